"""CPU oracle of Opymize's PDHG path -- TEST INFRASTRUCTURE ONLY.

This package restates, in numpy/scipy, the reference's CPU implementation of
the PDHG solver (opymize/solvers/pdhg.py), its linear operators
(opymize/linear/*), functionals (opymize/functionals/*) and prox operators
(opymize/operators/*).  Each function cites the reference file:line it
follows.

It is the checker, never the product: only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg and
``--impl reference`` arm import it.  The ``opymize_gb300`` package never
imports it and has no CPU fallback.

Pinning: ``tests/test_oracle.py`` checks every function here against the
fixtures in ``tests/golden/``, which ``tests/golden/make_golden.py`` produced
by running the reference's own Python code (and the golden gradient values
held in the reference's tests/sparse.py:59-93).
"""

from oracle.linops import (Gradient, Divergence, Laplacian, MatrixMult,   # noqa: F401
                           MatrixMultR, MatrixMultRBatched, TangledMatrixMultR,
                           DiagMatrixMultR, IndexedMult, IndexedMultAdj,
                           ZeroOp, ScaleOp, IdentityOp, BlockOp, normest)
from oracle.functionals import (SSD, L1Norms, L1NormsConj, HuberL1Norms,  # noqa: F401
                                HuberL1NormsConj, QuadEpiInd, QuadEpiSupp,
                                HuberPerspective, TruncQuadEpiInd, SplitSum,
                                PositivityFct, NegativityFct, ZeroFct,
                                IndicatorFct, AffineFct, ConstrainFct,
                                MaskedAffineFct)
from oracle.prox import (l1_projection, quadepi_projection,               # noqa: F401
                         solve_reduced_monic_cubic, truncate)
from oracle.pdhg import PDHG                                               # noqa: F401
