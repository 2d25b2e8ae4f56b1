"""Functionals (opymize/functionals) evaluated and proxed on the GPU."""

import numpy as np

from opymize_gb300 import Variable, Functional
from opymize_gb300.gpuarray import DeviceArray
from opymize_gb300.operators import SplitOp
from opymize_gb300.functionals.quad import SSD                                  # noqa: F401
from opymize_gb300.functionals.l1norms import (L1Norms, L1NormsConj,            # noqa: F401
                                               HuberL1Norms, HuberL1NormsConj)
from opymize_gb300.functionals.epigraph import (QuadEpiInd, QuadEpiSupp,        # noqa: F401
                                                QuadSupport, HuberPerspective,
                                                TruncQuadEpiInd, quad_dual_coefficients,
                                                EpigraphInd, EpigraphFct, EpigraphSupp,
                                                EpigraphSupportFct)
from opymize_gb300.functionals.indicators import (AffineFct, ConstFct, ZeroFct,  # noqa: F401
                                                  MaskedAffineFct, IndicatorFct,
                                                  ConstrainFct, PositivityFct,
                                                  NegativityFct)


class SplitSum(Functional):
    """F(x1, x2, ...) = F1(x1) + F2(x2) + ... (opymize/functionals/__init__.py:10-39)."""

    def __init__(self, fcts, conj=None):
        Functional.__init__(self)
        self.x = Variable(*[(F.x.size,) for F in fcts])
        self.fcts = fcts
        self.conj = SplitSum([F.conj for F in fcts], conj=self) if conj is None else conj

    def _eval_gpu(self, x):
        res = [F(xi) for F, xi in zip(self.fcts, self.x.vars(x))]
        return sum(r[0] for r in res), max(r[1] for r in res)

    def prox(self, tau):
        if isinstance(tau, DeviceArray):
            return SplitOp([F.prox(t) for F, t in zip(self.fcts, self.x.vars(tau))])
        if isinstance(tau, np.ndarray):
            raise TypeError("per-element steps must be DeviceArrays on the GPU path")
        return SplitOp([F.prox(tau) for F in self.fcts])
