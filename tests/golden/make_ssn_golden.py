"""Golden fixtures for the semismooth Newton solver, generated by the
reference itself (its CPU-only ``SemismoothNewton``, opymize/solvers/
semismooth_newton.py:250-427, and ``L12ProjJacobian``, opymize/operators/
proj.py:228-276).  Run where the reference is mounted::

    python tests/golden/make_ssn_golden.py          # writes tests/golden/ssn.npz

Cases: gray 2-D ROF with SSD data and Frobenius L1 norms (the centered
gradient, the reference default), started from a few hundred reference PDHG iterations (the
reference's own example starts its Newton solver from a PDHG result,
examples/rof.py:79-85) or from zero; the Newton iterates after 1, 2 and 3
steps (each from the same start, ``np.random`` seeded before every solve
because the step bound comes from ``normest``), and the projection's
Jacobian applied to random vectors for one and three channels.  (On a
colour ROF case the reference's Armijo search stops with "Not a descent
direction", so the solver fixtures are gray.)
"""

import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("OPYMIZE_REF", "/root/reference")

_numba = types.ModuleType("numba")
_numba.jit = lambda *a, **k: (a[0] if a and callable(a[0]) else (lambda f: f))
sys.modules.setdefault("numba", _numba)
sys.path.insert(0, REF)
sys.path.insert(0, REPO)

from opymize.solvers import PDHG, SemismoothNewton              # noqa: E402
from opymize.functionals import SSD, L1Norms                     # noqa: E402
from opymize.linear.diff import GradientOp                      # noqa: E402
from opymize.operators.proj import L1NormsProj                  # noqa: E402

from opymize_gb300.tools.synthetic import piecewise_constant    # noqa: E402

CASES = [("gray", (24, 20), 1, 0.1, 300), ("zero", (24, 20), 1, 0.1, 0),
         ("gray2", (20, 28), 1, 0.05, 200)]
JACOBIAN_CASES = [("jac1", 480, 1, 0.1), ("jac3", 192, 3, 0.08)]


def main():
    out = {}
    for name, dims, C, lbd, pdhg_iters in CASES:
        f = piecewise_constant(dims, C, sigma=0.1, seed=31)
        N = int(np.prod(dims))
        D = len(dims)
        # GradientOp with its default centered scheme, as examples/rof.py:73
        G, F, A = SSD(f.reshape(N, C)), L1Norms(N, (C, D), lbd), GradientOp(dims, C)
        if pdhg_iters:
            np.random.seed(0)
            s = PDHG(G, F, A)
            s.solve(steps="precond", term_pd_gap=1e-300, term_maxiter=pdhg_iters,
                    granularity=pdhg_iters, use_gpu=False)
            start = np.concatenate([v.ravel() for v in s.state])
        else:
            start = np.zeros(N * C * (1 + D))
        out[name + "_f"] = f
        out[name + "_lbd"] = lbd
        out[name + "_start"] = start
        for k in (1, 2, 3):
            np.random.seed(1)
            ssn = SemismoothNewton(G, F, A)
            info = ssn.solve(continue_at=start.copy(), granularity=1, term_relgap=1e-300,
                             term_maxiter=k)
            x, y = ssn.state
            out["%s_xy%d" % (name, k)] = np.concatenate([x.ravel(), y.ravel()])
            out["%s_info%d" % (name, k)] = np.array([info[q] for q in
                                                     ("objp", "objd", "infeasp", "infeasd", "relgap")])
            out["%s_lbd%d" % (name, k)] = ssn.lbd
            out["%s_steps%d" % (name, k)] = np.array([ssn.constvars["tau"], ssn.constvars["sigma"]])
    for name, N, C, lbd in JACOBIAN_CASES:
        D = 2
        # the projection's Jacobian (Frobenius) at a point with interior and exterior groups
        rng = np.random.default_rng(5)
        xv = rng.standard_normal((N, C * D)) * lbd
        v = rng.standard_normal((N, C * D))
        proj = L1NormsProj(N, (C, D), lbd, "frobenius")
        xp = xv.copy().ravel()
        J = proj(xp, jacobian=True)
        jv = np.zeros(N * C * D)
        J(v.ravel(), jv)
        out[name + "_jac_x"] = xv
        out[name + "_jac_v"] = v
        out[name + "_jac_proj"] = xp
        out[name + "_jac_Jv"] = jv
    np.savez_compressed(os.path.join(HERE, "ssn.npz"), **out)
    print("wrote", os.path.join(HERE, "ssn.npz"), sorted(out))


if __name__ == "__main__":
    main()
