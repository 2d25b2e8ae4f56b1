"""Generate tests/golden/sublabel_*.npz: the sublabel lifting model of
opymize_gb300/tools/lifting.py assembled from the REFERENCE's classes and
solved by the reference's own CPU PDHG (opymize/solvers/pdhg.py:229-315,
precision="double").

    python oracle/build_ref.py
    python tests/golden/make_sublabel_golden.py

The reference's EpigraphProj CPU path needs cvxpy + MOSEK (absent here); it
is replaced by the reference's own GPU QP (`epigraphproj`, proj.cu:222-831)
compiled for the host by oracle/build_ref.py.  The shims of
make_epigraph_golden.py (identity numba.jit, cvxpy stand-in for
EpigraphProj.__init__, numpy-1 meaning of np.linalg.solve in EpigraphSupp's
constructor) apply.  Only the model's constant data comes from this package
(tools/lifting.py: labels, sample points, b, P, Bc, hull faces).
"""

import importlib.util
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_spec = importlib.util.spec_from_file_location("make_epigraph_golden",
                                               os.path.join(HERE, "make_epigraph_golden.py"))
meg = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(meg)

from opymize.solvers import PDHG                                     # noqa: E402
from opymize.functionals import (SplitSum, PositivityFct, ZeroFct,     # noqa: E402
                                 IndicatorFct, L1Norms)
from opymize.linear import BlockOp                                     # noqa: E402
from opymize.linear.diff import GradientOp                             # noqa: E402
from opymize.linear.einsum import MatrixMultR                          # noqa: E402
from opymize.linear.indexed import IndexedMultAdj                      # noqa: E402
from opymize.linear.scale import IdentityOp, ScaleOp                   # noqa: E402
from opymize.operators.proj import EpigraphProj                        # noqa: E402

from opymize_gb300.tools import lifting                                # noqa: E402
from opymize_gb300.tools.synthetic import piecewise_constant           # noqa: E402


def _call_cpu(self, x, y=None, add=False, jacobian=False):
    """EpigraphProj on the CPU through the reference's own QP kernel."""
    assert not add and not jacobian
    shape = self.x[0]['shape']
    out = x if y is None else y
    out[:] = meg.ref_proj(self.I, self.J, self.v, self.b, x.reshape(shape)).ravel()


EpigraphProj._call_cpu = _call_cpu


def ref_model(img, L, lbd, samples, trunc):
    dims = img.shape
    N, D = int(np.prod(dims)), len(dims)
    d = lifting.sublabel_data(img.ravel(), L, samples, trunc)
    If = lifting.faces(d)
    nmu = (L - 1) * N * 2
    g = SplitSum([PositivityFct(N * L), ZeroFct(N), ZeroFct(nmu)])
    supp = meg.ref_supp(d["I"], If, d["J"], d["v"], d["b"], with_conj=True)
    f = SplitSum([IndicatorFct(N * L), IndicatorFct(N), L1Norms(N, (1, D), lbd),
                  IndicatorFct(N, c1=1.0), supp])
    A = BlockOp([
        [IdentityOp(N * L), 0, IndexedMultAdj(L, N, d["P"], d["Bc"])],
        [MatrixMultR(N, d["t"][:, None]), ScaleOp(N, -1.0), 0],
        [0, GradientOp(dims, 1, scheme="forward"), 0],
        [MatrixMultR(N, np.ones((L, 1))), 0, 0],
        [0, 0, IdentityOp(nmu)]])
    return g, f, A, d, If


def run(name, shape, L, lbd, samples, trunc, steps, iters, gran, seed):
    img = piecewise_constant(shape, 1, sigma=0.05, seed=seed, salt_pepper=0.1)[..., 0]
    img = np.clip(img, 0.0, 1.0)
    g, f, A, d, If = ref_model(img, L, lbd, samples, trunc)
    solver = PDHG(g, f, A)
    dumps, infos = [], []

    def cb(state, info):
        dumps.append((info["iter"], state[0].copy(), state[1].copy()))
        infos.append((info["iter"], info["objp"], info["objd"], info["gap"],
                      info["infeasp"], info["infeasd"]))

    np.random.seed(0)
    solver.solve(steps=steps, precision="double", term_pd_gap=1e-300, term_maxiter=iters,
                 granularity=gran, use_gpu=False, cbfun=cb)
    faces_flat = np.concatenate([np.concatenate(row) for row in If])
    nfaces = np.array([[len(fc) for fc in row] for row in If])
    np.savez_compressed(
        os.path.join(HERE, name + ".npz"), img=img, L=L, lbd=lbd, samples=samples, trunc=trunc,
        steps=steps, iters=iters, gran=gran, faces=faces_flat, nfaces=nfaces,
        dump_iters=np.array([t for t, _, _ in dumps]), x=np.stack([x for _, x, _ in dumps]),
        y=np.stack([y for _, _, y in dumps]), info=np.array(infos))
    print(name, "final gap", infos[-1])


def main():
    run("sublabel_small_precond", (9, 8), 5, 0.1, 5, 0.04, "precond", 200, 50, 4)
    run("sublabel_small_adaptive", (7, 10), 4, 0.15, 4, 0.04, "adaptive", 150, 50, 9)


if __name__ == "__main__":
    main()
