"""The benchmarked configurations at their full sizes against the FP64 oracle.

* colour: 2048 x 2048 x 3 FP32, Huber-smoothed joint TV (alpha 0.01,
  lambda 0.05), preconditioned steps, single sweeps, gap every 6 iterations
  -- the bench's headline problem, same seed;
* volume: 256^3 FP32 TV (lambda 0.08), preconditioned steps, 3-D sweeps.

The oracle is the numpy/scipy port of the reference's CPU solver
(opymize/solvers/pdhg.py:229-315), run over every host thread by
oracle.threaded (bit-identical to the one-thread oracle; tests/
test_oracle_threaded.py).  Bars: relative L2 error of x and y <= 1e-5 after
the same iteration count, the gap at every check to 1e-6 absolute, and the
iteration at which the stop test |relgap| < 1e-4 first holds."""

import numpy as np
import pytest

from oracle.threaded import ThreadedROF

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


def rel(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return np.linalg.norm(a - b) / max(1e-300, np.linalg.norm(b))


def gpu_solve(f, dims, lbd, huber, iters, gran, tol=1e-300):
    from opymize_gb300 import _lib
    from opymize_gb300.solvers import PDHG
    from opymize_gb300.functionals import SSD, L1Norms, HuberL1Norms
    from opymize_gb300.linear import GradientOp
    N, C, D = int(np.prod(dims)), f.shape[-1], len(dims)
    F = HuberL1Norms(N, (C, D), lbd, huber) if huber > 0 else L1Norms(N, (C, D), lbd)
    s = PDHG(SSD(f.reshape(N, C)), F, GradientOp(dims, C, scheme="forward"))
    gaps = {}
    s.solve(steps="precond", precision="float", term_pd_gap=tol, term_maxiter=iters,
            granularity=gran, cbfun=lambda st, info: gaps.__setitem__(info["iter"],
                                                                     info["relgap"]))
    assert s.path == "fused"
    fz = s._fused
    assert fz["y2"] is not None
    assert bool(_lib.load().opyx_rof_uses_sweep(fz["problem"], fz["buffers"]))
    return s, gaps


def oracle_solve(f, dims, lbd, huber, iters, gran, tol=1e-300):
    t = ThreadedROF(f.reshape(-1, f.shape[-1]), dims, lbd, huber)
    gaps = {}
    t._setup()
    it = 0
    while it < iters:
        it += 1
        t._iterate()
        if it % gran == 0:
            g = t.pd_gap()
            gaps[it] = g["relgap"]
            if abs(g["relgap"]) < tol:
                break
    state = (t.state[0].copy(), t.state[1].copy())
    t.close()
    return state, gaps, it


def test_colour_2048x2048x3_bench_problem():
    from opymize_gb300.tools.synthetic import piecewise_constant
    dims, C = (2048, 2048), 3
    f = piecewise_constant(dims, C, sigma=0.1, seed=0)
    # fixed 30 iterations (the bench's solve stops at 30)
    s, g_gpu = gpu_solve(f, dims, 0.05, 0.01, 30, 6)
    (xo, yo), g_or, _ = oracle_solve(f, dims, 0.05, 0.01, 30, 6)
    ex, ey = rel(s.state[0], xo), rel(s.state[1], yo)
    assert ex <= 1e-5 and ey <= 1e-5, (ex, ey)
    for it in g_or:
        assert abs(g_gpu[it] - g_or[it]) <= 1e-6, (it, g_gpu[it], g_or[it])
    # the stop test fires at the same check
    s2, g2 = gpu_solve(f, dims, 0.05, 0.01, 5000, 6, tol=1e-4)
    _, _, it_or = oracle_solve(f, dims, 0.05, 0.01, 5000, 6, tol=1e-4)
    assert s2.info["iter"] == it_or, (s2.info["iter"], it_or)


def test_volume_256cubed_bench_problem():
    from opymize_gb300.tools.synthetic import piecewise_constant
    dims = (256, 256, 256)
    f = piecewise_constant(dims, 1, sigma=0.1, seed=0)
    s, g_gpu = gpu_solve(f, dims, 0.08, 0.0, 30, 10)
    (xo, yo), g_or, _ = oracle_solve(f, dims, 0.08, 0.0, 30, 10)
    ex, ey = rel(s.state[0], xo), rel(s.state[1], yo)
    assert ex <= 1e-5 and ey <= 1e-5, (ex, ey)
    for it in g_or:
        assert abs(g_gpu[it] - g_or[it]) <= 1e-6 + 1e-4 * abs(g_or[it]), (it, g_gpu[it], g_or[it])
