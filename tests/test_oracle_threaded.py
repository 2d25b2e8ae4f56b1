"""The oracle's PDHG over a thread pool (oracle.threaded, the CPU baseline
of bench.py) against the one-thread oracle: the same iterates bit for bit,
the same gap to rounding, the same stop iteration."""

import numpy as np
import pytest

import oracle
from oracle.threaded import ThreadedROF
from opymize_gb300.tools.synthetic import piecewise_constant


@pytest.mark.parametrize("dims,C,huber,threads", [((64, 48), 3, 0.01, 5), ((70, 33), 1, 0.0, 3),
                                                  ((12, 10, 9), 1, 0.0, 4)])
def test_threaded_matches_oracle(dims, C, huber, threads):
    f = piecewise_constant(dims, C, sigma=0.1, seed=1)
    N = int(np.prod(dims))
    D = len(dims)
    F = oracle.HuberL1Norms(N, (C, D), 0.05, huber) if huber > 0 else oracle.L1Norms(N, (C, D), 0.05)
    so = oracle.PDHG(oracle.SSD(f.reshape(N, C)), F, oracle.Gradient(dims, C, "forward"))
    so.solve(steps="precond", term_pd_gap=1e-300, term_maxiter=40, granularity=10)
    t = ThreadedROF(f.reshape(N, C), dims, 0.05, huber, threads=threads)
    info = t.solve(term_pd_gap=1e-300, term_maxiter=40, granularity=10)
    t.close()
    for a, b in zip(t.state, so.state):
        assert np.array_equal(a, b)
    for k in ("objp", "objd", "relgap", "infeasd"):
        assert abs(info[k] - so.info[k]) <= 1e-12 * max(1.0, abs(so.info[k]))


def test_threaded_stops_where_oracle_stops():
    dims, C = (40, 36), 1
    f = piecewise_constant(dims, C, sigma=0.1, seed=2)
    N = dims[0] * dims[1]
    so = oracle.PDHG(oracle.SSD(f.reshape(N, C)), oracle.L1Norms(N, (C, 2), 0.1),
                     oracle.Gradient(dims, C, "forward"))
    so.solve(steps="precond", term_pd_gap=1e-4, term_maxiter=5000, granularity=10)
    t = ThreadedROF(f.reshape(N, C), dims, 0.1, threads=4)
    info = t.solve(term_pd_gap=1e-4, term_maxiter=5000, granularity=10)
    t.close()
    assert info["iter"] == so.info["iter"]
