"""Device-side stop test of the fused path.

The fused solve queues check chunks ahead of the host's reads; the gap
kernel evaluates the reference's stop test (opymize/solvers/pdhg.py:290-305)
and every kernel queued after the passing check returns at once.  These tests
check that the result equals a loop that waits at every check: the stop
iteration derived from the reference's own gap records (tests/golden), the
state bit for bit, and that kernels after the stop leave the state alone."""

import os

import numpy as np
import pytest

from tests.conftest import GOLDEN
from tests.test_gpu_pdhg import gpu_problem

pytestmark = pytest.mark.gpu


def expected_stop(d, tol):
    """First check of the reference's run that passes |relgap| < tol and
    max(infeasp, infeasd) < tol, from the fixture's info records."""
    for j, it in enumerate(d["info_iters"]):
        if abs(d["info_relgap"][j]) < tol and \
                max(d["info_infeasp"][j], d["info_infeasd"][j]) < tol:
            return int(it)
    return None


def solve(d, tol, precision="double", waits=False, graph=True, maxiter=100000, **kw):
    from opymize_gb300.solvers import PDHG
    G, F, A = gpu_problem(d)
    s = PDHG(G, F, A)
    cb = (lambda state, info: None) if waits else None
    np.random.seed(0)      # constant steps come from normest's random draws
    s.solve(steps=str(d["steps"]), precision=precision, term_pd_gap=tol,
            term_maxiter=maxiter, granularity=int(d["gran"]), cbfun=cb, graph=graph, **kw)
    assert s.path == "fused"
    return s


@pytest.mark.parametrize("case", ["g2d_precond_fwd", "c2d_huber_precond", "g2d_const_fwd",
                                  "v3d_precond_fwd"])
def test_stop_iteration_matches_reference(case):
    d = np.load(os.path.join(GOLDEN, case + ".npz"))
    rg = np.abs(d["info_relgap"])
    # a tolerance halfway (geometrically) between the third and fourth checks
    tol = float(np.sqrt(rg[2] * rg[3])) if rg[3] < rg[2] else float(rg[2]) * 0.999
    want = expected_stop(d, tol)
    if want is None:
        pytest.skip("the fixture's run never passes the stop test")
    ahead = solve(d, tol)
    wait = solve(d, tol, waits=True)
    eager = solve(d, tol, graph=False)
    for s in (ahead, wait, eager):
        assert s.info["iter"] == want, (case, s.info["iter"], want)
    for s in (wait, eager):
        np.testing.assert_array_equal(ahead.state[0], s.state[0])
        np.testing.assert_array_equal(ahead.state[1], s.state[1])
        for k in ("objp", "objd", "gap", "relgap", "infeasd"):
            assert ahead.info[k] == s.info[k], (k, ahead.info[k], s.info[k])
    j = list(d["info_iters"]).index(want)
    assert abs(ahead.info["objp"] - d["info_objp"][j]) <= 1e-10 * max(1, abs(d["info_objp"][j]))


def test_kernels_return_after_stop():
    from opymize_gb300 import _lib
    from opymize_gb300.gpuarray import stream_ptr
    d = np.load(os.path.join(GOLDEN, "g2d_precond_fwd.npz"))
    s = solve(d, 1e30)                 # the first check passes
    assert s.info["iter"] == int(d["gran"])
    fz = s._fused
    x0, y0 = fz["x"].get().copy(), fz["y"].get().copy()
    off = _lib.load().opyx_rof_info_offset() // 8
    nrec = len(_lib.ROF_INFO_FIELDS)
    rec0 = fz["ws"][off:off + nrec].get().copy()
    names = _lib.ROF_INFO_FIELDS
    assert rec0[names.index("checks")] == 1 and rec0[names.index("done")] == 1  # stopped
    assert rec0[names.index("fault")] == 0
    _lib.call("opyx_rof_iterate", fz["problem"], fz["buffers"], 7, stream_ptr())
    _lib.call("opyx_rof_gap", fz["problem"], fz["buffers"], stream_ptr())
    np.testing.assert_array_equal(fz["x"].get(), x0)
    np.testing.assert_array_equal(fz["y"].get(), y0)
    np.testing.assert_array_equal(fz["ws"][off:off + nrec].get(), rec0)
    # opyx_rof_init clears the flag: the same buffers iterate again
    _lib.call("opyx_rof_init", fz["problem"], fz["buffers"], stream_ptr())
    _lib.call("opyx_rof_iterate", fz["problem"], fz["buffers"], 1, stream_ptr())
    assert not np.array_equal(fz["x"].get(), x0)


def test_fp32_stop_matches_waiting_loop():
    d = np.load(os.path.join(GOLDEN, "c2d_precond_fwd.npz"))
    tol = float(np.abs(d["info_relgap"][1])) * 0.9
    ahead = solve(d, tol, precision="float")
    wait = solve(d, tol, precision="float", waits=True)
    assert ahead.info["iter"] == wait.info["iter"]
    np.testing.assert_array_equal(ahead.state[0], wait.state[0])
    np.testing.assert_array_equal(ahead.state[1], wait.state[1])


def test_residual_stop_adaptive():
    """term_pd_res (adaptive steps, residual test pdhg.py:295-298)."""
    from opymize_gb300.solvers import PDHG
    d = np.load(os.path.join(GOLDEN, "c2d_huber_adaptive.npz"))
    res = {}
    for waits in (False, True):
        G, F, A = gpu_problem(d)
        s = PDHG(G, F, A)
        seen = []
        cb = (lambda state, info: seen.append((info["iter"], info["resp"], info["epsp"],
                                               info["resd"], info["epsd"]))) if waits else None
        np.random.seed(0)
        s.solve(precision="double", term_pd_res=1e-3, term_maxiter=20000,
                granularity=int(d["gran"]), cbfun=cb)
        assert s.path == "fused"
        res[waits] = (s, seen)
    ahead, (wait, seen) = res[False][0], res[True]
    assert ahead.info["iter"] == wait.info["iter"] < 20000
    it, rp, ep, rd, ed = seen[-1]
    assert it == wait.info["iter"] and rp < ep and rd < ed
    assert all(not (r[1] < r[2] and r[3] < r[4]) for r in seen[:-1])
    np.testing.assert_array_equal(ahead.state[0], wait.state[0])
