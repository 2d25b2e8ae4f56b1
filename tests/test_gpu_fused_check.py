"""opyx_rof_gap_iterate: the check at the end of one granularity chunk
(opymize/solvers/pdhg.py:285-305) queued with the next chunk's iterations.
With single sweeps the first sweep computes the gap of the state it reads;
the result must equal opyx_rof_gap followed by opyx_rof_iterate -- the state
bit for bit, the info record up to the order of the FP64 sums -- and a check
that passes the stop test must leave the checked state in place."""

import os

import numpy as np
import pytest

from tests.conftest import GOLDEN
from tests.test_gpu_pdhg import gpu_problem

pytestmark = pytest.mark.gpu

FIXTURES = ["g2d_precond_fwd", "g2d_const_fwd", "g2d_const_imageh", "c2d_precond_fwd",
            "c2d_huber_precond", "c2d_volmask_const"]
# (H, W, C, huber): several tiles with a ragged last one, rows of one narrow
# tile (128 / 256 pixels), two and four channels
SHAPES = [(70, 1028, 1, 0.0), (33, 300, 1, 0.0), (48, 20, 2, 0.0), (30, 260, 4, 0.0),
          (64, 516, 3, 0.02), (5, 132, 1, 0.0)]


def fused_solver(G, F, A, steps, iters=6):
    """A solver whose fused FP32 buffers (single sweeps) hold the state after
    `iters` iterations."""
    from opymize_gb300.solvers import PDHG
    s = PDHG(G, F, A)
    s.solve(steps=steps, precision="float", term_pd_gap=1e-300, term_maxiter=iters,
            granularity=3)
    assert s.path == "fused"
    return s


def from_fixture(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    return fused_solver(*gpu_problem(d), steps=str(d["steps"]))


def from_shape(H, W, C, huber):
    from opymize_gb300.functionals import SSD, L1Norms, HuberL1Norms
    from opymize_gb300.linear import GradientOp
    from opymize_gb300.tools.synthetic import piecewise_constant
    f = piecewise_constant((H, W), C, sigma=0.1, seed=H + W + C)
    N = H * W
    F = HuberL1Norms(N, (C, 2), 0.1, huber) if huber > 0 else L1Norms(N, (C, 2), 0.1)
    return fused_solver(SSD(f.reshape(N, C)), F, GradientOp((H, W), C, scheme="forward"),
                        steps="precond")


def info(fz):
    from opymize_gb300 import _lib
    off = _lib.load().opyx_rof_info_offset() // 8
    rec = fz["ws"][off:off + len(_lib.ROF_INFO_FIELDS)].get().copy()
    return dict(zip(_lib.ROF_INFO_FIELDS, rec))


def both_ways(s, iters, relgap_tol=1e-300):
    """(state, info) after gap + iterate and after gap_iterate, from the same
    start."""
    from opymize_gb300 import _lib
    from opymize_gb300.gpuarray import stream_ptr
    fz = s._fused
    p, b = fz["problem"], fz["buffers"]
    assert _lib.load().opyx_rof_uses_sweep(p, b)
    p.term_mode, p.term_relgap, p.term_infeas = 1, relgap_tol, 1e300
    x0, y0 = fz["x"].get().copy(), fz["y"].get().copy()
    out = []
    for fused in (False, True):
        fz["x"].set(x0)
        fz["y"].set(y0)
        _lib.call("opyx_rof_init", p, b, stream_ptr())
        if fused:
            _lib.call("opyx_rof_gap_iterate", p, b, iters, stream_ptr())
        else:
            _lib.call("opyx_rof_gap", p, b, stream_ptr())
            _lib.call("opyx_rof_iterate", p, b, iters, stream_ptr())
        out.append((fz["x"].get().copy(), fz["y"].get().copy(), info(fz)))
    return (x0, y0), out


def check_equal(out):
    (xa, ya, ra), (xb, yb, rb) = out
    np.testing.assert_array_equal(xa, xb)
    np.testing.assert_array_equal(ya, yb)
    assert ra["checks"] == rb["checks"] == 1 and rb["fault"] == 0
    for k in ("objp", "objd"):
        assert abs(ra[k] - rb[k]) <= 1e-6 * max(1.0, abs(ra[k])), (k, ra[k], rb[k])
    # FP32 partial sums in another order: the gap's absolute bar of the
    # batched tests (1e-7 of |objd|)
    assert abs(ra["relgap"] - rb["relgap"]) <= 1e-7 + 1e-5 * abs(ra["relgap"])
    assert ra["infeasd"] == rb["infeasd"]          # a max: order-free


@pytest.mark.parametrize("name", FIXTURES)
def test_fixture_problems(name):
    _, out = both_ways(from_fixture(name), 4)
    check_equal(out)


@pytest.mark.parametrize("shape", SHAPES)
def test_tilings_and_channels(shape):
    _, out = both_ways(from_shape(*shape), 6)
    check_equal(out)


def test_odd_iteration_count():
    _, out = both_ways(from_shape(70, 1028, 1, 0.0), 5)
    check_equal(out)


def test_passing_check_keeps_the_checked_state():
    (x0, y0), out = both_ways(from_shape(64, 516, 3, 0.02), 6, relgap_tol=1e30)
    for x, y, rec in out:
        np.testing.assert_array_equal(x, x0)
        np.testing.assert_array_equal(y, y0)
        assert rec["done"] == 1 and rec["checks"] == 1


@pytest.mark.parametrize("dims,C,huber,lbd,gran", [((256, 256), 1, 0.0, 0.1, 10),
                                                   ((128, 200), 3, 0.01, 0.05, 6)])
def test_solve_matches_loop_waiting_at_checks(dims, C, huber, lbd, gran):
    """PDHG.solve queues each check with the next chunk (no callback) or runs
    the gap kernel after each chunk (with one): the same stop iteration and
    state, the gap records equal up to summation order."""
    from opymize_gb300.functionals import SSD, L1Norms, HuberL1Norms
    from opymize_gb300.linear import GradientOp
    from opymize_gb300.solvers import PDHG
    from opymize_gb300.tools.synthetic import piecewise_constant
    f = piecewise_constant(dims, C, sigma=0.1, seed=5)
    N = dims[0] * dims[1]
    res = []
    for waits in (False, True):
        F = HuberL1Norms(N, (C, 2), lbd, huber) if huber > 0 else L1Norms(N, (C, 2), lbd)
        s = PDHG(SSD(f.reshape(N, C)), F, GradientOp(dims, C, scheme="forward"))
        seen = []
        cb = (lambda state, info: seen.append(info["relgap"])) if waits else None
        s.solve(steps="precond", precision="float", term_pd_gap=1e-3, term_maxiter=5000,
                granularity=gran, cbfun=cb)
        assert s.path == "fused"
        res.append(s)
    ahead, wait = res
    assert 0 < ahead.info["iter"] == wait.info["iter"] < 5000
    np.testing.assert_array_equal(ahead.state[0], wait.state[0])
    np.testing.assert_array_equal(ahead.state[1], wait.state[1])
    assert abs(ahead.info["relgap"] - wait.info["relgap"]) <= 1e-7 + 1e-5 * abs(wait.info["relgap"])
