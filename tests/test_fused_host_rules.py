"""CPU checks of the fused path's host-side rules in libopyx.

The batched solve's work list (`opyx_rof_batch_describe`): the sizing call,
every pixel of every active instance in exactly one work item, items of one
instance consecutive and in one tile-width class, tiles of equal width (a
multiple of 4) in the class that leaves the fewest lanes idle, inactive
instances without items, and the argument errors.  The single-sweep
selection (`opyx_rof_uses_sweep`).  No device memory is touched: the buffers
are aligned placeholder addresses that the host code only copies."""

import ctypes as C

import numpy as np
import pytest

from opymize_gb300 import _lib

CLASS_TW = (128, 256, 512)
ITEM_BYTES = 20          # five int32: inst, r0, r1, q_beg, q_end


@pytest.fixture(scope="module")
def lib():
    import os
    if not os.path.exists(_lib.LIB_PATH):
        from opymize_gb300 import build
        build.build()
    return _lib.load()


def problems(shapes, C_=1, steps=2):
    n = len(shapes)
    probs = (_lib.opyx_rof_problem * n)()
    bufs = (_lib.opyx_rof_buffers * n)()
    base = 1 << 40
    for i, (H, W) in enumerate(shapes):
        p = probs[i]
        p.dtype, p.ndim, p.nchannels, p.steps = _lib.OPYX_F32, 2, C_, steps
        p.dims[0], p.dims[1] = H, W
        p.h[0] = p.h[1] = 1.0
        for k in range(C_):
            p.weights[k] = p.vol[k] = 1.0
        p.lbd, p.theta, p.tau, p.sigma = 0.1, 1.0, 0.3, 0.3
        p.term_mode, p.term_relgap, p.term_infeas = 1, 1e-4, 1e-4
        b = bufs[i]
        addr = base + i * (1 << 32)
        b.x, b.xbar, b.y, b.y2, b.f = (addr + j * (1 << 28) for j in range(5))
    return probs, bufs


def describe(lib, probs, bufs, active, rows, records=1 << 39):
    n = len(probs)
    act = None if active is None else np.ascontiguousarray(active, dtype=np.uint8)
    aptr = None if act is None else act.ctypes.data
    nitems = C.c_int(-1)
    st = lib.opyx_rof_batch_describe(probs, bufs, n, C.c_void_p(records), aptr, rows, None, 0,
                                     C.byref(nitems))
    assert st == _lib.OPYX_ERR_WORKSPACE and nitems.value >= 0
    nbytes = lib.opyx_rof_batch_desc_bytes(n, nitems.value)
    host = np.zeros(nbytes, np.uint8)
    st = lib.opyx_rof_batch_describe(probs, bufs, n, C.c_void_p(records), aptr, rows,
                                     host.ctypes.data, nbytes, C.byref(nitems))
    assert st == _lib.OPYX_OK
    hdr = host[:32].view(np.int32)
    items = host[nbytes - nitems.value * ITEM_BYTES:].view(np.int32).reshape(-1, 5)
    return hdr, items, nitems.value


def expected_class(W):
    costs = [-(-W // tw) * tw for tw in CLASS_TW]
    best = min(costs)
    return max(c for c in range(3) if costs[c] == best)      # ties to the wider class


SHAPES = [(1, 4), (7, 124), (64, 128), (129, 132), (33, 300), (16, 512), (9, 700),
          (40, 1024), (5, 1100), (300, 260)]


@pytest.mark.parametrize("rows", [1, 8, 16])
@pytest.mark.parametrize("masked", [False, True])
def test_items_cover_every_pixel_once(lib, rows, masked):
    probs, bufs = problems(SHAPES)
    active = np.array([1, 0, 1, 1, 0, 1, 1, 1, 0, 1]) if masked else None
    hdr, items, nitems = describe(lib, probs, bufs, active, rows)
    ninst, n_items, nch = hdr[0], hdr[1], hdr[2]
    class_beg = hdr[4:8]
    assert (ninst, n_items, nch) == (len(SHAPES), nitems, 1)
    assert class_beg[0] == 0 and class_beg[3] == nitems and np.all(np.diff(class_beg) >= 0)
    seen = set()
    for i, (H, W) in enumerate(SHAPES):
        own = np.nonzero(items[:, 0] == i)[0]
        if active is not None and not active[i]:
            assert own.size == 0
            continue
        # consecutive, in the class that fills the most lanes, equal tiles
        assert own.size and np.all(np.diff(own) == 1)
        cls = expected_class(W)
        assert class_beg[cls] <= own[0] and own[-1] < class_beg[cls + 1]
        it = items[own]
        widths = it[:, 4] - it[:, 3]
        assert np.all(it[:, 3] % 4 == 0) and np.all(widths > 0)
        assert widths.max() <= CLASS_TW[cls] and len(set(widths[it[:, 4] < W])) <= 1
        assert np.all(it[:, 2] - it[:, 1] <= rows) and np.all(it[:, 1] < it[:, 2])
        cover = np.zeros((H, W), np.int32)
        for _, r0, r1, q0, q1 in it:
            assert 0 <= r0 < r1 <= H and 0 <= q0 < q1 <= W
            cover[r0:r1, q0:q1] += 1
        assert np.all(cover == 1)
        ntiles = -(-W // CLASS_TW[cls])
        assert len(set(it[:, 3])) == ntiles and own.size == ntiles * -(-H // rows)
        seen.update(own.tolist())
    assert seen == set(range(nitems))


def test_argument_errors(lib):
    probs, bufs = problems(SHAPES[:3])
    n = C.c_int(0)
    rec = C.c_void_p(1 << 39)
    assert lib.opyx_rof_batch_describe(probs, bufs, 3, rec, None, 0, None, 0,
                                       C.byref(n)) == _lib.OPYX_ERR_ARG
    assert lib.opyx_rof_batch_describe(probs, bufs, 3, C.c_void_p((1 << 39) + 64), None, 8,
                                       None, 0, C.byref(n)) == _lib.OPYX_ERR_WORKSPACE
    # one channel count per batch
    probs[1].nchannels = 2
    probs[1].vol[1] = probs[1].weights[1] = 1.0
    assert lib.opyx_rof_batch_describe(probs, bufs, 3, rec, None, 8, None, 0,
                                       C.byref(n)) == _lib.OPYX_ERR_ARG
    # FP32 constant or preconditioned steps only
    probs, bufs = problems(SHAPES[:3], steps=1)
    for p, b in zip(probs, bufs):
        p.alpha0, p.eta, p.Delta = 0.5, 0.95, 1.5
        b.xgrad, b.gp = b.x + (1 << 27), b.y + (1 << 27)
    assert lib.opyx_rof_batch_describe(probs, bufs, 3, rec, None, 8, None, 0,
                                       C.byref(n)) == _lib.OPYX_ERR_UNSUPPORTED
    probs, bufs = problems(SHAPES[:3])
    probs[2].dtype = _lib.OPYX_F64
    assert lib.opyx_rof_batch_describe(probs, bufs, 3, rec, None, 8, None, 0,
                                       C.byref(n)) == _lib.OPYX_ERR_UNSUPPORTED
    # rows whose length is not a multiple of 4 cannot stream as quads
    probs, bufs = problems([(8, 130)])
    assert lib.opyx_rof_batch_describe(probs, bufs, 1, rec, None, 8, None, 0,
                                       C.byref(n)) == _lib.OPYX_ERR_ARG


def _one(ndim, dims, C_=1, steps=2, dtype=None, y2=True):
    p = _lib.opyx_rof_problem()
    p.dtype = _lib.OPYX_F32 if dtype is None else dtype
    p.ndim, p.nchannels, p.steps = ndim, C_, steps
    for t, n in enumerate(dims):
        p.dims[t], p.h[t] = n, 1.0
    for k in range(C_):
        p.weights[k] = p.vol[k] = 1.0
    p.lbd, p.theta, p.tau, p.sigma = 0.1, 1.0, 0.3, 0.3
    p.alpha0, p.eta, p.Delta = 0.5, 0.95, 1.5
    b = _lib.opyx_rof_buffers()
    a = 1 << 40
    b.x, b.xbar, b.y, b.f, b.ws = a, a + (1 << 30), a + (2 << 30), a + (3 << 30), a + (4 << 30)
    b.xgrad, b.gp = a + (5 << 30), a + (6 << 30)
    if y2:
        b.y2 = a + (7 << 30)
    return p, b


SWEEP_CASES = [
    (dict(ndim=2, dims=(64, 128)), 1),
    (dict(ndim=2, dims=(64, 128), C_=3), 1),
    (dict(ndim=2, dims=(64, 128), steps=0), 1),                   # constant steps
    (dict(ndim=2, dims=(64, 128), steps=1), 0),                   # adaptive: two passes and R
    (dict(ndim=2, dims=(64, 128), dtype=_lib.OPYX_F64), 0),
    (dict(ndim=2, dims=(64, 128), y2=False), 0),                  # no ping-pong buffer for y
    (dict(ndim=2, dims=(64, 130)), 0),                            # rows not in quads
    (dict(ndim=3, dims=(16, 32, 256)), 1),
    (dict(ndim=3, dims=(16, 32, 128)), 1),
    (dict(ndim=3, dims=(16, 32, 512)), 1),
    (dict(ndim=3, dims=(16, 32, 64)), 0),                         # other row lengths: two passes
    (dict(ndim=3, dims=(16, 32, 256), C_=2), 0),                  # several channels: two passes
    (dict(ndim=1, dims=(4096,)), 0),
]


@pytest.mark.parametrize("case", range(len(SWEEP_CASES)))
def test_single_sweep_selection(lib, case):
    """opyx_rof_uses_sweep (host code): the single sweep runs for FP32 with
    constant or preconditioned steps and a y2 buffer -- 2-D, or 3-D with one
    channel and rows of 128, 256 or 512 pixels, unmasked."""
    kw, want = SWEEP_CASES[case]
    p, b = _one(**kw)
    assert lib.opyx_rof_uses_sweep(C.byref(p), C.byref(b)) == want
    if kw["ndim"] == 3 and want:
        b.mask = (1 << 40) + (8 << 30)
        assert lib.opyx_rof_uses_sweep(C.byref(p), C.byref(b)) == 0
    b.y2 = (b.y2 or 0) + 4                                          # misaligned y2
    assert lib.opyx_rof_uses_sweep(C.byref(p), C.byref(b)) == 0


@pytest.mark.parametrize("t_persist,t_graphs,want", [(0.92, 0.89, "persistent"),
                                                      (0.756, 0.74, "persistent"),
                                                      (1.00, 1.05, "persistent"),
                                                      (1.20, 1.00, "graphs")])
def test_batch_mode_choice(t_persist, t_graphs, want):
    """BatchROF.autotune for one-channel batches without a fixed mode: both
    modes tuned, the persistent launch kept unless the graphs' iteration with
    every instance active is more than PERSIST_MARGIN times faster (host
    rule; the timings are given)."""
    from types import SimpleNamespace
    from opymize_gb300.solvers.batch import BatchROF

    def tune(ms, rows, gran):
        def f(iters):
            s.tuning = {"rows_per_item": rows, "ms_per_iteration": ms}
            s.rows_per_item, s.gran = rows, gran
            return rows
        return f

    s = SimpleNamespace(_persistent_req=None, C=1, PERSIST_MARGIN=BatchROF.PERSIST_MARGIN,
                        tuning=None, gran=None, rows_per_item=None, persistent=None)
    s._autotune_persistent = tune(t_persist, 32, 58)
    s._autotune_graphs = tune(t_graphs, 8, 70)
    rows = BatchROF.autotune(s)
    assert s.tuning["mode"] == want and s.persistent == (want == "persistent")
    assert (rows, s.gran) == ((32, 58) if want == "persistent" else (8, 70))
    assert s.tuning["ms_per_iteration_other_mode"] == (t_graphs if s.persistent else t_persist)
