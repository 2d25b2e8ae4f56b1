"""GPU test of opyx_rof_iterate_noalloc, the entry point for callers that
cannot allocate device memory (code inside another framework's memory pool,
or hosts that only hold device pointers for the image and the iterates): its
scratch lives in a static device array of the library instead of a
caller-sized workspace.

The test calls it through the C ABI twice in a row (the second call
continues from the first call's output, and both reuse the same static
scratch) and compares x, y and the duality gap with the workspace entry
points (opyx_rof_init + opyx_rof_iterate + opyx_rof_gap) on the same
inputs, at the tolerances of the other GPU parity tests.  It lives in a file
of its own that pytest collects last."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problem(dtype, steps, dims, C, huber):
    from opymize_gb300 import _lib
    p = _lib.opyx_rof_problem()
    p.dtype = _lib.OPYX_F32 if dtype == np.float32 else _lib.OPYX_F64
    p.ndim, p.nchannels, p.steps = len(dims), C, _lib.STEPS[steps]
    for t, n in enumerate(dims):
        p.dims[t], p.h[t] = n, 1.0
    for k in range(C):
        p.weights[k], p.vol[k] = 1.0, 1.0
    p.lbd, p.huber_alpha, p.theta = 0.05, huber, 1.0
    p.tau = p.sigma = 0.35
    p.alpha0, p.eta, p.Delta = 0.5, 0.95, 1.5
    for j in range(4):
        p.eps[j] = 1e-4
    return p


@pytest.mark.parametrize("dtype,steps,dims,C,huber", [
    (np.float32, "precond", (384, 256), 3, 0.01),
    (np.float64, "adaptive", (96, 80), 1, 0.0),
    (np.float32, "const", (40, 30, 20), 1, 0.0),
])
def test_noalloc_matches_workspace_entry_point(dtype, steps, dims, C, huber):
    from opymize_gb300 import _lib
    from opymize_gb300.gpuarray import DeviceArray, stream_ptr, torch
    from opymize_gb300.tools.synthetic import piecewise_constant
    lib = _lib.load()
    f = piecewise_constant(dims, C, sigma=0.1, seed=5).astype(dtype).ravel()
    N = int(np.prod(dims))
    D = len(dims)
    p = _problem(dtype, steps, dims, C, huber)
    fd = DeviceArray.to_gpu(f, dtype)

    # workspace entry points
    x1 = DeviceArray.zeros((N * C,), dtype)
    y1 = DeviceArray.zeros((N * D * C,), dtype)
    xbar = DeviceArray.zeros((N * C,), dtype)
    xgrad = DeviceArray.zeros((N * C,), dtype)
    gp = DeviceArray.zeros((N * C,), dtype)
    ws = DeviceArray.zeros(((lib.opyx_rof_workspace_size() + 7) // 8,), np.float64)
    b = _lib.opyx_rof_buffers()
    b.x, b.xbar, b.y, b.f, b.ws = x1.ptr, xbar.ptr, y1.ptr, fd.ptr, ws.ptr
    if steps == "adaptive":
        b.xgrad, b.gp = xgrad.ptr, gp.ptr
    info_off = lib.opyx_rof_info_offset() // 8

    # allocation-free entry point (the caller still owns f, x, y and the gap output)
    x2 = DeviceArray.zeros((N * C,), dtype)
    y2 = DeviceArray.zeros((N * D * C,), dtype)
    gap2 = DeviceArray.zeros((6,), np.float64)

    tol = 1e-12 if dtype == np.float64 else 1e-5
    for call in range(2):
        s = stream_ptr()
        _lib.call("opyx_rof_init", p, b, s)
        _lib.call("opyx_rof_iterate", p, b, 25, s)
        _lib.call("opyx_rof_gap", p, b, s)
        _lib.call("opyx_rof_iterate_noalloc", p, x2.ptr, y2.ptr, fd.ptr, None, 25, gap2.ptr, s)
        torch().cuda.synchronize()
        xa, xb_ = x1.get(), x2.get()
        ya, yb = y1.get(), y2.get()
        assert np.linalg.norm(xb_ - xa) <= tol * np.linalg.norm(xa), (call, "x")
        assert np.linalg.norm(yb - ya) <= tol * max(1e-30, np.linalg.norm(ya)), (call, "y")
        g1 = ws[info_off:info_off + 6].get()
        g2 = gap2.get()
        assert np.all(np.abs(g2 - g1) <= tol * np.maximum(1.0, np.abs(g1))), (call, g1, g2)


def test_noalloc_rejects_problems_beyond_its_scratch():
    from opymize_gb300 import _lib
    lib = _lib.load()
    p = _problem(np.float32, "precond", (4096, 4096), 1, 0.0)   # 64 MiB of xbar
    st = lib.opyx_rof_iterate_noalloc(p, None, None, None, None, 1, None, None)
    assert st == 6
    assert "static scratch" in _lib.status_string(st)
