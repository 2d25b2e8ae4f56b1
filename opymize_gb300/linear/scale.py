"""Trivial linear operators (opymize/linear/scale.py) on libopyx kernels."""

import numpy as np

from opymize_gb300 import Variable, LinOp, _lib
from opymize_gb300.gpuarray import DeviceArray, stream_ptr


class ZeroOp(LinOp):
    """(Ax)_i = 0 (opymize/linear/scale.py:14-31)."""

    def __init__(self, M, N=None, adjoint=None):
        LinOp.__init__(self)
        N = M if N is None else N
        self.x = Variable(N)
        self.y = Variable(M)
        self.adjoint = ZeroOp(N, M, adjoint=self) if adjoint is None else adjoint

    def _call_gpu(self, x, y=None, add=False):
        if not add:
            (x if y is None else y).fill(0.0)

    def rowwise_lp(self, y, p=1, add=False):
        if not add:
            y.fill(0.0)


class ScaleOp(LinOp):
    """(Ax)_i = fact*x_i, fact a scalar or an array (opymize/linear/scale.py:33-73)."""

    def __init__(self, N, fact):
        LinOp.__init__(self)
        self.x = Variable(N)
        self.y = Variable(N)
        self.adjoint = self
        self.fact = fact
        self._fact_dev = {}

    def _fvec(self, dtype):
        key = np.dtype(dtype).str
        if key not in self._fact_dev:
            self._fact_dev[key] = DeviceArray.to_gpu(np.ascontiguousarray(
                np.broadcast_to(np.asarray(self.fact, dtype=np.float64), (self.x.size,))), dtype)
        return self._fact_dev[key]

    def _call_gpu(self, x, y=None, add=False):
        y = x if y is None else y
        if np.isscalar(self.fact):
            _lib.call("opyx_axpby", x.dcode, x.size, float(self.fact), x.ptr,
                      1.0 if add else 0.0, y.ptr, stream_ptr())
        else:
            f = self._fvec(x.dtype)
            _lib.call("opyx_shiftscale", x.dcode, x.size, f.ptr, 0.0, None, 0.0, None, 0.0,
                      x.ptr, y.ptr, int(bool(add)), stream_ptr())

    def rowwise_lp(self, y, p=1, add=False):
        v = np.broadcast_to(np.abs(np.asarray(self.fact, dtype=np.float64)) ** p, (y.size,))
        tmp = DeviceArray.to_gpu(v, y.dtype)
        if add:
            y.axpy(1.0, tmp)
        else:
            y.assign(tmp)


class IdentityOp(LinOp):
    """(Ax)_i = x_i (opymize/linear/scale.py:75-94)."""

    def __init__(self, N):
        LinOp.__init__(self)
        self.x = Variable(N)
        self.y = Variable(N)
        self.adjoint = self

    def _call_gpu(self, x, y=None, add=False):
        if y is None and not add:
            return
        y = x if y is None else y
        if add:
            y.axpy(1.0, x)
        else:
            y.assign(x)

    def rowwise_lp(self, y, p=1, add=False):
        if add:
            y += 1.0
        else:
            y.fill(1.0)


class NihilOp(LinOp):
    """(Ax)_i = x_i if keep_i else 0 (opymize/linear/scale.py:96-115)."""

    def __init__(self, N, keep):
        LinOp.__init__(self)
        self.x = Variable(N)
        self.y = Variable(N)
        self.adjoint = self
        self.keep = np.asarray(keep).astype(bool)

    def _call_gpu(self, x, y=None, add=False):
        y = x if y is None else y
        k = DeviceArray.to_gpu(self.keep.astype(np.float64), x.dtype)
        _lib.call("opyx_shiftscale", x.dcode, x.size, k.ptr, 0.0, None, 0.0, None, 0.0,
                  x.ptr, y.ptr, int(bool(add)), stream_ptr())

    def rowwise_lp(self, y, p=1, add=False):
        k = DeviceArray.to_gpu(self.keep.astype(np.float64), y.dtype)
        if add:
            y.axpy(1.0, k)
        else:
            y.assign(k)
