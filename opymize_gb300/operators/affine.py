"""Affine prox operators (opymize/operators/affine.py) on libopyx kernels."""

import numpy as np

from opymize_gb300 import Variable, Operator, _lib
from opymize_gb300.gpuarray import DeviceArray, stream_ptr
from opymize_gb300.steps import step_struct


def _dev_cache(owner, name, host, dtype):
    """Device copy of a host array in `dtype`, cached on `owner`."""
    cache = owner.__dict__.setdefault("_devcache", {})
    key = (name, np.dtype(dtype).str)
    if key not in cache:
        cache[key] = DeviceArray.to_gpu(host, dtype)   # float casts run on the device
    return cache[key]


class ConstOp(Operator):
    """T(x) = const (opymize/operators/affine.py:15-44)."""

    def __init__(self, N, const):
        Operator.__init__(self)
        self.x = Variable(N)
        self.y = Variable(const.size)
        self.const = np.asarray(const)

    def _call_gpu(self, x, y=None, add=False, jacobian=False):
        y = x if y is None else y
        c = _dev_cache(self, "const", self.const.ravel(), x.dtype)
        if add:
            y.axpy(1.0, c)
        else:
            y.assign(c)
        if jacobian:
            from opymize_gb300.linear.scale import ZeroOp
            return ZeroOp(self.x.size, self.y.size)


class ConstrainOp(Operator):
    """y[mask,:] = const[mask,:], identity elsewhere (opymize/operators/affine.py:46-83)."""

    def __init__(self, mask, const):
        Operator.__init__(self)
        self.x = Variable(const.shape)
        self.y = self.x
        self.mask = np.asarray(mask, dtype=bool)
        self.const = np.asarray(const)

    def _call_gpu(self, x, y=None, add=False, jacobian=False):
        y = x if y is None else y
        N, M = self.const.shape
        c = _dev_cache(self, "const", self.const, x.dtype)
        m = _dev_cache(self, "mask", self.mask.astype(np.uint8), np.uint8)
        _lib.call("opyx_constrain", x.dcode, N, M, m.ptr, c.ptr, x.ptr, y.ptr, int(bool(add)),
                  stream_ptr())
        if jacobian:
            from opymize_gb300.linear.scale import ScaleOp
            scale = np.ones_like(self.const, dtype=np.float64)
            scale[self.mask, :] = 0.0
            return ScaleOp(self.x.size, scale.ravel())


class ShiftScaleOp(Operator):
    """T(x) = a*(x + b*shift), each of a, b, shift a scalar or an array
    (opymize/operators/affine.py:85-146)."""

    def __init__(self, N, shift, a, b):
        Operator.__init__(self)
        self.shift, self.a, self.b = shift, a, b
        self.x = Variable(N)
        self.y = Variable(N)

    def _arg(self, name, v, dtype):
        if isinstance(v, DeviceArray):
            return v.ptr, 0.0
        if isinstance(v, np.ndarray) and v.size > 1:
            return _dev_cache(self, name + str(id(v)), v.ravel(), dtype).ptr, 0.0
        return None, float(np.asarray(v).ravel()[0]) if isinstance(v, np.ndarray) else float(v)

    def _call_gpu(self, x, y=None, add=False, jacobian=False):
        y = x if y is None else y
        ap, av = self._arg("a", self.a, x.dtype)
        bp, bv = self._arg("b", self.b, x.dtype)
        sp_, sv = self._arg("shift", self.shift, x.dtype)
        _lib.call("opyx_shiftscale", x.dcode, x.size, ap, av, bp, bv, sp_, sv, x.ptr, y.ptr,
                  int(bool(add)), stream_ptr())
        if jacobian:
            from opymize_gb300.linear.scale import ScaleOp
            return ScaleOp(self.x.size, self.a)


class AffineProxOp(Operator):
    """T(x) = a*(x - tau*c): the prox of tau*(b + <c, x>), masked by a
    (AffineFct / MaskedAffineFct.prox, opymize/functionals/affine.py:38-42,
    :86-90).  ``tau`` is a scalar, a per-element DeviceArray or a
    DeviceScalar (adaptive steps), read by the kernel at launch."""

    def __init__(self, N, a, c, tau):
        Operator.__init__(self)
        self.a, self.c, self.tau = a, c, tau
        self.x = Variable(N)
        self.y = Variable(N)

    def _arg(self, name, v, dtype):
        if isinstance(v, np.ndarray) and v.size > 1:
            return _dev_cache(self, name, v.ravel(), dtype).ptr, 0.0
        return None, float(np.asarray(v).ravel()[0]) if isinstance(v, np.ndarray) else float(v)

    def _call_gpu(self, x, y=None, add=False, jacobian=False):
        assert not add
        y = x if y is None else y
        ap, av = self._arg("a", self.a, x.dtype)
        cp, cv = self._arg("c", self.c, x.dtype)
        _lib.call("opyx_affine_prox", x.dcode, x.size, ap, av, cp, cv,
                  step_struct(self.tau, x.dtype), x.ptr, y.ptr, stream_ptr())
        if jacobian:
            from opymize_gb300.linear.scale import ScaleOp
            return ScaleOp(self.x.size, self.a)


class SSDProxOp(Operator):
    """prox of tau*SSD: x <- (x + t*f)/(1 + t), t = tau*vol on masked pixels
    (opymize/functionals/quad.py:45-55 builds the same map as a ShiftScaleOp
    with host-computed arrays a, b).  ``tau`` is a scalar, a per-element
    DeviceArray or a DeviceScalar, read by the kernel at launch."""

    def __init__(self, ssd, tau):
        Operator.__init__(self)
        self.ssd = ssd
        self.tau = tau
        self.x = Variable(ssd.x.size)
        self.y = self.x

    def _call_gpu(self, x, y=None, add=False, jacobian=False):
        assert not add
        y = x if y is None else y
        N, C = self.ssd.f.shape
        f = self.ssd.f_dev(x.dtype)
        vol = self.ssd.vol_dev()
        mask = self.ssd.mask_dev()
        _lib.call("opyx_ssd_prox", x.dcode, N, C, f.ptr, vol.ptr, None if mask is None else mask.ptr,
                  step_struct(self.tau, x.dtype), x.ptr, y.ptr, stream_ptr())
        if jacobian:
            # the map is a*(x + b*f) with a = 1/(1 + tau*vol) on masked pixels and
            # 1 elsewhere (quad.py:45-55); its Jacobian is the ScaleOp diag(a)
            return self._jacobian_op()

    def _jacobian_op(self):
        from opymize_gb300.linear.scale import ScaleOp
        if getattr(self, "_jac", None) is None:
            if not np.isscalar(self.tau):
                raise NotImplementedError("the Jacobian needs a scalar step")
            N, C = self.ssd.f.shape
            tv = np.zeros((N, C))
            msk = np.ones(N, dtype=bool) if self.ssd.mask is None else np.asarray(self.ssd.mask, bool)
            tv[msk, :] = float(self.tau) * np.asarray(self.ssd.vol, dtype=np.float64)
            self._jac = ScaleOp(N * C, 1.0 / (1.0 + tv.ravel()))
        return self._jac
