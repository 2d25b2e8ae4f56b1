"""Projection operators (opymize/operators/proj.py) on libopyx kernels."""

import numpy as np

from opymize_gb300 import Variable, Operator, _lib
from opymize_gb300.gpuarray import DeviceArray, stream_ptr
from opymize_gb300.steps import step_struct


def _inplace(x, y):
    """The projections work in place: copy x to y first when y is given."""
    if y is None:
        return x
    if y.ptr != x.ptr:
        y.assign(x)
    return y


class PosProj(Operator):
    """T(x) = max(0, x) (opymize/operators/proj.py:19-50)."""

    def __init__(self, N):
        Operator.__init__(self)
        self.x = Variable(N)
        self.y = Variable(N)

    def _call_gpu(self, x, y=None, add=False, jacobian=False):
        y = x if y is None else y
        _lib.call("opyx_posproj", x.dcode, x.size, x.ptr, y.ptr, int(bool(add)), stream_ptr())
        if jacobian:
            from opymize_gb300.linear.scale import NihilOp
            return NihilOp(self.x.size, x.get() > 0)


class NegProj(Operator):
    """T(x) = min(0, x) (opymize/operators/proj.py:52-85)."""

    def __init__(self, N):
        Operator.__init__(self)
        self.x = Variable(N)
        self.y = Variable(N)

    def _call_gpu(self, x, y=None, add=False, jacobian=False):
        y = x if y is None else y
        _lib.call("opyx_negproj", x.dcode, x.size, x.ptr, y.ptr, int(bool(add)), stream_ptr())
        if jacobian:
            from opymize_gb300.linear.scale import NihilOp
            return NihilOp(self.x.size, x.get() < 0)


class L1NormsProj(Operator):
    """x_i <- proj onto {|x_i| <= lbd}, Frobenius or spectral norm
    (opymize/operators/proj.py:170-226).  For the spectral norm the per-group
    buffer is read in the (M[1], M[0]) order of the reference's GPU kernel
    (operators/proj.cu:11-21), i.e. the (D, C) layout of GradientOp output."""

    def __init__(self, N, M, lbd, matrixnorm):
        Operator.__init__(self)
        assert matrixnorm in ['frobenius', 'spectral']
        self.M, self.N = tuple(M), int(N)
        self.x = Variable((self.N,) + self.M)
        self.y = self.x
        self.lbd = float(lbd)
        self.matrixnorm = matrixnorm

    def _call_gpu(self, x, y=None, add=False, jacobian=False):
        assert not add and not jacobian
        y = _inplace(x, y)
        _lib.call("opyx_l1normsproj", y.dcode, self.N, self.M[0], self.M[1], self.lbd,
                  _lib.NORM[self.matrixnorm], y.ptr, stream_ptr())


class HuberConjProj(Operator):
    """prox of sigma*F* for F = lbd*sum_i huber_alph(|x_i|_F):
    x_i <- proj_{|.|_F <= lbd}(x_i / (1 + sigma*alph/lbd)); ``sigma`` is a
    scalar, a per-element DeviceArray or a DeviceScalar."""

    def __init__(self, N, M, lbd, alph, sigma):
        Operator.__init__(self)
        self.M, self.N = tuple(M), int(N)
        self.x = Variable((self.N,) + self.M)
        self.y = self.x
        self.lbd, self.alph, self.sigma = float(lbd), float(alph), sigma

    def _call_gpu(self, x, y=None, add=False, jacobian=False):
        assert not add and not jacobian
        y = _inplace(x, y)
        _lib.call("opyx_huber_conj_prox", y.dcode, self.N, self.M[0] * self.M[1], self.lbd,
                  self.alph, step_struct(self.sigma, y.dtype), y.ptr, stream_ptr())


class QuadEpiProj(Operator):
    """T(z)[i] = projection of z[i] onto epi(f_i), f_i(x) = 0.5*alph*|x - s1_i|^2
    + s2_i (or from b, c), optionally truncated at |x - s1_i| <= lbd
    (opymize/operators/proj.py:278-374).  The cubic root-solve runs in FP64."""

    def __init__(self, N, M, alph=1.0, shift=None, b=None, c=None, lbd=np.inf):
        Operator.__init__(self)
        assert lbd > 0
        assert alph > 0
        self.N, self.M = int(N), int(M)
        self.x = Variable((self.N, self.M + 1))
        self.y = self.x
        self.lbd, self.alph, self.shift = float(lbd), float(alph), shift
        if not (b is None and c is None):
            assert self.shift is None
            self.b = np.zeros((N, M)) if b is None else b
            self.c = np.zeros((N,)) if c is None else c
            self.shift = np.zeros((N, M + 1))
            self.shift[:, :-1] = -self.b / self.alph
            self.shift[:, -1] = -(0.5 / self.alph * (self.b ** 2).sum(axis=-1) - self.c)
        self._shift_dev = {}

    def _sptr(self, dtype):
        if self.shift is None:
            return None
        key = np.dtype(dtype).str
        if key not in self._shift_dev:
            self._shift_dev[key] = DeviceArray.to_gpu(np.ascontiguousarray(self.shift).ravel(), dtype)
        return self._shift_dev[key].ptr

    def _call_gpu(self, x, y=None, add=False, jacobian=False):
        assert not add and not jacobian
        y = _inplace(x, y)
        _lib.call("opyx_quadepiproj", y.dcode, self.N, self.M, self.alph, self._sptr(y.dtype),
                  self.lbd, y.ptr, stream_ptr())
