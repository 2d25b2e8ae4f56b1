"""Label gather / scatter operators (opymize/linear/indexed.py) on libopyx kernels."""

import numpy as np

from opymize_gb300 import Variable, LinOp, _lib
from opymize_gb300.gpuarray import DeviceArray, stream_ptr


def _lp_vals(v, p):
    v = np.abs(v)
    return v.sum(axis=-1) if p == 1 else (v ** p).sum(axis=-1) ** (1.0 / p)


class _IndexedBase(LinOp):
    def _setup(self, K, N, B, P):
        self.B = np.ascontiguousarray(B, dtype=np.float64)
        self.P = np.ascontiguousarray(P, dtype=np.int64)
        assert self.P.shape[0] == self.B.shape[0]
        assert self.P.shape[1] == self.B.shape[2]
        if self.P.size and (self.P.min() < 0 or self.P.max() >= K):
            raise ValueError("label indices P must lie in [0, %d)" % K)
        self.K, self.N = int(K), int(N)
        self.J, self.M, self.L = self.B.shape
        self._dev = None

    def _bufs(self):
        if self._dev is None:
            self._dev = (DeviceArray.to_gpu(self.B), DeviceArray.to_gpu(self.P))
        return self._dev

    def _check(self, x, y):
        if y is None:
            raise ValueError("this operator needs an output array y")
        if x.size != self.x.size or y.size != self.y.size or x.dtype != y.dtype:
            raise ValueError("size or dtype mismatch")

    def _merged(self):
        """Coefficients merged over equal labels: W[j, m, k] = sum_{l: P[j,l]=k} B[j,m,l]."""
        W = np.zeros((self.J, self.M, self.K))
        for j in range(self.J):
            for l in range(self.L):
                W[j, :, self.P[j, l]] += self.B[j, :, l]
        return W


class IndexedMult(_IndexedBase):
    """(Ax)[j,i,m] = -sum_l B[j,m,l] x[i,P[j,l]] (opymize/linear/indexed.py:63-94)."""

    def __init__(self, K, N, B, P, adjoint=None):
        LinOp.__init__(self)
        self._setup(K, N, B, P)
        self.x = Variable((self.N, self.K))
        self.y = Variable((self.J, self.N, self.M))
        self.adjoint = IndexedMultAdj(K, N, P, B, adjoint=self) if adjoint is None else adjoint

    def _call_gpu(self, x, y=None, add=False):
        self._check(x, y)
        Bd, Pd = self._bufs()
        _lib.call("opyx_indexedmult", x.dcode, self.J, self.N, self.M, self.L, self.K,
                  Bd.ptr, Pd.ptr, x.ptr, y.ptr, int(bool(add)), stream_ptr())

    def rowwise_lp(self, y, p=1, add=False):
        pat = _lp_vals(self._merged(), p)                       # (J, M)
        pdev = DeviceArray.to_gpu(np.ascontiguousarray(pat).ravel())
        _lib.call("opyx_broadcast_mid", y.dcode, pdev.ptr, self.J, self.N, self.M, y.ptr,
                  int(bool(add)), stream_ptr())


class IndexedMultAdj(_IndexedBase):
    """(Ax)[i,P[j,l]] -= sum_m B[j,m,l] x[j,i,m] (opymize/linear/indexed.py:34-61)."""

    def __init__(self, K, N, P, B, adjoint=None):
        LinOp.__init__(self)
        self._setup(K, N, B, P)
        self.x = Variable((self.J, self.N, self.M))
        self.y = Variable((self.N, self.K))
        self.adjoint = IndexedMult(K, N, B, P, adjoint=self) if adjoint is None else adjoint

    def _call_gpu(self, x, y=None, add=False):
        self._check(x, y)
        Bd, Pd = self._bufs()
        _lib.call("opyx_indexedmult_adj", x.dcode, self.J, self.N, self.M, self.L, self.K,
                  Bd.ptr, Pd.ptr, x.ptr, y.ptr, int(bool(add)), stream_ptr())

    def rowwise_lp(self, y, p=1, add=False):
        W = self._merged()                                      # (J, M, K)
        pat = _lp_vals(W.transpose(2, 0, 1).reshape(self.K, -1), p)  # (K,)
        pdev = DeviceArray.to_gpu(np.ascontiguousarray(pat))
        _lib.call("opyx_broadcast_mid", y.dcode, pdev.ptr, 1, self.N, self.K, y.ptr,
                  int(bool(add)), stream_ptr())
