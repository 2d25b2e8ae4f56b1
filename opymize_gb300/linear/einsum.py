"""Per-pixel small matrix products (opymize/linear/einsum.py) on libopyx kernels."""

import numpy as np

from opymize_gb300 import Variable, LinOp, _lib
from opymize_gb300.gpuarray import DeviceArray, stream_ptr


def _lp(a, p, axis):
    a = np.abs(a)
    return a.sum(axis=axis) if p == 1 else (a ** p).sum(axis=axis) ** (1.0 / p)


class _SmallMatOp(LinOp):
    """Holds the (double) matrix on the device and the rowwise-norm pattern."""

    def _dev_A(self):
        if getattr(self, "_A_dev", None) is None:
            self._A_dev = DeviceArray.to_gpu(np.ascontiguousarray(self.A, dtype=np.float64))
        return self._A_dev

    def _check(self, x, y):
        if y is None:
            raise ValueError("this operator needs an output array y")
        if x.size != self.x.size or y.size != self.y.size:
            raise ValueError("size mismatch: x %d (want %d), y %d (want %d)"
                             % (x.size, self.x.size, y.size, self.y.size))
        if x.dtype != y.dtype:
            raise TypeError("x and y must share a dtype")

    def _rowlp_pattern(self, p):
        raise NotImplementedError

    def rowwise_lp(self, y, p=1, add=False):
        pat, outer, N, inner = self._rowlp_pattern(p)
        pdev = DeviceArray.to_gpu(np.ascontiguousarray(pat, dtype=np.float64).ravel())
        _lib.call("opyx_broadcast_mid", y.dcode, pdev.ptr, outer, N, inner, y.ptr,
                  int(bool(add)), stream_ptr())


class MatrixMult(_SmallMatOp):
    """y_ji = sum_k A_jk x_ki (opymize/linear/einsum.py:17-56); trans uses A^T.
    x is (K, N) with K the contracted side of A, so non-square A works too."""

    def __init__(self, N, A, trans=False, adjoint=None):
        LinOp.__init__(self)
        self.A, self.trans, self.N = np.asarray(A), trans, int(N)
        J, K = (self.A.shape[1], self.A.shape[0]) if trans else self.A.shape
        self.J, self.K = J, K
        self.x = Variable((K, self.N))
        self.y = Variable((J, self.N))
        self.adjoint = MatrixMult(N, A, trans=not trans, adjoint=self) if adjoint is None else adjoint

    def _call_gpu(self, x, y=None, add=False):
        self._check(x, y)
        _lib.call("opyx_matrixmult", x.dcode, self.N, self.J, self.K, self._dev_A().ptr,
                  int(self.trans), x.ptr, y.ptr, int(bool(add)), stream_ptr())

    def _rowlp_pattern(self, p):
        return _lp(self.A, p, 0 if self.trans else 1), self.J, self.N, 1


class MatrixOp(MatrixMult):
    """y_i = sum_j A_ij x_j (opymize/linear/einsum.py:99-102)."""

    def __init__(self, A):
        MatrixMult.__init__(self, 1, A)


class MatrixMultR(_SmallMatOp):
    """y_ij = sum_k x_ik A_kj (opymize/linear/einsum.py:58-97)."""

    def __init__(self, N, A, trans=False, adjoint=None):
        LinOp.__init__(self)
        self.A, self.trans, self.N = np.asarray(A), trans, int(N)
        K, J = (self.A.shape[1], self.A.shape[0]) if trans else self.A.shape
        self.J, self.K = J, K
        self.x = Variable((self.N, K))
        self.y = Variable((self.N, J))
        self.adjoint = MatrixMultR(N, A, trans=not trans, adjoint=self) if adjoint is None else adjoint

    def _call_gpu(self, x, y=None, add=False):
        self._check(x, y)
        _lib.call("opyx_matrixmultr", x.dcode, self.N, self.K, self.J, self._dev_A().ptr,
                  int(self.trans), x.ptr, y.ptr, int(bool(add)), stream_ptr())

    def _rowlp_pattern(self, p):
        return _lp(self.A, p, 1 if self.trans else 0), 1, self.N, self.J


class DiagMatrixMultR(_SmallMatOp):
    """y_ik = x_ik A_k (opymize/linear/einsum.py:104-128)."""

    def __init__(self, N, A):
        LinOp.__init__(self)
        self.A, self.N = np.asarray(A).ravel(), int(N)
        self.x = Variable((self.N, self.A.size))
        self.y = Variable((self.N, self.A.size))
        self.adjoint = self

    def _call_gpu(self, x, y=None, add=False):
        self._check(x, y)
        _lib.call("opyx_diag_matrixmultr", x.dcode, self.N, self.A.size, self._dev_A().ptr,
                  x.ptr, y.ptr, int(bool(add)), stream_ptr())

    def _rowlp_pattern(self, p):
        return np.abs(self.A), 1, self.N, self.A.size


class TangledMatrixMultR(_SmallMatOp):
    """y_mik = sum_jl x_jil A_jlmk (opymize/linear/einsum.py:130-173)."""

    def __init__(self, N, A, trans=False, adjoint=None):
        LinOp.__init__(self)
        self.A, self.trans, self.N = np.asarray(A), trans, int(N)
        J0, L0, M0, K0 = self.A.shape
        # kernel dims: contraction (J, L), output (M, K)
        self.kd = (M0, K0, J0, L0) if trans else (J0, L0, M0, K0)
        J, L, M, K = self.kd
        self.x = Variable((J, self.N, L))
        self.y = Variable((M, self.N, K))
        self.adjoint = TangledMatrixMultR(N, A, trans=not trans, adjoint=self) \
            if adjoint is None else adjoint

    def _call_gpu(self, x, y=None, add=False):
        self._check(x, y)
        J, L, M, K = self.kd
        _lib.call("opyx_tangled_matrixmultr", x.dcode, J, self.N, L, M, K, self._dev_A().ptr,
                  int(self.trans), x.ptr, y.ptr, int(bool(add)), stream_ptr())

    def _rowlp_pattern(self, p):
        J, L, M, K = self.kd
        pat = _lp(self.A, p, (2, 3)) if self.trans else _lp(self.A, p, (0, 1))
        return pat, M, self.N, K


class MatrixMultRBatched(_SmallMatOp):
    """y_jlk = sum_m x_jlm A_jmk (opymize/linear/einsum.py:175-214)."""

    def __init__(self, N, A, trans=False, adjoint=None):
        LinOp.__init__(self)
        self.A, self.trans, self.N = np.asarray(A), trans, int(N)
        J, M0, K0 = self.A.shape
        self.J = J
        self.M, self.K = (K0, M0) if trans else (M0, K0)   # contraction, output
        self.x = Variable((J, self.N, self.M))
        self.y = Variable((J, self.N, self.K))
        self.adjoint = MatrixMultRBatched(N, A, trans=not trans, adjoint=self) \
            if adjoint is None else adjoint

    def _call_gpu(self, x, y=None, add=False):
        self._check(x, y)
        _lib.call("opyx_matrixmultr_batched", x.dcode, self.J, self.N, self.M, self.K,
                  self._dev_A().ptr, int(self.trans), x.ptr, y.ptr, int(bool(add)), stream_ptr())

    def _rowlp_pattern(self, p):
        pat = _lp(self.A, p, 2) if self.trans else _lp(self.A, p, 1)
        return pat, self.J, self.N, self.K
