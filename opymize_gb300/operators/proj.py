"""Projection operators (opymize/operators/proj.py) on libopyx kernels."""

import numpy as np

from opymize_gb300 import Variable, Operator, LinOp, _lib
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
        self._jacobian = L12ProjJacobian(self.N, self.M, self.lbd) \
            if matrixnorm == "frobenius" else None

    def _call_gpu(self, x, y=None, add=False, jacobian=False):
        assert not add
        assert self.matrixnorm == "frobenius" or not jacobian
        y = _inplace(x, y)
        if jacobian:
            # the projection and its Jacobian at x in one pass (proj.py:206-226)
            J = self._jacobian
            J._buffers(y.dtype)
            _lib.call("opyx_l1normsproj_jac", y.dcode, self.N, self.M[0] * self.M[1], self.lbd,
                      y.ptr, J.xn.ptr, J.s.ptr, stream_ptr())
            return J
        _lib.call("opyx_l1normsproj", y.dcode, self.N, self.M[0], self.M[1], self.lbd,
                  _lib.NORM[self.matrixnorm], y.ptr, stream_ptr())


class L12ProjJacobian(LinOp):
    """Jacobian of the projection onto the Frobenius lbd-balls at the point
    of the last L1NormsProj call with jacobian=True (opymize/operators/
    proj.py:228-276): the identity on groups inside the ball, lbd/|x|
    (v - <n, v> n) with n = x/|x| outside.  Symmetric.  The state (n and the
    scale per group) lives on the device and is written by the projection."""

    def __init__(self, N, M, lbd):
        LinOp.__init__(self)
        self.N, self.M = int(N), tuple(M)
        self.x = Variable((self.N, self.M[0] * self.M[1]))
        self.y = self.x
        self.lbd = float(lbd)
        self.adjoint = self
        self.xn = self.s = None

    def _buffers(self, dtype):
        if self.xn is None or self.xn.dtype != np.dtype(dtype):
            m = self.M[0] * self.M[1]
            self.xn = DeviceArray.zeros((self.N * m,), dtype)
            self.s = DeviceArray.empty((self.N,), dtype)
            self.s.fill(1.0)

    def _call_gpu(self, x, y=None, add=False):
        self._buffers(x.dtype)
        out = x if y is None else y
        if y is None and add:
            raise ValueError("in-place application with add is ambiguous")
        _lib.call("opyx_l12proj_jacobian", x.dcode, self.N, self.M[0] * self.M[1], self.xn.ptr,
                  self.s.ptr, x.ptr, out.ptr, int(bool(add)), stream_ptr())


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


def epigraph_Ab(I, J, v, b):
    """The constraint system of EpigraphProj as one block-diagonal CSR matrix
    and right-hand side (opymize/operators/proj.py:376-386): instance (j, i)
    contributes the rows (v[l], -1) <= b[i, l] for l in J[j] with I[i, l]."""
    import scipy.sparse as sp
    nfuns, npoints = I.shape
    blocks, rhs = [], []
    for j in range(J.shape[0]):
        for i in range(nfuns):
            ls = [int(l) for l in J[j] if I[i, l]]
            A = -np.ones((len(ls), v.shape[1] + 1))
            A[:, :-1] = v[ls]
            blocks.append(A)
            rhs.append(np.asarray(b[i, ls], dtype=np.float64))
    return sp.block_diag(blocks, format="csr"), np.concatenate(rhs)


class _EpigraphData(object):
    """Device copies of (I, J, v, b) and the opyx_epigraph descriptor."""

    def __init__(self, I, J, v, b):
        I, J = np.asarray(I), np.asarray(J)
        v, b = np.asarray(v, dtype=np.float64), np.asarray(b, dtype=np.float64)
        assert I.shape == b.shape and I.shape[1] == v.shape[0]
        assert J.ndim == 2 and v.ndim == 2
        if J.size and (J.min() < 0 or J.max() >= I.shape[1]):
            raise ValueError("J holds indices outside [0, npoints)")
        if not 1 <= v.shape[1] <= 3:
            raise NotImplementedError("epigraph projections support ndim 1..3")
        self.I, self.J, self.v, self.b = I, J, v, b
        self.nfuns, self.npoints = I.shape
        self.nregions, self.nsubpoints = J.shape
        self.ndim = v.shape[1]
        self._dev = {}
        self._ij = None

    def struct(self, dtype, supp=None):
        # ndim 1 projections read transposed copies of I and b (instances of
        # one region with consecutive functions read consecutive values)
        tr = self.ndim == 1
        if self._ij is None:
            self._ij = (DeviceArray.to_gpu(np.ascontiguousarray(self.I, dtype=np.uint8)),
                        DeviceArray.to_gpu(np.ascontiguousarray(self.J, dtype=np.int64)),
                        DeviceArray.to_gpu(np.ascontiguousarray(self.I.T, dtype=np.uint8))
                        if tr else None)
        key = np.dtype(dtype).str
        if key not in self._dev:
            self._dev[key] = (DeviceArray.to_gpu(np.ascontiguousarray(self.v), dtype),
                              DeviceArray.to_gpu(np.ascontiguousarray(self.b), dtype),
                              DeviceArray.to_gpu(np.ascontiguousarray(self.b.T), dtype)
                              if tr else None)
        e = _lib.opyx_epigraph()
        e.ndim, e.nsubpoints = self.ndim, self.nsubpoints
        e.nfuns, e.nregions, e.npoints = self.nfuns, self.nregions, self.npoints
        e.I, e.J = self._ij[0].ptr, self._ij[1].ptr
        e.v, e.b = self._dev[key][0].ptr, self._dev[key][1].ptr
        if tr:
            e.It, e.bt = self._ij[2].ptr, self._dev[key][2].ptr
        if supp is not None:
            e.eq_off, e.eqns, e.checks = (None if a is None else a.ptr for a in supp)
        return e


class EpigraphProj(Operator):
    """T(x)[j,i] = projection of x[j,i] onto the epigraph of the conjugate
    of the convex piece j of the piecewise-linear function i, i.e. onto
    {y : <v[k], y[:-1]> - y[-1] <= b[i,k] for k in J[j] with I[i,k]}
    (opymize/operators/proj.py:388-480).

    Every instance is solved by one thread with an active-set QP (the
    reference's GPU method, proj.cu:660-790); the iteration bound and the
    tolerance are the reference's (ndim*nsubpoints, 1e-9).  Instances that
    hit the bound keep their last iterate and are counted in
    ``nonconverged`` (the reference prints a warning).  For ndim 1 with at
    most 16 points per region the same projection is computed directly: the
    nearest of the epigraph boundary's line pieces, no iterations."""

    def __init__(self, I, J, v, b, Ab=None):
        Operator.__init__(self)
        self.data = _EpigraphData(I, J, v, b)
        d = self.data
        self.I, self.J, self.v, self.b = d.I, d.J, d.v, d.b
        self._Ab = Ab
        self.x = Variable((d.nregions, d.nfuns, d.ndim + 1))
        self.y = self.x
        self.maxiter = d.ndim * d.nsubpoints
        self.tol = 1e-9
        self._count = None

    @property
    def Ab(self):
        if self._Ab is None:
            self._Ab = epigraph_Ab(self.I, self.J, self.v, self.b)
        return self._Ab

    @property
    def nonconverged(self):
        """Instances that hit the iteration bound, over all calls so far."""
        return 0 if self._count is None else int(self._count.t.item())

    def _call_gpu(self, x, y=None, add=False, jacobian=False):
        assert not add
        assert not jacobian
        assert x.size == self.x.size, "x must hold (nregions, nfuns, ndim+1) values"
        out = x if y is None else y
        assert out.size == x.size and out.dtype == x.dtype
        if self._count is None:
            from opymize_gb300.gpuarray import torch
            self._count = DeviceArray(torch().zeros(1, dtype=torch().int32, device="cuda"))
        _lib.call("opyx_epigraph_proj", self.data.struct(x.dtype), x.dcode, x.ptr, out.ptr,
                  int(self.maxiter), float(self.tol), self._count.ptr, stream_ptr())
