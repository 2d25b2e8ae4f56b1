"""Finite-difference operators (opymize/linear/diff.py) on libopyx kernels."""

import numpy as np

from opymize_gb300 import Variable, LinOp, _lib
from opymize_gb300.gpuarray import DeviceArray, stream_ptr


def make_grid(imagedims, nchannels, imageh):
    g = _lib.opyx_grid()
    D = len(imagedims)
    if D > _lib.MAX_DIMS:
        raise ValueError("at most %d image dimensions are supported" % _lib.MAX_DIMS)
    g.ndim, g.nchannels = D, int(nchannels)
    for t in range(D):
        g.dims[t] = int(imagedims[t])
        g.h[t] = float(imageh[t])
    return g


def _check_pair(x, y, nx, ny):
    if y is None:
        raise ValueError("this operator needs an output array y")
    if x.size != nx or y.size != ny:
        raise ValueError("size mismatch: x %d (want %d), y %d (want %d)" % (x.size, nx, y.size, ny))
    if x.dtype != y.dtype:
        raise TypeError("x and y must share a dtype")


class _DiffBase(LinOp):
    def _setup(self, imagedims, nchannels, imageh, weights):
        self.imagedims = tuple(int(d) for d in imagedims)
        self.nchannels = int(nchannels)
        ndims = len(self.imagedims)
        self.imageh = np.ones(ndims) if imageh is None else np.asarray(imageh, dtype=np.float64)
        self.weights = np.ones(nchannels) if weights is None else np.asarray(weights, dtype=np.float64)
        self._grid = make_grid(self.imagedims, self.nchannels, self.imageh)
        self._w_dev = None

    def _wptr(self):
        if np.all(self.weights == 1.0):
            return None
        if self._w_dev is None:
            self._w_dev = DeviceArray.to_gpu(self.weights, np.float64)
        return self._w_dev.ptr


class GradientOp(_DiffBase):
    """y[i,t,k] = w_k D_t x[i,k] on a cartesian grid, scheme "centered"
    (default) or "forward", Neumann boundary (opymize/linear/diff.py:67-144)."""

    def __init__(self, imagedims, nchannels, scheme="centered", imageh=None, weights=None,
                 adjoint=None):
        LinOp.__init__(self)
        if scheme not in _lib.SCHEME:
            raise ValueError("unsupported scheme: %s" % scheme)
        self._setup(imagedims, nchannels, imageh, weights)
        self.scheme = scheme
        npoints = int(np.prod(self.imagedims))
        ndims = len(self.imagedims)
        self.x = Variable((npoints, self.nchannels))
        self.y = Variable((npoints, ndims, self.nchannels))
        self.adjoint = DivergenceOp(imagedims, nchannels, imageh=self.imageh,
                                    weights=self.weights, adjoint=self, scheme=scheme) \
            if adjoint is None else adjoint

    def prepare_gpu(self, kernels=None, type_t="double"):
        pass

    def _call_gpu(self, x, y=None, add=False):
        _check_pair(x, y, self.x.size, self.y.size)
        _lib.call("opyx_gradient", self._grid, _lib.SCHEME[self.scheme], self._wptr(),
                  x.dcode, x.ptr, y.ptr, int(bool(add)), stream_ptr())

    def rowwise_lp(self, y, p=1, add=False):
        _lib.call("opyx_gradient_rowlp", self._grid, _lib.SCHEME[self.scheme], self._wptr(),
                  0, float(p), y.dcode, y.ptr, int(bool(add)), stream_ptr())


class DivergenceOp(_DiffBase):
    """Negative divergence, the adjoint of GradientOp
    (opymize/linear/diff.py:146-183)."""

    def __init__(self, imagedims, nchannels, imageh=None, weights=None, adjoint=None,
                 scheme="centered"):
        LinOp.__init__(self)
        self._setup(imagedims, nchannels, imageh, weights)
        npoints = int(np.prod(self.imagedims))
        ndims = len(self.imagedims)
        self.x = Variable((npoints, ndims, self.nchannels))
        self.y = Variable((npoints, self.nchannels))
        if adjoint is None:
            adjoint = GradientOp(imagedims, nchannels, scheme=scheme, imageh=self.imageh,
                                 weights=self.weights, adjoint=self)
        self.adjoint = adjoint
        self.scheme = adjoint.scheme

    def prepare_gpu(self, kernels=None, type_t="double"):
        pass

    def _call_gpu(self, x, y=None, add=False):
        _check_pair(x, y, self.x.size, self.y.size)
        _lib.call("opyx_divergence", self._grid, _lib.SCHEME[self.scheme], self._wptr(),
                  x.dcode, x.ptr, y.ptr, int(bool(add)), stream_ptr())

    def rowwise_lp(self, y, p=1, add=False):
        _lib.call("opyx_gradient_rowlp", self._grid, _lib.SCHEME[self.scheme], self._wptr(),
                  1, float(p), y.dcode, y.ptr, int(bool(add)), stream_ptr())


class LaplacianOp(LinOp):
    """Laplacian with "neumann", "curvature(_adj)" or "second-order(_adj)"
    boundary (opymize/linear/diff.py:185-249)."""

    supported_bc = ["curvature", "curvature_adj", "second-order", "second-order_adj",
                    "neumann"]

    def __init__(self, imagedims, nchannels, imageh=None, boundary="neumann", adjoint=None):
        LinOp.__init__(self)
        if boundary not in self.supported_bc:
            raise Exception("Unknown boundary conditions: %s" % boundary)
        self.imagedims = tuple(int(d) for d in imagedims)
        ndims = len(self.imagedims)
        self.imageh = np.ones(ndims) if imageh is None else np.asarray(imageh, dtype=np.float64)
        self.bc = boundary
        self.nchannels = int(nchannels)
        npoints = int(np.prod(self.imagedims))
        self.x = Variable((npoints, self.nchannels))
        self.y = Variable((npoints, self.nchannels))
        self._grid = make_grid(self.imagedims, self.nchannels, self.imageh)
        self._is_adj = boundary.endswith("_adj")
        self._base = boundary[:-4] if self._is_adj else boundary
        if boundary == "neumann":
            self.adjoint = self
        elif adjoint is None:
            adj_bc = self._base if self._is_adj else boundary + "_adj"
            self.adjoint = LaplacianOp(imagedims, nchannels, imageh=self.imageh,
                                       boundary=adj_bc, adjoint=self)
        else:
            self.adjoint = adjoint

    def _call_gpu(self, x, y=None, add=False):
        _check_pair(x, y, self.x.size, self.y.size)
        _lib.call("opyx_laplacian", self._grid, _lib.BC[self._base], int(self._is_adj),
                  x.dcode, x.ptr, y.ptr, int(bool(add)), stream_ptr())

    def rowwise_lp(self, y, p=1, add=False):
        _lib.call("opyx_laplacian_rowlp", self._grid, _lib.BC[self._base], int(self._is_adj),
                  float(p), y.dcode, y.ptr, int(bool(add)), stream_ptr())
