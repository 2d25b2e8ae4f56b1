"""Device arrays: the subset of ``pycuda.gpuarray.GPUArray`` the reference's
PDHG path touches (``to_gpu``, ``get``, ``fill``, ``copy``, slicing,
``reshape``, ``y[:] = x``, ``y += x``, ``y *= a``; opymize/solvers/pdhg.py:81-91,
opymize/linear/__init__.py:99-105, opymize/operators/*), on GB300 memory.

Storage and streams come from PyTorch (a CUDA tensor underneath, allocated by
its caching allocator on the current device); every arithmetic operation is a
libopyx kernel launched on the current stream.
"""

import numpy as np

from opymize_gb300 import _lib

_torch = None


def torch():
    global _torch
    if _torch is None:
        import torch as t
        if not t.cuda.is_available():
            raise _lib.OpyxLibraryError("no CUDA device: opymize_gb300 runs on the GPU only")
        _torch = t
    return _torch


_NP2T = {np.dtype(np.float32): "float32", np.dtype(np.float64): "float64",
         np.dtype(np.uint8): "uint8", np.dtype(np.bool_): "uint8",
         np.dtype(np.int64): "int64", np.dtype(np.int32): "int32"}


def _tdtype(dtype):
    return getattr(torch(), _NP2T[np.dtype(dtype)])


def stream_ptr():
    """Raw cudaStream_t of torch's current stream."""
    return torch().cuda.current_stream().cuda_stream


def dtype_code(dtype):
    dt = np.dtype(dtype)
    if dt == np.float32:
        return _lib.OPYX_F32
    if dt == np.float64:
        return _lib.OPYX_F64
    raise TypeError("unsupported iterate dtype %s (float32 or float64)" % dt)


class DeviceArray(object):
    """A contiguous array in device memory (torch tensor underneath)."""

    __array_priority__ = 100

    def __init__(self, tensor, dtype=None):
        self.t = tensor
        self._dtype = np.dtype(dtype) if dtype is not None else \
            np.dtype(str(tensor.dtype).replace("torch.", ""))

    # --- construction
    @classmethod
    def empty(cls, shape, dtype=np.float64):
        shape = (shape,) if np.isscalar(shape) else tuple(int(s) for s in shape)
        return cls(torch().empty(shape, dtype=_tdtype(dtype), device="cuda"), dtype)

    @classmethod
    def zeros(cls, shape, dtype=np.float64):
        a = cls.empty(shape, dtype)
        if a.size:
            a.fill(0)
        return a

    @classmethod
    def to_gpu(cls, ary, dtype=None):
        ary = np.asarray(ary)
        want = np.dtype(dtype) if dtype is not None else ary.dtype
        floats = (np.dtype(np.float32), np.dtype(np.float64))
        if ary.dtype != want and ary.dtype in floats and want in floats:
            # upload in the host precision, convert on the device
            src = cls.to_gpu(ary)
            out = cls.empty(ary.shape, want)
            if src.size:
                _lib.call("opyx_cast", dtype_code(ary.dtype), dtype_code(want), src.size,
                          src.ptr, out.ptr, stream_ptr())
            return out
        ary = np.ascontiguousarray(ary, dtype=want)
        if not ary.flags.writeable:     # torch.from_numpy wants a writable buffer
            ary = ary.copy()
        src = ary.view(np.uint8) if ary.dtype == np.bool_ else ary
        t = torch().from_numpy(src).to("cuda", non_blocking=False)
        return cls(t, np.uint8 if ary.dtype == np.bool_ else ary.dtype)

    # --- attributes
    @property
    def shape(self):
        return tuple(self.t.shape)

    @property
    def dtype(self):
        return self._dtype

    @property
    def size(self):
        return int(self.t.numel())

    @property
    def nbytes(self):
        return self.size * self._dtype.itemsize

    @property
    def ptr(self):
        return self.t.data_ptr()

    gpudata = ptr

    @property
    def dcode(self):
        return dtype_code(self._dtype)

    def __len__(self):
        return self.shape[0]

    def __repr__(self):
        return "DeviceArray(shape=%s, dtype=%s)" % (self.shape, self._dtype)

    # --- host transfers
    def get(self, ary=None):
        """Copy to the host (through page-locked memory from torch's
        caching host allocator); synchronises."""
        t = torch()
        h = t.empty(tuple(self.t.shape), dtype=self.t.dtype, pin_memory=True)
        h.copy_(self.t)
        h = h.numpy()
        if ary is None:
            return h
        ary[...] = h.reshape(ary.shape)
        return ary

    def set(self, ary):
        ary = np.ascontiguousarray(ary, dtype=self._dtype).reshape(self.shape)
        self.t.copy_(torch().from_numpy(ary))

    # --- views
    def reshape(self, *shape):
        if len(shape) == 1 and not np.isscalar(shape[0]):
            shape = tuple(shape[0])
        return DeviceArray(self.t.view(*shape), self._dtype)

    def ravel(self):
        return DeviceArray(self.t.view(-1), self._dtype)

    def __getitem__(self, idx):
        v = self.t[idx]
        if not v.is_contiguous():
            raise ValueError("only contiguous views of a DeviceArray are supported")
        return DeviceArray(v, self._dtype)

    # --- kernels
    def fill(self, value):
        if self.size:
            _lib.call("opyx_fill", self.dcode, self.ptr, self.size, float(value), stream_ptr())
        return self

    def copy(self):
        out = DeviceArray.empty(self.shape, self._dtype)
        out.assign(self)
        return out

    def assign(self, other, scale=1.0):
        """self[:] = scale*other (other a DeviceArray of the same size)."""
        if other.size != self.size:
            raise ValueError("size mismatch: %d vs %d" % (other.size, self.size))
        if self.size:
            _lib.call("opyx_axpby", self.dcode, self.size, float(scale), other.ptr, 0.0,
                      self.ptr, stream_ptr())
        return self

    def axpy(self, a, other):
        """self += a*other."""
        if other.size != self.size:
            raise ValueError("size mismatch: %d vs %d" % (other.size, self.size))
        if self.size:
            _lib.call("opyx_axpby", self.dcode, self.size, float(a), other.ptr, 1.0,
                      self.ptr, stream_ptr())
        return self

    def __setitem__(self, idx, value):
        view = self if (isinstance(idx, slice) and idx == slice(None)) else self[idx]
        if isinstance(value, DeviceArray):
            view.assign(value)
        elif np.isscalar(value):
            view.fill(value)
        else:
            view.set(np.asarray(value))

    def __iadd__(self, other):
        if isinstance(other, DeviceArray):
            return self.axpy(1.0, other)
        if np.isscalar(other):
            tmp = DeviceArray.empty(self.shape, self._dtype).fill(other)
            return self.axpy(1.0, tmp)
        return self.axpy(1.0, DeviceArray.to_gpu(np.asarray(other), self._dtype))

    def __imul__(self, a):
        if not np.isscalar(a):
            raise TypeError("DeviceArray *= supports scalars only")
        if self.size:
            _lib.call("opyx_axpby", self.dcode, self.size, float(a), self.ptr, 0.0,
                      self.ptr, stream_ptr())
        return self


_copy_streams = {}   # device index -> streams of get_all


def get_all(arrays):
    """Host copies of several device arrays (as DeviceArray.get), each
    transfer on its own stream after the work queued so far, so that they
    run on separate copy engines at once; synchronises."""
    t = torch()
    cur = t.cuda.current_stream()
    streams = _copy_streams.setdefault(t.cuda.current_device(), [])
    while len(streams) < len(arrays):
        streams.append(t.cuda.Stream())
    outs = []
    for a, st in zip(arrays, streams):
        h = t.empty(tuple(a.t.shape), dtype=a.t.dtype, pin_memory=True)
        st.wait_stream(cur)
        with t.cuda.stream(st):
            h.copy_(a.t, non_blocking=True)
        outs.append(h)
    for st in streams[:len(arrays)]:
        st.synchronize()
    return [h.numpy() for h in outs]


def to_gpu(ary, dtype=None):
    return DeviceArray.to_gpu(ary, dtype)


def is_device(x):
    return isinstance(x, DeviceArray)


class Workspace(object):
    """A zero-initialised device scratch buffer (reduction partials and
    tickets), allocated once per size and reused by later calls."""

    _cache = {}

    @classmethod
    def get(cls, nbytes, key="reduce"):
        k = (key, int(nbytes), torch().cuda.current_device())
        ws = cls._cache.get(k)
        if ws is None:
            ws = DeviceArray.zeros((int(nbytes) + 255) // 8 + 32, np.float64)
            cls._cache[k] = ws
        return ws


def norms(x):
    """(sum of squares, max |x_i|) of a DeviceArray, reduced in FP64 on the
    device; synchronises to return host floats."""
    ws = Workspace.get(_lib.load().opyx_reduce_workspace_size())
    out = DeviceArray.zeros((2,), np.float64)
    _lib.call("opyx_norms", x.dcode, x.size, x.ptr, out.ptr, ws.ptr, stream_ptr())
    h = out.get()
    return float(h[0]), float(h[1])


def dot(x, y):
    """<x, y> of two DeviceArrays of the same size and dtype, reduced in
    FP64 on the device (deterministic); synchronises to return a float."""
    if x.size != y.size or x.dtype != y.dtype:
        raise ValueError("dot: size or dtype mismatch")
    ws = Workspace.get(_lib.load().opyx_reduce_workspace_size(), key="dot")
    out = DeviceArray.zeros((1,), np.float64)
    _lib.call("opyx_dot", x.dcode, x.size, x.ptr, y.ptr, out.ptr, ws.ptr, stream_ptr())
    return float(out.get()[0])


def norm(x):
    """Euclidean norm of a DeviceArray (FP64 reduction)."""
    return float(np.sqrt(norms(x)[0]))


def abs_(x, out=None):
    out = x if out is None else out
    _lib.call("opyx_abs", x.dcode, x.size, x.ptr, out.ptr, stream_ptr())
    return out
