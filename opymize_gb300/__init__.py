"""opymize_gb300 -- GB300-native PDHG path with Opymize's Python API.

Core types mirror opymize/__init__.py:6-179 (``Variable``, ``Operator``,
``LinOp``, ``Functional``).  Operators dispatch on ``DeviceArray`` (this
package's stand-in for ``pycuda.gpuarray.GPUArray``) and run sm_103a kernels
from libopyx.so; there is no CPU path, so numpy inputs raise ``TypeError``.
"""

import numpy as np

from opymize_gb300.gpuarray import DeviceArray, to_gpu, is_device   # noqa: F401

__version__ = "1.0.0"


class Variable(object):
    """Flat buffer with named, reshaped sub-views (opymize/__init__.py:6-46)."""

    def __init__(self, *args):
        if len(args) == 1 and type(args[0]) in [np.int64, int]:
            args = [(args[0],)]
        if type(args[0][0]) is not str:
            args = list([('v%d' % i, a) for i, a in enumerate(args)])
        self._descr = {}
        self._args = args
        self.size = 0
        for name, dim in args:
            self._descr[name] = {
                'name': name,
                'offset': self.size,
                'shape': dim,
                'size': int(np.prod(dim)),
            }
            self.size += int(np.prod(dim))

    def vars(self, data=None, named=False):
        if data is None:
            if named:
                return self._descr
            return [self._descr[a[0]] for a in self._args]
        result = {} if named else [None for a in self._args]
        for i, a in enumerate(self._args):
            d = self._descr[a[0]]
            start, end = d['offset'], d['offset'] + int(np.prod(d['shape']))
            idx = d['name'] if named else i
            shape = d['shape'] if isinstance(d['shape'], tuple) else (d['shape'],)
            result[idx] = data[start:end].reshape(shape)
        return result

    def __getitem__(self, idx):
        if type(idx) is str:
            return self._descr[idx]
        return self._descr[self._args[idx][0]]

    def new(self, dtype=np.float64):
        """Host zeros of this size (as the reference's Variable.new)."""
        return np.zeros((self.size,), order='C', dtype=dtype)

    def new_gpu(self, dtype=np.float64):
        """Device zeros of this size."""
        return DeviceArray.zeros((self.size,), dtype)


def _require_device(x):
    if not isinstance(x, DeviceArray):
        raise TypeError("opymize_gb300 operators run on the GPU only: pass a DeviceArray "
                        "(opymize_gb300.to_gpu), got %s" % type(x).__name__)


class Operator(object):
    """T(x) (opymize/__init__.py:48-84)."""

    def __init__(self):
        self.x = None
        self.y = None

    def prepare_gpu(self, type_t="double"):
        pass

    def _call_gpu(self, x, y=None, add=False, jacobian=False):
        raise NotImplementedError("%s has no GPU implementation" % type(self).__name__)

    def __call__(self, x, y=None, add=False, jacobian=False):
        """Evaluate T(x); the result goes to y (to x if y is None), added to
        its current value if ``add``."""
        _require_device(x)
        return self._call_gpu(x, y=y, add=add, jacobian=jacobian)


class LinOp(Operator):
    """Matrix-free linear operator A (opymize/__init__.py:86-142)."""

    def __init__(self):
        Operator.__init__(self)
        self.adjoint = None

    def _call_gpu(self, x, y=None, add=False):
        raise NotImplementedError("%s has no GPU implementation" % type(self).__name__)

    def __call__(self, x, y=None, add=False, jacobian=False):
        _require_device(x)
        self._call_gpu(x, y=y, add=add)
        return self if jacobian else None

    def rowwise_lp(self, y, p=1, add=False):
        """y_i = |A_i|_p (p-norm of row i; sum_j |A_ij| for p = 1), on the device."""
        raise NotImplementedError("%s has no rowwise_lp" % type(self).__name__)


class Functional(object):
    """F with value/infeasibility, prox and conjugate (opymize/__init__.py:144-179)."""

    def __init__(self):
        self.x = None
        self.conj = None

    def __call__(self, x, grad=False):
        """(val, infeas) of F at a DeviceArray x, reduced in FP64 on the device."""
        _require_device(x)
        if grad:
            raise NotImplementedError("gradients of functionals are not on the PDHG path")
        return self._eval_gpu(x)

    def _eval_gpu(self, x):
        raise NotImplementedError("%s cannot be evaluated" % type(self).__name__)

    def prox(self, tau):
        raise NotImplementedError("%s has no prox" % type(self).__name__)
