"""Step sizes as the kernels take them (``opyx_step``): a per-element device
vector (diagonal preconditioning), a device double written by the solver
(adaptive steps, read by every kernel at run time so that no iteration waits
for the host), or a constant."""

import numpy as np

from opymize_gb300 import _lib
from opymize_gb300.gpuarray import DeviceArray


class DeviceScalar(object):
    """A double in device memory: ``ptr`` is its address.  ``host_value`` is
    the value the host last wrote or read (for logging and for ``float()``)."""

    def __init__(self, ptr, owner=None, host_value=None):
        self.ptr = int(ptr)
        self.owner = owner          # keeps the backing allocation alive
        self.host_value = host_value

    def __float__(self):
        if self.host_value is None:
            raise ValueError("device scalar has no host copy")
        return float(self.host_value)


def step_struct(tau, dtype=None):
    s = _lib.opyx_step()
    if isinstance(tau, DeviceArray):
        if dtype is not None and np.dtype(tau.dtype) != np.dtype(dtype):
            raise TypeError("step vector dtype %s does not match iterates %s" % (tau.dtype, dtype))
        s.vec = tau.ptr
    elif isinstance(tau, DeviceScalar):
        s.dev = tau.ptr
    elif isinstance(tau, np.ndarray):
        raise TypeError("per-element steps must be DeviceArrays on the GPU path")
    else:
        s.value = float(tau)
    return s
