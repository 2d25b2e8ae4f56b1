"""Device evaluation of functionals through ``opyx_fct_eval``."""

import numpy as np

from opymize_gb300 import _lib
from opymize_gb300.gpuarray import DeviceArray, Workspace, stream_ptr


def fct(kind, ngroups, m1, m2=1, **kw):
    f = _lib.opyx_fct()
    f.kind = _lib.FCT[kind]
    f.ngroups, f.m1, f.m2 = int(ngroups), int(m1), int(m2)
    for k, v in kw.items():
        setattr(f, k, v)
    return f


def evaluate(f, x):
    """Run the reduction; returns host (val, infeas)."""
    ws = Workspace.get(_lib.load().opyx_reduce_workspace_size())
    out = DeviceArray.zeros((2,), np.float64)
    _lib.call("opyx_fct_eval", f, x.dcode, x.ptr, out.ptr, ws.ptr, stream_ptr())
    h = out.get()
    return float(h[0]), float(h[1])


def devcopy(owner, name, host, dtype):
    cache = owner.__dict__.setdefault("_devcache", {})
    key = (name, np.dtype(dtype).str)
    if key not in cache:
        # float data is uploaded in its host precision and converted on the
        # device (a host-side cast of a 2048^2 x 3 image costs more than
        # the whole solve)
        cache[key] = DeviceArray.to_gpu(host, dtype)
    return cache[key]
