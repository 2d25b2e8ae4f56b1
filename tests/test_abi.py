"""CPU checks of the C ABI boundary: the library loads, exports every entry
point that include/opyx.h declares, the ctypes mirror in
opymize_gb300/_lib.py binds them all, and the ctypes structures have the
sizes and field offsets that a C compiler gives the header's structs.  No
compute call is made (no GPU here)."""

import ctypes as C
import os
import re
import shutil
import subprocess

import pytest

from opymize_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "opyx.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(opyx_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_lib.LIB_PATH):
        from opymize_gb300 import build
        build.build()
    return _lib.load()


def test_header_declares_entry_points():
    names = declared_functions()
    assert len(names) >= 40
    assert "opyx_rof_iterate" in names and "opyx_gradient" in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_ctypes_mirror_binds_every_declared_symbol():
    assert sorted(_lib.SIGNATURES) == declared_functions()


def test_status_strings(lib):
    assert _lib.status_string(0) == "ok"
    assert "argument" in _lib.status_string(1)


STRUCTS = {
    "opyx_grid": _lib.opyx_grid,
    "opyx_step": _lib.opyx_step,
    "opyx_adaptive_state": _lib.opyx_adaptive_state,
    "opyx_fct": _lib.opyx_fct,
    "opyx_epigraph": _lib.opyx_epigraph,
    "opyx_rof_problem": _lib.opyx_rof_problem,
    "opyx_rof_buffers": _lib.opyx_rof_buffers,
    "opyx_rof_info": _lib.opyx_rof_info,
    "opyx_sublabel": _lib.opyx_sublabel,
    "opyx_conv3x3_desc": _lib.opyx_conv3x3_desc,
}


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_struct_layout_matches_header(tmp_path):
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "opyx.h"', 'int main(void){']
    for name, cls in STRUCTS.items():
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (name, name))
        for fname, _ in cls._fields_:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (name, fname, name, fname))
    lines.append("return 0;}")
    c = tmp_path / "layout.c"
    c.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(c), "-o", str(exe)])
    out = dict(l.split() for l in subprocess.check_output([str(exe)]).decode().splitlines())
    for name, cls in STRUCTS.items():
        import ctypes
        assert int(out[name]) == ctypes.sizeof(cls), name
        for fname, _ in cls._fields_:
            assert int(out[name + "." + fname]) == getattr(cls, fname).offset, (name, fname)


def test_no_cpu_fallback_without_gpu():
    """Operators refuse host arrays instead of computing on the CPU."""
    import numpy as np
    from opymize_gb300.linear import GradientOp
    op = GradientOp((4, 5), 1, scheme="forward")
    with pytest.raises(TypeError):
        op(np.zeros(20), np.zeros(40))
    from opymize_gb300.solvers import PDHG
    from opymize_gb300.functionals import SSD, L1Norms
    s = PDHG(SSD(np.zeros((20, 1))), L1Norms(20, (1, 2), 0.1), op)
    with pytest.raises(NotImplementedError):
        s.solve(use_gpu=False)


# Fake device addresses: aligned, never dereferenced, because each call below
# fails its argument checks (or has no work) before it touches the device.
_P = 1 << 40


def _grid(ndim=2, dims=(4, 5), h=1.0, C=1):
    g = _lib.opyx_grid()
    g.ndim, g.nchannels = ndim, C
    for t in range(min(ndim, len(dims))):
        g.dims[t], g.h[t] = dims[t], h
    return g


def _epigraph(ndim=1, nsub=2, nfuns=3, nregions=2, npoints=3):
    e = _lib.opyx_epigraph()
    e.ndim, e.nsubpoints, e.nfuns, e.nregions, e.npoints = ndim, nsub, nfuns, nregions, npoints
    e.I, e.J, e.v, e.b = _P, _P + 4096, _P + 8192, _P + 12288
    return e


def _conv(**kw):
    d = _lib.opyx_conv3x3_desc()
    d.batch, d.height, d.width = 1, 8, 8
    d.in_channels = d.in_stride = 32
    d.out_channels = d.out_stride = 32
    d.x, d.w, d.y = _P, _P + 65536, _P + 131072
    for k, v in kw.items():
        setattr(d, k, v)
    return d


def _rof(dims, C=1):
    p = _lib.opyx_rof_problem()
    p.dtype, p.ndim, p.nchannels, p.steps = _lib.OPYX_F32, len(dims), C, 2   # precond
    for t, n in enumerate(dims):
        p.dims[t], p.h[t] = n, 1.0
    for k in range(C):
        p.weights[k] = p.vol[k] = 1.0
    p.lbd, p.theta = 0.1, 1.0
    return p


def _rof_buffers():
    b = _lib.opyx_rof_buffers()
    b.x, b.xbar, b.y, b.f, b.ws, b.y2 = _P, _P + 4096, _P + 8192, _P + 12288, _P + 65536, \
        _P + 131072
    return b


ARG, UNSUP, WS, OK = (_lib.OPYX_ERR_ARG, _lib.OPYX_ERR_UNSUPPORTED, _lib.OPYX_ERR_WORKSPACE,
                      _lib.OPYX_OK)

ERROR_CASES = [
    ("opyx_fill", (0, None, 10, 0.0, None), ARG),
    ("opyx_fill", (0, None, 0, 0.0, None), OK),                         # nothing to do
    ("opyx_axpby", (0, -1, 1.0, _P, 0.0, _P, None), ARG),
    ("opyx_matrixmult", (0, -1, 2, 2, _P, 0, _P, _P, 0, None), ARG),
    ("opyx_matrixmult", (0, 10, 0, 2, _P, 0, _P, _P, 0, None), OK),     # J = 0: no output
    ("opyx_matrixmultr", (0, 10, 2, 2, None, 0, _P, _P, 0, None), ARG),
    ("opyx_matrixmultr", (7, 10, 2, 2, _P, 0, _P, _P, 0, None), ARG),    # unknown dtype
    ("opyx_indexedmult", (0, 2, 10, 1, 1, 0, _P, _P, _P, _P, 0, None), ARG),      # K < 1
    ("opyx_indexedmult_adj", (0, 2, 10, 1, 1, 0, _P, _P, _P, _P, 0, None), ARG),
    ("opyx_indexedmult_adj", (0, 2, 10, 1, 1, 3, _P, None, _P, _P, 0, None), ARG),  # no P
    ("opyx_l1normsproj", (0, 10, 1, 2, 0.1, 99, _P, None), ARG),       # unknown norm
    ("opyx_l1normsproj", (0, 10, 3, 3, 0.1, 1, _P, None), UNSUP),      # spectral, 3 x 3
    ("opyx_l1normsproj_jac", (0, 10, 2, 0.0, _P, _P, _P, None), ARG),  # lbd <= 0
    ("opyx_dot", (0, 10, _P, _P, _P, _P + 4, None), WS),               # misaligned workspace
    ("opyx_dot", (0, 10, _P, _P, None, _P, None), ARG),
    ("opyx_gradient", (None, 0, None, 0, _P, _P, 0, None), ARG),
    ("opyx_gradient", (_grid(h=0.0), 0, None, 0, _P, _P, 0, None), ARG),
    ("opyx_gradient", (_grid(), 9, None, 0, _P, _P, 0, None), ARG),    # unknown scheme
    ("opyx_epigraph_proj", (_epigraph(ndim=4), 0, _P, _P, 10, 1e-9, None, None), UNSUP),
    ("opyx_epigraph_proj", (_epigraph(), 0, _P, _P, 0, 1e-9, None, None), ARG),  # maxiter 0
    ("opyx_epigraph_proj", (_epigraph(nregions=0), 0, _P, _P, 10, 1e-9, None, None), OK),
    ("opyx_conv3x3", (None, None), ARG),
    ("opyx_conv3x3", (_conv(in_channels=24, in_stride=24), None), ARG),  # channels per chunk
    ("opyx_conv3x3", (_conv(out_channels=48, out_stride=48), None), UNSUP),
    ("opyx_conv3x3", (_conv(x=_P + 8), None), ARG),                    # 16-byte alignment
    # dims whose product wraps int64 ({2^62 + 1, 4} would wrap to 4 pixels)
    ("opyx_rof_init", (_rof((2 ** 62 + 1, 4)), _rof_buffers(), None), ARG),
    ("opyx_rof_iterate", (_rof((2 ** 62 + 1, 4)), _rof_buffers(), 1, None), ARG),
    ("opyx_rof_init", (_rof((2 ** 21, 2 ** 21, 2 ** 21)), _rof_buffers(), None), ARG),
    ("opyx_rof_init", (_rof((2 ** 20, 2 ** 19), C=4), _rof_buffers(), None), ARG),  # > 2^40 values
    ("opyx_rof_init", (_rof((0, 4)), _rof_buffers(), None), ARG),
    ("opyx_rof_gap_iterate", (_rof((64, 64)), _rof_buffers(), -1, None), ARG),
    ("opyx_rof_gap_iterate", (_rof((2 ** 62 + 1, 4)), _rof_buffers(), 2, None), ARG),
    ("opyx_rof_iterate_noalloc", (_rof((2 ** 62 + 1, 4)), _P, _P, _P, None, 1, None, None),
     _lib.OPYX_ERR_SCRATCH_LIMIT),
    ("opyx_rof_iterate_noalloc", (_rof((4096, 4096)), _P, _P, _P, None, 1, None, None),
     _lib.OPYX_ERR_SCRATCH_LIMIT),                                     # xbar does not fit
    ("opyx_rof_iterate_noalloc", (_rof((0, 4)), _P, _P, _P, None, 1, None, None), ARG),
    ("opyx_rof_batch_persist", (None, None, None, 10, 100, None), ARG),
    ("opyx_rof_batch_persist", (_P, _P, _P, 7, 100, None), ARG),     # odd check interval
    ("opyx_rof_batch_persist", (_P, _P, _P, 10, 99, None), ARG),     # odd iteration count
]


@pytest.mark.parametrize("case", range(len(ERROR_CASES)))
def test_argument_checks_precede_device_work(lib, case):
    """The entry points' error behaviour: invalid arguments return their
    status without a launch (the reference's PyCUDA kernels return none;
    this boundary reports one per call, see opyx_status_string)."""
    name, args, want = ERROR_CASES[case]
    args = tuple(C.byref(a) if isinstance(a, C.Structure) else a for a in args)
    assert getattr(lib, name)(*args) == want, (name, _lib.status_string(getattr(lib, name)(*args)))
