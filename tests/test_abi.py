"""CPU checks of the C ABI boundary: the library loads, exports every entry
point that include/opyx.h declares, the ctypes mirror in
opymize_gb300/_lib.py binds them all, and the ctypes structures have the
sizes and field offsets that a C compiler gives the header's structs.  No
compute call is made (no GPU here)."""

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
