"""Compile the reference's own host-buildable kernels as test oracles.

Outputs go to oracle/_ref/ only (git-ignored).  Needs the reference sources
(opymize/operators/proj.cu) at REF_ROOT (default /root/reference); without
them nothing is built and the tests that need these libraries skip.  Used
only by tests/ and tests/golden/ scripts.

    python oracle/build_ref.py
"""

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REF_ROOT = os.environ.get("REF_ROOT", "/root/reference")
PROJ_DIR = os.path.join(REF_ROOT, "opymize", "operators")


def lib_path(ndim):
    return os.path.join(OUT, "libref_epigraph_%d.so" % ndim)


def build(verbose=True):
    if not os.path.exists(os.path.join(PROJ_DIR, "proj.cu")):
        if verbose:
            print("oracle/_ref: reference sources not found; skipped")
        return False
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(HERE, "ref_epigraph.cpp")
    procs = []
    for nd in (1, 2, 3):
        cmd = ["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-w", "-Dndim=%d" % nd,
               "-I", PROJ_DIR, src, "-o", lib_path(nd)]
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE,
                                            stderr=subprocess.STDOUT)))
    ok = True
    for cmd, p in procs:
        out = p.communicate()[0].decode()
        if p.returncode != 0:
            ok = False
            print("oracle/_ref build failed: %s\n%s" % (" ".join(cmd), out), file=sys.stderr)
    return ok


if __name__ in ("__main__", "__graft_build__"):
    build()
