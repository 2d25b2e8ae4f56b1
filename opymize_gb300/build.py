"""In-tree build of libopyx.so (the sm_103a CUDA kernels behind the C ABI).

    python -m opymize_gb300.build        # or opymize_gb300.build.build()

Each ``csrc/*.cu`` is compiled in parallel with ``nvcc -gencode
arch=compute_103a,code=sm_103a`` and linked into ``opymize_gb300/libopyx.so``
against the shared CUDA runtime.  Objects go to ``opymize_gb300/_build/``.
"""

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libopyx.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              "-I" + INCLUDE, "-I" + CSRC]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"),
                 "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libopyx")


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    return p.returncode, p.stdout, cmd


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False, jobs=None, extra_flags=()):
    """Compile every csrc/*.cu and link libopyx.so; returns the library path."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))
    cc = nvcc()
    jobs_list = []
    objs = []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs_list.append([cc, "-c", s, "-o", o] + ARCH + NVCC_FLAGS + list(extra_flags))
    workers = jobs or min(len(jobs_list), os.cpu_count() or 4) or 1
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        for rc, out, cmd in ex.map(_run, jobs_list):
            if verbose or rc != 0:
                sys.stdout.write(" ".join(cmd) + "\n" + out)
            if rc != 0:
                raise RuntimeError("nvcc failed on %s" % cmd[2])
    if force or jobs_list or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        cmd = [cc, "-shared", "-o", tmp] + objs + ARCH + ["-cudart", "shared",
                                                         "-Xlinker", "-rpath,/usr/local/cuda/lib64"]
        rc, out, _ = _run(cmd)
        if rc != 0:
            sys.stdout.write(out)
            raise RuntimeError("linking libopyx.so failed")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
