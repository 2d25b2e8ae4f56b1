"""A fused ROF solve of a seeded synthetic image or volume for a fixed
number of iterations -- a small, repeatable case for profilers:

    python -m opymize_gb300.solvers --dims 256 256 256 --iters 20
    python -m opymize_gb300.solvers --dims 2048 2048 --channels 3 --huber 0.01 --lbd 0.05
    python -m opymize_gb300.solvers --dims 512 512 --sublabel 16 --lbd 0.1 --iters 10
    python -m opymize_gb300.solvers --dims 2048 2048 --lbd 0.1 --iters 20 --gran 10

``--gran`` is the check interval (default: one check after the last
iteration); with 2-D single sweeps each check but the last is computed by the
first sweep of the next chunk.

With ``--sublabel L`` the problem is the sublabel-lifted model of
``tools.lifting.sublabel_problem`` (L labels on [0, 1], 8 samples per
interval) on the generic PDHG path.
"""

import argparse
import json
import time

import numpy as np

from opymize_gb300.functionals import SSD, L1Norms, HuberL1Norms
from opymize_gb300.gpuarray import torch
from opymize_gb300.linear import GradientOp
from opymize_gb300.solvers import PDHG
from opymize_gb300.tools.synthetic import piecewise_constant


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--dims", type=int, nargs="+", default=[256, 256, 256])
    ap.add_argument("--channels", type=int, default=1)
    ap.add_argument("--lbd", type=float, default=0.08)
    ap.add_argument("--huber", type=float, default=0.0)
    ap.add_argument("--iters", type=int, default=20)
    ap.add_argument("--steps", default="precond")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--sublabel", type=int, default=0)
    ap.add_argument("--gran", type=int, default=0)
    a = ap.parse_args(argv)
    gran = a.gran if a.gran > 0 else a.iters
    if a.sublabel:
        return sublabel(a)
    dims, C = tuple(a.dims), a.channels
    N, D = int(np.prod(dims)), len(dims)
    f = piecewise_constant(dims, C, sigma=0.1, seed=a.seed)
    F = HuberL1Norms(N, (C, D), a.lbd, a.huber) if a.huber > 0 else L1Norms(N, (C, D), a.lbd)
    s = PDHG(SSD(f.reshape(N, C)), F, GradientOp(dims, C, scheme="forward"))
    s.solve(steps=a.steps, precision="float", term_pd_gap=1e-300, term_maxiter=a.iters,
            granularity=gran)
    torch().cuda.synchronize()
    print(json.dumps({"dims": list(dims), "channels": C, "path": s.path, "iters": s.info["iter"],
                      "relgap": s.info["relgap"]}))


def sublabel(a):
    from opymize_gb300.tools import lifting
    dims = tuple(a.dims)
    img = np.clip(piecewise_constant(dims, 1, sigma=0.05, seed=a.seed, salt_pepper=0.1)[..., 0], 0, 1)
    g, f, A, _ = lifting.sublabel_problem(img, L=a.sublabel, lbd=a.lbd, samples=8)
    s = PDHG(g, f, A)
    el = []
    for _ in range(2):          # the second solve is timed (setup cached)
        torch().cuda.synchronize()
        t0 = time.perf_counter()
        s.solve(steps=a.steps, precision="float", term_pd_gap=1e-300, term_maxiter=a.iters,
                granularity=a.iters)
        torch().cuda.synchronize()
        el.append(time.perf_counter() - t0)
    print(json.dumps({"dims": list(dims), "labels": a.sublabel, "path": s.path,
                      "iters": s.info["iter"], "relgap": s.info["relgap"],
                      "iters_per_s": round(a.iters / el[-1], 1)}))


if __name__ == "__main__":
    main()
