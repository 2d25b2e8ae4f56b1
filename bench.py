#!/usr/bin/env python
"""ROF time-to-gap benchmark of the fused GB300 PDHG path.

Workload (one "step" = one full solve): colour TV denoising, 2048 x 2048 x 3
fp32, joint Frobenius coupling of the per-pixel 3x2 Jacobian with Huber
smoothing alpha = 0.01, lambda = 0.05, f from the seeded piecewise-constant
generator (sigma = 0.1), diagonally preconditioned steps, until the relative
primal-dual gap is <= 1e-4 (gap checked every --gran iterations).

value   -- milliseconds per solve with f resident in HBM (x, y reset to 0
           inside the timed region), CUDA events, max over ranks.
e2e     -- the same solve through the public API PDHG(...).solve(use_gpu=True)
           from host numpy data: host->device copies of f and the start
           point, device->host copies of x and y, all inside the timed region.
roofline-- the dominant fused pass: algorithmic bytes per launch / average
           launch time (CUDA events on the launching stream) vs the measured
           HBM copy bandwidth.
cpu_baseline / --impl reference -- the CPU oracle (a numpy/scipy port of the
           reference's CPU PDHG, FP64) on the same input.

Multi-GPU: independent replicas (the path does not shard); N ranks each solve
their own instance, the reported time is the max over ranks.
"""

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ROF time-to-gap 1e-4 (ms)"
UNIT = "ms"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="opyx", choices=["opyx", "reference"])
    ap.add_argument("--size", type=int, default=2048)
    ap.add_argument("--channels", type=int, default=3)
    ap.add_argument("--huber", type=float, default=0.01)
    ap.add_argument("--lbd", type=float, default=0.05)
    ap.add_argument("--tol", type=float, default=1e-4)
    ap.add_argument("--gran", type=int, default=6)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline leg")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the volume and sublabel configurations")
    return ap.parse_args()


def workload_config(a, world):
    ws_mb = 4 * a.size * a.size * a.channels * 7 // 2 ** 20
    return {
        "workload": "colour Huber-TV ROF %dx%dx%d fp32, alpha=%g, lambda=%g, precond steps, "
                    "until relgap<=%g" % (a.size, a.size, a.channels, a.huber, a.lbd, a.tol),
        "image": [a.size, a.size, a.channels], "lambda": a.lbd, "huber_alpha": a.huber,
        "steps": "precond", "tol": a.tol, "gap_check_every": a.gran, "seed": a.seed,
        "l2": "working set (x, xbar, y, y2, f = %d MB) %s than L2 (126 MB)" %
              (ws_mb, "larger" if ws_mb > 126 else "smaller"),
        "parallelism": "replicas x%d" % world,
    }


def make_image(a):
    from opymize_gb300.tools.synthetic import piecewise_constant
    return piecewise_constant((a.size, a.size), a.channels, sigma=0.1, seed=a.seed)


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class ClockSampler(object):
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 7:
                self.rows.append((time.time(), parts))

    def mark(self):
        """Host time stamp of the timed region's start or end."""
        return time.time()

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self, t0=None, t1=None):
        """Median SM clock and throttle reasons of the samples taken between
        host times t0 and t1 (the timed region)."""
        rows = [r for (t, r) in self.rows if (t0 is None or t >= t0) and (t1 is None or t <= t1)]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in rows if r[0].replace('.', '', 1).isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace('.', '', 1).isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[j] for r in rows for j in range(4)
                          if r[3 + j].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


# ----------------------------------------------------------------- GPU arm
class ResidentSolver(object):
    """The fused ROF solve with f, x, y, xbar and the workspace resident in HBM."""

    def __init__(self, a, f, dims=None, lbd=None, huber=None, gran=None):
        from opymize_gb300 import _lib
        from opymize_gb300.gpuarray import DeviceArray
        from opymize_gb300.functionals import SSD, L1Norms, HuberL1Norms
        from opymize_gb300.linear import GradientOp
        from opymize_gb300.solvers import PDHG
        self.lib = _lib
        dims = (a.size, a.size) if dims is None else tuple(dims)
        C = f.shape[-1]
        D = len(dims)
        N = int(np.prod(dims))
        lbd = a.lbd if lbd is None else lbd
        huber = a.huber if huber is None else huber
        self.N, self.C, self.K = N, C, D * C
        self.gran, self.tol = (a.gran if gran is None else gran), a.tol
        F = HuberL1Norms(N, (C, D), lbd, huber) if huber > 0 else L1Norms(N, (C, D), lbd)
        self.solver = PDHG(SSD(f.reshape(N, C)), F, GradientOp(dims, C, scheme="forward"))
        s = self.solver
        s.constvars.update(theta=1.0, precond=True)
        self.p = s._rof_problem(np.float32, "precond")
        self.f = s.g.f_dev(np.float32)
        self.x = DeviceArray.zeros((N * C,), np.float32)
        self.y = DeviceArray.zeros((N * D * C,), np.float32)
        self.xbar = DeviceArray.zeros((N * C,), np.float32)
        self.y2 = DeviceArray.zeros((N * D * C,), np.float32)   # single-sweep ping-pong
        wsb = _lib.load().opyx_rof_workspace_size()
        self.ws = DeviceArray.zeros(((wsb + 7) // 8,), np.float64)
        b = _lib.opyx_rof_buffers()
        b.x, b.xbar, b.y, b.f, b.ws = self.x.ptr, self.xbar.ptr, self.y.ptr, self.f.ptr, self.ws.ptr
        b.y2 = self.y2.ptr
        self.b = b
        self.p.term_mode = 1
        self.p.term_relgap = self.p.term_infeas = self.tol
        from opymize_gb300.solvers.pdhg import _FusedLoop
        self.loop = _FusedLoop(self.p, self.b, self.ws, self.gran)
        self.launches = 0

    def solve(self, maxiter=5000):
        """The solver's own check loop (chunks queued ahead of their checks,
        device-side stop test) from a zero start."""
        from opymize_gb300.gpuarray import stream_ptr
        self.x.fill(0.0)
        self.y.fill(0.0)
        self.lib.call("opyx_rof_init", self.p, self.b, stream_ptr())
        l0 = self.loop.launches
        it, rec = self.loop.run(maxiter)
        self.launches += 3 + self.loop.launches - l0
        self.iters, self.relgap = it, float(rec[5])
        return it

    def time_pass(self, which, reps=20):
        from opymize_gb300.gpuarray import torch, stream_ptr
        t = torch()
        s = t.cuda.current_stream()
        # clears the stop flag of the last solve (the passes would return at once)
        self.lib.call("opyx_rof_init", self.p, self.b, stream_ptr())
        for _ in range(3):
            self.lib.call("opyx_rof_pass", self.p, self.b, which, stream_ptr())
        e0, e1 = t.cuda.Event(enable_timing=True), t.cuda.Event(enable_timing=True)
        t.cuda.synchronize()
        e0.record(s)
        for _ in range(reps):
            self.lib.call("opyx_rof_pass", self.p, self.b, which, stream_ptr())
        e1.record(s)
        t.cuda.synchronize()
        return e0.elapsed_time(e1) / reps * 1e-3   # seconds per launch


def volume_case(a):
    """The volume configuration: 256^3, one channel, TV (lambda = 0.08),
    ellipsoids + noise 0.1, precond steps, until relgap <= 1e-4, data resident
    (3-D single sweeps: plane tiles streamed along z; the two passes they
    replace are timed beside them)."""
    from opymize_gb300.gpuarray import torch
    from opymize_gb300.tools.synthetic import piecewise_constant
    t = torch()
    f = piecewise_constant((256, 256, 256), 1, sigma=0.1, seed=a.seed)
    rs = ResidentSolver(a, f, dims=(256, 256, 256), lbd=0.08, huber=0.0, gran=10)
    rs.solve()
    e0, e1 = t.cuda.Event(enable_timing=True), t.cuda.Event(enable_timing=True)
    reps = 3
    t.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        rs.solve()
    e1.record()
    t.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    N, C, K = rs.N, rs.C, rs.K
    it_bytes = 4.0 * N * (5 * C + 3 * K)
    sw_bytes = 4.0 * N * (3 * C + 2 * K)
    tA, tB = rs.time_pass(0), rs.time_pass(1)
    tS = rs.time_pass(3)
    peak = measured_peaks().get("hbm_gbs")
    return {"workload": "TV volume 256^3 fp32, lambda=0.08, precond steps, until relgap<=1e-4",
            "time_to_gap_ms": round(ms, 3), "iters_to_gap": rs.iters, "final_relgap": rs.relgap,
            "sweep_us": round(tS * 1e6, 2),
            "sweep_GBps": round(sw_bytes / tS / 1e9, 1),
            "sweep_frac_of_measured_hbm": round(sw_bytes / tS / 1e9 / peak, 3) if peak else None,
            "sweep_algorithmic_bytes": sw_bytes,
            "two_pass": {"passA_us": round(tA * 1e6, 2), "passB_us": round(tB * 1e6, 2),
                         "GBps": round(it_bytes / (tA + tB) / 1e9, 1)},
            "data": "synthetic ellipsoids, resident in HBM"}


def gray_case(a, size=2048, lbd=0.1, gran=10, cpu_iters=20):
    """Plain gray ROF (the reference example's model, examples/rof.py:60-80,
    with its preconditioned steps): size^2, one channel, SSD + lambda*L1Norms
    of the forward gradient, lambda = 0.1, noise 0.1, until relgap <= 1e-4
    (gap every `gran` iterations), data resident; the public API from host
    data; the one-channel sweep's share of the roofline; and the oracle on
    the host cores (its set-up and one gap timed once, `cpu_iters`
    iterations timed without set-up, scaled to the solve's counts)."""
    from opymize_gb300.gpuarray import torch
    from opymize_gb300.tools.synthetic import piecewise_constant
    from opymize_gb300.functionals import SSD, L1Norms
    from opymize_gb300.linear import GradientOp
    from opymize_gb300.solvers import PDHG
    t = torch()
    dims = (size, size)
    N = size * size
    f = piecewise_constant(dims, 1, sigma=0.1, seed=a.seed)
    rs = ResidentSolver(a, f, dims=dims, lbd=lbd, huber=0.0, gran=gran)
    rs.solve(maxiter=100000)
    e0, e1 = t.cuda.Event(enable_timing=True), t.cuda.Event(enable_timing=True)
    reps = 3
    t.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        rs.solve(maxiter=100000)
    e1.record()
    t.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    iters = rs.iters
    sw_bytes = 4.0 * N * (3 + 2 * 2)
    tS = rs.time_pass(3)
    peak = measured_peaks().get("hbm_gbs")
    del rs
    # the public API, host data in and out
    s = PDHG(SSD(f.reshape(N, 1)), L1Norms(N, (1, 2), lbd), GradientOp(dims, 1, scheme="forward"))
    s.solve(steps="precond", precision="float", term_pd_gap=a.tol, granularity=gran,
            term_maxiter=100000)
    t.cuda.synchronize()
    t0 = time.perf_counter()
    s = PDHG(SSD(f.reshape(N, 1)), L1Norms(N, (1, 2), lbd), GradientOp(dims, 1, scheme="forward"))
    s.solve(steps="precond", precision="float", term_pd_gap=a.tol, granularity=gran,
            term_maxiter=100000)
    x, y = s.state
    t.cuda.synchronize()
    e2e_ms = (time.perf_counter() - t0) * 1e3
    rec = {"workload": "gray TV ROF %dx%d fp32, lambda=%g, precond steps, until relgap<=%g"
                       % (size, size, lbd, a.tol),
           "time_to_gap_ms": round(ms, 3), "iters_to_gap": iters,
           "e2e_ms": round(e2e_ms, 3),
           "sweep_us": round(tS * 1e6, 2), "sweep_GBps": round(sw_bytes / tS / 1e9, 1),
           "sweep_frac_of_measured_hbm": round(sw_bytes / tS / 1e9 / peak, 3) if peak else None,
           "sweep_algorithmic_bytes": sw_bytes,
           "data": "synthetic piecewise-constant image + noise 0.1, resident in HBM"}
    if not a.no_cpu:
        so = cpu_solver(a, f, dims=dims, lbd=lbd, huber=0.0)
        t0 = time.perf_counter()
        so._setup()
        t_setup = time.perf_counter() - t0
        t0 = time.perf_counter()
        so.iterate(cpu_iters)
        t_it = (time.perf_counter() - t0) / cpu_iters
        t0 = time.perf_counter()
        so.pd_gap()
        t_gap = time.perf_counter() - t0
        so.close()
        cpu_ms = (t_setup + t_it * iters + t_gap * (iters // gran)) * 1e3
        rec["cpu_baseline"] = {
            "value": round(cpu_ms, 1), "unit": "ms", "cores": so.threads, "kind": "port",
            "sample": "oracle (numpy/scipy port of the reference CPU PDHG, FP64) on the same "
                      "input over %d host threads: set-up (%.3f s) and one gap (%.3f s) timed "
                      "once, %d iterations timed without set-up (%.4f s/it), scaled to the "
                      "solve's %d iterations and %d checks" % (so.threads, t_setup, t_gap,
                                                               cpu_iters, t_it, iters,
                                                               iters // gran)}
        rec["cpu_over_gpu"] = round(cpu_ms / ms, 1)
        rec["cpu_over_gpu_e2e"] = round(cpu_ms / e2e_ms, 1)
    return rec


def sublabel_case(a, iters=5000):
    """The sublabel-lifted configuration: 512^2, 16 labels on [0, 1],
    rho = min((u - f)^2, 0.04) sampled at 8 points per interval, 10%
    salt-and-pepper, TV weight 0.1, preconditioned steps, `iters`
    iterations in FP32 (the fused sublabel passes) and the same solve in
    FP64 (pinned to the reference's CPU solver at 1e-10 on the fixtures):
    iterations per second, the HBM fraction of the iteration, the gap and
    infeasibilities of both and the FP32 error against FP64."""
    from opymize_gb300.gpuarray import torch
    from opymize_gb300.solvers import PDHG
    from opymize_gb300.tools import lifting
    from opymize_gb300.tools.synthetic import piecewise_constant
    t = torch()
    img = np.clip(piecewise_constant((512, 512), 1, sigma=0.05, seed=a.seed,
                                     salt_pepper=0.1)[..., 0], 0, 1)
    res = {"workload": "sublabel lifting 512^2, 16 labels, 8 samples/interval, truncated "
                       "quadratic data term, lambda 0.1, precond steps, %d iterations" % iters}
    states = {}
    for precision in ("float", "double"):
        g, f, A, _ = lifting.sublabel_problem(img, L=16, lbd=0.1, samples=8)
        s = PDHG(g, f, A)
        s.solve(steps="precond", precision=precision, term_pd_gap=1e-300, term_maxiter=20,
                granularity=20)
        t.cuda.synchronize()
        t0 = time.perf_counter()
        s.solve(steps="precond", precision=precision, term_pd_gap=1e-300, term_maxiter=iters,
                granularity=iters)
        t.cuda.synchronize()
        el = time.perf_counter() - t0
        states[precision] = s.state
        res[precision] = {"path": s.path, "wall_s": round(el, 3),
                          "iters_per_s": round(iters / el, 1),
                          "loop_iters_per_s": round(float(s.info["it_per_s"]), 1),
                          "relgap": s.info["relgap"], "objp": s.info["objp"],
                          "objd": s.info["objd"], "infeasp": s.info["infeasp"],
                          "infeasd": s.info["infeasd"]}
    (x32, y32), (x64, y64) = states["float"], states["double"]
    res["fp32_vs_fp64"] = {
        "x_rel_l2": float(np.linalg.norm(x32 - x64) / np.linalg.norm(x64)),
        "y_rel_l2": float(np.linalg.norm(y32 - y64) / np.linalg.norm(y64)),
        "relgap_abs_diff": abs(res["float"]["relgap"] - res["double"]["relgap"])}
    N, L = 512 * 512, 16
    n_p, n_d = L + 1 + 2 * (L - 1), 3 * L + 2
    alg = 4.0 * N * (5 * n_p + 3 * n_d)               # iterates, two-pass count
    data = 4.0 * N * 8 * (L - 1)                       # the data term at the interval points
    it_s = res["float"]["loop_iters_per_s"]
    peak = measured_peaks().get("hbm_gbs")
    res["hbm"] = {"algorithmic_bytes_per_iter": alg, "data_term_bytes_per_iter": data,
                  "GBps": round((alg + data) * it_s / 1e9, 1),
                  "frac_of_measured_hbm": round((alg + data) * it_s / 1e9 / peak, 3)
                  if peak else None}
    res["note"] = ("wall time of solve() includes its set-up (steps, initial A x, the fused "
                   "passes' tables) and the final gap; loop_iters_per_s is the iteration loop")
    return res


def batch_specs(seed, n=512):
    """Sizes, noise levels and weights of the batched configuration's
    instances (sides log-uniform in [64, 1024], aspect U[0.5, 2], lambda
    U[0.02, 0.3], sigma U[0.05, 0.2])."""
    rng = np.random.default_rng(seed)
    specs = []
    for k in range(n):
        side = np.exp(rng.uniform(np.log(64), np.log(1024)))
        asp = rng.uniform(0.5, 2.0)
        H = max(8, int(round(side)))
        W = max(4, int(round(side * asp / 4)) * 4)
        sigma = rng.uniform(0.05, 0.2)
        lbd = rng.uniform(0.02, 0.3)
        specs.append((H, W, sigma, lbd, 1000 + k))
    return specs


def batch_case(a, world=1, rank=0):
    """The batched configuration: 512 independent 2-D instances, FP32; every
    instance retires at its own relgap 1e-4; rows per work item and the check
    interval chosen by the autotuner (BatchROF).  With several ranks the
    instances are sharded by size (solvers.batch.shard, no collective on the
    data path) and the per-instance stats gathered once at the end."""
    from opymize_gb300.gpuarray import torch
    from opymize_gb300.solvers import BatchROF
    from opymize_gb300.solvers.batch import shard, gather_stats
    from opymize_gb300.tools.synthetic import piecewise_constant
    t = torch()
    specs = batch_specs(a.seed)
    mine = shard([H * W for (H, W, _, _, _) in specs], rank, world)
    imgs = [piecewise_constant((specs[i][0], specs[i][1]), 1, sigma=specs[i][2],
                               seed=specs[i][4]) for i in mine]
    lbds = [specs[i][3] for i in mine]
    b = BatchROF(imgs, lbds, tol=1e-4, granularity=None)   # rows per item and check interval tuned
    b.autotune()
    t.cuda.synchronize()
    t0 = time.perf_counter()
    info = b.solve(maxiter=20000)
    t.cuda.synchronize()
    el = time.perf_counter() - t0
    stats = {int(i): (int(d["iter"]), bool(d["converged"]), el) for i, d in zip(mine, info)}
    merged = {}
    for d in gather_stats(stats):
        merged.update(d)
    el = max(v[2] for v in merged.values())          # the slowest rank's wall time
    its = np.array([merged[i][0] for i in range(len(specs))])
    npx = np.array([H * W for (H, W, _, _, _) in specs])
    byts = float((28.0 * npx * its).sum())     # single sweep: 4 N (3C + 2K) bytes, C = 1, K = 2
    peak = measured_peaks().get("hbm_gbs")
    gbs = byts / el / 1e9
    return {"workload": "512 ROF instances, sides log-uniform [64, 1024], aspect U[0.5, 2], "
                        "lambda U[0.02, 0.3], sigma U[0.05, 0.2], fp32, retire at relgap 1e-4",
            "ranks": world,
            "solves_per_s": round(len(specs) / el, 2), "wall_s": round(el, 3),
            "converged": int(sum(v[1] for v in merged.values())), "maxiter": 20000,
            "iters_median": float(np.median(its)), "iters_max": int(its.max()),
            "pixels": int(npx.sum()), "sum_bytes_per_wall_GBps": round(gbs, 1),
            "frac_of_measured_hbm": round(gbs / peak / world, 3) if peak else None,
            "rows_per_item": b.rows_per_item, "granularity": b.gran,
            "tuning": {k: (round(v, 4) if isinstance(v, float) else v) for k, v in b.tuning.items()},
            "launches": b.launches,
            "data": "synthetic piecewise-constant images, resident in HBM"}


def warm_start_case(a, n_eval=32):
    """The learned warm start on 512^2: the committed U-Net's proposals vs
    the zero start on held-out seeds, same solver (BatchROF) and stop test;
    plus the tcgen05 convolutions' throughput (forward of a 32-image batch,
    and the largest layer alone) against the measured bf16 peak."""
    from opymize_gb300.gpuarray import torch
    from opymize_gb300.warmstart import UNet, evaluate, instances
    t = torch()
    path = os.path.join(ROOT, "opymize_gb300", "warmstart", "unet512.npz")
    net = UNet.load(path)
    seeds = range(3 * 10 ** 6, 3 * 10 ** 6 + n_eval)
    res = {"workload": "ROF 512^2, lambda U[0.02, 0.3], sigma U[0.05, 0.2]: U-Net proposal "
                       "(0.64M params, bf16 tensor cores) + fused PDHG vs zero start",
           "held_out": n_eval}
    for tol in (1e-4, 1e-3):
        ev = evaluate(net, seeds, S=512, tol=tol)
        res["relgap_%g" % tol] = {
            "iters_cold_mean": float(np.mean(ev["iters_cold"])),
            "iters_warm_mean": float(np.mean(ev["iters_warm"])),
            "solve_cold_ms": round(1e3 * ev["solve_cold_s"], 2),
            "solve_warm_ms": round(1e3 * ev["solve_warm_s"], 2),
            "net_ms": round(1e3 * ev["net_s"], 2),
            "time_ratio_cold_over_warm": round(ev["speedup"], 3),
            "converged": [ev["converged_cold"], ev["converged_warm"]]}
    # restart mode: the network corrects the iterate after 100 plain iterations
    from opymize_gb300.warmstart import evaluate_restart
    rnet = UNet.load(os.path.join(ROOT, "opymize_gb300", "warmstart", "unet512_restart.npz"))
    ev = evaluate_restart(rnet, seeds, 100, S=512, tol=1e-4)
    res["restart_after_100_relgap_0.0001"] = {
        "iters_cold_mean": float(np.mean(ev["iters_cold"])),
        "iters_warm_mean": float(np.mean(ev["iters_warm"])),
        "solve_cold_ms": round(1e3 * ev["solve_cold_s"], 2),
        "solve_warm_ms": round(1e3 * ev["solve_warm_s"], 2),
        "net_ms": round(1e3 * ev["net_s"], 2),
        "time_ratio_cold_over_warm": round(ev["speedup"], 3),
        "converged": [ev["converged_cold"], ev["converged_warm"]]}
    del rnet
    # the metric's own form: one 512^2 image at a time through the public
    # fused PDHG, zero start vs the network's proposal (continue_at), time to
    # relgap 1e-4 including the network's inference for that image
    from opymize_gb300.functionals import SSD, L1Norms
    from opymize_gb300.linear import GradientOp
    from opymize_gb300.solvers import PDHG
    fs, lams = instances(list(seeds)[:8], 512)
    N = 512 * 512
    rows = []
    for k in range(len(lams)):
        rec = {}
        for warm in (False, True):
            s = PDHG(SSD(fs[k].reshape(N, 1)), L1Norms(N, (1, 2), float(lams[k])),
                     GradientOp((512, 512), 1, scheme="forward"))
            t.cuda.synchronize()
            t0 = time.perf_counter()
            kw = {}
            if warm:
                x0, y0 = net.predict(t.from_numpy(fs[k:k + 1]).cuda(),
                                     t.tensor([float(lams[k])], device="cuda"))
                kw["continue_at"] = (x0.view(-1).cpu().numpy().astype(np.float64),
                                     y0.view(-1).cpu().numpy().astype(np.float64))
            s.solve(steps="precond", precision="float", term_pd_gap=1e-4, term_maxiter=20000,
                    granularity=10, **kw)
            t.cuda.synchronize()
            rec[warm] = (1e3 * (time.perf_counter() - t0), s.info["iter"])
        rows.append(rec)
    res["single_image_fused_relgap_1e-4"] = {
        "images": len(rows),
        "plain_ms_mean": round(float(np.mean([r[False][0] for r in rows])), 2),
        "warm_ms_mean": round(float(np.mean([r[True][0] for r in rows])), 2),
        "plain_iters_mean": float(np.mean([r[False][1] for r in rows])),
        "warm_iters_mean": float(np.mean([r[True][1] for r in rows])),
        "note": "wall time of PDHG.solve from host data incl. set-up; warm includes the network "
                "forward of that image and the proposal's round trip through the host"}
    B, S = 32, 512
    f, lam = instances(range(B), S)
    fd, ld = t.from_numpy(f).cuda(), t.from_numpy(lam).cuda()
    for _ in range(3):
        net.forward(fd, ld, keep=False)
    e0, e1 = t.cuda.Event(enable_timing=True), t.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(5):
        net.forward(fd, ld, keep=False)
    e1.record()
    t.cuda.synchronize()
    fwd_s = e0.elapsed_time(e1) / 1e3 / 5
    peak = measured_peaks().get("bf16_tflops")
    layer_s, layer_fl = net.time_conv("d0", B, S)
    res["network"] = {"batch": B, "forward_ms": round(1e3 * fwd_s, 3), "mode": "inference",
                      "forward_conv_TFLOPs": round(net.conv_flops(B, S) / fwd_s / 1e12, 1),
                      "largest_layer": "d0 (64 -> 32 channels at 512^2)",
                      "layer_us": round(1e6 * layer_s, 1),
                      "layer_TFLOPs": round(layer_fl / layer_s / 1e12, 1),
                      "layer_frac_of_measured_bf16": round(layer_fl / layer_s / 1e12 / peak, 3)
                      if peak else None}
    net.check_fault()
    return res


def ssn_case(a, newton_steps=3):
    """Semismooth Newton (the reference's CPU-only method, here on the
    device) on 256^2 gray ROF (lambda = 0.1, centered gradient as the
    reference default) from 300 preconditioned PDHG iterations: time per
    Newton step and CG iterations, beside the oracle's CPU restatement of one
    step on the host (the reference's own code is numpy on one core)."""
    import oracle
    from oracle.ssn import SemismoothNewton as OracleSSN
    from opymize_gb300.gpuarray import torch
    from opymize_gb300.functionals import SSD, L1Norms
    from opymize_gb300.linear import GradientOp
    from opymize_gb300.solvers import PDHG, SemismoothNewton
    from opymize_gb300.tools.synthetic import piecewise_constant
    t = torch()
    dims = (256, 256)
    N = dims[0] * dims[1]
    f = piecewise_constant(dims, 1, sigma=0.1, seed=a.seed)
    p = PDHG(SSD(f.reshape(N, 1)), L1Norms(N, (1, 2), 0.1), GradientOp(dims, 1))
    p.solve(steps="precond", precision="double", term_pd_gap=1e-300, term_maxiter=300,
            granularity=300)
    start = np.concatenate([v.ravel() for v in p.state])
    s = SemismoothNewton(SSD(f.reshape(N, 1)), L1Norms(N, (1, 2), 0.1), GradientOp(dims, 1))
    np.random.seed(1)
    t.cuda.synchronize()
    t0 = time.perf_counter()
    info = s.solve(continue_at=start.copy(), granularity=newton_steps, term_relgap=1e-300,
                   term_maxiter=newton_steps)
    t.cuda.synchronize()
    gpu_s = (time.perf_counter() - t0) / newton_steps
    o = OracleSSN(f, 0.1, oracle.Gradient(dims, 1, "centered"), 2)
    t0 = time.perf_counter()
    o.solve(start, 1)
    cpu_s = time.perf_counter() - t0
    return {"workload": "semismooth Newton, ROF 256^2 gray, lambda 0.1, FP64, from 300 precond PDHG "
                        "iterations", "newton_steps": newton_steps,
            "gpu_s_per_step": round(gpu_s, 4), "cg_iters": s.cg_iters,
            "relgap_start": p.info["relgap"], "relgap_after": info["relgap"],
            "cpu_oracle_s_per_step": round(cpu_s, 3),
            "note": "per step: normest once per solve, one CG solve (3 FP64 device inner products "
                    "per CG iteration read by the host), Armijo search"}


def guarded(case, a):
    """One extra workload's record, or the error that stopped it: the
    headline line does not depend on the other configurations."""
    try:
        return case(a)
    except Exception as err:          # noqa: BLE001
        return {"error": "%s: %s" % (type(err).__name__, str(err)[:300])}


def e2e_solve(a, f):
    """The public-API call a user makes, host data in and out."""
    from opymize_gb300.functionals import SSD, HuberL1Norms
    from opymize_gb300.linear import GradientOp
    from opymize_gb300.solvers import PDHG
    from opymize_gb300.gpuarray import torch
    n, C = a.size, a.channels
    N = n * n
    s = PDHG(SSD(f.reshape(N, C)), HuberL1Norms(N, (C, 2), a.lbd, a.huber),
             GradientOp((n, n), C, scheme="forward"))
    t0 = time.perf_counter()
    s.solve(steps="precond", precision="float", term_pd_gap=a.tol, granularity=a.gran)
    x, y = s.state
    torch().cuda.synchronize()
    dt = time.perf_counter() - t0
    # the solver and its host results are dropped before the next call, as a
    # caller that consumes them would
    return dt, None, x.nbytes + y.nbytes


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return {}


def profile_traffic():
    """Per-launch DRAM bytes of the fused kernels from the committed ncu
    summaries (profiles/*.txt lines `traffic_bytes_per_launch <kernel> <bytes>`)."""
    out = {}
    pdir = os.path.join(ROOT, "profiles")
    try:
        names = sorted(os.listdir(pdir))
    except OSError:
        return out
    for fn in names:
        if not fn.endswith(".txt"):
            continue
        for line in open(os.path.join(pdir, fn)):
            if line.startswith("traffic_bytes_per_launch"):
                _, name, val = line.split()
                out[name] = float(val)
    return out


def cpu_sample(a, f):
    """One whole solve of the oracle (CPU port of the reference, FP64, every
    host thread) on the same input, wall clock: set-up, iterations, gaps."""
    so = cpu_solver(a, f)
    t0 = time.perf_counter()
    info = so.solve(term_pd_gap=a.tol, term_maxiter=100000, granularity=a.gran)
    dt = time.perf_counter() - t0
    so.close()
    return dt * 1e3, int(info["iter"]), so.threads


def run_gpu_arm(a, world, rank, local):
    from opymize_gb300.gpuarray import torch
    t = torch()
    t.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=t.device("cuda", local))
    f = make_image(a)
    rs = ResidentSolver(a, f)
    s = t.cuda.current_stream()
    e0, e1 = t.cuda.Event(enable_timing=True), t.cuda.Event(enable_timing=True)
    # the sampler starts before the warm-up (nvidia-smi takes a while to give
    # its first line); only samples inside the timed region are kept
    with ClockSampler(local) as clk:
        for _ in range(max(3, a.warmup)):
            rs.solve()
        launches0 = rs.launches
        if dist:
            dist.barrier()
        t.cuda.synchronize()
        t_start = clk.mark()
        e0.record(s)
        for _ in range(a.steps):
            rs.solve()
        e1.record(s)
        t.cuda.synchronize()
        t_end = clk.mark()
        if dist:
            dist.barrier()
    clocks = clk.summary(t_start, t_end)
    ms = e0.elapsed_time(e1) / a.steps
    launches = rs.launches - launches0
    if dist:
        v = t.tensor([ms], device="cuda")
        dist.all_reduce(v, op=dist.ReduceOp.MAX)
        ms = float(v.item())

    # roofline of the dominant kernel: the single-sweep iteration (precond:
    # no step-size arrays; xbar stays on chip), with the two passes it
    # replaces timed beside it
    C, K, N = rs.C, rs.K, rs.N
    tS = rs.time_pass(3)
    tA, tB = rs.time_pass(0), rs.time_pass(1)
    bytesS = 4.0 * N * (3 * C + 2 * K)
    peaks = measured_peaks()
    peak = peaks.get("hbm_gbs")
    peak_src = "measured" if peak else "fallback"
    peak = peak or 6800.0
    ach = bytesS / tS / 1e9
    two_pass_bytes = 4.0 * N * (5 * C + 3 * K)
    roof = {"bound": "hbm", "kernel": "k_sweep (one PDHG iteration)",
            "achieved": round(ach, 1), "peak": peak, "peak_source": peak_src, "unit": "GB/s",
            "frac": round(ach / peak, 4), "traffic": profile_traffic().get("sweep"),
            "algorithmic_bytes_per_launch": bytesS,
            "sweep_us": round(tS * 1e6, 2),
            "two_pass": {"passA_us": round(tA * 1e6, 2), "passB_us": round(tB * 1e6, 2),
                         "algorithmic_bytes": two_pass_bytes,
                         "GBps": round(two_pass_bytes / (tA + tB) / 1e9, 1)},
            "speedup_vs_two_pass": round((tA + tB) / tS, 3)}

    # e2e through the public API (rank-local)
    e2e_times = []
    for _ in range(2):
        e2e_solve(a, f)                      # warm
    for _ in range(max(1, min(a.steps, 3))):
        dt, s_api, d2h = e2e_solve(a, f)
        e2e_times.append(dt)
    h2d = f.nbytes          # the FP64 host image; the zero start point is filled on the device
    e2e_ms = float(np.median(e2e_times) * 1e3)
    if dist:
        v = t.tensor([e2e_ms], device="cuda")
        dist.all_reduce(v, op=dist.ReduceOp.MAX)
        e2e_ms = float(v.item())

    # with several ranks the batched configuration is split across them (every
    # rank takes part in the one gather of its stats)
    batch_rec = guarded(lambda aa: batch_case(aa, world, rank), a) \
        if world > 1 and not a.no_extra else None
    out = None
    if rank == 0:
        out = {
            "metric": METRIC, "value": round(ms, 4), "unit": UNIT, "n_gpus": world,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": round(ms, 4),
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded piecewise-constant image + noise)",
            "config": workload_config(a, world),
            "iters_to_gap": rs.iters, "final_relgap": rs.relgap,
            "e2e": {"value": round(e2e_ms, 4), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h),
                    "api": "PDHG(SSD, HuberL1Norms, GradientOp).solve(use_gpu=True, "
                           "steps='precond', precision='float')"},
            "roofline": roof,
            "clocks": clocks,
            "gpu_launches": int(launches),
        }
        if world > 1 and not a.no_extra:
            out["other_workloads"] = {"batched_512_instances": batch_rec}
        if world == 1 and not a.no_extra:
            # the other configurations of the path, outside the headline metric
            del rs
            out["other_workloads"] = {"gray_2048x2048": guarded(gray_case, a),
                                      "volume_256x256x256": guarded(volume_case, a),
                                      "sublabel_512x512_L16": guarded(sublabel_case, a),
                                      "batched_512_instances": guarded(batch_case, a),
                                      "warm_start_512x512": guarded(warm_start_case, a),
                                      "semismooth_newton_256x256": guarded(ssn_case, a)}
        if world == 1 and not a.no_cpu:
            cpu_ms, cpu_iters, thr = cpu_sample(a, f)
            out["cpu_baseline"] = {
                "value": round(cpu_ms, 1), "unit": UNIT, "cores": thr, "kind": "port",
                "sample": "one whole solve of the oracle (numpy/scipy port of the reference CPU "
                          "PDHG, FP64) on the same %dx%dx%d input from a zero start to relgap %g "
                          "(%d iterations, gap every %d), array operations split over %d host "
                          "threads" % (a.size, a.size, a.channels, a.tol, cpu_iters, a.gran, thr),
                "host_cpus": os.cpu_count()}
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return out


# ------------------------------------------------------------ reference arm
def cpu_solver(a, f, dims=None, lbd=None, huber=None):
    """The oracle's PDHG (numpy/scipy port of the reference's CPU solver,
    FP64) over every host thread (oracle.threaded: pixel ranges of each
    array operation on a thread pool; same iterates as the one-thread port)."""
    from oracle.threaded import ThreadedROF
    dims = (a.size, a.size) if dims is None else tuple(dims)
    return ThreadedROF(f.reshape(-1, f.shape[-1]), dims, a.lbd if lbd is None else lbd,
                       a.huber if huber is None else huber)


def run_reference_arm(a, world, rank):
    """Each step is one whole CPU solve to the gap (set-up, iterations and
    gap checks, as a caller of solve() sees it), timed on the wall clock."""
    if rank != 0:
        return None
    f = make_image(a)
    so = cpu_solver(a, f)
    times, iters = [], None
    for k in range(a.warmup + a.steps):
        t0 = time.perf_counter()
        info = so.solve(term_pd_gap=a.tol, term_maxiter=100000, granularity=a.gran)
        dt = time.perf_counter() - t0
        iters = int(info["iter"])
        if k >= a.warmup:
            times.append(dt)
    so.close()
    ms = float(np.mean(times)) * 1e3
    return {
        "metric": METRIC, "value": round(ms, 1), "unit": UNIT, "n_gpus": world,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": round(ms, 1),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded piecewise-constant image + noise)",
        "config": workload_config(a, world), "impl": "reference",
        "iters_to_gap": iters, "final_relgap": info["relgap"],
        "step_ms_min_max": [round(1e3 * min(times), 1), round(1e3 * max(times), 1)],
        "cpu_baseline": {"value": round(ms, 1), "unit": UNIT, "cores": so.threads, "kind": "port",
                         "sample": "each step: one whole solve of the oracle (numpy/scipy port of "
                                   "the reference CPU PDHG, FP64) on the full input from a zero "
                                   "start to relgap %g: set-up, %d iterations, %d gap checks; "
                                   "array operations split over %d host threads"
                                   % (a.tol, iters, iters // a.gran, so.threads),
                         "host_cpus": os.cpu_count()},
        "e2e": {"value": round(ms, 1), "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def relaunch_ranks(n):
    """`bench.py --gpus N` started as one process: run it again as N ranks
    (one per GPU) under torch.distributed.run on 127.0.0.1, and return their
    exit status.  Rank 0 prints the line."""
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
           "--nproc-per-node=%d" % n, "--master-addr=127.0.0.1", "--master-port=%d" % port,
           os.path.abspath(__file__)] + sys.argv[1:]
    env = dict(os.environ, MASTER_ADDR="127.0.0.1")
    return subprocess.call(cmd, env=env)


def main():
    a = parse()
    if a.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(relaunch_ranks(a.gpus))
    world, rank, local = dist_setup()
    if "WORLD_SIZE" in os.environ and world != a.gpus:
        raise SystemExit("bench.py: --gpus %d but WORLD_SIZE=%d" % (a.gpus, world))
    if a.impl == "reference":
        out = run_reference_arm(a, world, rank)
    else:
        out = run_gpu_arm(a, world, rank, local)
    if out is not None:
        print(json.dumps(out))
        sys.stdout.flush()


if __name__ == "__main__":
    main()
