"""Batched ROF-type solves: many independent images, one launch per iteration.

The reference solves one problem per `PDHG` object (opymize/solvers/pdhg.py:
229-315); workloads of many images (a data set, tiles of a mosaic) then pay a
full solver set-up and a chain of small launches per image.  `BatchROF` runs
the fused single-sweep iteration of every active image in one launch (the
images' tiles form one work list), evaluates every image's gap in one launch
pair, and retires each image as soon as its own stop test passes (the
reference's test, pdhg.py:290-305).  The arithmetic per pixel is that of the
single-image fused path, so an image's iterates are identical to its own
`PDHG.solve(steps="precond", precision="float")` run.

Restrictions (those of the single sweep): 2-D images whose last axis is a
multiple of 4, one channel count for the whole batch, FP32, preconditioned
steps.  The gap check interval must be even (iterations run in pairs).
"""

import time

import numpy as np

from opymize_gb300 import _lib
from opymize_gb300.gpuarray import DeviceArray, stream_ptr, torch
from opymize_gb300.functionals import SSD, L1Norms, HuberL1Norms
from opymize_gb300.linear import GradientOp
from opymize_gb300.solvers.pdhg import PDHG, INFO_KEYS


class BatchROF(object):
    """min_x 0.5*|x - f_i|^2 + lbd_i * TV(x) (Huber-smoothed with alpha > 0)
    for every image f_i of `images` ((H, W) or (H, W, C) arrays)."""

    ROWS_CANDIDATES = (8, 16, 32, 64)

    GRAN_RANGE = (10, 100)
    GRAN_PRIOR_ITERS = 1000   # iterations an instance is assumed to need when tuning the interval
    PERSIST_MARGIN = 1.1      # persistent kept unless the graphs' full iteration is this much faster

    def __init__(self, images, lbd, huber=0.0, tol=1e-4, granularity=10, rows_per_item=None,
                 persistent=None):
        if not images:
            raise ValueError("empty batch")
        self.n = len(images)
        lbds = np.broadcast_to(np.asarray(lbd, dtype=np.float64), (self.n,))
        self.tol = float(tol)
        # granularity=None: the interval between stop tests is tuned with the rows per item
        self.gran_auto = granularity is None
        g = 10 if granularity is None else int(granularity)
        self.gran = g + (g & 1)   # iterations run in pairs
        self.rows_per_item = rows_per_item
        self.class_streams = True    # width classes on separate streams inside the graphs
        self._persistent_req = persistent
        lib = _lib.load()
        self.problems = (_lib.opyx_rof_problem * self.n)()
        self.buffers = (_lib.opyx_rof_buffers * self.n)()
        self.dims, self.arrays = [], []
        C = None
        for i, img in enumerate(images):
            img = np.asarray(img)
            img = img[..., None] if img.ndim == 2 else img
            if img.ndim != 3:
                raise ValueError("images must be 2-D (optionally with a channel axis)")
            H, W, Ci = img.shape
            C = Ci if C is None else C
            if Ci != C:
                raise ValueError("all images of a batch need the same channel count")
            if W % 4:
                raise ValueError("the last axis of every image must be a multiple of 4")
            N = H * W
            F = HuberL1Norms(N, (C, 2), lbds[i], huber) if huber > 0 else L1Norms(N, (C, 2), lbds[i])
            s = PDHG(SSD(img.reshape(N, C)), F, GradientOp((H, W), C, scheme="forward"))
            s.constvars.update(theta=1.0, precond=True)
            p = s._rof_problem(np.float32, "precond")
            p.term_mode = 1
            p.term_relgap = p.term_infeas = self.tol
            self.problems[i] = p
            arr = dict(x=DeviceArray.zeros((N * C,), np.float32),
                       y=DeviceArray.zeros((N * 2 * C,), np.float32),
                       xbar=DeviceArray.empty((N * C,), np.float32),
                       y2=DeviceArray.empty((N * 2 * C,), np.float32),
                       f=s.g.f_dev(np.float32))
            b = self.buffers[i]
            b.x, b.xbar, b.y, b.y2, b.f = (arr[k].ptr for k in ("x", "xbar", "y", "y2", "f"))
            self.arrays.append(arr)
            self.dims.append((H, W, C))
        self.C = C
        # one channel: the whole solve in one persistent launch or chains of
        # per-iteration launches captured in graphs, whichever the autotuner
        # times faster (persistent until then); more channels: graphs
        self.persistent = (C == 1) if persistent is None else bool(persistent)
        if self.persistent and C != 1:
            raise ValueError("the persistent batched solve takes one-channel images")
        self.rec_bytes = lib.opyx_rof_batch_record_bytes()
        self.records = DeviceArray.zeros((self.n * self.rec_bytes // 8,), np.float64)
        self.launches = 0
        self.info = []

    @classmethod
    def check_interval(cls, t_gap, t_iter):
        """Iterations between stop tests for a test costing t_gap and an
        iteration costing t_iter (any one time unit): g = sqrt(2 n t_gap /
        t_iter) for n = GRAN_PRIOR_ITERS, rounded, made even (iterations run
        in pairs) and clipped to GRAN_RANGE."""
        g = int(round(np.sqrt(2.0 * cls.GRAN_PRIOR_ITERS * t_gap / max(t_iter, 1e-9))))
        return int(np.clip(g + (g & 1), *cls.GRAN_RANGE))

    # ------------------------------------------------------------ plumbing
    def _describe(self, active, rows):
        lib = _lib.load()
        act = np.ascontiguousarray(active, dtype=np.uint8)
        nitems = _lib.C.c_int(0)
        # a first call without a buffer returns the item count to size it
        st = lib.opyx_rof_batch_describe(self.problems, self.buffers, self.n, self.records.ptr,
                                         act.ctypes.data, int(rows), None, 0, _lib.C.byref(nitems))
        if st not in (_lib.OPYX_OK, _lib.OPYX_ERR_WORKSPACE):
            raise _lib.OpyxError("opyx_rof_batch_describe", st, _lib.status_string(st))
        nbytes = lib.opyx_rof_batch_desc_bytes(self.n, nitems.value)
        t = torch()
        # pinned host copy, uploaded without a synchronisation: chunks queued
        # on the stream keep running on the previous descriptor (its device
        # copy stays alive in their graphs' tuples) while this one is built
        pinned = t.zeros(nbytes, dtype=t.uint8, pin_memory=True)
        host = pinned.numpy()
        _lib.call("opyx_rof_batch_describe", self.problems, self.buffers, self.n,
                  self.records.ptr, act.ctypes.data, int(rows), host.ctypes.data, nbytes,
                  _lib.C.byref(nitems))
        cb = host[16:32].view(np.int32)              # the header's class_beg[0..3]
        self._classes = int(np.count_nonzero(np.diff(cb)))
        self._class_ids = [c for c in range(3) if cb[c + 1] > cb[c]]
        dev = t.empty(nbytes, dtype=t.uint8, device="cuda")
        dev.copy_(pinned, non_blocking=True)
        part = DeviceArray.empty((max(1, nitems.value) * 5,), np.float64)
        return (host, dev, pinned), nitems.value, part

    def _reset(self):
        for arr in self.arrays:
            arr["x"].fill(0.0)
            arr["y"].fill(0.0)

    def _iterate(self, desc, nitems, n):
        _lib.call("opyx_rof_batch_iterate", desc[0].ctypes.data, desc[1].data_ptr(), n,
                  stream_ptr())
        self.launches += n * self._classes

    def _gap(self, desc, nitems, part):
        _lib.call("opyx_rof_batch_gap", desc[0].ctypes.data, desc[1].data_ptr(), part.ptr,
                  stream_ptr())
        self.launches += 2

    def _init(self, desc):
        _lib.call("opyx_rof_batch_init", desc[0].ctypes.data, desc[1].data_ptr(), stream_ptr())
        self.launches += 1

    # ------------------------------------------------- persistent solve
    def _persist(self, desc, gran, maxiter):
        """One cooperative launch: `maxiter` (even) iterations of every active
        image with a gap check every `gran` (even) iterations, images retiring
        on the device; returns the control record (error, active, strips,
        iterations at the last check) once the launch has finished."""
        lib = _lib.load()
        wsb = lib.opyx_rof_batch_persist_ws_bytes(desc[0].ctypes.data)
        if getattr(self, "_pws", None) is None or self._pws.size * 8 < wsb:
            self._pws = DeviceArray.zeros(((wsb + 7) // 8,), np.float64)
        _lib.call("opyx_rof_batch_persist", desc[0].ctypes.data, desc[1].data_ptr(),
                  self._pws.ptr, int(gran), int(maxiter), stream_ptr())
        self.launches += 2            # the control block's memset and the solve
        ctl = self._pws.t[:6].cpu().numpy().view(np.int32)
        # (arrive: u64, grab[4]: u32, error, nact, nwork, iters, rows, nwork_gap: i32)
        error, nact, nwork, iters, rows = (int(v) for v in ctl[6:11])
        if error:
            raise _lib.OpyxError("opyx_rof_batch_persist", _lib.OPYX_ERR_LAUNCH,
                                 "a grid barrier of the persistent solve timed out")
        return {"active": nact, "items": nwork, "iters": iters, "item_rows": rows}

    def _autotune_persistent(self, iters):
        t = torch()
        best = None
        active = np.ones(self.n, np.uint8)
        big = 1 << 30                 # no gap check within the timed iterations
        for rows in self.ROWS_CANDIDATES:
            desc, _, _ = self._describe(active, rows)
            self._init(desc)
            self._persist(desc, big, 2)   # warm
            e0, e1 = t.cuda.Event(enable_timing=True), t.cuda.Event(enable_timing=True)
            e0.record()
            self._persist(desc, big, iters)
            e1.record()
            t.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            if best is None or ms < best[0]:
                best = (ms, rows, desc)
        self.rows_per_item = best[1]
        t_it = best[0] / iters
        self.tuning = {"rows_per_item": best[1], "ms_per_iteration": t_it}
        if self.gran_auto:
            desc = best[2]
            e0, e1 = t.cuda.Event(enable_timing=True), t.cuda.Event(enable_timing=True)
            self._init(desc)
            e0.record()
            self._persist(desc, 2, 2)      # two iterations and one gap check
            e1.record()
            t.cuda.synchronize()
            t_gap = max(e0.elapsed_time(e1) - 2 * t_it, 1e-3)
            g = self.check_interval(t_gap, t_it)
            self.gran = g
            self.tuning.update(ms_per_gap=t_gap, granularity=g)
        self._reset()
        return best[1]

    def _solve_persistent(self, maxiter):
        active = np.ones(self.n, np.uint8)
        desc, _, _ = self._describe(active, self.rows_per_item)
        self._init(desc)
        t = torch()
        t0 = time.perf_counter()
        m = maxiter + (maxiter & 1)
        self.persist_ctl = self._persist(desc, self.gran, m)
        t.cuda.synchronize()
        self.elapsed = time.perf_counter() - t0
        return self._read_info(maxiter)

    def _read_info(self, maxiter):
        names = _lib.ROF_INFO_FIELDS
        nrec = self.rec_bytes // 8
        i_done, i_fault = names.index("done"), names.index("fault")
        i_checks = names.index("checks")
        off = 256 // 8
        final = self.records.get().reshape(self.n, nrec)[:, off:off + len(names)]
        if (final[:, i_fault] != 0).any():
            raise _lib.OpyxError("batched PDHG iteration", _lib.OPYX_ERR_LAUNCH,
                                 "a kernel gave up waiting for its own copies")
        self.info = []
        for i in range(self.n):
            d = {k: float(final[i, names.index(k)]) for k in INFO_KEYS}
            d["iter"] = int(min(maxiter, round(final[i, i_checks]) * self.gran))
            d["converged"] = bool(final[i, i_done] != 0)
            self.info.append(d)
        return self.info

    def autotune(self, iters=4):
        """Rows per work item (and the check interval with granularity=None);
        for one-channel batches whose mode was not fixed by `persistent`,
        also the mode: the persistent launch and the graph-captured
        per-iteration launches are both tuned and the faster iteration over
        the whole batch is kept, the persistent launch unless the graphs'
        iteration is more than PERSIST_MARGIN times faster (the persistent
        launch won on a batch of 512 mixed sizes, the graphs on 32 equal
        512^2 images)."""
        if self._persistent_req is None and self.C == 1:
            self.persistent = True
            rp = self._autotune_persistent(iters)
            tp = dict(self.tuning)
            gp = self.gran
            self.persistent = False
            rg = self._autotune_graphs(iters)
            tg = dict(self.tuning)
            # the tuning times iterations with every instance active; the
            # persistent launch gains in the tail (no per-check host round
            # trips or descriptor rebuilds: 512 mixed instances 3.89 s against
            # 4.03 s with graphs at 0.756 against ~0.74 ms per full iteration),
            # so it is kept unless the graphs are clearly faster
            if tp["ms_per_iteration"] <= self.PERSIST_MARGIN * tg["ms_per_iteration"]:
                self.persistent, self.rows_per_item, self.tuning, self.gran = True, rp, tp, gp
            self.tuning["mode"] = "persistent" if self.persistent else "graphs"
            self.tuning["ms_per_iteration_other_mode"] = (
                tg if self.persistent else tp)["ms_per_iteration"]
            return self.rows_per_item
        if self.persistent:
            return self._autotune_persistent(iters)
        return self._autotune_graphs(iters)

    def _autotune_graphs(self, iters=4):
        """Rows per work item: each candidate runs `iters` iterations from the
        zero start, timed with CUDA events; the fastest is kept and the state
        reset (the tuning iterations do not count).  With granularity=None
        the interval g between stop tests is chosen too: a test costs t_gap
        and an instance runs on average g/2 iterations past its stop, so g
        minimises t_gap/g + t_iter g/(2 n) for n = GRAN_PRIOR_ITERS, i.e.
        g = sqrt(2 n t_gap / t_iter), even, within GRAN_RANGE."""
        t = torch()
        best = None
        active = np.ones(self.n, np.uint8)
        for rows in self.ROWS_CANDIDATES:
            desc, nitems, part = self._describe(active, rows)
            self._init(desc)
            self._iterate(desc, nitems, 2)            # warm
            e0, e1 = t.cuda.Event(enable_timing=True), t.cuda.Event(enable_timing=True)
            e0.record()
            self._iterate(desc, nitems, iters)
            e1.record()
            t.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            if best is None or ms < best[0]:
                best = (ms, rows, desc, nitems, part)
        self.rows_per_item = best[1]
        self.tuning = {"rows_per_item": best[1], "ms_per_iteration": best[0] / iters}
        if self.gran_auto:
            _, _, desc, nitems, part = best
            self._gap(desc, nitems, part)             # warm
            e0, e1 = t.cuda.Event(enable_timing=True), t.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(3):
                self._gap(desc, nitems, part)
            e1.record()
            t.cuda.synchronize()
            t_gap = e0.elapsed_time(e1) / 3
            t_it = best[0] / iters
            g = self.check_interval(t_gap, t_it)
            self.gran = g
            self.tuning.update(ms_per_gap=t_gap, granularity=g)
        self._reset()
        return best[1]

    # ---------------------------------------------------------------- solve
    DEPTH = 2     # chunks queued ahead of the host's reads

    def _capture(self, desc, nitems, part, n, slot):
        """`n` iterations, the gap and the copy of the info records into
        pinned slot `slot`, captured into one CUDA graph (on a private capture
        stream) for the current active set."""
        t = torch()
        stream = t.cuda.Stream()
        graph = t.cuda.CUDAGraph()
        stream.wait_stream(t.cuda.current_stream())
        with t.cuda.graph(graph, stream=stream):
            if len(self._class_ids) > 1 and self.class_streams:
                # the classes' instances are disjoint: one chain of iterations
                # per class on its own stream, joined before the gap
                if not hasattr(self, "_side"):
                    self._side = [t.cuda.Stream() for _ in range(3)]
                fork = t.cuda.Event()
                fork.record(stream)
                joins = []
                for c in self._class_ids:
                    side = self._side[c]
                    side.wait_event(fork)
                    with t.cuda.stream(side):
                        _lib.call("opyx_rof_batch_iterate_class", desc[0].ctypes.data,
                                  desc[1].data_ptr(), c, n, stream_ptr())
                        ev = t.cuda.Event()
                        ev.record(side)
                        joins.append(ev)
                for ev in joins:
                    stream.wait_event(ev)
            else:
                self._iterate(desc, nitems, n)
            self._gap(desc, nitems, part)
            self._pinned[slot].copy_(self.records.t, non_blocking=True)
        return graph

    def solve(self, maxiter=5000, init=None, graph=True):
        """Iterate until every image passed its stop test or `maxiter`
        iterations; returns per image a dict with the reference's info keys
        and `iter`.  States: `self.state(i)` (x as an (H, W, C) array),
        `self.dual(i)` (y as (H, W, 2, C)).  `init`: optional starting
        points, a sequence of (x, y) per image (device tensors or arrays of
        N*C and N*2*C values; the reference's `continue_at`,
        opymize/solvers/pdhg.py:254-255); zero otherwise.

        Chunks of `granularity` iterations + gap are captured into CUDA
        graphs per active set and queued DEPTH ahead of the host's reads:
        the device-side stop test makes the kernels skip finished images, so
        chunks queued past an image's stop leave it alone, and its iteration
        count comes from its device check counter."""
        if self.rows_per_item is None:
            self.autotune()
        self._reset()
        if init is not None:
            t = torch()
            for arr, (x0, y0) in zip(self.arrays, init):
                for key, v in (("x", x0), ("y", y0)):
                    src = v if hasattr(v, "data_ptr") else t.from_numpy(
                        np.ascontiguousarray(v, dtype=np.float32))
                    arr[key].t.copy_(src.reshape(-1))
        if self.persistent:
            return self._solve_persistent(maxiter)
        t = torch()
        names = _lib.ROF_INFO_FIELDS
        nrec = self.rec_bytes // 8
        i_done, i_fault = names.index("done"), names.index("fault")
        i_checks = names.index("checks")
        off = 256 // 8
        self._pinned = [t.empty(self.records.t.shape, dtype=self.records.t.dtype,
                                pin_memory=True) for _ in range(self.DEPTH)]
        active = np.ones(self.n, np.uint8)
        desc, nitems, part = self._describe(active, self.rows_per_item)
        described = active.copy()
        self._pix = np.array([H * W for H, W, _ in self.dims], dtype=np.int64)
        self._init(desc)
        gran = self.gran
        graphs = None
        t0 = time.perf_counter()
        launched = 0          # iterations queued
        pending = []          # (slot, event, iterations after the chunk)
        chunks = 0
        last = None
        while True:
            while len(pending) < self.DEPTH and launched < maxiter and active.any():
                n = min(gran, maxiter - launched)
                n += n & 1
                slot = chunks % self.DEPTH
                if graph and n == gran:
                    if graphs is None:
                        graphs = [self._capture(desc, nitems, part, gran, k)
                                  for k in range(self.DEPTH)]
                    graphs[slot].replay()
                    self.launches += n * self._classes + 2
                else:
                    self._iterate(desc, nitems, n)
                    self._gap(desc, nitems, part)
                    self._pinned[slot].copy_(self.records.t, non_blocking=True)
                ev = t.cuda.Event()
                ev.record()
                launched += n
                pending.append((slot, ev, launched))
                chunks += 1
            if not pending:
                break
            slot, ev, it = pending.pop(0)
            ev.synchronize()
            last = self._pinned[slot].numpy().reshape(self.n, nrec)[:, off:off + len(names)].copy()
            if (last[:, i_fault] != 0).any():
                raise _lib.OpyxError("batched PDHG iteration", _lib.OPYX_ERR_LAUNCH,
                                     "a kernel gave up waiting for its own copies")
            done = (last[:, i_done] != 0) & (active != 0)
            if done.any():
                active[done] = 0
                # finished images are skipped on the device, so the descriptor
                # is rebuilt only once a tenth of its pixels have finished;
                # chunks already queued keep the previous one
                gone = self._pix[(described != 0) & (active == 0)].sum()
                if active.any() and gone >= 0.1 * self._pix[described != 0].sum():
                    desc, nitems, part = self._describe(active, self.rows_per_item)
                    described = active.copy()
                    graphs = None
        t.cuda.synchronize()
        self.elapsed = time.perf_counter() - t0
        final = self.records.get().reshape(self.n, nrec)[:, off:off + len(names)]
        self.info = []
        for i in range(self.n):
            d = {k: float(final[i, names.index(k)]) for k in INFO_KEYS}
            d["iter"] = int(min(maxiter, round(final[i, i_checks]) * gran))
            d["converged"] = bool(final[i, i_done] != 0)
            self.info.append(d)
        return self.info

    def state(self, i):
        H, W, C = self.dims[i]
        return self.arrays[i]["x"].get().reshape(H, W, C)

    def dual(self, i):
        H, W, C = self.dims[i]
        return self.arrays[i]["y"].get().reshape(H, W, 2, C)

    def pixels(self):
        return sum(H * W for H, W, _ in self.dims)


def shard(sizes, rank, world):
    """Indices of the instances rank `rank` of `world` solves: instances are
    independent, so the batch splits across GPUs with no collective on the
    data path.  Greedy by size (largest first onto the least loaded rank, ties
    to the lower rank), deterministic on every rank."""
    sizes = np.asarray(sizes, dtype=np.int64)
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    load = np.zeros(world, dtype=np.int64)
    owner = np.empty(len(sizes), dtype=np.int64)
    for i in sorted(range(len(sizes)), key=lambda k: (-int(sizes[k]), k)):
        r = int(np.argmin(load))
        owner[i] = r
        load[r] += sizes[i]
    return [i for i in range(len(sizes)) if owner[i] == rank]


def gather_stats(stats, group=None):
    """The one collective of a sharded batch: every rank's stats (a
    picklable object, e.g. {instance index: info}) gathered on all ranks;
    without an initialised process group, [stats]."""
    try:
        import torch.distributed as dist
    except ImportError:
        return [stats]
    if not dist.is_available() or not dist.is_initialized():
        return [stats]
    out = [None] * dist.get_world_size(group)
    dist.all_gather_object(out, stats, group=group)
    return out


def _main(argv=None):
    """A seeded mixed-size batch (sides log-uniform in [64, 1024], aspect
    U[0.5, 2], lambda U[0.02, 0.3], sigma U[0.05, 0.2]) solved for a few
    iterations -- a small case for profilers:

        python -m opymize_gb300.solvers.batch --n 96 --maxiter 10
    """
    import argparse
    import json
    from opymize_gb300.tools.synthetic import piecewise_constant
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=96)
    ap.add_argument("--maxiter", type=int, default=10)
    ap.add_argument("--rows", type=int, default=8)
    ap.add_argument("--tol", type=float, default=1e-4)
    a = ap.parse_args(argv)
    rng = np.random.default_rng(0)
    imgs, lbds = [], []
    for k in range(a.n):
        side = np.exp(rng.uniform(np.log(64), np.log(1024)))
        asp = rng.uniform(0.5, 2.0)
        H = max(8, int(round(side)))
        W = max(4, int(round(side * asp / 4)) * 4)
        imgs.append(piecewise_constant((H, W), 1, sigma=rng.uniform(0.05, 0.2), seed=1000 + k))
        lbds.append(rng.uniform(0.02, 0.3))
    b = BatchROF(imgs, lbds, tol=a.tol, granularity=10, rows_per_item=a.rows)
    info = b.solve(maxiter=a.maxiter)
    torch().cuda.synchronize()
    print(json.dumps({"instances": a.n, "pixels": b.pixels(), "launches": b.launches,
                      "iters": max(d["iter"] for d in info)}))


if __name__ == "__main__":
    _main()
