"""Training data, training loop and evaluation of the learned warm start.

Data: seeded synthetic ROF instances (piecewise-constant images, noise
sigma ~ U[0.05, 0.2], lambda ~ U[0.02, 0.3]) solved by the project's own
batched fused PDHG (`BatchROF`, preconditioned steps, FP32 iterates, FP64
gap) to a tight relative gap; the targets are (x* - f, y* / lambda).

Evaluation: held-out seeds solved to relative gap 1e-4 from zero and from
the network's proposal, by the same solver with the same stop test, so the
plain method stays the arbiter of the warm start: a proposal only changes
where the iteration starts, never the accepted gap.
"""

import time

import numpy as np

from opymize_gb300.gpuarray import torch
from opymize_gb300.solvers.batch import BatchROF
from opymize_gb300.tools.synthetic import piecewise_constant

SIGMA_RANGE = (0.05, 0.2)
LAMBDA_RANGE = (0.02, 0.3)


def instance(seed, S=512):
    """One seeded instance: (f (S, S) float32, lambda)."""
    rng = np.random.default_rng([seed, 7919])
    sigma = rng.uniform(*SIGMA_RANGE)
    lam = float(rng.uniform(*LAMBDA_RANGE))
    f = piecewise_constant((S, S), 1, sigma=sigma, seed=seed)[..., 0].astype(np.float32)
    return f, lam


def instances(seeds, S=512):
    fs, lams = zip(*(instance(s, S) for s in seeds))
    return np.stack(fs), np.asarray(lams, dtype=np.float32)


def solve_batch(f, lam, tol, maxiter, init=None, chunk=256, granularity=10):
    """Solve ROF for the images f (n, S, S) with BatchROF in chunks; returns
    x (n, S, S), y (n, S, S, 2) as device tensors, the per-image info and
    the summed wall time of the solves (set-up excluded)."""
    t = torch()
    n, S = f.shape[0], f.shape[1]
    xs = t.empty(n, S, S, device="cuda")
    ys = t.empty(n, S, S, 2, device="cuda")
    infos = []
    elapsed = 0.0
    for c0 in range(0, n, chunk):
        c1 = min(n, c0 + chunk)
        imgs = [np.asarray(f[i].cpu() if hasattr(f[i], "cpu") else f[i]) for i in range(c0, c1)]
        b = BatchROF(imgs, [float(l) for l in lam[c0:c1]], tol=tol, granularity=granularity)
        ini = None if init is None else [(init[0][i], init[1][i]) for i in range(c0, c1)]
        b.autotune()
        t.cuda.synchronize()
        t0 = time.perf_counter()
        infos += b.solve(maxiter=maxiter, init=ini)
        t.cuda.synchronize()
        elapsed += time.perf_counter() - t0
        for k, i in enumerate(range(c0, c1)):
            xs[i].view(-1).copy_(b.arrays[k]["x"].t)
            ys[i].view(-1).copy_(b.arrays[k]["y"].t)
    return xs, ys, infos, elapsed


def make_dataset(seeds, S=512, tol=1e-5, maxiter=8000, chunk=256, restart=0):
    """Device tensors f (n, S, S), lam (n,), target (n, S, S, 3) and the
    solver infos for the given seeds.  restart=K: the inputs also hold the
    iterate after K plain iterations from zero ("state") and the targets are
    the corrections (x* - x_K, (y* - y_K) / lambda) of that iterate."""
    t = torch()
    f, lam = instances(seeds, S)
    fd = t.from_numpy(f).cuda()
    ld = t.from_numpy(lam).cuda()
    n = len(seeds)
    state = None
    if restart:
        xk, yk, _, _ = solve_batch(f, lam, 1e-300, restart, chunk=chunk)
        xs, ys, infos, _ = solve_batch(f, lam, tol, maxiter, chunk=chunk,
                                       init=(xk.view(n, -1), yk.view(n, -1)))
        state = (xk, yk)
        base_x, base_y = xk, yk
    else:
        xs, ys, infos, _ = solve_batch(f, lam, tol, maxiter, chunk=chunk)
        base_x, base_y = fd, t.zeros_like(ys)
    tgt = t.empty(n, S, S, 3, device="cuda")
    tgt[..., 0] = xs - base_x
    tgt[..., 1:] = (ys - base_y) / ld.view(-1, 1, 1, 1)
    return dict(f=fd, lam=ld, target=tgt, infos=infos, state=state)


def train(net, data, epochs=4, batch=32, lr=1e-3, seed=0, log=None, cosine=True):
    """Adam on the warm-start loss (primal residual, lambda * divergence of
    the dual error, dual error); returns the mean loss of every epoch and
    the median step time (ms)."""
    t = torch()
    n = data["f"].shape[0]
    g = t.Generator(device="cpu").manual_seed(seed)
    losses, step_ms = [], []
    total = epochs * (n // batch)
    step = 0
    for ep in range(epochs):
        perm = t.randperm(n, generator=g)
        tot, cnt = 0.0, 0
        for b0 in range(0, n - batch + 1, batch):
            idx = perm[b0:b0 + batch].cuda()
            f = data["f"].index_select(0, idx)
            lam = data["lam"].index_select(0, idx)
            tgt = data["target"].index_select(0, idx)
            st = None
            if data.get("state") is not None:
                st = (data["state"][0].index_select(0, idx), data["state"][1].index_select(0, idx))
            t.cuda.synchronize()
            t0 = time.perf_counter()
            net.forward(f, lam, state=st)
            loss = net.loss_warm(tgt)
            net.backward()
            # cosine decay of the learning rate over the run
            lr_t = lr * 0.5 * (1.0 + np.cos(np.pi * step / max(1, total))) if cosine else lr
            net.adam_step(lr=lr_t)
            step += 1
            t.cuda.synchronize()
            step_ms.append(1e3 * (time.perf_counter() - t0))
            tot += float(loss)
            cnt += 1
        net.check_fault()
        losses.append(tot / max(1, cnt))
        if log:
            log("epoch %d loss %.5f (%.1f ms/step)" % (ep, losses[-1], np.median(step_ms)))
    return losses, float(np.median(step_ms)) if step_ms else None


def predict(net, f, lam, batch=32, state=None):
    """Network proposals for device tensors f (n, S, S), lam (n,) (and, in
    the restart mode, the iterates state = (x (n, S, S), y (n, S, S, 2)))."""
    t = torch()
    n, S = f.shape[0], f.shape[1]
    x0 = t.empty(n, S, S, device="cuda")
    y0 = t.empty(n, S, S, 2, device="cuda")

    def pad(v, b0, b1):
        v = v[b0:b1].contiguous()
        if b1 - b0 < batch:   # keep one buffer shape: pad the last batch
            v = t.cat([v, v[:1].expand((batch - (b1 - b0),) + tuple(v.shape[1:]))])
        return v

    for b0 in range(0, n, batch):
        b1 = min(n, b0 + batch)
        st = None if state is None else (pad(state[0], b0, b1), pad(state[1], b0, b1))
        xb, yb = net.predict(pad(f, b0, b1), pad(lam, b0, b1), state=st)
        x0[b0:b1] = xb[:b1 - b0]
        y0[b0:b1] = yb[:b1 - b0]
    return x0, y0


def evaluate(net, seeds, S=512, tol=1e-4, maxiter=20000, batch=32):
    """Held-out comparison, zero start vs network start, same solver and
    stop test.  Returns per-image iterations, gaps and wall times."""
    t = torch()
    f, lam = instances(seeds, S)
    fd, ld = t.from_numpy(f).cuda(), t.from_numpy(lam).cuda()
    if getattr(net, "restart", False):
        raise ValueError("use evaluate_restart for a restart-mode network")
    _, _, cold, t_cold = solve_batch(f, lam, tol, maxiter)
    t.cuda.synchronize()
    t0 = time.perf_counter()
    x0, y0 = predict(net, fd, ld, batch=batch)
    t.cuda.synchronize()
    t_net = time.perf_counter() - t0
    n = len(seeds)
    _, _, warm, t_warm = solve_batch(f, lam, tol, maxiter, init=(x0.view(n, -1), y0.view(n, -1)))
    it_c = np.array([d["iter"] for d in cold])
    it_w = np.array([d["iter"] for d in warm])

    return dict(seeds=list(seeds), iters_cold=it_c.tolist(), iters_warm=it_w.tolist(),
                relgap_cold=[d["relgap"] for d in cold], relgap_warm=[d["relgap"] for d in warm],
                converged_cold=int(sum(d["converged"] for d in cold)),
                converged_warm=int(sum(d["converged"] for d in warm)),
                solve_cold_s=t_cold, solve_warm_s=t_warm, net_s=t_net,
                speedup=t_cold / (t_warm + t_net),
                mean_iter_ratio=float(it_c.mean() / max(1.0, it_w.mean())))


def evaluate_restart(net, seeds, K, S=512, tol=1e-4, maxiter=20000, batch=32):
    """The restart mode on held-out seeds: K plain iterations from zero (the
    stop test active), the network's correction of that iterate, then PDHG
    to the same stop test; against the plain solve from zero.  Iterations
    and times include the first K (or fewer) iterations and the network."""
    t = torch()
    f, lam = instances(seeds, S)
    fd, ld = t.from_numpy(f).cuda(), t.from_numpy(lam).cuda()
    n = len(seeds)
    _, _, cold, t_cold = solve_batch(f, lam, tol, maxiter)
    xk, yk, first, t_first = solve_batch(f, lam, tol, K)
    t.cuda.synchronize()
    t0 = time.perf_counter()
    x0, y0 = predict(net, fd, ld, batch=batch, state=(xk, yk))
    t.cuda.synchronize()
    t_net = time.perf_counter() - t0
    _, _, rest, t_rest = solve_batch(f, lam, tol, maxiter, init=(x0.view(n, -1), y0.view(n, -1)))
    it_c = np.array([d["iter"] for d in cold])
    it_w = np.array([d["iter"] for d in first]) + np.array([d["iter"] for d in rest])
    return dict(seeds=list(seeds), K=K, iters_cold=it_c.tolist(), iters_warm=it_w.tolist(),
                relgap_cold=[d["relgap"] for d in cold], relgap_warm=[d["relgap"] for d in rest],
                converged_cold=int(sum(d["converged"] for d in cold)),
                converged_warm=int(sum(d["converged"] for d in rest)),
                solve_cold_s=t_cold, solve_warm_s=t_first + t_rest, net_s=t_net,
                speedup=t_cold / (t_first + t_rest + t_net),
                mean_iter_ratio=float(it_c.mean() / max(1.0, it_w.mean())))
