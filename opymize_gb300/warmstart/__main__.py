"""Generate training data, train the warm-start U-Net and evaluate it on
held-out seeds; prints one JSON line with the results.

    python -m opymize_gb300.warmstart --train 4096 --epochs 6 --eval 256 \
        --out opymize_gb300/warmstart/unet512.npz
"""

import argparse
import json
import sys
import time

import numpy as np

from opymize_gb300.warmstart import UNet, make_dataset, train, evaluate, evaluate_restart

EVAL_SEED0 = 10 ** 6     # held-out seeds start here; training seeds are 0 .. n-1


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, default=512)
    ap.add_argument("--train", type=int, default=4096)
    ap.add_argument("--data-tol", type=float, default=1e-5)
    ap.add_argument("--data-maxiter", type=int, default=8000)
    ap.add_argument("--epochs", type=int, default=6)
    ap.add_argument("--batch", type=int, default=32)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--eval", type=int, default=256)
    ap.add_argument("--eval-tols", default="1e-4", help="comma-separated relative gaps")
    ap.add_argument("--init", default=None, help="start from these weights")
    ap.add_argument("--out", default=None)
    ap.add_argument("--restart", type=int, default=0,
                    help="restart mode: correct the iterate after this many plain iterations")
    ap.add_argument("--profile-steps", type=int, default=0,
                    help="only run this many training steps on --batch seeded images (for profilers)")
    a = ap.parse_args(argv)
    log = lambda m: print(m, file=sys.stderr, flush=True)
    t0 = time.perf_counter()
    net = UNet.load(a.init) if a.init else UNet(seed=0, restart=a.restart > 0)
    res = dict(size=a.size, params=net.nparams())
    if a.profile_steps > 0:
        import torch
        from opymize_gb300.warmstart import instances
        f, lam = instances(range(a.batch), a.size)
        fd, ld = torch.from_numpy(f).cuda(), torch.from_numpy(lam).cuda()
        tgt = torch.zeros(a.batch, a.size, a.size, 3, device="cuda")
        for _ in range(a.profile_steps):
            net.forward(fd, ld)
            net.loss_warm(tgt)
            net.backward()
            net.adam_step(lr=a.lr)
        torch.cuda.synchronize()
        net.check_fault()
        res["profile_steps"] = a.profile_steps
        print(json.dumps(res))
        return
    if a.train > 0:
        data = make_dataset(range(a.train), S=a.size, tol=a.data_tol, maxiter=a.data_maxiter,
                            restart=a.restart)
        its = np.array([d["iter"] for d in data["infos"]])
        res.update(train_n=a.train, data_tol=a.data_tol, data_converged=int(sum(d["converged"] for d in data["infos"])),
                   data_iters_median=float(np.median(its)), data_s=time.perf_counter() - t0)
        log("data: %d images, median %d iterations, %.1f s" % (a.train, np.median(its), res["data_s"]))
        t1 = time.perf_counter()
        losses, step_ms = train(net, data, epochs=a.epochs, batch=a.batch, lr=a.lr, log=log)
        res.update(epochs=a.epochs, batch=a.batch, lr=a.lr, losses=losses, step_ms=step_ms,
                   train_s=time.perf_counter() - t1)
        del data
        if a.out:
            net.save(a.out)
    if a.eval > 0:
        res["eval"] = {}
        for tol in (float(v) for v in a.eval_tols.split(",")):
            seeds = range(EVAL_SEED0, EVAL_SEED0 + a.eval)
            if net.restart:
                ev = evaluate_restart(net, seeds, a.restart, S=a.size, tol=tol, batch=a.batch)
            else:
                ev = evaluate(net, seeds, S=a.size, tol=tol, batch=a.batch)
            r = {k: v for k, v in ev.items() if not isinstance(v, list)}
            r.update(n=a.eval, iters_cold_mean=float(np.mean(ev["iters_cold"])),
                     iters_warm_mean=float(np.mean(ev["iters_warm"])),
                     iters_cold_median=float(np.median(ev["iters_cold"])),
                     iters_warm_median=float(np.median(ev["iters_warm"])))
            res["eval"]["%g" % tol] = r
            log("tol %g: %s" % (tol, r))
    print(json.dumps(res))


if __name__ == "__main__":
    main()
