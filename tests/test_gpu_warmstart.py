"""Learned warm start: the U-Net's forward output and every parameter
gradient (tcgen05 convolutions, hand-written backward) against torch CPU
autograd in FP64 on the same weights; training lowers the loss; the trained
network's proposals let the fused PDHG reach the same relative gap in fewer
iterations than the zero start, with the plain solver's stop test deciding."""

import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

WEIGHTS = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                       "opymize_gb300", "warmstart", "unet512.npz")


def torch_unet(T, params, f, lam, lam_scale):
    """The network of opymize_gb300.warmstart.unet in plain torch (NCHW)."""
    F = T.nn.functional
    B, S = f.shape[0], f.shape[1]
    x = T.zeros(B, 32, S, S, dtype=f.dtype)
    x[:, 0] = f
    x[:, 1] = (lam * lam_scale).view(B, 1, 1)

    def conv(x, name):
        w = params[name + ".w"]                       # (9, cout, cin), tap = 3 (dy+1) + (dx+1)
        wt = w.reshape(3, 3, w.shape[1], w.shape[2]).permute(2, 3, 0, 1)
        return F.gelu(F.conv2d(x, wt, params[name + ".b"], padding=1), approximate="tanh")

    def up(x):
        return x.repeat_interleave(2, 2).repeat_interleave(2, 3)

    e0 = conv(conv(x, "e0a"), "e0b")
    e1 = conv(conv(F.avg_pool2d(e0, 2), "e1a"), "e1b")
    e2 = conv(conv(F.avg_pool2d(e1, 2), "e2a"), "e2b")
    m = conv(F.avg_pool2d(e2, 2), "mid")
    d2 = conv(T.cat([up(m), e2], 1), "d2")
    d1 = conv(T.cat([up(d2), e1], 1), "d1")
    d0 = conv(T.cat([up(d1), e0], 1), "d0")
    out = T.einsum("bchw,kc->bhwk", d0, params["head.w"]) + params["head.b"]
    return out


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def test_unet_matches_torch_autograd():
    import torch as T
    from opymize_gb300.warmstart import UNet
    from opymize_gb300.warmstart.unet import LAM_SCALE
    net = UNet(seed=3)
    # larger head weights than the initialisation so every layer's gradient is sizeable
    net.params["head.w"].normal_(0.0, 0.3)
    B, S = 2, 128
    g = T.Generator().manual_seed(0)
    f = T.rand(B, S, S, generator=g)
    lam = T.tensor([0.05, 0.25])
    tgt = T.randn(B, S, S, 3, generator=g)
    out = net.forward(f.cuda(), lam.cuda())
    loss = net.loss(tgt.cuda())
    net.backward()
    T.cuda.synchronize()
    net.check_fault()
    ref_params = {k: v.detach().cpu().double().requires_grad_(True) for k, v in net.params.items()}
    ro = torch_unet(T, ref_params, f.double(), lam.double(), LAM_SCALE)
    rl = ((ro - tgt.double()) ** 2).mean()
    rl.backward()
    # bf16 activations and operands (8-bit mantissa) against FP64: a few 1e-3 per layer
    assert rel(out.cpu().double().numpy(), ro.detach().numpy()) < 2e-2
    assert abs(float(loss) - float(rl.detach())) <= 2e-2 * float(rl.detach())
    for k in net.params:
        gk = net.grads[k].cpu().double().numpy()
        rk = ref_params[k].grad.numpy()
        if k == "e0a.w":
            gk, rk = gk[:, :, :2], rk[:, :, :2]      # the zero input channels
        assert rel(gk, rk) < 5e-2, (k, rel(gk, rk))


def test_training_lowers_the_loss():
    import torch as T
    from opymize_gb300.warmstart import UNet, make_dataset, train
    data = make_dataset(range(8), S=128, tol=1e-4, maxiter=4000)
    net = UNet(seed=1)
    losses, step_ms = train(net, data, epochs=60, batch=8, lr=2e-3, cosine=False)
    assert np.isfinite(losses).all()
    assert losses[-1] < 0.8 * losses[0], losses
    net.check_fault()


def test_batch_init_matches_continue_at():
    """BatchROF's `init` and PDHG's `continue_at` (the reference's warm
    start hook, pdhg.py:254-255) start from the same point: same iterates."""
    import torch as T
    from opymize_gb300.warmstart import instances, solve_batch
    from opymize_gb300.functionals import SSD, L1Norms
    from opymize_gb300.linear import GradientOp
    from opymize_gb300.solvers import PDHG
    f, lam = instances([5, 6], S=64)
    g = np.random.default_rng(0)
    x0 = (f + 0.01 * g.standard_normal(f.shape)).astype(np.float32)
    y0 = (0.5 * lam.reshape(-1, 1, 1, 1) * g.uniform(-1, 1, (2, 64, 64, 2))).astype(np.float32)
    xs, ys, infos, _ = solve_batch(f, lam, 1e-300, 20, init=(T.from_numpy(x0).cuda().view(2, -1),
                                                           T.from_numpy(y0).cuda().view(2, -1)))
    for i in range(2):
        N = 64 * 64
        s = PDHG(SSD(f[i].reshape(N, 1)), L1Norms(N, (1, 2), float(lam[i])),
                 GradientOp((64, 64), 1, scheme="forward"))
        s.solve(steps="precond", precision="float", term_pd_gap=1e-300, term_maxiter=20,
                granularity=10, continue_at=(x0[i].ravel().astype(np.float64),
                                             y0[i].ravel().astype(np.float64)))
        assert s.path == "fused"
        np.testing.assert_array_equal(xs[i].cpu().numpy().ravel(),
                                      s.state[0].ravel().astype(np.float32))


def test_trained_warm_start_beats_zero_start():
    """The committed network (trained on seeds 0..2047) on 32 held-out
    seeds: the same stop test is met from both starts; the proposal saves
    a third of the iterations to relative gap 1e-3 and is never worse on
    average at 1e-4 (where the slow modes that the network does not resolve
    dominate both runs)."""
    from opymize_gb300.warmstart import UNet, evaluate
    net = UNet.load(WEIGHTS)
    seeds = range(2 * 10 ** 6, 2 * 10 ** 6 + 32)
    for tol, ratio in ((1e-3, 0.85), (1e-4, 1.0)):
        ev = evaluate(net, seeds, S=512, tol=tol)
        assert ev["converged_cold"] == ev["converged_warm"] == 32
        assert all(abs(r) < tol for r in ev["relgap_warm"])
        it_c, it_w = np.array(ev["iters_cold"]), np.array(ev["iters_warm"])
        assert it_w.mean() <= ratio * it_c.mean(), (tol, it_c.mean(), it_w.mean())


def test_warm_loss_matches_torch_autograd():
    """opyx_warm_loss: value and gradient against torch autograd of the same
    formula (divergence adjoint to the forward gradient)."""
    import ctypes as C
    import torch as T
    from opymize_gb300 import _lib
    B, H, W = 2, 32, 48
    g = T.Generator().manual_seed(3)
    out = T.randn(B, H, W, 3, generator=g, dtype=T.float64)
    tgt = T.randn(B, H, W, 3, generator=g, dtype=T.float64)
    lam = T.tensor([0.05, 0.2], dtype=T.float64)
    w = (1.0, 0.7, 0.05, 0.3)
    o = out.clone().requires_grad_(True)
    e = o[..., 1:] - tgt[..., 1:]
    d = T.zeros(B, H, W, dtype=T.float64)
    d[:, :-1, :] += e[:, :-1, :, 0]
    d[:, 1:, :] -= e[:, :-1, :, 0]
    d[:, :, :-1] += e[:, :, :-1, 1]
    d[:, :, 1:] -= e[:, :, :-1, 1]
    ld = lam.view(B, 1, 1) * d
    L = (w[0] * (o[..., 0] - tgt[..., 0]) ** 2 + w[1] * ld ** 2 + w[2] * (e ** 2).sum(-1)).mean()
    pool = lambda v: v.reshape(B, H // 8, 8, W // 8, 8).mean(dim=(2, 4))
    L = L + w[3] * 4096.0 / (B * H * W) * ((pool(o[..., 0] - tgt[..., 0]) ** 2).sum()
                                           + (pool(ld) ** 2).sum())
    L.backward()
    od, td, ld = out.float().cuda(), tgt.float().cuda(), lam.float().cuda()
    grad = T.empty_like(od)
    scr = T.empty(B * H * W + B * H * W // 32, device="cuda")
    parts = T.empty(64, device="cuda", dtype=T.float64)
    _lib.call("opyx_warm_loss", B, H, W, od.data_ptr(), td.data_ptr(), ld.data_ptr(), w[0], w[1], w[2],
              w[3], grad.data_ptr(), scr.data_ptr(), parts.data_ptr(), 64, None)
    assert abs(parts.sum().item() - L.item()) <= 1e-5 * L.item()
    assert rel(grad.cpu().double().numpy(), o.grad.numpy()) < 1e-5


def test_restart_mode_beats_zero_start():
    """The committed restart-mode network (corrections of the iterate after
    100 plain iterations, trained on seeds 0..2047) on 32 held-out seeds:
    the same stop test from both runs; the first 100 iterations count."""
    from opymize_gb300.warmstart import UNet, evaluate_restart
    net = UNet.load(WEIGHTS.replace("unet512.npz", "unet512_restart.npz"))
    assert net.restart
    seeds = range(2 * 10 ** 6, 2 * 10 ** 6 + 32)
    for tol, ratio in ((1e-3, 0.8), (1e-4, 0.95)):
        ev = evaluate_restart(net, seeds, 100, S=512, tol=tol)
        assert ev["converged_cold"] == ev["converged_warm"] == 32
        assert all(abs(r) < tol for r in ev["relgap_warm"])
        it_c, it_w = np.array(ev["iters_cold"]), np.array(ev["iters_warm"])
        assert it_w.mean() <= ratio * it_c.mean(), (tol, it_c.mean(), it_w.mean())
