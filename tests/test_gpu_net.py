"""Warm-start network kernels against plain PyTorch FP32 references of the
same ops (on bf16-rounded operands, so only the summation order differs):
the tcgen05 3x3 convolution (GELU / FP32 / BF16 epilogues, channel slices),
its weight gradient, and the elementwise, pooling, head, loss and Adam
kernels around them."""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch
    torch.backends.cudnn.allow_tf32 = False
    torch.backends.cuda.matmul.allow_tf32 = False
    return torch


def lib():
    from opymize_gb300 import _lib
    return _lib


def desc(B, H, W, cin, cout, x, w, y, bias=None, z=None, in_stride=None, in_off=0,
         out_stride=None, out_off=0, epilogue=0, accumulate=0):
    L = lib()
    d = L.opyx_conv3x3_desc()
    d.batch, d.height, d.width = B, H, W
    d.in_channels, d.in_stride, d.in_offset = cin, in_stride or cin, in_off
    d.out_channels, d.out_stride, d.out_offset = cout, out_stride or cout, out_off
    d.epilogue, d.accumulate = epilogue, accumulate
    d.x, d.w = x.data_ptr(), w.data_ptr()
    d.bias = bias.data_ptr() if bias is not None else None
    d.y = y.data_ptr()
    d.z = z.data_ptr() if z is not None else None
    return d


def ref_conv(torch, x, w, bias=None):
    """x (B, H, W, Cin) float, w (9, Cout, Cin) float -> (B, H, W, Cout)."""
    wt = w.reshape(3, 3, w.shape[1], w.shape[2]).permute(2, 3, 0, 1)   # (Cout, Cin, 3, 3)
    y = torch.nn.functional.conv2d(x.permute(0, 3, 1, 2), wt, bias=bias, padding=1)
    return y.permute(0, 2, 3, 1)


def gelu(torch, z):
    return torch.nn.functional.gelu(z, approximate="tanh")


def no_fault():
    L = lib()
    f = C.c_uint(0)
    L.call("opyx_net_fault", C.byref(f))
    assert f.value == 0


CASES = [  # B, H, W, cin, cout, in_stride, in_off
    (2, 64, 64, 32, 32, 32, 0),
    (1, 128, 128, 64, 64, 96, 32),
    (1, 256, 256, 32, 128, 32, 0),
    (2, 64, 64, 128, 256, 128, 0),
    (1, 32, 512, 96, 64, 96, 0),
]


@pytest.mark.parametrize("case", CASES)
def test_conv3x3_gelu_matches_torch(torch, case):
    B, H, W, cin, cout, stride, off = case
    g = torch.Generator(device="cuda").manual_seed(1)
    x = (torch.randn(B, H, W, stride, device="cuda", generator=g)).to(torch.bfloat16)
    w = (torch.randn(9, cout, cin, device="cuda", generator=g) / np.sqrt(9 * cin)).to(torch.bfloat16)
    bias = torch.randn(cout, device="cuda", generator=g) * 0.1
    y = torch.empty(B, H, W, cout, device="cuda", dtype=torch.bfloat16)
    z = torch.empty(B, H, W, cout, device="cuda", dtype=torch.bfloat16)
    d = desc(B, H, W, cin, cout, x, w, y, bias=bias, z=z, in_stride=stride, in_off=off)
    lib().call("opyx_conv3x3", C.byref(d), None)
    torch.cuda.synchronize()
    no_fault()
    zr = ref_conv(torch, x[..., off:off + cin].float(), w.float(), bias)
    # z is acc + bias rounded to bf16; y = gelu(acc + bias) rounded to bf16
    assert torch.allclose(z.float(), zr, rtol=2 ** -7, atol=1e-3)
    yr = gelu(torch, zr)
    assert torch.allclose(y.float(), yr, rtol=2 ** -7, atol=2e-3)


def test_conv3x3_f32_accumulate_into_slice(torch):
    B, H, W, cin, cout = 1, 64, 64, 64, 32
    g = torch.Generator(device="cuda").manual_seed(2)
    x = torch.randn(B, H, W, cin, device="cuda", generator=g).to(torch.bfloat16)
    w = (torch.randn(9, cout, cin, device="cuda", generator=g) / 24).to(torch.bfloat16)
    y = torch.randn(B, H, W, 96, device="cuda", generator=g)
    y0 = y.clone()
    d = desc(B, H, W, cin, cout, x, w, y, out_stride=96, out_off=64, epilogue=1, accumulate=1)
    lib().call("opyx_conv3x3", C.byref(d), None)
    torch.cuda.synchronize()
    no_fault()
    ref = ref_conv(torch, x.float(), w.float())
    assert torch.equal(y[..., :64], y0[..., :64])
    err = (y[..., 64:] - y0[..., 64:] - ref).abs().max().item()
    assert err <= 1e-5 * max(1.0, ref.abs().max().item()), err


@pytest.mark.parametrize("case", [(2, 64, 64, 32, 32), (1, 128, 128, 64, 64), (1, 64, 64, 256, 128),
                                  (1, 256, 256, 32, 32)])
def test_conv3x3_wgrad_matches_torch(torch, case):
    B, H, W, cin, cout = case
    g = torch.Generator(device="cuda").manual_seed(3)
    x = torch.randn(B, H, W, cin, device="cuda", generator=g).to(torch.bfloat16)
    dy = torch.randn(B, H, W, cout, device="cuda", generator=g).to(torch.bfloat16)
    w = torch.zeros(9, cout, cin, device="cuda", dtype=torch.bfloat16)
    y = torch.empty(B, H, W, cout, device="cuda", dtype=torch.bfloat16)
    d = desc(B, H, W, cin, cout, x, w, y)
    L = lib()
    nws = L.load().opyx_conv3x3_wgrad_workspace(C.byref(d))
    ws = torch.empty(nws // 4 + 4, device="cuda")
    dw = torch.empty(9, cout, cin, device="cuda")
    L.call("opyx_conv3x3_wgrad", C.byref(d), dy.data_ptr(), dw.data_ptr(), 0, ws.data_ptr(), nws, None)
    torch.cuda.synchronize()
    no_fault()
    xf = x.float().permute(0, 3, 1, 2)
    wt = torch.zeros(cout, cin, 3, 3, device="cuda", requires_grad=True)
    out = torch.nn.functional.conv2d(xf, wt, padding=1)
    out.backward(dy.float().permute(0, 3, 1, 2))
    ref = wt.grad.permute(2, 3, 0, 1).reshape(9, cout, cin)
    scale = ref.abs().max().item()
    err = (dw - ref).abs().max().item()
    assert err <= 5e-5 * scale, (err, scale)


def test_input_gradient_is_a_flipped_convolution(torch):
    """dX of a convolution = a 3x3 convolution of dY with the tap-flipped,
    in/out-transposed weights (opyx_conv_weights makes that copy)."""
    B, H, W, cin, cout = 1, 64, 64, 64, 32
    g = torch.Generator(device="cuda").manual_seed(4)
    x = torch.randn(B, H, W, cin, device="cuda", generator=g)
    w32 = torch.randn(9, cout, cin, device="cuda", generator=g) / 24
    dy = torch.randn(B, H, W, cout, device="cuda", generator=g).to(torch.bfloat16)
    wb = torch.empty(9, cout, cin, device="cuda", dtype=torch.bfloat16)
    wt = torch.empty(9, cin, cout, device="cuda", dtype=torch.bfloat16)
    L = lib()
    L.call("opyx_conv_weights", cin, cout, w32.data_ptr(), wb.data_ptr(), wt.data_ptr(), None)
    dx = torch.empty(B, H, W, cin, device="cuda")
    d = desc(B, H, W, cout, cin, dy, wt, dx, epilogue=1)
    L.call("opyx_conv3x3", C.byref(d), None)
    torch.cuda.synchronize()
    no_fault()
    assert torch.equal(wb.float(), w32.to(torch.bfloat16).float())
    xf = x.permute(0, 3, 1, 2).clone().requires_grad_(True)
    wref = wb.float().reshape(3, 3, cout, cin).permute(2, 3, 0, 1)
    out = torch.nn.functional.conv2d(xf, wref, padding=1)
    out.backward(dy.float().permute(0, 3, 1, 2))
    ref = xf.grad.permute(0, 2, 3, 1)
    err = (dx - ref).abs().max().item()
    assert err <= 1e-5 * ref.abs().max().item(), err


def test_elementwise_kernels(torch):
    L = lib()
    B, H, W, C2 = 2, 64, 64, 32
    g = torch.Generator(device="cuda").manual_seed(5)
    # pooling of a channel slice and its backward
    x = torch.randn(B, H, W, 96, device="cuda", generator=g).to(torch.bfloat16)
    p = torch.empty(B, H // 2, W // 2, C2, device="cuda", dtype=torch.bfloat16)
    L.call("opyx_pool2", B, H, W, C2, x.data_ptr(), 96, 32, p.data_ptr(), None)
    ref = torch.nn.functional.avg_pool2d(x[..., 32:64].float().permute(0, 3, 1, 2), 2).permute(0, 2, 3, 1)
    assert torch.allclose(p.float(), ref, rtol=2 ** -8, atol=1e-6)
    dp = torch.randn(B, H // 2, W // 2, C2, device="cuda", generator=g)
    dx = torch.randn(B, H, W, 96, device="cuda", generator=g)
    dx0 = dx.clone()
    L.call("opyx_pool2_bwd", B, H, W, C2, dp.data_ptr(), dx.data_ptr(), 96, 32, 1, None)
    up = dp.repeat_interleave(2, 1).repeat_interleave(2, 2) * 0.25
    assert torch.allclose(dx[..., 32:64], dx0[..., 32:64] + up, atol=1e-6)
    assert torch.equal(dx[..., :32], dx0[..., :32])
    # nearest upsampling into a slice and its backward
    a = torch.randn(B, H // 2, W // 2, C2, device="cuda", generator=g).to(torch.bfloat16)
    cat = torch.zeros(B, H, W, 64, device="cuda", dtype=torch.bfloat16)
    L.call("opyx_up2", B, H // 2, W // 2, C2, a.data_ptr(), cat.data_ptr(), 64, 0, None)
    assert torch.equal(cat[..., :32], a.repeat_interleave(2, 1).repeat_interleave(2, 2))
    dcat = torch.randn(B, H, W, 64, device="cuda", generator=g)
    da = torch.empty(B, H // 2, W // 2, C2, device="cuda")
    L.call("opyx_up2_bwd", B, H // 2, W // 2, C2, dcat.data_ptr(), 64, 0, da.data_ptr(), None)
    ref = dcat[..., :32].reshape(B, H // 2, 2, W // 2, 2, C2).sum(dim=(2, 4))
    assert torch.allclose(da, ref, atol=1e-5)
    # gelu backward with bias grad
    npix = B * H * W
    zz = torch.randn(npix, C2, device="cuda", generator=g).to(torch.bfloat16)
    dA = torch.randn(B, H, W, 96, device="cuda", generator=g)
    dz = torch.empty(npix, C2, device="cuda", dtype=torch.bfloat16)
    db = torch.empty(C2, device="cuda")
    nws = L.load().opyx_gelu_bwd_workspace(npix, C2)
    ws = torch.empty(nws // 4, device="cuda")
    L.call("opyx_gelu_bwd", npix, C2, dA.data_ptr(), 96, 64, zz.data_ptr(), dz.data_ptr(), db.data_ptr(),
           0, ws.data_ptr(), nws, None)
    zr = zz.float().clone().requires_grad_(True)
    gelu(torch, zr).backward(dA[..., 64:].reshape(npix, C2))
    assert torch.allclose(dz.float(), zr.grad, rtol=2 ** -7, atol=1e-6)
    assert torch.allclose(db, dz.float().sum(0), rtol=1e-5, atol=1e-4)


def test_head_loss_adam(torch):
    L = lib()
    npix = 128 * 128
    g = torch.Generator(device="cuda").manual_seed(6)
    a = torch.randn(npix, 32, device="cuda", generator=g).to(torch.bfloat16)
    w = torch.randn(3, 32, device="cuda", generator=g) * 0.2
    b = torch.randn(3, device="cuda", generator=g)
    out = torch.empty(npix, 3, device="cuda")
    L.call("opyx_head", npix, 3, a.data_ptr(), w.data_ptr(), b.data_ptr(), out.data_ptr(), None)
    ref = a.float() @ w.t() + b
    assert torch.allclose(out, ref, rtol=1e-5, atol=1e-5)
    tgt = torch.randn(npix, 3, device="cuda", generator=g)
    wk = torch.tensor([1.0, 2.0, 0.5], device="cuda")
    grad = torch.empty(npix, 3, device="cuda")
    parts = torch.empty(64, device="cuda", dtype=torch.float64)
    L.call("opyx_mse", npix * 3, 3, out.data_ptr(), tgt.data_ptr(), wk.data_ptr(), grad.data_ptr(),
           parts.data_ptr(), 64, None)
    loss_ref = ((out - tgt) ** 2 * wk).mean()
    assert abs(parts.sum().item() - loss_ref.item()) <= 1e-5 * loss_ref.item()
    assert torch.allclose(grad, 2 * wk * (out - tgt) / (npix * 3), rtol=1e-6, atol=1e-12)
    da = torch.empty(npix, 32, device="cuda")
    dw = torch.empty(3, 32, device="cuda")
    db = torch.empty(3, device="cuda")
    nws = L.load().opyx_head_bwd_workspace(npix, 3)
    ws = torch.empty(nws // 4, device="cuda")
    L.call("opyx_head_bwd", npix, 3, a.data_ptr(), w.data_ptr(), grad.data_ptr(), da.data_ptr(),
           dw.data_ptr(), db.data_ptr(), ws.data_ptr(), nws, None)
    af = a.float()
    assert torch.allclose(da, grad @ w, rtol=1e-5, atol=1e-9)
    assert torch.allclose(dw, grad.t() @ af, rtol=1e-4, atol=1e-7)
    assert torch.allclose(db, grad.sum(0), rtol=1e-4, atol=1e-8)
    # Adam against torch.optim.Adam on the same gradient
    p = torch.randn(9 * 32 * 64, device="cuda", generator=g)
    gr = torch.randn_like(p)
    m = torch.zeros_like(p)
    v = torch.zeros_like(p)
    pr = p.clone().requires_grad_(True)
    opt = torch.optim.Adam([pr], lr=1e-3, betas=(0.9, 0.999), eps=1e-8)
    wb = torch.empty(p.numel(), device="cuda", dtype=torch.bfloat16)
    for step in (1, 2, 3):
        L.call("opyx_adam", p.numel(), p.data_ptr(), gr.data_ptr(), m.data_ptr(), v.data_ptr(), 1e-3, 0.9,
               0.999, 1e-8, step, wb.data_ptr(), None, 64, 32, None)
        pr.grad = gr.clone()
        opt.step()
    assert torch.allclose(p, pr.detach(), rtol=1e-5, atol=1e-7)
    assert torch.equal(wb, p.to(torch.bfloat16))
