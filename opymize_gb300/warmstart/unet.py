"""U-Net that proposes a PDHG starting point (x0, y0) for ROF denoising.

Inputs per pixel: the noisy image f and the image's lambda; outputs: the
primal correction x - f and the dual y / lambda (2 components, the forward
gradient's directions).  Four levels (512, 256, 128, 64 pixels for 512^2
inputs) with 32, 64, 128 and 128 channels; the decoder upsamples (nearest),
concatenates the skip connection and applies one 3x3 convolution per level;
a 1x1 head maps the last 32 channels to the 3 outputs.  ~0.64M parameters.

Every 3x3 convolution -- forward, input gradient and weight gradient -- runs
in libopyx's tcgen05 kernels (BF16 operands, FP32 accumulation); the
pooling, upsampling, GELU backward, head, loss and Adam steps are libopyx
CUDA-core kernels.  PyTorch only allocates the device buffers.  There is no
counterpart in the reference, whose solvers start from zero or from a
caller's `continue_at` (opymize/solvers/pdhg.py:229-255).

Activation buffers (NHWC bf16), per level l with H_l = S / 2^l:
  in0 (32: f, lambda, zeros)  a0a (32)  cat0 (64: [up(d1) | e0b])  ad0 (32)
  p0 (32)  a1a (64)  cat1 (128: [up(d2) | e1b])  ad1 (32)
  p1 (64)  a2a (128) cat2 (256: [up(mid) | e2b]) ad2 (64)
  p2 (128) a3 (128)
The skip activations are written by their convolutions straight into the
upper channel slice of the concatenation buffers, and the upsampled decoder
activations into the lower slice, so no concatenation copy exists.
"""

import ctypes as C

import numpy as np

from opymize_gb300 import _lib
from opymize_gb300.gpuarray import stream_ptr, torch

# name, input buffer, input channel offset, input stride, cin, cout,
# output buffer, output stride, output offset, level
LAYERS = [
    ("e0a", "in0", 0, 32, 32, 32, "a0a", 32, 0, 0),
    ("e0b", "a0a", 0, 32, 32, 32, "cat0", 64, 32, 0),
    ("e1a", "p0", 0, 32, 32, 64, "a1a", 64, 0, 1),
    ("e1b", "a1a", 0, 64, 64, 64, "cat1", 128, 64, 1),
    ("e2a", "p1", 0, 64, 64, 128, "a2a", 128, 0, 2),
    ("e2b", "a2a", 0, 128, 128, 128, "cat2", 256, 128, 2),
    ("mid", "p2", 0, 128, 128, 128, "a3", 128, 0, 3),
    ("d2", "cat2", 0, 256, 256, 64, "ad2", 64, 0, 2),
    ("d1", "cat1", 0, 128, 128, 32, "ad1", 32, 0, 1),
    ("d0", "cat0", 0, 64, 64, 32, "ad0", 32, 0, 0),
]
LAYER = {l[0]: l for l in LAYERS}
HEAD_K = 3
LAM_SCALE = 1.0 / 0.3          # lambda channel scaled to about [0, 1]
LOSS_WEIGHTS = (1.0, 1.0, 1.0)
# warm-start loss: primal residual, lambda * divergence of the dual error, dual
# error, 8x8 block means of the first two (the slow, low-frequency modes; off
# by default: weighting them did not shorten the solves that follow)
WARM_WEIGHTS = (1.0, 1.0, 0.05, 0.0)


def _p(t):
    return t.data_ptr() if t is not None else None


class UNet(object):
    """Parameters (FP32 masters with bf16 working copies), Adam state and
    per-shape activation buffers.  `forward` / `backward` / `adam_step` run
    one training step; `predict` proposes (x0, y0) for a batch of images."""

    def __init__(self, seed=0, restart=False):
        """restart=False: proposals from (f, lambda) alone.  restart=True:
        corrections of a PDHG iterate (x, y), which is fed as three more
        input channels (x - f, y / lambda)."""
        t = torch()
        g = t.Generator(device="cpu").manual_seed(seed)
        self.restart = bool(restart)
        self.nin = 5 if self.restart else 2          # input channels in use
        self.params = {}
        for name, _, _, _, cin, cout, _, _, _, _ in LAYERS:
            # He initialisation for GELU layers
            w = t.randn(9, cout, cin, generator=g) * np.sqrt(2.0 / (9 * cin))
            if name == "e0a":
                w[:, :, self.nin:] = 0.0     # the padding input channels stay zero
            self.params[name + ".w"] = w
            self.params[name + ".b"] = t.zeros(cout)
        self.params["head.w"] = t.randn(HEAD_K, 32, generator=g) * np.sqrt(1.0 / 32) * 0.1
        self.params["head.b"] = t.zeros(HEAD_K)
        self.params = {k: v.float().cuda().contiguous() for k, v in self.params.items()}
        self.m = {k: t.zeros_like(v) for k, v in self.params.items()}
        self.v = {k: t.zeros_like(v) for k, v in self.params.items()}
        self.grads = {k: t.zeros_like(v) for k, v in self.params.items()}
        self.wb, self.wt = {}, {}
        for name, _, _, _, cin, cout, _, _, _, _ in LAYERS:
            self.wb[name] = t.empty(9, cout, cin, device="cuda", dtype=t.bfloat16)
            self.wt[name] = t.empty(9, cin, cout, device="cuda", dtype=t.bfloat16)
        self.steps = 0
        self._bufs = {}
        self.loss_weights = t.tensor(LOSS_WEIGHTS, device="cuda", dtype=t.float32)
        self.refresh_weights()

    # ------------------------------------------------------------ plumbing
    def refresh_weights(self):
        for name, _, _, _, cin, cout, _, _, _, _ in LAYERS:
            _lib.call("opyx_conv_weights", cin, cout, _p(self.params[name + ".w"]),
                      _p(self.wb[name]), _p(self.wt[name]), stream_ptr())

    def nparams(self):
        """Trainable parameters (e0a's zero padding input channels excluded)."""
        return sum(v.numel() for v in self.params.values()) - 9 * 32 * (32 - self.nin)

    def buffers(self, B, S):
        key = (B, S)
        if key in self._bufs:
            return self._bufs[key]
        for lev in range(4):
            h = S >> lev
            if (S % 8) or not (h % 128 == 0 or (128 % h == 0 and h * h >= 128)):
                raise ValueError("image side must be 128, 256, 512 or a multiple of 1024 "
                                 "(128-pixel convolution tiles of whole rows on every level)")
        t = torch()
        bf = t.bfloat16

        def act(l, c, dtype=bf):
            s = S >> l
            return t.empty(B, s, s, c, device="cuda", dtype=dtype)

        b = dict(in0=act(0, 32), a0a=act(0, 32), cat0=act(0, 64), ad0=act(0, 32),
                 p0=act(1, 32), a1a=act(1, 64), cat1=act(1, 128), ad1=act(1, 32),
                 p1=act(2, 64), a2a=act(2, 128), cat2=act(2, 256), ad2=act(2, 64),
                 p2=act(3, 128), a3=act(3, 128),
                 out=t.empty(B, S, S, HEAD_K, device="cuda"),
                 f=t.empty(B, S, S, device="cuda"), lam=t.empty(B, device="cuda"),
                 xb=t.empty(B, S, S, device="cuda") if self.restart else None,
                 yb=t.empty(B, S, S, 2, device="cuda") if self.restart else None)
        for name, _, _, _, _, cout, _, _, _, lev in LAYERS:
            b["z." + name] = act(lev, cout)
        self._bufs = {key: b}
        self._grad_bufs = None
        return b

    def grad_buffers(self, B, S):
        if self._grad_bufs is not None and self._grad_bufs[0] == (B, S):
            return self._grad_bufs[1]
        t = torch()

        def act(l, c, dtype=t.float32):
            s = S >> l
            return t.empty(B, s, s, c, device="cuda", dtype=dtype)

        g = dict(dout=act(0, HEAD_K), dad0=act(0, 32), dcat0=act(0, 64), dad1=act(1, 32),
                 dcat1=act(1, 128), dad2=act(2, 64), dcat2=act(2, 256), da3=act(3, 128),
                 dp2=act(3, 128), da2a=act(2, 128), dp1=act(2, 64), da1a=act(1, 64),
                 dp0=act(1, 32), da0a=act(0, 32))
        for name, _, _, _, _, cout, _, _, _, lev in LAYERS:
            g["dz." + name] = act(lev, cout, t.bfloat16)
        L = _lib.load()
        need = 0
        for name, src, ioff, istr, cin, cout, _, _, _, lev in LAYERS:
            d = self._desc(name, B, S, None, None, None)
            need = max(need, L.opyx_conv3x3_wgrad_workspace(C.byref(d)))
            need = max(need, L.opyx_gelu_bwd_workspace(B * (S >> lev) ** 2, cout))
        need = max(need, L.opyx_head_bwd_workspace(B * S * S, HEAD_K))
        g["ws"] = t.empty(need // 4 + 64, device="cuda")
        g["ws_bytes"] = need
        g["loss_parts"] = t.empty(1024, device="cuda", dtype=t.float64)
        self._grad_bufs = ((B, S), g)
        return g

    def _desc(self, name, B, S, x, y, z, epilogue=_lib.OPYX_CONV_GELU, bias=None, w=None,
              transpose=False, out_stride=None, out_off=0):
        _, _, ioff, istr, cin, cout, _, ostr, ooff, lev = LAYER[name]
        d = _lib.opyx_conv3x3_desc()
        d.batch, d.height, d.width = B, S >> lev, S >> lev
        if not transpose:
            d.in_channels, d.in_stride, d.in_offset = cin, istr, ioff
            d.out_channels = cout
            d.out_stride, d.out_offset = (out_stride or ostr), (out_off if out_stride else ooff)
        else:
            d.in_channels, d.in_stride, d.in_offset = cout, cout, 0
            d.out_channels, d.out_stride, d.out_offset = cin, out_stride or cin, out_off
        d.epilogue, d.accumulate = epilogue, 0
        d.x = _p(x) if x is not None else 16
        d.w = _p(w) if w is not None else 16
        d.bias = _p(bias)
        d.y = _p(y) if y is not None else 16
        d.z = _p(z)
        return d

    # ------------------------------------------------------------- forward
    def forward(self, f, lam, keep=True, state=None):
        """f: (B, S, S) fp32 device tensor, lam: (B,) fp32 device tensor,
        state: the restart mode's iterate (x (B, S, S), y (B, S, S, 2)).
        Returns the (B, S, S, 3) fp32 head output: (x - f, y / lambda), or in
        the restart mode the corrections of (x, y / lambda).  keep=False
        skips storing the pre-activations the backward needs (inference: a
        third less traffic in the convolutions' epilogues)."""
        B, S = f.shape[0], f.shape[1]
        b = self.buffers(B, S)
        s = stream_ptr()
        if f.data_ptr() != b["f"].data_ptr():
            b["f"].copy_(f)
            b["lam"].copy_(lam)
        if self.restart:
            if state is None:
                raise ValueError("the restart mode needs the current iterate")
            b["xb"].copy_(state[0].reshape(B, S, S))
            b["yb"].copy_(state[1].reshape(B, S, S, 2))
            _lib.call("opyx_pack_input_state", B, S * S, _p(b["f"]), _p(b["lam"]), LAM_SCALE,
                      _p(b["xb"]), _p(b["yb"]), _p(b["in0"]), s)
        else:
            _lib.call("opyx_pack_input", B, S * S, _p(b["f"]), _p(b["lam"]), LAM_SCALE, _p(b["in0"]), s)

        def conv(name):
            _, src, _, _, _, _, dst, _, _, _ = LAYER[name]
            d = self._desc(name, B, S, b[src], b[dst], b["z." + name] if keep else None,
                           bias=self.params[name + ".b"], w=self.wb[name])
            _lib.call("opyx_conv3x3", C.byref(d), s)

        def pool(lev, src, off, stride, c, dst):
            h = S >> lev
            _lib.call("opyx_pool2", B, h, h, c, _p(b[src]), stride, off, _p(b[dst]), s)

        def up(lev, src, c, dst, stride):
            h = S >> lev          # the coarse level's side
            _lib.call("opyx_up2", B, h, h, c, _p(b[src]), _p(b[dst]), stride, 0, s)

        conv("e0a"); conv("e0b"); pool(0, "cat0", 32, 64, 32, "p0")
        conv("e1a"); conv("e1b"); pool(1, "cat1", 64, 128, 64, "p1")
        conv("e2a"); conv("e2b"); pool(2, "cat2", 128, 256, 128, "p2")
        conv("mid")
        up(3, "a3", 128, "cat2", 256); conv("d2")
        up(2, "ad2", 64, "cat1", 128); conv("d1")
        up(1, "ad1", 32, "cat0", 64); conv("d0")
        _lib.call("opyx_head", B * S * S, HEAD_K, _p(b["ad0"]), _p(self.params["head.w"]),
                  _p(self.params["head.b"]), _p(b["out"]), s)
        return b["out"]

    # ------------------------------------------------------------ backward
    def loss(self, target):
        """Weighted MSE of the last forward output against `target`
        (B, S, S, 3); writes dL/dout.  Returns the loss as a device scalar."""
        out = self._bufs[next(iter(self._bufs))]["out"]
        B, S = out.shape[0], out.shape[1]
        g = self.grad_buffers(B, S)
        _lib.call("opyx_mse", out.numel(), HEAD_K, _p(out), _p(target), _p(self.loss_weights),
                  _p(g["dout"]), _p(g["loss_parts"]), g["loss_parts"].numel(), stream_ptr())
        return g["loss_parts"].sum()

    def loss_warm(self, target, weights=WARM_WEIGHTS):
        """The warm-start loss (opyx_warm_loss) of the last forward output:
        w_x |o0 - t0|^2 + w_div |lambda div(o12 - t12)|^2 + w_u |o12 - t12|^2
        per pixel, averaged, plus w_pool times the 8x8-block-mean version of
        the first two; writes dL/dout.  Returns a device scalar."""
        b = self._bufs[next(iter(self._bufs))]
        out = b["out"]
        B, S = out.shape[0], out.shape[1]
        g = self.grad_buffers(B, S)
        if "scratch" not in g:
            g["scratch"] = torch().empty(B * S * S + B * S * S // 32 + 64, device="cuda")
        _lib.call("opyx_warm_loss", B, S, S, _p(out), _p(target), _p(b["lam"]), weights[0],
                  weights[1], weights[2], weights[3], _p(g["dout"]), _p(g["scratch"]),
                  _p(g["loss_parts"]), g["loss_parts"].numel(), stream_ptr())
        return g["loss_parts"].sum()

    def backward(self):
        key = next(iter(self._bufs))
        B, S = key
        b = self._bufs[key]
        g = self.grad_buffers(B, S)
        s = stream_ptr()
        ws, nws = _p(g["ws"]), g["ws_bytes"]
        P = B * S * S
        _lib.call("opyx_head_bwd", P, HEAD_K, _p(b["ad0"]), _p(self.params["head.w"]), _p(g["dout"]),
                  _p(g["dad0"]), _p(self.grads["head.w"]), _p(self.grads["head.b"]), ws, nws, s)

        def layer(name, da, da_stride, da_off, dx=None, dx_stride=None):
            _, src, _, _, cin, cout, _, _, _, lev = LAYER[name]
            npix = B * (S >> lev) ** 2
            dz = g["dz." + name]
            _lib.call("opyx_gelu_bwd", npix, cout, _p(g[da]), da_stride, da_off, _p(b["z." + name]),
                      _p(dz), _p(self.grads[name + ".b"]), 0, ws, nws, s)
            d = self._desc(name, B, S, b[src], None, None)
            _lib.call("opyx_conv3x3_wgrad", C.byref(d), _p(dz), _p(self.grads[name + ".w"]), 0, ws,
                      nws, s)
            if dx is not None:
                d = self._desc(name, B, S, dz, g[dx], None, epilogue=_lib.OPYX_CONV_F32,
                               w=self.wt[name], transpose=True)
                _lib.call("opyx_conv3x3", C.byref(d), s)

        def up_bwd(lev, dsrc, stride, c, dst):
            h = S >> lev
            _lib.call("opyx_up2_bwd", B, h, h, c, _p(g[dsrc]), stride, 0, _p(g[dst]), s)

        def pool_bwd(lev, dsrc, c, dst, stride, off):
            h = S >> lev
            _lib.call("opyx_pool2_bwd", B, h, h, c, _p(g[dsrc]), _p(g[dst]), stride, off, 1, s)

        layer("d0", "dad0", 32, 0, "dcat0")
        up_bwd(1, "dcat0", 64, 32, "dad1")
        layer("d1", "dad1", 32, 0, "dcat1")
        up_bwd(2, "dcat1", 128, 64, "dad2")
        layer("d2", "dad2", 64, 0, "dcat2")
        up_bwd(3, "dcat2", 256, 128, "da3")
        layer("mid", "da3", 128, 0, "dp2")
        pool_bwd(2, "dp2", 128, "dcat2", 256, 128)
        layer("e2b", "dcat2", 256, 128, "da2a")
        layer("e2a", "da2a", 128, 0, "dp1")
        pool_bwd(1, "dp1", 64, "dcat1", 128, 64)
        layer("e1b", "dcat1", 128, 64, "da1a")
        layer("e1a", "da1a", 64, 0, "dp0")
        pool_bwd(0, "dp0", 32, "dcat0", 64, 32)
        layer("e0b", "dcat0", 64, 32, "da0a")
        layer("e0a", "da0a", 32, 0)

    def adam_step(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        self.steps += 1
        s = stream_ptr()
        self.grads["e0a.w"].view(9, 32, 32)[:, :, self.nin:] = 0.0
        for k, w in self.params.items():
            name = k.split(".")[0]
            conv = k.endswith(".w") and name in LAYER
            cin, cout = (LAYER[name][4], LAYER[name][5]) if conv else (0, 0)
            _lib.call("opyx_adam", w.numel(), _p(w), _p(self.grads[k]), _p(self.m[k]), _p(self.v[k]),
                      lr, b1, b2, eps, self.steps, _p(self.wb[name]) if conv else None,
                      _p(self.wt[name]) if conv else None, cin, cout, s)

    def check_fault(self):
        f = C.c_uint(0)
        _lib.call("opyx_net_fault", C.byref(f))
        if f.value:
            raise _lib.OpyxError("warm-start network", _lib.OPYX_ERR_LAUNCH,
                                 "a convolution gave up waiting for its own copies")

    # ------------------------------------------------------------- inference
    def predict(self, f, lam, state=None):
        """(x0, y0) for images f (B, S, S) and lambdas (B,) (device tensors):
        x0 = f + out0, y0 = lambda * out[1:3] projected onto the unit ball
        (feasible for F* = indicator of the lambda-ball); in the restart mode
        the corrected iterate (x + out0, lambda * proj(y / lambda + out[1:3])).
        Returns (B, S, S) and (B, S, S, 2) fp32 device tensors."""
        t = torch()
        out = self.forward(f, lam, keep=False, state=state)
        b = self._bufs[next(iter(self._bufs))]
        B, S = out.shape[0], out.shape[1]
        x0 = t.empty(B, S, S, device="cuda")
        y0 = t.empty(B, S, S, 2, device="cuda")
        if self.restart:
            _lib.call("opyx_warm_unpack_rel", B, S * S, _p(b["xb"]), _p(b["yb"]), _p(b["lam"]),
                      _p(out), _p(x0), _p(y0), stream_ptr())
        else:
            _lib.call("opyx_warm_unpack", B, S * S, _p(b["f"]), _p(b["lam"]), _p(out), _p(x0),
                      _p(y0), stream_ptr())
        return x0, y0

    # ------------------------------------------------------------ measurement
    def conv_flops(self, B, S, backward=False):
        """Tensor-core FLOPs of the 3x3 convolutions as executed (e0a with
        its 32 padded input channels): forward, or forward + input gradient
        (every layer but e0a) + weight gradient."""
        fwd = sum(2.0 * B * (S >> l[9]) ** 2 * l[4] * l[5] * 9 for l in LAYERS)
        if not backward:
            return fwd
        dgrad = sum(2.0 * B * (S >> l[9]) ** 2 * l[4] * l[5] * 9 for l in LAYERS if l[0] != "e0a")
        return 2 * fwd + dgrad

    def time_conv(self, name, B, S, reps=20):
        """Mean time (s) of one forward launch of layer `name` on the
        current buffers, CUDA events on the current stream."""
        t = torch()
        b = self.buffers(B, S)
        _, src, _, _, cin, cout, dst, _, _, lev = LAYER[name]
        d = self._desc(name, B, S, b[src], b[dst], b["z." + name], bias=self.params[name + ".b"],
                       w=self.wb[name])
        s = stream_ptr()
        for _ in range(3):
            _lib.call("opyx_conv3x3", C.byref(d), s)
        e0, e1 = t.cuda.Event(enable_timing=True), t.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            _lib.call("opyx_conv3x3", C.byref(d), s)
        e1.record()
        t.cuda.synchronize()
        flops = 2.0 * B * (S >> lev) ** 2 * cin * cout * 9
        return e0.elapsed_time(e1) / 1e3 / reps, flops

    # -------------------------------------------------------------- storage
    def state_dict(self):
        d = {k: v.detach().cpu().numpy() for k, v in self.params.items()}
        d["restart"] = np.array(int(self.restart))
        return d

    def load_state_dict(self, sd):
        t = torch()
        for k in self.params:
            self.params[k].copy_(t.from_numpy(np.asarray(sd[k], dtype=np.float32)))
        self.refresh_weights()

    def save(self, path):
        np.savez(path, **self.state_dict())

    @classmethod
    def load(cls, path):
        with np.load(path) as d:
            sd = {k: d[k] for k in d.files}
        net = cls(restart=bool(int(sd.pop("restart", 0))))
        net.load_state_dict(sd)
        return net
