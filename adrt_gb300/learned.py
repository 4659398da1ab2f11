"""Learned starting image for batched CG on the ADRT normal equations.

A 4-level convolutional encoder-decoder (32/64/128/256 channels, 3 x 3
kernels, ReLU, 2 x 2 average pooling down, nearest 2x upsampling up, skip
connections added before the decoder's first activation) maps the scaled
back-projection u = s * A^T b of the data to an image x0; CG then starts from
x0 instead of 0.  The reference has no learned component: its reconstruction
is CG from zero (docs/examples.cginverse.md:40-67), which stays the fallback;
every solve uses CG's own stopping rule (a solve counts when CG reaches the
tolerance).  The learned convolution preconditioner of
adrt_gb300.precond is the other learned component.

Everything runs in the library's kernels (include/adrt_gb300_net.h): the
3 x 3 convolutions with 32..256 channels on the tcgen05 tensor cores (bf16
weights and activations, f32 accumulation) for forward, input gradient and
weight gradient; the 1-channel input/output layers, pooling, upsampling,
loss and a fused Adam step as plain CUDA kernels.  PyTorch only provides
device memory, streams and CUDA-graph capture.

Training pairs come from the method itself: random phantoms -> adrt ->
noisy data b -> plain CG run to convergence; the network learns
u -> x_cg (mean squared error).

Layout: activations bf16 NHWC; parameters one flat f32 vector (per conv:
weights [9][c_out][c_in], tap = 3 * dy + dx, then bias [c_out]); the Adam
kernel keeps bf16 copies of the tensor-core weights in forward layout and in
the tap-flipped, transposed layout the input gradient uses.
"""

from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass

import torch

from . import _lib
from ._ops import adrt as _adrt
from .autograd import _adjoint_raw as _adjoint

__all__ = ["PreconditionerNet", "LAYERS", "training_pairs", "train", "learned_cg", "normal_op_norm", "TrainLog"]

# Tensor-core layers: name -> (c_in, c_out).  Level l works at (h >> l, w >> l).
LAYERS = (
    ("enc0b", 32, 32),
    ("enc1a", 32, 64),
    ("enc1b", 64, 64),
    ("enc2a", 64, 128),
    ("enc2b", 128, 128),
    ("enc3a", 128, 256),
    ("enc3b", 256, 256),
    ("dec2a", 256, 128),
    ("dec2b", 128, 128),
    ("dec1a", 128, 64),
    ("dec1b", 64, 64),
    ("dec0a", 64, 32),
    ("dec0b", 32, 32),
)
C0 = 32


class _Segment(ctypes.Structure):
    _fields_ = [
        ("offset", ctypes.c_int64),
        ("count", ctypes.c_int64),
        ("kind", ctypes.c_int32),
        ("c_in", ctypes.c_int32),
        ("c_out", ctypes.c_int32),
        ("pad_", ctypes.c_int32),
        ("w_offset", ctypes.c_int64),
        ("wt_offset", ctypes.c_int64),
    ]


def _sizes_ok(h: int, w: int) -> bool:
    """Every level (h >> l, w >> l), l < 4, must tile into the tensor-core
    convolutions' 128-pixel rows (forward) and 64-pixel K stages (weight
    gradient): true for powers of two >= 128."""
    return all(x >= 128 and x & (x - 1) == 0 for x in (h, w))


def _p(t):
    return None if t is None else t.data_ptr()


def _stream(dev):
    return torch.cuda.current_stream(dev).cuda_stream


class PreconditionerNet:
    """Parameters, optimizer state and the forward/backward passes."""

    def __init__(self, device="cuda", seed: int = 0):
        self.dev = torch.device(device)
        if self.dev.type != "cuda":
            raise TypeError("the preconditioner runs on CUDA devices only")
        self.lib = _lib.load()
        # Flat parameter layout.
        self.offsets = {}
        off = 0
        woff = 0
        segs = []

        def plain(name, count):
            nonlocal off
            self.offsets[name] = (off, count)
            segs.append((off, count, 0, 0, 0, 0, 0))
            off += count

        plain("in_w", 9 * C0)
        plain("in_b", C0)
        self.wofs = {}
        for name, ci, co in LAYERS:
            cnt = 9 * ci * co
            self.offsets[name + "_w"] = (off, cnt)
            self.wofs[name] = (woff, woff + cnt)
            segs.append((off, cnt, 1, ci, co, woff, woff + cnt))
            off += cnt
            woff += 2 * cnt
            plain(name + "_b", co)
        plain("out_w", 9 * C0)
        plain("out_b", 1)
        self.n_params = off
        arr = (_Segment * len(segs))()
        for i, (o, c, k, ci, co, wo, wto) in enumerate(segs):
            arr[i] = _Segment(o, c, k, ci, co, 0, wo, wto)
        self.nseg = len(segs)
        raw = torch.frombuffer(bytearray(bytes(arr)), dtype=torch.uint8)
        self.segs = raw.to(self.dev)

        g = torch.Generator().manual_seed(seed)
        p = torch.zeros(self.n_params, dtype=torch.float32)
        o, c = self.offsets["in_w"]
        p[o:o + c] = torch.randn(c, generator=g) * math.sqrt(2.0 / 9)
        for name, ci, co in LAYERS:
            o, c = self.offsets[name + "_w"]
            p[o:o + c] = torch.randn(c, generator=g) * math.sqrt(2.0 / (9 * ci))
        o, c = self.offsets["out_w"]
        p[o:o + c] = torch.randn(c, generator=g) * math.sqrt(1.0 / (9 * C0))
        self.params = p.to(self.dev)
        self.grads = torch.zeros_like(self.params)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.step_count = torch.zeros(1, dtype=torch.int64, device=self.dev)
        self.wbuf = torch.empty(max(1, woff), dtype=torch.bfloat16, device=self.dev)
        self.in_scale = 1.0
        self.loss_terms = (1.0, 0.0, 0)  # (alpha, mu, k): see loss_and_grad
        self._bufs = {}
        self.refresh_weights()

    # ---- parameter views ---------------------------------------------------
    def view(self, name, t=None):
        o, c = self.offsets[name]
        return (self.params if t is None else t)[o:o + c]

    def wt(self, name, transposed=False):
        a, b = self.wofs[name]
        n = b - a
        return self.wbuf[(b if transposed else a):(b if transposed else a) + n]

    def state_dict(self):
        return {"params": self.params.detach().cpu().clone(), "in_scale": self.in_scale}

    def load_state_dict(self, sd):
        self.params.copy_(sd["params"].to(self.dev))
        self.in_scale = float(sd["in_scale"])
        self.refresh_weights()

    def refresh_weights(self):
        rc = self.lib.adrtnet_adam(_p(self.params), None, None, None, _p(self.segs), self.nseg, self.n_params,
                                   0.0, 0.0, 0.0, 0.0, None, 0, _p(self.wbuf), _stream(self.dev))
        _lib.check(rc, "adrtnet_adam")

    # ---- buffers -------------------------------------------------------------
    def _buffers(self, B, H, W):
        key = (B, H, W)
        if key in self._bufs:
            return self._bufs[key]
        if not _sizes_ok(H, W):
            raise ValueError("image sides must be powers of two, at least 128")

        def act(level, c):
            return torch.empty((B, H >> level, W >> level, c), dtype=torch.bfloat16, device=self.dev)

        b = {}
        for nm, lv, c in [("a0", 0, 32), ("e0", 0, 32), ("d0", 0, 32), ("f0", 0, 32), ("u0", 0, 64),
                          ("p0", 1, 32), ("a1", 1, 64), ("e1", 1, 64), ("d1", 1, 64), ("f1", 1, 64), ("u1", 1, 128),
                          ("p1", 2, 64), ("a2", 2, 128), ("e2", 2, 128), ("d2", 2, 128), ("f2", 2, 128),
                          ("u2", 2, 256), ("p2", 3, 128), ("a3", 3, 256), ("e3", 3, 256),
                          # gradients
                          ("gf0", 0, 32), ("gd0", 0, 32), ("gu0", 0, 64), ("ge0", 0, 32), ("ga0", 0, 32),
                          ("gf1", 1, 64), ("gd1", 1, 64), ("gu1", 1, 128), ("gp0", 1, 32), ("ge1", 1, 64),
                          ("ga1", 1, 64), ("gf2", 2, 128), ("gd2", 2, 128), ("gu2", 2, 256), ("gp1", 2, 64),
                          ("ge2", 2, 128), ("ga2", 2, 128), ("ge3", 3, 256), ("ga3", 3, 256), ("gp2", 3, 128)]:
            b[nm] = act(lv, c)
        b["out"] = torch.empty((B, H, W), dtype=torch.float32, device=self.dev)
        b["gout"] = torch.empty((B, H, W), dtype=torch.float32, device=self.dev)
        b["dres"] = torch.empty((B, H, W), dtype=torch.float32, device=self.dev)
        b["loss"] = torch.zeros(1, dtype=torch.float32, device=self.dev)
        self._bufs[key] = b
        return b

    # ---- kernels -------------------------------------------------------------
    def _conv(self, x, name, out, B, h, w, addend=None, mask=None, relu=True, bias=True, grad=False):
        ci, co = self._shape(name)
        if grad:
            ci, co = co, ci
        rc = self.lib.adrtnet_conv3x3(_p(x), ci, _p(self.wt(name, transposed=grad)), co,
                                      _p(self.view(name + "_b")) if bias else None, _p(addend), _p(mask),
                                      1 if relu else 0, _p(out), B, h, w, _stream(self.dev))
        _lib.check(rc, "adrtnet_conv3x3")

    def _wgrad(self, x, gy, name, B, h, w):
        ci, co = self._shape(name)
        rc = self.lib.adrtnet_conv3x3_wgrad(_p(x), ci, _p(gy), co, _p(self.view(name + "_w", self.grads)), B, h, w,
                                            _stream(self.dev))
        _lib.check(rc, "adrtnet_conv3x3_wgrad")
        rc = self.lib.adrtnet_bias_grad(_p(gy), _p(self.view(name + "_b", self.grads)), B * h * w, co,
                                        _stream(self.dev))
        _lib.check(rc, "adrtnet_bias_grad")

    def _shape(self, name):
        for nm, ci, co in LAYERS:
            if nm == name:
                return ci, co
        raise KeyError(name)

    def _call(self, fn, *args):
        _lib.check(getattr(self.lib, fn)(*args, _stream(self.dev)), fn)

    # ---- forward / backward ----------------------------------------------------
    def forward(self, u: torch.Tensor) -> torch.Tensor:
        """u: (B, H, W) float32 CUDA, already scaled; returns the (B, H, W)
        float32 network output (a buffer reused by the next call of the same
        shape)."""
        if not (u.is_cuda and u.dtype == torch.float32 and u.ndim == 3 and u.is_contiguous()):
            raise TypeError("forward expects a contiguous float32 CUDA tensor (B, H, W)")
        B, H, W = u.shape
        b = self._buffers(B, H, W)
        L = [(H >> k, W >> k) for k in range(4)]
        self._call("adrtnet_conv_in", _p(u), _p(self.view("in_w")), _p(self.view("in_b")), _p(b["a0"]), B, H, W)
        self._conv(b["a0"], "enc0b", b["e0"], B, *L[0])
        self._call("adrtnet_pool2", _p(b["e0"]), _p(b["p0"]), B, *L[0], 32)
        self._conv(b["p0"], "enc1a", b["a1"], B, *L[1])
        self._conv(b["a1"], "enc1b", b["e1"], B, *L[1])
        self._call("adrtnet_pool2", _p(b["e1"]), _p(b["p1"]), B, *L[1], 64)
        self._conv(b["p1"], "enc2a", b["a2"], B, *L[2])
        self._conv(b["a2"], "enc2b", b["e2"], B, *L[2])
        self._call("adrtnet_pool2", _p(b["e2"]), _p(b["p2"]), B, *L[2], 128)
        self._conv(b["p2"], "enc3a", b["a3"], B, *L[3])
        self._conv(b["a3"], "enc3b", b["e3"], B, *L[3])
        self._call("adrtnet_up2", _p(b["e3"]), _p(b["u2"]), B, *L[3], 256)
        self._conv(b["u2"], "dec2a", b["d2"], B, *L[2], addend=b["e2"])
        self._conv(b["d2"], "dec2b", b["f2"], B, *L[2])
        self._call("adrtnet_up2", _p(b["f2"]), _p(b["u1"]), B, *L[2], 128)
        self._conv(b["u1"], "dec1a", b["d1"], B, *L[1], addend=b["e1"])
        self._conv(b["d1"], "dec1b", b["f1"], B, *L[1])
        self._call("adrtnet_up2", _p(b["f1"]), _p(b["u0"]), B, *L[1], 64)
        self._conv(b["u0"], "dec0a", b["d0"], B, *L[0], addend=b["e0"])
        self._conv(b["d0"], "dec0b", b["f0"], B, *L[0])
        self._call("adrtnet_conv_out", _p(b["f0"]), _p(self.view("out_w")), _p(self.view("out_b")), _p(b["out"]),
                   B, H, W)
        return b["out"]

    def backward(self, u: torch.Tensor, gout: torch.Tensor) -> None:
        """Accumulates parameter gradients (+=) for the last forward(u) given
        d loss / d out."""
        B, H, W = u.shape
        b = self._buffers(B, H, W)
        L = [(H >> k, W >> k) for k in range(4)]
        G = self.grads
        self._call("adrtnet_conv_out_bwd", _p(gout), _p(self.view("out_w")), _p(b["f0"]), _p(b["gf0"]),
                   _p(self.view("out_w", G)), _p(self.view("out_b", G)), B, H, W)
        # decoder, level 0
        self._wgrad(b["d0"], b["gf0"], "dec0b", B, *L[0])
        self._conv(b["gf0"], "dec0b", b["gd0"], B, *L[0], mask=b["d0"], relu=False, bias=False, grad=True)
        self._wgrad(b["u0"], b["gd0"], "dec0a", B, *L[0])
        self._conv(b["gd0"], "dec0a", b["gu0"], B, *L[0], relu=False, bias=False, grad=True)
        self._call("adrtnet_up2_bwd", _p(b["gu0"]), _p(b["f1"]), _p(b["gf1"]), B, *L[1], 64)
        # level 1
        self._wgrad(b["d1"], b["gf1"], "dec1b", B, *L[1])
        self._conv(b["gf1"], "dec1b", b["gd1"], B, *L[1], mask=b["d1"], relu=False, bias=False, grad=True)
        self._wgrad(b["u1"], b["gd1"], "dec1a", B, *L[1])
        self._conv(b["gd1"], "dec1a", b["gu1"], B, *L[1], relu=False, bias=False, grad=True)
        self._call("adrtnet_up2_bwd", _p(b["gu1"]), _p(b["f2"]), _p(b["gf2"]), B, *L[2], 128)
        # level 2
        self._wgrad(b["d2"], b["gf2"], "dec2b", B, *L[2])
        self._conv(b["gf2"], "dec2b", b["gd2"], B, *L[2], mask=b["d2"], relu=False, bias=False, grad=True)
        self._wgrad(b["u2"], b["gd2"], "dec2a", B, *L[2])
        self._conv(b["gd2"], "dec2a", b["gu2"], B, *L[2], relu=False, bias=False, grad=True)
        self._call("adrtnet_up2_bwd", _p(b["gu2"]), _p(b["e3"]), _p(b["ge3"]), B, *L[3], 256)
        # bottom
        self._wgrad(b["a3"], b["ge3"], "enc3b", B, *L[3])
        self._conv(b["ge3"], "enc3b", b["ga3"], B, *L[3], mask=b["a3"], relu=False, bias=False, grad=True)
        self._wgrad(b["p2"], b["ga3"], "enc3a", B, *L[3])
        self._conv(b["ga3"], "enc3a", b["gp2"], B, *L[3], relu=False, bias=False, grad=True)
        # encoder, level 2: e2 feeds pool and the dec2a skip
        self._call("adrtnet_pool2_bwd", _p(b["gp2"]), _p(b["gd2"]), _p(b["e2"]), _p(b["ge2"]), B, *L[2], 128)
        self._wgrad(b["a2"], b["ge2"], "enc2b", B, *L[2])
        self._conv(b["ge2"], "enc2b", b["ga2"], B, *L[2], mask=b["a2"], relu=False, bias=False, grad=True)
        self._wgrad(b["p1"], b["ga2"], "enc2a", B, *L[2])
        self._conv(b["ga2"], "enc2a", b["gp1"], B, *L[2], relu=False, bias=False, grad=True)
        # level 1
        self._call("adrtnet_pool2_bwd", _p(b["gp1"]), _p(b["gd1"]), _p(b["e1"]), _p(b["ge1"]), B, *L[1], 64)
        self._wgrad(b["a1"], b["ge1"], "enc1b", B, *L[1])
        self._conv(b["ge1"], "enc1b", b["ga1"], B, *L[1], mask=b["a1"], relu=False, bias=False, grad=True)
        self._wgrad(b["p0"], b["ga1"], "enc1a", B, *L[1])
        self._conv(b["ga1"], "enc1a", b["gp0"], B, *L[1], relu=False, bias=False, grad=True)
        # level 0
        self._call("adrtnet_pool2_bwd", _p(b["gp0"]), _p(b["gd0"]), _p(b["e0"]), _p(b["ge0"]), B, *L[0], 32)
        self._wgrad(b["a0"], b["ge0"], "enc0b", B, *L[0])
        self._conv(b["ge0"], "enc0b", b["ga0"], B, *L[0], mask=b["a0"], relu=False, bias=False, grad=True)
        self._call("adrtnet_conv_in_wgrad", _p(u), _p(b["ga0"]), _p(self.view("in_w", G)), _p(self.view("in_b", G)),
                   B, H, W)

    def adam(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        self.step_count += 1
        rc = self.lib.adrtnet_adam(_p(self.params), _p(self.grads), _p(self.m), _p(self.v), _p(self.segs), self.nseg,
                                   self.n_params, lr, beta1, beta2, eps, _p(self.step_count), 1, _p(self.wbuf),
                                   _stream(self.dev))
        _lib.check(rc, "adrtnet_adam")

    def loss_and_grad(self, out, target, scale=1.0):
        """Loss and d loss / d out for d = scale * out - target:
        (alpha |d|^2 + mu d.(A^T A)^k d) / numel, with (alpha, mu, k) =
        self.loss_terms.  k = 0 is the mean squared error; k = 1 adds the
        energy norm |A d|^2 that CG on the normal equations minimises; k = 2
        the normal-equation residual |A^T A d|^2 that its stopping rule
        measures."""
        b = self._buffers(*out.shape)
        b["loss"].zero_()
        n = out.numel()
        self._call("adrtnet_diff", _p(out), _p(target), scale, _p(b["dres"]), n)
        alpha, mu, k = self.loss_terms
        e = None
        if k > 0 and mu != 0.0:
            e = b["dres"]
            for _ in range(k):
                e = _adjoint(_adrt(e))
        self._call("adrtnet_loss_grad", _p(b["dres"]), _p(e), alpha, mu if e is not None else 0.0, scale,
                   _p(b["gout"]), _p(b["loss"]), n)
        return b["gout"], b["loss"]

    def train_step(self, u, target, lr=1e-3):
        self.grads.zero_()
        out = self.forward(u)
        gout, loss = self.loss_and_grad(out, target)
        self.backward(u, gout)
        self.adam(lr)
        return loss

    def check_status(self):
        _lib.check(self.lib.adrtnet_status(_stream(self.dev)), "adrtnet kernels")

    # ---- inference ------------------------------------------------------------
    def predict(self, b: torch.Tensor, batch: int = 256) -> torch.Tensor:
        """Starting images x0 (B, n, n) for data b (B, 4, 2n-1, n)."""
        bt = _adjoint(b.contiguous())
        out = torch.empty_like(bt)
        for i in range(0, bt.shape[0], batch):
            u = (bt[i:i + batch] * self.in_scale).contiguous()
            out[i:i + batch] = self.forward(u)
        return out


class _GraphedTrainer:
    """One training step captured in a CUDA graph on static input buffers."""

    def __init__(self, net: PreconditionerNet, batch: int, n: int, lr: float):
        self.net = net
        self.u = torch.zeros((batch, n, n), dtype=torch.float32, device=net.dev)
        self.t = torch.zeros_like(self.u)
        self.lr = lr
        s = torch.cuda.Stream(device=net.dev)
        s.wait_stream(torch.cuda.current_stream(net.dev))
        # Warm-up outside the graph must not change the parameters: run the
        # pieces without the Adam update.
        with torch.cuda.stream(s):
            net.grads.zero_()
            out = net.forward(self.u)
            gout, _ = net.loss_and_grad(out, self.t)
            net.backward(self.u, gout)
        torch.cuda.current_stream(net.dev).wait_stream(s)
        torch.cuda.synchronize(net.dev)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.loss = net.train_step(self.u, self.t, lr)

    def step(self, u, t):
        self.u.copy_(u, non_blocking=True)
        self.t.copy_(t, non_blocking=True)
        self.graph.replay()
        return self.loss


@dataclass
class TrainLog:
    losses: list
    seconds: float
    steps: int


def training_pairs(count: int, n: int, seed: int, noise: float = 1e-3, tol: float = 1e-5, device="cuda",
                   chunk: int = 512):
    """(b, x_cg) pairs: ellipse phantoms -> adrt -> Gaussian noise of
    `noise` * max|b| per image -> plain CG to `tol`."""
    from . import cg as cgmod
    from .data import ellipse_phantoms

    bs, xs = [], []
    for i in range(0, count, chunk):
        k = min(chunk, count - i)
        xt = ellipse_phantoms(k, n, seed=seed + i, device=device)
        b = _adrt(xt)
        sigma = noise * b.abs().amax(dim=(1, 2, 3), keepdim=True)
        g = torch.Generator(device=device)
        g.manual_seed(seed * 7919 + i)
        b = b + sigma * torch.randn(b.shape, generator=g, device=device)
        res = cgmod.cg(b, tol=tol, max_iters=2000, graph=True)
        bs.append(b)
        xs.append(res.x)
    return torch.cat(bs), torch.cat(xs)


def normal_op_norm(n: int, device="cuda", iters: int = 30) -> float:
    """Largest eigenvalue of A^T A on n x n images (power iteration)."""
    g = torch.Generator(device=device)
    g.manual_seed(12345)
    x = torch.rand((1, n, n), generator=g, device=device)
    lam = 0.0
    for _ in range(iters):
        y = _adjoint(_adrt(x))
        lam = float(y.norm() / x.norm())
        x = y / y.norm()
    return lam


def train(net: PreconditionerNet, b: torch.Tensor, x_cg: torch.Tensor, *, epochs: int = 10, batch: int = 16,
          lr: float = 1e-3, seed: int = 0, graph: bool = True, loss_power: int = 0, loss_mu: float = 1.0,
          loss_alpha: float = 1.0) -> TrainLog:
    """Fits u = s * A^T b -> x_cg; s is set from the data so that u and x_cg
    have the same mean norm.  Loss: loss_alpha |d|^2 + loss_mu d.(A^T A /
    lambda_max)^loss_power d for d = x0 - x_cg.  Learning rate `lr` for the
    first 70 % of the epochs, lr / 10 after (each phase one captured
    training step)."""
    import time

    n = b.shape[-1]
    if loss_power > 0:
        lam = normal_op_norm(n, net.dev)
        net.loss_terms = (loss_alpha, loss_mu / lam ** loss_power, loss_power)
    else:
        net.loss_terms = (loss_alpha, 0.0, 0)
    bt = _adjoint(b.contiguous())
    net.in_scale = float(x_cg.norm() / bt.norm())
    u_all = bt * net.in_scale
    N = u_all.shape[0]
    gen = torch.Generator(device="cpu").manual_seed(seed)
    losses = []
    steps = 0
    torch.cuda.synchronize(net.dev)
    t0 = time.perf_counter()
    trainer = None
    phase_lr = None
    for ep in range(epochs):
        lr_ep = lr if ep < max(1, int(0.7 * epochs)) else lr / 10
        if graph and lr_ep != phase_lr:
            trainer = _GraphedTrainer(net, batch, n, lr_ep)
            phase_lr = lr_ep
        perm = torch.randperm(N, generator=gen).to(net.dev)
        ep_loss = torch.zeros((), dtype=torch.float32, device=net.dev)
        nb = N // batch
        for k in range(nb):
            idx = perm[k * batch:(k + 1) * batch]
            if graph:
                loss = trainer.step(u_all[idx], x_cg[idx])
            else:
                loss = net.train_step(u_all[idx].contiguous(), x_cg[idx].contiguous(), lr_ep)
            ep_loss += loss[0]
            steps += 1
        losses.append(float(ep_loss) / max(1, nb))
    torch.cuda.synchronize(net.dev)
    net.check_status()
    return TrainLog(losses, time.perf_counter() - t0, steps)


def learned_cg(net: PreconditionerNet, b: torch.Tensor, *, tol: float = 1e-4, max_iters: int = 1000,
               graph: bool = True, check_every: int = 4, precond=None):
    """CG from the network's starting image (preconditioned CG with
    `precond`); same stopping rule as plain CG."""
    from . import cg as cgmod

    x0 = net.predict(b)
    return cgmod.cg(b, x0=x0, tol=tol, max_iters=max_iters, graph=graph, check_every=check_every,
                    precond=precond)
