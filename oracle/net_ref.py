"""CPU reference of the learned preconditioner network in plain PyTorch.

TEST INFRASTRUCTURE ONLY: used by tests/ as the checker of the network's
CUDA kernels (forward values and parameter gradients).  The ``adrt_gb300``
package never imports this module.

Same architecture and flat parameter layout as ``adrt_gb300.learned``:
per tensor-core layer weights [9][c_out][c_in] (tap = 3 * dy + dx over the
zero-padded 3 x 3 window, i.e. torch's conv2d cross-correlation with kernel
index [dy][dx]) then bias [c_out]; first layer weights [9][32] + bias [32];
last layer weights [9][32] + bias [1].  Computes in float32 or float64 with
autograd; the CUDA path rounds activations to bf16, so comparisons use
relative tolerances.
"""

from __future__ import annotations

import torch
import torch.nn.functional as F

LAYERS = (
    ("enc0b", 32, 32), ("enc1a", 32, 64), ("enc1b", 64, 64), ("enc2a", 64, 128), ("enc2b", 128, 128),
    ("enc3a", 128, 256), ("enc3b", 256, 256), ("dec2a", 256, 128), ("dec2b", 128, 128), ("dec1a", 128, 64),
    ("dec1b", 64, 64), ("dec0a", 64, 32), ("dec0b", 32, 32),
)


def offsets():
    """name -> (offset, count, shape of the torch conv weight or bias)."""
    out = {}
    off = 0

    def put(name, count, shape):
        nonlocal off
        out[name] = (off, count, shape)
        off += count

    put("in_w", 9 * 32, None)
    put("in_b", 32, None)
    for name, ci, co in LAYERS:
        put(name + "_w", 9 * ci * co, (ci, co))
        put(name + "_b", co, None)
    put("out_w", 9 * 32, None)
    put("out_b", 1, None)
    return out, off


def conv_weight(flat: torch.Tensor, ci: int, co: int) -> torch.Tensor:
    """[9][co][ci] -> torch (co, ci, 3, 3)."""
    return flat.reshape(3, 3, co, ci).permute(2, 3, 0, 1)


def forward(params: torch.Tensor, u: torch.Tensor) -> torch.Tensor:
    """params: flat vector; u: (B, H, W).  Returns (B, H, W)."""
    offs, _ = offsets()

    def get(name):
        o, c, _ = offs[name]
        return params[o:o + c]

    def conv(x, name, addend=None):
        ci, co = offs[name + "_w"][2]
        y = F.conv2d(x, conv_weight(get(name + "_w"), ci, co), get(name + "_b"), padding=1)
        if addend is not None:
            y = y + addend
        return F.relu(y)

    x = u[:, None]
    w_in = get("in_w").reshape(3, 3, 32).permute(2, 0, 1)[:, None]  # (32, 1, 3, 3)
    a0 = F.relu(F.conv2d(x, w_in, get("in_b"), padding=1))
    e0 = conv(a0, "enc0b")
    a1 = conv(F.avg_pool2d(e0, 2), "enc1a")
    e1 = conv(a1, "enc1b")
    a2 = conv(F.avg_pool2d(e1, 2), "enc2a")
    e2 = conv(a2, "enc2b")
    a3 = conv(F.avg_pool2d(e2, 2), "enc3a")
    e3 = conv(a3, "enc3b")
    up = lambda t: F.interpolate(t, scale_factor=2, mode="nearest")  # noqa: E731
    d2 = conv(up(e3), "dec2a", e2)
    f2 = conv(d2, "dec2b")
    d1 = conv(up(f2), "dec1a", e1)
    f1 = conv(d1, "dec1b")
    d0 = conv(up(f1), "dec0a", e0)
    f0 = conv(d0, "dec0b")
    w_out = get("out_w").reshape(3, 3, 32).permute(2, 0, 1)[None]  # (1, 32, 3, 3)
    return F.conv2d(f0, w_out, get("out_b"), padding=1)[:, 0]


def loss_and_grads(params: torch.Tensor, u: torch.Tensor, target: torch.Tensor):
    """mean((out - target)^2) and its gradient with respect to the flat
    parameter vector."""
    p = params.detach().clone().requires_grad_(True)
    out = forward(p, u)
    loss = ((out - target) ** 2).mean()
    loss.backward()
    return out.detach(), float(loss.detach()), p.grad.detach()
