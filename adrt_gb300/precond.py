"""Learned convolution preconditioner for CG on the ADRT normal equations.

M = convolution with a (2h+1) x (2h+1) kernel K ("same" size, zero padding),
applied by the library's ``adrt_gb300_precond_conv`` kernel.  K is learned as
a least-squares approximate inverse of the normal operator A^T A:

    minimise  sum_s || K * (A^T A e_s) - e_s ||^2

over noise images e_s whose spectrum is |w|^tilt (tilt = 0: white noise,
every frequency weighted equally; a slight low-frequency tilt of -0.25
measured 9.9 instead of 11.0 PCG iterations for an 11 x 11 kernel on noisy
256 x 256 phantoms), with K restricted to the symmetries of the
square (invariant under the eight flips and transposes), so that M is
symmetric.  M is positive definite when K's symbol
sum_d K[d] cos(w . d) is positive at every frequency w; ``fit`` checks that
on a fine frequency grid and raises the centre weight if needed.

A^T A behaves like a convolution with a kernel whose symbol falls as 1/|w|
(the continuous Radon transform's normal operator), so the learned K acts
like a short ramp filter; on 256 x 256 phantoms preconditioned CG needs about
a third of plain CG's iterations for the same tolerance.
"""

from __future__ import annotations

import ctypes
import json

import numpy as np
import torch

from . import _lib
from ._wrappers import float_code

__all__ = ["ConvPreconditioner", "basis", "fit"]

MAX_H = 7


class ConvPreconditioner:
    """y = K * x per image; K: (2h+1, 2h+1) float64 weights (host)."""

    def __init__(self, weights):
        w = np.ascontiguousarray(np.asarray(weights, dtype=np.float64))
        if w.ndim != 2 or w.shape[0] != w.shape[1] or w.shape[0] % 2 != 1:
            raise ValueError("weights must be a (2h+1, 2h+1) array")
        self.h = (w.shape[0] - 1) // 2
        if self.h > MAX_H:
            raise ValueError(f"kernel half-width must be at most {MAX_H}")
        self.weights = w
        self._cw = w.ctypes.data_as(ctypes.POINTER(ctypes.c_double))

    def apply(self, x: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        """M x for a batch (B, n, n) of images on the device."""
        if not (isinstance(x, torch.Tensor) and x.is_cuda and x.ndim == 3 and x.shape[-1] == x.shape[-2]):
            raise TypeError("apply expects a CUDA tensor of shape (B, n, n)")
        x = x.contiguous()
        if out is None:
            out = torch.empty_like(x)
        rc = _lib.load().adrt_gb300_precond_conv(x.data_ptr(), out.data_ptr(), x.shape[0], x.shape[-1], self._cw,
                                                 self.h, float_code(x),
                                                 torch.cuda.current_stream(x.device).cuda_stream)
        _lib.check(rc, "precond_conv")
        return out

    def apply_dot(self, x: torch.Tensor, out: torch.Tensor, dot: torch.Tensor, workspace: torch.Tensor) -> None:
        """out = M x and dot[i] = <x_i, (M x)_i> (float64) in one kernel;
        `workspace` from ``dot_workspace``."""
        rc = _lib.load().adrt_gb300_precond_conv_dot(x.data_ptr(), out.data_ptr(), x.shape[0], x.shape[-1],
                                                     self._cw, self.h, float_code(x), dot.data_ptr(),
                                                     workspace.data_ptr(), workspace.numel(),
                                                     torch.cuda.current_stream(x.device).cuda_stream)
        _lib.check(rc, "precond_conv_dot")

    @staticmethod
    def dot_workspace(batch: int, n: int, device) -> torch.Tensor:
        size = _lib.load().adrt_gb300_precond_dot_workspace_size(batch, n)
        return torch.empty(max(int(size), 1), dtype=torch.uint8, device=device)

    def symbol_range(self, grid: int = 512) -> tuple[float, float]:
        """(min, max) of the symbol sum_d K[d] cos(w . d) over a grid x grid
        frequency lattice."""
        return symbol_range(self.weights, grid)

    def save(self, path: str) -> None:
        with open(path, "w") as f:
            json.dump({"weights": self.weights.tolist()}, f)

    @classmethod
    def load(cls, path: str) -> "ConvPreconditioner":
        with open(path) as f:
            return cls(json.load(f)["weights"])


def symbol_range(K: np.ndarray, grid: int = 512) -> tuple[float, float]:
    h = (K.shape[0] - 1) // 2
    emb = np.zeros((grid, grid))
    for i in range(-h, h + 1):
        for j in range(-h, h + 1):
            emb[i % grid, j % grid] += K[h + i, h + j]
    s = np.real(np.fft.fft2(emb))
    return float(s.min()), float(s.max())


def basis(h: int) -> list[np.ndarray]:
    """Kernels spanning the (2h+1)^2 kernels invariant under the square's
    eight symmetries: one per orbit {(+-i, +-j), (+-j, +-i)}, 0 <= j <= i <= h."""
    out = []
    for i in range(h + 1):
        for j in range(i + 1):
            B = np.zeros((2 * h + 1, 2 * h + 1))
            for a, b in {(i, j), (j, i)}:
                for sa in (1, -1):
                    for sb in (1, -1):
                        B[h + sa * a, h + sb * b] = 1.0
            out.append(B)
    return out


def _samples(samples: int, n: int, seed: int, tilt: float) -> np.ndarray:
    """Gaussian noise images whose spectrum is shaped by |w|^tilt (0: white)."""
    e = np.random.default_rng(seed).standard_normal((samples, n, n))
    if tilt:
        f = np.fft.fftfreq(n)
        w = np.sqrt(f[:, None] ** 2 + f[None, :] ** 2)
        w[0, 0] = 1.0 / n
        e = np.real(np.fft.ifft2(np.fft.fft2(e) * w ** tilt))
    return e


def fit(n: int, h: int = 4, samples: int = 16, seed: int = 0, device="cuda",
        dtype=torch.float32, ridge_param: float = 0.0, tilt: float = 0.0) -> ConvPreconditioner:
    """Least-squares fit of K ~ (A^T A + 4 ridge_param I)^{-1} on noise images
    with spectrum |w|^tilt (white for tilt = 0; untimed set-up work)."""
    from .cg import normal_op

    if not 0 <= h <= MAX_H:
        raise ValueError(f"h must be in [0, {MAX_H}]")
    e = torch.from_numpy(_samples(samples, n, seed, tilt)).to(device=device, dtype=dtype)
    y = normal_op(e, 4.0 * ridge_param)
    Bs = basis(h)
    feats = torch.stack([ConvPreconditioner(B).apply(y) for B in Bs]).reshape(len(Bs), -1).double()
    G = (feats @ feats.T).cpu().numpy()
    rhs = (feats @ e.reshape(-1).double()).cpu().numpy()
    w = np.linalg.solve(G, rhs)
    K = sum(wi * B for wi, B in zip(w, Bs))
    lo, hi = symbol_range(K)
    if lo <= 1e-6 * hi:
        K[h, h] += 1e-6 * hi - lo
    return ConvPreconditioner(K)
