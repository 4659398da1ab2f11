"""Seeded synthetic inputs: uniform images and random-ellipse phantoms.

Phantom recipe (per image, its own seed = base seed + image index):
K ~ U{5..15} ellipses; centre uniform in a disk of radius 0.8 (r = 0.8 sqrt(u));
semi-axes U[0.05, 0.4]; rotation U[0, pi); intensity U[-0.5, 1.0]; the
ellipses' indicator functions weighted by intensity are summed on the
[-1, 1]^2 grid and the sum is clipped at 0.  Parameters are drawn on the host
with NumPy; the rasterisation runs on the device.
"""

from __future__ import annotations

import numpy as np
import torch


def ellipse_params(seed: int):
    rng = np.random.default_rng(seed)
    k = int(rng.integers(5, 16))
    r = 0.8 * np.sqrt(rng.random(k))
    t = 2 * np.pi * rng.random(k)
    cx, cy = r * np.cos(t), r * np.sin(t)
    a = rng.uniform(0.05, 0.4, k)
    b = rng.uniform(0.05, 0.4, k)
    phi = rng.uniform(0.0, np.pi, k)
    val = rng.uniform(-0.5, 1.0, k)
    return np.stack([cx, cy, a, b, phi, val], axis=1)


def ellipse_phantoms(batch: int, n: int, seed: int = 0, device="cuda", dtype=torch.float32):
    """(batch, n, n) phantoms; image i uses seed + i."""
    lin = torch.linspace(-1.0, 1.0, n, device=device, dtype=torch.float64)
    yy, xx = torch.meshgrid(lin, lin, indexing="ij")
    out = torch.empty((batch, n, n), device=device, dtype=dtype)
    for i in range(batch):
        p = torch.as_tensor(ellipse_params(seed + i), device=device)
        img = torch.zeros((n, n), device=device, dtype=torch.float64)
        for cx, cy, a, b, phi, val in p:
            dx, dy = xx - cx, yy - cy
            c, s = torch.cos(phi), torch.sin(phi)
            u = (dx * c + dy * s) / a
            v = (-dx * s + dy * c) / b
            img += val * ((u * u + v * v) <= 1.0)
        out[i] = img.clamp_min(0.0).to(dtype)
    return out


def uniform_images(batch: int, n: int, seed: int = 0, device="cuda", dtype=torch.float32):
    """(batch, n, n) i.i.d. uniform [0, 1) values from a seeded generator."""
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    return torch.rand((batch, n, n), generator=g, device=device, dtype=dtype)


def mixed_batch(batch: int, n: int, seed: int = 0, device="cuda", dtype=torch.float32):
    """First half uniform [0, 1), second half ellipse phantoms."""
    h = batch // 2
    x = torch.empty((batch, n, n), device=device, dtype=dtype)
    x[:h] = uniform_images(h, n, seed, device, dtype)
    x[h:] = ellipse_phantoms(batch - h, n, seed + 100_000, device, dtype)
    return x


RAGGED_SIZES = (32, 64, 128, 256, 512, 1024)
RAGGED_WEIGHTS = (0.3, 0.25, 0.2, 0.15, 0.07, 0.03)


def ragged_sizes(count: int, seed: int = 0):
    """Image sides of the ragged workload: N drawn from {32, ..., 1024} with
    weights {.3, .25, .2, .15, .07, .03}."""
    rng = np.random.default_rng(seed)
    return [int(v) for v in rng.choice(RAGGED_SIZES, size=count, p=RAGGED_WEIGHTS)]


def ragged_phantoms(count: int, seed: int = 0, device="cuda", dtype=torch.float32):
    """A list of `count` ellipse phantoms with sides from ragged_sizes."""
    return [ellipse_phantoms(1, n, seed + i, device, dtype)[0] for i, n in enumerate(ragged_sizes(count, seed))]
