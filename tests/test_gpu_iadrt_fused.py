"""The exact inverse with its last five stages fused into one sweep (one warp
per group of 32 chains, shared-memory rings for the levels in between)
against the oracle, bit for bit: arbitrary (4, 2n-1, n) arrays with signed
zeros, infinities and NaNs (the recurrences propagate them along whole
chains), float32 and float64, n = 32 (all five stages fused) up to 1024.

Reference: src/adrt/adrt_cdefs_iadrt.hpp:53-105 (iadrt_core stages)."""

import numpy as np
import pytest
import torch

import adrt_gb300 as adrt
from conftest import bits_equal, first_mismatch

pytestmark = pytest.mark.gpu


def _hard(rng, b, n, dt):
    y = rng.standard_normal((b, 4, 2 * n - 1, n)).astype(dt)
    y[rng.random(y.shape) < 0.02] = -0.0
    y[:, :, -3:, :] = np.where(rng.random((b, 4, 3, n)) < 0.5, -0.0, y[:, :, -3:, :])
    y[:, :, :, rng.integers(0, n, size=2)] = -0.0
    y[0, 1, rng.integers(0, 2 * n - 1), rng.integers(0, n)] = np.inf
    y[-1, 2, rng.integers(0, 2 * n - 1), rng.integers(0, n)] = np.nan
    return y


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("n,b", [(32, 3), (64, 2), (128, 2), (512, 1), (1024, 1)])
def test_iadrt_fused_bit_exact(oracle_mod, dt, n, b):
    if dt == np.float64 and n == 1024:
        pytest.skip("float64 covered to n = 512")
    rng = np.random.default_rng(n * 7 + b)
    y = _hard(rng, b, n, dt)
    got = adrt.iadrt(torch.from_numpy(y).cuda()).cpu().numpy()
    want = oracle_mod.iadrt(y)
    assert bits_equal(got, want), first_mismatch(got, want)


def test_iadrt_fused_many_images(oracle_mod):
    # 96 images at n = 256 (adrt outputs): one batched call, compared with
    # the per-image call and, for three images, with the oracle.  (The exact
    # inverse is ill-conditioned; the comparison is bit for bit, not with the
    # original image.)
    g = torch.Generator(device="cuda")
    g.manual_seed(3)
    x = torch.rand((96, 256, 256), generator=g, device="cuda", dtype=torch.float64)
    y = adrt.adrt(x)
    inv = adrt.iadrt(y)
    for i in (0, 37, 95):
        assert torch.equal(inv[i], adrt.iadrt(y[i]))
        want = oracle_mod.iadrt(y[i].cpu().numpy())
        assert bits_equal(inv[i].cpu().numpy(), want)
