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


@pytest.mark.parametrize("n,b,dt", [(64, 640, np.float32), (256, 160, np.float32), (128, 320, np.float64)])
def test_iadrt_row_sweep_bit_exact(oracle_mod, n, b, dt):
    # Batches with at least 32 warps of chains per SM (4 b n >= 152 x 1024)
    # take the single-stage kernels' row sweep for the odd chains; each
    # image must equal its own (per-lane sweep) call and the oracle.
    assert 4 * b * n >= 152 * 1024
    rng = np.random.default_rng(n + b)
    y = _hard(rng, b, n, dt)
    yd = torch.from_numpy(y).cuda()
    got = adrt.iadrt(yd)
    g = got.cpu().numpy()
    for i in (0, 1, b // 2, b - 1):  # bit patterns: the last image holds a NaN
        one = adrt.iadrt(yd[i]).cpu().numpy()
        assert bits_equal(g[i], one), (i, first_mismatch(g[i], one))
    for i in (0, b - 1):
        want = oracle_mod.iadrt(y[i])
        assert bits_equal(g[i], want), first_mismatch(g[i], want)
