"""The register-level bdrt passes (float32, 128 <= n <= 1024: the last five
forward stages undone by the first pass, the first L-5 by the second) against
the oracle, bit for bit: signed zeros, infinities and NaNs spread over whole rows,
dense near the row ends (where the reference's copy and zero rules act, in the
tiles the generic kernel keeps) and around the offsets where the register
tiles end; the truncated bdrt of the adjoint; batches large enough to need
several launches' worth of grid rows and chunks.

Reference: src/adrt/adrt_cdefs_bdrt.hpp:56-187 (bdrt_core, bdrt_basic),
src/adrt/_wrappers.py:283-284 (the transpose identity)."""

import numpy as np
import pytest
import torch

import adrt_gb300 as adrt
from adrt_gb300 import autograd as ag
from conftest import bits_equal, first_mismatch

pytestmark = pytest.mark.gpu


def _hard_input(rng, b, n, dtype=np.float32):
    C = 2 * n - 1
    y = rng.standard_normal((b, 4, C, n)).astype(dtype)
    # whole rows of signed zeros, scattered -0 / +inf / -inf / NaN
    y[:, :, rng.integers(0, C, size=8), :] = -0.0
    mask = rng.random(y.shape) < 0.01
    y[mask] = -0.0
    y[rng.random(y.shape) < 1e-4] = np.inf
    y[rng.random(y.shape) < 1e-4] = -np.inf
    y[rng.random(y.shape) < 1e-4] = np.nan
    # the last offsets of every row (copy/zero rules), and the offsets where
    # the register tiles hand over to the generic kernel (multiples of 448)
    y[:, :, C - 40 :, :] = np.where(rng.random((b, 4, 40, n)) < 0.5, -0.0, y[:, :, C - 40 :, :])
    for c in range(448, C, 448):
        y[:, :, max(0, c - 8) : c + 8, :] *= -1
    return y


@pytest.mark.parametrize("n,b", [(128, 5), (256, 3), (512, 2), (1024, 2)])
def test_bdrt_fast_bit_exact(oracle_mod, n, b):
    rng = np.random.default_rng(n)
    y = _hard_input(rng, b, n)
    got = adrt.bdrt(torch.from_numpy(y).cuda()).cpu().numpy()
    want = oracle_mod.bdrt(y)
    assert bits_equal(got, want), first_mismatch(got, want)


@pytest.mark.parametrize("n", [128, 256, 512, 1024])
def test_adjoint_fast_bit_exact(oracle_mod, n):
    rng = np.random.default_rng(n + 1)
    y = rng.standard_normal((2, 4, 2 * n - 1, n)).astype(np.float32)
    y[0, :, :, : n // 3] = -0.0
    got = ag.adjoint(torch.from_numpy(y).cuda()).cpu().numpy()
    want = oracle_mod.adjoint(y)
    assert bits_equal(got, want), first_mismatch(got, want)


@pytest.mark.parametrize("n,b", [(256, 40), (512, 12), (128, 64)])
def test_bdrt_fast_many_images(oracle_mod, n, b):
    # Many images: one chunk, one launch per pass; every image checked.
    g = torch.Generator(device="cuda")
    g.manual_seed(7)
    y = torch.randn((b, 4, 2 * n - 1, n), generator=g, device="cuda")
    got = adrt.bdrt(y).cpu().numpy()
    want = oracle_mod.bdrt(y.cpu().numpy())
    assert bits_equal(got, want), first_mismatch(got, want)


def test_bdrt_float64_unchanged(oracle_mod):
    # float64 keeps the generic passes (unpadded buffer rows).
    rng = np.random.default_rng(3)
    y = rng.standard_normal((1, 4, 1023, 512))
    got = adrt.bdrt(torch.from_numpy(y).cuda()).cpu().numpy()
    assert bits_equal(got, oracle_mod.bdrt(y))
