"""The register-level first pass of the float32 forward at n = 64 .. 512
(the first log2(n) - 5 stages, then the five-stage second pass) against the
oracle, bit for bit: signed zeros along whole rows and columns (the four
quadrants read rows from the right end and columns up and down), infinities
and NaNs near the row ends, and batches of several images.

Reference: src/adrt/adrt_cdefs_adrt.hpp:56-96 (adrt_core stages),
:123-186 (quadrant flips)."""

import numpy as np
import pytest
import torch

import adrt_gb300 as adrt
from conftest import bits_equal, first_mismatch

pytestmark = pytest.mark.gpu


def _hard_image(rng, b, n):
    x = rng.standard_normal((b, n, n)).astype(np.float32)
    x[:, rng.integers(0, n, size=3), :] = -0.0
    x[:, :, rng.integers(0, n, size=3)] = -0.0
    x[rng.random(x.shape) < 0.02] = -0.0
    for v in (np.inf, -np.inf, np.nan):
        x[rng.random(x.shape) < 2e-4] = v
    # corners and edges: the first and last offsets of every quadrant's rows
    x[:, :2, :] *= -1
    x[:, -2:, -3:] = np.where(rng.random((b, 2, 3)) < 0.5, -0.0, x[:, -2:, -3:])
    return x


@pytest.mark.parametrize("n,b", [(64, 7), (128, 5), (256, 3), (512, 2)])
def test_first_pass_bit_exact(oracle_mod, n, b):
    rng = np.random.default_rng(n + 17)
    x = _hard_image(rng, b, n)
    got = adrt.adrt(torch.from_numpy(x).cuda()).cpu().numpy()
    want = oracle_mod.adrt(x)
    assert bits_equal(got, want), first_mismatch(got, want)


@pytest.mark.parametrize("n", [64, 128, 256, 512])
def test_first_pass_many_images(oracle_mod, n):
    # Enough images for several CTAs per SM at every size; all checked.
    b = 64 if n < 512 else 24
    g = torch.Generator(device="cuda")
    g.manual_seed(n)
    x = torch.rand((b, n, n), generator=g, device="cuda")
    got = adrt.adrt(x).cpu().numpy()
    want = oracle_mod.adrt(x.cpu().numpy())
    assert bits_equal(got, want), first_mismatch(got, want)
