"""Batched full-multigrid inverse: every image's result equals the
single-array iadrt_fmg (same iterations, same stopping rule) bit for bit."""

import pytest
import torch

import adrt_gb300 as adrt
from adrt_gb300.data import ellipse_phantoms, uniform_images
from adrt_gb300.ragged import iadrt_fmg_ragged

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [8, 32, 128])
@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("max_iters", [None, 1, 3])
def test_batched_matches_single(n, dtype, max_iters):
    x = torch.cat([ellipse_phantoms(3, n, seed=11, device="cuda", dtype=dtype),
                   uniform_images(2, n, seed=12, device="cuda", dtype=dtype)])
    y = adrt.adrt(x)
    got = adrt.iadrt_fmg_batched(y, max_iters=max_iters)
    assert got.shape == (5, n, n) and got.dtype == dtype
    for i in range(5):
        want = adrt.iadrt_fmg(y[i], max_iters=max_iters)
        assert torch.equal(got[i], want), i


def test_ragged_groups_by_size():
    ys = [adrt.adrt(ellipse_phantoms(1, n, seed=20 + i, device="cuda")[0]) for i, n in enumerate([16, 64, 16, 32])]
    got = iadrt_fmg_ragged(ys)
    for y, g in zip(ys, got):
        assert torch.equal(g, adrt.iadrt_fmg(y))


def test_rejects():
    y = adrt.adrt(torch.zeros((2, 16, 16), device="cuda"))
    with pytest.raises(ValueError):
        adrt.iadrt_fmg_batched(y[0])
    with pytest.raises(ValueError):
        adrt.iadrt_fmg_batched(y, max_iters=0)
