"""Ragged batches in one persistent launch: every image's result equals the
regular transform bit for bit; an injected stall makes a device-side wait
expire, which the host reads as a timeout status while the context stays
usable."""

import numpy as np
import pytest
import torch

import adrt_gb300 as adrt
from adrt_gb300 import ragged
from adrt_gb300.data import ellipse_phantoms
from conftest import bits_equal

pytestmark = pytest.mark.gpu

ERR_TIMEOUT = 7


@pytest.mark.parametrize("dt", [torch.float32, torch.float64])
def test_ragged_matches_regular(dt):
    sizes = [1, 2, 1024, 4, 32, 64, 8, 128, 256, 512, 16, 64, 1024]
    g = torch.Generator(device="cuda")
    g.manual_seed(1)
    imgs = [torch.randn((n, n), generator=g, device="cuda", dtype=dt) for n in sizes]
    imgs[2][:100] = -0.0
    outs = ragged.adrt_ragged(imgs)
    for im, o in zip(imgs, outs):
        assert bits_equal(o.cpu().numpy(), adrt.adrt(im).cpu().numpy())


def test_ragged_round_trip_distribution():
    # Sizes drawn like the ragged workload (weights .3/.25/.2/.15/.07/.03 over
    # 32..1024), ellipse phantoms; exact inverse and FMG inverse round trips.
    rng = np.random.default_rng(0)
    choices = [32, 64, 128, 256, 512, 1024]
    sizes = rng.choice(choices, size=48, p=[0.3, 0.25, 0.2, 0.15, 0.07, 0.03])
    imgs = [ellipse_phantoms(1, int(n), seed=100 + i, device="cuda")[0] for i, n in enumerate(sizes)]
    outs = ragged.adrt_ragged(imgs)
    for im, o in zip(imgs, outs):
        assert bits_equal(o.cpu().numpy(), adrt.adrt(im).cpu().numpy())
    small = [(im, o) for im, o in zip(imgs, outs) if im.shape[0] <= 64]
    invs = ragged.iadrt_ragged([o for _, o in small])
    for (im, o), inv in zip(small, invs):
        assert bits_equal(inv.cpu().numpy(), adrt.iadrt(o).cpu().numpy())
    # Unbounded FMG (stops when the residual stops decreasing); float32 FMG
    # round trips at n <= 64 recover the image to about 1e-7 relative.
    fm = ragged.iadrt_fmg_ragged([o for _, o in small[:4]])
    for (im, _), x in zip(small[:4], fm):
        rel = (x - im).norm() / im.norm()
        assert rel < 1e-3, rel


def test_ragged_wait_expires_and_context_survives():
    imgs = [torch.rand((n, n), device="cuda") for n in (64, 1024, 32, 256)]
    # Image 1 waits for a first-pass tile that does not exist; 50 ms limit.
    views, status = ragged._launch(imgs, wait_ns=50_000_000, starve_image=1)
    assert status == ERR_TIMEOUT
    # The context is still usable and the regular path still exact.
    outs = ragged.adrt_ragged(imgs)
    for im, o in zip(imgs, outs):
        assert bits_equal(o.cpu().numpy(), adrt.adrt(im).cpu().numpy())


def test_ragged_rejects():
    with pytest.raises(ValueError, match="up to 1024"):
        ragged.adrt_ragged([torch.zeros((2048, 2048), device="cuda")])
    with pytest.raises(ValueError, match="power of two"):
        ragged.adrt_ragged([torch.zeros((6, 6), device="cuda")])


def test_ragged_plan_repeated_launches():
    # One plan, several back-to-back launches on one stream (descriptor
    # uploads staged through pinned memory), then a second plan whose
    # descriptors are larger: results equal the list API's bit for bit.
    sizes = [1024, 32, 256, 64, 1024, 128, 512]
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    imgs = [torch.randn((n, n), generator=g, device="cuda") for n in sizes]
    want = ragged.adrt_ragged(imgs)
    plan = ragged.RaggedPlan(sizes)
    packed = plan.packed_input(imgs)
    for _ in range(4):
        plan.launch(packed)
    assert plan.status() == 0
    for a, b in zip(plan.views(), want):
        assert bits_equal(a.cpu().numpy(), b.cpu().numpy())
    big = ragged.RaggedPlan(sizes * 40)
    big.launch(big.packed_input(imgs * 40))
    plan.launch(packed)
    assert big.status() == 0 and plan.status() == 0
    for a, b in zip(big.views(), want * 40):
        assert bits_equal(a.cpu().numpy(), b.cpu().numpy())
    with pytest.raises(ValueError, match="packed input"):
        plan.launch(packed[:-1])
