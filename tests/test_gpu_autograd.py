"""Differentiable ADRT: the backward is the exact transpose.

Checks: the adjoint kernel equals the reference's transpose
truncate(bdrt(y)) summed over quadrants (tests/test_bdrt.py:310-325) bit for
bit; the dot-product test <A x, y> = <x, A^T y> in float64 to rounding; central
finite differences in float64 at n = 32, batch 8, step 1e-6 (gradcheck); the
loss ||adrt(x) - y||^2 on 512 x 512 images with the data model of the
differentiable workload (y = adrt(phantom) + Gaussian noise of 1e-3 max|y|)."""

import numpy as np
import pytest
import torch

import adrt_gb300 as adrt
from adrt_gb300 import autograd as ag
from adrt_gb300.data import ellipse_phantoms
from conftest import bits_equal

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dt", [torch.float32, torch.float64])
@pytest.mark.parametrize("n,b", [(1, 3), (2, 2), (8, 3), (64, 2), (256, 1), (1024, 1)])
def test_adjoint_kernel_matches_reference_composition(oracle_mod, dt, n, b):
    g = torch.Generator(device="cuda")
    g.manual_seed(n)
    y = torch.randn((b, 4, 2 * n - 1, n), generator=g, device="cuda", dtype=dt)
    got = ag.adjoint(y).cpu().numpy()
    want = oracle_mod.adjoint(y.cpu().numpy())
    assert bits_equal(got, want)


@pytest.mark.parametrize("n", [16, 64, 256])
def test_dot_product(n):
    g = torch.Generator(device="cuda")
    g.manual_seed(7)
    x = torch.randn((4, n, n), generator=g, device="cuda", dtype=torch.float64)
    y = torch.randn((4, 4, 2 * n - 1, n), generator=g, device="cuda", dtype=torch.float64)
    lhs = (ag.adrt(x) * y).sum(dim=(1, 2, 3))
    rhs = (x * ag.adjoint(y)).sum(dim=(1, 2))
    rel = ((lhs - rhs).abs() / lhs.abs().clamp_min(1e-300)).max().item()
    assert rel < 1e-12, rel


def test_gradcheck_finite_differences():
    g = torch.Generator(device="cuda")
    g.manual_seed(3)
    x = torch.randn((8, 32, 32), generator=g, device="cuda", dtype=torch.float64, requires_grad=True)
    assert torch.autograd.gradcheck(ag.adrt, (x,), eps=1e-6, atol=1e-7, rtol=1e-6)
    y = torch.randn((2, 4, 15, 8), generator=g, device="cuda", dtype=torch.float64, requires_grad=True)
    assert torch.autograd.gradcheck(ag.adjoint, (y,), eps=1e-6, atol=1e-7, rtol=1e-6)


def test_least_squares_gradient_512():
    n, b = 512, 4
    x_true = ellipse_phantoms(b, n, seed=11, device="cuda")
    y = adrt.adrt(x_true)
    y = y + 1e-3 * y.abs().max() * torch.randn_like(y)
    x = torch.zeros_like(x_true, requires_grad=True)
    loss = ((ag.adrt(x) - y) ** 2).sum()
    loss.backward()
    # d/dx ||Ax - y||^2 at x = 0 is -2 A^T y.
    want = -2.0 * ag.adjoint(y)
    torch.testing.assert_close(x.grad, want, rtol=1e-6, atol=1e-3)
