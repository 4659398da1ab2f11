"""Learned convolution preconditioner and preconditioned CG: the convolution
kernel against torch's float64 CPU convolution, symmetry of the operator, the
least-squares fit, and PCG against a float64 SciPy CG on the oracle operator."""

import numpy as np
import pytest
import torch
import torch.nn.functional as F

import adrt_gb300 as adrt
from adrt_gb300 import cg as cgmod
from adrt_gb300 import precond
from adrt_gb300.data import ellipse_phantoms

pytestmark = pytest.mark.gpu


def _sym_kernel(h, seed):
    rng = np.random.default_rng(seed)
    return sum(rng.standard_normal() * B for B in precond.basis(h))


@pytest.mark.parametrize("n", [1, 5, 40, 64])
@pytest.mark.parametrize("h", [0, 2, 4, 7])
@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_conv_matches_torch(n, h, dtype):
    rng = np.random.default_rng(n * 10 + h)
    K = rng.standard_normal((2 * h + 1, 2 * h + 1))  # any kernel: the op is a correlation
    x = torch.from_numpy(rng.standard_normal((3, n, n)))
    want = F.conv2d(x[:, None], torch.from_numpy(K)[None, None], padding=h)[:, 0]
    got = precond.ConvPreconditioner(K).apply(x.to("cuda", dtype)).cpu().double()
    tol = 1e-5 if dtype == torch.float32 else 1e-12
    scale = want.abs().max().item() + 1e-30
    assert (got - want).abs().max().item() <= tol * scale * (2 * h + 1)


def test_symmetric_operator():
    M = precond.ConvPreconditioner(_sym_kernel(4, 1))
    g = torch.Generator(device="cuda")
    g.manual_seed(0)
    x = torch.randn((2, 64, 64), generator=g, device="cuda", dtype=torch.float64)
    y = torch.randn((2, 64, 64), generator=g, device="cuda", dtype=torch.float64)
    a = (M.apply(x) * y).sum().item()
    b = (x * M.apply(y)).sum().item()
    assert abs(a - b) <= 1e-12 * abs(a)


def test_fit_is_positive_definite_and_approximates_inverse():
    M = precond.fit(64, h=4, samples=8, seed=3)
    lo, hi = M.symbol_range()
    assert lo > 0 and hi > lo
    assert np.allclose(M.weights, M.weights.T) and np.allclose(M.weights, M.weights[::-1, ::-1])
    # On fresh white noise, M A^T A e is much closer to e than A^T A e scaled.
    g = torch.Generator(device="cuda")
    g.manual_seed(99)
    e = torch.randn((4, 64, 64), generator=g, device="cuda")
    y = cgmod.normal_op(e)
    err_m = ((M.apply(y) - e).norm() / e.norm()).item()
    s = (y * e).sum() / (y * y).sum()
    err_s = ((s * y - e).norm() / e.norm()).item()
    assert err_m < 0.5 * err_s


def _noisy(n, B, seed):
    xt = ellipse_phantoms(B, n, seed=seed, device="cuda")
    b = adrt.adrt(xt)
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    return xt, b + 1e-3 * b.abs().amax(dim=(1, 2, 3), keepdim=True) * torch.randn(b.shape, generator=g, device="cuda")


@pytest.mark.parametrize("graph", [False, True])
def test_pcg_reaches_tolerance_with_fewer_iterations(graph):
    n, B = 128, 8
    xt, b = _noisy(n, B, 71)
    M = precond.fit(n, h=4, samples=8, seed=5)
    plain = cgmod.cg(b, tol=1e-4, max_iters=300, graph=graph)
    pcg = cgmod.cg(b, tol=1e-4, max_iters=300, graph=graph, precond=M)
    assert (pcg.normal_residual <= 1.5e-4).all(), pcg.normal_residual
    assert pcg.iterations.double().mean() < 0.6 * plain.iterations.double().mean()
    # Both solve the same system to the same tolerance.
    d = (pcg.x - plain.x).reshape(B, -1).norm(dim=1) / plain.x.reshape(B, -1).norm(dim=1)
    assert (d < 5e-2).all()


def test_pcg_float64_matches_scipy_oracle(oracle_mod):
    from test_gpu_cg import scipy_cg

    n = 32
    xt = ellipse_phantoms(2, n, seed=5, device="cuda", dtype=torch.float64)
    b = adrt.adrt(xt)
    M = precond.fit(n, h=3, samples=8, seed=1, dtype=torch.float64)
    res = cgmod.cg(b, tol=1e-10, max_iters=2000, precond=M)
    for i in range(2):
        want = scipy_cg(oracle_mod, b[i].cpu().numpy(), 1e-12)
        got = res.x[i].cpu().numpy()
        assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-6
    assert (res.normal_residual <= 1e-9).all()


def test_pcg_compaction_and_graph_identical():
    n, B = 64, 12
    xt, b = _noisy(n, B, 83)
    b[: B // 2] *= 1e-3
    M = precond.fit(n, h=4, samples=8, seed=7)
    full = cgmod.cg(b, tol=1e-5, max_iters=400, compact=0.0, check_every=1, precond=M)
    comp = cgmod.cg(b, tol=1e-5, max_iters=400, compact=0.9, check_every=1, graph=True, precond=M)
    assert torch.equal(full.iterations, comp.iterations)
    assert torch.equal(full.x, comp.x)


@pytest.mark.parametrize("n", [5, 64, 100])
def test_fused_dot_matches_separate(n):
    M = precond.ConvPreconditioner(_sym_kernel(3, 2))
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    x = torch.randn((3, n, n), generator=g, device="cuda")
    out = torch.empty_like(x)
    dot = torch.empty(3, dtype=torch.float64, device="cuda")
    M.apply_dot(x, out, dot, M.dot_workspace(3, n, x.device))
    assert torch.equal(out, M.apply(x))
    want = (x.double() * out.double()).sum(dim=(1, 2))
    assert torch.allclose(dot, want, rtol=1e-5, atol=1e-6)
