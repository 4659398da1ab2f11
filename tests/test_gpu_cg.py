"""Batched CG on the ADRT normal equations against a float64 SciPy CG oracle
on the CPU oracle operator (the reference recipe, docs/examples.cginverse.md:40-67)."""

import numpy as np
import pytest
import torch

import adrt_gb300 as adrt
from adrt_gb300 import cg as cgmod
from adrt_gb300.data import ellipse_phantoms

pytestmark = pytest.mark.gpu


def scipy_cg(oracle_mod, b, tol):
    sla = pytest.importorskip("scipy.sparse.linalg")
    n = b.shape[-1]

    def mv(v):
        return oracle_mod.adjoint(oracle_mod.adrt(v.reshape(n, n))).ravel()

    op = sla.LinearOperator((n * n, n * n), matvec=mv, dtype=np.float64)
    rhs = oracle_mod.adjoint(b).ravel()
    x, info = sla.cg(op, rhs, rtol=tol, maxiter=5000)
    assert info == 0
    return x.reshape(n, n)


def test_float64_matches_scipy_oracle(oracle_mod):
    n = 32
    xt = ellipse_phantoms(2, n, seed=5, device="cuda", dtype=torch.float64)
    b = adrt.adrt(xt)
    res = cgmod.cg(b, tol=1e-10, max_iters=2000)
    for i in range(2):
        want = scipy_cg(oracle_mod, b[i].cpu().numpy(), 1e-12)
        got = res.x[i].cpu().numpy()
        assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-6
    assert (res.normal_residual <= 1e-9).all()


@pytest.mark.parametrize("graph", [False, True])
def test_float32_noisy_phantoms_reach_tolerance(graph):
    n, B = 256, 8
    xt = ellipse_phantoms(B, n, seed=17, device="cuda")
    b = adrt.adrt(xt)
    sigma = 1e-3 * b.abs().amax(dim=(1, 2, 3), keepdim=True)
    g = torch.Generator(device="cuda")
    g.manual_seed(0)
    b = b + sigma * torch.randn(b.shape, generator=g, device="cuda")
    res = cgmod.cg(b, tol=1e-4, max_iters=300, graph=graph)
    assert (res.normal_residual <= 1.5e-4).all(), res.normal_residual
    assert (res.iterations > 5).all() and (res.iterations < 300).all()
    # Noise floor of the data residual at this noise level is about 6e-3.
    assert (res.data_residual < 2e-2).all()
    err = (res.x - xt).reshape(B, -1).norm(dim=1) / xt.reshape(B, -1).norm(dim=1)
    assert (err < 0.5).all()


def test_graph_and_eager_agree():
    n, B = 64, 4
    xt = ellipse_phantoms(B, n, seed=23, device="cuda")
    b = adrt.adrt(xt)
    r1 = cgmod.cg(b, tol=1e-5, max_iters=200, graph=False, check_every=1)
    r2 = cgmod.cg(b, tol=1e-5, max_iters=200, graph=True, check_every=1)
    assert torch.equal(r1.iterations, r2.iterations)
    assert torch.equal(r1.x, r2.x)


def test_warm_start_converges_faster():
    n, B = 64, 4
    xt = ellipse_phantoms(B, n, seed=29, device="cuda")
    b = adrt.adrt(xt)
    cold = cgmod.cg(b, tol=1e-5, max_iters=500)
    warm = cgmod.cg(b, x0=xt + 1e-3 * torch.randn_like(xt), tol=1e-5, max_iters=500)
    assert warm.iterations.sum() < cold.iterations.sum()


def test_graphed_forward_matches_eager():
    from adrt_gb300.graphs import GraphedCall

    x = torch.rand((2, 1024, 1024), device="cuda")
    g = GraphedCall(adrt.adrt, x.clone())
    for seed in range(3):
        torch.manual_seed(seed)
        xn = torch.rand((2, 1024, 1024), device="cuda")
        assert torch.equal(g(xn), adrt.adrt(xn))


def scipy_ridge_cg(oracle_mod, b, ridge_param, tol):
    """The reference's ADRTRidgeOperator recipe (docs/examples.tomography.md:
    63-76) on the oracle operator in float64."""
    sla = pytest.importorskip("scipy.sparse.linalg")
    n = b.shape[-1]

    def mv(v):
        img = v.reshape(n, n)
        return (oracle_mod.adjoint(oracle_mod.adrt(img)) / 4 + ridge_param * img).ravel()

    op = sla.LinearOperator((n * n, n * n), matvec=mv, dtype=np.float64)
    rhs = (oracle_mod.adjoint(b) / 4).ravel()
    x, info = sla.cg(op, rhs, rtol=tol, maxiter=5000)
    assert info == 0
    return x.reshape(n, n)


@pytest.mark.parametrize("ridge_param", [0.5, 20.0])
def test_ridge_matches_scipy_oracle(oracle_mod, ridge_param):
    n = 32
    xt = ellipse_phantoms(2, n, seed=41, device="cuda", dtype=torch.float64)
    b = adrt.adrt(xt)
    res = cgmod.cg(b, tol=1e-11, max_iters=2000, ridge_param=ridge_param)
    for i in range(2):
        want = scipy_ridge_cg(oracle_mod, b[i].cpu().numpy(), ridge_param, 1e-13)
        got = res.x[i].cpu().numpy()
        assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-8
    plain = cgmod.cg(b, tol=1e-11, max_iters=2000)
    # The ridge term shrinks the solution.
    assert (res.x.norm(dim=(1, 2)) < plain.x.norm(dim=(1, 2))).all()
    assert (res.normal_residual <= 1e-10).all()


def test_compaction_gives_identical_results():
    """Shrinking the batch to the active images changes no image's result."""
    n, B = 64, 16
    xt = ellipse_phantoms(B, n, seed=57, device="cuda")
    b = adrt.adrt(xt)
    # widely different difficulty: scale half of the batch's data
    b[: B // 2] *= 1e-3
    g = torch.Generator(device="cuda")
    g.manual_seed(3)
    b = b + 1e-3 * b.abs().amax() * torch.randn(b.shape, generator=g, device="cuda")
    full = cgmod.cg(b, tol=1e-5, max_iters=400, compact=0.0, check_every=1)
    comp = cgmod.cg(b, tol=1e-5, max_iters=400, compact=0.9, check_every=1, graph=True)
    assert torch.equal(full.iterations, comp.iterations)
    assert torch.equal(full.x, comp.x)
    assert torch.equal(full.normal_residual, comp.normal_residual)
