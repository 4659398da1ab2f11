"""Parity on the exact benchmarked configuration: 256 images of 1024 x 1024
float32 (the first half uniform [0, 1), the second half ellipse phantoms, the
generator and seed bench.py uses on rank 0), through the same public call the
benchmark times (``adrt_gb300.adrt`` on a CUDA batch, which runs the fast
two-pass kernels over the whole batch in balanced chunks), compared bit for
bit with the CPU oracle image by image.  Also ``bdrt`` of that output and the
64-image float64 leg of the benchmark (``adrt`` and ``bdrt``).

Reference routines: src/adrt/adrt_cdefs_adrt.hpp:101-212 (adrt_basic),
src/adrt/adrt_cdefs_bdrt.hpp:121-187 (bdrt_basic)."""

import numpy as np
import pytest
import torch

import adrt_gb300 as adrt
from adrt_gb300.data import mixed_batch
from conftest import bits_equal, first_mismatch

pytestmark = pytest.mark.gpu

N = 1024
BATCH = 256
CHUNK = 32  # images compared per oracle call (bounds host memory)


@pytest.fixture(scope="module")
def batch():
    return mixed_batch(BATCH, N, seed=0, device="cuda", dtype=torch.float32)


def _compare(oracle_fn, x_dev, y_dev):
    for i in range(0, x_dev.shape[0], CHUNK):
        xs = x_dev[i : i + CHUNK].cpu().numpy()
        got = y_dev[i : i + CHUNK].cpu().numpy()
        want = oracle_fn(xs)
        assert bits_equal(got, want), f"images {i}..{i + xs.shape[0] - 1}: {first_mismatch(got, want)}"


def test_bench_batch_is_the_benchmarked_one(batch):
    # Half uniform in [0, 1), half phantoms (clipped at 0, piecewise constant).
    assert batch.shape == (BATCH, N, N) and batch.dtype == torch.float32
    u, p = batch[: BATCH // 2], batch[BATCH // 2 :]
    assert float(u.min()) >= 0.0 and float(u.max()) < 1.0
    assert float(p.min()) >= 0.0 and float((p == 0).float().mean()) > 0.3


def test_adrt_bdrt_float32_full_batch(oracle_mod, batch):
    y = adrt.adrt(batch)
    torch.cuda.synchronize()
    assert y.shape == (BATCH, 4, 2 * N - 1, N)
    _compare(oracle_mod.adrt, batch, y)
    z = adrt.bdrt(y)
    torch.cuda.synchronize()
    _compare(oracle_mod.bdrt, y, z)


def test_adrt_bdrt_float64_leg(oracle_mod, batch):
    x64 = batch[:64].double()
    y = adrt.adrt(x64)
    _compare(oracle_mod.adrt, x64, y)
    z = adrt.bdrt(y)
    _compare(oracle_mod.bdrt, y, z)


def test_repeated_calls_identical(batch):
    # The benchmark times back-to-back calls into reused allocations.
    a = adrt.adrt(batch[:130])
    b = adrt.adrt(batch[:130])
    assert torch.equal(a.view(torch.int32), b.view(torch.int32))
