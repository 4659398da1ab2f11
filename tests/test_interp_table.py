"""interp_to_cart's selection table (host arithmetic, no GPU): applied with
NumPy it reproduces the compiled reference's interp_to_cart bit for bit, at
every power-of-two size up to 1024, in float32 and float64.  The GPU kernel
applies the same table (tests/test_gpu_next.py)."""

import ctypes

import numpy as np
import pytest

from adrt_gb300 import _lib


def table(n):
    idx = np.empty((n, 4 * n), dtype=np.int32)
    f32 = np.empty(4 * n, dtype=np.float32)
    f64 = np.empty(4 * n, dtype=np.float64)
    rc = _lib.load().adrt_gb300_interp_table(n, idx.ctypes.data, f32.ctypes.data, f64.ctypes.data)
    _lib.check(rc, "interp_table")
    return idx, f32, f64


def apply(y, idx, fac):
    flat = y.reshape(y.shape[0], -1)
    out = np.zeros((y.shape[0],) + idx.shape, dtype=y.dtype)
    m = idx >= 0
    out[:, m] = (fac[None, :] * np.ones(idx.shape, dtype=y.dtype))[m] * flat[:, idx[m]]
    return out


@pytest.fixture(scope="module")
def reference():
    from oracle import ref

    A = ref.load()
    if A is None:
        pytest.skip("compiled reference not available")
    return A


@pytest.mark.parametrize("n", [2, 4, 8, 16, 32, 64, 128, 256, 512, 1024])
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_table_matches_reference(reference, n, dt):
    rng = np.random.default_rng(n)
    y = rng.standard_normal((1, 4, 2 * n - 1, n)).astype(dt)
    want = reference.utils.interp_to_cart(y)
    idx, f32, f64 = table(n)
    got = apply(y, idx, f32 if dt == np.float32 else f64)
    assert got.dtype == want.dtype
    assert np.array_equal(got.view(np.uint8), want.view(np.uint8))


def test_table_rejects():
    buf = np.empty(64, dtype=np.int64)
    p = buf.ctypes.data
    lib = _lib.load()
    assert lib.adrt_gb300_interp_table(3, p, p, p) == _lib.ERR_SHAPE
    assert lib.adrt_gb300_interp_table(1, p, p, p) == _lib.ERR_SHAPE
    assert lib.adrt_gb300_interp_table(4, None, p, p) == _lib.ERR_NULL
