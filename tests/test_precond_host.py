"""Host-side checks of the convolution preconditioner (no GPU)."""

import ctypes

import numpy as np
import pytest

from adrt_gb300 import _lib
from adrt_gb300 import precond


@pytest.mark.parametrize("h", [0, 1, 4, 7])
def test_basis_spans_square_symmetric_kernels(h):
    Bs = precond.basis(h)
    assert len(Bs) == (h + 1) * (h + 2) // 2
    total = sum(Bs)
    assert np.all(total == 1.0)  # the orbits partition the kernel's entries
    for B in Bs:
        assert np.array_equal(B, B.T) and np.array_equal(B, B[::-1]) and np.array_equal(B, B[:, ::-1])


def test_symbol_range():
    K = np.zeros((3, 3))
    K[1, 1] = 2.0
    assert precond.symbol_range(K) == (2.0, 2.0)
    K[1, 0] = K[1, 2] = K[0, 1] = K[2, 1] = -0.25  # 2 - 0.5 (cos wx + cos wy)
    lo, hi = precond.symbol_range(K, grid=64)
    assert abs(lo - 1.0) < 1e-12 and abs(hi - 3.0) < 1e-12


def test_rejects_bad_kernels():
    with pytest.raises(ValueError):
        precond.ConvPreconditioner(np.zeros((2, 2)))
    with pytest.raises(ValueError):
        precond.ConvPreconditioner(np.zeros((17, 17)))


def test_abi_argument_checks():
    lib = _lib.load()
    fake = ctypes.c_void_p(16)
    w = (ctypes.c_double * 9)()
    assert lib.adrt_gb300_precond_conv(None, fake, 1, 8, w, 1, _lib.F32, None) == _lib.ERR_NULL
    assert lib.adrt_gb300_precond_conv(fake, fake, 1, 8, None, 1, _lib.F32, None) == _lib.ERR_NULL
    assert lib.adrt_gb300_precond_conv(fake, fake, 1, 8, w, 1, 7, None) == _lib.ERR_DTYPE
    assert lib.adrt_gb300_precond_conv(fake, fake, 0, 8, w, 1, _lib.F32, None) == _lib.ERR_SHAPE
    assert lib.adrt_gb300_precond_conv(fake, fake, 1, 8, w, 8, _lib.F32, None) == _lib.ERR_SHAPE
    assert lib.adrt_gb300_precond_conv(fake, fake, 1, 65536, w, 1, _lib.F32, None) == _lib.ERR_TOO_LARGE


def test_fused_dot_abi_argument_checks():
    lib = _lib.load()
    fake = ctypes.c_void_p(16)
    w = (ctypes.c_double * 9)()
    ws = lib.adrt_gb300_precond_dot_workspace_size(4, 64)
    assert ws == 8 * 4 * 2 * 2
    assert lib.adrt_gb300_precond_dot_workspace_size(0, 64) == 0
    assert lib.adrt_gb300_precond_conv_dot(fake, fake, 4, 64, w, 1, _lib.F32, None, fake, ws, None) == _lib.ERR_NULL
    assert lib.adrt_gb300_precond_conv_dot(fake, fake, 4, 64, w, 1, _lib.F32, fake, None, ws, None) == _lib.ERR_NULL
    assert lib.adrt_gb300_precond_conv_dot(fake, fake, 4, 64, w, 1, _lib.F32, fake, fake, ws - 1, None) == \
        _lib.ERR_WORKSPACE
    assert lib.adrt_gb300_precond_conv_dot(fake, fake, 4, 64, w, 9, _lib.F32, fake, fake, ws, None) == _lib.ERR_SHAPE


def test_sumsq_batched_abi_argument_checks():
    lib = _lib.load()
    fake = ctypes.c_void_p(16)
    assert lib.adrt_gb300_sumsq_batched_workspace_size(3) == 3 * lib.adrt_gb300_sumsq_workspace_size()
    assert lib.adrt_gb300_sumsq_batched_workspace_size(0) == 0
    assert lib.adrt_gb300_sumsq_batched(None, 2, 16, _lib.F32, fake, fake, None) == _lib.ERR_NULL
    assert lib.adrt_gb300_sumsq_batched(fake, 0, 16, _lib.F32, fake, fake, None) == _lib.ERR_SHAPE
    assert lib.adrt_gb300_sumsq_batched(fake, 2, 16, 7, fake, fake, None) == _lib.ERR_DTYPE
    assert lib.adrt_gb300_sumsq_batched(fake, 70000, 16, _lib.F32, fake, fake, None) == _lib.ERR_TOO_LARGE
