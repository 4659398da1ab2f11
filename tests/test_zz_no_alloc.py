"""The no-allocation forward ADRT (adrt_gb300_adrt_noalloc) against the
regular entry point, through the C ABI.

adrt_gb300_adrt_noalloc serves callers that receive input and output buffers
but may not allocate device memory (a process that reserves its device memory
budget up front, a plugin inside a framework that owns the pool, a binding
with no allocator).  It keeps its intermediate in a static device array of
ADRT_GB300_NOALLOC_SCRATCH_BYTES (32 MiB) instead of a caller workspace.  Two
calls in a row must both reproduce the regular entry point bit for bit: the
second call finds the first call's data in the shared scratch.

This file is named to be collected last."""

import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

F32, F64 = 0, 1
OK, ERR_TOO_LARGE = 0, 8
SCRATCH_BYTES = 32 << 20


def _lib():
    from adrt_gb300 import _lib as lib_mod

    return lib_mod


def _regular(lib_mod, x, n, code, stream):
    b = x.shape[0]
    out = torch.empty((b, 4, 2 * n - 1, n), dtype=x.dtype, device=x.device)
    nbytes = lib_mod.workspace_size(lib_mod.OP_ADRT, b, n, code)
    ws = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=x.device)
    rc = lib_mod.load().adrt_gb300_adrt(x.data_ptr(), out.data_ptr(), b, n, code,
                                        ws.data_ptr(), nbytes, stream)
    assert rc == OK
    return out


def _noalloc(lib_mod, x, n, code, stream):
    b = x.shape[0]
    out = torch.full((b, 4, 2 * n - 1, n), float("nan"), dtype=x.dtype, device=x.device)
    rc = lib_mod.load().adrt_gb300_adrt_noalloc(x.data_ptr(), out.data_ptr(), b, n, code, stream)
    assert rc == OK, lib_mod.status_string(rc)
    return out


@pytest.mark.parametrize(
    "n,batch,dtype",
    [(1024, 3, torch.float32), (64, 5, torch.float32), (256, 2, torch.float64), (16, 4, torch.float64)],
)
def test_noalloc_matches_regular_twice(n, batch, dtype):
    lib_mod = _lib()
    code = F32 if dtype == torch.float32 else F64
    stream = torch.cuda.current_stream().cuda_stream
    g = torch.Generator(device="cuda")
    g.manual_seed(n + batch)
    x1 = torch.rand((batch, n, n), generator=g, device="cuda", dtype=dtype)
    x2 = torch.rand((batch, n, n), generator=g, device="cuda", dtype=dtype) - 0.5
    x2[0, : n // 4] = -0.0
    for x in (x1, x2):  # two calls in a row; the scratch keeps the previous call's data
        want = _regular(lib_mod, x, n, code, stream)
        got = _noalloc(lib_mod, x, n, code, stream)
        torch.cuda.synchronize()
        a = got.cpu().numpy()
        b = want.cpu().numpy()
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8))


def test_noalloc_rejects_sizes_beyond_scratch():
    lib_mod = _lib()
    lib = lib_mod.load()
    fake = ctypes.c_void_p(256)
    # float32 n = 2048 needs two 268 MB intermediates; float64 n = 1024 one 67 MB.
    assert lib.adrt_gb300_adrt_noalloc(fake, fake, 1, 2048, F32, None) == ERR_TOO_LARGE
    assert lib.adrt_gb300_adrt_noalloc(fake, fake, 1, 1024, F64, None) == ERR_TOO_LARGE
    assert lib_mod.workspace_size(lib_mod.OP_ADRT, 1, 1024, F32) <= SCRATCH_BYTES
