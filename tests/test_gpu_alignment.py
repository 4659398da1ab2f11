"""Buffers that are not 32-byte aligned (a C caller's pointer into the middle
of an allocation): the fast float32 kernels use 16- and 32-byte vector
accesses, so such calls take the generic kernels; results are bit-identical
to the aligned calls.  Ragged batches pack images back to back, so their
images are aligned or not depending on the sizes before them."""

import numpy as np
import pytest
import torch

import adrt_gb300 as adrt
from adrt_gb300 import _lib, ragged
from conftest import bits_equal

pytestmark = pytest.mark.gpu


def _call(fn, op, x, n, b, out_elems, offset):
    """Runs a C-ABI transform with input and output shifted by `offset`
    floats inside their allocations."""
    lib = _lib.load()
    xin = torch.empty(x.numel() + 8, device="cuda")
    xin[offset:offset + x.numel()] = x.reshape(-1)
    out = torch.full((out_elems + 8,), float("nan"), device="cuda")
    nbytes = _lib.workspace_size(op, b, n, _lib.F32)
    ws = torch.empty(max(nbytes, 1), dtype=torch.uint8, device="cuda")
    rc = getattr(lib, fn)(xin.data_ptr() + 4 * offset, out.data_ptr() + 4 * offset, b, n, _lib.F32,
                          ws.data_ptr(), nbytes, torch.cuda.current_stream().cuda_stream)
    assert rc == _lib.OK, _lib.status_string(rc)
    return out[offset:offset + out_elems].cpu().numpy()


@pytest.mark.parametrize("n,b", [(1024, 2), (256, 3)])
def test_unaligned_forward_and_bdrt(n, b):
    g = torch.Generator(device="cuda")
    g.manual_seed(n)
    x = torch.randn((b, n, n), generator=g, device="cuda")
    m = 4 * n * (2 * n - 1) * b
    aligned = _call("adrt_gb300_adrt", _lib.OP_ADRT, x, n, b, m, 0)
    shifted = _call("adrt_gb300_adrt", _lib.OP_ADRT, x, n, b, m, 1)
    assert bits_equal(aligned, shifted)
    y = torch.from_numpy(aligned).cuda()
    za = _call("adrt_gb300_bdrt", _lib.OP_BDRT, y, n, b, m, 0)
    zs = _call("adrt_gb300_bdrt", _lib.OP_BDRT, y, n, b, m, 3)
    assert bits_equal(za, zs)


def test_ragged_mixed_alignment():
    # 1024, 64, 256 aligned (fast tiles); after the 1 x 1 and 2 x 2 images the
    # rest start 5 floats off a 32-byte boundary (generic tiles).
    sizes = [1024, 64, 256, 1, 2, 512, 128, 1024]
    g = torch.Generator(device="cuda")
    g.manual_seed(2)
    imgs = [torch.randn((n, n), generator=g, device="cuda") for n in sizes]
    outs = ragged.adrt_ragged(imgs)
    for im, o in zip(imgs, outs):
        assert bits_equal(o.cpu().numpy(), adrt.adrt(im).cpu().numpy())
