"""Kernels whose dynamic shared-memory limit the library raises must work on
every device of a process, not only the first one used: the limit is a
per-device attribute.  Runs the fast forward (both passes), the generic
passes, bdrt and the no-allocation forward on device 1 after device 0, each
compared bit for bit with device 0's result.  Needs two visible GPUs; skipped
otherwise.  Nothing here waits on another device."""

import numpy as np
import pytest
import torch

import adrt_gb300 as adrt

pytestmark = pytest.mark.gpu


def _noalloc(x, n):
    from adrt_gb300 import _lib

    out = torch.empty((x.shape[0], 4, 2 * n - 1, n), dtype=x.dtype, device=x.device)
    with torch.cuda.device(x.device):
        rc = _lib.load().adrt_gb300_adrt_noalloc(x.data_ptr(), out.data_ptr(), x.shape[0], n, _lib.F32,
                                                torch.cuda.current_stream(x.device).cuda_stream)
    assert rc == _lib.OK, _lib.status_string(rc)
    return out


@pytest.mark.skipif(torch.cuda.device_count() < 2, reason="needs two GPUs")
@pytest.mark.parametrize("n", [1024, 256, 32])
def test_second_device_matches_first(n):
    x0 = torch.rand((2, n, n), device="cuda:0")
    x1 = x0.to("cuda:1")
    outs = []
    for x in (x0, x1):
        with torch.cuda.device(x.device):
            y = adrt.adrt(x)
            z = adrt.bdrt(y)
            w = _noalloc(x, n)
            torch.cuda.synchronize(x.device)
        outs.append([t.cpu().numpy() for t in (y, z, w)])
    for a, b in zip(*outs):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
