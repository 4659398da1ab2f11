"""interp_to_cart, unstitch_adrt, coord_adrt and coord_cart_to_adrt on the
GPU against fixtures produced by the reference (tests/golden/golden_next.npz).

interp_to_cart and unstitch_adrt are bit-exact.  The coordinate maps are
NumPy code in the reference; their arctan/sin/cos/tan come from a different
math library here, so float outputs are compared to 1e-13 relative and
integer outputs may differ only where an ulp crosses a rounding tie."""

import numpy as np
import pytest
import torch

import adrt_gb300 as adrt
from conftest import bits_equal

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dt", ["float32", "float64"])
@pytest.mark.parametrize("n", [2, 4, 8, 16, 32, 64])
def test_interp_to_cart_golden(golden_next, dt, n):
    y = golden_next[f"interp_{dt}_n{n}_in"]
    want = golden_next[f"interp_{dt}_n{n}_out"]
    got = adrt.utils.interp_to_cart(torch.from_numpy(y).cuda()).cpu().numpy()
    assert bits_equal(got, want)
    # host arrays in, host arrays out; 3-d input without batch
    got_h = adrt.utils.interp_to_cart(y[0])
    assert isinstance(got_h, np.ndarray) and bits_equal(got_h, want[0])


def test_interp_to_cart_large_consistent():
    """n = 1024: the kernel's gather equals the selection table applied on the host."""
    from adrt_gb300 import _lib

    n = 1024
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    y = torch.randn((2, 4, 2 * n - 1, n), generator=g, device="cuda")
    got = adrt.utils.interp_to_cart(y).cpu().numpy()
    idx = np.empty((n, 4 * n), dtype=np.int32)
    f32 = np.empty(4 * n, dtype=np.float32)
    f64 = np.empty(4 * n, dtype=np.float64)
    _lib.check(_lib.load().adrt_gb300_interp_table(n, idx.ctypes.data, f32.ctypes.data, f64.ctypes.data), "table")
    flat = y.reshape(2, -1).cpu().numpy()
    m = idx >= 0
    want = np.zeros((2, n, 4 * n), dtype=np.float32)
    want[:, m] = np.broadcast_to(f32, idx.shape)[m] * flat[:, idx[m]]
    assert bits_equal(got, want)


@pytest.mark.parametrize("n,rr", [(1, 0), (4, 0), (4, 1), (16, 0), (16, 1)])
def test_unstitch_golden(golden_next, n, rr):
    s = golden_next[f"unstitch_n{n}_rr{rr}_in"]
    want = golden_next[f"unstitch_n{n}_rr{rr}_out"]
    got = adrt.utils.unstitch_adrt(torch.from_numpy(s).cuda()).cpu().numpy()
    assert bits_equal(got, want)
    assert bits_equal(adrt.utils.unstitch_adrt(s), want)


def test_stitch_unstitch_round_trip():
    n = 64
    x = torch.rand((3, n, n), device="cuda", dtype=torch.float64)
    y = adrt.adrt(x)
    assert torch.equal(adrt.utils.unstitch_adrt(adrt.utils.stitch_adrt(y)), y)
    # remove_repeated drops columns that are redundant for a real ADRT output
    z = adrt.utils.unstitch_adrt(adrt.utils.stitch_adrt(y, remove_repeated=True))
    assert z.shape == y.shape


@pytest.mark.parametrize("n", [2, 4, 16, 64])
def test_coord_adrt_golden(golden_next, n):
    c = adrt.utils.coord_adrt(n)
    assert c.offset.dtype == torch.float64 and c.offset.shape == (4, 2 * n - 1, n)
    assert c.angle.shape == (4, 1, n)
    np.testing.assert_allclose(c.offset.cpu().numpy(), golden_next[f"coord_n{n}_offset"], rtol=1e-13, atol=1e-15)
    np.testing.assert_allclose(c.angle.cpu().numpy(), golden_next[f"coord_n{n}_angle"], rtol=1e-14, atol=1e-15)


@pytest.mark.parametrize("dt", ["float32", "float64"])
@pytest.mark.parametrize("n", [4, 64])
def test_coord_cart_to_adrt_golden(golden_next, dt, n):
    k = f"cart_{dt}_n{n}"
    theta, t = golden_next[f"{k}_theta"], golden_next[f"{k}_t"]
    r = adrt.utils.coord_cart_to_adrt(theta, t, n)
    assert isinstance(r.quadrant, np.ndarray)
    assert r.quadrant.dtype == np.uint8 and r.height.dtype == np.int64
    assert r.slope.dtype == np.uint64 and r.factor.dtype == np.float64
    assert np.array_equal(r.quadrant, golden_next[f"{k}_q"])
    allowed = 0 if dt == "float64" else 5  # ulp differences of tan/cos at ties (float32)
    for got, want in ((r.height, golden_next[f"{k}_h"]), (r.slope, golden_next[f"{k}_s"])):
        diff = got.astype(np.int64) - want.astype(np.int64)
        assert np.count_nonzero(diff) <= allowed and np.abs(diff).max() <= 1
    same = r.slope == golden_next[f"{k}_s"]
    np.testing.assert_allclose(r.factor[same], golden_next[f"{k}_f"][same], rtol=1e-15)
    rc = adrt.utils.coord_cart_to_adrt(torch.from_numpy(theta).cuda(), torch.from_numpy(t).cuda(), n)
    assert rc.quadrant.is_cuda and np.array_equal(rc.height.cpu().numpy(), r.height)


@pytest.mark.parametrize("dtype", [torch.int8, torch.float16, torch.int32, torch.float64, torch.complex128])
def test_stitch_unstitch_round_trip_any_element_size(dtype):
    g = torch.Generator(device="cuda")
    g.manual_seed(4)
    y = (torch.rand((2, 4, 63, 32), generator=g, device="cuda") * 100).to(dtype)
    for rr in (False, True):
        s = adrt.utils.stitch_adrt(y, remove_repeated=rr)
        z = adrt.utils.unstitch_adrt(s)
        if rr:
            # stitch drops one column per quadrant (the last of even quadrants,
            # the first of odd ones, which are flipped); unstitch fills it from
            # the neighbouring quadrant
            assert torch.equal(z[:, 0::2, :, :-1], y[:, 0::2, :, :-1])
            assert torch.equal(z[:, 1::2, :, 1:], y[:, 1::2, :, 1:])
        else:
            assert torch.equal(z, y)
