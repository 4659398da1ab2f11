"""GPU parity: every transform, bit for bit against the golden fixtures (made
by the reference's compiled code) and against the CPU oracle on seeded inputs,
through the public API and hence the C ABI."""

import numpy as np
import pytest
import torch

import adrt_gb300 as adrt
from conftest import bits_equal, first_mismatch

pytestmark = pytest.mark.gpu

DTYPES = ("float32", "float64")
SIZES = (1, 2, 4, 8, 16, 32)


def dev(x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def host(t):
    return t.cpu().numpy()


def test_config1_adrt_bdrt(golden):
    x = golden["cfg1_x"]
    y = adrt.adrt(dev(x))
    assert y.shape == (4, 127, 64) and y.dtype == torch.float32
    assert bits_equal(host(y), golden["cfg1_adrt"]), first_mismatch(host(y), golden["cfg1_adrt"])
    z = adrt.bdrt(y)
    assert bits_equal(host(z), golden["cfg1_bdrt"])


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("n", SIZES)
def test_golden_transforms(golden, dt, n):
    g = lambda s: golden[f"{dt}_n{n}_{s}"]  # noqa: E731
    for inp, want, fn in [
        ("x", "adrt", adrt.adrt),
        ("xb", "adrt_b", adrt.adrt),
        ("yz", "bdrt", adrt.bdrt),
        ("adrt_b", "bdrt_b", adrt.bdrt),
        ("adrt", "iadrt", adrt.iadrt),
        ("adrt_b", "iadrt_b", adrt.iadrt),
    ]:
        got = host(fn(dev(g(inp))))
        assert bits_equal(got, g(want)), (fn.__name__, inp, first_mismatch(got, g(want)))


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("n", SIZES)
def test_golden_steps(golden, dt, n):
    k = f"{dt}_n{n}"
    init = adrt.core.adrt_init(dev(golden[f"{k}_x"]))
    yz = dev(golden[f"{k}_yz"])
    for s in range(adrt.core.num_iters(n)):
        assert bits_equal(host(adrt.core.adrt_step(init, s)), golden[f"{k}_adrt_step{s}"])
        assert bits_equal(host(adrt.core.bdrt_step(yz, s)), golden[f"{k}_bdrt_step{s}"])


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("n", SIZES)
def test_golden_fmg(golden, dt, n):
    k = f"{dt}_n{n}"
    xb, yb = dev(golden[f"{k}_xb"]), dev(golden[f"{k}_adrt_b"])
    assert bits_equal(host(adrt.core._prolong(xb)), golden[f"{k}_prolong"])
    if n >= 2:
        assert bits_equal(host(adrt.core._restrict(yb)), golden[f"{k}_restrict"])
        assert bits_equal(host(adrt.core._highpass(xb)), golden[f"{k}_highpass"])
        got = host(adrt.core.iadrt_fmg_step(yb))
        assert bits_equal(got, golden[f"{k}_fmg_step"]), first_mismatch(got, golden[f"{k}_fmg_step"])


def test_golden_iadrt_fmg(golden):
    y = adrt.adrt(dev(golden["fmg_src"]))
    got = host(adrt.iadrt_fmg(y))
    want = golden["fmg_inv"]
    assert got.shape == want.shape
    # The stopping rule compares float64 residual norms (NumPy uses float32),
    # so the iteration count may differ only on near-ties; values agree to 1e-5.
    np.testing.assert_allclose(got, want, atol=1e-5, rtol=0)
    got2 = host(adrt.iadrt_fmg(y, max_iters=2))
    assert bits_equal(got2, golden["fmg_inv_max2"]) or np.allclose(got2, golden["fmg_inv_max2"], atol=1e-6)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("n,b", [(64, 3), (128, 2), (256, 2), (512, 1), (1024, 2), (2048, 1)])
def test_oracle_large(oracle_mod, dt, n, b):
    rng = np.random.default_rng(n + b)
    x = rng.random((b, n, n)).astype(dt)
    x[0, : n // 4] = -0.0
    y = adrt.adrt(dev(x))
    want = oracle_mod.adrt(x)
    assert bits_equal(host(y), want), first_mismatch(host(y), want)
    yz = want.copy()
    yz[:, :, -5:] = -0.0
    z = adrt.bdrt(dev(yz))
    assert bits_equal(host(z), oracle_mod.bdrt(yz))
    if n <= 1024:
        inv = adrt.iadrt(dev(want))
        assert bits_equal(host(inv), oracle_mod.iadrt(want))


@pytest.mark.parametrize("n", [64, 256])
def test_steps_chain_equals_fused(oracle_mod, n):
    rng = np.random.default_rng(5)
    x = dev(rng.standard_normal((2, n, n)).astype(np.float32))
    a = adrt.core.adrt_init(x)
    for s in range(adrt.core.num_iters(n)):
        a = adrt.core.adrt_step(a, s)
    assert bits_equal(host(a), host(adrt.adrt(x)))
    y = adrt.adrt(x)
    for s in range(adrt.core.num_iters(n)):
        got = host(adrt.core.bdrt_step(y, s))
        assert bits_equal(got, oracle_mod.bdrt_step(host(y), s))


def test_host_inputs_roundtrip(golden):
    x = golden["float32_n16_xb"]
    y = adrt.adrt(x)  # numpy in -> numpy out, computed on the GPU
    assert isinstance(y, np.ndarray) and bits_equal(y, golden["float32_n16_adrt_b"])
    yt = adrt.adrt(torch.from_numpy(x))  # CPU tensor in -> CPU tensor out
    assert isinstance(yt, torch.Tensor) and not yt.is_cuda
    assert bits_equal(yt.numpy(), golden["float32_n16_adrt_b"])
    # Non-contiguous / Fortran-order / byte-swapped inputs are accepted.
    assert bits_equal(adrt.adrt(np.asfortranarray(x)), golden["float32_n16_adrt_b"])
    assert bits_equal(adrt.adrt(x.astype(x.dtype.newbyteorder(">"))), golden["float32_n16_adrt_b"])
    xt = torch.from_numpy(x).cuda().transpose(-1, -2).contiguous().transpose(-1, -2)
    assert bits_equal(host(adrt.adrt(xt)), golden["float32_n16_adrt_b"])


@pytest.mark.parametrize("n,b,dt", [(1024, 19, np.float32), (512, 37, np.float64), (64, 5, np.float32)])
def test_host_pipeline_chunks(n, b, dt):
    # Host batches run chunk by chunk with overlapped copies; results must
    # equal the device path bit for bit, for every chunk including the last,
    # partial one.
    rng = np.random.default_rng(n + b)
    x = rng.standard_normal((b, n, n)).astype(dt)
    y_host = adrt.adrt(x)
    y_dev = host(adrt.adrt(dev(x)))
    assert isinstance(y_host, np.ndarray) and bits_equal(y_host, y_dev)
    z_host = adrt.bdrt(torch.from_numpy(y_host))
    assert isinstance(z_host, torch.Tensor) and not z_host.is_cuda
    assert bits_equal(z_host.numpy(), host(adrt.bdrt(dev(y_dev))))


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64, torch.int32, torch.int64,
                                   torch.int8, torch.float16, torch.complex128, torch.bool])
def test_init_truncate_stitch_any_dtype(oracle_mod, dtype):
    n = 8
    x = (torch.arange(3 * n * n) % 7).reshape(3, n, n).to(dtype)
    xn = x.numpy()
    init = adrt.core.adrt_init(x.cuda())
    assert init.dtype == dtype
    assert np.array_equal(host(init), oracle_mod.adrt_init(xn))
    tr = adrt.utils.truncate(init)
    assert np.array_equal(host(tr), oracle_mod.truncate(oracle_mod.adrt_init(xn)))
    for rr in (False, True):
        st = adrt.utils.stitch_adrt(init, remove_repeated=rr)
        assert np.array_equal(host(st), oracle_mod.stitch_adrt(oracle_mod.adrt_init(xn), rr))


def test_truncate_stitch_leading_dims(oracle_mod):
    rng = np.random.default_rng(3)
    y = rng.standard_normal((2, 3, 4, 15, 8)).astype(np.float32)
    assert bits_equal(host(adrt.utils.truncate(dev(y))), oracle_mod.truncate(y))
    assert bits_equal(host(adrt.utils.stitch_adrt(dev(y))), oracle_mod.stitch_adrt(y))


def test_nan_inf_positions(oracle_mod):
    rng = np.random.default_rng(11)
    x = rng.standard_normal((2, 64, 64)).astype(np.float32)
    x[0, 3, 5] = np.nan
    x[1, 10, 10] = np.inf
    x[1, 11, 12] = -np.inf
    assert bits_equal(host(adrt.adrt(dev(x))), oracle_mod.adrt(x))


def test_device_status_clean_after_fast_path():
    from adrt_gb300 import _lib

    x = torch.rand((3, 1024, 1024), device="cuda")
    adrt.adrt(x)
    for n in (64, 256, 512):
        adrt.adrt(torch.rand((2, n, n), device="cuda"))
    rc = _lib.load().adrt_gb300_device_status(torch.cuda.current_stream().cuda_stream)
    assert rc == _lib.OK
