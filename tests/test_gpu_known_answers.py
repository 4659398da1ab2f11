"""Known-answer tests of the reference suite, run on the GPU path.

These restate the reference's own expectations: sums along recursively
generated digital lines (tests/test_adrt.py:40-72,233-284), the empty lower
triangle of each quadrant (:170-183), the spot values for edge lines
(:286-396), delta backprojections (tests/test_bdrt.py:211-300), the transpose
relation by materialising both matrices (tests/test_bdrt.py:310-325,
tests/test_bdrt_step.py:76-91), exact-inverse round trips
(tests/test_iadrt.py:185-239) and the full-multigrid stopping behaviour
(tests/test_iadrt_fmg.py:57-114, tests/test_iadrt_fmg_iter.py:105-117)."""

import contextlib
import functools
import itertools

import numpy as np
import pytest
import torch

import adrt_gb300 as adrt

pytestmark = pytest.mark.gpu


def digital_line(n, h, s):
    """Pixels (row, col) of the digital line of height offset h and slope s
    across n rows: split in halves, the lower half shifted by ceil(s/2)."""
    if n == 1:
        return {(0, h)}
    half = s // 2
    top = digital_line(n // 2, h, half)
    bot = digital_line(n // 2, h + half + (s & 1), half)
    return top | {(i + n // 2, j) for i, j in bot}


def naive_adrt(img):
    n = img.shape[0]
    res = np.zeros((4, 2 * n - 1, n), dtype=img.dtype)
    views = [img, img.T, np.flipud(img).T, np.flipud(img)]
    for q, v in enumerate(views):
        for hi, h in enumerate(range(n - 1, -n, -1)):
            for s in range(n):
                res[q, hi, s] = sum(
                    v[i, j] for i, j in digital_line(n, h, s) if 0 <= i < n and 0 <= j < n
                )
    return res


def lower_triangles_zero(a):
    n = a.shape[-1]
    return all(np.all(np.tril(a[q, -n:], k=-1) == 0) for q in range(4))


@pytest.mark.parametrize(
    "img",
    [
        np.ones((16, 16)),
        np.pad(np.ones((16, 1)), ((0, 0), (8, 7))),
        np.arange(256, dtype=np.float32).reshape(16, 16),
    ],
    ids=["ones", "vertical_line", "arange"],
)
def test_digital_line_sums(img):
    out = adrt.adrt(img)
    assert np.allclose(out, naive_adrt(img))
    assert lower_triangles_zero(out)


def test_batch_digital_lines():
    x = np.arange(4 * 8 * 8).reshape(4, 8, 8).astype(np.float32)
    out = adrt.adrt(x)
    assert np.allclose(out, np.stack([naive_adrt(x[i]) for i in range(4)]))


def test_zeros_and_1x1():
    assert np.all(adrt.adrt(np.zeros((32, 32))) == 0)
    assert np.allclose(adrt.adrt(np.ones((1, 1))), np.ones((4, 1, 1)))
    x = np.arange(5, dtype=np.float64).reshape(5, 1, 1) + 1
    assert np.allclose(adrt.adrt(x), np.stack([x] * 4, axis=1))


def test_spot_values_edge_line():
    x = np.zeros((8, 8))
    x[:, 0] = 1
    out = adrt.adrt(x)
    assert out.shape == (4, 15, 8) and lower_triangles_zero(out)
    assert out[0, 7, 0] == 8 and np.count_nonzero(out[0, :, 0]) == 1
    assert np.all(out[0, :7, -1] == 0) and np.all(out[0, -8:, -1] == 1)
    assert np.all(out[1, 8:, 0] == 0) and np.all(out[1, :8, -1] == 1)


def test_bdrt_delta_levels():
    n = 16
    x = np.zeros((n, n))
    x[n // 2, n // 2] = 1.0
    sq = np.mean(adrt.utils.truncate(adrt.bdrt(adrt.adrt(x))), axis=0)
    assert np.allclose(1.0 * (sq == 16.0), x)
    assert np.sum(sq == 4) == 8
    assert np.sum(sq == 2) == 19


def test_bdrt_digital_line_quadrant0():
    n = 16
    want = np.zeros((n, n))
    for i, j in digital_line(n, n - 5, 3):
        want[i, j] = 0.25
    y = np.zeros((4, 2 * n - 1, n))
    y[0, 4, 3] = 1.0
    assert np.allclose(np.mean(adrt.utils.truncate(adrt.bdrt(y)), axis=0), want)


def test_bdrt_zero_region():
    n = 16
    out = adrt.bdrt(adrt.adrt(np.ones((n, n))))
    for q in range(4):
        assert np.linalg.norm(np.tril(out[q, n:, ::-1]), ord="fro") == 0.0


@pytest.mark.parametrize("n", [1, 2, 4, 8])
def test_materialized_transpose(n):
    full, asz = n * n, 4 * n * (2 * n - 1)
    A = adrt.adrt(np.eye(full, dtype=np.float32).reshape(full, n, n)).reshape(full, -1).T
    bt = adrt.utils.truncate(adrt.bdrt(np.eye(asz, dtype=np.float32).reshape(asz, 4, 2 * n - 1, n)))
    B = np.sum(bt, axis=1).reshape(asz, full)
    assert np.allclose(A, B)


@pytest.mark.parametrize("n", [2, 4, 8])
def test_materialized_step_transpose(n):
    full = 4 * n * (2 * n - 1)
    basis = torch.eye(full, dtype=torch.float32).reshape(full, 4, 2 * n - 1, n).cuda()
    L = adrt.core.num_iters(n)
    for bs, fs in zip(range(L), reversed(range(L))):
        bm = adrt.core.bdrt_step(basis, bs).reshape(full, full).cpu().numpy()
        fm = adrt.core.adrt_step(basis, fs).reshape(full, full).cpu().numpy()
        assert np.array_equal(fm, bm.T)


@pytest.mark.parametrize("n", [16, 32])
def test_iadrt_round_trip(n):
    for x in (np.zeros((n, n), np.float32), np.ones((n, n), np.float32),
              np.arange(n * n).reshape(n, n).astype(np.float32)):
        inv = np.mean(adrt.utils.truncate(adrt.iadrt(adrt.adrt(x))), axis=0)
        assert inv.shape == x.shape and inv.dtype == x.dtype
        assert np.allclose(inv, x)
    xb = np.arange(4 * n * n).reshape(4, n, n).astype(np.float32)
    inv = np.mean(adrt.utils.truncate(adrt.iadrt(adrt.adrt(xb))), axis=1)
    assert np.allclose(inv, xb)


def test_iadrt_1x1():
    x = np.arange(5, dtype=np.float64).reshape(5, 1, 1) + 1
    out = adrt.iadrt(np.stack([x] * 4, axis=1))
    assert np.allclose(np.mean(adrt.utils.truncate(out), axis=1), x)


@pytest.fixture
def count_fmg_steps(monkeypatch):
    calls = 0
    orig = adrt.core.iadrt_fmg_step

    @functools.wraps(orig)
    def counting(*args, **kwargs):
        nonlocal calls
        calls += 1
        return orig(*args, **kwargs)

    monkeypatch.setattr(adrt.core, "iadrt_fmg_step", counting)
    return lambda: calls


@pytest.mark.parametrize("dtype", ["float32", "float64"])
def test_iadrt_fmg_recovers(dtype):
    x = np.arange(64).reshape(8, 8).astype(dtype)
    inv = adrt.iadrt_fmg(adrt.adrt(x), max_iters=50)
    assert inv.dtype == x.dtype and inv.shape == x.shape and inv.flags.writeable
    assert np.allclose(inv, x, atol=1e-3)


@pytest.mark.parametrize("val", [0, np.nan, np.inf, -np.inf])
def test_iadrt_fmg_stops_on_edge_cases(count_fmg_steps, val):
    a = np.full((4, 15, 8), val, dtype=np.float32)
    with np.errstate(invalid="ignore") if np.isinf(val) else contextlib.nullcontext():
        inv = adrt.iadrt_fmg(a, max_iters=50)
    assert count_fmg_steps() <= 2
    assert inv.shape == (8, 8) and inv.dtype == a.dtype
    assert np.isinf(val) or np.allclose(inv, val, equal_nan=True)


@pytest.mark.parametrize("max_iters", [1, 2, 3, 4])
def test_iadrt_fmg_max_iters(count_fmg_steps, max_iters):
    x = np.arange(256).reshape(16, 16).astype(np.float64)
    adrt.iadrt_fmg(adrt.adrt(x), max_iters=max_iters)
    assert count_fmg_steps() == max_iters


def test_iadrt_fmg_rejects_float_max_iters():
    with pytest.raises(ValueError, match=r"must be.*int"):
        adrt.iadrt_fmg(np.zeros((4, 15, 8), np.float32), max_iters=2.0)


def test_iadrt_fmg_iter_monotone_residual():
    n = 16
    yy, xx = np.mgrid[-1:1:n * 1j, -1:1:n * 1j]
    img = np.exp(-4 * (xx**2 + yy**2)).astype(np.float64)
    a = adrt.adrt(img)
    res = [np.linalg.norm(adrt.adrt(x) - a) for x in itertools.islice(adrt.core.iadrt_fmg_iter(a), 10)]
    assert all(r2 <= r1 for r1, r2 in itertools.pairwise(res))


def test_iadrt_fmg_iter_copies():
    a = adrt.adrt(np.ones((8, 8), np.float32))
    it = adrt.core.iadrt_fmg_iter(a, copy=False)
    v = next(it)
    assert not v.flags.writeable
    w = next(adrt.core.iadrt_fmg_iter(a))
    assert w.flags.writeable


def test_adrt_iter_matches():
    x = np.random.default_rng(0).standard_normal((16, 16)).astype(np.float32)
    steps = list(adrt.core.adrt_iter(x))
    assert len(steps) == adrt.core.num_iters(16) + 1
    assert np.array_equal(steps[-1], adrt.adrt(x))
    y = adrt.adrt(x)
    bs = list(adrt.core.bdrt_iter(y))
    assert len(bs) == 4
