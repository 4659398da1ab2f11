"""Argument checking at the public API, mirroring the reference boundary's
exception types and messages (src/adrt/adrt_cdefs_py.cpp:77-269 and the
per-function bodies; reference tests tests/test_adrt.py:85-166,
tests/test_bdrt.py:55-147, tests/test_iadrt.py:40-132,
tests/test_adrt_step.py:40-72, tests/test_bdrt_step.py:40-72,
tests/test_press_fmg_*.py, tests/test_adrt_init.py, tests/test_truncate.py,
tests/test_stitch_adrt.py, tests/test_num_iters.py, tests/test_iadrt_fmg.py).

All of these fail before any device work, so they run without a GPU."""

import numpy as np
import pytest

import adrt_gb300 as adrt


def z(*shape, dtype=np.float32):
    return np.zeros(shape, dtype=dtype)


class TestAdrt:
    def test_refuses_int32(self):
        with pytest.raises(TypeError, match="int32"):
            adrt.adrt(z(16, 16, dtype=np.int32))

    def test_refuses_non_square(self):
        with pytest.raises(ValueError, match="must be square"):
            adrt.adrt(z(16, 32))

    def test_refuses_four_dim(self):
        with pytest.raises(ValueError, match="between 2 and 3 dimensions, but had 4"):
            adrt.adrt(z(5, 3, 16, 16))

    def test_refuses_one_dim(self):
        with pytest.raises(ValueError, match="between 2 and 3 dimensions, but had 1"):
            adrt.adrt(z(16))

    def test_refuses_non_power_of_two(self):
        with pytest.raises(ValueError, match="power of two shape"):
            adrt.adrt(z(31, 31))

    def test_refuses_non_array(self):
        with pytest.raises(TypeError, match="must be torch.Tensor or numpy.ndarray"):
            adrt.adrt([[1.0, 2.0], [3.0, 4.0]])
        with pytest.raises(TypeError, match="but got NoneType"):
            adrt.adrt(None)

    def test_refuses_zero_axis(self):
        with pytest.raises(ValueError, match="found zero in dimension 0"):
            adrt.adrt(z(0, 32, 32))

    def test_shape_checked_before_dtype(self):
        with pytest.raises(ValueError, match="power of two"):
            adrt.adrt(z(3, 3, dtype=np.int32))


@pytest.mark.parametrize("fn", [adrt.bdrt, adrt.iadrt])
class TestAdrtShaped:
    def test_refuses_int32(self, fn):
        with pytest.raises(TypeError, match="int32"):
            fn(z(4, 31, 16, dtype=np.int32))

    def test_refuses_mismatched_shape(self, fn):
        with pytest.raises(ValueError, match="must have a valid ADRT output shape"):
            fn(z(4, 32, 16))
        with pytest.raises(ValueError, match="must have a valid ADRT output shape"):
            fn(z(3, 31, 16))

    def test_refuses_five_dim(self, fn):
        with pytest.raises(ValueError, match="between 3 and 4 dimensions, but had 5"):
            fn(z(2, 3, 4, 31, 16))

    def test_refuses_non_power_of_two(self, fn):
        with pytest.raises(ValueError, match="must have a valid ADRT output shape"):
            fn(z(4, 23, 12))

    def test_refuses_zero_axis(self, fn):
        with pytest.raises(ValueError, match="found zero in dimension 0"):
            fn(z(0, 4, 31, 16))

    def test_refuses_non_array(self, fn):
        with pytest.raises(TypeError, match="must be torch.Tensor or numpy.ndarray"):
            fn(None)


@pytest.mark.parametrize("fn", [adrt.core.adrt_step, adrt.core.bdrt_step])
class TestSteps:
    def test_refuses_step_out_of_range(self, fn):
        with pytest.raises(ValueError, match=r"step -1 is out of range.*num_iters"):
            fn(z(4, 31, 16), -1)
        with pytest.raises(ValueError, match=r"step 4 is out of range.*num_iters"):
            fn(z(4, 31, 16), 4)

    def test_refuses_huge_step(self, fn):
        with pytest.raises(OverflowError, match="too large to convert to C int"):
            fn(z(4, 31, 16), 2**40)

    def test_refuses_non_int_step(self, fn):
        with pytest.raises(TypeError):
            fn(z(4, 31, 16), 1.0)

    def test_refuses_int32(self, fn):
        with pytest.raises(TypeError, match="int32"):
            fn(z(4, 31, 16, dtype=np.int32), 0)

    def test_refuses_bad_shape(self, fn):
        with pytest.raises(ValueError, match="shape"):
            fn(z(4, 30, 16), 0)

    def test_missing_step(self, fn):
        with pytest.raises(TypeError):
            fn(z(4, 31, 16))


def test_adrt_step_shape_message():
    with pytest.raises(ValueError, match="use adrt.core.adrt_init"):
        adrt.core.adrt_step(z(4, 30, 16), 0)


class TestFmgOps:
    def test_restriction_rejects(self):
        with pytest.raises(ValueError, match="valid ADRT output shape"):
            adrt.core._restrict(z(4, 1, 1))
        with pytest.raises(ValueError, match="between 3 and 4 dimensions"):
            adrt.core._restrict(z(31, 16))
        with pytest.raises(TypeError, match="int32"):
            adrt.core._restrict(z(4, 31, 16, dtype=np.int32))

    def test_highpass_rejects(self):
        with pytest.raises(ValueError, match="too small to high-pass"):
            adrt.core._highpass(z(1, 5))
        with pytest.raises(ValueError, match="between 2 and 3 dimensions, but had 4"):
            adrt.core._highpass(z(1, 2, 5, 5))

    def test_prolongation_rejects(self):
        with pytest.raises(ValueError, match="found zero in dimension 1"):
            adrt.core._prolong(z(3, 0, 2))
        with pytest.raises(TypeError, match="int64"):
            adrt.core._prolong(z(3, 2, dtype=np.int64))


class TestAdrtInit:
    def test_refuses_non_array(self):
        with pytest.raises(TypeError, match="but got list"):
            adrt.core.adrt_init([[1, 2], [3, 4]])

    def test_refuses_dims(self):
        with pytest.raises(ValueError, match="between 2 and 3 dimensions, but had 4"):
            adrt.core.adrt_init(z(1, 1, 4, 4))

    def test_refuses_non_square(self):
        with pytest.raises(ValueError, match="square with a power of two"):
            adrt.core.adrt_init(z(4, 8))
        with pytest.raises(ValueError, match="square with a power of two"):
            adrt.core.adrt_init(z(6, 6))

    def test_refuses_zero(self):
        with pytest.raises(ValueError, match="found zero in dimension 0"):
            adrt.core.adrt_init(z(0, 4, 4))


@pytest.mark.parametrize("fn", [adrt.utils.truncate, adrt.utils.stitch_adrt])
@pytest.mark.parametrize("shape", [(4, 0, 0), (4, 4, 2), (7, 4), (3, 7, 4)])
def test_layout_rejects(fn, shape):
    with pytest.raises(ValueError, match=r"unsuitable shape .*ADRT output"):
        fn(np.ones(shape, dtype=np.float32))


class TestNumIters:
    @pytest.mark.parametrize(
        "n,want", [(0, 0), (1, 0), (2, 1), (3, 2), (4, 2), (5, 3), (16, 4), (17, 5)]
    )
    def test_values(self, n, want):
        assert adrt.core.num_iters(n) == want

    def test_numpy_ints(self):
        assert adrt.core.num_iters(np.int64(16)) == 4
        assert adrt.core.num_iters(np.uint8(8)) == 3

    def test_huge(self):
        assert adrt.core.num_iters(2**128) == 128
        assert adrt.core.num_iters(2**128 + 1) == 129
        assert adrt.core.num_iters(2**128 - 1) == 128

    def test_rejects(self):
        with pytest.raises(ValueError, match="non-negative value required"):
            adrt.core.num_iters(-1)
        with pytest.raises(TypeError):
            adrt.core.num_iters(4.0)


class TestIadrtFmgArgs:
    def test_rejects_batch(self):
        with pytest.raises(ValueError, match="batch dimension not supported"):
            adrt.iadrt_fmg(z(2, 4, 31, 16))

    @pytest.mark.parametrize("mi", [0, -1])
    def test_rejects_max_iters(self, mi):
        with pytest.raises(ValueError, match="must allow at least one iteration"):
            adrt.iadrt_fmg(z(4, 31, 16), max_iters=mi)


def test_threading_enabled():
    assert adrt.core.threading_enabled() is True


def test_public_names():
    assert set(adrt.__all__) == {"adrt", "iadrt", "bdrt", "iadrt_fmg", "utils", "core"}
    for name in ("num_iters", "adrt_step", "adrt_init", "adrt_iter", "bdrt_step", "bdrt_iter",
                 "threading_enabled", "iadrt_fmg_step", "iadrt_fmg_iter"):
        assert name in adrt.core.__all__ and callable(getattr(adrt.core, name))
