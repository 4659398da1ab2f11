"""Pins the CPU oracle (oracle/adrt_oracle.c) to the golden fixtures, which
were produced by the reference's own compiled code (tests/golden/make_golden.py).
Runs without a GPU."""

import numpy as np
import pytest

from conftest import bits_equal, first_mismatch

DTYPES = ("float32", "float64")
SIZES = (1, 2, 4, 8, 16, 32)


def test_config1_adrt_bdrt(golden, oracle_mod):
    x = np.random.default_rng(0).random((64, 64), dtype=np.float32)
    assert bits_equal(x, golden["cfg1_x"])
    y = oracle_mod.adrt(x)
    assert y.shape == (4, 127, 64)
    assert bits_equal(y, golden["cfg1_adrt"]), first_mismatch(y, golden["cfg1_adrt"])
    z = oracle_mod.bdrt(y)
    assert bits_equal(z, golden["cfg1_bdrt"]), first_mismatch(z, golden["cfg1_bdrt"])


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("n", SIZES)
def test_transforms(golden, oracle_mod, dt, n):
    k = f"{dt}_n{n}"
    g = lambda s: golden[f"{k}_{s}"]  # noqa: E731
    assert bits_equal(oracle_mod.adrt(g("x")), g("adrt"))
    assert bits_equal(oracle_mod.adrt(g("xb")), g("adrt_b"))
    assert bits_equal(oracle_mod.bdrt(g("yz")), g("bdrt"))
    assert bits_equal(oracle_mod.bdrt(g("adrt_b")), g("bdrt_b"))
    assert bits_equal(oracle_mod.iadrt(g("adrt")), g("iadrt"))
    assert bits_equal(oracle_mod.iadrt(g("adrt_b")), g("iadrt_b"))


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("n", SIZES)
def test_steps(golden, oracle_mod, dt, n):
    k = f"{dt}_n{n}"
    init = oracle_mod.adrt_init(golden[f"{k}_x"])
    for s in range(oracle_mod.num_iters(n)):
        assert bits_equal(oracle_mod.adrt_step(init, s), golden[f"{k}_adrt_step{s}"])
        assert bits_equal(oracle_mod.bdrt_step(golden[f"{k}_yz"], s), golden[f"{k}_bdrt_step{s}"])


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("n", SIZES)
def test_fmg_ops(golden, oracle_mod, dt, n):
    k = f"{dt}_n{n}"
    xb, yb = golden[f"{k}_xb"], golden[f"{k}_adrt_b"]
    assert bits_equal(oracle_mod.press_fmg_prolongation(xb), golden[f"{k}_prolong"])
    if n >= 2:
        assert bits_equal(oracle_mod.press_fmg_restriction(yb), golden[f"{k}_restrict"])
        assert bits_equal(oracle_mod.press_fmg_highpass(xb), golden[f"{k}_highpass"])
        assert bits_equal(oracle_mod.iadrt_fmg_step(yb), golden[f"{k}_fmg_step"])


def test_num_iters(oracle_mod):
    for n, want in [(0, 0), (1, 0), (2, 1), (3, 2), (4, 2), (5, 3), (1024, 10), (1025, 11)]:
        assert oracle_mod.num_iters(n) == want
