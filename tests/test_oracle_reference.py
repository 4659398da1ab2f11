"""Cross-checks the CPU oracle against the reference package itself (installed
into baseline/_ref by ``make -C oracle install-ref``, its extension compiled
from its own sources by ``make -C oracle ref``).  Skipped where that install
is absent."""

import numpy as np
import pytest

from conftest import bits_equal


@pytest.fixture(scope="module")
def ref():
    from oracle import ref as refmod

    A = refmod.load()
    if A is None:
        pytest.skip("reference package not installed here (make -C oracle install-ref)")
    return A


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("n", [1, 2, 4, 8, 16, 32, 64, 128])
def test_random_and_signed_zero(ref, oracle_mod, dt, n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal((2, n, n)).astype(dt)
    x[0, : max(1, n // 2)] = -0.0
    y = ref.adrt(x)
    assert bits_equal(oracle_mod.adrt(x), y)
    yz = y.copy()
    yz[..., -3:, :] = -0.0
    assert bits_equal(oracle_mod.bdrt(yz), ref.bdrt(yz))
    assert bits_equal(oracle_mod.iadrt(y), ref.iadrt(y))
    for s in range(oracle_mod.num_iters(n)):
        assert bits_equal(oracle_mod.adrt_step(yz, s), ref.core.adrt_step(yz, s))
        assert bits_equal(oracle_mod.bdrt_step(yz, s), ref.core.bdrt_step(yz, s))
    if n >= 2:
        assert bits_equal(oracle_mod.press_fmg_restriction(y), ref._wrappers._press_fmg_restriction(y))
        assert bits_equal(oracle_mod.press_fmg_highpass(x), ref._wrappers._press_fmg_highpass(x))
        assert bits_equal(oracle_mod.iadrt_fmg_step(y), ref.core.iadrt_fmg_step(y))
    assert bits_equal(oracle_mod.press_fmg_prolongation(x), ref._wrappers._press_fmg_prolongation(x))


def test_layout_helpers(ref, oracle_mod):
    rng = np.random.default_rng(7)
    for n in (1, 2, 8):
        x = rng.standard_normal((3, n, n)).astype(np.float32)
        y = ref.adrt(x)
        assert bits_equal(oracle_mod.adrt_init(x), ref.core.adrt_init(x))
        assert bits_equal(oracle_mod.truncate(y), ref.utils.truncate(y))
        assert bits_equal(oracle_mod.stitch_adrt(y), ref.utils.stitch_adrt(y))
        assert bits_equal(
            oracle_mod.stitch_adrt(y, True), ref.utils.stitch_adrt(y, remove_repeated=True)
        )
        adj = ref.utils.truncate(ref.bdrt(y))
        want = ((adj[:, 0] + adj[:, 1]) + adj[:, 2]) + adj[:, 3]
        assert bits_equal(oracle_mod.adjoint(y), want)
