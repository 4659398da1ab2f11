"""Argument checks of interp_to_cart, unstitch_adrt and the coordinate maps,
with the reference's exception types and messages (no GPU needed: all are
raised before any device work)."""

import numpy as np
import pytest

import adrt_gb300 as adrt


def test_interp_to_cart_rejects():
    with pytest.raises(ValueError, match="valid ADRT output shape"):
        adrt.utils.interp_to_cart(np.zeros((4, 1, 1), dtype=np.float32))  # n = 1
    with pytest.raises(ValueError, match="valid ADRT output shape"):
        adrt.utils.interp_to_cart(np.zeros((4, 6, 4), dtype=np.float32))
    with pytest.raises(ValueError):
        adrt.utils.interp_to_cart(np.zeros((4, 7), dtype=np.float32))
    with pytest.raises(TypeError):
        adrt.utils.interp_to_cart(np.zeros((4, 7, 4), dtype=np.int32))
    with pytest.raises(TypeError):
        adrt.utils.interp_to_cart([[1.0]])


def test_unstitch_rejects():
    with pytest.raises(ValueError, match="unsuitable shape for ADRT unstitching"):
        adrt.utils.unstitch_adrt(np.zeros((10, 15), dtype=np.float32))
    with pytest.raises(ValueError, match="unsuitable shape for ADRT unstitching"):
        adrt.utils.unstitch_adrt(np.zeros((9, 15), dtype=np.float32))


def test_coord_rejects():
    with pytest.raises(ValueError, match="must be at least 2"):
        adrt.utils.coord_adrt(1)
    with pytest.raises(ValueError, match="must be a power of two"):
        adrt.utils.coord_adrt(12)
    with pytest.raises(TypeError):
        adrt.utils.coord_adrt(4.0)
    with pytest.raises(ValueError, match="mismatched shapes"):
        adrt.utils.coord_cart_to_adrt(np.zeros(3), np.zeros(4), 8)
    with pytest.raises(ValueError, match="must be a power of two"):
        adrt.utils.coord_cart_to_adrt(np.zeros(3), np.zeros(3), 6)


def test_exports():
    for name in ("interp_to_cart", "unstitch_adrt", "coord_adrt", "coord_cart_to_adrt"):
        assert name in adrt.utils.__all__
