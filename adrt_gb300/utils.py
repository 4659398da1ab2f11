"""Layout utilities for ADRT outputs.

GB300 counterpart of the reference's ``adrt.utils`` (src/adrt/utils.py) for
``truncate``, ``stitch_adrt``, ``unstitch_adrt``, ``coord_adrt`` and
``coord_cart_to_adrt``, and of ``adrt.utils.interp_to_cart``: the same names, signatures, shapes and
errors; the copies run as CUDA kernels.  Any element type is accepted, and any
number of leading dimensions, as in the reference.
"""

from __future__ import annotations

import collections.abc
import operator
import typing

import torch

from . import _lib
from ._wrappers import Staged, batch_of, check_array, check_ndim, check_nonzero, ensure_cuda, float_code, ptr
from ._wrappers import valid_adrt_output_shape

__all__: typing.Final[collections.abc.Sequence[str]] = [
    "stitch_adrt",
    "unstitch_adrt",
    "truncate",
    "interp_to_cart",
    "coord_adrt",
    "coord_cart_to_adrt",
    "ADRTCoord",
    "ADRTIndex",
]


def _check_adrt_output(a) -> int:
    shape = tuple(a.shape)
    n = shape[-1] if shape else 0
    if shape[-3:] != (4, 2 * n - 1, n):
        raise ValueError(f"unsuitable shape for ADRT output processing {shape}")
    return int(n)


def truncate(a, /):
    """Cut each quadrant to its top n x n square and rotate it back to the
    orientation of the image.  Output (..., 4, n, n).
    Reference: src/adrt/utils.py:191-242."""
    check_array(a)
    n = _check_adrt_output(a)
    ensure_cuda()
    st = Staged(a)
    out = st.empty((*a.shape[:-3], 4, n, n))
    b = batch_of(a.shape, 3)
    if b > 0 and n > 0:
        rc = _lib.load().adrt_gb300_truncate(ptr(st.t), ptr(out), b, n, st.t.element_size(), st.stream())
        _lib.check(rc, "truncate")
    return st.finish(out)


def stitch_adrt(a, /, *, remove_repeated: bool = False):
    """Place the four quadrants side by side in one (..., 3n-2, 4n) image (4n-4
    columns with `remove_repeated`), odd quadrants flipped, quadrants 2 and 3
    aligned to the bottom.  Reference: src/adrt/utils.py:65-134."""
    check_array(a)
    n = _check_adrt_output(a)
    ensure_cuda()
    st = Staged(a)
    vc = n - (1 if remove_repeated else 0)
    out = st.empty((*a.shape[:-3], 3 * n - 2, 4 * vc))
    b = batch_of(a.shape, 3)
    if b > 0 and out.numel() > 0:
        rc = _lib.load().adrt_gb300_stitch(
            ptr(st.t), ptr(out), b, n, 1 if remove_repeated else 0, st.t.element_size(), st.stream()
        )
        _lib.check(rc, "stitch_adrt")
    return st.finish(out)


def unstitch_adrt(a, /):
    """Slice a stitched ADRT output back into its four quadrants: the inverse
    of :func:`stitch_adrt` (with or without `remove_repeated`, detected from
    the width).  Output (..., 4, 2n-1, n).  Reference: src/adrt/utils.py:137-188."""
    check_array(a)
    shape = tuple(a.shape)
    n = (shape[-2] + 2) // 3
    if shape[-2] != 3 * n - 2 or (shape[-1] != 4 * n and shape[-1] != 4 * n - 4):
        raise ValueError(f"unsuitable shape for ADRT unstitching {shape}")
    removed = shape[-1] == 4 * n - 4
    ensure_cuda()
    st = Staged(a)
    out = st.empty((*shape[:-2], 4, 2 * n - 1, n))
    b = batch_of(shape, 2)
    if b > 0 and out.numel() > 0:
        rc = _lib.load().adrt_gb300_unstitch(ptr(st.t), ptr(out), b, n, 1 if removed else 0, st.t.element_size(),
                                             st.stream())
        _lib.check(rc, "unstitch_adrt")
    return st.finish(out)


def interp_to_cart(a, /):
    """Resample ADRT output (..., 4, 2n-1, n) onto the regular Cartesian
    Radon grid (..., n, 4n): each output takes the nearest digital line's
    entry times its length factor (zero outside the data).  Same selection
    and factors as the reference, bit for bit.
    Reference: src/adrt/_wrappers.py:329-362, src/adrt/adrt_cdefs_py.cpp:621-682,
    src/adrt/adrt_cdefs_interp_adrtcart.hpp:62-114."""
    check_array(a)
    check_ndim(a, 3, 4)
    check_nonzero(a)
    if not valid_adrt_output_shape(a.shape) or int(a.shape[-1]) < 2:
        raise ValueError("array must have a valid ADRT output shape")
    n = int(a.shape[-1])
    if n > (1 << 24) // 4:
        raise ValueError("array is too big for interpolation index calculations")
    code = float_code(a)
    ensure_cuda()
    st = Staged(a)
    out = st.empty((*a.shape[:-3], n, 4 * n))
    b = batch_of(a.shape, 3)
    rc = _lib.load().adrt_gb300_interp_to_cart(ptr(st.t), ptr(out), b, n, code, st.stream())
    _lib.check(rc, "interp_to_cart")
    return st.finish(out)


class ADRTCoord(typing.NamedTuple):
    """Offsets (4, 2n-1, n) and angles (4, 1, n) of the ADRT entries."""

    offset: torch.Tensor
    angle: torch.Tensor


class ADRTIndex(typing.NamedTuple):
    """Nearest ADRT entries (quadrant, height, slope) and scale factors."""

    quadrant: typing.Any
    height: typing.Any
    slope: typing.Any
    factor: typing.Any


def _radon_size(n) -> int:
    n = operator.index(n)
    if n < 2:
        raise ValueError(f"invalid Radon domain size {n}, must be at least 2")
    if n & (n - 1):
        raise ValueError(f"invalid Radon domain size {n}, must be a power of two")
    return n


def coord_adrt(n, /) -> ADRTCoord:
    """Offset and angle (radians) that every entry of an n x n ADRT output
    approximates, as float64 CUDA tensors on the current device: offset
    (4, 2n-1, n), angle (4, 1, n) (broadcastable).  Reference:
    src/adrt/utils.py:250-332."""
    n = _radon_size(n)
    ensure_cuda()
    dev = torch.device("cuda", torch.cuda.current_device())
    offset = torch.empty((4, 2 * n - 1, n), dtype=torch.float64, device=dev)
    angle = torch.empty((4, 1, n), dtype=torch.float64, device=dev)
    rc = _lib.load().adrt_gb300_coord_adrt(n, ptr(offset), ptr(angle), torch.cuda.current_stream(dev).cuda_stream)
    _lib.check(rc, "coord_adrt")
    return ADRTCoord(offset, angle)


def coord_cart_to_adrt(theta, t, n, /) -> ADRTIndex:
    """Nearest ADRT entry and scale factor for continuous Radon points
    (theta in radians, t in [-1/sqrt 2, 1/sqrt 2]): quadrant (uint8), height
    (int64), slope (uint64), factor (float64), each shaped like theta.  CUDA
    tensors in give CUDA tensors out; NumPy arrays give NumPy arrays.
    Reference: src/adrt/utils.py:335-435."""
    n = _radon_size(n)
    if tuple(theta.shape) != tuple(t.shape):
        raise ValueError(f"mismatched shapes for theta and t {tuple(theta.shape)} vs. {tuple(t.shape)}")
    check_array(theta)
    check_array(t)
    code = max(float_code(theta), float_code(t))
    ensure_cuda()
    st = Staged(theta)
    th = st.t.to(torch.float32 if code == _lib.F32 else torch.float64).contiguous()
    tt = torch.as_tensor(t).to(device=th.device, dtype=th.dtype).contiguous()
    shape = tuple(th.shape)
    q = torch.empty(shape, dtype=torch.uint8, device=th.device)
    h = torch.empty(shape, dtype=torch.int64, device=th.device)
    s = torch.empty(shape, dtype=torch.uint64, device=th.device)
    f = torch.empty(shape, dtype=torch.float64, device=th.device)
    rc = _lib.load().adrt_gb300_coord_cart_to_adrt(ptr(th), ptr(tt), th.numel(), n, code, ptr(q), ptr(h), ptr(s),
                                                   ptr(f), st.stream())
    _lib.check(rc, "coord_cart_to_adrt")
    return ADRTIndex(*(st.finish(x) for x in (q, h, s, f)))
