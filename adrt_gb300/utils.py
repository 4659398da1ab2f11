"""Layout utilities for ADRT outputs.

GB300 counterpart of the reference's ``adrt.utils`` (src/adrt/utils.py) for
``truncate`` and ``stitch_adrt``: the same names, signatures, shapes and
errors; the copies run as CUDA kernels.  Any element type is accepted, and any
number of leading dimensions, as in the reference.
"""

from __future__ import annotations

import collections.abc
import typing

from . import _lib
from ._wrappers import Staged, batch_of, check_array, ensure_cuda, ptr

__all__: typing.Final[collections.abc.Sequence[str]] = ["stitch_adrt", "truncate"]


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
