"""Low-level routines for observing or influencing the basic algorithms.

GB300 counterpart of the reference's ``adrt.core`` (src/adrt/core.py): the same
names, signatures and error behaviour, computed on the GPU.
"""

from __future__ import annotations

import collections.abc
import operator
import typing

import numpy as np
import torch

from . import _lib
from ._ops import adrt as _adrt
from ._ops import adrt_step, bdrt_step
from ._ops import bdrt as _bdrt
from ._ops import press_fmg_highpass as _highpass
from ._ops import press_fmg_prolongation as _prolong
from ._ops import press_fmg_restriction as _restrict
from ._wrappers import (
    Staged,
    _format_object_type,
    batch_of,
    check_array,
    ensure_cuda,
    float_code,
    ptr,
)

__all__: typing.Final[collections.abc.Sequence[str]] = [
    "num_iters",
    "adrt_step",
    "adrt_init",
    "adrt_iter",
    "bdrt_step",
    "bdrt_iter",
    "threading_enabled",
    "iadrt_fmg_step",
    "iadrt_fmg_iter",
]


def num_iters(n: typing.SupportsIndex, /) -> int:
    """ceil(log2(n)), with num_iters(0) == 0.  Reference: src/adrt/core.py:94-120."""
    n = operator.index(n)
    if n < 0:
        raise ValueError(f"non-negative value required for iteration count, but got {n}")
    return n.bit_length() - (n.bit_count() == 1)


def threading_enabled() -> bool:
    """The GPU routines are always parallel.  Reference: src/adrt/_wrappers.py:363-378."""
    return True


def adrt_init(a, /):
    """Stack the four flipped/transposed copies of `a` into the ADRT output
    layout, zeros below the top n rows.  Any dtype.
    Reference: src/adrt/core.py:123-176."""
    if not isinstance(a, (torch.Tensor, np.ndarray)):
        raise TypeError(
            f"array must be torch.Tensor or numpy.ndarray, but got {_format_object_type(a)}"
        )
    if a.ndim > 3 or a.ndim < 2:
        raise ValueError(f"array must have between 2 and 3 dimensions, but had {a.ndim}")
    n = int(a.shape[-1])
    if a.shape[-1] != a.shape[-2] or n.bit_count() != 1:
        raise ValueError("array must be square with a power of two shape")
    if not all(a.shape):
        raise ValueError(
            "all array dimensions must be nonzero, "
            f"but found zero in dimension {tuple(a.shape).index(0)}"
        )
    ensure_cuda()
    st = Staged(a)
    out = st.empty((*a.shape[:-2], 4, 2 * n - 1, n))
    rc = _lib.load().adrt_gb300_adrt_init(
        ptr(st.t), ptr(out), batch_of(a.shape, 2), n, st.t.element_size(), st.stream()
    )
    _lib.check(rc, "adrt_init")
    return st.finish(out)


def _readonly(x, copy):
    if isinstance(x, np.ndarray):
        x.setflags(write=False)
        return x.copy() if copy else x.view()
    return x.clone() if copy else x


def adrt_iter(a, /, *, copy: bool = True):
    """Yield adrt_init(a) and each of the num_iters(n) stages.
    Reference: src/adrt/core.py:179-223."""
    a = adrt_init(a)
    yield _readonly(a, copy)
    for i in range(num_iters(a.shape[-1])):
        a = adrt_step(a, i)
        yield _readonly(a, copy)


def bdrt_iter(a, /, *, copy: bool = True):
    """Yield each bdrt step of `a`.  Reference: src/adrt/core.py:226-262."""
    for i in range(num_iters(a.shape[-1])):
        a = bdrt_step(a, i)
        yield _readonly(a, copy)


def _sub(a: torch.Tensor, b: torch.Tensor, out: torch.Tensor = None) -> torch.Tensor:
    out = torch.empty_like(a) if out is None else out
    rc = _lib.load().adrt_gb300_elementwise(
        0, ptr(a), ptr(b), ptr(out), a.numel(), float_code(a), torch.cuda.current_stream(a.device).cuda_stream
    )
    _lib.check(rc, "elementwise")
    return out


def _add(a: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    out = torch.empty_like(a)
    rc = _lib.load().adrt_gb300_elementwise(
        1, ptr(a), ptr(b), ptr(out), a.numel(), float_code(a), torch.cuda.current_stream(a.device).cuda_stream
    )
    _lib.check(rc, "elementwise")
    return out


def _fmg_correction(y: torch.Tensor) -> torch.Tensor:
    n = int(y.shape[-1])
    out = torch.empty((*y.shape[:-3], n, n), dtype=y.dtype, device=y.device)
    rc = _lib.load().adrt_gb300_fmg_correction(
        ptr(y), ptr(out), batch_of(y.shape, 3), n, float_code(y), torch.cuda.current_stream(y.device).cuda_stream
    )
    _lib.check(rc, "fmg_correction")
    return out


def _fmg_step_device(a: torch.Tensor) -> torch.Tensor:
    """iadrt_fmg_step on a contiguous CUDA tensor (same operation order as
    src/adrt/core.py:318-330)."""
    stack = []
    for _ in range(num_iters(a.shape[-1])):
        stack.append(a)
        a = _restrict(a)
    ret = a[..., 0, :, :].contiguous()
    while stack:
        ret = _prolong(ret)
        resid = _sub(_adrt(ret), stack.pop())
        corr = _highpass(_fmg_correction(_bdrt(resid)))
        _sub(ret, corr, out=ret)
    return ret


def iadrt_fmg_step(a, /):
    """One full-multigrid estimate of the inverse ADRT.
    Reference: src/adrt/core.py:265-331."""
    check_array(a)
    ensure_cuda()
    st = Staged(a)
    return st.finish(_fmg_step_device(st.t))


def iadrt_fmg_iter(a, /, *, copy: bool = True):
    """Infinite iterator of refined inverses inv_{k+1} = inv_k + step(a - adrt(inv_k)).
    Reference: src/adrt/core.py:334-381."""
    check_array(a)
    ensure_cuda()
    st = Staged(a)
    t = st.t
    # iadrt_fmg_step is looked up at call time (as in the reference), and on a
    # CUDA tensor it returns a CUDA tensor.
    inv = iadrt_fmg_step(t)
    yield _readonly(st.finish(inv), copy) if st.kind != "cuda" else (inv.clone() if copy else inv)
    while True:
        inv = _add(inv, iadrt_fmg_step(_sub(t, _adrt(inv))))
        yield _readonly(st.finish(inv), copy) if st.kind != "cuda" else (inv.clone() if copy else inv)
