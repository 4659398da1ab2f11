"""GB300-native approximate discrete Radon transform (ADRT).

A drop-in for the public API of the ``adrt`` package (karlotness/adrt):
``adrt``, ``bdrt``, ``iadrt``, ``iadrt_fmg``, ``adrt_gb300.core`` and
``adrt_gb300.utils``, computed by hand-written sm_103a CUDA kernels behind the
C ABI in include/adrt_gb300.h.  Inputs may be CUDA tensors (results stay on
the device) or host arrays (NumPy / CPU tensors: copied in and out).
There is no CPU compute path.
"""

from __future__ import annotations

import collections.abc
import math
import operator
import sys
import typing

import torch

from . import core, utils
from . import _lib
from ._ops import adrt, bdrt, iadrt
from ._wrappers import Staged, float_code, ptr

__all__: typing.Final[collections.abc.Sequence[str]] = [
    "adrt",
    "iadrt",
    "bdrt",
    "iadrt_fmg",
    "utils",
    "core",
]

__version__: typing.Final[str] = "0.1.0"


def _residual_norm(x: torch.Tensor, a: torch.Tensor, ws: torch.Tensor, acc: torch.Tensor) -> float:
    """||adrt(x) - a||_2 accumulated in float64 on the device."""
    r = core._sub(adrt(x), a)
    rc = _lib.load().adrt_gb300_sumsq(
        ptr(r), r.numel(), float_code(r), ptr(acc), ptr(ws), torch.cuda.current_stream(r.device).cuda_stream
    )
    _lib.check(rc, "sumsq")
    return math.sqrt(float(acc.item()))


def _iteration_limit(max_iters):
    """max_iters as an int (None: unbounded).  The reference checks `< 1`
    first, then hands the value to itertools.islice, which takes only None or
    an index in [0, sys.maxsize] and raises ValueError otherwise; the same
    values are accepted and rejected here."""
    if max_iters is not None and max_iters < 1:
        raise ValueError(f"must allow at least one iteration, but specified {max_iters}")
    if max_iters is None:
        return None
    try:
        limit = operator.index(max_iters)
    except TypeError:
        limit = -1
    if not 0 <= limit <= sys.maxsize:
        raise ValueError(f"max_iters must be None or an integer in [0, {sys.maxsize}], got {max_iters!r}")
    return limit


def iadrt_fmg_batched(a, /, *, max_iters: int | None = None):
    """iadrt_fmg for every (4, 2n-1, n) array of a batch (B, 4, 2n-1, n) at
    once (not in the reference, whose iadrt_fmg takes one array): the images
    iterate together, each with iadrt_fmg's own stopping rule, and each result
    is bit-identical to iadrt_fmg of that image alone (the same kernels, and
    per-image residual norms summed with the single-array partition).
    Returns (B, n, n)."""
    max_iters = _iteration_limit(max_iters)
    if a.ndim != 4:
        raise ValueError(f"iadrt_fmg_batched expects a batch (B, 4, 2n-1, n), got {a.ndim} dimensions")
    st = Staged(a)
    t = st.t
    B = int(t.shape[0])
    lib = _lib.load()
    ws = torch.empty(lib.adrt_gb300_sumsq_batched_workspace_size(B), dtype=torch.uint8, device=st.device)
    acc = torch.empty(B, dtype=torch.float64, device=st.device)

    def norms(x):
        r = core._sub(adrt(x), t)
        rc = lib.adrt_gb300_sumsq_batched(ptr(r), B, r[0].numel(), float_code(r), ptr(acc), ptr(ws),
                                         torch.cuda.current_stream(r.device).cuda_stream)
        _lib.check(rc, "sumsq_batched")
        return torch.sqrt(acc)

    it = core.iadrt_fmg_iter(t, copy=False)
    x = next(it)
    best, res_best = x.clone(), norms(x)
    done = torch.zeros(B, dtype=torch.bool, device=st.device)
    made = 1
    while max_iters is None or made < max_iters:
        x = next(it)
        made += 1
        res = norms(x)
        improved = (res < res_best) & ~done  # the reference stops at the first non-decrease (or NaN)
        done |= ~improved
        best[improved] = x[improved]
        res_best = torch.where(improved, res, res_best)
        if bool(done.all()):
            break
    return st.finish(best)


def iadrt_fmg(a, /, *, max_iters: int | None = None):
    """Approximate inverse of the ADRT by the full multigrid method, refined
    until the residual norm stops decreasing or `max_iters` estimates were made.
    No batch dimension.  Reference: src/adrt/__init__.py:69-148 (the same
    estimates and stopping rule: keep an estimate while each new one has a
    strictly smaller residual norm; the norm is accumulated in float64)."""
    if a.ndim > 3:
        raise ValueError(f"batch dimension not supported for iadrt_fmg, got {a.ndim} dimensions")
    max_iters = _iteration_limit(max_iters)
    st = Staged(a)
    t = st.t
    ws = torch.empty(_lib.load().adrt_gb300_sumsq_workspace_size(), dtype=torch.uint8, device=st.device)
    acc = torch.empty((), dtype=torch.float64, device=st.device)
    estimates = core.iadrt_fmg_iter(t, copy=False)
    kept = next(estimates)
    kept_norm = _residual_norm(kept, t, ws, acc)
    made = 1
    while max_iters is None or made < max_iters:
        cand = next(estimates)
        made += 1
        cand_norm = _residual_norm(cand, t, ws, acc)
        if not cand_norm < kept_norm:  # no decrease, or a NaN norm: stop at the kept one
            break
        kept, kept_norm = cand, cand_norm
    return st.finish(kept.clone())
