"""Transform functions over the C ABI (the GB300 counterpart of the reference's
``adrt._adrt_cdefs`` as wrapped by src/adrt/_wrappers.py)."""

from __future__ import annotations

import operator

from . import _lib
from ._wrappers import (
    Staged,
    batch_of,
    c_int_step,
    check_array,
    check_ndim,
    check_nonzero,
    ensure_cuda,
    float_code,
    host_pipeline,
    is_host,
    is_pow2,
    ptr,
    valid_adrt_output_shape,
    workspace,
)


def adrt(a, /):
    """The Approximate Discrete Radon Transform (ADRT).

    Input: square images of side n (a power of two), shape (n, n) or
    (batch, n, n), float32 or float64.  Output: (…, 4, 2n-1, n).
    Bit-identical to the reference's ``adrt.adrt``
    (src/adrt/_wrappers.py:115-159, src/adrt/adrt_cdefs_py.cpp:275-341).
    """
    check_array(a)
    check_ndim(a, 2, 3)
    check_nonzero(a)
    if a.shape[-1] != a.shape[-2] or not is_pow2(int(a.shape[-1])):
        raise ValueError("array must be square with a power of two shape")
    code = float_code(a)
    ensure_cuda()
    n = int(a.shape[-1])
    if is_host(a) and a.ndim == 3 and a.shape[0] > 1:
        return _host_batched(a, _lib.OP_ADRT, "adrt_gb300_adrt", n, code, (4, 2 * n - 1, n))
    st = Staged(a)
    b = batch_of(a.shape, 2)
    out = st.empty((*a.shape[:-2], 4, 2 * n - 1, n))
    ws, nbytes = workspace(st, _lib.OP_ADRT, b, n, code)
    rc = _lib.load().adrt_gb300_adrt(ptr(st.t), ptr(out), b, n, code, ptr(ws), nbytes, st.stream())
    _lib.check(rc, "adrt")
    return st.finish(out)


def _adrt_shaped_prologue(a, shape_msg):
    check_array(a)
    check_ndim(a, 3, 4)
    check_nonzero(a)
    if not valid_adrt_output_shape(a.shape):
        raise ValueError(shape_msg)


def adrt_step(a, /, step):
    """One step of the ADRT in the output layout; reference:
    src/adrt/_wrappers.py:162-202, src/adrt/adrt_cdefs_py.cpp:343-412."""
    check_array(a)
    step = operator.index(step)
    _adrt_shaped_prologue(a, "array must have valid shape for ADRT, use adrt.core.adrt_init")
    return _step(a, step, "adrt_gb300_adrt_step")


def bdrt_step(a, /, step):
    """One step of the bdrt; reference: src/adrt/_wrappers.py:289-325,
    src/adrt/adrt_cdefs_py.cpp:550-619."""
    check_array(a)
    step = operator.index(step)
    _adrt_shaped_prologue(a, "array must have a valid ADRT output shape")
    return _step(a, step, "adrt_gb300_bdrt_step")


def _step(a, step, fn):
    step = c_int_step(step)
    n = int(a.shape[-1])
    L = _num_iters_int(n)
    if step < 0 or step >= L:
        raise ValueError(
            f"step {step} is out of range for array's shape, use adrt.core.num_iters"
        )
    code = float_code(a)
    ensure_cuda()
    st = Staged(a)
    out = st.empty(tuple(a.shape))
    rc = getattr(_lib.load(), fn)(ptr(st.t), ptr(out), batch_of(a.shape, 3), n, step, code, st.stream())
    _lib.check(rc, fn)
    return st.finish(out)


def _num_iters_int(n: int) -> int:
    return n.bit_length() - (1 if n > 0 and (n & (n - 1)) == 0 else 0)


def _host_chunk(n: int, elem: int) -> int:
    """Images per pipeline chunk for host inputs: about 256 MB of output."""
    per = 4 * n * (2 * n - 1) * elem
    return max(1, (256 << 20) // per)


def _host_batched(a, op, fn, n, code, out_tail):
    """Host batch: chunked device transform with overlapped copies."""
    import torch

    elem = 4 if code == _lib.F32 else 8
    chunk = min(_host_chunk(n, elem), int(a.shape[0]))
    dev = torch.device("cuda", torch.cuda.current_device())
    nbytes = _lib.workspace_size(op, chunk, n, code)
    ws = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=dev)
    lib = _lib.load()

    def run(d_in, d_out, k, stream):
        rc = getattr(lib, fn)(ptr(d_in), ptr(d_out), k, n, code, ptr(ws), nbytes, stream)
        _lib.check(rc, fn)

    return host_pipeline(a, out_tail, chunk, run)


def _transform3(a, op, fn, name):
    _adrt_shaped_prologue(a, "array must have a valid ADRT output shape")
    code = float_code(a)
    ensure_cuda()
    n = int(a.shape[-1])
    if is_host(a) and a.ndim == 4 and a.shape[0] > 1:
        return _host_batched(a, op, fn, n, code, (4, 2 * n - 1, n))
    st = Staged(a)
    b = batch_of(a.shape, 3)
    out = st.empty(tuple(a.shape))
    ws, nbytes = workspace(st, op, b, n, code)
    rc = getattr(_lib.load(), fn)(ptr(st.t), ptr(out), b, n, code, ptr(ws), nbytes, st.stream())
    _lib.check(rc, name)
    return st.finish(out)


def bdrt(a, /):
    """Backprojection (generalised transpose) of the ADRT; bit-identical to the
    reference's ``adrt.bdrt`` (src/adrt/_wrappers.py:248-286,
    src/adrt/adrt_cdefs_py.cpp:482-548)."""
    check_array(a)
    return _transform3(a, _lib.OP_BDRT, "adrt_gb300_bdrt", "bdrt")


def iadrt(a, /):
    """Exact inverse of the ADRT; bit-identical to the reference's ``adrt.iadrt``
    (src/adrt/_wrappers.py:205-245, src/adrt/adrt_cdefs_py.cpp:414-480)."""
    check_array(a)
    return _transform3(a, _lib.OP_IADRT, "adrt_gb300_iadrt", "iadrt")


def press_fmg_restriction(a, /):
    """Reference: src/adrt/_wrappers.py:381-382, src/adrt/adrt_cdefs_fmg.hpp:53-73."""
    check_array(a)
    check_ndim(a, 3, 4)
    check_nonzero(a)
    n = int(a.shape[-1])
    if not (a.shape[-3] == 4 and a.shape[-2] == 2 * n - 1 and n >= 2 and n % 2 == 0):
        raise ValueError("array must have a valid ADRT output shape")
    code = float_code(a)
    ensure_cuda()
    st = Staged(a)
    out = st.empty((*a.shape[:-2], n - 1, n // 2))
    rc = _lib.load().adrt_gb300_fmg_restriction(ptr(st.t), ptr(out), batch_of(a.shape, 3), n, code, st.stream())
    _lib.check(rc, "press_fmg_restriction")
    return st.finish(out)


def press_fmg_prolongation(a, /):
    """Reference: src/adrt/_wrappers.py:385-386, src/adrt/adrt_cdefs_fmg.hpp:75-95."""
    check_array(a)
    check_ndim(a, 2, 3)
    check_nonzero(a)
    code = float_code(a)
    ensure_cuda()
    st = Staged(a)
    h, w = int(a.shape[-2]), int(a.shape[-1])
    out = st.empty((*a.shape[:-2], 2 * h, 2 * w))
    rc = _lib.load().adrt_gb300_fmg_prolongation(ptr(st.t), ptr(out), batch_of(a.shape, 2), h, w, code, st.stream())
    _lib.check(rc, "press_fmg_prolongation")
    return st.finish(out)


def press_fmg_highpass(a, /):
    """Reference: src/adrt/_wrappers.py:389-390, src/adrt/adrt_cdefs_fmg.hpp:97-171."""
    check_array(a)
    check_ndim(a, 2, 3)
    check_nonzero(a)
    h, w = int(a.shape[-2]), int(a.shape[-1])
    if h < 2 or w < 2:
        raise ValueError("array is too small to high-pass filter")
    code = float_code(a)
    ensure_cuda()
    st = Staged(a)
    out = st.empty(tuple(a.shape))
    rc = _lib.load().adrt_gb300_fmg_highpass(ptr(st.t), ptr(out), batch_of(a.shape, 2), h, w, code, st.stream())
    _lib.check(rc, "press_fmg_highpass")
    return st.finish(out)
