"""Differentiable ADRT.

``adrt(x)`` is the forward ADRT as a ``torch.autograd.Function`` whose backward
is the exact transpose, computed by the library's adjoint kernel
(``adrt_gb300_adjoint``: backprojection followed by the quadrant sum, the
composition the reference documents as ``truncate(bdrt(y)).sum(-3)``,
src/adrt/_wrappers.py:283-284).  No autograd graph is built through the
butterfly stages.  ``adjoint(y)`` is the transpose as a Function whose
backward is the forward ADRT.

Both accept CUDA tensors of shape (n, n) / (B, n, n) resp. (4, 2n-1, n) /
(B, 4, 2n-1, n), float32 or float64.
"""

from __future__ import annotations

import torch

from . import _lib
from ._ops import adrt as _adrt_op
from ._wrappers import (
    batch_of,
    check_array,
    check_ndim,
    check_nonzero,
    ensure_cuda,
    float_code,
    valid_adrt_output_shape,
)

__all__ = ["adrt", "adjoint", "ADRTFunction", "AdjointFunction"]


def _adjoint_raw(y: torch.Tensor) -> torch.Tensor:
    """truncate(bdrt(y)) summed over quadrants in order, on the device."""
    check_array(y)
    check_ndim(y, 3, 4)
    check_nonzero(y)
    if not valid_adrt_output_shape(y.shape):
        raise ValueError("array must have a valid ADRT output shape")
    code = float_code(y)
    ensure_cuda()
    if not (isinstance(y, torch.Tensor) and y.is_cuda):
        raise TypeError("adjoint expects a CUDA tensor")
    y = y.contiguous()
    n = int(y.shape[-1])
    b = batch_of(y.shape, 3)
    out = torch.empty((*y.shape[:-3], n, n), dtype=y.dtype, device=y.device)
    nbytes = _lib.workspace_size(_lib.OP_ADJOINT, b, n, code)
    ws = torch.empty(nbytes, dtype=torch.uint8, device=y.device)
    rc = _lib.load().adrt_gb300_adjoint(
        y.data_ptr(), out.data_ptr(), b, n, code, ws.data_ptr(), nbytes,
        torch.cuda.current_stream(y.device).cuda_stream,
    )
    _lib.check(rc, "adjoint")
    return out


class ADRTFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x):
        if not x.is_cuda:
            raise TypeError("adrt_gb300.autograd.adrt expects a CUDA tensor")
        return _adrt_op(x)

    @staticmethod
    def backward(ctx, grad_out):
        return _adjoint_raw(grad_out)


class AdjointFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, y):
        return _adjoint_raw(y)

    @staticmethod
    def backward(ctx, grad_out):
        return _adrt_op(grad_out.contiguous())


def adrt(x: torch.Tensor) -> torch.Tensor:
    """Differentiable forward ADRT (backward = exact transpose)."""
    return ADRTFunction.apply(x)


def adjoint(y: torch.Tensor) -> torch.Tensor:
    """Differentiable transpose of the ADRT: truncate(bdrt(y)).sum(-3)."""
    return AdjointFunction.apply(y)
