"""Ragged batches: images of different power-of-two sizes.

``adrt_ragged(images)`` transforms a list of square images (sides 1..1024,
one dtype, one CUDA device) in a single persistent kernel launch that takes
(image, pass, tile) work items from a device-side queue; each result equals
``adrt_gb300.adrt`` of that image bit for bit.  ``iadrt_ragged`` and
``iadrt_fmg_ragged`` invert such a list (grouped by size, resp. image by image,
as the reference's ``iadrt_fmg`` takes no batch).
"""

from __future__ import annotations

import ctypes
from collections import defaultdict

import numpy as np
import torch

from . import _lib
from ._ops import iadrt as _iadrt
from ._wrappers import float_code, is_pow2

__all__ = ["adrt_ragged", "RaggedPlan", "iadrt_ragged", "iadrt_fmg_ragged"]


def _sizes_array(images):
    if not isinstance(images, (list, tuple)) or not images:
        raise TypeError("images must be a non-empty list of CUDA tensors")
    if not all(isinstance(im, torch.Tensor) for im in images):
        raise TypeError("images must be CUDA tensors")
    dt, dev = images[0].dtype, images[0].device
    if not dev.type == "cuda" or any(im.device != dev for im in images):
        if not all(im.is_cuda for im in images):
            raise TypeError("images must be CUDA tensors")
        raise ValueError("all images must share dtype and device")
    if any(im.dtype != dt for im in images):
        raise ValueError("all images must share dtype and device")
    shapes = [im.shape for im in images]
    for sh in shapes:
        if len(sh) != 2 or sh[0] != sh[1] or not is_pow2(int(sh[0])):
            raise ValueError("each image must be square with a power of two shape")
        if sh[0] > 1024:
            raise ValueError("ragged batches take sides up to 1024")
    return np.fromiter((sh[0] for sh in shapes), dtype=np.int64, count=len(shapes)), dt, dev


def _launch(images, wait_ns=0, starve_image=-1):
    sizes, dt, dev = _sizes_array(images)
    plan = RaggedPlan(sizes, dt, dev)
    plan.launch(plan.packed_input(images), wait_ns, starve_image)
    return plan.views(), plan.status()


def adrt_ragged(images):
    """Forward ADRT of each image of a ragged list, in one persistent launch.

    Raises RuntimeError if a device-side wait of the launch expired."""
    views, status = _launch(images)
    _lib.check(status, "adrt_ragged")
    return views


class RaggedPlan:
    """Buffers for repeated ragged launches over one list of sizes: the
    workspace and the packed output, allocated once.  `packed_input(images)`
    packs a list of images into one buffer (image after image, row-major);
    `launch(packed)` runs the persistent launch on torch's current stream and
    returns without waiting; `status()` then reads the launch's error word
    (waiting for the launch) and `views()` gives the (4, 2n-1, n) results."""

    def __init__(self, sizes, dtype=torch.float32, device="cuda"):
        self.sizes = np.ascontiguousarray(sizes, dtype=np.int64)
        if self.sizes.ndim != 1 or self.sizes.size == 0:
            raise ValueError("sizes must be a non-empty list of image sides")
        self.dtype = dtype
        self.device = torch.device(device)
        self.code = float_code(torch.empty(0, dtype=dtype))
        lib = _lib.load()
        self._sp = self.sizes.ctypes.data_as(ctypes.c_void_p)
        nbytes = ctypes.c_size_t(0)
        _lib.check(lib.adrt_gb300_ragged_workspace_size(self._sp, len(self.sizes), self.code,
                                                        ctypes.byref(nbytes)), "ragged")
        self.ws = torch.empty(max(nbytes.value, 1), dtype=torch.uint8, device=self.device)
        self.ws_bytes = nbytes.value
        self.in_elems = int((self.sizes * self.sizes).sum())
        self.out_lengths = [4 * int(n) * (2 * int(n) - 1) for n in self.sizes]
        self.out = torch.empty(sum(self.out_lengths), dtype=dtype, device=self.device)

    def packed_input(self, images):
        return torch.cat([im.reshape(-1) for im in images])

    def launch(self, packed, wait_ns=0, starve_image=-1):
        if not (isinstance(packed, torch.Tensor) and packed.device == self.out.device
                and packed.dtype == self.dtype and packed.is_contiguous()
                and packed.numel() == self.in_elems):
            raise ValueError("packed input must be one contiguous %s buffer of %d elements on %s"
                             % (self.dtype, self.in_elems, self.out.device))
        stream = torch.cuda.current_stream(self.out.device).cuda_stream
        rc = _lib.load().adrt_gb300_adrt_ragged_ex(packed.data_ptr(), self.out.data_ptr(), self._sp,
                                                   len(self.sizes), self.code, self.ws.data_ptr(),
                                                   self.ws_bytes, wait_ns, starve_image, stream)
        _lib.check(rc, "adrt_ragged")

    def status(self):
        stream = torch.cuda.current_stream(self.out.device).cuda_stream
        return _lib.load().adrt_gb300_ragged_status(self.ws.data_ptr(), self._sp, len(self.sizes),
                                                    self.code, stream)

    def views(self):
        return [t.view(4, 2 * n - 1, n) for t, n in zip(self.out.split(self.out_lengths), self.sizes.tolist())]


def iadrt_ragged(arrays):
    """Exact inverse of each (4, 2n-1, n) array; arrays of one size run as a batch."""
    groups = defaultdict(list)
    for i, a in enumerate(arrays):
        groups[int(a.shape[-1])].append(i)
    out = [None] * len(arrays)
    for n, idx in groups.items():
        res = _iadrt(torch.stack([arrays[i] for i in idx]))
        for k, i in enumerate(idx):
            out[i] = res[k]
    return out


def iadrt_fmg_ragged(arrays, max_iters=None):
    """Full-multigrid inverse of each array; arrays of one size iterate as a
    batch (``iadrt_fmg_batched``), each image with iadrt_fmg's own stopping
    rule and an identical result."""
    from . import iadrt_fmg_batched

    groups = defaultdict(list)
    for i, a in enumerate(arrays):
        groups[int(a.shape[-1])].append(i)
    out = [None] * len(arrays)
    for n, idx in groups.items():
        res = iadrt_fmg_batched(torch.stack([arrays[i] for i in idx]), max_iters=max_iters)
        for k, i in enumerate(idx):
            out[i] = res[k]
    return out
