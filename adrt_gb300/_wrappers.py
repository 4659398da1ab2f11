"""Argument handling shared by the public modules.

Mirrors the reference's boundary: ``_normalize_array`` (src/adrt/_wrappers.py:96-112)
and the checks of the CPython binding (src/adrt/adrt_cdefs_py.cpp:77-269 and the
per-function bodies), in the same order and with the same exception types and
messages, before calling the C ABI in ``libadrt_gb300.so``.

Accepted inputs:
  * CUDA ``torch.Tensor``: computed on its device, result is a CUDA tensor;
  * CPU ``torch.Tensor`` or ``numpy.ndarray``: copied to the current CUDA
    device, computed there, copied back (result is the same kind of object).
Anything else raises ``TypeError``.  There is no CPU compute path.
"""

from __future__ import annotations

import operator

import numpy as np
import torch

from . import _lib

_FLOAT_DTYPES = {torch.float32: _lib.F32, torch.float64: _lib.F64}
_NP_FLOAT = {np.dtype(np.float32): _lib.F32, np.dtype(np.float64): _lib.F64}


def _format_object_type(obj: object) -> str:
    t = type(obj)
    if t.__module__ == "builtins":
        return str(t.__qualname__)
    return f"{t.__module__}.{t.__qualname__}"


def check_array(a, what: str = "array") -> None:
    if not isinstance(a, (torch.Tensor, np.ndarray)):
        raise TypeError(
            f"{what} must be torch.Tensor or numpy.ndarray, but got {_format_object_type(a)}"
        )


def check_ndim(a, lo: int, hi: int) -> None:
    if a.ndim < lo or a.ndim > hi:
        raise ValueError(f"array must have between {lo} and {hi} dimensions, but had {a.ndim}")


def check_nonzero(a) -> None:
    for i, s in enumerate(a.shape):
        if s <= 0:
            raise ValueError(
                f"all array dimensions must be nonzero, but found zero in dimension {i}"
            )


def float_code(a) -> int:
    """dtype code for float32/float64 arrays, TypeError otherwise (checked last, as in the reference)."""
    if isinstance(a, torch.Tensor):
        code = _FLOAT_DTYPES.get(a.dtype)
    else:
        code = _NP_FLOAT.get(a.dtype.newbyteorder("="))
    if code is None:
        raise TypeError(f"unsupported array dtype {a.dtype}")
    return code


def is_pow2(v: int) -> bool:
    return v > 0 and (v & (v - 1)) == 0


def valid_adrt_output_shape(shape) -> bool:
    """(…, 4, 2n-1, n) with n a power of two; reference: adrt_step_is_valid_shape
    (src/adrt/adrt_cdefs_common.cpp:185-193)."""
    q, rows, n = shape[-3], shape[-2], shape[-1]
    return q == 4 and is_pow2(n) and rows == 2 * n - 1


def c_int_step(step) -> int:
    step = operator.index(step)
    if step < -(2**31) or step > 2**31 - 1:
        raise OverflowError("Python int too large to convert to C int")
    return step


class Staged:
    """A CUDA tensor for the kernel plus how to return results to the caller."""

    __slots__ = ("t", "kind", "device")

    def __init__(self, a):
        if isinstance(a, torch.Tensor):
            if a.is_cuda:
                self.kind = "cuda"
                self.device = a.device
                self.t = a.contiguous()
            else:
                self.kind = "torch_cpu"
                self.device = torch.device("cuda", torch.cuda.current_device())
                self.t = a.contiguous().to(self.device, non_blocking=False)
        else:
            self.kind = "numpy"
            self.device = torch.device("cuda", torch.cuda.current_device())
            host = np.ascontiguousarray(a, dtype=a.dtype.newbyteorder("="))
            if not host.flags.writeable:
                host = host.copy()
            self.t = torch.from_numpy(host).to(self.device)

    def empty(self, shape, dtype=None):
        return torch.empty(shape, dtype=dtype or self.t.dtype, device=self.device)

    def finish(self, out: torch.Tensor):
        if self.kind == "cuda":
            return out
        if self.kind == "torch_cpu":
            return out.cpu()
        return out.cpu().numpy()

    def stream(self) -> int:
        return torch.cuda.current_stream(self.device).cuda_stream


def is_host(a) -> bool:
    return isinstance(a, np.ndarray) or (isinstance(a, torch.Tensor) and not a.is_cuda)


_PIPELINE_STREAMS = {}


def _pipeline_streams(dev):
    """The three copy/transform streams of `host_pipeline` on device `dev`,
    created once: the device buffers of every call are then allocated on the
    same stream and come back from the caching allocator's pool for that
    stream (fresh pool streams per call left them on a different stream each
    time)."""
    import torch

    key = dev.index
    if key not in _PIPELINE_STREAMS:
        _PIPELINE_STREAMS[key] = tuple(torch.cuda.Stream(device=dev) for _ in range(3))
    return _PIPELINE_STREAMS[key]


def host_pipeline(a, out_tail, chunk, run_chunk):
    """Transform a host array batch by batch with copies overlapped.

    `a` is a host array (NumPy or CPU tensor) of shape (B, *in_tail).  The
    batch is split into chunks of `chunk` images; chunk i's host-to-device
    copy, chunk i-1's transform and chunk i-2's device-to-host copy run on
    three streams at once, through two device buffers.  The result is written
    into host memory and returned as the caller's kind (NumPy array or CPU
    tensor).
    `run_chunk(d_in, d_out, k, stream_handle)` enqueues the transform of k
    images on the given stream.
    """
    dev = torch.device("cuda", torch.cuda.current_device())
    if isinstance(a, np.ndarray):
        host = np.ascontiguousarray(a, dtype=a.dtype.newbyteorder("="))
        hin = torch.from_numpy(host if host.flags.writeable else host.copy())
    else:
        hin = a.contiguous()
    B = hin.shape[0]
    # Pinned result (torch's caching host allocator reuses it across calls).
    # Freshly allocated pageable memory is much slower to copy into: every
    # page faults on first touch (measured 119 vs ~5000 images/s end to end).
    hout = torch.empty((B, *out_tail), dtype=hin.dtype, pin_memory=True)
    cur = torch.cuda.current_stream(dev)
    s_in, s_run, s_out = _pipeline_streams(dev)
    for s in (s_in, s_run, s_out):
        s.wait_stream(cur)
    k0 = min(chunk, B)
    with torch.cuda.stream(s_run):
        din = [torch.empty((k0, *hin.shape[1:]), dtype=hin.dtype, device=dev) for _ in range(2)]
        dout = [torch.empty((k0, *out_tail), dtype=hin.dtype, device=dev) for _ in range(2)]
    in_done = [torch.cuda.Event() for _ in range(2)]
    run_done = [None, None]
    out_done = [None, None]
    for i, b0 in enumerate(range(0, B, k0)):
        k = min(k0, B - b0)
        j = i & 1
        if run_done[j] is not None:
            s_in.wait_event(run_done[j])      # transform i-2 finished reading din[j]
        with torch.cuda.stream(s_in):
            din[j][:k].copy_(hin[b0:b0 + k], non_blocking=True)
        in_done[j].record(s_in)
        s_run.wait_event(in_done[j])
        if out_done[j] is not None:
            s_run.wait_event(out_done[j])     # copy-out of chunk i-2 finished reading dout[j]
        run_chunk(din[j][:k], dout[j][:k], k, s_run.cuda_stream)
        run_done[j] = torch.cuda.Event()
        run_done[j].record(s_run)
        s_out.wait_event(run_done[j])
        with torch.cuda.stream(s_out):
            hout[b0:b0 + k].copy_(dout[j][:k], non_blocking=True)
        out_done[j] = torch.cuda.Event()
        out_done[j].record(s_out)
    s_out.synchronize()
    s_run.synchronize()
    s_in.synchronize()
    return hout.numpy() if isinstance(a, np.ndarray) else hout


def ensure_cuda() -> None:
    if not torch.cuda.is_available():
        raise RuntimeError("adrt_gb300 requires a CUDA device; there is no CPU fallback")
    _lib.load()


def workspace(st: Staged, op: int, batch: int, n: int, code: int):
    nbytes = _lib.workspace_size(op, batch, n, code)
    if nbytes == 0:
        return None, 0
    return torch.empty(nbytes, dtype=torch.uint8, device=st.device), nbytes


def ptr(t) -> int:
    return 0 if t is None else t.data_ptr()


def batch_of(shape, core_ndim: int) -> int:
    return int(np.prod(shape[: len(shape) - core_ndim], dtype=np.int64)) if len(shape) > core_ndim else 1
