"""Loads ``libadrt_gb300.so`` (the C ABI in include/adrt_gb300.h) with ctypes.

There is no CPU fallback: if the library is missing or cannot be loaded, every
call raises ``RuntimeError``.  Build it with ``python -m adrt_gb300.build`` (or
``__graft_entry__.build()``).
"""

from __future__ import annotations

import ctypes
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libadrt_gb300.so")

OK = 0
ERR_SHAPE = 1
ERR_STEP = 2
ERR_DTYPE = 3
ERR_WORKSPACE = 4
ERR_NULL = 5
ERR_CUDA = 6
ERR_TIMEOUT = 7
ERR_TOO_LARGE = 8

F32 = 0
F64 = 1

OP_ADRT = 0
OP_BDRT = 1
OP_IADRT = 2
OP_ADJOINT = 3

_lib = None
_lock = threading.Lock()

_v = ctypes.c_void_p
_i64 = ctypes.c_int64
_int = ctypes.c_int
_sz = ctypes.c_size_t

# name -> argtypes (all return int status unless listed in _RESTYPES)
SIGNATURES = {
    "adrt_gb300_status_string": [_int],
    "adrt_gb300_num_iters": [_i64],
    "adrt_gb300_launch_count": [],
    "adrt_gb300_device_status": [_v],
    "adrt_gb300_probe_dadd": [_v, _int, _int, _int, _v],
    "adrt_gb300_workspace_size": [_int, _i64, _i64, _int, ctypes.POINTER(_sz)],
    "adrt_gb300_adrt": [_v, _v, _i64, _i64, _int, _v, _sz, _v],
    "adrt_gb300_adrt_noalloc": [_v, _v, _i64, _i64, _int, _v],
    "adrt_gb300_adrt_step": [_v, _v, _i64, _i64, _int, _int, _v],
    "adrt_gb300_bdrt": [_v, _v, _i64, _i64, _int, _v, _sz, _v],
    "adrt_gb300_bdrt_step": [_v, _v, _i64, _i64, _int, _int, _v],
    "adrt_gb300_iadrt": [_v, _v, _i64, _i64, _int, _v, _sz, _v],
    "adrt_gb300_adjoint": [_v, _v, _i64, _i64, _int, _v, _sz, _v],
    "adrt_gb300_adrt_init": [_v, _v, _i64, _i64, _sz, _v],
    "adrt_gb300_truncate": [_v, _v, _i64, _i64, _sz, _v],
    "adrt_gb300_stitch": [_v, _v, _i64, _i64, _int, _sz, _v],
    "adrt_gb300_unstitch": [_v, _v, _i64, _i64, _int, _sz, _v],
    "adrt_gb300_interp_to_cart": [_v, _v, _i64, _i64, _int, _v],
    "adrt_gb300_interp_table": [_i64, _v, _v, _v],
    "adrt_gb300_coord_adrt": [_i64, _v, _v, _v],
    "adrt_gb300_coord_cart_to_adrt": [_v, _v, _i64, _i64, _int, _v, _v, _v, _v, _v],
    "adrt_gb300_fmg_restriction": [_v, _v, _i64, _i64, _int, _v],
    "adrt_gb300_fmg_prolongation": [_v, _v, _i64, _i64, _i64, _int, _v],
    "adrt_gb300_fmg_highpass": [_v, _v, _i64, _i64, _i64, _int, _v],
    "adrt_gb300_fmg_correction": [_v, _v, _i64, _i64, _int, _v],
    "adrt_gb300_elementwise": [_int, _v, _v, _v, _i64, _int, _v],
    "adrt_gb300_sumsq_workspace_size": [],
    "adrt_gb300_sumsq": [_v, _i64, _int, _v, _v, _v],
    "adrt_gb300_sumsq_batched_workspace_size": [_i64],
    "adrt_gb300_sumsq_batched": [_v, _i64, _i64, _int, _v, _v, _v],
    "adrt_gb300_cg_workspace_size": [_i64],
    "adrt_gb300_ragged_workspace_size": [_v, _i64, _int, ctypes.POINTER(_sz)],
    "adrt_gb300_adrt_ragged": [_v, _v, _v, _i64, _int, _v, _sz, _v],
    "adrt_gb300_adrt_ragged_ex": [_v, _v, _v, _i64, _int, _v, _sz, ctypes.c_uint64, _i64, _v],
    "adrt_gb300_ragged_status": [_v, _v, _i64, _int, _v],
    "adrt_gb300_batched_dot": [_v, _v, _v, _i64, _i64, _int, _v, _v],
    "adrt_gb300_cg_update": [_v, _v, _v, _v, _v, _v, _v, _v, _i64, _i64, _int, _v, _v],
    "adrt_gb300_cg_direction": [_v, _v, _v, _v, _v, _i64, _i64, _int, _v],
    "adrt_gb300_axpy": [ctypes.c_double, _v, _v, _i64, _int, _v],
    "adrt_gb300_precond_conv": [_v, _v, _i64, _i64, ctypes.POINTER(ctypes.c_double), _int, _int, _v],
    "adrt_gb300_precond_dot_workspace_size": [_i64, _i64],
    "adrt_gb300_precond_conv_dot": [_v, _v, _i64, _i64, ctypes.POINTER(ctypes.c_double), _int, _int, _v, _v, _sz, _v],
    "adrt_gb300_tune_set": [_int, _int, _i64, _int, _int, _int, _int],
    "adrt_gb300_tune_get": [_int, _int, _i64, ctypes.POINTER(_int), ctypes.POINTER(_int), ctypes.POINTER(_int),
                            ctypes.POINTER(_int)],
    "adrt_gb300_tune_reset": [],
    # learned preconditioner kernels (include/adrt_gb300_net.h)
    "adrtnet_conv3x3": [_v, _int, _v, _int, _v, _v, _v, _int, _v, _i64, _i64, _i64, _v],
    "adrtnet_conv3x3_wgrad": [_v, _int, _v, _int, _v, _i64, _i64, _i64, _v],
    "adrtnet_status": [_v],
    "adrtnet_conv_in": [_v, _v, _v, _v, _i64, _i64, _i64, _v],
    "adrtnet_conv_in_wgrad": [_v, _v, _v, _v, _i64, _i64, _i64, _v],
    "adrtnet_conv_out": [_v, _v, _v, _v, _i64, _i64, _i64, _v],
    "adrtnet_conv_out_bwd": [_v, _v, _v, _v, _v, _v, _i64, _i64, _i64, _v],
    "adrtnet_pool2": [_v, _v, _i64, _i64, _i64, _int, _v],
    "adrtnet_pool2_bwd": [_v, _v, _v, _v, _i64, _i64, _i64, _int, _v],
    "adrtnet_up2": [_v, _v, _i64, _i64, _i64, _int, _v],
    "adrtnet_up2_bwd": [_v, _v, _v, _i64, _i64, _i64, _int, _v],
    "adrtnet_bias_grad": [_v, _v, _i64, _int, _v],
    "adrtnet_diff": [_v, _v, ctypes.c_float, _v, _i64, _v],
    "adrtnet_loss_grad": [_v, _v, ctypes.c_float, ctypes.c_float, ctypes.c_float, _v, _v, _i64, _v],
    "adrtnet_adam": [_v, _v, _v, _v, _v, _int, _i64, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                     ctypes.c_float, _v, _int, _v, _v],
}
_RESTYPES = {
    "adrt_gb300_tune_reset": None,
    "adrt_gb300_status_string": ctypes.c_char_p,
    "adrt_gb300_sumsq_workspace_size": _sz,
    "adrt_gb300_sumsq_batched_workspace_size": _sz,
    "adrt_gb300_precond_dot_workspace_size": _sz,
    "adrt_gb300_launch_count": ctypes.c_uint64,
    "adrt_gb300_cg_workspace_size": _sz,
}


def launch_count() -> int:
    return int(load().adrt_gb300_launch_count())


def load() -> ctypes.CDLL:
    """Return the loaded library, raising RuntimeError if it is unavailable."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"adrt_gb300 CUDA library not found at {LIB_PATH}; "
                "build it with `python -m adrt_gb300.build`"
            )
        lib = ctypes.CDLL(LIB_PATH)
        for name, args in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = _RESTYPES.get(name, _int)
        _lib = lib
    return _lib


def status_string(code: int) -> str:
    return load().adrt_gb300_status_string(code).decode()


def workspace_size(op: int, batch: int, n: int, dtype_code: int) -> int:
    out = _sz(0)
    rc = load().adrt_gb300_workspace_size(op, batch, n, dtype_code, ctypes.byref(out))
    check(rc, "workspace_size")
    return int(out.value)


def check(rc: int, what: str) -> None:
    if rc == OK:
        return
    msg = f"{what}: {status_string(rc)}"
    if rc in (ERR_SHAPE, ERR_STEP, ERR_TOO_LARGE):
        raise ValueError(msg)
    if rc == ERR_DTYPE:
        raise TypeError(msg)
    raise RuntimeError(msg)
