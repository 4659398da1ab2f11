"""NumPy front end for the C restatement in ``oracle/adrt_oracle.c``.

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` as the checker.  The ``adrt_gb300``
package never imports this module.

Each function takes and returns C-contiguous NumPy arrays with the same shapes
as the reference's ``adrt._adrt_cdefs`` functions (src/adrt/_adrt_cdefs.pyi:40-50)
and computes the same values.  Batch dimensions are optional, as in the
reference.
"""

from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")
_lib = None

_i64 = ctypes.c_int64
_ptr = ctypes.c_void_p


def build(force: bool = False) -> str:
    """Compile liboracle.so with the Makefile beside this file."""
    if force or not os.path.exists(_LIB_PATH):
        subprocess.run(["make", "-s", "-C", _HERE, "all"], check=True)
    return _LIB_PATH


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(_LIB_PATH)
        for sfx in ("f32", "f64"):
            for name in ("adrt", "bdrt", "iadrt", "fmg_restriction"):
                fn = getattr(_lib, f"adrt_oracle_{name}_{sfx}")
                fn.argtypes = [_ptr, _i64, _i64, _ptr]
                fn.restype = ctypes.c_int
            for name in ("adrt_step", "bdrt_step"):
                fn = getattr(_lib, f"adrt_oracle_{name}_{sfx}")
                fn.argtypes = [_ptr, _i64, _i64, ctypes.c_int, _ptr]
                fn.restype = ctypes.c_int
            for name in ("fmg_prolongation", "fmg_highpass"):
                fn = getattr(_lib, f"adrt_oracle_{name}_{sfx}")
                fn.argtypes = [_ptr, _i64, _i64, _i64, _ptr]
                fn.restype = ctypes.c_int
        _lib.adrt_oracle_num_iters.argtypes = [_i64]
        _lib.adrt_oracle_num_iters.restype = ctypes.c_int
        _lib.adrt_oracle_threads.restype = ctypes.c_int
        _lib.adrt_oracle_set_threads.argtypes = [ctypes.c_int]
    return _lib


def threads() -> int:
    return lib().adrt_oracle_threads()


def set_threads(n: int) -> None:
    lib().adrt_oracle_set_threads(int(n))


def _sfx(a: np.ndarray) -> str:
    if a.dtype == np.float32:
        return "f32"
    if a.dtype == np.float64:
        return "f64"
    raise TypeError(f"unsupported array dtype {a.dtype}")


def _c(a: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(a)


def _call(name, a, *args):
    fn = getattr(lib(), f"adrt_oracle_{name}_{_sfx(a)}")
    rc = fn(*args)
    if rc != 0:
        raise MemoryError(f"oracle {name} failed ({rc})")


def num_iters(n: int) -> int:
    return lib().adrt_oracle_num_iters(int(n))


def adrt(a: np.ndarray) -> np.ndarray:
    a = _c(a)
    squeeze = a.ndim == 2
    x = a[None] if squeeze else a
    b, n = x.shape[0], x.shape[-1]
    out = np.empty((b, 4, 2 * n - 1, n), dtype=a.dtype)
    _call("adrt", a, x.ctypes.data, b, n, out.ctypes.data)
    return out[0] if squeeze else out


def _adrt_shaped(name, a, *extra):
    a = _c(a)
    squeeze = a.ndim == 3
    x = a[None] if squeeze else a
    b, n = x.shape[0], x.shape[-1]
    out = np.empty_like(x)
    _call(name, a, x.ctypes.data, b, n, *extra, out.ctypes.data)
    return out[0] if squeeze else out


def adrt_step(a: np.ndarray, step: int) -> np.ndarray:
    return _adrt_shaped("adrt_step", a, int(step))


def bdrt(a: np.ndarray) -> np.ndarray:
    return _adrt_shaped("bdrt", a)


def bdrt_step(a: np.ndarray, step: int) -> np.ndarray:
    return _adrt_shaped("bdrt_step", a, int(step))


def iadrt(a: np.ndarray) -> np.ndarray:
    return _adrt_shaped("iadrt", a)


def press_fmg_restriction(a: np.ndarray) -> np.ndarray:
    a = _c(a)
    squeeze = a.ndim == 3
    x = a[None] if squeeze else a
    b, n = x.shape[0], x.shape[-1]
    out = np.empty((b, 4, n - 1, n // 2), dtype=a.dtype)
    _call("fmg_restriction", a, x.ctypes.data, b, n, out.ctypes.data)
    return out[0] if squeeze else out


def _image_op(name, a, scale):
    a = _c(a)
    squeeze = a.ndim == 2
    x = a[None] if squeeze else a
    b, h, w = x.shape
    out = np.empty((b, h * scale, w * scale), dtype=a.dtype)
    _call(name, a, x.ctypes.data, b, h, w, out.ctypes.data)
    return out[0] if squeeze else out


def press_fmg_prolongation(a: np.ndarray) -> np.ndarray:
    return _image_op("fmg_prolongation", a, 2)


def press_fmg_highpass(a: np.ndarray) -> np.ndarray:
    return _image_op("fmg_highpass", a, 1)


# --- NumPy restatements of the reference's Python-level helpers -------------


def adrt_init(a: np.ndarray) -> np.ndarray:
    """Reference: src/adrt/core.py:123-176."""
    n = a.shape[-1]
    ret = np.zeros((*a.shape[:-2], 4, 2 * n - 1, n), dtype=a.dtype)
    ret[..., 0, :n, :] = np.flip(a, axis=-1).swapaxes(-1, -2)
    ret[..., 1, :n, :] = np.flip(a, axis=-2)
    ret[..., 2, :n, :] = a
    ret[..., 3, :n, :] = np.flip(a, axis=(-1, -2)).swapaxes(-1, -2)
    return ret


def truncate(a: np.ndarray) -> np.ndarray:
    """Reference: src/adrt/utils.py:191-242."""
    n = a.shape[-1]
    return np.stack(
        [
            np.flip(a[..., 0, :n, :n], axis=-2).swapaxes(-1, -2),
            np.flip(a[..., 1, :n, :n], axis=-2),
            a[..., 2, :n, :n],
            np.flip(a[..., 3, :n, :n], axis=(-1, -2)).swapaxes(-1, -2),
        ],
        axis=-3,
    )


def stitch_adrt(a: np.ndarray, remove_repeated: bool = False) -> np.ndarray:
    """Reference: src/adrt/utils.py:65-134."""
    n = a.shape[-1]
    in_rows, out_rows = 2 * n - 1, 3 * n - 2
    vc = n - (1 if remove_repeated else 0)
    ret = np.zeros((*a.shape[:-3], out_rows, 4, vc), dtype=a.dtype)
    for i in range(4):
        quad = a[..., i, :, :]
        if i % 2:
            quad = np.flip(quad, axis=(-1, -2))
        if remove_repeated:
            quad = quad[..., :-1]
        if i < 2:
            ret[..., :in_rows, i, :] = quad
        else:
            ret[..., -in_rows:, i, :] = quad
    return ret.reshape((*a.shape[:-3], out_rows, 4 * vc))


def adjoint(a: np.ndarray) -> np.ndarray:
    """Transpose of adrt: truncate(bdrt(a)).sum(-3), quadrants added in order.

    Reference: src/adrt/_wrappers.py:283-284 and tests/test_bdrt.py:310-325.
    """
    t = truncate(bdrt(a))
    return ((t[..., 0, :, :] + t[..., 1, :, :]) + t[..., 2, :, :]) + t[..., 3, :, :]


def iadrt_fmg_step(a: np.ndarray) -> np.ndarray:
    """Reference: src/adrt/core.py:265-331 (same operation order)."""
    stack = []
    for _ in range(num_iters(a.shape[-1])):
        stack.append(a)
        a = press_fmg_restriction(a)
    ret = a[..., 0, :, :]
    n = 1
    while stack:
        n *= 2
        ret = press_fmg_prolongation(ret)
        ret -= press_fmg_highpass(
            np.mean(truncate(bdrt(adrt(ret) - stack.pop())) / (n - 1), axis=-3)
        )
    return ret
