"""Autotuner for the launch configuration of the forward and transposed
(bdrt) transforms.

For one (op, n, dtype) it times every candidate configuration on a synthetic
batch with CUDA events, checks that each candidate's output is bit-identical
to the built-in configuration's (the knobs change tiling and staging only,
never the arithmetic), and installs the fastest in the library's table
(``adrt_gb300_tune_set``).  Knobs (see include/adrt_gb300.h):

* ``width``: forward tile width in offsets, 128 or 256;
* ``max_fused``: stages fused in shared memory per pass (3, 4 or 5), which
  sets the number of passes through HBM/L2;
* ``chunk_mb``: budget of one chunk's intermediate buffer (images per
  launch: small chunks keep it in L2, large ones cut launch tails);
* ``use_fast``: the float32 fast forward kernels (64 <= n <= 1024) or the
  generic pass kernels.

Tables persist as JSON keyed by the device name: ``save()`` / ``load()``
(default path ``$ADRT_GB300_TUNE_FILE`` or ``~/.cache/adrt_gb300/tune.json``).
"""

from __future__ import annotations

import ctypes
import itertools
import json
import os
from dataclasses import asdict, dataclass

import torch

from . import _lib

__all__ = ["Config", "get", "set_config", "reset", "candidates", "autotune", "save", "load", "TuneResult"]

OPS = {"adrt": _lib.OP_ADRT, "bdrt": _lib.OP_BDRT}


@dataclass(frozen=True)
class Config:
    width: int = 0
    max_fused: int = 0
    chunk_mb: int = 0
    use_fast: int = -1


@dataclass
class TuneResult:
    op: str
    n: int
    dtype: str
    best: Config
    best_ms: float
    default_ms: float
    timings: list  # (Config, ms per call)


def _dt(dtype) -> int:
    if dtype in (torch.float32, "float32", "f32"):
        return _lib.F32
    if dtype in (torch.float64, "float64", "f64"):
        return _lib.F64
    raise TypeError(f"unsupported dtype {dtype}")


def get(op: str, n: int, dtype) -> Config:
    vals = [ctypes.c_int() for _ in range(4)]
    rc = _lib.load().adrt_gb300_tune_get(OPS[op], _dt(dtype), n, *[ctypes.byref(v) for v in vals])
    _lib.check(rc, "tune_get")
    return Config(*[v.value for v in vals])


def set_config(op: str, n: int, dtype, cfg: Config) -> None:
    rc = _lib.load().adrt_gb300_tune_set(OPS[op], _dt(dtype), n, cfg.width, cfg.max_fused, cfg.chunk_mb,
                                         cfg.use_fast)
    _lib.check(rc, "tune_set")


def reset() -> None:
    _lib.load().adrt_gb300_tune_reset()


def candidates(op: str, n: int, dtype) -> list:
    """Configurations worth timing for (op, n, dtype); the built-in one first."""
    L = max(0, n.bit_length() - 1)
    fused = [0] + [m for m in (4, 3) if m < L and -(-L // m) != -(-L // 5)]
    chunks = [0, 96, 1024]
    out = [Config()]
    if op == "adrt":
        fast = [-1, 0] if (_dt(dtype) == _lib.F32 and 64 <= n <= 1024) else [-1]
        for uf, w, mf, ch in itertools.product(fast, (0, 128, 256), fused, chunks):
            if uf == -1 and _dt(dtype) == _lib.F32 and 64 <= n <= 1024 and mf != 0:
                continue  # the fast path has a fixed two-pass plan
            c = Config(w, mf, ch, uf)
            if c not in out:
                out.append(c)
    else:
        for mf, ch in itertools.product(fused, chunks):
            c = Config(0, mf, ch, -1)
            if c not in out:
                out.append(c)
    return out


def _runner(op):
    from ._ops import adrt, bdrt

    return adrt if op == "adrt" else bdrt


def _synthetic(op, n, dtype, batch, device):
    g = torch.Generator(device=device)
    g.manual_seed(1234 + n)
    x = torch.rand((batch, n, n), generator=g, device=device, dtype=torch.float32).to(dtype)
    if op == "bdrt":
        from ._ops import adrt

        x = adrt(x)
    return x


def autotune(op: str = "adrt", n: int = 1024, dtype=torch.float32, *, batch: int | None = None, reps: int = 5,
             apply: bool = True, device="cuda", min_gain: float = 0.01) -> TuneResult:
    """Times the candidates of (op, n, dtype) and installs the fastest, if it
    beats the built-in configuration by at least `min_gain` (relative);
    tune at the batch size the transform will run at."""
    dtype = torch.float32 if _dt(dtype) == _lib.F32 else torch.float64
    es = 4 if dtype == torch.float32 else 8
    if batch is None:
        per = 4 * n * (2 * n - 1) * es
        batch = max(1, min(64, (512 << 20) // per))
    fn = _runner(op)
    x = _synthetic(op, n, dtype, batch, device)
    previous = get(op, n, dtype)
    set_config(op, n, dtype, Config())
    ref = fn(x).clone()
    timings = []
    s = torch.cuda.current_stream(device)
    try:
        for cfg in candidates(op, n, dtype):
            set_config(op, n, dtype, cfg)
            y = fn(x)
            if not torch.equal(y.view(torch.int64 if es == 8 else torch.int32),
                               ref.view(torch.int64 if es == 8 else torch.int32)):
                raise RuntimeError(f"tuning candidate {cfg} changed the result of {op} n={n}")
            del y
            fn(x)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ms = []
            for _ in range(reps):
                e0.record(s)
                fn(x)
                e1.record(s)
                e1.synchronize()
                ms.append(e0.elapsed_time(e1))
            ms.sort()
            timings.append((cfg, ms[len(ms) // 2]))
    finally:
        set_config(op, n, dtype, previous)
    best, best_ms = select(timings, min_gain)
    default_ms = timings[0][1]
    if apply:
        set_config(op, n, dtype, best)
    return TuneResult(op, n, "float32" if es == 4 else "float64", best, best_ms, default_ms, timings)


def select(timings, min_gain: float = 0.01):
    """(config, ms) to install from [(config, ms), ...] whose first entry is
    the built-in configuration: the fastest candidate, unless it beats the
    built-in one by less than `min_gain` (relative) -- differences within
    timing noise, or candidates that launch identically at the tuning batch,
    must not pick a configuration that is worse elsewhere."""
    best, best_ms = min(timings, key=lambda t: t[1])
    if best_ms > (1.0 - min_gain) * timings[0][1]:
        return timings[0]
    return best, best_ms


def _default_path():
    return os.environ.get("ADRT_GB300_TUNE_FILE") or os.path.join(os.path.expanduser("~"), ".cache", "adrt_gb300",
                                                                   "tune.json")


def save(results, path: str | None = None) -> str:
    """Writes tuned entries (TuneResult list) for the current device."""
    path = path or _default_path()
    dev = torch.cuda.get_device_name()
    data = {}
    if os.path.exists(path):
        with open(path) as f:
            data = json.load(f)
    entries = data.setdefault(dev, [])
    for r in results:
        entries[:] = [e for e in entries if (e["op"], e["n"], e["dtype"]) != (r.op, r.n, r.dtype)]
        entries.append({"op": r.op, "n": r.n, "dtype": r.dtype, **asdict(r.best), "ms": r.best_ms})
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    with open(path, "w") as f:
        json.dump(data, f, indent=1)
    return path


def load(path: str | None = None) -> int:
    """Installs the saved entries for the current device; returns how many."""
    path = path or _default_path()
    if not os.path.exists(path):
        return 0
    with open(path) as f:
        data = json.load(f)
    k = 0
    for e in data.get(torch.cuda.get_device_name(), []):
        set_config(e["op"], e["n"], e["dtype"], Config(e["width"], e["max_fused"], e["chunk_mb"], e["use_fast"]))
        k += 1
    return k
