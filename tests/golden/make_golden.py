"""Generate the golden fixtures in this directory from the reference package.

Run here, where the reference checkout exists and its extension has been
compiled by ``make -C oracle ref``:

    python tests/golden/make_golden.py

Every array in ``golden.npz`` is the output of the reference's own compiled
code (karlotness/adrt, imported through oracle/ref.py) on seeded inputs.  The
GPU tests and the oracle tests compare against these arrays bit for bit.
"""

from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import ref  # noqa: E402


def signed_zero_image(rng, n, dtype):
    x = rng.standard_normal((n, n)).astype(dtype)
    x[: max(1, n // 2)] = -0.0
    return x


def main() -> None:
    A = ref.load()
    if A is None:
        raise SystemExit("reference not available: run `make -C oracle install-ref REF_SRC=<adrt checkout>`")
    out = {}
    # Small uniform [0,1) image: 64 x 64 float32, seed 0; adrt and bdrt of it.
    x = np.random.default_rng(0).random((64, 64), dtype=np.float32)
    y = A.adrt(x)
    out["cfg1_x"] = x
    out["cfg1_adrt"] = y
    out["cfg1_bdrt"] = A.bdrt(y)
    rng = np.random.default_rng(1234)
    for dt in ("float32", "float64"):
        for n in (1, 2, 4, 8, 16, 32):
            x = signed_zero_image(rng, n, dt)
            xb = rng.standard_normal((3, n, n)).astype(dt)
            y = A.adrt(x)
            yb = A.adrt(xb)
            yz = y.copy()
            yz[:, -2:] = -0.0
            k = f"{dt}_n{n}"
            out[f"{k}_x"] = x
            out[f"{k}_xb"] = xb
            out[f"{k}_adrt"] = y
            out[f"{k}_adrt_b"] = yb
            out[f"{k}_yz"] = yz
            out[f"{k}_bdrt"] = A.bdrt(yz)
            out[f"{k}_bdrt_b"] = A.bdrt(yb)
            out[f"{k}_iadrt"] = A.iadrt(y)
            out[f"{k}_iadrt_b"] = A.iadrt(yb)
            for s in range(A.core.num_iters(n)):
                out[f"{k}_adrt_step{s}"] = A.core.adrt_step(A.core.adrt_init(x), s)
                out[f"{k}_bdrt_step{s}"] = A.core.bdrt_step(yz, s)
            if n >= 2:
                out[f"{k}_restrict"] = A._wrappers._press_fmg_restriction(yb)
                out[f"{k}_highpass"] = A._wrappers._press_fmg_highpass(xb)
                out[f"{k}_fmg_step"] = A.core.iadrt_fmg_step(yb)
            out[f"{k}_prolong"] = A._wrappers._press_fmg_prolongation(xb)
    # Full-multigrid inverse on an exact ADRT of a smooth image.
    xs = np.arange(16 * 16, dtype=np.float32).reshape(16, 16) / 256.0
    out["fmg_src"] = xs
    out["fmg_inv"] = A.iadrt_fmg(A.adrt(xs))
    out["fmg_inv_max2"] = A.iadrt_fmg(A.adrt(xs), max_iters=2)
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    print(f"wrote {len(out)} arrays")


if __name__ == "__main__":
    main()
