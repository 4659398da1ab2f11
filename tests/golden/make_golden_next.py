"""Generate golden_next.npz: fixtures for interp_to_cart, unstitch_adrt,
coord_adrt and coord_cart_to_adrt from the reference package.

Run here, where the reference checkout exists and its extension has been
compiled by ``make -C oracle ref``:

    python tests/golden/make_golden_next.py

Every array is the output of the reference's own code (imported through
oracle/ref.py) on seeded inputs.
"""

from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import ref  # noqa: E402


def main() -> None:
    A = ref.load()
    if A is None:
        raise SystemExit("reference not available: run `make -C oracle install-ref REF_SRC=<adrt checkout>`")
    out = {}
    rng = np.random.default_rng(4321)
    for dt in ("float32", "float64"):
        for n in (2, 4, 8, 16, 32, 64):
            y = rng.standard_normal((2, 4, 2 * n - 1, n)).astype(dt)
            y[0, :, -3:] = -0.0
            out[f"interp_{dt}_n{n}_in"] = y
            out[f"interp_{dt}_n{n}_out"] = A.utils.interp_to_cart(y)
    for n in (1, 4, 16):
        y = rng.standard_normal((3, 4, 2 * n - 1, n)).astype(np.float32)
        for rr in (False, True):
            if rr and n == 1:
                continue
            s = A.utils.stitch_adrt(y, remove_repeated=rr)
            out[f"unstitch_n{n}_rr{int(rr)}_in"] = s
            out[f"unstitch_n{n}_rr{int(rr)}_out"] = A.utils.unstitch_adrt(s)
    for n in (2, 4, 16, 64):
        c = A.utils.coord_adrt(n)
        out[f"coord_n{n}_offset"] = c.offset
        out[f"coord_n{n}_angle"] = c.angle
    for dt in ("float32", "float64"):
        theta = rng.uniform(-4.0, 4.0, (1000,)).astype(dt)
        theta[:8] = np.array([0, np.pi / 4, -np.pi / 4, np.pi / 2, -np.pi / 2, np.pi, 3 * np.pi / 4, 1e-7], dtype=dt)
        t = rng.uniform(-0.75, 0.75, (1000,)).astype(dt)
        for n in (4, 64):
            r = A.utils.coord_cart_to_adrt(theta, t, n)
            k = f"cart_{dt}_n{n}"
            out[f"{k}_theta"] = theta
            out[f"{k}_t"] = t
            out[f"{k}_q"] = r.quadrant
            out[f"{k}_h"] = r.height
            out[f"{k}_s"] = r.slope
            out[f"{k}_f"] = r.factor
    np.savez_compressed(os.path.join(HERE, "golden_next.npz"), **out)
    print(f"wrote {len(out)} arrays")


if __name__ == "__main__":
    main()
