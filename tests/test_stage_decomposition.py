"""The stage decomposition the register-level forward passes compute, checked
on the CPU against the reference's stage recursion, bit for bit.

A pass of S stages (n = 32 * 2^S) over 32 consecutive rows runs group 1 (the
first min(S, 2) stages on each quad of rows), then, for group-1 angle L1,
pre-shifts quad h by L1 * (h mod 2^GS) and runs GS = S - 2 fresh stages on
each set of 2^GS quads; row group (32 >> S) R + set, angle 2^GS L1 + local
angle.  Operands the reference would skip (offset below 0: it copies) are
-0.0 here, as in the kernels: x + (-0) == x.

Reference: src/adrt/adrt_cdefs_adrt.hpp:56-96 (adrt_core: out[a][c] =
in[2r][a/2][c] + in[2r+1][a/2][c - ceil(a/2)], a copy where that offset is
negative)."""

import numpy as np
import pytest

f32 = np.float32


def reference_stages(rows, stages):
    """rows: [sections][angles][C] -> the reference's recursion, `stages` times."""
    buf = rows
    for _ in range(stages):
        R, A, C = buf.shape
        out = np.empty((R // 2, 2 * A, C), dtype=buf.dtype)
        for m in range(R // 2):
            for a in range(2 * A):
                sh = (a + 1) // 2
                e, o = buf[2 * m, a >> 1], buf[2 * m + 1, a >> 1]
                out[m, a] = e
                out[m, a, sh:] = e[sh:] + o[: C - sh]
        buf = out
    return buf


def fresh_stages(rows, stages):
    """The same recursion with absent operands read as -0 (the kernels' form)."""
    buf = rows
    for _ in range(stages):
        R, A, C = buf.shape
        out = np.empty((R // 2, 2 * A, C), dtype=buf.dtype)
        for m in range(R // 2):
            for a in range(2 * A):
                sh = (a + 1) // 2
                e, o = buf[2 * m, a >> 1], buf[2 * m + 1, a >> 1]
                shifted = np.full(C, -0.0, dtype=buf.dtype)
                shifted[sh:] = o[: C - sh]
                out[m, a] = e + shifted
        buf = out
    return buf


@pytest.mark.parametrize("S", [1, 2, 3, 4, 5])
def test_pass_a_decomposition_bit_exact(S):
    n = 32 << S
    C = 2 * n - 1
    rng = np.random.default_rng(S)
    x = np.zeros((32, 1, C), dtype=f32)
    x[:, 0, :n] = rng.standard_normal((32, n)).astype(f32)
    x[rng.random(x.shape) < 0.05] = -0.0
    x[:, 0, n:] = 0.0  # the zero padding
    want = reference_stages(x.copy(), S)  # [32 >> S][2^S][C]

    g1_stages = min(S, 2)
    g1 = np.stack([fresh_stages(x[4 * h:4 * h + 4].copy(), g1_stages)
                   .reshape(-1, C) for h in range(8)])  # [8 quads][2^g1 rows][C]
    got = np.empty_like(want)
    if S == 1:
        # group 1 did the only stage: quad h holds row groups 2h, 2h + 1, angles 0, 1
        for h in range(8):
            for l1 in range(4):
                got[2 * h + (l1 >> 1), l1 & 1] = g1[h, l1]
    else:
        GS = S - 2
        for L1 in range(4):
            for st in range(8 >> GS):
                members = []
                for hl in range(1 << GS):
                    sh = L1 * hl
                    z = np.full(C, -0.0, dtype=f32)
                    z[sh:] = g1[st * (1 << GS) + hl, L1, : C - sh]
                    members.append(z)
                w = fresh_stages(np.array(members)[:, None, :], GS)[0]  # [2^GS][C]
                for l in range(1 << GS):
                    got[st, (L1 << GS) + l] = w[l]
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
