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


def reference_bdrt_stages(buf, stages):
    """The reference's transposed stages on [angles][sections][R]: angle
    pair (2 si, 2 si + 1) of each section gives sections 2 sec (left, A + B)
    and 2 sec + 1 (right[u] = A[u + si] + B[u + si + 1], a copy of A where
    B's offset is R, +0 beyond).  src/adrt/adrt_cdefs_bdrt.hpp:56-116."""
    for _ in range(stages):
        H, S, R = buf.shape
        out = np.empty((H // 2, 2 * S, R), dtype=buf.dtype)
        for si in range(H // 2):
            for sec in range(S):
                A, B = buf[2 * si, sec], buf[2 * si + 1, sec]
                out[si, 2 * sec] = A + B
                right = np.zeros(R, dtype=buf.dtype)
                if R - 1 - si > 0:
                    right[: R - 1 - si] = A[si : R - 1] + B[si + 1 : R]
                right[R - 1 - si] = A[R - 1]
                out[si, 2 * sec + 1] = right
        buf = out
    return buf


@pytest.mark.parametrize("n,ap", [(128, 0), (128, 3), (256, 5), (256, 7)])
def test_bdrt_pass1_frame_bit_exact(n, ap):
    # The register-level bdrt's first pass on input angle group a' (angles
    # 32 a' .. 32 a' + 31), five stages undone with local shifts only, in one
    # frame: row (member prefix p, step j) sits at reference offset F - a' p
    # 2^(4-j); every row reads +0 past offset 2n-2 except a row in the B role,
    # which reads -0 at exactly 2n-1 (so A + B copies A); member i is finally
    # stored a' i to the left.  Also: every member value at frame positions
    # >= 2n-1 is +0 (the tiles there store +0 without computing).
    C = 2 * n - 1
    rng = np.random.default_rng(n + ap)
    y = rng.standard_normal((n, C)).astype(f32)  # [angle][offset] of one quadrant
    y[rng.random(y.shape) < 0.05] = -0.0
    y[:, C - 3 :] = np.where(rng.random((n, 3)) < 0.5, -0.0, y[:, C - 3 :])
    want = reference_bdrt_stages(y[:, None, :].copy(), 5)  # [n/32 angles][32 sections][C]

    E = C + 31 * ap + 64  # frame positions kept
    rows = {}
    for la in range(32):
        r = np.zeros(E, dtype=f32)
        r[:C] = y[32 * ap + la]
        if la & 1:
            r[C] = -0.0
        rows[(0, la)] = r
    for j in range(5):
        new = {}
        n_ang = 32 >> j
        for (p, la) in rows:
            if la & 1:
                continue
            li = la >> 1
            A, B = rows[(p, la)], rows[(p, la + 1)]
            left = A + B
            right = np.zeros(E, dtype=f32)
            right[: E - li - 1] = A[li : E - 1] + B[li + 1 : E]
            new[(2 * p, li)] = left
            new[(2 * p + 1, li)] = right
        rows = new
        # B rows of the next step: -0 at reference offset 2n-1
        if j < 4:
            for (p, la), r in rows.items():
                if la & 1:
                    r[C + ap * p * (1 << (4 - j))] = -0.0
        assert len(rows) == 32 and n_ang // 2 * (2 << j) == 32
    for i in range(32):
        member = rows[(i, 0)]
        got = member[ap * i : ap * i + C]
        assert np.array_equal(got.view(np.uint32), want[ap, i].view(np.uint32)), i
        beyond = member[C:]
        assert np.all(beyond.view(np.uint32) == 0), i  # +0, not -0


def iadrt_stage(x, s):
    """One stage of the reference's exact inverse on [row][chain] planes
    (x: (R, n)): chain (l, col), l < 2^(s+1), col < n / 2^(s+1), reads the
    input chains E = (l/2, 2 col), O = E + 1 and runs from row R-1 down:
      l even: v = (0 + E[r]) - O[r+1] + out[r+1]   (the last two if r+1 < R)
      l odd:  v = (0 + O[r+d]) - E[r+d] (if r+d < R, else 0), d = 1 + col;
              v += out[r+1] if r+1 < R.
    src/adrt/adrt_cdefs_iadrt.hpp:53-105."""
    R, n = x.shape
    Cc = n >> s
    C2 = Cc >> 1
    out = np.empty_like(x)
    z = x.dtype.type(0)
    for l in range(2 << s):
        for col in range(C2):
            ch = l * C2 + col
            e = (l >> 1) * Cc + 2 * col
            o = e + 1
            prev = z
            for r in range(R - 1, -1, -1):
                if l % 2 == 0:
                    v = z + x[r, e]
                    if r + 1 < R:
                        v = v - x[r + 1, o]
                        v = v + prev
                else:
                    d = 1 + col
                    v = z
                    if r + d < R:
                        v = v + x[r + d, o]
                        v = v - x[r + d, e]
                    if r + 1 < R:
                        v = v + prev
                out[r, ch] = v
                prev = v
    return out


def iadrt_last5_fused(x, s0):
    """The fused kernel's sweep for stages s0 .. s0+4: one group of 32 chains
    (indices 32A + lane at every level), rows from R-1 down, the five levels
    in order at each row; each level reads the previous one at rows r, r+1
    and r+d (d = 1 + col <= 16) from a 17-row ring."""
    R, n = x.shape
    z = x.dtype.type(0)
    out = np.empty_like(x)
    H = 17
    for A in range(n >> 5):
        ring = np.zeros((5, H, 32), dtype=x.dtype)
        prev = [[z] * 32 for _ in range(5)]
        for r in range(R - 1, -1, -1):
            slot = r % H
            ring[0, slot] = x[r, 32 * A:32 * A + 32]
            for t in range(5):
                vals = []
                for lane in range(32):
                    lam, col = lane >> (4 - t), lane & ((1 << (4 - t)) - 1)
                    e = ((lam >> 1) << (5 - t)) + 2 * col
                    o, d = e + 1, 1 + col
                    if lam % 2 == 0:
                        v = z + ring[t, slot, e]
                        if r + 1 < R:
                            v = v - ring[t, (r + 1) % H, o]
                            v = v + prev[t][lane]
                    else:
                        v = z
                        if r + d < R:
                            assert d <= 16
                            v = v + ring[t, (r + d) % H, o]
                            v = v - ring[t, (r + d) % H, e]
                        if r + 1 < R:
                            v = v + prev[t][lane]
                    prev[t][lane] = v
                    vals.append(v)
                if t < 4:
                    ring[t + 1, slot] = vals
                else:
                    out[r, 32 * A:32 * A + 32] = vals
    return out


@pytest.mark.parametrize("n", [32, 64])
def test_iadrt_fused_last5_equals_stages(oracle_mod, n):
    # The staged restatement against the oracle's inverse, then the fused
    # sweep against the staged one, bit for bit (float32, signed zeros).
    rng = np.random.default_rng(n)
    y = rng.standard_normal((4, 2 * n - 1, n)).astype(f32)
    y[rng.random(y.shape) < 0.05] = -0.0
    L = n.bit_length() - 1
    staged = np.stack([y[q] for q in range(4)])
    for s in range(L):
        staged = np.stack([iadrt_stage(staged[q], s) for q in range(4)])
    want = oracle_mod.iadrt(y)
    assert np.array_equal(staged.view(np.uint32), want.view(np.uint32))
    pre = np.stack([y[q] for q in range(4)])
    for s in range(L - 5):
        pre = np.stack([iadrt_stage(pre[q], s) for q in range(4)])
    fused = np.stack([iadrt_last5_fused(pre[q], L - 5) for q in range(4)])
    assert np.array_equal(fused.view(np.uint32), staged.view(np.uint32))


def iadrt_stage_row_sweep(x, s):
    """The single-stage kernel's odd chains swept by input row (stages with
    C2 >= 32): a warp holds 32 consecutive columns of one odd l, lane lags
    d0 + lane; at input row x each lane computes its output row x - d, into a
    32-row ring; row x - d0 is stored once lane 0 has written it.  Even
    chains as in the reference."""
    R, n = x.shape
    Cc = n >> s
    C2 = Cc >> 1
    assert C2 >= 32
    out = iadrt_stage(x, s)  # even chains (and, for now, odd ones)
    z = x.dtype.type(0)
    for l in range(1, 2 << s, 2):
        for col0 in range(0, C2, 32):
            ring = np.full((32, 32), np.nan, dtype=x.dtype)
            prev = [z] * 32
            d0 = 1 + col0
            stored = np.full((R, 32), np.nan, dtype=x.dtype)
            for xr in range(R - 1 + d0 + 31, d0 - 1, -1):
                for lane in range(32):
                    d = d0 + lane
                    y = xr - d
                    if y < 0 or y >= R:
                        continue
                    if xr >= R:
                        v = z  # rows R-d .. R-1: +0
                    else:
                        e = (l >> 1) * Cc + 2 * (col0 + lane)
                        v = z + x[xr, e + 1]
                        v = v - x[xr, e]
                        v = v + prev[lane]
                    prev[lane] = v
                    ring[y & 31, lane] = v
                yc = xr - d0
                if yc < R:
                    stored[yc] = ring[yc & 31]
            chs = l * C2 + col0 + np.arange(32)
            assert not np.isnan(stored).any()
            out[:, chs] = stored
    return out


@pytest.mark.parametrize("n,s", [(64, 0), (128, 0), (128, 1)])
def test_iadrt_row_sweep_equals_stage(n, s):
    rng = np.random.default_rng(n + s)
    x = rng.standard_normal((2 * n - 1, n)).astype(f32)
    x[rng.random(x.shape) < 0.05] = -0.0
    want = iadrt_stage(x, s)
    got = iadrt_stage_row_sweep(x, s)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("n", [32, 64, 128])
def test_forward_support_is_plus_zero(n):
    # After k stages a row at angle a is exactly +0 at offsets >= n + a (the
    # padding's sums): the bound behind the intermediate's row length and
    # pass B's zero tiles.  Inputs include -0 and NaN inside the image.
    C = 2 * n - 1
    rng = np.random.default_rng(n)
    x = np.zeros((n, 1, C), dtype=f32)
    x[:, 0, :n] = rng.standard_normal((n, n)).astype(f32)
    x[:, 0, :n][rng.random((n, n)) < 0.05] = -0.0
    x[n // 2, 0, n // 3] = np.nan
    buf = x
    for k in range(1, n.bit_length()):
        buf = reference_stages(buf, 1)
        for a in range(buf.shape[1]):
            tail = buf[:, a, n + a:]
            assert np.all(tail.view(np.uint32) == 0), (k, a)
