/*
 * adrt_oracle.c -- CPU restatement of the adrt reference algorithms.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA library
 * in adrt_gb300/ is compared against.  Only tests/, __graft_entry__.smoke()
 * and the CPU-baseline leg of bench.py load it.  The product path never calls
 * into it (the Python package raises when its CUDA library is missing).
 *
 * Parity of this restatement is pinned two ways:
 *   - bit-for-bit against the reference package itself (installed into
 *     baseline/_ref and its extension compiled from its own sources by
 *     oracle/Makefile, see tests/test_oracle_reference.py) on random inputs,
 *     signed zeros and edge sizes;
 *   - against the golden fixtures under tests/golden/, which were generated
 *     by that same compiled reference (tests/golden/make_golden.py).
 *
 * Every routine restates the arithmetic of one reference routine: the same
 * pairing of operands, the same operand order, the same copy-versus-add and
 * zero-fill rules.  The loops and memory layout are written fresh: stages
 * work on a per-quadrant buffer indexed [row][angle][offset] (adrt) or
 * [angle][section][offset] (bdrt), exactly the reference's 5-D buffer
 * shapes, but addressed with plain index arithmetic.
 *
 * Build: see oracle/Makefile (-O2 -fopenmp -ffp-contract=off, no fast-math:
 * the highpass filter multiplies and must not be FMA-contracted).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#define OMP(x) _Pragma(x)
#else
#define OMP(x)
#endif

typedef int64_t i64;

int adrt_oracle_num_iters(i64 n)
{
    /* ceil(log2(n)), num_iters(0) == 0.
     * Reference: src/adrt/adrt_cdefs_common.cpp:140-142, src/adrt/core.py:94-120 */
    if (n <= 1) return 0;
    int bits = 0;
    i64 v = n;
    while (v) { bits++; v >>= 1; }
    return bits - (((n & (n - 1)) == 0) ? 1 : 0);
}

int adrt_oracle_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void adrt_oracle_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ------------------------------------------------------------------------ */
/* Generic (float / double) bodies, instantiated below.                       */
/* ------------------------------------------------------------------------ */

#define DEFINE_ORACLE(T, SFX)                                                   \
                                                                                \
/* One forward butterfly stage on one quadrant buffer.                          \
 * in:  [R][A][C]  ->  out: [R/2][2A][C]                                        \
 * out[r][a][c] = in[2r][a/2][c] + in[2r+1][a/2][c - ceil(a/2)]                 \
 * when c >= ceil(a/2), otherwise a copy of the first operand.                 \
 * Reference: src/adrt/adrt_cdefs_adrt.hpp:56-96 (adrt_core).  */               \
static void fwd_stage_##SFX(const T *in, T *out, i64 R, i64 A, i64 C)          \
{                                                                               \
    const i64 R2 = R / 2, A2 = 2 * A;                                           \
    for (i64 r = 0; r < R2; ++r) {                                              \
        for (i64 a = 0; a < A2; ++a) {                                          \
            const i64 sh = (a + 1) / 2;                                         \
            const T *ea = in + ((2 * r) * A + a / 2) * C;                       \
            const T *ob = in + ((2 * r + 1) * A + a / 2) * C;                   \
            T *o = out + (r * A2 + a) * C;                                      \
            for (i64 c = 0; c < C; ++c) {                                       \
                if (c >= sh) o[c] = ea[c] + ob[c - sh];                         \
                else o[c] = ea[c];                                              \
            }                                                                   \
        }                                                                       \
    }                                                                           \
}                                                                               \
                                                                                \
/* Full forward ADRT.  in: (B, N, N)  out: (B, 4, 2N-1, N).                     \
 * Reference: src/adrt/adrt_cdefs_adrt.hpp:101-212 (adrt_basic): quadrant      \
 * flips into a [N][1][2N-1] buffer with +0 in offsets N..2N-2, log2(N)         \
 * stages, then out[q][c][a] = buf[q][0][a][c]. */                              \
int adrt_oracle_adrt_##SFX(const T *in, i64 B, i64 N, T *out)                   \
{                                                                               \
    const i64 C = 2 * N - 1;                                                    \
    const i64 QS = N * C;                                                       \
    const int L = adrt_oracle_num_iters(N);                                     \
    int err = 0;                                                                \
    OMP("omp parallel for collapse(2) schedule(dynamic)")                       \
    for (i64 b = 0; b < B; ++b) {                                               \
        for (int q = 0; q < 4; ++q) {                                           \
            T *x = (T *)malloc(sizeof(T) * (size_t)QS);                         \
            T *y = (T *)malloc(sizeof(T) * (size_t)QS);                         \
            if (!x || !y) { free(x); free(y); err = 1; continue; }              \
            const T *img = in + b * N * N;                                      \
            for (i64 r = 0; r < N; ++r) {                                       \
                T *row = x + r * C;                                             \
                for (i64 c = 0; c < N; ++c) {                                   \
                    T v;                                                        \
                    switch (q) {                                                \
                    case 0: v = img[r * N + (N - 1 - c)]; break;                \
                    case 1: v = img[(N - 1 - c) * N + r]; break;                \
                    case 2: v = img[c * N + r]; break;                          \
                    default: v = img[(N - 1 - r) * N + (N - 1 - c)]; break;     \
                    }                                                           \
                    row[c] = v;                                                 \
                }                                                               \
                for (i64 c = N; c < C; ++c) row[c] = (T)0;                      \
            }                                                                   \
            i64 R = N, A = 1;                                                   \
            for (int s = 0; s < L; ++s) {                                       \
                fwd_stage_##SFX(x, y, R, A, C);                                 \
                T *t = x; x = y; y = t;                                         \
                R /= 2; A *= 2;                                                 \
            }                                                                   \
            T *o = out + (b * 4 + q) * QS;                                      \
            for (i64 c = 0; c < C; ++c)                                         \
                for (i64 a = 0; a < N; ++a)                                     \
                    o[c * N + a] = x[a * C + c];                                \
            free(x); free(y);                                                   \
        }                                                                       \
    }                                                                           \
    return err;                                                                 \
}                                                                               \
                                                                                \
/* One forward stage in the output layout (B, 4, 2N-1, N).                     \
 * Column index of the last axis = block * 2^(k+1) + angle.                    \
 * Reference: src/adrt/adrt_cdefs_adrt.hpp:215-258 (adrt_step). */             \
int adrt_oracle_adrt_step_##SFX(const T *in, i64 B, i64 N, int k, T *out)      \
{                                                                               \
    const i64 C = 2 * N - 1;                                                    \
    const i64 E = (i64)1 << k, E2 = E * 2;                                      \
    OMP("omp parallel for collapse(3)")                                         \
    for (i64 b = 0; b < B; ++b)                                                 \
        for (int q = 0; q < 4; ++q)                                             \
            for (i64 row = 0; row < C; ++row) {                                 \
                const T *src = in + (b * 4 + q) * C * N;                        \
                T *dst = out + (b * 4 + q) * C * N;                             \
                for (i64 col = 0; col < N; ++col) {                             \
                    const i64 blk = col / E2, ang = col % E2;                   \
                    const i64 ca = 2 * blk * E + ang / 2;                       \
                    const i64 cb = (2 * blk + 1) * E + ang / 2;                 \
                    const i64 sh = (ang + 1) / 2;                               \
                    const T av = src[row * N + ca];                             \
                    if (row >= sh) dst[row * N + col] = av + src[(row - sh) * N + cb]; \
                    else dst[row * N + col] = av;                               \
                }                                                               \
            }                                                                   \
    return 0;                                                                   \
}                                                                               \
                                                                                \
/* One backprojection stage on one quadrant buffer.                             \
 * in: [S][P][C] (S angle pairs halve, P sections double) -> out [S/2][2P][C]   \
 * left  = out[s][2p][c]       = in[2s][p][c] + in[2s+1][p][c]                  \
 * right = out[s][2p+1][c - s] = in[2s][p][c] + in[2s+1][p][c+1]                \
 * right at c = C-1 is a copy of in[2s][p][C-1]; right[C-s..C) = +0.           \
 * Reference: src/adrt/adrt_cdefs_bdrt.hpp:56-116 (bdrt_core). */              \
static void bwd_stage_##SFX(const T *in, T *out, i64 S, i64 P, i64 C)          \
{                                                                               \
    const i64 S2 = S / 2, P2 = 2 * P;                                           \
    for (i64 s = 0; s < S2; ++s) {                                              \
        for (i64 p = 0; p < P; ++p) {                                           \
            const T *la = in + ((2 * s) * P + p) * C;                           \
            const T *lb = in + ((2 * s + 1) * P + p) * C;                       \
            T *left = out + (s * P2 + 2 * p) * C;                               \
            T *right = out + (s * P2 + 2 * p + 1) * C;                          \
            for (i64 c = 0; c < C; ++c) left[c] = la[c] + lb[c];                \
            for (i64 c = s; c < C - 1; ++c) right[c - s] = la[c] + lb[c + 1];   \
            right[C - 1 - s] = la[C - 1];                                       \
            for (i64 c = C - s; c < C; ++c) right[c] = (T)0;                    \
        }                                                                       \
    }                                                                           \
}                                                                               \
                                                                                \
/* Full backprojection.  in/out: (B, 4, 2N-1, N).                               \
 * Reference: src/adrt/adrt_cdefs_bdrt.hpp:121-187 (bdrt_basic): transpose     \
 * into [N][1][2N-1], log2(N) stages, transpose back. */                        \
int adrt_oracle_bdrt_##SFX(const T *in, i64 B, i64 N, T *out)                   \
{                                                                               \
    const i64 C = 2 * N - 1;                                                    \
    const i64 QS = N * C;                                                       \
    const int L = adrt_oracle_num_iters(N);                                     \
    int err = 0;                                                                \
    OMP("omp parallel for collapse(2) schedule(dynamic)")                       \
    for (i64 b = 0; b < B; ++b) {                                               \
        for (int q = 0; q < 4; ++q) {                                           \
            T *x = (T *)malloc(sizeof(T) * (size_t)QS);                         \
            T *y = (T *)malloc(sizeof(T) * (size_t)QS);                         \
            if (!x || !y) { free(x); free(y); err = 1; continue; }              \
            const T *src = in + (b * 4 + q) * QS;                               \
            for (i64 c = 0; c < C; ++c)                                         \
                for (i64 a = 0; a < N; ++a)                                     \
                    x[a * C + c] = src[c * N + a];                              \
            i64 S = N, P = 1;                                                   \
            for (int s = 0; s < L; ++s) {                                       \
                bwd_stage_##SFX(x, y, S, P, C);                                 \
                T *t = x; x = y; y = t;                                         \
                S /= 2; P *= 2;                                                 \
            }                                                                   \
            T *o = out + (b * 4 + q) * QS;                                      \
            for (i64 c = 0; c < C; ++c)                                         \
                for (i64 p = 0; p < N; ++p)                                     \
                    o[c * N + p] = x[p * C + c];                                \
            free(x); free(y);                                                   \
        }                                                                       \
    }                                                                           \
    return err;                                                                 \
}                                                                               \
                                                                                \
/* One backprojection step in the output layout.  Transposes forward stage     \
 * L-1-k; missing operands are +0 and are ADDED (unlike bdrt_core's copy).      \
 * Reference: src/adrt/adrt_cdefs_bdrt.hpp:190-244 (bdrt_step). */              \
int adrt_oracle_bdrt_step_##SFX(const T *in, i64 B, i64 N, int k, T *out)      \
{                                                                               \
    const i64 C = 2 * N - 1;                                                    \
    const int L = adrt_oracle_num_iters(N);                                     \
    const i64 E = (i64)1 << (L - k - 1);                                        \
    OMP("omp parallel for collapse(3)")                                         \
    for (i64 b = 0; b < B; ++b)                                                 \
        for (int q = 0; q < 4; ++q)                                             \
            for (i64 row = 0; row < C; ++row) {                                 \
                const T *src = in + (b * 4 + q) * C * N;                        \
                T *dst = out + (b * 4 + q) * C * N;                             \
                for (i64 col = 0; col < N; ++col) {                             \
                    const i64 blk = col / E, i = col % E;                       \
                    const i64 base = 2 * (i + E * (blk / 2));                   \
                    if ((blk & 1) == 0) {                                       \
                        dst[row * N + col] = src[row * N + base] + src[row * N + base + 1]; \
                    } else {                                                    \
                        const i64 r0 = row + i;                                 \
                        T av = (T)0, bv = (T)0;                                 \
                        if (r0 < C) av = src[r0 * N + base];                    \
                        if (r0 + 1 < C) bv = src[(r0 + 1) * N + base + 1];      \
                        dst[row * N + col] = av + bv;                           \
                    }                                                           \
                }                                                               \
            }                                                                   \
    return 0;                                                                   \
}                                                                               \
                                                                                \
/* One exact-inverse stage on one quadrant buffer.                              \
 * in: [Lc][Cc][R] -> out: [2Lc][Cc/2][R]; each (l, col) is a serial chain      \
 * from the last row down: v = 0; v += A; v -= B; v += out[row+1].              \
 * Reference: src/adrt/adrt_cdefs_iadrt.hpp:53-105 (iadrt_core). */            \
static void inv_stage_##SFX(const T *in, T *out, i64 Lc, i64 Cc, i64 R)        \
{                                                                               \
    const i64 L2 = 2 * Lc, C2 = Cc / 2;                                         \
    for (i64 l = 0; l < L2; ++l) {                                              \
        const i64 pl = l / 2;                                                   \
        for (i64 col = 0; col < C2; ++col) {                                    \
            const T *e = in + (pl * Cc + 2 * col) * R;                          \
            const T *od = in + (pl * Cc + 2 * col + 1) * R;                     \
            const int has_odd = (2 * col + 1) < Cc;                             \
            T *o = out + (l * C2 + col) * R;                                    \
            for (i64 row = R - 1; row >= 0; --row) {                            \
                T v = (T)0;                                                     \
                if ((l & 1) == 0) {                                             \
                    v += e[row];                                                \
                    if (row + 1 < R && has_odd) v -= od[row + 1];               \
                } else if (row + 1 + col < R) {                                 \
                    if (has_odd) v += od[row + 1 + col];                        \
                    v -= e[row + 1 + col];                                      \
                }                                                               \
                if (row + 1 < R) v += o[row + 1];                               \
                o[row] = v;                                                     \
            }                                                                   \
        }                                                                       \
    }                                                                           \
}                                                                               \
                                                                                \
/* Exact inverse.  in/out: (B, 4, 2N-1, N).                                     \
 * Reference: src/adrt/adrt_cdefs_iadrt.hpp:110-176 (iadrt_basic). */          \
int adrt_oracle_iadrt_##SFX(const T *in, i64 B, i64 N, T *out)                  \
{                                                                               \
    const i64 C = 2 * N - 1;                                                    \
    const i64 QS = N * C;                                                       \
    const int L = adrt_oracle_num_iters(N);                                     \
    int err = 0;                                                                \
    OMP("omp parallel for collapse(2) schedule(dynamic)")                       \
    for (i64 b = 0; b < B; ++b) {                                               \
        for (int q = 0; q < 4; ++q) {                                           \
            T *x = (T *)malloc(sizeof(T) * (size_t)QS);                         \
            T *y = (T *)malloc(sizeof(T) * (size_t)QS);                         \
            if (!x || !y) { free(x); free(y); err = 1; continue; }              \
            const T *src = in + (b * 4 + q) * QS;                               \
            for (i64 c = 0; c < N; ++c)                                         \
                for (i64 r = 0; r < C; ++r)                                     \
                    x[c * C + r] = src[r * N + c];                              \
            i64 Lc = 1, Cc = N;                                                 \
            for (int s = 0; s < L; ++s) {                                       \
                inv_stage_##SFX(x, y, Lc, Cc, C);                               \
                T *t = x; x = y; y = t;                                         \
                Lc *= 2; Cc /= 2;                                               \
            }                                                                   \
            T *o = out + (b * 4 + q) * QS;                                      \
            for (i64 r = 0; r < C; ++r)                                         \
                for (i64 c = 0; c < N; ++c)                                     \
                    o[r * N + c] = x[c * C + r];                                \
            free(x); free(y);                                                   \
        }                                                                       \
    }                                                                           \
    return err;                                                                 \
}                                                                               \
                                                                                \
/* Multigrid restriction: (B,4,2n-1,n) -> (B,4,n-1,n/2);                        \
 * out[r][c] = (x[2r][2c] + x[2r+1][2c]) / 4.                                   \
 * Reference: src/adrt/adrt_cdefs_fmg.hpp:53-73. */                             \
int adrt_oracle_fmg_restriction_##SFX(const T *in, i64 B, i64 n, T *out)       \
{                                                                               \
    const i64 Ri = 2 * n - 1, Ro = n - 1, Co = n / 2;                           \
    OMP("omp parallel for collapse(2)")                                         \
    for (i64 bq = 0; bq < B * 4; ++bq)                                          \
        for (i64 r = 0; r < Ro; ++r)                                            \
            for (i64 c = 0; c < Co; ++c) {                                      \
                const T va = in[(bq * Ri + 2 * r) * n + 2 * c];                 \
                const T vb = in[(bq * Ri + 2 * r + 1) * n + 2 * c];             \
                out[(bq * Ro + r) * Co + c] = (va + vb) / (T)4;                 \
            }                                                                   \
    return 0;                                                                   \
}                                                                               \
                                                                                \
/* Multigrid prolongation: (B,h,w) -> (B,2h,2w), 2x2 nearest repeat.            \
 * Reference: src/adrt/adrt_cdefs_fmg.hpp:75-95. */                             \
int adrt_oracle_fmg_prolongation_##SFX(const T *in, i64 B, i64 h, i64 w, T *out) \
{                                                                               \
    OMP("omp parallel for collapse(2)")                                         \
    for (i64 b = 0; b < B; ++b)                                                 \
        for (i64 r = 0; r < 2 * h; ++r)                                         \
            for (i64 c = 0; c < 2 * w; ++c)                                     \
                out[(b * 2 * h + r) * 2 * w + c] = in[(b * h + r / 2) * w + c / 2]; \
    return 0;                                                                   \
}                                                                               \
                                                                                \
/* Multigrid high-pass: 3x3 kernel [[a,b,a],[b,c,b],[a,b,a]] with              \
 * a=-1/16, b=-1/8, c=3/4, reflected edges; each tap is one rounded multiply    \
 * and the sum is (v11+v21+v31) + (v12+v22+v32) + (v13+v23+v33), left to right.\
 * Reference: src/adrt/adrt_cdefs_fmg.hpp:97-171. */                            \
int adrt_oracle_fmg_highpass_##SFX(const T *in, i64 B, i64 h, i64 w, T *out)   \
{                                                                               \
    const T ka = (T)-0.0625, kb = (T)-0.125, kc = (T)0.75;                      \
    OMP("omp parallel for collapse(2)")                                         \
    for (i64 b = 0; b < B; ++b)                                                 \
        for (i64 r = 0; r < h; ++r) {                                           \
            const T *x = in + b * h * w;                                        \
            const i64 rp = (r == 0) ? 1 : r - 1;                                \
            const i64 rn = (r == h - 1) ? r - 1 : r + 1;                        \
            for (i64 c = 0; c < w; ++c) {                                       \
                const i64 cp = (c == 0) ? 1 : c - 1;                            \
                const i64 cn = (c == w - 1) ? c - 1 : c + 1;                    \
                const T v11 = ka * x[rp * w + cp], v12 = kb * x[rp * w + c], v13 = ka * x[rp * w + cn]; \
                const T v21 = kb * x[r * w + cp], v22 = kc * x[r * w + c], v23 = kb * x[r * w + cn];    \
                const T v31 = ka * x[rn * w + cp], v32 = kb * x[rn * w + c], v33 = ka * x[rn * w + cn]; \
                out[(b * h + r) * w + c] = (v11 + v21 + v31) + (v12 + v22 + v32) + (v13 + v23 + v33);  \
            }                                                                   \
        }                                                                       \
    return 0;                                                                   \
}

DEFINE_ORACLE(float, f32)
DEFINE_ORACLE(double, f64)
