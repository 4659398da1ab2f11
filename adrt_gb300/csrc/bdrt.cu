// Backprojection (bdrt): the transpose of the forward butterfly, fused into
// multi-stage passes.
//
// The reference runs log2(n) stages over a per-quadrant buffer [S][P][2n-1]
// (S angles halving, P sections doubling, src/adrt/adrt_cdefs_bdrt.hpp:56-116):
//   left   out[s][2p][c]       = in[2s][p][c] + in[2s+1][p][c]
//   right  out[s][2p+1][c]     = in[2s][p][c+s] + in[2s+1][p][c+s+1]   (c+s+1 <= C-1)
//          out[s][2p+1][C-1-s] = in[2s][p][C-1]                         (copy)
//          out[s][2p+1][c]     = +0                                     (c >= C-s)
// after transposing the (4, 2n-1, n) input to [n][1][2n-1] (:144-161) and
// before transposing back (:170-185).
//
// bdrt stage j undoes forward stage L-1-j, so bdrt passes are forward passes
// run backwards.  One CTA owns forward row group r at forward input angle a'
// (i.e. bdrt angles a'*2^S + l, l < 2^S) and a window of W tile positions.
// Member i of the pass output lives at tile position t <-> reference offset
// t - a'*i, the same pre-shift as the forward pass, so inside the tile the
// gathers are the small residual shifts l and l+1.  Loads are one window per
// angle; stores go to a per-member shifted window.  Copy and zero rules are
// evaluated on reference offsets, exactly as in the reference.
#include "common.cuh"
#include "tune.cuh"

namespace adrtg {

// Tile width in stored offsets: 224 for float32 (tile rows of 256 positions
// with the halo, three CTAs per SM), 128 for float64 (two CTAs per SM).
template <typename T> constexpr int bwd_width() { return sizeof(T) == 4 ? 224 : 128; }
constexpr int kBwdHalo = 32;   // right halo (>= 2^S - 1)
// Threads per CTA: 512 for passes of five stages (32 tile rows; measured
// 1.4x faster than 256 at n = 1024), 256 for shorter passes (slightly faster
// there).  Occupancy is bound by shared memory, three CTAs per SM.
template <int S> constexpr int bwd_threads() { return S >= 5 ? 512 : 256; }

struct BwdPassArgs {
  const void *in;  // final-layout array (first pass) or bdrt buffer
  void *out;       // bdrt buffer, or final-layout output (last pass)
  i64 n;
  int k0;          // first forward stage covered by this pass
  i64 batch;
  i64 c_need;      // pass outputs are needed at reference offsets < c_need
  i64 cs = 0;      // row stride of the bdrt buffers (0: 2n-1)
};

// Buffer layout between passes, per (b, q): [angle s][section p][offset c],
// the reference's bdrt buffer.  After forward stage k0 there are A = 2^k0
// angles and R = n / 2^k0 sections.
// Shared-memory rows of one tile, with the forward kernel's layout rules: a
// stage sweeps each row with TPR consecutive threads, and the row stride is
// padded so the transposing first-pass loads and last-pass stores hit
// distinct banks.  A 32-element tail pad keeps the right-shifted reads of the
// last row in bounds.
template <typename T, int ROWS, int NT>
struct BwdTile {
  static constexpr int W = bwd_width<T>();
  static constexpr int TWP = W + kBwdHalo;
  static constexpr int WF = sizeof(T) == 4 ? 32 : 16;  // lanes per wavefront
  static constexpr int PAD = ROWS == 1 ? 0 : (ROWS >= WF ? 1 : WF / ROWS);
  static constexpr int RS = TWP + PAD;
  static constexpr int BUF = ROWS * RS + 32;
  static constexpr int TPR = ROWS >= 8 ? 32 : NT / ROWS;
  static constexpr int ROW_STEP = NT / TPR;
  static_assert(TWP % 32 == 0, "tile width plus halo must be a multiple of 32");
};

// Column tiles of one pass: tile positions span [0, C + a'_max * (2^S - 1)) so
// every member's pre-shifted window is covered.
static __host__ __device__ inline int bwd_col_tiles(i64 n, int k0, int S, int W) {
  const i64 C = 2 * n - 1;
  const i64 max_ext = ((i64(1) << k0) - 1) * ((1 << S) - 1);
  return (int)((C + max_ext + W - 1) / W);
}

// Per-quadrant index arithmetic is 32-bit: a quadrant holds n (2n-1) < 2^32
// elements for every n the host accepts here (checked in bdrt_forward).
template <typename T, int S, bool FIRST, bool LAST>
__global__ void __launch_bounds__(bwd_threads<S>())
bwd_pass_kernel(BwdPassArgs args) {
  constexpr int ROWS = 1 << S, NT = bwd_threads<S>();
  using TL = BwdTile<T, ROWS, NT>;
  constexpr int W = TL::W, TWP = TL::TWP, RS = TL::RS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *buf0 = reinterpret_cast<T *>(smem_raw);
  T *buf1 = buf0 + TL::BUF;

  const unsigned n = (unsigned)args.n;
  const int C = (int)(2 * args.n - 1);
  const int k0 = args.k0;
  const unsigned A_lo = 1u << k0;      // angles after this pass (pass output)
  const unsigned R_lo = n >> k0;       // sections after this pass
  const unsigned R_hi = R_lo >> S;     // sections at pass input
  const int col_tiles = bwd_col_tiles(args.n, k0, S, W);
  const unsigned cs = args.cs ? (unsigned)args.cs : (unsigned)C;  // bdrt buffer row stride

  unsigned t = blockIdx.x;
  const int ct = (int)(t % (unsigned)col_tiles); t /= (unsigned)col_tiles;
  const unsigned ap = t % A_lo; t /= A_lo;
  const unsigned r = t % R_hi; t /= R_hi;
  const unsigned q = t & 3u; t >>= 2;
  const unsigned b = t;
  const int c0 = ct * W;
  // Skip tiles that hold no member's needed offsets (member i of this tile
  // stores reference offsets >= c0 - a'*i).
  if ((i64)c0 >= args.c_need + (i64)ap * (ROWS - 1)) return;
  const size_t qoff = ((size_t)b * 4 + q) * (size_t)n * (size_t)C;  // quadrant base, final layout
  const size_t qbuf = ((size_t)b * 4 + q) * (size_t)n * (size_t)cs; // quadrant base, bdrt buffer

  // ---- load angle l = a'*2^S + l of section r, tile positions [c0, c0+TWP).
  if (FIRST) {
    // in[b][q][c][angle], angle innermost; here R_hi == 1, A_hi == n.
    const T *src = static_cast<const T *>(args.in) + qoff + ap * ROWS;
#pragma unroll 4
    for (int idx = threadIdx.x; idx < ROWS * TWP; idx += NT) {
      const int l = idx % ROWS, u = idx / ROWS;
      const int c = c0 + u;
      T v = T(0);
      if (c < C) v = src[(unsigned)c * n + l];
      buf0[l * RS + u] = v;
    }
  } else {
    const T *src = static_cast<const T *>(args.in) + qbuf + ((size_t)ap * ROWS * R_hi + r) * cs + c0;
    for (int l = threadIdx.x / TL::TPR; l < ROWS; l += TL::ROW_STEP) {
      const T *rowp = src + (size_t)l * R_hi * cs;
#pragma unroll 4
      for (int u = threadIdx.x % TL::TPR; u < TWP; u += TL::TPR) {
        T v = T(0);
        if (c0 + u < C) v = rowp[u];
        buf0[l * RS + u] = v;
      }
    }
  }
  __syncthreads();

  // ---- S transposed stages, forward local stage j = S-1 down to 0.
  // Level j+1 buffer rows: combo m, local angle la -> row m * 2^(j+1) + la.
  // Level j buffer rows:   combo m', local angle li -> row m' * 2^j + li.
  // Right rows: tile position u holds reference offset base + u of la; the
  // reference adds la + lbb while that offset is <= C - 2, copies la at C - 1
  // and writes +0 beyond.  The three ranges are computed once per row.
  T *cur = buf0, *nxt = buf1;
  const int lr = threadIdx.x % TL::TPR;
#pragma unroll
  for (int j = S - 1; j >= 0; --j) {
    const int Al_hi = 2 << j;          // local angles at level j+1
    const int Al_lo = 1 << j;          // local angles at level j
    for (int rowo = threadIdx.x / TL::TPR; rowo < ROWS; rowo += TL::ROW_STEP) {
      const int mm = rowo / Al_lo, li = rowo % Al_lo;  // level-j combo, angle
      const int m = mm >> 1;                           // parent combo at level j+1
      const T *ya = cur + (m * Al_hi + 2 * li) * RS;
      const T *yb = ya + RS;
      T *np = nxt + rowo * RS;
      if ((mm & 1) == 0) {
        // left: la + lb (positions past the buffer end are never used)
#pragma unroll
        for (int u = lr; u < TWP; u += TL::TPR) np[u] = add_rn(ya[u], yb[u]);
      } else {
        // right: reference offset of la is base + u, with the parent mapping a'*2m*2^j.
        const int base = c0 + li - (int)(ap * (unsigned)((2 * m) << j));
        const int copy_at = C - 1 - base;  // la + lbb below, copy of la here, +0 beyond
        ya += li;
        yb += li + 1;
        if (copy_at >= TWP) {
#pragma unroll
          for (int u = lr; u < TWP; u += TL::TPR) np[u] = add_rn(ya[u], yb[u]);
        } else {
#pragma unroll
          for (int u = lr; u < TWP; u += TL::TPR)
            np[u] = u < copy_at ? add_rn(ya[u], yb[u]) : (u == copy_at ? ya[u] : T(0));
        }
      }
    }
    __syncthreads();
    T *tmp = cur; cur = nxt; nxt = tmp;
  }

  // ---- store member i (section r*2^S + i at angle a') at reference offset u + c0 - a'*i.
  if (LAST) {
    // out[b][q][c][section], section innermost; A_lo == 1, a' == 0.
    T *dst = static_cast<T *>(args.out) + qoff + r * ROWS;
#pragma unroll 4
    for (int idx = threadIdx.x; idx < W * ROWS; idx += NT) {
      const int i = idx % ROWS, w = idx / ROWS;
      const int c = c0 + w;
      if (c < C) st_stream(&dst[(unsigned)c * n + i], cur[i * RS + w]);
    }
  } else {
    T *dst = static_cast<T *>(args.out) + qbuf + ((size_t)ap * R_lo + r * ROWS) * cs;
    for (int i = threadIdx.x / TL::TPR; i < ROWS; i += TL::ROW_STEP) {
      T *rowp = dst + (size_t)i * cs;
      const int cb = c0 - (int)ap * i;
#pragma unroll 4
      for (int w = threadIdx.x % TL::TPR; w < W; w += TL::TPR) {
        const int c = cb + w;
        if (c >= 0 && c < C) rowp[c] = cur[i * RS + w];
      }
    }
  }
}

// Passes of at most 5 stages (or the tuned maximum), as even as possible.
static int plan_passes_bwd(i64 n, size_t elem, int *sizes) {
  const int mf = tune_lookup(ADRT_GB300_OP_BDRT, elem == 4 ? ADRT_GB300_F32 : ADRT_GB300_F64, n).max_fused;
  return plan_stage_split(num_iters(n), mf, sizes);
}

template <typename T, int S, bool FIRST, bool LAST>
static int launch_bwd_pass(const BwdPassArgs &a, cudaStream_t st) {
  constexpr int ROWS = 1 << S, NT = bwd_threads<S>();
  const size_t smem = 2 * sizeof(T) * BwdTile<T, ROWS, NT>::BUF;
  auto kern = bwd_pass_kernel<T, S, FIRST, LAST>;
  static std::atomic<unsigned long long> configured{0};
  if (const int rc = smem_limit_once((const void *)kern, smem, configured)) return rc;
  const i64 A_lo = i64(1) << a.k0;
  const i64 col_tiles = bwd_col_tiles(a.n, a.k0, S, BwdTile<T, ROWS, NT>::W);
  const i64 tiles = a.batch * 4 * ((a.n >> a.k0) >> S) * A_lo * col_tiles;
  kern<<<(unsigned)tiles, NT, smem, st>>>(a);
  return launch_status();
}

template <typename T, bool FIRST, bool LAST>
static int bwd_dispatch_S(int S, const BwdPassArgs &a, cudaStream_t st) {
  switch (S) {
    case 0: return launch_bwd_pass<T, 0, FIRST, LAST>(a, st);
    case 1: return launch_bwd_pass<T, 1, FIRST, LAST>(a, st);
    case 2: return launch_bwd_pass<T, 2, FIRST, LAST>(a, st);
    case 3: return launch_bwd_pass<T, 3, FIRST, LAST>(a, st);
    case 4: return launch_bwd_pass<T, 4, FIRST, LAST>(a, st);
    case 5: return launch_bwd_pass<T, 5, FIRST, LAST>(a, st);
  }
  return ADRT_GB300_ERR_SHAPE;
}

template <typename T>
static int bwd_dispatch(int S, bool first, bool last, const BwdPassArgs &a, cudaStream_t st) {
  if (first && last) return bwd_dispatch_S<T, true, true>(S, a, st);
  if (first) return bwd_dispatch_S<T, true, false>(S, a, st);
  if (last) return bwd_dispatch_S<T, false, true>(S, a, st);
  return bwd_dispatch_S<T, false, false>(S, a, st);
}

// Register-level passes (bdrt_fast.cu), float32, 128 <= n <= 1024: the first
// bdrt pass undoes forward stages L-1 .. L-5, the second L-6 .. 0.
int bdrt_fast_pass1(const float *in, float *buf, i64 batch, i64 n, i64 cs, i64 need, cudaStream_t st);
int bdrt_fast_pass2(const float *buf, float *out, i64 batch, i64 n, i64 cs, i64 need, cudaStream_t st);

static bool bwd_fast_eligible(i64 n, size_t elem) {
  if (elem != 4 || n < 128 || n > 1024 || !is_pow2(n)) return false;
  const TuneConfig tc = tune_lookup(ADRT_GB300_OP_BDRT, ADRT_GB300_F32, n);
  return tc.use_fast != 0 && (tc.max_fused == 0 || tc.max_fused == 5);
}

// Pass plan: the fast path splits the forward's stages as its forward does,
// [0, L-5) and [L-5, L): the first bdrt pass undoes the last five stages, the
// second the first L-5.
static int plan_bwd(i64 n, size_t elem, int *sizes) {
  if (bwd_fast_eligible(n, elem)) {
    sizes[0] = num_iters(n) - 5;
    sizes[1] = 5;
    return 2;
  }
  return plan_passes_bwd(n, elem, sizes);
}

// Row stride of the bdrt buffers: 2n-1, padded to 8 elements on the fast
// path (16-byte aligned rows for its vector loads and stores).
static i64 bwd_cs(i64 n, size_t elem) {
  const i64 C = 2 * n - 1;
  return bwd_fast_eligible(n, elem) ? (C + 7) / 8 * 8 : C;
}

// Images per chunk.  One chunk's intermediate has a built-in budget of 1 GB
// (bdrt at n = 1024, float32, 128 images: 9.9k img/s against 8.5k with
// 48 MB chunks whose intermediate stays in L2: fewer launch tails), or the
// tuned one; chunks are balanced.
static i64 bwd_chunk(i64 batch, i64 n, size_t elem) {
  const size_t per = (size_t)4 * n * bwd_cs(n, elem) * elem;
  const int mb = tune_lookup(ADRT_GB300_OP_BDRT, elem == 4 ? ADRT_GB300_F32 : ADRT_GB300_F64, n).chunk_mb;
  const size_t budget = (size_t)(mb > 0 ? mb : 1024) << 20;
  i64 k = (i64)(budget / per);
  if (k < 1) k = 1;
  if (batch <= k) return batch;
  const i64 nchunks = (batch + k - 1) / k;
  return (batch + nchunks - 1) / nchunks;
}

size_t bwd_workspace_bytes(i64 batch, i64 n, size_t elem) {
  int sizes[16];
  const int P = plan_bwd(n, elem, sizes);
  if (P <= 1) return 0;
  const size_t per = (size_t)4 * n * bwd_cs(n, elem) * elem;
  return per * (P >= 3 ? 2 : 1) * (size_t)bwd_chunk(batch, n, elem);
}

// rows_needed: offsets of each quadrant of the result the caller reads (2n-1
// for bdrt itself, n for the adjoint, which truncates).  Undoing forward stage
// k reads offsets at most 2^k to the right of the one it writes, so the pass
// starting at forward stage k0 only has to produce offsets below
// rows_needed + 2^k0 - 1; tiles beyond are skipped and left unwritten.
template <typename T>
int bdrt_forward(const T *in, T *out, i64 batch, i64 n, void *ws, size_t ws_bytes,
                 cudaStream_t st, i64 rows_needed) {
  // The pass kernels index one quadrant (n (2n-1) elements) in 32 bits.
  if (n > 32768) return ADRT_GB300_ERR_TOO_LARGE;
  int sizes[16];
  int P = plan_bwd(n, sizeof(T), sizes);
  // Unaligned buffers take the generic passes (unpadded rows fit in the
  // workspace sized for padded ones).
  const bool fast = bwd_fast_eligible(n, sizeof(T)) && aligned32(in) && aligned32(out);
  const i64 cs = fast ? bwd_cs(n, sizeof(T)) : 2 * n - 1;
  if (!fast && bwd_fast_eligible(n, sizeof(T))) P = plan_passes_bwd(n, sizeof(T), sizes);
  const size_t per = (size_t)4 * n * cs * sizeof(T);
  const int nbuf = P <= 1 ? 0 : (P >= 3 ? 2 : 1);
  i64 chunk = bwd_chunk(batch, n, sizeof(T));
  if (nbuf) {
    const i64 fit = (i64)(ws_bytes / (per * nbuf));
    if (fit < 1 || ws == nullptr) return ADRT_GB300_ERR_WORKSPACE;
    if (fit < chunk) chunk = fit;
  }
  T *bufs[2] = {static_cast<T *>(ws),
                nbuf == 2 ? reinterpret_cast<T *>(static_cast<char *>(ws) + per * chunk) : nullptr};
  // Forward pass p covers stages [k_p, k_p + sizes[p]); run them last to first.
  int kstart[16];
  int k = 0;
  for (int p = 0; p < P; ++p) { kstart[p] = k; k += sizes[p]; }
  for (i64 b0 = 0; b0 < batch; b0 += chunk) {
    const i64 nb = (batch - b0) < chunk ? (batch - b0) : chunk;
    const void *src = in + b0 * 4 * n * (2 * n - 1);
    for (int s = 0; s < P; ++s) {
      const int p = P - 1 - s;
      const bool first = s == 0, last = s == P - 1;
      void *dst = last ? static_cast<void *>(out + b0 * 4 * n * (2 * n - 1)) : bufs[s & 1];
      const i64 C = 2 * n - 1;
      const i64 need = rows_needed + (i64(1) << kstart[p]) - 1;
      BwdPassArgs a{src, dst, n, kstart[p], nb, need < C ? need : C};
      a.cs = cs;
      int rc = ADRT_GB300_OK;
      bool done = false;
      if constexpr (sizeof(T) == 4) {
        if (fast) {
          rc = last ? bdrt_fast_pass2(static_cast<const float *>(src), static_cast<float *>(dst), nb, n, cs,
                                      a.c_need, st)
                    : bdrt_fast_pass1(static_cast<const float *>(src), static_cast<float *>(dst), nb, n, cs,
                                      a.c_need, st);
          done = true;
        }
      }
      if (!done) rc = bwd_dispatch<T>(sizes[p], first, last, a, st);
      if (rc) return rc;
      src = dst;
    }
  }
  return ADRT_GB300_OK;
}

template int bdrt_forward<float>(const float *, float *, i64, i64, void *, size_t, cudaStream_t, i64);
template int bdrt_forward<double>(const double *, double *, i64, i64, void *, size_t, cudaStream_t, i64);

}  // namespace adrtg
