// Forward ADRT: fused multi-stage passes.
//
// The reference runs log2(n) butterfly stages over a per-quadrant buffer of
// shape [R][A][2n-1] (rows, angles, offsets), each stage
//   out[r][a][c] = in[2r][a/2][c] + in[2r+1][a/2][c - ceil(a/2)]   (c >= ceil(a/2))
//   out[r][a][c] = in[2r][a/2][c]                                   (otherwise)
// (src/adrt/adrt_cdefs_adrt.hpp:56-96), after flipping the image into four
// quadrants (:123-186) and before transposing to (4, 2n-1, n) (:195-210).
//
// Here the stages are grouped into passes of S <= 5 stages.  One CTA of a pass
// owns 2^S consecutive input rows (row groups) at one input angle a', and a
// window of W output offsets.  Within the pass, the stage that merges members
// with local angle l and parity p shifts the odd member by (a' * 2^j + l + p);
// the part a' * 2^j summed over the pass is a' * i for member i, so member i is
// loaded already shifted by a' * i and only the small residual shift l + p
// (< 2^S) remains inside the tile.  The copy-versus-add decision is still made
// on the reference's own offset index, so every output is the same sequence of
// adds as in the reference.
//
// The first pass reads the image directly (the quadrant flips and the +0 pad
// are fused into its load); the last pass writes the (4, 2n-1, n) layout
// directly (the transpose is fused into its store).  Passes in between use a
// workspace laid out like the reference's buffer: [b][q][R][A][2n-1].
#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "fwd_fast.cuh"
#include "tune.cuh"

namespace adrtg {

// Output offsets per tile: 256 for n >= 128, else 128 (narrow images waste
// wide tiles; measured 2x faster at n = 32 with 128, 1.2-1.3x slower at
// n = 128..256), unless the autotuner's table says otherwise.
constexpr int kFwdWNarrow = 128, kFwdWWide = 256;
static int fwd_width(long long n, int dtype) {
  const int w = tune_lookup(ADRT_GB300_OP_ADRT, dtype, n).width;
  if (w == kFwdWNarrow || w == kFwdWWide) return w;
  return n >= 128 ? kFwdWWide : kFwdWNarrow;
}
template <typename T> constexpr int dtype_code() { return sizeof(T) == 4 ? ADRT_GB300_F32 : ADRT_GB300_F64; }
constexpr int kFwdHalo = 32;  // halo columns kept left of the tile (>= 2^S - 1)
constexpr int kFwdThreads = 256;
// Threads per CTA of the pass kernels (the ragged kernel uses kFwdThreads):
// 512 for float64 passes of five stages (measured 1.15x faster at n = 1024),
// 256 otherwise (float32 five-stage passes measured 3 % slower with 512).
template <typename T, int S> constexpr int fwd_threads() { return (sizeof(T) == 8 && S >= 5) ? 512 : 256; }

struct FwdPassArgs {
  const void *in;  // image (first pass) or stage-k0 buffer
  void *out;       // stage-(k0+S) buffer, or final output (last pass)
  i64 n;           // image side
  int k0;          // index of the first stage of this pass
  i64 batch;
  i64 cs_out = 0;  // row stride of a non-final output buffer (0: 2n-1)
};

// Shared-memory rows of one tile.  During a stage a row is swept by TPR
// consecutive threads (a whole warp, or several warps for few rows), so stage
// accesses never conflict.  The transposing accesses (first-pass loads of
// quadrants 1 and 2, last-pass stores) have consecutive threads on
// consecutive rows: the row stride is TWP (a multiple of 32) plus PAD, chosen
// so that the rows and positions one shared-memory wavefront covers (32 lanes
// of 4-byte, 16 of 8-byte elements) fall in distinct banks.
template <typename T, int ROWS, int W, int NT = kFwdThreads>
struct FwdTile {
  static constexpr int TWP = W + kFwdHalo;                  // positions per row
  static constexpr int WF = sizeof(T) == 4 ? 32 : 16;       // lanes per wavefront
  static constexpr int PAD = ROWS == 1 ? 0 : (ROWS >= WF ? 1 : WF / ROWS);
  static constexpr int RS = TWP + PAD;
  static constexpr int BUF = ROWS * RS;
  static constexpr int TPR = ROWS >= 8 ? 32 : NT / ROWS;  // threads per row
  static constexpr int ROW_STEP = NT / TPR;               // rows in flight
  static_assert(TWP % 32 == 0, "tile width plus halo must be a multiple of 32");
};

// Loads for non-first passes go through L2 only (the ragged kernel reads
// intermediates written by other CTAs of the same launch).
template <typename T>
__device__ __forceinline__ T ld_l2(const T *p) { return __ldcg(p); }

// One tile of one pass.  `tile` enumerates (b, q, r, a', column tile), column
// tile fastest; `smem_raw` holds two tile buffers.
template <typename T, int S, bool FIRST, bool LAST, int kFwdW, int NT = kFwdThreads>
__device__ __forceinline__ void fwd_tile(const FwdPassArgs &args, i64 tile,
                                         unsigned char *smem_raw) {
  constexpr int ROWS = 1 << S;
  using TL = FwdTile<T, ROWS, kFwdW, NT>;
  constexpr int TWP = TL::TWP, RS = TL::RS;
  T *buf0 = reinterpret_cast<T *>(smem_raw);
  T *buf1 = buf0 + TL::BUF;

  const i64 n = args.n;
  const i64 C = 2 * n - 1;
  const int k0 = args.k0;
  const i64 A_in = i64(1) << k0;            // angles at the pass input
  const i64 R_in = n >> k0;                 // row groups at the pass input
  const i64 R_out = R_in >> S;
  const i64 A_out = A_in << S;
  const int col_tiles = (int)((C + kFwdW - 1) / kFwdW);

  // Decode the tile: (b, q, r, a', column tile), column tile fastest.
  // 32-bit decode: tile indices fit in 32 bits, and 64-bit division is a
  // long instruction sequence that small tiles cannot amortise.
  unsigned t = (unsigned)tile;
  const int ct = (int)(t % (unsigned)col_tiles); t /= (unsigned)col_tiles;
  const i64 ap = t % (unsigned)A_in; t /= (unsigned)A_in;
  const i64 r = t % (unsigned)R_out; t /= (unsigned)R_out;
  const int q = (int)(t & 3u); t >>= 2;
  const i64 b = t;
  const i64 c0 = (i64)ct * kFwdW;
  const i64 tbase = c0 - kFwdHalo;  // reference offset of tile position 0 (before pre-shift)

  // Support: after k stages a row at angle a is +0 at offsets >= n + a (a
  // digital line over the row group rises by at most a, and every term past
  // the image is the +0 padding).  This pass's outputs have angles below
  // (a'+1) 2^S, so from offset sup_out on the whole tile is +0: a last pass
  // stores zeros there without computing, other passes skip the tile (the
  // next pass bounds its loads by each input row's own support, n + a').  A
  // padded fast-path intermediate (cs_out set) is read in whole 16-byte
  // chunks up to its row length, so there every offset below cs_out is
  // written.
  const i64 sup_out = n + (ap + 1) * ROWS - 1;
  const i64 skip_from = (!LAST && args.cs_out > sup_out) ? args.cs_out : sup_out;
  if (c0 >= skip_from) {
    if (LAST) {
      T *dst = static_cast<T *>(args.out) + ((size_t)b * 4 + q) * (size_t)C * (unsigned)n + (unsigned)ap * ROWS;
      for (int idx = threadIdx.x; idx < kFwdW * ROWS; idx += NT) {
        const int l = idx % ROWS, w = idx / ROWS;
        const int c = (int)c0 + w;
        if (c < (int)C) st_stream(&dst[(unsigned)c * (unsigned)n + l], T(0));
      }
    }
    return;
  }
  const int sup_in = (int)(FIRST ? n : (n + ap < C ? n + ap : C));

  // ---- load: member i, tile position u  <->  reference offset tbase + u - a'*i.
  // Offsets below 0 do not exist in the reference (it copies instead of adding
  // there); they are stored as -0.0, and e + (-0) == e for every e, so the
  // stages below add unconditionally.  Offsets n..2n-2 of the first pass are
  // the reference's +0 padding.  Offsets inside one image or quadrant are
  // 32-bit (n <= 32768, checked by the host).
  const unsigned un = (unsigned)n;
  const int lr = threadIdx.x % TL::TPR;
  if (FIRST) {
    const T *img = static_cast<const T *>(args.in) + (size_t)b * un * un;
    if (q == 1 || q == 2) {
      // Columns of the image: consecutive threads take consecutive rows i
      // (adjacent in memory).  Quadrant 1 runs up the column, 2 down.
#pragma unroll 4
      for (int idx = threadIdx.x; idx < ROWS * TWP; idx += NT) {
        const int i = idx % ROWS, u = idx / ROWS;
        const int ref = (int)tbase + u;  // a' == 0 in the first pass
        T v = ref < 0 ? T(-0.0) : T(0);
        if (ref >= 0 && ref < (int)un) {
          const unsigned c = (unsigned)ref, row = q == 1 ? un - 1 - c : c;
          v = img[row * un + (unsigned)r * ROWS + i];
        }
        buf0[i * RS + u] = v;
      }
    } else {
      // Rows of the image read from their right end (quadrant 0 row R0,
      // quadrant 3 row n-1-R0).
      for (int i = threadIdx.x / TL::TPR; i < ROWS; i += TL::ROW_STEP) {
        const unsigned R0 = (unsigned)r * ROWS + i;
        const T *rowp = img + (q == 0 ? R0 : un - 1 - R0) * un + (un - 1);
#pragma unroll 4
        for (int u = lr; u < TWP; u += TL::TPR) {
          const int ref = (int)tbase + u;
          T v = ref < 0 ? T(-0.0) : T(0);
          if (ref >= 0 && ref < (int)un) v = rowp[-ref];
          buf0[i * RS + u] = v;
        }
      }
    }
  } else {
    const T *src = static_cast<const T *>(args.in) + ((size_t)b * 4 + q) * un * (size_t)C;
    const unsigned row0 = (unsigned)r * ROWS * (unsigned)A_in + (unsigned)ap;
    for (int i = threadIdx.x / TL::TPR; i < ROWS; i += TL::ROW_STEP) {
      const T *rowp = src + (size_t)(row0 + (unsigned)i * (unsigned)A_in) * (unsigned)C;
      const int rb = (int)tbase - (int)ap * i;
#pragma unroll 4
      for (int u = lr; u < TWP; u += TL::TPR) {
        const int ref = rb + u;
        T v = ref < 0 ? T(-0.0) : T(0);
        if (ref >= 0 && ref < sup_in) v = ld_l2(&rowp[ref]);
        buf0[i * RS + u] = v;
      }
    }
  }
  __syncthreads();

  // ---- S stages in shared memory: row m*2A + 2li + p of the output is
  // row 2m*A + li plus row (2m+1)*A + li shifted by li + p.
  T *cur = buf0, *nxt = buf1;
#pragma unroll
  for (int j = 0; j < S; ++j) {
    const int Al_in = 1 << j, Al_out = 2 << j;
    for (int rowo = threadIdx.x / TL::TPR; rowo < ROWS; rowo += TL::ROW_STEP) {
      const int m = rowo / Al_out, lo = rowo % Al_out;
      const int li = lo >> 1, sh = li + (lo & 1);
      const T *ep = cur + ((2 * m) * Al_in + li) * RS;
      const T *op = cur + ((2 * m + 1) * Al_in + li) * RS - sh;  // row index >= 1, so in bounds
      T *np = nxt + rowo * RS;
      for (int u = lr; u < TWP; u += TL::TPR) np[u] = add_rn(ep[u], op[u]);
    }
    __syncthreads();
    T *tmp = cur; cur = nxt; nxt = tmp;
  }

  // ---- store: local angle l is global angle a' * 2^S + l of row group r.
  if (LAST) {
    // out[b][q][c][a], angle innermost; here R_out == 1 and A_out == n.
    T *dst = static_cast<T *>(args.out) + ((size_t)b * 4 + q) * (size_t)C * un + (unsigned)ap * ROWS;
#pragma unroll 4
    for (int idx = threadIdx.x; idx < kFwdW * ROWS; idx += NT) {
      const int l = idx % ROWS, w = idx / ROWS;
      const int c = (int)c0 + w;
      if (c < (int)C) st_stream(&dst[(unsigned)c * un + l], cur[l * RS + kFwdHalo + w]);
    }
  } else {
    // Rows of the buffer hold cs offsets (cs <= C: a padded fast-path
    // intermediate keeps only its rows' supports).
    const unsigned cs = args.cs_out ? (unsigned)args.cs_out : (unsigned)C;
    T *dst = static_cast<T *>(args.out) + ((size_t)b * 4 + q) * un * (size_t)cs +
             ((size_t)r * A_out + (size_t)ap * ROWS) * cs + c0;
#pragma unroll 4
    for (int idx = threadIdx.x; idx < ROWS * kFwdW; idx += NT) {
      const int l = idx / kFwdW, w = idx % kFwdW;
      if ((unsigned)c0 + w < cs) dst[(unsigned)l * cs + (unsigned)w] = cur[l * RS + kFwdHalo + w];
    }
  }
}

template <typename T, int S, bool FIRST, bool LAST, int W>
__global__ void __launch_bounds__(fwd_threads<T, S>())
fwd_pass_kernel(FwdPassArgs args) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  fwd_tile<T, S, FIRST, LAST, W, fwd_threads<T, S>()>(args, blockIdx.x, smem_raw);
}

// Tiles in one pass of one image for tile width W.
static __host__ __device__ i64 fwd_pass_tiles(i64 n, int S, int W) {
  const i64 C = 2 * n - 1;
  return 4 * (n >> S) * ((C + W - 1) / W);
}

// ---- host side --------------------------------------------------------------

// Split L stages into passes of at most 5 stages (or the tuned maximum), as
// even as possible.
static int plan_passes(int L, int *sizes, int max_fused = 5) { return plan_stage_split(L, max_fused, sizes); }

template <typename T, int S, bool FIRST, bool LAST, int W>
static int launch_fwd_pass_w(const FwdPassArgs &a, cudaStream_t st) {
  constexpr int ROWS = 1 << S;
  const size_t smem = 2 * sizeof(T) * FwdTile<T, ROWS, W>::BUF;
  auto kern = fwd_pass_kernel<T, S, FIRST, LAST, W>;
  static std::atomic<unsigned long long> configured{0};  // per instantiation: devices done
  if (const int rc = smem_limit_once((const void *)kern, smem, configured)) return rc;
  const i64 tiles = a.batch * fwd_pass_tiles(a.n, S, W);
  kern<<<(unsigned)tiles, fwd_threads<T, S>(), smem, st>>>(a);
  return launch_status();
}

template <typename T, int S, bool FIRST, bool LAST>
static int launch_fwd_pass(const FwdPassArgs &a, cudaStream_t st) {
  if (fwd_width(a.n, dtype_code<T>()) == kFwdWWide) return launch_fwd_pass_w<T, S, FIRST, LAST, kFwdWWide>(a, st);
  return launch_fwd_pass_w<T, S, FIRST, LAST, kFwdWNarrow>(a, st);
}

template <typename T, bool FIRST, bool LAST>
static int dispatch_S(int S, const FwdPassArgs &a, cudaStream_t st) {
  switch (S) {
    case 0: return launch_fwd_pass<T, 0, FIRST, LAST>(a, st);
    case 1: return launch_fwd_pass<T, 1, FIRST, LAST>(a, st);
    case 2: return launch_fwd_pass<T, 2, FIRST, LAST>(a, st);
    case 3: return launch_fwd_pass<T, 3, FIRST, LAST>(a, st);
    case 4: return launch_fwd_pass<T, 4, FIRST, LAST>(a, st);
    case 5: return launch_fwd_pass<T, 5, FIRST, LAST>(a, st);
  }
  return ADRT_GB300_ERR_SHAPE;
}

template <typename T>
static int dispatch_pass(int S, bool first, bool last, const FwdPassArgs &a, cudaStream_t st) {
  if (first && last) return dispatch_S<T, true, true>(S, a, st);
  if (first) return dispatch_S<T, true, false>(S, a, st);
  if (last) return dispatch_S<T, false, true>(S, a, st);
  return dispatch_S<T, false, false>(S, a, st);
}

// Images per chunk: the intermediate of one chunk is meant to stay in L2
// (48 MB, or the tuned budget).
static i64 fwd_chunk(i64 batch, i64 n, size_t elem) {
  const size_t per = (size_t)4 * n * (2 * n - 1) * elem;
  const int mb = tune_lookup(ADRT_GB300_OP_ADRT, elem == 4 ? ADRT_GB300_F32 : ADRT_GB300_F64, n).chunk_mb;
  const size_t budget = (size_t)(mb > 0 ? mb : 48) << 20;
  i64 k = (i64)(budget / per);
  if (k < 1) k = 1;
  return k < batch ? k : batch;
}

// Fast path for float32, 64 <= n <= 1024 (adrt_fwd_fast.cu).
bool fast_forward_eligible(i64 n, size_t elem);
size_t fast_workspace_bytes(i64 batch, i64 n);
int fast_inter_cs(i64 n);
int adrt_forward_fast(const float *in, float *out, i64 batch, i64 n, void *ws, size_t ws_bytes,
                      cudaStream_t st);


static bool use_fast_path(i64 n, size_t elem) {
  return fast_forward_eligible(n, elem) && tune_lookup(ADRT_GB300_OP_ADRT, ADRT_GB300_F32, n).use_fast != 0;
}

static int fwd_max_fused(i64 n, size_t elem) {
  return tune_lookup(ADRT_GB300_OP_ADRT, elem == 4 ? ADRT_GB300_F32 : ADRT_GB300_F64, n).max_fused;
}

size_t fwd_workspace_bytes(i64 batch, i64 n, size_t elem) {
  if (use_fast_path(n, elem)) return fast_workspace_bytes(batch, n);
  int sizes[16];
  const int P = plan_passes(num_iters(n), sizes, fwd_max_fused(n, elem));
  if (P <= 1) return 0;
  const size_t per = (size_t)4 * n * (2 * n - 1) * elem;
  return per * (P >= 3 ? 2 : 1) * (size_t)fwd_chunk(batch, n, elem);
}

template <typename T>
int adrt_forward(const T *in, T *out, i64 batch, i64 n, void *ws, size_t ws_bytes,
                 cudaStream_t st) {
  if constexpr (sizeof(T) == 4) {
    if (use_fast_path(n, sizeof(T)) && aligned32(in) && aligned32(out))
      return adrt_forward_fast(reinterpret_cast<const float *>(in), reinterpret_cast<float *>(out),
                               batch, n, ws, ws_bytes, st);
  }
  // The pass kernels index one image or quadrant (n (2n-1) elements) in 32 bits.
  if (n > 32768) return ADRT_GB300_ERR_TOO_LARGE;
  int sizes[16];
  const int P = plan_passes(num_iters(n), sizes, fwd_max_fused(n, sizeof(T)));
  const size_t per = (size_t)4 * n * (2 * n - 1) * sizeof(T);
  const int nbuf = P <= 1 ? 0 : (P >= 3 ? 2 : 1);
  i64 chunk = fwd_chunk(batch, n, sizeof(T));
  if (nbuf) {
    const i64 fit = (i64)(ws_bytes / (per * nbuf));
    if (fit < 1 || ws == nullptr) return ADRT_GB300_ERR_WORKSPACE;
    if (fit < chunk) chunk = fit;
  }
  T *bufs[2] = {static_cast<T *>(ws), nbuf == 2 ? reinterpret_cast<T *>(static_cast<char *>(ws) + per * chunk) : nullptr};
  for (i64 b0 = 0; b0 < batch; b0 += chunk) {
    const i64 nb = (batch - b0) < chunk ? (batch - b0) : chunk;
    int k0 = 0;
    const void *src = in + b0 * n * n;
    for (int p = 0; p < P; ++p) {
      const bool first = p == 0, last = p == P - 1;
      void *dst = last ? static_cast<void *>(out + b0 * 4 * n * (2 * n - 1)) : bufs[p & 1];
      FwdPassArgs a{src, dst, n, k0, nb};
      int rc = dispatch_pass<T>(sizes[p], first, last, a, st);
      if (rc) return rc;
      k0 += sizes[p];
      src = dst;
    }
  }
  return ADRT_GB300_OK;
}

template int adrt_forward<float>(const float *, float *, i64, i64, void *, size_t, cudaStream_t);
template int adrt_forward<double>(const double *, double *, i64, i64, void *, size_t, cudaStream_t);



// ---------------------------------------------------------------------------
// Ragged batches: images of different power-of-two sizes in one persistent
// launch.  CTAs take tickets from a device queue of (image, pass, tile) items
// (all first-pass items, largest images first, then all second-pass items).
// A second-pass item waits until every first-pass tile of its image has been
// counted.  Every item a waiting CTA depends on has a smaller ticket and is
// held by a CTA that is already running and never waits itself, so the waits
// always end; each wait is still bounded (by %globaltimer), and on expiry the
// kernel raises the error word and stops taking work.
// ---------------------------------------------------------------------------

// Item kinds: a generic pass tile, or a tile of the fast float32 passes
// (pass A at n = 1024; pass B for 64 <= n <= 1024, reading the padded
// intermediate [q][32][n/32][cs] that pass A wrote).
enum { RAGGED_GENERIC = 0, RAGGED_FAST_A = 1, RAGGED_FAST_B = 2 };

struct RaggedImage {
  i64 in_off, out_off, inter_off;  // element offsets in the packed buffers
  int n, s0, s1;                   // side, stages of pass 0 and pass 1 (0: none)
  int tiles0;                      // tiles of pass 0
  int kind0, kind1;                // item kinds of pass 0 and pass 1
  int cs;                          // intermediate row stride (0: 2n-1)
  int pad;
};

// An item is `count` consecutive tiles of one pass of one image (small
// generic tiles are grouped so that the per-item ticket and barriers are paid
// on enough work).
struct RaggedItem {
  int image, pass, tile, count;
};

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

template <typename T, bool FIRST, bool LAST>
__device__ __forceinline__ void ragged_tile_S(int S, const FwdPassArgs &a, i64 tile,
                                              unsigned char *smem) {
  switch (S) {
    case 0: fwd_tile<T, 0, FIRST, LAST, kFwdWNarrow>(a, tile, smem); break;
    case 1: fwd_tile<T, 1, FIRST, LAST, kFwdWNarrow>(a, tile, smem); break;
    case 2: fwd_tile<T, 2, FIRST, LAST, kFwdWNarrow>(a, tile, smem); break;
    case 3: fwd_tile<T, 3, FIRST, LAST, kFwdWNarrow>(a, tile, smem); break;
    case 4: fwd_tile<T, 4, FIRST, LAST, kFwdWNarrow>(a, tile, smem); break;
    default: fwd_tile<T, 5, FIRST, LAST, kFwdWNarrow>(a, tile, smem); break;
  }
}

// Item bodies of the ragged kernel, each kept out of line: inlined into one
// loop, the generic and fast tiles' register needs add up and spill.
template <typename T, bool FIRST, bool LAST>
__device__ __noinline__ void ragged_generic_item(int S, const FwdPassArgs a, i64 tile, unsigned char *smem) {
  ragged_tile_S<T, FIRST, LAST>(S, a, tile, smem);
}

// Register first pass of n = 32 * 2^S: item t = (quadrant, 32-row block R,
// column tile), column tile fastest.
// The sweep length is fixed per column tile at compile time: every tile but
// the last is full; the last sweeps only its own iterations.
template <int S, class Hook>
__device__ __forceinline__ void ragged_fast_a_tile(const float *img, float *inter_img, int t, float *xs,
                                                   const Hook &hook) {
  using P = fast::PassA<S>;
  constexpr int last = P::TILES - 1;
  const int q = t / (P::TILES * (P::n / 32)), R = (t / P::TILES) % (P::n / 32), ct = t % P::TILES;
  if (ct == last)
    fast::pass_a_tile<S, fast::pass_a_nit<S>(last)>(img, inter_img, q, R, ct, xs, hook);
  else
    fast::pass_a_tile<S, fast::NCH / 32>(img, inter_img, q, R, ct, xs, hook);
}

template <class Hook>
__device__ __forceinline__ void ragged_fast_a_item(int S, const float *img, float *inter_img, int t, float *xs,
                                                   const Hook &hook) {
  switch (S) {
    case 5: ragged_fast_a_tile<5>(img, inter_img, t, xs, hook); break;
    case 4: ragged_fast_a_tile<4>(img, inter_img, t, xs, hook); break;
    case 3: ragged_fast_a_tile<3>(img, inter_img, t, xs, hook); break;
    case 2: ragged_fast_a_tile<2>(img, inter_img, t, xs, hook); break;
    default: ragged_fast_a_tile<1>(img, inter_img, t, xs, hook); break;
  }
}

template <class Hook>
__device__ __forceinline__ void ragged_fast_b_item(const float *inter_img, float *out_img, int n, int cs, int t,
                                                   float *xs, const Hook &hook) {
  const int ctn = fast::pass_b_col_tiles(n);
  fast::pass_b_tile<fast::LD_CG, true>(inter_img, out_img, n, cs, (t / ctn) % 4, t / (ctn * 4), t % ctn, xs,
                                       hook);
}

// Descriptors of the item a CTA works on and of the one it fetched next
// (image -1: no item).
struct RaggedSlots {
  RaggedItem item[2];
  RaggedImage image[2];
};

// Thread 0 only: item `t` (a ticket) and its image into slot `s`.
__device__ __forceinline__ void ragged_fetch(RaggedSlots &sl, int s, unsigned t, int n_items,
                                             const RaggedImage *__restrict__ imgs,
                                             const RaggedItem *__restrict__ items) {
  RaggedItem it;
  it.image = -1;
  if (t < (unsigned)n_items) {
    it = items[t];
    sl.image[s] = imgs[it.image];
  }
  sl.item[s] = it;
}

// Fetches the next item when a fast tile calls it (thread 0; the others do
// nothing).
struct RaggedPrefetch {
  RaggedSlots *sl;
  int s;
  unsigned t;
  int n_items;
  const RaggedImage *imgs;
  const RaggedItem *items;
  __device__ __forceinline__ void operator()() const {
    if (threadIdx.x == 0) ragged_fetch(*sl, s, t, n_items, imgs, items);
  }
};

// ctl[0]: next ticket, ctl[1]: error word.
// Two CTAs per SM: the persistent loop inlines every stage count, and without
// a bound the compiler spends registers that halve the resident CTAs.
// Each CTA claims its next ticket when it starts an item and reads that
// item's descriptors during the current one (in a fast tile once its loads
// are in flight, after a generic item's tiles), so that no item starts with
// a chain of dependent global loads.  A CTA that has seen an image's first
// pass complete does not poll that image's counter again.
template <typename T>
__global__ void __launch_bounds__(kFwdThreads, 2)
ragged_fwd_kernel(const T *__restrict__ in, T *__restrict__ out, T *__restrict__ inter,
                  const RaggedImage *__restrict__ imgs, const RaggedItem *__restrict__ items,
                  int n_items, unsigned *ctl, unsigned *counters, unsigned long long wait_ns) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ RaggedSlots sl;
  __shared__ int s_ok;
  __shared__ int s_seen;  // last image whose first pass this CTA saw complete
  if (threadIdx.x == 0) {
    ragged_fetch(sl, 0, atomicAdd(&ctl[0], 1u), n_items, imgs, items);
    s_seen = -1;
  }
  __syncthreads();
  for (int slot = 0;; slot ^= 1) {
    const RaggedItem item = sl.item[slot];
    if (item.image < 0) break;
    const RaggedImage im = sl.image[slot];
    unsigned next = 0;
    if (threadIdx.x == 0) next = atomicAdd(&ctl[0], 1u);
    const RaggedPrefetch prefetch{&sl, slot ^ 1, next, n_items, imgs, items};
    if (item.pass == 1) {
      if (threadIdx.x == 0) {
        int ok = 1;
        if (s_seen != item.image) {
          const unsigned long long t0 = global_ns();
          const volatile unsigned *done = counters + item.image;
          const volatile unsigned *err = ctl + 1;
          while (*done < (unsigned)im.tiles0) {
            if (*err != 0u || global_ns() - t0 > wait_ns) {
              ok = 0;
              atomicExch(&ctl[1], 1u);
              break;
            }
            __nanosleep(128);
          }
          __threadfence();
          if (ok) s_seen = item.image;
        }
        s_ok = ok;
      }
      __syncthreads();
      if (!s_ok) break;
    }
    if constexpr (sizeof(T) == 4) {
      float *xs = reinterpret_cast<float *>(smem_raw);
      const int kind = item.pass == 0 ? im.kind0 : im.kind1;
      if (kind == RAGGED_FAST_A)
        ragged_fast_a_item(im.s0, reinterpret_cast<const float *>(in) + im.in_off,
                           reinterpret_cast<float *>(inter) + im.inter_off, item.tile, xs, prefetch);
      else if (kind == RAGGED_FAST_B)
        ragged_fast_b_item(reinterpret_cast<const float *>(inter) + im.inter_off,
                           reinterpret_cast<float *>(out) + im.out_off, im.n, im.cs, item.tile, xs, prefetch);
      if (kind != RAGGED_GENERIC) {
        __syncthreads();
        if (item.pass == 0 && im.s1 > 0 && threadIdx.x == 0) {
          __threadfence();
          atomicAdd(&counters[item.image], 1u);
        }
        continue;
      }
    }
    FwdPassArgs a;
    a.n = im.n;
    a.batch = 1;
    a.cs_out = im.cs;
    for (int t = item.tile; t < item.tile + item.count; ++t) {
      if (t > item.tile) __syncthreads();  // the previous tile is done with shared memory
      if (item.pass == 0) {
        a.in = in + im.in_off;
        a.k0 = 0;
        if (im.s1 == 0) {
          a.out = out + im.out_off;
          ragged_generic_item<T, true, true>(im.s0, a, t, smem_raw);
        } else {
          a.out = inter + im.inter_off;
          ragged_generic_item<T, true, false>(im.s0, a, t, smem_raw);
        }
      } else {
        a.in = inter + im.inter_off;
        a.out = out + im.out_off;
        a.k0 = im.s0;
        ragged_generic_item<T, false, true>(im.s1, a, t, smem_raw);
      }
    }
    prefetch();
    __syncthreads();
    if (item.pass == 0 && im.s1 > 0 && threadIdx.x == 0) {
      __threadfence();
      atomicAdd(&counters[item.image], 1u);
    }
  }
}

// Workspace: [images][items][ctl x2 + counters][intermediates], each part
// 256-byte aligned.
struct RaggedPlan {
  size_t off_imgs, off_items, off_ctl, off_inter, total;
  i64 n_items, inter_elems;
};

static size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

// Per-image plan of a ragged batch: passes, item kinds, tiles, intermediate.
struct RaggedImagePlan {
  int s0, s1, kind0, kind1, cs;
  i64 tiles0, tiles1, inter_elems;
};

// Tiles per item: generic tiles of S stages hold 2^S rows x 160 positions;
// they are grouped to about 16k elements per item.  Fast tiles: one each.
static int ragged_group(int kind, int S) {
  if (kind != RAGGED_GENERIC) return 1;
  const int per = (1 << S) * (kFwdWNarrow + kFwdHalo);
  const int g = 16384 / per;
  return g < 1 ? 1 : g;
}

static i64 ragged_items(i64 tiles, int kind, int S) {
  const int g = ragged_group(kind, S);
  return (tiles + g - 1) / g;
}

static bool ragged_fast_size(i64 n, size_t elem) {
  return elem == 4 && fast_forward_eligible(n, elem) && tune_lookup(ADRT_GB300_OP_ADRT, ADRT_GB300_F32, n).use_fast != 0;
}

// fast: the image may use the fast tiles (its size allows it, and its input
// and output are 32-byte aligned for their vector loads and stores).
static RaggedImagePlan ragged_image_plan(i64 n, size_t elem, bool fast) {
  RaggedImagePlan ip{};
  const int L = num_iters(n);
  if (fast && ragged_fast_size(n, elem)) {
    ip.s0 = L - 5;
    ip.s1 = 5;
    ip.cs = fast_inter_cs(n);
    // The register first pass (S = L - 5 >= 1 stages).
    ip.kind0 = RAGGED_FAST_A;
    ip.kind1 = RAGGED_FAST_B;
    ip.tiles0 = 4 * (n / 32) * ((ip.cs + fast::W - 1) / fast::W);
    ip.tiles1 = 4 * (n / 32) * fast::pass_b_col_tiles((int)n);
    ip.inter_elems = 4 * n * ip.cs;
    return ip;
  }
  int sz[16];
  const int P = plan_passes(L, sz);
  ip.s0 = sz[0];
  ip.s1 = P == 2 ? sz[1] : 0;
  ip.tiles0 = fwd_pass_tiles(n, ip.s0, kFwdWNarrow);
  ip.tiles1 = P == 2 ? fwd_pass_tiles(n, ip.s1, kFwdWNarrow) : 0;
  ip.inter_elems = P == 2 ? 4 * n * (2 * n - 1) : 0;
  return ip;
}

// One image's slot in the intermediate buffer: room for either plan, a
// multiple of 64 elements so that every slot starts 256-byte aligned.
static i64 ragged_inter_slot(i64 n, size_t elem) {
  i64 e = ragged_image_plan(n, elem, false).inter_elems;
  if (ragged_fast_size(n, elem)) {
    const i64 f = ragged_image_plan(n, elem, true).inter_elems;
    if (f > e) e = f;
  }
  return (e + 63) / 64 * 64;
}

// Workspace layout from per-image upper bounds (the items and intermediate
// of either plan), so that it does not depend on the buffers' alignment.
static int ragged_plan(const int64_t *sizes, i64 count, size_t elem, RaggedPlan &p) {
  i64 items = 0, inter = 0;
  for (i64 i = 0; i < count; ++i) {
    const i64 n = sizes[i];
    if (n < 1 || !is_pow2(n) || n > 1024) return ADRT_GB300_ERR_SHAPE;
    const RaggedImagePlan g = ragged_image_plan(n, elem, false);
    i64 it = ragged_items(g.tiles0, g.kind0, g.s0) + ragged_items(g.tiles1, g.kind1, g.s1);
    if (ragged_fast_size(n, elem)) {
      const RaggedImagePlan f = ragged_image_plan(n, elem, true);
      const i64 fi = ragged_items(f.tiles0, f.kind0, f.s0) + ragged_items(f.tiles1, f.kind1, f.s1);
      if (fi > it) it = fi;
    }
    items += it;
    inter += ragged_inter_slot(n, elem);
  }
  p.n_items = items;
  p.inter_elems = inter;
  p.off_imgs = 0;
  p.off_items = align256(sizeof(RaggedImage) * (size_t)count);
  p.off_ctl = p.off_items + align256(sizeof(RaggedItem) * (size_t)items);
  p.off_inter = p.off_ctl + align256(sizeof(unsigned) * (size_t)(2 + count));
  p.total = p.off_inter + align256(elem * (size_t)inter);
  return ADRT_GB300_OK;
}

size_t ragged_workspace_bytes(const int64_t *sizes, i64 count, size_t elem, int *rc) {
  RaggedPlan p;
  *rc = ragged_plan(sizes, count, elem, p);
  return *rc ? 0 : p.total;
}

// Pinned host staging for a launch's descriptors, one per device, so that
// their upload is asynchronous (a copy from pageable memory would first wait
// for the stream's earlier work).  Reused once its previous upload has
// completed (an event recorded after it); grown as needed.  The first call
// on a device allocates it: that call should come before any stream capture.
struct RaggedStaging {
  std::mutex mu;
  void *host = nullptr;
  size_t cap = 0;
  cudaEvent_t done = nullptr;
};

static RaggedStaging &ragged_staging(int dev) {
  static RaggedStaging st[64];
  return st[dev & 63];
}

// Wall-clock bound on one wait (the whole batch runs in far less).
constexpr unsigned long long kRaggedWaitNs = 4000000000ull;

template <typename T>
int adrt_ragged(const T *in, T *out, const int64_t *sizes, i64 count, void *ws, size_t ws_bytes,
                unsigned long long wait_ns, i64 starve_image, cudaStream_t st) {
  RaggedPlan p;
  int rc = ragged_plan(sizes, count, sizeof(T), p);
  if (rc) return rc;
  if (ws == nullptr || ws_bytes < p.total) return ADRT_GB300_ERR_WORKSPACE;
  if (p.n_items > 0x7fffffff) return ADRT_GB300_ERR_TOO_LARGE;
  // Host-side descriptors.
  std::vector<RaggedImage> imgs((size_t)count);
  i64 in_off = 0, out_off = 0, inter_off = 0;
  std::vector<RaggedImagePlan> plans((size_t)count);
  for (i64 i = 0; i < count; ++i) {
    const i64 n = sizes[i];
    const bool fast = aligned32(in + in_off) && aligned32(out + out_off);
    const RaggedImagePlan ip = plans[(size_t)i] = ragged_image_plan(n, sizeof(T), fast);
    RaggedImage &im = imgs[(size_t)i];
    im.in_off = in_off;
    im.out_off = out_off;
    im.inter_off = inter_off;
    im.n = (int)n;
    im.s0 = ip.s0;
    im.s1 = ip.s1;
    im.tiles0 = (int)ragged_items(ip.tiles0, ip.kind0, ip.s0);  // pass-0 items the counter reaches
    im.kind0 = ip.kind0;
    im.kind1 = ip.kind1;
    im.cs = ip.cs;
    im.pad = 0;
    // Fault injection for tests: the image's second pass waits for one more
    // first-pass tile than exists, so its wait can only expire.
    if (i == starve_image && im.s1 > 0) im.tiles0 += 1;
    in_off += n * n;
    out_off += 4 * n * (2 * n - 1);
    inter_off += ragged_inter_slot(n, sizeof(T));
  }
  // Items: first passes (largest images first), then second passes.
  std::vector<i64> order((size_t)count);
  for (i64 i = 0; i < count; ++i) order[(size_t)i] = i;
  std::stable_sort(order.begin(), order.end(), [&](i64 a, i64 b) { return sizes[a] > sizes[b]; });
  std::vector<RaggedItem> items;
  items.reserve((size_t)p.n_items);
  for (int pass = 0; pass < 2; ++pass)
    for (i64 oi : order) {
      const RaggedImagePlan &ip = plans[(size_t)oi];
      const i64 nt = pass == 0 ? ip.tiles0 : ip.tiles1;
      const int g = ragged_group(pass == 0 ? ip.kind0 : ip.kind1, pass == 0 ? ip.s0 : ip.s1);
      for (i64 t = 0; t < nt; t += g)
        items.push_back(RaggedItem{(int)oi, pass, (int)t, (int)(nt - t < g ? nt - t : g)});
    }
  char *base = static_cast<char *>(ws);
  {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return ADRT_GB300_ERR_CUDA;
    RaggedStaging &sg = ragged_staging(dev);
    std::lock_guard<std::mutex> lock(sg.mu);
    const size_t bi = sizeof(RaggedImage) * imgs.size(), bt = sizeof(RaggedItem) * items.size();
    if (sg.done == nullptr && cudaEventCreateWithFlags(&sg.done, cudaEventDisableTiming) != cudaSuccess)
      return ADRT_GB300_ERR_CUDA;
    if (cudaEventSynchronize(sg.done) != cudaSuccess) return ADRT_GB300_ERR_CUDA;  // previous upload done
    if (sg.cap < bi + bt) {
      if (sg.host) cudaFreeHost(sg.host);
      sg.host = nullptr;
      sg.cap = 0;
      if (cudaMallocHost(&sg.host, bi + bt) != cudaSuccess) return ADRT_GB300_ERR_CUDA;
      sg.cap = bi + bt;
    }
    char *h = static_cast<char *>(sg.host);
    std::memcpy(h, imgs.data(), bi);
    std::memcpy(h + bi, items.data(), bt);
    if (cudaMemcpyAsync(base + p.off_imgs, h, bi, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(base + p.off_items, h + bi, bt, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaEventRecord(sg.done, st) != cudaSuccess ||
        cudaMemsetAsync(base + p.off_ctl, 0, sizeof(unsigned) * (size_t)(2 + count), st) != cudaSuccess)
      return ADRT_GB300_ERR_CUDA;
  }
  // float32 items may be fast-pass tiles, which need fast::SMEM.
  constexpr size_t smem_generic = 2 * sizeof(T) * FwdTile<T, 32, kFwdWNarrow>::BUF;
  constexpr size_t smem = sizeof(T) == 4 && fast::SMEM > smem_generic ? fast::SMEM : smem_generic;
  auto kern = ragged_fwd_kernel<T>;
  static std::atomic<unsigned long long> configured{0};
  if (const int rc = smem_limit_once((const void *)kern, smem, configured)) return rc;
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kFwdThreads, smem);
  if (per_sm < 1) per_sm = 1;
  i64 grid = (i64)sms * per_sm;
  const i64 n_items = (i64)items.size();  // <= p.n_items, the layout's capacity
  if (grid > n_items) grid = n_items;
  if (grid < 1) return ADRT_GB300_OK;
  unsigned *ctl = reinterpret_cast<unsigned *>(base + p.off_ctl);
  kern<<<(unsigned)grid, kFwdThreads, smem, st>>>(
      in, out, reinterpret_cast<T *>(base + p.off_inter),
      reinterpret_cast<const RaggedImage *>(base + p.off_imgs),
      reinterpret_cast<const RaggedItem *>(base + p.off_items), (int)n_items, ctl, ctl + 2,
      wait_ns ? wait_ns : kRaggedWaitNs);
  return launch_status();
}

template int adrt_ragged<float>(const float *, float *, const int64_t *, i64, void *, size_t,
                                unsigned long long, i64, cudaStream_t);
template int adrt_ragged<double>(const double *, double *, const int64_t *, i64, void *, size_t,
                                 unsigned long long, i64, cudaStream_t);

// Byte offset of the error word in the workspace of a ragged call.
size_t ragged_error_offset(const int64_t *sizes, i64 count, size_t elem) {
  RaggedPlan p;
  if (ragged_plan(sizes, count, elem, p)) return 0;
  return p.off_ctl + sizeof(unsigned);
}

}  // namespace adrtg
