// 3x3 convolutions of the learned CG preconditioner on the tcgen05 tensor
// cores: bf16 operands staged by TMA, f32 accumulators in TMEM.
//
// Activations are bf16 NHWC (batch, h, w, c); weights bf16 [9][c_out][c_in]
// (tap = 3 * dy + dx).  Zero padding of the 3x3 window comes from the TMA
// unit's zero fill of out-of-range coordinates.
//
// conv_kernel (forward, and input gradient with flipped/transposed weights):
//   one CTA computes a 128-pixel x c_out tile; the K loop runs over 9 taps x
//   (c_in / ck) channel chunks; A (pixels x ck, K-major) is one TMA box of the
//   activation tensor shifted by the tap, B (c_out x ck, K-major) one box of
//   the weights.  Epilogue: v = acc (+ bias) (+ addend); relu; mask select.
// wgrad_kernel (weight gradient):
//   D[(tap, ci)][co] = sum over pixels of x[p + d_tap][ci] * dy[p][co]; M rows
//   are (tap, channel block) segments of the activation tensor, N = c_out, K
//   = pixels.  Both operands are MN-major (channels contiguous, as stored).
//   The pixel range is split across CTAs, which add their partial sums into
//   the f32 gradient with atomics.
//
// Warp roles (128 threads): warp 0 lane 0 issues TMA, warp 1 allocates TMEM
// and lane 0 issues MMAs, all four warps run the epilogue (warp w owns TMEM
// lanes 32w..32w+31 = tile rows).

#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "../../include/adrt_gb300_net.h"
#include "common.cuh"
#include "sm100.cuh"

namespace adrtg {
namespace net {

using namespace sm100;
using bf16 = __nv_bfloat16;

constexpr int kThreads = 128;
constexpr int kStages = 4;
constexpr int kWgradK = 64;  // pixels per wgrad K stage

// Error bits of the network kernels' bounded waits.
constexpr unsigned kErrProducer = 1u, kErrMma = 2u, kErrEpilogue = 4u;

static __device__ unsigned g_net_err;
static unsigned *g_net_err_ptr[64];
static std::mutex g_net_err_mu;

unsigned *net_error_word() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lock(g_net_err_mu);
  if (!g_net_err_ptr[dev]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_net_err) != cudaSuccess) return nullptr;
    g_net_err_ptr[dev] = static_cast<unsigned *>(p);
  }
  return g_net_err_ptr[dev];
}

struct ConvArgs {
  bf16 *out;
  const float *bias;
  const bf16 *addend;
  const bf16 *mask;
  int c_out;
  int ck;       // channels per K chunk (32 or 64)
  int kchunks;  // c_in / ck
  int relu;
  int w;
  int tiles_per_image;
  int rows_per_tile;  // 128 / w when w < 128
  unsigned *err;
};

__device__ __forceinline__ bool bf16_positive(unsigned short h) { return !(h & 0x8000u) && (h & 0x7FFFu); }

__device__ __forceinline__ float bf16_lo(unsigned u) { return __uint_as_float(u << 16); }
__device__ __forceinline__ float bf16_hi(unsigned u) { return __uint_as_float(u & 0xFFFF0000u); }

__device__ __forceinline__ unsigned pack_bf16(float a, float b) {
  const unsigned lo = __bfloat16_as_ushort(__float2bfloat16_rn(a));
  const unsigned hi = __bfloat16_as_ushort(__float2bfloat16_rn(b));
  return lo | (hi << 16);
}

__device__ __forceinline__ unsigned char *align1024(unsigned char *p) {
  return reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(p) + 1023) & ~uintptr_t(1023));
}

__global__ void __launch_bounds__(kThreads) conv_kernel(const __grid_constant__ CUtensorMap tx,
                                                        const __grid_constant__ CUtensorMap tw, ConvArgs a) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char *smem = align1024(smem_raw);
  const int N = a.c_out;
  const unsigned a_bytes = 128u * a.ck * 2u;
  const unsigned b_bytes = (unsigned)N * a.ck * 2u;
  const unsigned stage_bytes = a_bytes + b_bytes;
  uint64_t *full = reinterpret_cast<uint64_t *>(smem + kStages * stage_bytes);
  uint64_t *empty = full + kStages;
  uint64_t *done = empty + kStages;
  unsigned *tmem_slot = reinterpret_cast<unsigned *>(done + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tile = blockIdx.x;
  const int img = tile / a.tiles_per_image;
  const int tin = tile % a.tiles_per_image;
  int x0, y0;
  if (a.w >= 128) {
    const int p0 = tin * 128;
    y0 = p0 / a.w;
    x0 = p0 % a.w;
  } else {
    y0 = tin * a.rows_per_tile;
    x0 = 0;
  }
  const unsigned tcols = N < 32 ? 32u : (unsigned)N;
  const int KT = 9 * a.kchunks;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    fence_mbar_init();
    tma_prefetch_desc(&tx);
    tma_prefetch_desc(&tw);
  }
  if (warp == 1) tmem_alloc(tmem_slot, tcols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const unsigned tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    for (int kt = 0; kt < KT; ++kt) {
      const int s = kt % kStages;
      if (kt >= kStages) mbar_wait(&empty[s], ((kt / kStages) - 1) & 1, a.err, kErrProducer);
      unsigned char *sa = smem + s * stage_bytes;
      mbar_arrive_expect_tx(&full[s], stage_bytes);
      const int tap = kt / a.kchunks, c0 = (kt % a.kchunks) * a.ck;
      tma_load_4d(sa, &tx, &full[s], c0, x0 + tap % 3 - 1, y0 + tap / 3 - 1, img);
      tma_load_3d(sa + a_bytes, &tw, &full[s], c0, 0, tap);
    }
  } else if (warp == 1 && lane == 0) {
    const uint32_t idesc = idesc_bf16_f32(128, N, 0, 0);
    const unsigned layout = a.ck == 64 ? 2u : 4u;
    const unsigned sbo = a.ck == 64 ? 1024u : 512u;
    for (int kt = 0; kt < KT; ++kt) {
      const int s = kt % kStages;
      mbar_wait(&full[s], (kt / kStages) & 1, a.err, kErrMma);
      tc_fence_after();
      const unsigned sa = smem_u32(smem + s * stage_bytes);
      const unsigned sb = sa + a_bytes;
      for (int kk = 0; kk < a.ck / 16; ++kk)
        mma_bf16(tmem, smem_desc(sa + kk * 32, 16, sbo, layout), smem_desc(sb + kk * 32, 16, sbo, layout), idesc,
                 (kt | kk) != 0);
      mma_commit(&empty[s]);
    }
    mma_commit(done);
  }
  __syncwarp();

  mbar_wait(done, 0, a.err, kErrEpilogue);
  tc_fence_after();
  const int m = warp * 32 + lane;
  const long long pix = (long long)tile * 128 + m;
  const size_t row = (size_t)pix * N;
  for (int j = 0; j < N / 32; ++j) {
    float v[32];
    tmem_ld32(tmem + ((unsigned)(warp * 32) << 16) + (unsigned)(j * 32), v);
    const int n0 = j * 32;
    if (a.bias) {
#pragma unroll
      for (int i = 0; i < 32; ++i) v[i] += __ldg(a.bias + n0 + i);
    }
    if (a.addend) {
      const uint4 *src = reinterpret_cast<const uint4 *>(a.addend + row + n0);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const uint4 u = src[q];
        const unsigned w4[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          v[q * 8 + 2 * e] += bf16_lo(w4[e]);
          v[q * 8 + 2 * e + 1] += bf16_hi(w4[e]);
        }
      }
    }
    if (a.relu) {
#pragma unroll
      for (int i = 0; i < 32; ++i) v[i] = fmaxf(v[i], 0.0f);
    }
    if (a.mask) {
      const uint4 *src = reinterpret_cast<const uint4 *>(a.mask + row + n0);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const uint4 u = src[q];
        const unsigned w4[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          if (!bf16_positive((unsigned short)(w4[e] & 0xFFFFu))) v[q * 8 + 2 * e] = 0.0f;
          if (!bf16_positive((unsigned short)(w4[e] >> 16))) v[q * 8 + 2 * e + 1] = 0.0f;
        }
      }
    }
    uint4 *dst = reinterpret_cast<uint4 *>(a.out + row + n0);
#pragma unroll
    for (int q = 0; q < 4; ++q)
      dst[q] = make_uint4(pack_bf16(v[q * 8 + 0], v[q * 8 + 1]), pack_bf16(v[q * 8 + 2], v[q * 8 + 3]),
                          pack_bf16(v[q * 8 + 4], v[q * 8 + 5]), pack_bf16(v[q * 8 + 6], v[q * 8 + 7]));
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) tmem_dealloc(tmem, tcols);
}

struct WgradArgs {
  float *dw;
  int c_in, c_out;
  int ma;             // channels per A segment (32 or 64)
  int na;             // channels per B atom (32 or 64)
  int segs_total;     // 9 * c_in / ma
  int segs_per_tile;  // 128 / ma
  int ptiles_per_image;
  int w;
  int kt_per_cta;
  int ptiles_total;
  unsigned *err;
};

__global__ void __launch_bounds__(kThreads) wgrad_kernel(const __grid_constant__ CUtensorMap tx,
                                                         const __grid_constant__ CUtensorMap tdy, WgradArgs a) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char *smem = align1024(smem_raw);
  const int N = a.c_out;
  const unsigned seg_bytes = (unsigned)kWgradK * a.ma * 2u;
  const unsigned a_bytes = 128u * kWgradK * 2u;
  const unsigned atom_b = (unsigned)kWgradK * a.na * 2u;
  const unsigned b_bytes = (unsigned)N * kWgradK * 2u;
  const unsigned stage_bytes = a_bytes + b_bytes;
  uint64_t *full = reinterpret_cast<uint64_t *>(smem + kStages * stage_bytes);
  uint64_t *empty = full + kStages;
  uint64_t *done = empty + kStages;
  unsigned *tmem_slot = reinterpret_cast<unsigned *>(done + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g0 = blockIdx.x * a.segs_per_tile;
  const int nseg = min(a.segs_per_tile, a.segs_total - g0);
  const int q0 = blockIdx.y * a.kt_per_cta;
  const int KT = min(a.kt_per_cta, a.ptiles_total - q0);
  const int cblocks = a.c_in / a.ma;
  const unsigned tcols = N < 32 ? 32u : (unsigned)N;
  const unsigned tx_bytes = (unsigned)nseg * seg_bytes + b_bytes;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    fence_mbar_init();
    tma_prefetch_desc(&tx);
    tma_prefetch_desc(&tdy);
  }
  if (warp == 1) tmem_alloc(tmem_slot, tcols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const unsigned tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    for (int kt = 0; kt < KT; ++kt) {
      const int s = kt % kStages;
      if (kt >= kStages) mbar_wait(&empty[s], ((kt / kStages) - 1) & 1, a.err, kErrProducer);
      unsigned char *sa = smem + s * stage_bytes;
      mbar_arrive_expect_tx(&full[s], tx_bytes);
      const int q = q0 + kt;
      const int img = q / a.ptiles_per_image;
      const int p0 = (q % a.ptiles_per_image) * kWgradK;
      const int y0 = p0 / a.w, x0 = p0 % a.w;
      for (int i = 0; i < nseg; ++i) {
        const int g = g0 + i, tap = g / cblocks, cb = g % cblocks;
        tma_load_4d(sa + i * seg_bytes, &tx, &full[s], cb * a.ma, x0 + tap % 3 - 1, y0 + tap / 3 - 1, img);
      }
      for (int nb = 0; nb < N / a.na; ++nb)
        tma_load_4d(sa + a_bytes + nb * atom_b, &tdy, &full[s], nb * a.na, x0, y0, img);
    }
  } else if (warp == 1 && lane == 0) {
    const uint32_t idesc = idesc_bf16_f32(128, N, 1, 1);
    const unsigned la = a.ma == 64 ? 2u : 4u, lb = a.na == 64 ? 2u : 4u;
    const unsigned sbo_a = 8u * a.ma * 2u, sbo_b = 8u * a.na * 2u;
    for (int kt = 0; kt < KT; ++kt) {
      const int s = kt % kStages;
      mbar_wait(&full[s], (kt / kStages) & 1, a.err, kErrMma);
      tc_fence_after();
      const unsigned sa = smem_u32(smem + s * stage_bytes);
      const unsigned sb = sa + a_bytes;
      for (int kk = 0; kk < kWgradK / 16; ++kk)
        mma_bf16(tmem, smem_desc(sa + kk * 2 * sbo_a, seg_bytes, sbo_a, la),
                 smem_desc(sb + kk * 2 * sbo_b, atom_b, sbo_b, lb), idesc, (kt | kk) != 0);
      mma_commit(&empty[s]);
    }
    mma_commit(done);
  }
  __syncwarp();

  mbar_wait(done, 0, a.err, kErrEpilogue);
  tc_fence_after();
  const int m = warp * 32 + lane;
  const int seg = m / a.ma;
  const bool live = seg < nseg && KT > 0;
  const int g = g0 + seg;
  const int tap = g / cblocks;
  const int ci = (g % cblocks) * a.ma + m % a.ma;
  for (int j = 0; j < N / 32; ++j) {
    float v[32];
    tmem_ld32(tmem + ((unsigned)(warp * 32) << 16) + (unsigned)(j * 32), v);
    if (live) {
      float *dst = a.dw + ((size_t)tap * N + j * 32) * a.c_in + ci;
#pragma unroll
      for (int e = 0; e < 32; ++e) atomicAdd(dst + (size_t)e * a.c_in, v[e]);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) tmem_dealloc(tmem, tcols);
}

// ---- host side ------------------------------------------------------------

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

static CUtensorMapSwizzle swizzle_for(int inner_channels) {
  return inner_channels == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B;
}

// NHWC bf16 activation map: dims (c, w, h, batch), box (bc, bw, bh, 1).
static bool act_map(CUtensorMap *m, const void *base, int c, i64 w, i64 h, i64 batch, int bc, int bw, int bh) {
  auto fn = encode_fn();
  if (!fn) return false;
  const cuuint64_t dims[4] = {(cuuint64_t)c, (cuuint64_t)w, (cuuint64_t)h, (cuuint64_t)batch};
  const cuuint64_t strides[3] = {(cuuint64_t)c * 2, (cuuint64_t)(w * c * 2), (cuuint64_t)(h * w * c * 2)};
  const cuuint32_t box[4] = {(cuuint32_t)bc, (cuuint32_t)bw, (cuuint32_t)bh, 1};
  const cuuint32_t es[4] = {1, 1, 1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void *>(base), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle_for(bc), CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Weight map over [9][c_out][c_in]: dims (c_in, c_out, 9), box (bc, c_out, 1).
static bool weight_map(CUtensorMap *m, const void *base, int c_in, int c_out, int bc) {
  auto fn = encode_fn();
  if (!fn) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)c_in, (cuuint64_t)c_out, 9};
  const cuuint64_t strides[2] = {(cuuint64_t)c_in * 2, (cuuint64_t)c_in * c_out * 2};
  const cuuint32_t box[3] = {(cuuint32_t)bc, (cuuint32_t)c_out, 1};
  const cuuint32_t es[3] = {1, 1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void *>(base), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle_for(bc), CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

static bool channels_ok(int c) { return c == 32 || c == 64 || c == 128 || c == 256; }
static bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

static size_t conv_smem(int ck, int n) { return (size_t)kStages * (128 + n) * ck * 2 + 1024 + 256; }
static size_t wgrad_smem(int n) { return (size_t)kStages * (128 + n) * kWgradK * 2 + 1024 + 256; }

}  // namespace net
}  // namespace adrtg

using namespace adrtg;
using namespace adrtg::net;

extern "C" int adrtnet_conv3x3(const void *x, int c_in, const void *w, int c_out, const float *bias,
                               const void *addend, const void *mask, int relu, void *out, int64_t batch,
                               int64_t h, int64_t wd, void *stream) {
  if (!x || !w || !out) return ADRT_GB300_ERR_NULL;
  if (!channels_ok(c_in) || !channels_ok(c_out)) return ADRT_GB300_ERR_SHAPE;
  if (batch < 1 || h < 1 || wd < 1 || (h * wd) % 128 != 0) return ADRT_GB300_ERR_SHAPE;
  if (!(wd % 128 == 0 || (wd < 128 && 128 % wd == 0))) return ADRT_GB300_ERR_SHAPE;
  if (batch * h * wd / 128 > 0x7FFFFFFFll || h > 0x7FFFFFFF || wd > 0x7FFFFFFF) return ADRT_GB300_ERR_TOO_LARGE;
  if (!aligned16(x) || !aligned16(w) || !aligned16(out) || (addend && !aligned16(addend)) ||
      (mask && !aligned16(mask)))
    return ADRT_GB300_ERR_SHAPE;
  unsigned *err = net_error_word();
  if (!err) return ADRT_GB300_ERR_CUDA;
  const int ck = c_in < 64 ? c_in : 64;
  const int bw = wd >= 128 ? 128 : (int)wd;
  const int bh = 128 / bw;
  CUtensorMap tx, tw;
  if (!act_map(&tx, x, c_in, wd, h, batch, ck, bw, bh) || !weight_map(&tw, w, c_in, c_out, ck))
    return ADRT_GB300_ERR_CUDA;
  ConvArgs a;
  a.out = static_cast<bf16 *>(out);
  a.bias = bias;
  a.addend = static_cast<const bf16 *>(addend);
  a.mask = static_cast<const bf16 *>(mask);
  a.c_out = c_out;
  a.ck = ck;
  a.kchunks = c_in / ck;
  a.relu = relu ? 1 : 0;
  a.w = (int)wd;
  a.tiles_per_image = (int)(h * wd / 128);
  a.rows_per_tile = bh;
  a.err = err;
  const size_t smem = conv_smem(ck, c_out);
  if (cudaFuncSetAttribute(conv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return ADRT_GB300_ERR_CUDA;
  const unsigned grid = (unsigned)(batch * h * wd / 128);
  conv_kernel<<<grid, kThreads, smem, static_cast<cudaStream_t>(stream)>>>(tx, tw, a);
  return launch_status();
}

extern "C" int adrtnet_conv3x3_wgrad(const void *x, int c_in, const void *dy, int c_out, float *dw,
                                     int64_t batch, int64_t h, int64_t wd, void *stream) {
  if (!x || !dy || !dw) return ADRT_GB300_ERR_NULL;
  if (!channels_ok(c_in) || !channels_ok(c_out)) return ADRT_GB300_ERR_SHAPE;
  if (batch < 1 || h < 1 || wd < 1 || (h * wd) % kWgradK != 0) return ADRT_GB300_ERR_SHAPE;
  if (!(wd % kWgradK == 0 || (wd < kWgradK && kWgradK % wd == 0))) return ADRT_GB300_ERR_SHAPE;
  if (batch * h * wd / kWgradK > 0x7FFFFFFFll) return ADRT_GB300_ERR_TOO_LARGE;
  if (!aligned16(x) || !aligned16(dy) || !aligned16(dw)) return ADRT_GB300_ERR_SHAPE;
  unsigned *err = net_error_word();
  if (!err) return ADRT_GB300_ERR_CUDA;
  const int ma = c_in < 64 ? c_in : 64;
  const int na = c_out < 64 ? c_out : 64;
  const int bw = wd >= kWgradK ? kWgradK : (int)wd;
  const int bh = kWgradK / bw;
  CUtensorMap tx, tdy;
  if (!act_map(&tx, x, c_in, wd, h, batch, ma, bw, bh) || !act_map(&tdy, dy, c_out, wd, h, batch, na, bw, bh))
    return ADRT_GB300_ERR_CUDA;
  WgradArgs a;
  a.dw = dw;
  a.c_in = c_in;
  a.c_out = c_out;
  a.ma = ma;
  a.na = na;
  a.segs_total = 9 * c_in / ma;
  a.segs_per_tile = 128 / ma;
  a.ptiles_per_image = (int)(h * wd / kWgradK);
  a.w = (int)wd;
  a.ptiles_total = (int)(batch * h * wd / kWgradK);
  const int mtiles = (a.segs_total + a.segs_per_tile - 1) / a.segs_per_tile;
  // Enough CTAs to fill the GPU a few times over, each with at least 8 stages.
  int per = (int)((a.ptiles_total * (long long)mtiles + 4 * 152 - 1) / (4 * 152));
  if (per < 8) per = 8;
  a.kt_per_cta = per;
  a.err = err;
  const size_t smem = wgrad_smem(c_out);
  if (cudaFuncSetAttribute(wgrad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return ADRT_GB300_ERR_CUDA;
  const dim3 grid((unsigned)mtiles, (unsigned)((a.ptiles_total + per - 1) / per));
  wgrad_kernel<<<grid, kThreads, smem, static_cast<cudaStream_t>(stream)>>>(tx, tdy, a);
  return launch_status();
}

extern "C" int adrtnet_status(void *stream) {
  unsigned *w = net_error_word();
  if (!w) return ADRT_GB300_ERR_CUDA;
  unsigned word = 0;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (cudaMemcpyAsync(&word, w, sizeof(word), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return ADRT_GB300_ERR_CUDA;
  if (word) {
    const unsigned zero = 0;
    if (cudaMemcpyAsync(w, &zero, sizeof(zero), cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return ADRT_GB300_ERR_CUDA;
    return ADRT_GB300_ERR_TIMEOUT;
  }
  return ADRT_GB300_OK;
}
