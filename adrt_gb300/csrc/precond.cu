// Convolution preconditioner for CG on the ADRT normal equations.
//
// y[b][i][j] = sum_{di, dj in [-h, h]} K[di][dj] x[b][i+di][j+dj], with x = 0
// outside the n x n image ("same" size, zero padding).  For a point-symmetric
// K (K[d] = K[-d]) this is a symmetric operator, and it is positive definite
// when K's symbol sum_d K[d] e^{i w.d} is positive at every frequency w; then
// it is a valid preconditioner for conjugate gradients.  The weights are
// learned (adrt_gb300.precond) as a least-squares approximate inverse of
// A^T A.  They travel in the launch parameters, so the multiply-adds read
// them as uniform constant operands and a captured CUDA graph keeps them.
//
// Each CTA computes a 32 x 32 output tile of one image from a shared-memory
// input tile with an h-wide halo; a thread computes four rows of one column.
// Accumulation order is fixed (dy, then dx), so results are deterministic.
#include "common.cuh"

namespace adrtg {

constexpr int kPcTile = 32;
constexpr int kPcThreads = 256;          // 32 columns x 8 row groups of 4
constexpr int kPcMaxH = 7;

template <typename T, int H>
struct PcWeights {
  T w[(2 * H + 1) * (2 * H + 1)];
};

// With `partial` non-null the kernel also writes the tile's share of the dot
// product <x, y> (PCG's <r, M r>): per-thread sums of its four products in
// the data type, then a fixed float64 warp-shuffle tree and the warps in
// order; precond_dot_final_kernel adds an image's tiles in order.
template <typename T, int H>
__global__ void __launch_bounds__(kPcThreads) precond_conv_kernel(const T *__restrict__ x, T *__restrict__ y,
                                                                 int n, const __grid_constant__ PcWeights<T, H> K,
                                                                 double *__restrict__ partial) {
  constexpr int KS = 2 * H + 1, TIN = kPcTile + 2 * H;
  __shared__ T sx[TIN][TIN + 1];
  const int tx0 = blockIdx.x * kPcTile, ty0 = blockIdx.y * kPcTile;
  const size_t off = (size_t)blockIdx.z * (unsigned)n * (unsigned)n;
  const T *xi = x + off;
  for (int idx = threadIdx.x; idx < TIN * TIN; idx += kPcThreads) {
    const int r = idx / TIN, c = idx % TIN;
    const int gy = ty0 - H + r, gx = tx0 - H + c;
    T v = T(0);
    if (gy >= 0 && gy < n && gx >= 0 && gx < n) v = xi[(unsigned)gy * (unsigned)n + (unsigned)gx];
    sx[r][c] = v;
  }
  __syncthreads();
  const int col = threadIdx.x & 31, r0 = (threadIdx.x >> 5) * 4;
  T acc[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
  for (int dx = 0; dx < KS; ++dx) {
    T v[4 + 2 * H];
#pragma unroll
    for (int k = 0; k < 4 + 2 * H; ++k) v[k] = sx[r0 + k][col + dx];
#pragma unroll
    for (int dy = 0; dy < KS; ++dy) {
      const T w = K.w[dy * KS + dx];
#pragma unroll
      for (int k = 0; k < 4; ++k) acc[k] = fma_rn(w, v[k + dy], acc[k]);
    }
  }
  T *yo = y + off;
  const int gx = tx0 + col;
  T d = T(0);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int gy = ty0 + r0 + k;
    if (gy < n && gx < n) {
      yo[(unsigned)gy * (unsigned)n + (unsigned)gx] = acc[k];
      d = add_rn(d, mul_rn(sx[r0 + k + H][col + H], acc[k]));
    }
  }
  if (partial != nullptr) {
    __shared__ double wsum[kPcThreads / 32];
    double v = (double)d;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_down_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int w = 0; w < kPcThreads / 32; ++w) t = __dadd_rn(t, wsum[w]);
      partial[(size_t)blockIdx.z * gridDim.x * gridDim.y + blockIdx.y * gridDim.x + blockIdx.x] = t;
    }
  }
}

__global__ void precond_dot_final_kernel(const double *__restrict__ partial, double *__restrict__ out, int batch,
                                         int tiles) {
  const int img = blockIdx.x * blockDim.x + threadIdx.x;
  if (img >= batch) return;
  double t = 0.0;
  for (int k = 0; k < tiles; ++k) t = __dadd_rn(t, partial[(size_t)img * tiles + k]);
  out[img] = t;
}

template <typename T, int H>
static int precond_launch_h(const T *x, T *y, i64 batch, i64 n, const double *w, double *partial,
                            cudaStream_t st) {
  PcWeights<T, H> K;
  for (int i = 0; i < (2 * H + 1) * (2 * H + 1); ++i) K.w[i] = (T)w[i];
  const unsigned tiles = (unsigned)((n + kPcTile - 1) / kPcTile);
  const dim3 grid(tiles, tiles, (unsigned)batch);
  precond_conv_kernel<T, H><<<grid, kPcThreads, 0, st>>>(x, y, (int)n, K, partial);
  return launch_status();
}

template <typename T>
static int precond_launch(const T *x, T *y, i64 batch, i64 n, const double *w, int h, double *partial,
                          cudaStream_t st) {
  switch (h) {
    case 0: return precond_launch_h<T, 0>(x, y, batch, n, w, partial, st);
    case 1: return precond_launch_h<T, 1>(x, y, batch, n, w, partial, st);
    case 2: return precond_launch_h<T, 2>(x, y, batch, n, w, partial, st);
    case 3: return precond_launch_h<T, 3>(x, y, batch, n, w, partial, st);
    case 4: return precond_launch_h<T, 4>(x, y, batch, n, w, partial, st);
    case 5: return precond_launch_h<T, 5>(x, y, batch, n, w, partial, st);
    case 6: return precond_launch_h<T, 6>(x, y, batch, n, w, partial, st);
    case 7: return precond_launch_h<T, 7>(x, y, batch, n, w, partial, st);
  }
  return ADRT_GB300_ERR_SHAPE;
}

static i64 pc_tiles(i64 n) { const i64 t = (n + kPcTile - 1) / kPcTile; return t * t; }

}  // namespace adrtg

extern "C" int adrt_gb300_precond_conv(const void *x, void *y, int64_t batch, int64_t n, const double *weights,
                                       int h, int dtype, void *stream) {
  if (!x || !y || !weights) return ADRT_GB300_ERR_NULL;
  if (dtype != ADRT_GB300_F32 && dtype != ADRT_GB300_F64) return ADRT_GB300_ERR_DTYPE;
  if (batch < 1 || n < 1 || h < 0 || h > adrtg::kPcMaxH) return ADRT_GB300_ERR_SHAPE;
  if (n > 32768 || batch > 65535) return ADRT_GB300_ERR_TOO_LARGE;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == ADRT_GB300_F32)
    return adrtg::precond_launch<float>(static_cast<const float *>(x), static_cast<float *>(y), batch, n, weights, h,
                                        nullptr, st);
  return adrtg::precond_launch<double>(static_cast<const double *>(x), static_cast<double *>(y), batch, n, weights,
                                       h, nullptr, st);
}

extern "C" size_t adrt_gb300_precond_dot_workspace_size(int64_t batch, int64_t n) {
  if (batch < 1 || n < 1) return 0;
  return sizeof(double) * (size_t)batch * (size_t)adrtg::pc_tiles(n);
}

extern "C" int adrt_gb300_precond_conv_dot(const void *x, void *y, int64_t batch, int64_t n, const double *weights,
                                           int h, int dtype, double *dot, void *workspace, size_t workspace_bytes,
                                           void *stream) {
  if (!x || !y || !weights || !dot || !workspace) return ADRT_GB300_ERR_NULL;
  if (dtype != ADRT_GB300_F32 && dtype != ADRT_GB300_F64) return ADRT_GB300_ERR_DTYPE;
  if (batch < 1 || n < 1 || h < 0 || h > adrtg::kPcMaxH) return ADRT_GB300_ERR_SHAPE;
  if (n > 32768 || batch > 65535) return ADRT_GB300_ERR_TOO_LARGE;
  if (workspace_bytes < adrt_gb300_precond_dot_workspace_size(batch, n)) return ADRT_GB300_ERR_WORKSPACE;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double *partial = static_cast<double *>(workspace);
  int rc;
  if (dtype == ADRT_GB300_F32)
    rc = adrtg::precond_launch<float>(static_cast<const float *>(x), static_cast<float *>(y), batch, n, weights, h,
                                      partial, st);
  else
    rc = adrtg::precond_launch<double>(static_cast<const double *>(x), static_cast<double *>(y), batch, n, weights,
                                       h, partial, st);
  if (rc) return rc;
  adrtg::precond_dot_final_kernel<<<(unsigned)((batch + 127) / 128), 128, 0, st>>>(
      partial, dot, (int)batch, (int)adrtg::pc_tiles(n));
  return adrtg::launch_status();
}
