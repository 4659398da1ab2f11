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

template <typename T, int H>
__global__ void __launch_bounds__(kPcThreads) precond_conv_kernel(const T *__restrict__ x, T *__restrict__ y,
                                                                 int n, const __grid_constant__ PcWeights<T, H> K) {
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
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int gy = ty0 + r0 + k;
    if (gy < n && gx < n) yo[(unsigned)gy * (unsigned)n + (unsigned)gx] = acc[k];
  }
}

template <typename T, int H>
static int precond_launch_h(const T *x, T *y, i64 batch, i64 n, const double *w, cudaStream_t st) {
  PcWeights<T, H> K;
  for (int i = 0; i < (2 * H + 1) * (2 * H + 1); ++i) K.w[i] = (T)w[i];
  const unsigned tiles = (unsigned)((n + kPcTile - 1) / kPcTile);
  const dim3 grid(tiles, tiles, (unsigned)batch);
  precond_conv_kernel<T, H><<<grid, kPcThreads, 0, st>>>(x, y, (int)n, K);
  return launch_status();
}

template <typename T>
static int precond_launch(const T *x, T *y, i64 batch, i64 n, const double *w, int h, cudaStream_t st) {
  switch (h) {
    case 0: return precond_launch_h<T, 0>(x, y, batch, n, w, st);
    case 1: return precond_launch_h<T, 1>(x, y, batch, n, w, st);
    case 2: return precond_launch_h<T, 2>(x, y, batch, n, w, st);
    case 3: return precond_launch_h<T, 3>(x, y, batch, n, w, st);
    case 4: return precond_launch_h<T, 4>(x, y, batch, n, w, st);
    case 5: return precond_launch_h<T, 5>(x, y, batch, n, w, st);
    case 6: return precond_launch_h<T, 6>(x, y, batch, n, w, st);
    case 7: return precond_launch_h<T, 7>(x, y, batch, n, w, st);
  }
  return ADRT_GB300_ERR_SHAPE;
}

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
                                        st);
  return adrtg::precond_launch<double>(static_cast<const double *>(x), static_cast<double *>(y), batch, n, weights,
                                       h, st);
}
