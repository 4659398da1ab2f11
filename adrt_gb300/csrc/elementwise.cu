// Small kernels that replace the NumPy glue of the full-multigrid inverse
// (src/adrt/core.py:318-330, src/adrt/core.py:378, src/adrt/__init__.py:135).
#include "common.cuh"

namespace adrtg {

// Pixel (i, j) of quadrant q under truncate (src/adrt/utils.py:234-242).
__device__ __forceinline__ i64 trunc_idx(int q, i64 i, i64 j, i64 n) {
  switch (q) {
    case 0: return (n - 1 - j) * n + i;
    case 1: return (n - 1 - i) * n + j;
    case 2: return i * n + j;
    default: return (n - 1 - j) * n + (n - 1 - i);
  }
}

// out = np.mean(truncate(y) / (n - 1), axis=-3): each quadrant value is divided
// by (n-1) (one rounding), the four are summed in quadrant order, then divided
// by 4, exactly as NumPy evaluates the expression at src/adrt/core.py:328-329.
// Index arithmetic in I (32-bit unsigned when the sizes allow); n is a power
// of two here (lg = log2 n), so the decomposition is shifts and masks.
template <typename T, typename I>
__global__ void fmg_correction_kernel(const T *__restrict__ y, T *__restrict__ out, I total, I n, int lg,
                                      T divisor) {
  const I C = 2 * n - 1;
  for (I idx = blockIdx.x * (I)blockDim.x + threadIdx.x; idx < total; idx += (I)gridDim.x * blockDim.x) {
    const I j = idx & (n - 1), i = (idx >> lg) & (n - 1);
    const T *yb = y + (idx >> (2 * lg)) * 4 * C * n;
    T s = add_rn(div_rn(yb[trunc_idx(0, i, j, n)], divisor),
                 div_rn(yb[C * n + trunc_idx(1, i, j, n)], divisor));
    s = add_rn(s, div_rn(yb[2 * C * n + trunc_idx(2, i, j, n)], divisor));
    s = add_rn(s, div_rn(yb[3 * C * n + trunc_idx(3, i, j, n)], divisor));
    out[idx] = div_rn(s, T(4));
  }
}

// op 0: out = a - b;  op 1: out = a + b.
template <typename T>
__global__ void binary_kernel(const T *__restrict__ a, const T *__restrict__ b, T *out, i64 count,
                              int op) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < count;
       i += (i64)gridDim.x * blockDim.x)
    out[i] = op == 0 ? sub_rn(a[i], b[i]) : add_rn(a[i], b[i]);
}

// Deterministic sum of squares in float64: fixed grid, fixed per-thread
// stride order, fixed tree in shared memory, then one block sums the partials.
constexpr int kSqThreads = 256;
constexpr int kSqBlocks = 512;

// blockIdx.y selects an image of `count` elements (a batch of sums computed
// with exactly the single-array partition, image by image).
template <typename T>
__global__ void sumsq_partial_kernel(const T *__restrict__ a, i64 count, double *partial) {
  __shared__ double sh[kSqThreads];
  a += (i64)blockIdx.y * count;
  partial += (size_t)blockIdx.y * kSqBlocks;
  double acc = 0.0;
  for (i64 i = blockIdx.x * (i64)kSqThreads + threadIdx.x; i < count; i += (i64)kSqBlocks * kSqThreads) {
    const double v = (double)a[i];
    acc = __dadd_rn(acc, __dmul_rn(v, v));
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kSqThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = __dadd_rn(sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

__global__ void sumsq_final_kernel(const double *partial, double *out) {
  __shared__ double sh[kSqBlocks];
  partial += (size_t)blockIdx.x * kSqBlocks;
  out += blockIdx.x;
  for (int i = threadIdx.x; i < kSqBlocks; i += blockDim.x) sh[i] = partial[i];
  __syncthreads();
  for (int s = kSqBlocks / 2; s > 0; s >>= 1) {
    for (int i = threadIdx.x; i < s; i += blockDim.x) sh[i] = __dadd_rn(sh[i], sh[i + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

static unsigned grid_e(i64 total) {
  i64 g = (total + 255) / 256;
  if (g > 152 * 32) g = 152 * 32;
  return (unsigned)(g < 1 ? 1 : g);
}

template <typename T>
int fmg_correction_launch(const T *y, T *out, i64 batch, i64 n, cudaStream_t st) {
  const i64 total = batch * n * n;
  const int lg = num_iters(n);
  if (total * 8 < (i64(1) << 32))
    fmg_correction_kernel<T, unsigned><<<grid_e(total), 256, 0, st>>>(y, out, (unsigned)total, (unsigned)n, lg,
                                                                      T(n - 1));
  else
    fmg_correction_kernel<T, unsigned long long><<<grid_e(total), 256, 0, st>>>(
        y, out, (unsigned long long)total, (unsigned long long)n, lg, T(n - 1));
  return launch_status();
}

template <typename T>
int binary_launch(const T *a, const T *b, T *out, i64 count, int op, cudaStream_t st) {
  binary_kernel<T><<<grid_e(count), 256, 0, st>>>(a, b, out, count, op);
  return launch_status();
}

size_t sumsq_workspace_bytes() { return sizeof(double) * kSqBlocks; }

template <typename T>
int sumsq_launch(const T *a, i64 count, double *out, void *ws, cudaStream_t st, i64 batch) {
  double *partial = static_cast<double *>(ws);
  sumsq_partial_kernel<T><<<dim3(kSqBlocks, (unsigned)batch), kSqThreads, 0, st>>>(a, count, partial);
  sumsq_final_kernel<<<(unsigned)batch, 256, 0, st>>>(partial, out);
  return launch_status();
}

#define INST(T)                                                                   \
  template int fmg_correction_launch<T>(const T *, T *, i64, i64, cudaStream_t);  \
  template int binary_launch<T>(const T *, const T *, T *, i64, int, cudaStream_t); \
  template int sumsq_launch<T>(const T *, i64, double *, void *, cudaStream_t, i64);
INST(float)
INST(double)
#undef INST

}  // namespace adrtg
