// Batched conjugate-gradient vector kernels for the ADRT normal equations.
//
// Every image of a batch runs its own CG recurrence; scalars (dot products,
// alpha, beta) are per image.  A dot product is reduced in a fixed order:
// each thread sums its strided slice in the data type (products and sums
// rounded separately, no FMA), the per-thread sums are combined in float64
// by a fixed warp-shuffle tree, then across the block's warps and the
// image's blocks in index order -- so results do not depend on scheduling.
// (float64 arithmetic is slow on this GPU: the per-element work stays in the
// data type; float64 data therefore accumulates in float64 throughout.)
// An image whose `active` flag is 0 is frozen: its alpha is 0 and its
// direction is left unchanged.
#include "common.cuh"

namespace adrtg {

constexpr int kDotThreads = 256;
constexpr int kDotBlocksPerImage = 32;

// Sum over the block in a fixed order: shuffle tree within each warp, then
// the warps' sums in warp order.
__device__ __forceinline__ double block_sum(double v, double *sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_down_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < kDotThreads / 32; ++w) s = __dadd_rn(s, sh[w]);
  return s;
}

// partial[img][blk] = sum over the block's strided slice of a*b.
template <typename T>
__global__ void __launch_bounds__(kDotThreads) dot_partial_kernel(const T *__restrict__ a, const T *__restrict__ b,
                                                                 i64 per, double *partial) {
  __shared__ double sh[kDotThreads / 32];
  const int img = blockIdx.y, blk = blockIdx.x;
  const T *pa = a + (i64)img * per, *pb = b + (i64)img * per;
  T acc = T(0);
  for (i64 i = (i64)blk * kDotThreads + threadIdx.x; i < per; i += (i64)kDotBlocksPerImage * kDotThreads)
    acc = add_rn(acc, mul_rn(pa[i], pb[i]));
  const double s = block_sum((double)acc, sh);
  if (threadIdx.x == 0) partial[img * kDotBlocksPerImage + blk] = s;
}

__global__ void dot_final_kernel(const double *partial, double *out, int batch) {
  const int img = blockIdx.x * blockDim.x + threadIdx.x;
  if (img >= batch) return;
  double s = 0.0;
  for (int k = 0; k < kDotBlocksPerImage; ++k) s = __dadd_rn(s, partial[img * kDotBlocksPerImage + k]);
  out[img] = s;
}

// alpha = rs / pAp (0 if frozen or pAp == 0); x += alpha p; r -= alpha Ap;
// partial sums of r*r for rs_new.
template <typename T>
__global__ void __launch_bounds__(kDotThreads) cg_update_kernel(T *__restrict__ x, T *__restrict__ r,
                                                               const T *__restrict__ p, const T *__restrict__ Ap,
                                                               const double *rs, const double *pAp,
                                                               const int *active, i64 per, double *partial) {
  __shared__ double sh[kDotThreads / 32];
  const int img = blockIdx.y, blk = blockIdx.x;
  const double den = pAp[img];
  const bool on = active[img] != 0 && den != 0.0;
  const T alpha = on ? (T)(rs[img] / den) : T(0);
  T *px = x + (i64)img * per, *pr = r + (i64)img * per;
  const T *pp = p + (i64)img * per, *pAp_ = Ap + (i64)img * per;
  T acc = T(0);
  for (i64 i = (i64)blk * kDotThreads + threadIdx.x; i < per; i += (i64)kDotBlocksPerImage * kDotThreads) {
    T rv = pr[i];
    if (on) {
      px[i] = add_rn(px[i], mul_rn(alpha, pp[i]));
      rv = sub_rn(rv, mul_rn(alpha, pAp_[i]));
      pr[i] = rv;
    }
    acc = add_rn(acc, mul_rn(rv, rv));
  }
  const double s = block_sum((double)acc, sh);
  if (threadIdx.x == 0) partial[img * kDotBlocksPerImage + blk] = s;
}

// beta = rs_new / rs; p = r + beta p; rs = rs_new (active images only).
template <typename T>
__global__ void cg_direction_kernel(T *__restrict__ p, const T *__restrict__ r, const double *rs_new,
                                    double *rs, const int *active, i64 per) {
  const int img = blockIdx.y;
  if (!active[img]) return;
  const double old = rs[img];
  const T beta = old != 0.0 ? (T)(rs_new[img] / old) : T(0);
  T *pp = p + (i64)img * per;
  const T *pr = r + (i64)img * per;
  for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < per; i += (i64)gridDim.x * blockDim.x)
    pp[i] = add_rn(pr[i], mul_rn(beta, pp[i]));
}

__global__ void cg_commit_kernel(double *rs, const double *rs_new, const int *active, int batch) {
  const int img = blockIdx.x * blockDim.x + threadIdx.x;
  if (img < batch && active[img]) rs[img] = rs_new[img];
}

size_t cg_workspace_bytes(i64 batch) { return sizeof(double) * (size_t)batch * kDotBlocksPerImage; }

template <typename T>
int batched_dot_launch(const T *a, const T *b, double *out, i64 batch, i64 per, void *ws,
                       cudaStream_t st) {
  double *partial = static_cast<double *>(ws);
  dot_partial_kernel<T><<<dim3(kDotBlocksPerImage, (unsigned)batch), kDotThreads, 0, st>>>(a, b, per, partial);
  int rc = launch_status();
  if (rc) return rc;
  dot_final_kernel<<<(unsigned)((batch + 127) / 128), 128, 0, st>>>(partial, out, (int)batch);
  return launch_status();
}

template <typename T>
int cg_update_launch(T *x, T *r, const T *p, const T *Ap, const double *rs, const double *pAp,
                     const int *active, double *rs_new, i64 batch, i64 per, void *ws, cudaStream_t st) {
  double *partial = static_cast<double *>(ws);
  cg_update_kernel<T><<<dim3(kDotBlocksPerImage, (unsigned)batch), kDotThreads, 0, st>>>(
      x, r, p, Ap, rs, pAp, active, per, partial);
  int rc = launch_status();
  if (rc) return rc;
  dot_final_kernel<<<(unsigned)((batch + 127) / 128), 128, 0, st>>>(partial, rs_new, (int)batch);
  return launch_status();
}

template <typename T>
int cg_direction_launch(T *p, const T *r, const double *rs_new, double *rs, const int *active,
                        i64 batch, i64 per, cudaStream_t st) {
  cg_direction_kernel<T><<<dim3(32, (unsigned)batch), 256, 0, st>>>(p, r, rs_new, rs, active, per);
  int rc = launch_status();
  if (rc) return rc;
  cg_commit_kernel<<<(unsigned)((batch + 127) / 128), 128, 0, st>>>(rs, rs_new, active, (int)batch);
  return launch_status();
}

// y += alpha * x (one rounding for the product, one for the sum; no FMA).
template <typename T>
__global__ void axpy_kernel(T alpha, const T *__restrict__ x, T *__restrict__ y, i64 count) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < count; i += (i64)gridDim.x * blockDim.x)
    y[i] = add_rn(y[i], mul_rn(alpha, x[i]));
}

template <typename T>
int axpy_launch(double alpha, const T *x, T *y, i64 count, cudaStream_t st) {
  const i64 blocks = (count + 255) / 256;
  axpy_kernel<T><<<(unsigned)(blocks < 8192 ? blocks : 8192), 256, 0, st>>>((T)alpha, x, y, count);
  return launch_status();
}

#define INST(T)                                                                                \
  template int batched_dot_launch<T>(const T *, const T *, double *, i64, i64, void *, cudaStream_t); \
  template int cg_update_launch<T>(T *, T *, const T *, const T *, const double *, const double *, \
                                   const int *, double *, i64, i64, void *, cudaStream_t);     \
  template int cg_direction_launch<T>(T *, const T *, const double *, double *, const int *, i64, \
                                      i64, cudaStream_t);                                      \
  template int axpy_launch<T>(double, const T *, T *, i64, cudaStream_t);
INST(float)
INST(double)
#undef INST

}  // namespace adrtg
