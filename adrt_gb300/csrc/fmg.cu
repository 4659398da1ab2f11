// Multigrid operators used by the full-multigrid inverse (Press 2006).
#include "common.cuh"

namespace adrtg {

// out[p][r][c] = (x[p][2r][2c] + x[p][2r+1][2c]) / 4,  (4, 2n-1, n) -> (4, n-1, n/2).
// Reference: src/adrt/adrt_cdefs_fmg.hpp:53-73.
// Index arithmetic of these kernels runs in I: 32-bit unsigned when every
// index fits (64-bit division is a long instruction sequence), else 64-bit.
template <typename T, typename I>
__global__ void fmg_restriction_kernel(const T *__restrict__ in, T *__restrict__ out,
                                       I planes, I n) {
  const I Ri = 2 * n - 1, Ro = n - 1, Co = n / 2;
  const I total = planes * Ro * Co;
  for (I idx = blockIdx.x * (I)blockDim.x + threadIdx.x; idx < total;
       idx += (I)gridDim.x * blockDim.x) {
    const I c = idx % Co;
    const I pr = idx / Co;
    const I r = pr % Ro;
    const I p = pr / Ro;
    const T va = in[(p * Ri + 2 * r) * n + 2 * c];
    const T vb = in[(p * Ri + 2 * r + 1) * n + 2 * c];
    out[idx] = div_rn(add_rn(va, vb), T(4));
  }
}

// 2x2 nearest-neighbour repeat, (h, w) -> (2h, 2w).
// Reference: src/adrt/adrt_cdefs_fmg.hpp:75-95.
template <typename T, typename I>
__global__ void fmg_prolongation_kernel(const T *__restrict__ in, T *__restrict__ out,
                                        I batch, I h, I w) {
  const I total = batch * 4 * h * w;
  for (I idx = blockIdx.x * (I)blockDim.x + threadIdx.x; idx < total;
       idx += (I)gridDim.x * blockDim.x) {
    const I c = idx % (2 * w);
    const I br = idx / (2 * w);
    const I r = br % (2 * h);
    const I b = br / (2 * h);
    out[idx] = in[(b * h + r / 2) * w + c / 2];
  }
}

// 3x3 high-pass with kernel [[a,b,a],[b,c,b],[a,b,a]], a=-1/16, b=-1/8, c=3/4,
// reflected borders; taps multiplied then summed column by column:
// (v11+v21+v31) + (v12+v22+v32) + (v13+v23+v33).
// Reference: src/adrt/adrt_cdefs_fmg.hpp:97-171.
template <typename T, typename I>
__global__ void fmg_highpass_kernel(const T *__restrict__ in, T *__restrict__ out,
                                    I batch, I h, I w) {
  const T ka = T(-0.0625), kb = T(-0.125), kc = T(0.75);
  const I total = batch * h * w;
  for (I idx = blockIdx.x * (I)blockDim.x + threadIdx.x; idx < total;
       idx += (I)gridDim.x * blockDim.x) {
    const I c = idx % w;
    const I br = idx / w;
    const I r = br % h;
    const T *x = in + (br / h) * h * w;
    const I rp = r == 0 ? 1 : r - 1, rn = r == h - 1 ? r - 1 : r + 1;
    const I cp = c == 0 ? 1 : c - 1, cn = c == w - 1 ? c - 1 : c + 1;
    const T v11 = mul_rn(ka, x[rp * w + cp]), v12 = mul_rn(kb, x[rp * w + c]),
            v13 = mul_rn(ka, x[rp * w + cn]);
    const T v21 = mul_rn(kb, x[r * w + cp]), v22 = mul_rn(kc, x[r * w + c]),
            v23 = mul_rn(kb, x[r * w + cn]);
    const T v31 = mul_rn(ka, x[rn * w + cp]), v32 = mul_rn(kb, x[rn * w + c]),
            v33 = mul_rn(ka, x[rn * w + cn]);
    const T s1 = add_rn(add_rn(v11, v21), v31);
    const T s2 = add_rn(add_rn(v12, v22), v32);
    const T s3 = add_rn(add_rn(v13, v23), v33);
    out[idx] = add_rn(add_rn(s1, s2), s3);
  }
}

static unsigned grid_1d(i64 total) {
  i64 g = (total + 255) / 256;
  if (g > 152 * 32) g = 152 * 32;
  return (unsigned)(g < 1 ? 1 : g);
}

// 32-bit indices when every index of the input and output, plus one grid
// stride, stays below 2^32.
static bool fits_u32(i64 max_index) { return max_index < (i64(1) << 32) - (i64(1) << 24); }

template <typename T>
int fmg_restriction_launch(const T *in, T *out, i64 batch, i64 n, cudaStream_t st) {
  const i64 total = batch * 4 * (n - 1) * (n / 2);
  if (fits_u32(batch * 4 * (2 * n - 1) * n))
    fmg_restriction_kernel<T, unsigned><<<grid_1d(total), 256, 0, st>>>(in, out, (unsigned)(batch * 4), (unsigned)n);
  else
    fmg_restriction_kernel<T, unsigned long long><<<grid_1d(total), 256, 0, st>>>(
        in, out, (unsigned long long)(batch * 4), (unsigned long long)n);
  return launch_status();
}

template <typename T>
int fmg_prolongation_launch(const T *in, T *out, i64 batch, i64 h, i64 w, cudaStream_t st) {
  const i64 total = batch * 4 * h * w;
  if (fits_u32(total))
    fmg_prolongation_kernel<T, unsigned><<<grid_1d(total), 256, 0, st>>>(in, out, (unsigned)batch, (unsigned)h,
                                                                         (unsigned)w);
  else
    fmg_prolongation_kernel<T, unsigned long long><<<grid_1d(total), 256, 0, st>>>(
        in, out, (unsigned long long)batch, (unsigned long long)h, (unsigned long long)w);
  return launch_status();
}

template <typename T>
int fmg_highpass_launch(const T *in, T *out, i64 batch, i64 h, i64 w, cudaStream_t st) {
  const i64 total = batch * h * w;
  if (fits_u32(total))
    fmg_highpass_kernel<T, unsigned><<<grid_1d(total), 256, 0, st>>>(in, out, (unsigned)batch, (unsigned)h,
                                                                     (unsigned)w);
  else
    fmg_highpass_kernel<T, unsigned long long><<<grid_1d(total), 256, 0, st>>>(
        in, out, (unsigned long long)batch, (unsigned long long)h, (unsigned long long)w);
  return launch_status();
}

#define INST(T)                                                                        \
  template int fmg_restriction_launch<T>(const T *, T *, i64, i64, cudaStream_t);      \
  template int fmg_prolongation_launch<T>(const T *, T *, i64, i64, i64, cudaStream_t); \
  template int fmg_highpass_launch<T>(const T *, T *, i64, i64, i64, cudaStream_t);
INST(float)
INST(double)
#undef INST

}  // namespace adrtg
