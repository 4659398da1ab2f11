// Multigrid operators used by the full-multigrid inverse (Press 2006).
#include "common.cuh"

namespace adrtg {

// out[p][r][c] = (x[p][2r][2c] + x[p][2r+1][2c]) / 4,  (4, 2n-1, n) -> (4, n-1, n/2).
// Reference: src/adrt/adrt_cdefs_fmg.hpp:53-73.
template <typename T>
__global__ void fmg_restriction_kernel(const T *__restrict__ in, T *__restrict__ out,
                                       i64 planes, i64 n) {
  const i64 Ri = 2 * n - 1, Ro = n - 1, Co = n / 2;
  const i64 total = planes * Ro * Co;
  for (i64 idx = blockIdx.x * (i64)blockDim.x + threadIdx.x; idx < total;
       idx += (i64)gridDim.x * blockDim.x) {
    const i64 c = idx % Co;
    const i64 r = (idx / Co) % Ro;
    const i64 p = idx / (Co * Ro);
    const T va = in[(p * Ri + 2 * r) * n + 2 * c];
    const T vb = in[(p * Ri + 2 * r + 1) * n + 2 * c];
    out[idx] = div_rn(add_rn(va, vb), T(4));
  }
}

// 2x2 nearest-neighbour repeat, (h, w) -> (2h, 2w).
// Reference: src/adrt/adrt_cdefs_fmg.hpp:75-95.
template <typename T>
__global__ void fmg_prolongation_kernel(const T *__restrict__ in, T *__restrict__ out,
                                        i64 batch, i64 h, i64 w) {
  const i64 total = batch * 4 * h * w;
  for (i64 idx = blockIdx.x * (i64)blockDim.x + threadIdx.x; idx < total;
       idx += (i64)gridDim.x * blockDim.x) {
    const i64 c = idx % (2 * w);
    const i64 r = (idx / (2 * w)) % (2 * h);
    const i64 b = idx / (4 * h * w);
    out[idx] = in[(b * h + r / 2) * w + c / 2];
  }
}

// 3x3 high-pass with kernel [[a,b,a],[b,c,b],[a,b,a]], a=-1/16, b=-1/8, c=3/4,
// reflected borders; taps multiplied then summed column by column:
// (v11+v21+v31) + (v12+v22+v32) + (v13+v23+v33).
// Reference: src/adrt/adrt_cdefs_fmg.hpp:97-171.
template <typename T>
__global__ void fmg_highpass_kernel(const T *__restrict__ in, T *__restrict__ out,
                                    i64 batch, i64 h, i64 w) {
  const T ka = T(-0.0625), kb = T(-0.125), kc = T(0.75);
  const i64 total = batch * h * w;
  for (i64 idx = blockIdx.x * (i64)blockDim.x + threadIdx.x; idx < total;
       idx += (i64)gridDim.x * blockDim.x) {
    const i64 c = idx % w;
    const i64 r = (idx / w) % h;
    const T *x = in + (idx / (h * w)) * h * w;
    const i64 rp = r == 0 ? 1 : r - 1, rn = r == h - 1 ? r - 1 : r + 1;
    const i64 cp = c == 0 ? 1 : c - 1, cn = c == w - 1 ? c - 1 : c + 1;
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

template <typename T>
int fmg_restriction_launch(const T *in, T *out, i64 batch, i64 n, cudaStream_t st) {
  const i64 total = batch * 4 * (n - 1) * (n / 2);
  fmg_restriction_kernel<T><<<grid_1d(total), 256, 0, st>>>(in, out, batch * 4, n);
  return launch_status();
}

template <typename T>
int fmg_prolongation_launch(const T *in, T *out, i64 batch, i64 h, i64 w, cudaStream_t st) {
  fmg_prolongation_kernel<T><<<grid_1d(batch * 4 * h * w), 256, 0, st>>>(in, out, batch, h, w);
  return launch_status();
}

template <typename T>
int fmg_highpass_launch(const T *in, T *out, i64 batch, i64 h, i64 w, cudaStream_t st) {
  fmg_highpass_kernel<T><<<grid_1d(batch * h * w), 256, 0, st>>>(in, out, batch, h, w);
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
