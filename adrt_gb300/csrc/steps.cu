// Single-stage kernels in the (batch, 4, 2n-1, n) output layout.
#include "common.cuh"

namespace adrtg {

// One forward stage k.  The last axis packs (block, angle) as
// col = block * 2^(k+1) + angle; operand a at (row, 2*block*2^k + angle/2),
// operand b at (row - ceil(angle/2), (2*block+1)*2^k + angle/2); copy of a
// when row < ceil(angle/2).
// Reference: src/adrt/adrt_cdefs_adrt.hpp:215-258 (adrt_step).
template <typename T>
__global__ void adrt_step_kernel(const T *__restrict__ in, T *__restrict__ out, i64 planes,
                                 i64 n, int k) {
  const i64 C = 2 * n - 1;
  const i64 total = planes * C * n;
  const i64 E = i64(1) << k;
  for (i64 idx = blockIdx.x * (i64)blockDim.x + threadIdx.x; idx < total;
       idx += (i64)gridDim.x * blockDim.x) {
    const i64 col = idx % n;
    const i64 row = (idx / n) % C;
    const i64 base = idx - row * n - col;  // start of this plane
    const i64 blk = col >> (k + 1), ang = col & (2 * E - 1);
    const i64 ca = 2 * blk * E + (ang >> 1);
    const i64 cb = ca + E;
    const i64 sh = (ang + 1) >> 1;
    const T av = in[base + row * n + ca];
    out[idx] = row >= sh ? add_rn(av, in[base + (row - sh) * n + cb]) : av;
  }
}

// One backprojection step k (undoes forward stage L-1-k).  Even blocks add
// two neighbours in the same row; odd blocks add along the diagonal
// (row+i, row+i+1), where a missing operand is +0 and is still added.
// Reference: src/adrt/adrt_cdefs_bdrt.hpp:190-244 (bdrt_step).
template <typename T>
__global__ void bdrt_step_kernel(const T *__restrict__ in, T *__restrict__ out, i64 planes,
                                 i64 n, int ek) {
  const i64 C = 2 * n - 1;
  const i64 total = planes * C * n;
  const i64 E = i64(1) << ek;
  for (i64 idx = blockIdx.x * (i64)blockDim.x + threadIdx.x; idx < total;
       idx += (i64)gridDim.x * blockDim.x) {
    const i64 col = idx % n;
    const i64 row = (idx / n) % C;
    const i64 base = idx - row * n - col;
    const i64 blk = col >> ek, i = col & (E - 1);
    const i64 bc = 2 * (i + E * (blk >> 1));
    T v;
    if ((blk & 1) == 0) {
      v = add_rn(in[base + row * n + bc], in[base + row * n + bc + 1]);
    } else {
      const i64 r0 = row + i;
      const T av = r0 < C ? in[base + r0 * n + bc] : T(0);
      const T bv = r0 + 1 < C ? in[base + (r0 + 1) * n + bc + 1] : T(0);
      v = add_rn(av, bv);
    }
    out[idx] = v;
  }
}

static unsigned grid_for(i64 total, int threads) {
  i64 g = (total + threads - 1) / threads;
  const i64 cap = 152 * 32;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (unsigned)g;
}

template <typename T>
int adrt_step_launch(const T *in, T *out, i64 batch, i64 n, int k, cudaStream_t st) {
  const i64 total = batch * 4 * (2 * n - 1) * n;
  adrt_step_kernel<T><<<grid_for(total, 256), 256, 0, st>>>(in, out, batch * 4, n, k);
  return launch_status();
}

template <typename T>
int bdrt_step_launch(const T *in, T *out, i64 batch, i64 n, int k, cudaStream_t st) {
  const int L = num_iters(n);
  const i64 total = batch * 4 * (2 * n - 1) * n;
  bdrt_step_kernel<T><<<grid_for(total, 256), 256, 0, st>>>(in, out, batch * 4, n, L - k - 1);
  return launch_status();
}

template int adrt_step_launch<float>(const float *, float *, i64, i64, int, cudaStream_t);
template int adrt_step_launch<double>(const double *, double *, i64, i64, int, cudaStream_t);
template int bdrt_step_launch<float>(const float *, float *, i64, i64, int, cudaStream_t);
template int bdrt_step_launch<double>(const double *, double *, i64, i64, int, cudaStream_t);

}  // namespace adrtg
