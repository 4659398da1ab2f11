// Single-stage kernels in the (batch, 4, 2n-1, n) output layout.
#include "common.cuh"

namespace adrtg {

// One forward stage k.  The last axis packs (block, angle) as
// col = block * 2^(k+1) + angle; operand a at (row, 2*block*2^k + angle/2),
// operand b at (row - ceil(angle/2), (2*block+1)*2^k + angle/2); copy of a
// when row < ceil(angle/2).
// Reference: src/adrt/adrt_cdefs_adrt.hpp:215-258 (adrt_step).
// Index arithmetic runs in I: 32-bit unsigned whenever the element count
// allows (64-bit division is a long instruction sequence), 64-bit otherwise.
// n is a power of two (lg = log2 n): the column is a mask, the row one
// division by C = 2n-1.
template <typename T, typename I>
__global__ void adrt_step_kernel(const T *__restrict__ in, T *__restrict__ out, I total, I n, int lg, int k) {
  const I C = 2 * n - 1;
  const I E = I(1) << k;
  for (I idx = blockIdx.x * (I)blockDim.x + threadIdx.x; idx < total; idx += (I)gridDim.x * blockDim.x) {
    const I col = idx & (n - 1);
    const I rp = idx >> lg;  // plane * C + row
    const I row = rp % C;
    const I base = (rp - row) << lg;  // start of this plane
    const I blk = col >> (k + 1), ang = col & (2 * E - 1);
    const I ca = 2 * blk * E + (ang >> 1);
    const I cb = ca + E;
    const I sh = (ang + 1) >> 1;
    const T av = in[base + (row << lg) + ca];
    out[idx] = row >= sh ? add_rn(av, in[base + ((row - sh) << lg) + cb]) : av;
  }
}

// One backprojection step k (undoes forward stage L-1-k).  Even blocks add
// two neighbours in the same row; odd blocks add along the diagonal
// (row+i, row+i+1), where a missing operand is +0 and is still added.
// Reference: src/adrt/adrt_cdefs_bdrt.hpp:190-244 (bdrt_step).
template <typename T, typename I>
__global__ void bdrt_step_kernel(const T *__restrict__ in, T *__restrict__ out, I total, I n, int lg, int ek) {
  const I C = 2 * n - 1;
  const I E = I(1) << ek;
  for (I idx = blockIdx.x * (I)blockDim.x + threadIdx.x; idx < total; idx += (I)gridDim.x * blockDim.x) {
    const I col = idx & (n - 1);
    const I rp = idx >> lg;
    const I row = rp % C;
    const I base = (rp - row) << lg;
    const I blk = col >> ek, i = col & (E - 1);
    const I bc = 2 * (i + E * (blk >> 1));
    T v;
    if ((blk & 1) == 0) {
      v = add_rn(in[base + (row << lg) + bc], in[base + (row << lg) + bc + 1]);
    } else {
      const I r0 = row + i;
      const T av = r0 < C ? in[base + (r0 << lg) + bc] : T(0);
      const T bv = r0 + 1 < C ? in[base + ((r0 + 1) << lg) + bc + 1] : T(0);
      v = add_rn(av, bv);
    }
    out[idx] = v;
  }
}

// 32-bit indices when every index (plus one grid stride) stays below 2^32.
inline bool fits_u32(i64 total) { return total < (i64(1) << 32) - (i64(1) << 24); }

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
  const int lg = num_iters(n);
  if (fits_u32(total))
    adrt_step_kernel<T, unsigned><<<grid_for(total, 256), 256, 0, st>>>(in, out, (unsigned)total, (unsigned)n, lg, k);
  else
    adrt_step_kernel<T, unsigned long long><<<grid_for(total, 256), 256, 0, st>>>(
        in, out, (unsigned long long)total, (unsigned long long)n, lg, k);
  return launch_status();
}

template <typename T>
int bdrt_step_launch(const T *in, T *out, i64 batch, i64 n, int k, cudaStream_t st) {
  const int L = num_iters(n);
  const i64 total = batch * 4 * (2 * n - 1) * n;
  if (fits_u32(total))
    bdrt_step_kernel<T, unsigned><<<grid_for(total, 256), 256, 0, st>>>(in, out, (unsigned)total, (unsigned)n, L,
                                                                        L - k - 1);
  else
    bdrt_step_kernel<T, unsigned long long><<<grid_for(total, 256), 256, 0, st>>>(
        in, out, (unsigned long long)total, (unsigned long long)n, L, L - k - 1);
  return launch_status();
}

template int adrt_step_launch<float>(const float *, float *, i64, i64, int, cudaStream_t);
template int adrt_step_launch<double>(const double *, double *, i64, i64, int, cudaStream_t);
template int bdrt_step_launch<float>(const float *, float *, i64, i64, int, cudaStream_t);
template int bdrt_step_launch<double>(const double *, double *, i64, i64, int, cudaStream_t);

}  // namespace adrtg
