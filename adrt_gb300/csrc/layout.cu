// Layout kernels: adrt_init, truncate, stitch (pure copies, any element size)
// and the quadrant sum of the adjoint.
#include "common.cuh"

namespace adrtg {

// Element-size-generic storage types (copies only move bits).
template <int B> struct word;
template <> struct word<1> { using t = uint8_t; };
template <> struct word<2> { using t = uint16_t; };
template <> struct word<4> { using t = uint32_t; };
template <> struct word<8> { using t = uint64_t; };
struct alignas(16) w16 {
  uint64_t lo, hi;
  w16() = default;
  __host__ __device__ explicit w16(int) : lo(0), hi(0) {}
};
template <> struct word<16> { using t = w16; };

// (n, n) image -> (4, 2n-1, n):  q0[c][a] = x[a][n-1-c], q1[c][a] = x[n-1-c][a],
// q2[c][a] = x[c][a], q3[c][a] = x[n-1-a][n-1-c]; zero for c >= n.
// Reference: src/adrt/core.py:170-175.
// Index arithmetic of the copy kernels runs in I: 32-bit unsigned when every
// index fits (64-bit division is a long instruction sequence), else 64-bit.
template <typename W, typename I>
__device__ __forceinline__ void init_body(const W *__restrict__ in, W *__restrict__ out, I batch, I n) {
  const I C = 2 * n - 1;
  const I total = batch * 4 * C * n;
  for (I idx = blockIdx.x * (I)blockDim.x + threadIdx.x; idx < total;
       idx += (I)gridDim.x * blockDim.x) {
    const I a = idx % n;
    const I rq = idx / n;
    const I c = rq % C;
    const I bq = rq / C;
    const int q = (int)(bq & 3);
    const I b = bq >> 2;
    const W *x = in + b * n * n;
    W v = W(0);
    if (c < n) {
      switch (q) {
        case 0: v = x[a * n + (n - 1 - c)]; break;
        case 1: v = x[(n - 1 - c) * n + a]; break;
        case 2: v = x[c * n + a]; break;
        default: v = x[(n - 1 - a) * n + (n - 1 - c)]; break;
      }
    }
    out[idx] = v;
  }
}

// Index into quadrant q of an ADRT array for truncate's output (i, j).
// Reference: src/adrt/utils.py:234-242.
__device__ __forceinline__ i64 trunc_src(int q, i64 i, i64 j, i64 n) {
  switch (q) {
    case 0: return (n - 1 - j) * n + i;
    case 1: return (n - 1 - i) * n + j;
    case 2: return i * n + j;
    default: return (n - 1 - j) * n + (n - 1 - i);
  }
}

template <typename W, typename I>
__device__ __forceinline__ void truncate_body(const W *__restrict__ in, W *__restrict__ out, I batch, I n) {
  const I C = 2 * n - 1;
  const I total = batch * 4 * n * n;
  for (I idx = blockIdx.x * (I)blockDim.x + threadIdx.x; idx < total;
       idx += (I)gridDim.x * blockDim.x) {
    const I j = idx % n;
    const I r = idx / n;
    const I i = r % n;
    const I bq = r / n;
    out[idx] = in[bq * C * n + (I)trunc_src((int)(bq & 3), i, j, n)];
  }
}

// (4, 2n-1, n) -> (3n-2, 4, vc): quadrant k flipped on both axes when k is
// odd, last column dropped when remove_repeated, rows offset by n-1 for k >= 2.
// Reference: src/adrt/utils.py:111-134.
template <typename W>
__global__ void __launch_bounds__(256) stitch_kernel(const W *__restrict__ in, W *__restrict__ out, i64 batch,
                                                     i64 n_, int remove_repeated) {
  // One block per output segment (b, row, k): vc contiguous outputs, read
  // from one input row (reversed for odd k), or zeros outside quadrant k.
  const unsigned n = (unsigned)n_;
  const unsigned C = 2 * n - 1, OR = 3 * n - 2;
  const unsigned vc = n - (remove_repeated ? 1 : 0);
  const i64 seg = blockIdx.x;
  const unsigned k = (unsigned)(seg & 3);
  const i64 brow = seg >> 2;
  const unsigned row = (unsigned)(brow % OR);
  const i64 b = brow / OR;
  W *o = out + seg * (i64)vc;
  const int rr = (int)row - (k >= 2 ? (int)n - 1 : 0);
  if (rr < 0 || rr >= (int)C) {
    for (unsigned c = threadIdx.x; c < vc; c += 256) o[c] = W(0);
    return;
  }
  const unsigned sr = (k & 1) ? C - 1 - (unsigned)rr : (unsigned)rr;
  const W *irow = in + ((b * 4 + k) * C + sr) * (i64)n;
  for (unsigned c = threadIdx.x; c < vc; c += 256) o[c] = irow[(k & 1) ? n - 1 - c : c];
}

// (3n-2, 4, vc) -> (4, 2n-1, n), the inverse of stitch_kernel: quadrant q
// read from rows [0, 2n-1) (q < 2) or [n-1, 3n-2) (q >= 2), flipped on both
// axes when q is odd; with vc = n-1 the last column comes from column 0 of
// quadrant q+1 (rows reversed for q = 3).  Reference: src/adrt/utils.py:137-188.
template <typename W>
__global__ void __launch_bounds__(256) unstitch_kernel(const W *__restrict__ in, W *__restrict__ out, i64 batch,
                                                       i64 n_, i64 vc_) {
  // One block per output row (b, q, r): per-row index work once, then a
  // contiguous (or reversed, for odd q) sweep over the row's n columns.
  const unsigned n = (unsigned)n_, vc = (unsigned)vc_;
  const unsigned C = 2 * n - 1, OR = 3 * n - 2;
  const i64 row_id = blockIdx.x;
  const unsigned r = (unsigned)(row_id % C);
  const i64 bq = row_id / C;
  const unsigned q = (unsigned)(bq & 3);
  const i64 b = bq >> 2;
  const unsigned rs = (q & 1) ? C - 1 - r : r;
  const unsigned R = rs + (q >= 2 ? n - 1 : 0);
  const W *srow = in + ((b * OR + R) * 4 + q) * (i64)vc;
  const unsigned R2 = q == 3 ? OR - 1 - R : R;
  const W *sext = in + ((b * OR + R2) * 4 + ((q + 1) & 3)) * (i64)vc;
  W *orow = out + row_id * (i64)n;
  for (unsigned c = threadIdx.x; c < n; c += 256) {
    const unsigned cs = (q & 1) ? n - 1 - c : c;
    orow[c] = cs < vc ? srow[cs] : sext[0];
  }
}

// Adjoint tail: out[b][i][j] = ((t0 + t1) + t2) + t3 with t_q = truncate(y)[q].
// n is a power of two (lg = log2 n): index arithmetic is shifts and masks, in
// 32-bit unsigned when the element count allows.
template <typename T, typename I>
__global__ void quad_sum_kernel(const T *__restrict__ y, T *__restrict__ out, I total, I n, int lg) {
  const I C = 2 * n - 1;
  for (I idx = blockIdx.x * (I)blockDim.x + threadIdx.x; idx < total; idx += (I)gridDim.x * blockDim.x) {
    const I j = idx & (n - 1);
    const I i = (idx >> lg) & (n - 1);
    const T *yb = y + (idx >> (2 * lg)) * 4 * C * n;
    T s = add_rn(yb[trunc_src(0, i, j, n)], yb[C * n + trunc_src(1, i, j, n)]);
    s = add_rn(s, yb[2 * C * n + trunc_src(2, i, j, n)]);
    out[idx] = add_rn(s, yb[3 * C * n + trunc_src(3, i, j, n)]);
  }
}

// The same sum for n >= 32 on 32 x 32 output tiles: quadrants 0 and 3 are
// read along their rows (coalesced) into shared memory and taken transposed
// from there; quadrants 1 and 2 are read directly.  Same operand order.
template <typename T>
__global__ void __launch_bounds__(256) quad_sum_tiled_kernel(const T *__restrict__ y, T *__restrict__ out,
                                                             unsigned n) {
  __shared__ T t0[32][33], t3[32][33];
  const unsigned C = 2 * n - 1;
  const unsigned i0 = blockIdx.y * 32, j0 = blockIdx.x * 32;
  const T *yb = y + (size_t)blockIdx.z * 4 * C * n;
  const unsigned tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
#pragma unroll
  for (unsigned k = 0; k < 4; ++k) {
    const unsigned jj = ty + 8 * k;
    const unsigned srow = n - 1 - (j0 + jj);
    t0[jj][tx] = yb[srow * n + (i0 + tx)];                          // quadrant 0: (n-1-j, i)
    t3[jj][tx] = yb[3 * (size_t)C * n + srow * n + (n - 1 - (i0 + tx))];  // quadrant 3: (n-1-j, n-1-i)
  }
  __syncthreads();
  T *ob = out + (size_t)blockIdx.z * n * n;
#pragma unroll
  for (unsigned k = 0; k < 4; ++k) {
    const unsigned ii = ty + 8 * k;
    const unsigned i = i0 + ii, j = j0 + tx;
    T s = add_rn(t0[tx][ii], yb[(size_t)C * n + (n - 1 - i) * n + j]);
    s = add_rn(s, yb[2 * (size_t)C * n + i * n + j]);
    ob[i * n + j] = add_rn(s, t3[tx][ii]);
  }
}

template <typename W>
__global__ void init_kernel_u32(const W *__restrict__ in, W *__restrict__ out, unsigned batch, unsigned n) {
  init_body<W, unsigned>(in, out, batch, n);
}
template <typename W>
__global__ void init_kernel_u64(const W *__restrict__ in, W *__restrict__ out, unsigned long long batch,
                                unsigned long long n) {
  init_body<W, unsigned long long>(in, out, batch, n);
}
template <typename W>
__global__ void truncate_kernel_u32(const W *__restrict__ in, W *__restrict__ out, unsigned batch, unsigned n) {
  truncate_body<W, unsigned>(in, out, batch, n);
}
template <typename W>
__global__ void truncate_kernel_u64(const W *__restrict__ in, W *__restrict__ out, unsigned long long batch,
                                    unsigned long long n) {
  truncate_body<W, unsigned long long>(in, out, batch, n);
}

static unsigned grid_l(i64 total) {
  i64 g = (total + 255) / 256;
  if (g > 152 * 32) g = 152 * 32;
  return (unsigned)(g < 1 ? 1 : g);
}

#define BY_SIZE(ES, KERNEL, TOTAL, ...)                                                     \
  switch (ES) {                                                                             \
    case 1: KERNEL<word<1>::t><<<grid_l(TOTAL), 256, 0, st>>>(                              \
        (const word<1>::t *)in, (word<1>::t *)out, __VA_ARGS__); break;                     \
    case 2: KERNEL<word<2>::t><<<grid_l(TOTAL), 256, 0, st>>>(                              \
        (const word<2>::t *)in, (word<2>::t *)out, __VA_ARGS__); break;                     \
    case 4: KERNEL<word<4>::t><<<grid_l(TOTAL), 256, 0, st>>>(                              \
        (const word<4>::t *)in, (word<4>::t *)out, __VA_ARGS__); break;                     \
    case 8: KERNEL<word<8>::t><<<grid_l(TOTAL), 256, 0, st>>>(                              \
        (const word<8>::t *)in, (word<8>::t *)out, __VA_ARGS__); break;                     \
    case 16: KERNEL<word<16>::t><<<grid_l(TOTAL), 256, 0, st>>>(                            \
        (const word<16>::t *)in, (word<16>::t *)out, __VA_ARGS__); break;                   \
    default: return ADRT_GB300_ERR_DTYPE;                                                   \
  }

static bool fits_u32(i64 max_index) { return max_index < (i64(1) << 32) - (i64(1) << 24); }

int init_launch(const void *in, void *out, i64 batch, i64 n, size_t es, cudaStream_t st) {
  const i64 total = batch * 4 * (2 * n - 1) * n;
  if (fits_u32(total)) {
    const unsigned B = (unsigned)batch, N = (unsigned)n;
    BY_SIZE(es, init_kernel_u32, total, B, N)
  } else {
    BY_SIZE(es, init_kernel_u64, total, (unsigned long long)batch, (unsigned long long)n)
  }
  return launch_status();
}

int truncate_launch(const void *in, void *out, i64 batch, i64 n, size_t es, cudaStream_t st) {
  const i64 total = batch * 4 * (2 * n - 1) * n;  // largest input index
  if (fits_u32(total)) {
    const unsigned B = (unsigned)batch, N = (unsigned)n;
    BY_SIZE(es, truncate_kernel_u32, batch * 4 * n * n, B, N)
  } else {
    BY_SIZE(es, truncate_kernel_u64, batch * 4 * n * n, (unsigned long long)batch, (unsigned long long)n)
  }
  return launch_status();
}

int stitch_launch(const void *in, void *out, i64 batch, i64 n, int rr, size_t es, cudaStream_t st) {
  const i64 segs = batch * (3 * n - 2) * 4;
  if (segs > 0x7fffffffll || n > 32768) return ADRT_GB300_ERR_TOO_LARGE;
  const unsigned grid = (unsigned)segs;
  switch (es) {
    case 1: stitch_kernel<word<1>::t><<<grid, 256, 0, st>>>((const word<1>::t *)in, (word<1>::t *)out, batch, n, rr); break;
    case 2: stitch_kernel<word<2>::t><<<grid, 256, 0, st>>>((const word<2>::t *)in, (word<2>::t *)out, batch, n, rr); break;
    case 4: stitch_kernel<word<4>::t><<<grid, 256, 0, st>>>((const word<4>::t *)in, (word<4>::t *)out, batch, n, rr); break;
    case 8: stitch_kernel<word<8>::t><<<grid, 256, 0, st>>>((const word<8>::t *)in, (word<8>::t *)out, batch, n, rr); break;
    case 16: stitch_kernel<word<16>::t><<<grid, 256, 0, st>>>((const word<16>::t *)in, (word<16>::t *)out, batch, n, rr); break;
    default: return ADRT_GB300_ERR_DTYPE;
  }
  return launch_status();
}

int unstitch_launch(const void *in, void *out, i64 batch, i64 n, i64 vc, size_t es, cudaStream_t st) {
  const i64 rows = batch * 4 * (2 * n - 1);
  if (rows > 0x7fffffffll || n > 32768) return ADRT_GB300_ERR_TOO_LARGE;
  const unsigned grid = (unsigned)rows;
  switch (es) {
    case 1: unstitch_kernel<word<1>::t><<<grid, 256, 0, st>>>((const word<1>::t *)in, (word<1>::t *)out, batch, n, vc); break;
    case 2: unstitch_kernel<word<2>::t><<<grid, 256, 0, st>>>((const word<2>::t *)in, (word<2>::t *)out, batch, n, vc); break;
    case 4: unstitch_kernel<word<4>::t><<<grid, 256, 0, st>>>((const word<4>::t *)in, (word<4>::t *)out, batch, n, vc); break;
    case 8: unstitch_kernel<word<8>::t><<<grid, 256, 0, st>>>((const word<8>::t *)in, (word<8>::t *)out, batch, n, vc); break;
    case 16: unstitch_kernel<word<16>::t><<<grid, 256, 0, st>>>((const word<16>::t *)in, (word<16>::t *)out, batch, n, vc); break;
    default: return ADRT_GB300_ERR_DTYPE;
  }
  return launch_status();
}

template <typename T>
int quad_sum_launch(const T *y, T *out, i64 batch, i64 n, cudaStream_t st) {
  const i64 total = batch * n * n;
  const int lg = num_iters(n);
  if (n >= 32 && n <= 32768 && batch <= 65535) {
    const unsigned t = (unsigned)(n / 32);
    quad_sum_tiled_kernel<T><<<dim3(t, t, (unsigned)batch), 256, 0, st>>>(y, out, (unsigned)n);
    return launch_status();
  }
  if (total * 8 < (i64(1) << 32))
    quad_sum_kernel<T, unsigned><<<grid_l(total), 256, 0, st>>>(y, out, (unsigned)total, (unsigned)n, lg);
  else
    quad_sum_kernel<T, unsigned long long><<<grid_l(total), 256, 0, st>>>(y, out, (unsigned long long)total,
                                                                            (unsigned long long)n, lg);
  return launch_status();
}
template int quad_sum_launch<float>(const float *, float *, i64, i64, cudaStream_t);
template int quad_sum_launch<double>(const double *, double *, i64, i64, cudaStream_t);

}  // namespace adrtg
