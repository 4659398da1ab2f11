// Exact inverse ADRT.
//
// The reference (src/adrt/adrt_cdefs_iadrt.hpp:53-105) runs log2(n) stages; in
// stage s every chain (l, col), l < 2^(s+1), col < n / 2^(s+1), is a serial
// recurrence from the last offset row down to row 0:
//   l even: v = (0 + E[row]) - O[row+1]             (O term if row+1 < R)
//   l odd:  v = (0 + O[row+1+col]) - E[row+1+col]   (if row+1+col < R, else 0)
//   v += out[row+1]                                  (if row+1 < R)
// with E, O the input chains (l/2, 2col) and (l/2, 2col+1), R = 2n-1.
//
// The recurrence is kept serial per chain (same operation order, so the
// ill-conditioned result is bit-identical).  The GPU layout is
// [row][chain] per (batch, quadrant), chain = l * (n/2^(s+1)) + col, so that a
// warp's chains are adjacent in memory at every row; the reference's input
// (4, 2n-1, n) is already this layout with chain = angle, and so is its output.
#include "common.cuh"

namespace adrtg {

// Loads for a chain never depend on its running value, so each thread keeps
// the operands of the next U rows in a register ring (slot u holds row
// row0 - u): the latency of a load is hidden behind U serial steps instead of
// stalling every step.  U = 32 (float32) / 16 (float64) for n >= 1024, where
// few chains run per SM and the deeper ring hides more latency (n = 1024,
// batch 2: 1.9k img/s against 1.6k with 16); half that below, where more
// chains are resident and the smaller register footprint wins (n = 256,
// batch 64: 111k against 97k img/s).  Threads are ordered so that the first n/2 of a plane
// run even-l chains and the rest odd-l chains: warps do not diverge between
// the two recurrences.

template <typename T>
__device__ __forceinline__ T ld_or_zero(const T *p, bool ok) { return ok ? __ldg(p) : T(0); }

// Index arithmetic is 32-bit: a plane holds n (2n-1) < 2^31 elements for the
// sizes the host accepts (n <= 32768).
template <typename T, int U>
__global__ void __launch_bounds__(128)
iadrt_stage_kernel(const T *__restrict__ in, T *__restrict__ out, i64 planes, i64 n_, int s, int row_sweep) {
  const int n = (int)n_;
  const int R = 2 * n - 1;
  const int Cc = n >> s;           // input chains per l
  const int C2 = Cc >> 1;          // output chains per l
  const int half = n >> 1;         // even-l (and odd-l) chains per plane
  const i64 gid = blockIdx.x * (i64)blockDim.x + threadIdx.x;
  if (gid >= planes * n) return;
  const i64 plane = gid / n;
  const int t = (int)(gid - plane * n);
  const bool odd = t >= half;
  const int tt = odd ? t - half : t;
  const int l = 2 * (tt / C2) + (odd ? 1 : 0), col = tt % C2;
  const int ch = l * C2 + col;
  const int pl = l >> 1;
  const T *src = in + plane * (i64)R * n;
  T *dst = out + plane * (i64)R * n;
  const int e_ch = pl * Cc + 2 * col;
  const int o_ch = e_ch + 1;
  T ea[U], oa[U];
  T prev = T(0);
  if (!odd) {
    // v = (0 + E[row]) - O[row + 1] + prev   (O and prev only if row + 1 < R)
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int r = R - 1 - u;
      ea[u] = ld_or_zero(src + r * n + e_ch, r >= 0);
      oa[u] = ld_or_zero(src + (r + 1) * n + o_ch, r >= 0 && r + 1 < R);
    }
    for (int row0 = R - 1; row0 >= 0; row0 -= U) {
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int row = row0 - u;
        if (row >= 0) {
          T v = add_rn(T(0), ea[u]);
          if (row + 1 < R) {
            v = sub_rn(v, oa[u]);
            v = add_rn(v, prev);
          }
          dst[row * n + ch] = v;
          prev = v;
        }
        const int r = row - U;
        ea[u] = ld_or_zero(src + r * n + e_ch, r >= 0);
        oa[u] = ld_or_zero(src + (r + 1) * n + o_ch, r >= 0);
      }
    }
  } else if (C2 < 32 || !row_sweep) {
    // Each lane sweeps its own output rows (reading the input d rows below:
    // one row per lane).  Stages with fewer than 32 columns per l (n <= 16)
    // always do (a warp mixes columns of several l); others when few chains
    // run (the row sweep below pays more latency per step, which only
    // enough resident warps hide).
    // v = (0 + O[row + d]) - E[row + d]  (if row + d < R, else 0); v += prev (row + 1 < R)
    const int d = 1 + col;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int r = R - 1 - u + d;
      const bool ok = r < R && r >= d;
      ea[u] = ld_or_zero(src + r * n + e_ch, ok);
      oa[u] = ld_or_zero(src + r * n + o_ch, ok);
    }
    for (int row0 = R - 1; row0 >= 0; row0 -= U) {
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int row = row0 - u;
        if (row >= 0) {
          T v = T(0);
          if (row + d < R) {
            v = add_rn(v, oa[u]);
            v = sub_rn(v, ea[u]);
          }
          if (row + 1 < R) v = add_rn(v, prev);
          dst[row * n + ch] = v;
          prev = v;
        }
        const int r = row - U + d;
        const bool ok = r < R && r >= d;
        ea[u] = ld_or_zero(src + r * n + e_ch, ok);
        oa[u] = ld_or_zero(src + r * n + o_ch, ok);
      }
    }
  } else {
    // v = (0 + O[row + d]) - E[row + d]  (if row + d < R, else 0); v += prev (row + 1 < R),
    // d = 1 + col.  With C2 >= 32 a warp's lanes are 32 consecutive columns
    // of one l, so d_lane = d0 + lane with d0 the same for the whole warp.
    // The warp sweeps the input row x: every lane reads row x (one coalesced
    // row per load) and computes its output row y = x - d_lane.  Rows
    // R-d .. R-1 have no operand and are +0 (0, then 0 + prev): they are the
    // steps x >= R.  Outputs go to a 32-row shared ring; row x - d0 is
    // complete once lane 0 has written it (the other lanes wrote it at
    // earlier steps, x + lane), and the warp stores it as one coalesced row.
    // The ring is dynamic shared memory (32 x 32 values per warp), given only
    // to launches that take this path.
    extern __shared__ __align__(16) unsigned char stage_smem[];
    T(*rg)[32] = reinterpret_cast<T(*)[32]>(stage_smem) + 32 * (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    const int d = 1 + col, d0 = d - lane;
    const int ch0 = ch - lane;
    const int x_top = R - 1 + d0 + 31;  // lane 31's row R-1
    // steps x >= R: the +0 rows
    for (int x = x_top; x >= R; --x) {
      const int y = x - d;
      if (y >= 0 && y < R) rg[y & 31][lane] = T(0);
      __syncwarp();
      const int yc = x - d0;
      if (yc < R) dst[yc * n + ch0 + lane] = rg[yc & 31][lane];
      __syncwarp();
    }
    // steps d0 <= x <= R-1: operands from input row x
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int x = R - 1 - u;
      const bool ok = x >= d0;
      ea[u] = ld_or_zero(src + x * n + e_ch, ok);
      oa[u] = ld_or_zero(src + x * n + o_ch, ok);
    }
    for (int x0 = R - 1; x0 >= d0; x0 -= U) {
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int x = x0 - u;
        if (x >= d0) {  // warp-uniform
          const int y = x - d;
          if (y >= 0) {
            T v = add_rn(T(0), oa[u]);
            v = sub_rn(v, ea[u]);
            v = add_rn(v, prev);  // y <= R - 2
            prev = v;
            rg[y & 31][lane] = v;
          }
          __syncwarp();
          const int yc = x - d0;
          dst[yc * n + ch0 + lane] = rg[yc & 31][lane];
          __syncwarp();
        }
        const int xn = x - U;
        const bool ok = xn >= d0;
        ea[u] = ld_or_zero(src + xn * n + e_ch, ok);
        oa[u] = ld_or_zero(src + xn * n + o_ch, ok);
      }
    }
  }
}

// The last five stages (s0 = L-5 .. L-1) in one sweep.  Across them the
// chains form closed groups: output chains of level L with angles
// [32A, 32A + 32) depend only on the level-s0 chains of angle A (its 32
// sections), and at every level s0 + t in between the group's 32 chains sit
// at chain indices 32A .. 32A + 31 (angle A 2^t + (lane >> (5-t)), section
// lane mod 2^(5-t)).  One warp runs one group of one plane: it walks the rows
// from R-1 down to 0 and, at each row, computes the five levels in order, each
// lane one chain per level with the recurrence above (same operations, same
// order).  A level reads the previous one at rows r, r + 1 and r + d, d = 1 +
// col <= 16, so each level's last 17 rows stay in a shared-memory ring.  The
// five intermediate levels never leave the SM: one read of the input and one
// write of the output replace five of each.
constexpr int kLast5Ring = 17;      // rows r .. r + 16
constexpr int kLast5Prefetch = 8;   // input rows loaded ahead
// Warps (groups) per CTA: the rings of a CTA stay under 48 KB of static
// shared memory (44.9 KB for float32 x 4 warps, float64 x 2).
template <typename T> constexpr int last5_warps() { return sizeof(T) == 4 ? 4 : 2; }

// One row of the fused sweep for this lane: the five levels in order.  Both
// recurrences read two values of the previous level: even chains E[r] and
// O[r + 1], odd chains O[r + d] and E[r + d]; the lane's ring rows and
// lanes are chosen by select, so the warp does not diverge between them.
// EDGE: a row within 16 of the top (some operands lie past row R-1: the
// reference's conditions apply); elsewhere every operand exists.
template <typename T, bool EDGE>
__device__ __forceinline__ void last5_row(T (*rg)[kLast5Ring][33], int r, int R, int slot, const int (&la)[5],
                                          const int (&lb)[5], const int (&dd)[5], const bool (&odd)[5],
                                          T (&prev)[5], T *dst_row, int lane) {
  constexpr int H = kLast5Ring;
  const int s1 = slot + 1 == H ? 0 : slot + 1;
#pragma unroll
  for (int t = 0; t < 5; ++t) {
    int sd = slot + dd[t];
    sd -= sd >= H ? H : 0;
    const T x1 = rg[t][odd[t] ? sd : slot][la[t]];  // E[r] or O[r + d]
    const T x2 = rg[t][odd[t] ? sd : s1][lb[t]];    // O[r + 1] or E[r + d]
    T v;
    if (!EDGE) {
      v = add_rn(T(0), x1);
      v = sub_rn(v, x2);
      v = add_rn(v, prev[t]);
    } else {
      // even: v = (0 + E[r]); if r + 1 < R: v = v - O[r + 1] + prev
      // odd:  v = 0; if r + d < R: v = (0 + O[r + d]) - E[r + d]; if r + 1 < R: v += prev
      const bool in1 = r + 1 < R, ind = r + dd[t] < R;
      const bool first = odd[t] ? ind : true, second = odd[t] ? ind : in1;
      v = first ? add_rn(T(0), x1) : T(0);
      if (second) v = sub_rn(v, x2);
      if (in1) v = add_rn(v, prev[t]);
    }
    prev[t] = v;
    if (t < 4) {
      rg[t + 1][slot][lane] = v;
      __syncwarp();
    } else {
      *dst_row = v;
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(32 * last5_warps<T>())
iadrt_last5_kernel(const T *__restrict__ in, T *__restrict__ out, i64 groups, int n) {
  constexpr int WPB = last5_warps<T>();
  constexpr int H = kLast5Ring, LS = 33;  // ring row stride: lanes reading rows r and r + d hit distinct banks
  __shared__ T ring[WPB][5][H][LS];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const i64 g = blockIdx.x * (i64)WPB + w;
  if (g >= groups) return;  // whole warps only: the sweep below synchronises within the warp
  const int gpp = n >> 5;   // groups per plane
  const i64 plane = g / gpp;
  const int A = (int)(g - plane * gpp);
  const int R = 2 * n - 1;
  const T *src = in + plane * (i64)R * n + 32 * A + lane;
  T *dst = out + plane * (i64)R * n + 32 * A + lane;
  T(*rg)[H][LS] = ring[w];
  // Per output level t + 1: parity, input lanes and lag of this lane's chain
  // (la: the lane of the first operand, E for even chains, O for odd ones).
  int la[5], lb[5], dd[5];
  bool odd[5];
#pragma unroll
  for (int t = 0; t < 5; ++t) {
    const int lam = lane >> (4 - t), col = lane & ((1 << (4 - t)) - 1);
    const int e = ((lam >> 1) << (5 - t)) + 2 * col;
    odd[t] = lam & 1;
    la[t] = odd[t] ? e + 1 : e;
    lb[t] = odd[t] ? e : e + 1;
    dd[t] = 1 + col;
  }
  T prev[5];
#pragma unroll
  for (int t = 0; t < 5; ++t) prev[t] = T(0);
  constexpr int U = kLast5Prefetch;
  T q[U];
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int r = R - 1 - u;
    q[u] = r >= 0 ? __ldg(src + (size_t)r * n) : T(0);
  }
  int slot = (R - 1) % H;  // ring slot of row r
  for (int row0 = R - 1; row0 >= 0; row0 -= U) {
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int r = row0 - u;
      if (r >= 0) {  // warp-uniform
        rg[0][slot][lane] = q[u];
        __syncwarp();
        if (r >= R - 16)
          last5_row<T, true>(rg, r, R, slot, la, lb, dd, odd, prev, dst + (size_t)r * n, lane);
        else
          last5_row<T, false>(rg, r, R, slot, la, lb, dd, odd, prev, dst + (size_t)r * n, lane);
        slot = slot == 0 ? H - 1 : slot - 1;
      }
      const int rn = r - U;
      q[u] = rn >= 0 ? __ldg(src + (size_t)rn * n) : T(0);
    }
  }
}

template <typename T>
__global__ void copy_kernel(const T *__restrict__ in, T *__restrict__ out, i64 total) {
  for (i64 i = blockIdx.x * (i64)blockDim.x + threadIdx.x; i < total;
       i += (i64)gridDim.x * blockDim.x)
    out[i] = in[i];
}

size_t iadrt_workspace_bytes(i64 batch, i64 n, size_t elem) {
  const int L = num_iters(n);
  const size_t per = (size_t)batch * 4 * n * (2 * n - 1) * elem;
  return L >= 3 ? 2 * per : (L == 2 ? per : 0);
}

template <typename T>
int iadrt_launch(const T *in, T *out, i64 batch, i64 n, void *ws, size_t ws_bytes,
                 cudaStream_t st) {
  const int L = num_iters(n);
  if (n > 32768) return ADRT_GB300_ERR_TOO_LARGE;  // 32-bit in-plane offsets
  const i64 planes = batch * 4;
  const i64 elems = planes * n * (2 * n - 1);
  if (L == 0) {
    copy_kernel<T><<<(unsigned)((elems + 255) / 256), 256, 0, st>>>(in, out, elems);
    return launch_status();
  }
  if (ws_bytes < iadrt_workspace_bytes(batch, n, sizeof(T)) || (L >= 2 && ws == nullptr))
    return ADRT_GB300_ERR_WORKSPACE;
  T *bufs[2] = {static_cast<T *>(ws), static_cast<T *>(ws) + elems};
  const T *src = in;
  const i64 threads = planes * n;
  // Few chains (small batches): 32-thread blocks so that they spread over
  // all SMs; otherwise 128.
  const int bs = threads >= (i64)152 * 4 * 128 ? 128 : 32;
  // Odd chains swept by input row (coalesced loads and stores through a
  // shared ring) when at least 32 warps of chains per SM run: measured
  // n = 1024 x 64 images 7.8k -> 8.8k img/s, n = 64 x 1024 +7 %; with fewer
  // (n = 256 x 64, n = 1024 x 2) the per-lane sweep is faster.
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int row_sweep = threads >= (i64)sms * 32 * 32 ? 1 : 0;
  const unsigned grid = (unsigned)((threads + bs - 1) / bs);
  constexpr int U_DEEP = sizeof(T) == 4 ? 32 : 16;
  // n >= 32: the first L-5 stages one kernel each, the last five fused.
  const int single = L >= 5 ? L - 5 : L;
  for (int s = 0; s < single; ++s) {
    T *dst = (s == L - 1) ? out : bufs[s & 1];
    const size_t smem = row_sweep ? (size_t)(bs / 32) * 32 * 32 * sizeof(T) : 0;
    if (n >= 1024)
      iadrt_stage_kernel<T, U_DEEP><<<grid, bs, smem, st>>>(src, dst, planes, n, s, row_sweep);
    else
      iadrt_stage_kernel<T, U_DEEP / 2><<<grid, bs, smem, st>>>(src, dst, planes, n, s, row_sweep);
    const int rc = launch_status();
    if (rc) return rc;
    src = dst;
  }
  if (L >= 5) {
    const i64 groups = planes * (n >> 5);
    constexpr int WPB = last5_warps<T>();
    const unsigned g5 = (unsigned)((groups + WPB - 1) / WPB);
    iadrt_last5_kernel<T><<<g5, 32 * WPB, 0, st>>>(src, out, groups, (int)n);
    return launch_status();
  }
  return ADRT_GB300_OK;
}

template int iadrt_launch<float>(const float *, float *, i64, i64, void *, size_t, cudaStream_t);
template int iadrt_launch<double>(const double *, double *, i64, i64, void *, size_t, cudaStream_t);

}  // namespace adrtg
