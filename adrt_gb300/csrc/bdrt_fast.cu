// Register-level bdrt passes for float32, n = 128..1024 (the transpose of the
// fast forward's pass structure): pass 1 undoes the last five forward stages,
// pass 2 the first S = log2(n) - 5.
//
// The generic pass (bdrt.cu) holds a tile of 32 rows in shared memory and
// runs each transposed stage through it.  Here a pass's five stages run in
// registers, for the tiles where none of the reference's copy/zero rules
// applies.  Inside a tile every row is kept in the tile frame (the pass's
// pre-shift a' * i is applied only when member i is stored), so an undone
// stage at local output angle li is
//     left  [u] = A[u] + B[u]
//     right [u] = A[u + li] + B[u + li + 1]
// with A, B the rows of local angles 2 li and 2 li + 1 (src/adrt/
// adrt_cdefs_bdrt.hpp:56-116).  The reference's copy and zero rules (right =
// copy of A where B's offset is 2n-1, +0 beyond) are what these formulas give
// when every row reads as +0 at reference offsets >= 2n-1, except a row used
// as B, which must read -0 at exactly 2n-1 (A + (-0) == A bit for bit).  The
// sums beyond 2n-1 come out +0 by themselves, so in tiles that reach that
// offset ("edge" tiles) the inputs there are filled that way and, after each
// undone stage, the one position of each B row at offset 2n-1 is set to -0.
// Row (combo m, level J) sits at tile position u <-> reference offset
// c0 + u - a' m 2^J; in group 2t's frame (below) also + L1 m 2^(J-2).
//
//  group 2t (stages 4, 3, 2 undone; in a pass 2 of S < 5 stages, S - 2 of
//    them on per-section sets of rows): a lane holds the 8 angles 8 L1 + l3
//    at 8 consecutive positions (block b); operands to the right come from
//    lane+1 by shuffle.  The L1-dependent part of the shifts (4 L1, 2 L1, L1)
//    is left out, so level-2 combo h comes out L1 * h positions to the right
//    of its tile position; the exchange write puts it back.
//  exchange: level-2 rows (combo h, angle L1) in shared memory, 16-byte chunks
//    XOR-swizzled as in the forward kernel.
//  group 1t (stages 1, 0 undone): a warp owns combo h, a lane one 4-position
//    chunk of its 4 angle rows; it produces members 4h..4h+3.
//
// The last lane of a warp cannot see its right neighbour, so it only seeds
// lane 30: group-2t warps cover blocks 0..31 and 30..61, group-1t warps take
// 31 chunks per sweep.
#include "common.cuh"

namespace adrtg {
namespace bfast {

constexpr int W = 448;             // stored tile positions per CTA (56 blocks of 8)
constexpr int TWI = 496;           // input positions per tile (62 blocks)
constexpr int NT = 256;
constexpr int NCH = 128;           // exchange chunks per row
constexpr int RS = 4 * (NCH + 1);  // exchange row stride in floats (odd chunk count)
constexpr size_t SMEM = sizeof(float) * 32 * RS;
constexpr unsigned FULL = 0xffffffffu;
// Both passes are instantiated per n (128 .. 1024): their geometry is
// compile-time (offsets fold into the loads' and stores' immediate fields).
// cs: the bdrt buffer's row, 2n - 1 padded to 8 floats.
template <int NN>
struct Geo {
  static constexpr int n = NN, C = 2 * NN - 1, cs = (C + 7) / 8 * 8;
  static constexpr int S = NN == 1024 ? 5 : NN == 512 ? 4 : NN == 256 ? 3 : 2;  // stages of pass 2
  static constexpr int GS = S - 2;                                                // of them in group 2t
  static_assert(NN == (32 << S), "n = 128, 256, 512 or 1024");
};
static_assert(TWI * 32 <= 32 * RS && W * 32 <= 32 * RS, "stagings fit in the exchange buffer");

__device__ __forceinline__ int swz(int ch) { return ch ^ ((ch >> 3) & 1); }

__device__ __forceinline__ float4 ld4_cs(const float *p) { return __ldcs(reinterpret_cast<const float4 *>(p)); }

// Streaming 16-byte load under a predicate: `fill` where it is false, with
// no memory access (predicated in PTX, so the choice costs no branch).
__device__ __forceinline__ float4 ld4_cs_if(const float *p, bool pred, float4 fill) {
  float4 v;
  asm("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %5, 0;\n\tmov.b32 %0, %6;\n\tmov.b32 %1, %7;\n\t"
      "mov.b32 %2, %8;\n\tmov.b32 %3, %9;\n\t@q ld.global.cs.v4.f32 {%0, %1, %2, %3}, [%4];\n\t}"
      : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
      : "l"(p), "r"((unsigned)pred), "f"(fill.x), "f"(fill.y), "f"(fill.z), "f"(fill.w));
  return v;
}

// Right output of one undone stage over 8 positions: d[k] = A[k + s] +
// B[k + s + 1], where positions 8.. come from lane + 1.
template <int S>
__device__ __forceinline__ void right8(const float (&A)[8], const float (&B)[8], float (&d)[8]) {
  float ea[S > 0 ? S : 1], eb[S + 1];
#pragma unroll
  for (int k = 0; k < S; ++k) ea[k] = __shfl_down_sync(FULL, A[k], 1);
#pragma unroll
  for (int k = 0; k <= S; ++k) eb[k] = __shfl_down_sync(FULL, B[k], 1);
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const float a = k + S < 8 ? A[(k + S) & 7] : ea[(k + S - 8) & (S > 0 ? 7 : 0)];
    const float b = k + S + 1 < 8 ? B[(k + S + 1) & 7] : eb[k + S + 1 - 8];
    d[k] = add_rn(a, b);
  }
}

__device__ __forceinline__ void left8(const float (&A)[8], const float (&B)[8], float (&d)[8]) {
#pragma unroll
  for (int k = 0; k < 8; k += 2) add_rn2(A[k], A[k + 1], B[k], B[k + 1], d[k], d[k + 1]);
}

// Sets v[f - base] to -0 when this lane holds position f.
template <int K>
__device__ __forceinline__ void neg0_at(float (&v)[K], int f_minus_base) {
#pragma unroll
  for (int k = 0; k < K; ++k)
    if (f_minus_base == k) v[k] = -0.f;
}

// Group 2t: a[l3] = angle 8 L1 + l3 at the lane's 8 positions -> t2[h] =
// level-2 combo h (undone stages 4, 3, 2 give its bits, first as MSB).  In
// edge tiles (edge set) the B rows of levels 4 and 3 get their -0 at offset
// 2n-1: fresh position kc + m (2^J a' + 2^(J-2) L1) for combo m at level J,
// kc = 2n-1 - c0; base = 8 b.
template <int L1>
__device__ __forceinline__ void group2t_three(float (&a)[8][8], float (&t2)[8][8], bool edge, int kc, int ap,
                                              int base) {
  float t4[2][4][8];
  left8(a[0], a[1], t4[0][0]);
  right8<0>(a[0], a[1], t4[1][0]);
  left8(a[2], a[3], t4[0][1]);
  right8<1>(a[2], a[3], t4[1][1]);
  left8(a[4], a[5], t4[0][2]);
  right8<2>(a[4], a[5], t4[1][2]);
  left8(a[6], a[7], t4[0][3]);
  right8<3>(a[6], a[7], t4[1][3]);
  if (edge) {
#pragma unroll
    for (int c4 = 0; c4 < 2; ++c4) {
      const int f = kc + c4 * (16 * ap + 4 * L1) - base;
      neg0_at(t4[c4][1], f);
      neg0_at(t4[c4][3], f);
    }
  }
  float t3[2][2][2][8];
#pragma unroll
  for (int c4 = 0; c4 < 2; ++c4) {
    left8(t4[c4][0], t4[c4][1], t3[c4][0][0]);
    right8<0>(t4[c4][0], t4[c4][1], t3[c4][1][0]);
    left8(t4[c4][2], t4[c4][3], t3[c4][0][1]);
    right8<1>(t4[c4][2], t4[c4][3], t3[c4][1][1]);
  }
  if (edge) {
#pragma unroll
    for (int c4 = 0; c4 < 2; ++c4)
#pragma unroll
      for (int c3 = 0; c3 < 2; ++c3) neg0_at(t3[c4][c3][1], kc + (2 * c4 + c3) * (8 * ap + 2 * L1) - base);
  }
#pragma unroll
  for (int c4 = 0; c4 < 2; ++c4)
#pragma unroll
    for (int c3 = 0; c3 < 2; ++c3) {
      left8(t3[c4][c3][0], t3[c4][c3][1], t2[4 * c4 + 2 * c3]);
      right8<0>(t3[c4][c3][0], t3[c4][c3][1], t2[4 * c4 + 2 * c3 + 1]);
    }
}

// GS < 3 (a pass of S = GS + 2 stages, n = 32 * 2^S): the lane's 8 rows form
// 8 >> GS sets of 2^GS angle rows (one set per section), each undone by GS
// stages: the last GS steps of the three-stage case, with set s in place of
// the level-(GS+2) combo bits.  Combo h = 2^GS s + (bits of this pass); its
// frame shift is L1 (h mod 2^GS), and a combo's level-J position in the edge
// rule counts only this pass's bits.
template <int L1, int GS>
__device__ __forceinline__ void group2t(float (&a)[8][8], float (&t2)[8][8], bool edge, int kc, int ap, int base) {
  static_assert(GS >= 0 && GS <= 3, "group 2t undoes 0 to 3 stages");
  if constexpr (GS == 0) {
#pragma unroll
    for (int h = 0; h < 8; ++h)
#pragma unroll
      for (int k = 0; k < 8; ++k) t2[h][k] = a[h][k];
  } else if constexpr (GS == 1) {
#pragma unroll
    for (int st = 0; st < 4; ++st) {
      left8(a[2 * st], a[2 * st + 1], t2[2 * st]);
      right8<0>(a[2 * st], a[2 * st + 1], t2[2 * st + 1]);
    }
  } else if constexpr (GS == 2) {
    float t3[2][2][2][8];
#pragma unroll
    for (int st = 0; st < 2; ++st) {
      left8(a[4 * st], a[4 * st + 1], t3[st][0][0]);
      right8<0>(a[4 * st], a[4 * st + 1], t3[st][1][0]);
      left8(a[4 * st + 2], a[4 * st + 3], t3[st][0][1]);
      right8<1>(a[4 * st + 2], a[4 * st + 3], t3[st][1][1]);
    }
    if (edge) {
#pragma unroll
      for (int st = 0; st < 2; ++st)
#pragma unroll
        for (int c3 = 0; c3 < 2; ++c3) neg0_at(t3[st][c3][1], kc + c3 * (8 * ap + 2 * L1) - base);
    }
#pragma unroll
    for (int st = 0; st < 2; ++st)
#pragma unroll
      for (int c3 = 0; c3 < 2; ++c3) {
        left8(t3[st][c3][0], t3[st][c3][1], t2[4 * st + 2 * c3]);
        right8<0>(t3[st][c3][0], t3[st][c3][1], t2[4 * st + 2 * c3 + 1]);
      }
  } else {
    group2t_three<L1>(a, t2, edge, kc, ap, base);
  }
}

// Writes combo h of angle L1 back to its tile positions: fresh position
// 8b + k is tile position 8b + k - L1 h (L1 (h mod 2^GS) for GS < 3).  Lanes 30 and 31 write nothing (31
// is a seed, 30's second chunk would need 31's values; the other half of the
// CTA covers those blocks).
template <int L1, int GS>
__device__ __forceinline__ void put_exchange_t(float *xs, int b, bool wr, const float (&t2)[8][8]) {
#pragma unroll
  for (int h = 0; h < 8; ++h) {
    constexpr int dummy = 0;
    (void)dummy;
    const int sh = L1 * (h & ((1 << GS) - 1)), qh = sh >> 2, mh = sh & 3;
    float nx[4];
#pragma unroll
    for (int k = 0; k < 3; ++k)
      if (k < mh) nx[k] = __shfl_down_sync(FULL, t2[h][k], 1);
    float v[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = k + mh < 8 ? t2[h][(k + mh) & 7] : nx[(k + mh - 8) & 3];
    // A chunk this lane does not write goes to the row's padding chunk
    // (NCH), which no read touches: the stores need no branch.
    float *row = xs + (h * 4 + L1) * RS;
    const int x0 = 2 * b - qh;
    const int c0w = wr && x0 >= 0 ? swz(x0) : NCH, c1w = wr && x0 + 1 >= 0 ? swz(x0 + 1) : NCH;
    *reinterpret_cast<float4 *>(row + c0w * 4) = make_float4(v[0], v[1], v[2], v[3]);
    *reinterpret_cast<float4 *>(row + c1w * 4) = make_float4(v[4], v[5], v[6], v[7]);
  }
}

// Group-2t lane: warp w takes angle group L1 = w & 3; half w >> 2 covers
// blocks 0..31 or 30..61.
__device__ __forceinline__ int g2_block() {
  const int lane = threadIdx.x & 31;
  return (threadIdx.x >> 7) ? 30 + lane : lane;
}

template <int L1, int GS = 3>
__device__ __forceinline__ void group2t_and_exchange(float (&a)[8][8], float *xs, bool edge, int kc, int ap) {
  float t2[8][8];
  const int b = g2_block();
  group2t<L1, GS>(a, t2, edge, kc, ap, 8 * b);
  const int lane = threadIdx.x & 31;
  put_exchange_t<L1, GS>(xs, b, lane < 30, t2);
}

// Group 1t for one sweep: chunk ch of combo h's four angle rows -> members
// 4h + m at the chunk's positions, o[m][k].
// Edge tiles: the B rows of level 2 (odd angles) and level 1 get -0 at tile
// position kc + 4 a' h and kc + 2 a' (2h + c1).
__device__ __forceinline__ void group1t(const float *xs, int h, int ch, float (&o)[4][4], bool edge, int kc,
                                        int ap) {
  float x[4][4];
#pragma unroll
  for (int l1 = 0; l1 < 4; ++l1) {
    const float4 v = *reinterpret_cast<const float4 *>(xs + (h * 4 + l1) * RS + swz(ch) * 4);
    x[l1][0] = v.x; x[l1][1] = v.y; x[l1][2] = v.z; x[l1][3] = v.w;
  }
  if (edge) {
    const int f = kc + 4 * ap * h - 4 * ch;
    neg0_at(x[1], f);
    neg0_at(x[3], f);
  }
  const float n10 = __shfl_down_sync(FULL, x[1][0], 1);
  const float n20 = __shfl_down_sync(FULL, x[2][0], 1);
  const float n30 = __shfl_down_sync(FULL, x[3][0], 1);
  const float n31 = __shfl_down_sync(FULL, x[3][1], 1);
  // undo stage 1: u[side][li][k]
  float u[2][2][5];
  add_rn2(x[0][0], x[0][1], x[1][0], x[1][1], u[0][0][0], u[0][0][1]);
  add_rn2(x[0][2], x[0][3], x[1][2], x[1][3], u[0][0][2], u[0][0][3]);
  add_rn2(x[2][0], x[2][1], x[3][0], x[3][1], u[0][1][0], u[0][1][1]);
  add_rn2(x[2][2], x[2][3], x[3][2], x[3][3], u[0][1][2], u[0][1][3]);
  u[0][1][4] = add_rn(n20, n30);
  const float x1e[5] = {x[1][0], x[1][1], x[1][2], x[1][3], n10};
  const float x2e[5] = {x[2][0], x[2][1], x[2][2], x[2][3], n20};
  const float x3e[6] = {x[3][0], x[3][1], x[3][2], x[3][3], n30, n31};
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    u[1][0][k] = add_rn(x[0][k], x1e[k + 1]);
    u[1][1][k] = add_rn(x2e[k + 1], x3e[k + 2]);
  }
  if (edge) {
    neg0_at(u[0][1], kc + 4 * ap * h - 4 * ch);  // positions 0..4 (4: next chunk's first)
    float t[4] = {u[1][1][0], u[1][1][1], u[1][1][2], u[1][1][3]};
    neg0_at(t, kc + 2 * ap * (2 * h + 1) - 4 * ch);
#pragma unroll
    for (int k = 0; k < 4; ++k) u[1][1][k] = t[k];
  }
  u[1][1][4] = __shfl_down_sync(FULL, u[1][1][0], 1);
  // undo stage 0: member 4h + 2 side + s0
#pragma unroll
  for (int c1 = 0; c1 < 2; ++c1) {
    add_rn2(u[c1][0][0], u[c1][0][1], u[c1][1][0], u[c1][1][1], o[2 * c1][0], o[2 * c1][1]);
    add_rn2(u[c1][0][2], u[c1][0][3], u[c1][1][2], u[c1][1][3], o[2 * c1][2], o[2 * c1][3]);
#pragma unroll
    for (int k = 0; k < 4; ++k) o[2 * c1 + 1][k] = add_rn(u[c1][0][k], u[c1][1][k + 1]);
  }
}

// ---- pass 1 (the last five forward stages undone, L-1 .. L-5) --------------
// Input: the (4, 2n-1, n) array, angles 32 a' .. 32 a' + 31 (128 bytes per
// offset), a' < n / 32; output: bdrt buffer rows (a', member i) = level L-5
// angle a', section i, at reference offset u - a' i, row stride cs.
// A4 = a' mod 4 fixes each member's sub-chunk shift.
template <int A4, int NN>
__device__ __forceinline__ void pass1_store(const float (&o)[4][4][4], float *rows_ap, int ap, int c0, int h) {
  using G = Geo<NN>;
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    const int i = 4 * h + m;
    const int D = ap * i;
    constexpr int dummy = 0;
    (void)dummy;
    const int mi = (A4 * m) & 3;  // == D & 3
    float *row = rows_ap + i * G::cs;
    // Chunk X = ch + c0/4 - D/4 of the member's row; stored when it holds
    // stored tile positions and lies in [0, 2n-1): X in [0, ceil(C/4)).
    const int X0 = lane + (c0 >> 2) - (D >> 2);
#pragma unroll
    for (int it = 0; it < 4; ++it) {
      // The chunk to the right: lane + 1's, except for lane 30, whose right
      // neighbour (lane 31) only seeds; that chunk is lane 0's next sweep.
      float nx[4];
#pragma unroll
      for (int k = 0; k < 3; ++k)
        if (k < mi) {
          const float va = __shfl_sync(FULL, o[it][m][k], (lane + 1) & 31);
          const float vb = it < 3 ? __shfl_sync(FULL, o[it < 3 ? it + 1 : it][m][k], 0) : va;
          nx[k] = lane == 30 ? vb : va;
        }
      float v[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) v[k] = k + mi < 4 ? o[it][m][(k + mi) & 3] : nx[(k + mi - 4) & 3];
      const int X = X0 + 31 * it;
      // lane < 31 and 4 ch + mi < W, ch = 31 it + lane
      const int lane_lim = min(31, (W - mi + 3) / 4 - 31 * it);
      if (lane < lane_lim && (unsigned)X < (unsigned)((G::C + 3) / 4))
        *reinterpret_cast<float4 *>(row + 4 * X) = make_float4(v[0], v[1], v[2], v[3]);
    }
  }
}

template <int NN>
__global__ void __launch_bounds__(NT, 2) pass1_kernel(const float *__restrict__ in, float *__restrict__ buf,
                                                      int need) {
  using G = Geo<NN>;
  extern __shared__ __align__(16) float xs[];
  constexpr int n = G::n, C = G::C;
  const int c0 = (int)blockIdx.x * W;
  const int bq = (int)blockIdx.y;  // image * 4 + quadrant
  const int ap = (int)blockIdx.z;
  // Member i stores reference offsets >= c0 - 31 a': nothing needed here.
  if (c0 >= need + 31 * ap) return;
  const int kc = C - c0;
  const bool edge = kc < TWI;
  if (kc <= 0) {
    // The whole tile lies at frame positions >= 2n-1, where every input row
    // reads +0 (a B row -0 only at its marker): an undone stage's outputs at
    // u read inputs at >= u, and each is A + B with A = +0, so +0 (IEEE
    // +0 + -0 = +0) at every level, and the final members, which get no
    // marker, are +0.  Their stored offsets (u - a' i < 2n-1 for the members
    // shifted that far) get +0 without loading or computing.
    const float(&o)[4][4][4] = {};
    float *rows_z = buf + ((size_t)bq * n + (size_t)ap * 32) * G::cs;
    const int hz = threadIdx.x >> 5;
    switch (ap & 3) {
      case 0: pass1_store<0, NN>(o, rows_z, ap, c0, hz); break;
      case 1: pass1_store<1, NN>(o, rows_z, ap, c0, hz); break;
      case 2: pass1_store<2, NN>(o, rows_z, ap, c0, hz); break;
      default: pass1_store<3, NN>(o, rows_z, ap, c0, hz); break;
    }
    return;
  }
  const float *src = in + (size_t)bq * C * n + 32 * ap;
  // Stage the tile's 496 offsets x 32 angles (128-byte rows), chunk j of row
  // r at swizzled chunk j ^ ((r >> 3) & 7).  Offsets >= 2n-1 read +0, and
  // -0 for the odd angles (B rows) at 2n-1 itself.
  {
    const int r0 = threadIdx.x >> 3, j = threadIdx.x & 7;
    float4 v[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const int r = r0 + 32 * i;
      if (r < TWI) {
        const float z = r == kc ? -0.f : 0.f;
        v[i] = ld4_cs_if(src + (size_t)(c0 + r) * n + 4 * j, r < kc, make_float4(0.f, z, 0.f, z));
      }
    }
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const int r = r0 + 32 * i;
      if (r < TWI) *reinterpret_cast<float4 *>(xs + r * 32 + 4 * (j ^ ((r >> 3) & 7))) = v[i];
    }
  }
  __syncthreads();
  const int L1 = (threadIdx.x >> 5) & 3, b = g2_block();
  float a[8][8];
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const int r = 8 * b + k, sw = b & 7;
    const float4 v0 = *reinterpret_cast<const float4 *>(xs + r * 32 + 4 * ((2 * L1) ^ sw));
    const float4 v1 = *reinterpret_cast<const float4 *>(xs + r * 32 + 4 * ((2 * L1 + 1) ^ sw));
    a[0][k] = v0.x; a[1][k] = v0.y; a[2][k] = v0.z; a[3][k] = v0.w;
    a[4][k] = v1.x; a[5][k] = v1.y; a[6][k] = v1.z; a[7][k] = v1.w;
  }
  __syncthreads();  // the exchange overlays the staging
  switch (L1) {
    case 0: group2t_and_exchange<0>(a, xs, edge, kc, ap); break;
    case 1: group2t_and_exchange<1>(a, xs, edge, kc, ap); break;
    case 2: group2t_and_exchange<2>(a, xs, edge, kc, ap); break;
    default: group2t_and_exchange<3>(a, xs, edge, kc, ap); break;
  }
  __syncthreads();
  const int h = threadIdx.x >> 5;
  float o[4][4][4];
#pragma unroll
  for (int it = 0; it < 4; ++it) group1t(xs, h, 31 * it + (threadIdx.x & 31), o[it], edge, kc, ap);
  float *rows_ap = buf + ((size_t)bq * n + (size_t)ap * 32) * G::cs;
  switch (ap & 3) {
    case 0: pass1_store<0, NN>(o, rows_ap, ap, c0, h); break;
    case 1: pass1_store<1, NN>(o, rows_ap, ap, c0, h); break;
    case 2: pass1_store<2, NN>(o, rows_ap, ap, c0, h); break;
    default: pass1_store<3, NN>(o, rows_ap, ap, c0, h); break;
  }
}

// ---- pass 2 (the first S = L-5 forward stages undone, S-1 .. 0) ----------
// Input: bdrt buffer rows of level S (2^S angles x 32 sections, row angle *
// 32 + section, row stride cs); a CTA takes the 32 rows of sections
// (32 >> S) R .. (32 >> S) R + (32 >> S) - 1, all angles; output: (4, 2n-1, n)
// sections 32 R .. 32 R + 31 (128 bytes per offset), staged in shared memory
// (chunk h of row p at chunk h ^ ((p >> 2) & 7)).
template <int NN>
__global__ void __launch_bounds__(NT, 2) pass2_kernel(const float *__restrict__ buf, float *__restrict__ out,
                                                      int need) {
  using G = Geo<NN>;
  extern __shared__ __align__(16) float xs[];
  constexpr int n = G::n, C = G::C, cs = G::cs, S = G::S, GS = G::GS;
  const int c0 = (int)blockIdx.x * W;
  if (c0 >= need) return;
  const int bq = (int)blockIdx.y;
  const int r = (int)blockIdx.z;
  const int L1 = (threadIdx.x >> 5) & 3, b = g2_block();
  const int kc = C - c0;
  const bool edge = kc < TWI;
  const int e0 = 8 * b;  // lane's first tile position
  const float *src = buf + (size_t)bq * n * cs + c0 + e0;
  // Row l3 of this lane: set l3 >> GS (section (32 >> S) r + that), angle
  // 2^GS L1 + (l3 mod 2^GS); at n = 1024 angle 8 L1 + l3 of section r.
  // Chunks that start at or past 2n-1 read +0 without a memory access (the
  // last chunk of a row ends exactly at 2n-1); offset 2n-1 itself is set
  // below: -0 on the odd angles (B rows), +0 on the even ones.
  float a[8][8];
#pragma unroll
  for (int l3 = 0; l3 < 8; ++l3) {
    const int angle = (L1 << GS) + (l3 & ((1 << GS) - 1)), section = (32 >> S) * r + (l3 >> GS);
    const float *p = src + (size_t)(angle * 32 + section) * cs;
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 v0 = ld4_cs_if(p, e0 < kc, zero), v1 = ld4_cs_if(p + 4, e0 + 4 < kc, zero);
    a[l3][0] = v0.x; a[l3][1] = v0.y; a[l3][2] = v0.z; a[l3][3] = v0.w;
    a[l3][4] = v1.x; a[l3][5] = v1.y; a[l3][6] = v1.z; a[l3][7] = v1.w;
  }
  if (edge) {
#pragma unroll
    for (int l3 = 0; l3 < 8; ++l3)
#pragma unroll
      for (int k = 0; k < 8; ++k)
        if (e0 + k == kc) a[l3][k] = ((GS > 0 ? l3 : L1) & 1) ? -0.f : 0.f;
  }
  switch (L1) {
    case 0: group2t_and_exchange<0, GS>(a, xs, edge, kc, 0); break;
    case 1: group2t_and_exchange<1, GS>(a, xs, edge, kc, 0); break;
    case 2: group2t_and_exchange<2, GS>(a, xs, edge, kc, 0); break;
    default: group2t_and_exchange<3, GS>(a, xs, edge, kc, 0); break;
  }
  __syncthreads();
  const int h = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float o[4][4][4];
#pragma unroll
  for (int it = 0; it < 4; ++it) group1t(xs, h, 31 * it + lane, o[it], edge, kc, 0);
  __syncthreads();  // the output staging overlays the exchange
  // Chunks past the tile (and lane 31's, a seed) go to a spare slot past the
  // staged rows (float W * 32), which no read touches: no branch.
  static_assert(W * 32 + 4 <= 32 * RS, "spare staging slot inside the buffer");
#pragma unroll
  for (int it = 0; it < 4; ++it) {
    const int ch = 31 * it + lane;
    const bool st = lane < 31 && ch < W / 4;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int p = 4 * ch + k;
      *reinterpret_cast<float4 *>(xs + (st ? p * 32 + 4 * (h ^ (ch & 7)) : W * 32)) =
          make_float4(o[it][0][k], o[it][1][k], o[it][2][k], o[it][3][k]);
    }
  }
  __syncthreads();
  const int p0 = threadIdx.x >> 3, j = threadIdx.x & 7;
  float *dst = out + (size_t)bq * C * n + 32 * r + 4 * j;
  const int lim = min(min(C, need) - c0, W);
  // Rows p < W are inside the staging: read them all, store the live ones.
#pragma unroll
  for (int i = 0; i < W / 32; ++i) {
    const int p = p0 + 32 * i;
    const float4 v = *reinterpret_cast<const float4 *>(xs + p * 32 + 4 * (j ^ ((p >> 2) & 7)));
    if (p < lim) __stcs(reinterpret_cast<float4 *>(dst + (size_t)(c0 + p) * n), v);
  }
}

}  // namespace bfast

// Column tiles: pass 2 covers offsets [0, 2n-1); pass 1 tile positions
// [0, 2n-1 + 31 (n/32 - 1)) (member i of input angle group a' is stored
// a' i positions to the left).
static int pass_tiles(i64 n, bool first) {
  const i64 span = 2 * n - 1 + (first ? 31 * (n / 32 - 1) : 0);
  return (int)((span + bfast::W - 1) / bfast::W);
}

template <int NN>
static int launch_pass1(const float *in, float *buf, i64 batch, i64 need, cudaStream_t st) {
  using G = bfast::Geo<NN>;
  static std::atomic<unsigned long long> configured{0};
  if (const int rc = smem_limit_once((const void *)bfast::pass1_kernel<NN>, bfast::SMEM, configured)) return rc;
  const int tiles = pass_tiles(NN, true);
  // Grid y counts (image, quadrant) pairs: launches of at most 16383 images.
  for (i64 b0 = 0; b0 < batch; b0 += 16383) {
    const i64 nb = batch - b0 < 16383 ? batch - b0 : 16383;
    const dim3 grid((unsigned)tiles, (unsigned)(nb * 4), (unsigned)(NN / 32));
    bfast::pass1_kernel<NN><<<grid, bfast::NT, bfast::SMEM, st>>>(in + b0 * 4 * G::C * NN,
                                                                    buf + b0 * 4 * NN * G::cs, (int)need);
    if (const int rc = launch_status()) return rc;
  }
  return ADRT_GB300_OK;
}

template <int NN>
static int launch_pass2(const float *buf, float *out, i64 batch, i64 need, cudaStream_t st) {
  using G = bfast::Geo<NN>;
  static std::atomic<unsigned long long> configured{0};
  if (const int rc = smem_limit_once((const void *)bfast::pass2_kernel<NN>, bfast::SMEM, configured)) return rc;
  const int tiles = pass_tiles(NN, false);
  for (i64 b0 = 0; b0 < batch; b0 += 16383) {
    const i64 nb = batch - b0 < 16383 ? batch - b0 : 16383;
    const dim3 grid((unsigned)tiles, (unsigned)(nb * 4), (unsigned)(NN / 32));
    bfast::pass2_kernel<NN><<<grid, bfast::NT, bfast::SMEM, st>>>(buf + b0 * 4 * NN * G::cs,
                                                                    out + b0 * 4 * G::C * NN, (int)need);
    if (const int rc = launch_status()) return rc;
  }
  return ADRT_GB300_OK;
}

// The bdrt buffer's rows are padded to 8 floats (cs = (2n - 1 + 7) / 8 * 8).
int bdrt_fast_pass1(const float *in, float *buf, i64 batch, i64 n, i64 cs, i64 need, cudaStream_t st) {
  if (cs != (2 * n - 1 + 7) / 8 * 8) return ADRT_GB300_ERR_SHAPE;
  switch (n) {
    case 128: return launch_pass1<128>(in, buf, batch, need, st);
    case 256: return launch_pass1<256>(in, buf, batch, need, st);
    case 512: return launch_pass1<512>(in, buf, batch, need, st);
    case 1024: return launch_pass1<1024>(in, buf, batch, need, st);
  }
  return ADRT_GB300_ERR_SHAPE;
}

int bdrt_fast_pass2(const float *buf, float *out, i64 batch, i64 n, i64 cs, i64 need, cudaStream_t st) {
  if (cs != (2 * n - 1 + 7) / 8 * 8) return ADRT_GB300_ERR_SHAPE;
  switch (n) {
    case 128: return launch_pass2<128>(buf, out, batch, need, st);
    case 256: return launch_pass2<256>(buf, out, batch, need, st);
    case 512: return launch_pass2<512>(buf, out, batch, need, st);
    case 1024: return launch_pass2<1024>(buf, out, batch, need, st);
  }
  return ADRT_GB300_ERR_SHAPE;
}

}  // namespace adrtg
