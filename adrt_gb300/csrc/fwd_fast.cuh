// Device code of the fast forward ADRT for float32, n = 64..1024, in two
// passes: pass A the first S = log2(n) - 5 stages (1 to 5), pass B the last
// five.  The per-tile functions the standalone pass kernels
// (adrt_fwd_fast.cu) and the ragged persistent kernel (adrt_fwd.cu) run.
//
// Same decomposition as adrt_fwd.cu: a pass merges 32 members (rows in pass A,
// row groups in pass B) at input angle a' into 32 angles, member i loaded with
// the pre-shift a'*i so that only residual shifts remain inside the tile.
// This kernel keeps those five stages out of shared memory as much as the
// hardware allows:
//
//  group 1 (stages 0-1; stage 0 only in a one-stage pass A): each lane owns
//    4 members x 4 consecutive positions
//    (one 16-byte chunk per member, loaded straight from global memory with
//    128-bit loads).  A warp sweeps the tile in iterations of 32 chunks; the
//    few operands that cross a chunk boundary come from the neighbouring lane
//    by shuffle, and lane 0 takes them from lane 31's previous iteration.
//  exchange: the 4 angles x 32 positions of each member quad go to shared
//    memory (16-byte stores, XOR-swizzled, rows padded to an odd chunk count).
//  group 2 (stages 2-4): each lane owns 8 combos x 8 positions of one angle
//    l1 of group 1.  Combo h is read pre-shifted by l1*h, which leaves a fresh
//    3-stage butterfly with shifts <= 4; boundary operands come from lane-1.
//    A pass A of S < 5 stages runs S - 2 of them on sets of combos.
//
// Operands whose reference offset is negative are "absent" (the reference
// copies instead of adding).  They are loaded as -0.0f, and e + (-0) == e bit
// for bit, so the kernel adds unconditionally and still reproduces the copy.
// Inductively every value at a negative offset stays -0.0f.
#pragma once

#include "common.cuh"

namespace adrtg {
namespace fast {

constexpr int W = 480;            // output offsets per tile
constexpr int HALO = 32;          // positions left of the outputs
constexpr int TW = W + HALO;      // 512 tile positions
constexpr int NCH = TW / 4;       // 128 chunks of 4 positions
constexpr int RS = 4 * (NCH + 1); // exchange row stride in floats (odd chunk count)
constexpr int NT = 256;           // threads per CTA
constexpr int N = 1024;
// After five stages a row group's values are non-zero only at offsets below
// n + 31 (shifts reach 31); beyond that every value is +0, the sum of the
// zero padding.  The intermediate rows end there (rounded up to 8 floats) and
// pass B reads anything past the row end as +0.  Pass A computes the tiles
// that hold those offsets; in its last tile only the iterations and warps
// that reach a stored offset run.
constexpr int A_TILES = (N + 31 + W - 1) / W;  // 3
constexpr int CS = (N + 31 + 7) / 8 * 8;       // 1056: intermediate row stride (128-byte multiple)
static_assert(A_TILES == 3 && CS == 1056, "n = 1024 pass A geometry");
constexpr unsigned FULL = 0xffffffffu;

// Pass A for n = 32 * 2^S (S = 2..5): the first S stages, after which the
// image's 32 row groups of 2^S rows each have 2^S angles.  A CTA still owns
// 32 consecutive image rows (or columns), i.e. 32 >> S row groups (one at
// S = 5, eight at S = 2), and the intermediate keeps each row's support:
// offsets below n + 2^S - 1, rounded up to 8 floats.
template <int S>
struct PassA {
  static_assert(S >= 1 && S <= 5, "pass A runs 1 to 5 stages");
  static constexpr int n = 32 << S;
  static constexpr int CS = (n + n / 32 - 1 + 7) / 8 * 8;  // 1056, 528, 264, 136, 72
  static constexpr int TILES = (CS + W - 1) / W;            // 3, 2, 1, 1, 1
  static constexpr int GS = S >= 2 ? S - 2 : 0;             // stages of group 2
  static constexpr int G1 = S >= 2 ? 2 : 1;                 // stages of group 1
};

// Sweep iterations pass A's column tile ct needs for n = 32 * 2^S (the
// compile-time form of sweep_iters(needed_positions(...))).
template <int S>
constexpr int pass_a_nit(int ct) {
  const int live = PassA<S>::CS - ct * W < W ? PassA<S>::CS - ct * W : W;
  const int it = (((live + 7) & ~7) + HALO + 127) >> 7;
  return it < NCH / 32 ? it : NCH / 32;
}
constexpr size_t SMEM = sizeof(float) * 32 * RS;
static_assert(W * 32 <= 32 * RS, "pass B output staging must fit in the exchange buffer");

__device__ __forceinline__ int swz(int ch) { return ch ^ ((ch >> 3) & 1); }

// Called by every thread of a tile once, after its group-1 loads have been
// issued and before the tile's first barrier (or at the start of a tile that
// only stores zeros): a persistent caller fetches its next work item there,
// where the fetch's latency overlaps the other warps' group-1 work.
struct NoHook {
  __device__ __forceinline__ void operator()() const {}
};

__device__ __forceinline__ float4 ld4_stream(const float *p) {
  return __ldcs(reinterpret_cast<const float4 *>(p));
}

__device__ __forceinline__ void st8(float *p, const float (&v)[8]) {
  asm volatile("st.global.v8.f32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"l"(p), "f"(v[0]), "f"(v[1]),
               "f"(v[2]), "f"(v[3]), "f"(v[4]), "f"(v[5]), "f"(v[6]), "f"(v[7])
               : "memory");
}


// Value of `cur` held by the lane D below (the previous chunk).  Lanes whose
// previous chunk was handled in the previous iteration (lane < D) receive the
// `saved` copy from lanes 32-D..31.
template <int D>
__device__ __forceinline__ float prev_chunk(float cur, float saved, int lane) {
  const float send = (lane >= 32 - D) ? saved : cur;
  return __shfl_sync(FULL, send, (lane - D) & 31);
}

// Tile positions (from tbase) that group 1 must produce when the tile stores
// `live` offsets from c0: group 2's block b reads positions up to 8b + 39,
// the position of its own last output.
__device__ __forceinline__ int needed_positions(int live) { return ((live + 7) & ~7) + HALO; }

// Group-1 sweep iterations (128 positions each) covering `pos` positions.
__device__ __forceinline__ int sweep_iters(int pos) {
  const int it = (pos + 127) >> 7;
  return it < NCH / 32 ? it : NCH / 32;
}


// ---------------------------------------------------------------------------
// Group 1: stages 0 and 1 on one member quad, 4 positions.
//   m[jj][k]  member jj of the quad, position k
//   o[l1][k]  angle l1 = 2*p0 + p1 of the quad's combo, position k
// The neighbour values come through `prev`.
// ---------------------------------------------------------------------------
struct G1Tail {
  float m1, m3;          // last position of members 1 and 3
  float s10, s11a, s11b; // stage-0 odd-pair outputs: li=0 pos 3, li=1 pos 3, li=1 pos 2
};

// ST = 1 (pass A at n = 64, one stage): stage 0 only, o[2 pair + p] =
// pair (0,1) or (2,3) at angle p.
template <int D, int ST = 2>
__device__ __forceinline__ void group1_compute(const float (&m)[4][4], float (&o)[4][4],
                                               G1Tail &saved, int lane) {
  // stage 0: pairs (0,1) and (2,3); shift p for the odd member.
  const float pm1 = prev_chunk<D>(m[1][3], saved.m1, lane);
  const float pm3 = prev_chunk<D>(m[3][3], saved.m3, lane);
  saved.m1 = m[1][3];
  saved.m3 = m[3][3];
  float s0[2][2][4];  // [pair][p][k]
#pragma unroll
  for (int k = 0; k < 4; k += 2) {
    add_rn2(m[0][k], m[0][k + 1], m[1][k], m[1][k + 1], s0[0][0][k], s0[0][0][k + 1]);
    add_rn2(m[2][k], m[2][k + 1], m[3][k], m[3][k + 1], s0[1][0][k], s0[1][0][k + 1]);
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    s0[0][1][k] = add_rn(m[0][k], k ? m[1][k - 1] : pm1);
    s0[1][1][k] = add_rn(m[2][k], k ? m[3][k - 1] : pm3);
  }
  if constexpr (ST == 1) {
#pragma unroll
    for (int l = 0; l < 4; ++l)
#pragma unroll
      for (int k = 0; k < 4; ++k) o[l][k] = s0[l >> 1][l & 1][k];
  } else {
    // stage 1: combo 0 (pair 0) + combo 1 (pair 1) shifted by li + p.
    const float q0 = prev_chunk<D>(s0[1][0][3], saved.s10, lane);   // li=0, position -1
    const float q1 = prev_chunk<D>(s0[1][1][3], saved.s11a, lane);  // li=1, position -1
    const float q2 = prev_chunk<D>(s0[1][1][2], saved.s11b, lane);  // li=1, position -2
    saved.s10 = s0[1][0][3];
    saved.s11a = s0[1][1][3];
    saved.s11b = s0[1][1][2];
    // ext[li][k + 2] = odd combo value at position k (k in [-2, 4))
    float ext0[6], ext1[6];
    ext0[0] = 0.f;  // never used (shift <= 1 for li = 0)
    ext0[1] = q0;
    ext1[0] = q2;
    ext1[1] = q1;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      ext0[k + 2] = s0[1][0][k];
      ext1[k + 2] = s0[1][1][k];
    }
#pragma unroll
    for (int k = 0; k < 4; k += 2) {
      add_rn2(s0[0][0][k], s0[0][0][k + 1], ext0[k + 2], ext0[k + 3], o[0][k], o[0][k + 1]);  // li=0, p=0
      add_rn2(s0[0][1][k], s0[0][1][k + 1], ext1[k], ext1[k + 1], o[3][k], o[3][k + 1]);      // li=1, p=1
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      o[1][k] = add_rn(s0[0][0][k], ext0[k + 1]);      // li=0, p=1
      o[2][k] = add_rn(s0[0][1][k], ext1[k + 1]);      // li=1, p=0
    }
  }
}

// Exchange row of member quad h at group-1 angle l1.  Pass A uses l1-major
// rows (its column-mode writes then spread over banks); pass B writes in place
// over its own input rows, member 4h + l1.
template <int XL>
__device__ __forceinline__ int xrow(int h, int l1) { return XL == 0 ? l1 * 8 + h : 4 * h + l1; }

template <int XL = 0>
__device__ __forceinline__ void put_exchange(float *xs, int mq, int ch, const float (&o)[4][4]) {
#pragma unroll
  for (int l1 = 0; l1 < 4; ++l1) {
    float4 v = make_float4(o[l1][0], o[l1][1], o[l1][2], o[l1][3]);
    *reinterpret_cast<float4 *>(xs + xrow<XL>(mq, l1) * RS + swz(ch) * 4) = v;
  }
}

// Chunk load with a fill value: a lane whose chunk lies outside [0, lim)
// gets the fill (-0 before the start: absent operands; +0 past the end: the
// zero padding and its sums) and issues no memory access.  Predicated in PTX
// so that the three cases cost no divergent branches.  Cache modes: LD_CA
// default (the image, which all four quadrants read); LD_CS evict-first (data
// read once); LD_CG L2 only (data other CTAs of the same launch wrote).
enum { LD_CA = 0, LD_CS = 1, LD_CG = 2 };
template <int MODE>
__device__ __forceinline__ float4 ld4_fill(const float *p, int g0, int lim) {
  float4 v;
  const float fill = __int_as_float(g0 & (int)0x80000000);
  const unsigned in = (unsigned)g0 < (unsigned)lim;
#define ADRTG_LD4_FILL(OP)                                                                                      \
  asm("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %5, 0;\n\tmov.b32 %0, %6;\n\tmov.b32 %1, %6;\n\t"               \
      "mov.b32 %2, %6;\n\tmov.b32 %3, %6;\n\t@q " OP " {%0, %1, %2, %3}, [%4];\n\t}"                           \
      : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)                                                             \
      : "l"(p), "r"(in), "f"(fill))
  if (MODE == LD_CS) ADRTG_LD4_FILL("ld.global.cs.v4.f32");
  else if (MODE == LD_CG) ADRTG_LD4_FILL("ld.global.cg.v4.f32");
  else ADRTG_LD4_FILL("ld.global.v4.f32");
#undef ADRTG_LD4_FILL
  return v;
}

// Loads of group 1 are all issued before any of them is consumed: a warp
// holds its whole sweep (4-5 chunks per member) in registers, so the load
// latency is paid once per tile rather than once per iteration.

// Pass A, quadrants 0 and 3: members are image rows, positions run along the
// row from its right end (offset c <-> column n-1-c).  Warp = member quad.
template <int NI, int NIT = 0>
__device__ __forceinline__ void group1_passA_rows(const float *img, int q, int r, int tbase, int pos,
                                                  float *xs) {
  const int lane = threadIdx.x & 31, mq = threadIdx.x >> 5;
  constexpr int IT = NCH / 32;
  const int nit = NIT ? NIT : sweep_iters(pos);
  float4 raw[IT][4];
#pragma unroll
  for (int it = 0; it < IT; ++it) {
    if (it >= nit) break;
    const int ref0 = tbase + 4 * (it * 32 + lane);
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) {
      const int R0 = 32 * r + 4 * mq + jj;
      const int irow = (q == 0) ? R0 : (NI - 1 - R0);
      raw[it][jj] = ld4_fill<LD_CA>(img + irow * NI + (NI - 4 - ref0), ref0, NI);
    }
  }
  G1Tail saved{-0.f, -0.f, -0.f, -0.f, -0.f};
#pragma unroll
  for (int it = 0; it < IT; ++it) {
    if (it >= nit) break;
    float m[4][4];
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) {
      m[jj][0] = raw[it][jj].w; m[jj][1] = raw[it][jj].z;
      m[jj][2] = raw[it][jj].y; m[jj][3] = raw[it][jj].x;
    }
    float o[4][4];
    group1_compute<1, NI == 64 ? 1 : 2>(m, o, saved, lane);
    put_exchange(xs, mq, it * 32 + lane, o);
  }
}

// Pass A, quadrants 1 and 2: members are image columns, positions run down
// (q2) or up (q1) the columns.  A lane loads one 16-byte row segment (4
// members) per position and transposes in registers.  Lanes: mq = lane & 7,
// position group = lane >> 3; warp w sweeps chunks [16w - 1, 16w + 16), the
// first one only to seed the boundary values.  Warps whose chunks start at or
// beyond `pos` have nothing to produce.
template <int NI>
__device__ __forceinline__ void group1_passA_cols(const float *img, int q, int r, int tbase, int pos,
                                                  float *xs) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (64 * w >= pos) return;
  const int mq = lane & 7, pg = lane >> 3;
  constexpr int IT = 5;
  float4 raw[IT][4];
#pragma unroll
  for (int it = 0; it < IT; ++it) {
    const int ch = 16 * w - 1 + 4 * it + pg;
    const bool live = ch <= 16 * w + 15;
    const int ref0 = tbase + 4 * ch;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int ref = ref0 + k;
      const int irow = (q == 2) ? ref : (NI - 1 - ref);
      // A chunk past this warp's range only seeds nothing: load it as absent.
      raw[it][k] = ld4_fill<LD_CA>(img + irow * NI + 32 * r + 4 * mq, live ? ref : -1, NI);
    }
  }
  G1Tail saved{-0.f, -0.f, -0.f, -0.f, -0.f};
#pragma unroll
  for (int it = 0; it < IT; ++it) {
    const int ch = 16 * w - 1 + 4 * it + pg;
    const bool live = ch <= 16 * w + 15;
    float m[4][4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      m[0][k] = raw[it][k].x; m[1][k] = raw[it][k].y;
      m[2][k] = raw[it][k].z; m[3][k] = raw[it][k].w;
    }
    float o[4][4];
    group1_compute<8, NI == 64 ? 1 : 2>(m, o, saved, lane);
    if (live && ch >= 16 * w) put_exchange(xs, mq, ch, o);
  }
}

// Pass B: members are the 32 row groups of pass A's output at angle a'.
// Member j's window is shifted by a'*j; a'*j mod 4 = (a' mod 4)*jj mod 4 is a
// compile-time constant per A4 = a' mod 4, so the realignment is a fixed
// selection of this lane's and the previous lane's 16-byte chunk.  Slot 0 of
// `raw` holds the chunk that precedes the first one, seeding lane 0.
// NIT: sweep iterations when known at compile time (full tiles), else 0;
// LD: cache mode of the intermediate's loads.
template <int A4, int NIT, int LD>
__device__ __forceinline__ void group1_passB(const float *src, int ap, int tbase, int pos, float *xs,
                                             size_t mstride, int cs) {
  const int lane = threadIdx.x & 31, mq = threadIdx.x >> 5;
  constexpr int IT = NCH / 32;
  const int nit = NIT ? NIT : sweep_iters(pos);
  float4 raw[IT + 1][4];
  // Member j's sweep starts at gb_j = tbase - 4 floor(a' j / 4), which falls
  // with j: when the warp's first member ends inside the row and its last
  // starts past the first chunk, every load of the warp is inside (one
  // warp-uniform branch for all four members).
  const int gb_hi = tbase - 4 * ((ap * (4 * mq)) >> 2), gb_lo = tbase - 4 * ((ap * (4 * mq + 3)) >> 2);
  if (gb_lo >= 4 && gb_hi + 128 * nit <= cs) {
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) {
      const int j = 4 * mq + jj;
      const float *row = src + (size_t)j * mstride;
      const int gb = tbase - 4 * ((ap * j) >> 2);
#pragma unroll
      for (int it = 0; it <= IT; ++it) {
        if (it > nit) break;
        const int g0 = it == 0 ? gb - 4 : gb + 4 * ((it - 1) * 32 + lane);
        raw[it][jj] = LD == LD_CG ? __ldcg(reinterpret_cast<const float4 *>(row + g0)) : ld4_stream(row + g0);
      }
    }
  } else {
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) {
      const int j = 4 * mq + jj;
      const float *row = src + (size_t)j * mstride;
      const int gb = tbase - 4 * ((ap * j) >> 2);
#pragma unroll
      for (int it = 0; it <= IT; ++it) {
        if (it > nit) break;
        // slot 0: the chunk before chunk 0 (only lane 31's copy is used)
        const int g0 = it == 0 ? gb - 4 : gb + 4 * ((it - 1) * 32 + lane);
        raw[it][jj] = ld4_fill<LD>(row + g0, g0, cs);
      }
    }
  }
  G1Tail saved{-0.f, -0.f, -0.f, -0.f, -0.f};
#pragma unroll
  for (int it = 1; it <= IT; ++it) {
    if (it > nit) break;
    float m[4][4];
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) {
      const float wv[4] = {raw[it][jj].x, raw[it][jj].y, raw[it][jj].z, raw[it][jj].w};
      const float pv[4] = {raw[it - 1][jj].x, raw[it - 1][jj].y, raw[it - 1][jj].z, raw[it - 1][jj].w};
      const int vsh = (A4 * jj) & 3;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        if (k >= vsh) m[jj][k] = wv[k - vsh];
        else m[jj][k] = prev_chunk<1>(wv[4 - vsh + k], pv[4 - vsh + k], lane);
      }
    }
    float o[4][4];
    group1_compute<1>(m, o, saved, lane);
    put_exchange(xs, mq, (it - 1) * 32 + lane, o);
  }
}


// Group 2's three stages (the fresh butterfly after the pre-shift).
__device__ __forceinline__ void group2_stage_a(const float (&r)[8][8], float (&t0)[4][2][8]) {
  // stage a: pairs (2P, 2P+1), shift p.
#pragma unroll
  for (int P = 0; P < 4; ++P) {
    const float pv = __shfl_up_sync(FULL, r[2 * P + 1][7], 1);
#pragma unroll
    for (int k = 0; k < 8; k += 2)
      add_rn2(r[2 * P][k], r[2 * P][k + 1], r[2 * P + 1][k], r[2 * P + 1][k + 1], t0[P][0][k], t0[P][0][k + 1]);
#pragma unroll
    for (int k = 0; k < 8; ++k) t0[P][1][k] = add_rn(r[2 * P][k], k ? r[2 * P + 1][k - 1] : pv);
  }
}

__device__ __forceinline__ void group2_stage_b(const float (&t0)[4][2][8], float (&t1)[2][4][8]) {
  // stage b: combos (2Q, 2Q+1), li in {0,1}, shift li + p.
#pragma unroll
  for (int Q = 0; Q < 2; ++Q) {
#pragma unroll
    for (int li = 0; li < 2; ++li) {
      float ext[10];  // ext[k + 2] = odd value at position k, k in [-2, 8)
      ext[0] = __shfl_up_sync(FULL, t0[2 * Q + 1][li][6], 1);
      ext[1] = __shfl_up_sync(FULL, t0[2 * Q + 1][li][7], 1);
#pragma unroll
      for (int k = 0; k < 8; ++k) ext[k + 2] = t0[2 * Q + 1][li][k];
#pragma unroll
      for (int p = 0; p < 2; ++p) {
        const int sh = li + p;
        if (sh % 2 == 0) {
#pragma unroll
          for (int k = 0; k < 8; k += 2)
            add_rn2(t0[2 * Q][li][k], t0[2 * Q][li][k + 1], ext[k + 2 - sh], ext[k + 3 - sh], t1[Q][2 * li + p][k],
                    t1[Q][2 * li + p][k + 1]);
        } else {
#pragma unroll
          for (int k = 0; k < 8; ++k) t1[Q][2 * li + p][k] = add_rn(t0[2 * Q][li][k], ext[k + 2 - sh]);
        }
      }
    }
  }
}

__device__ __forceinline__ void group2_stage_c(const float (&t1)[2][4][8], float (&out)[8][8]) {
  // stage c: li in [0,4), shift li + p.
#pragma unroll
  for (int li = 0; li < 4; ++li) {
    float ext[12];  // ext[k + 4] = odd value at position k, k in [-4, 8)
#pragma unroll
    for (int k = 0; k < 4; ++k) ext[k] = __shfl_up_sync(FULL, t1[1][li][4 + k], 1);
#pragma unroll
    for (int k = 0; k < 8; ++k) ext[k + 4] = t1[1][li][k];
#pragma unroll
    for (int p = 0; p < 2; ++p) {
      const int sh = li + p;
      if (sh % 2 == 0) {
#pragma unroll
        for (int k = 0; k < 8; k += 2)
          add_rn2(t1[0][li][k], t1[0][li][k + 1], ext[k + 4 - sh], ext[k + 5 - sh], out[2 * li + p][k],
                  out[2 * li + p][k + 1]);
      } else {
#pragma unroll
        for (int k = 0; k < 8; ++k) out[2 * li + p][k] = add_rn(t1[0][li][k], ext[k + 4 - sh]);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Group 2: stages 2-4 for angle L1 of group 1; lane owns 8 combos x 8
// positions (block b).  Returns out[l][k], l = local angle (tile angle 8*L1 + l).
// GS < 3 (pass A with S = GS + 2 stages): the 8 combos form 8 >> GS
// independent sets of 2^GS (one per row group), each merged by GS stages:
// combo h is pre-shifted by L1 * (h mod 2^GS), and out[e] holds set
// e >> GS at local angle e mod 2^GS (row-group angle 2^GS * L1 + that).
// ---------------------------------------------------------------------------
template <int L1, int XL = 0, int GS = 3>
__device__ __forceinline__ void group2_compute(const float *xs, int b, bool active,
                                               float (&out)[8][8]) {
  static_assert(GS >= 0 && GS <= 3, "group 2 runs 0 to 3 stages");
  const int bl = active ? b : W / 8 - 1;
  float r[8][8];
#pragma unroll
  for (int h = 0; h < 8; ++h) {
    const int hl = h & ((1 << GS) - 1);
    const int qh = (L1 * hl) >> 2, mh = (L1 * hl) & 3;
    const float *row = xs + xrow<XL>(h, L1) * RS;
    // Every lane reads, without a branch: the two lanes past the tile (half 1,
    // lanes 30-31) at the last block, in bounds (chunks <= 127 of 129); their
    // values only travel to higher lanes by shuffle, so no stored lane sees them.
    const float4 B = *reinterpret_cast<const float4 *>(row + swz(8 + 2 * bl - qh) * 4);
    const float4 Cc = *reinterpret_cast<const float4 *>(row + swz(9 + 2 * bl - qh) * 4);
    // Lane 0 has no left neighbour: it takes the preceding chunk, which every
    // lane reads (chunk 5 - qh >= 0 at block -1).
    float4 A = B;
    if (mh > 0) A = *reinterpret_cast<const float4 *>(row + swz(7 + 2 * bl - qh) * 4);
    const float bv[4] = {B.x, B.y, B.z, B.w};
    const float cv[4] = {Cc.x, Cc.y, Cc.z, Cc.w};
    const float av[4] = {A.x, A.y, A.z, A.w};
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      if (k < mh) {
        const float s = __shfl_up_sync(FULL, cv[4 - mh + k], 1);
        r[h][k] = (threadIdx.x & 31) ? s : av[4 - mh + k];
      } else if (k - mh < 4) {
        r[h][k] = bv[k - mh];
      } else {
        r[h][k] = cv[k - mh - 4];
      }
    }
  }
  if constexpr (GS == 0) {
#pragma unroll
    for (int h = 0; h < 8; ++h)
#pragma unroll
      for (int k = 0; k < 8; ++k) out[h][k] = r[h][k];
  } else {
    float t0[4][2][8];
    group2_stage_a(r, t0);
    if constexpr (GS == 1) {
#pragma unroll
      for (int e = 0; e < 8; ++e)
#pragma unroll
        for (int k = 0; k < 8; ++k) out[e][k] = t0[e >> 1][e & 1][k];
    } else {
      float t1[2][4][8];
      group2_stage_b(t0, t1);
      if constexpr (GS == 2) {
#pragma unroll
        for (int e = 0; e < 8; ++e)
#pragma unroll
          for (int k = 0; k < 8; ++k) out[e][k] = t1[e >> 2][e & 3][k];
      } else {
        group2_stage_c(t1, out);
      }
    }
  }
}

// Block b of this lane: warps 0-3 (half 0) cover blocks -1..30 (block -1 only
// seeds the boundary values), warps 4-7 cover 30..61 (block 30 seeds).
__device__ __forceinline__ void group2_lane(int &b, bool &active, bool &store) {
  const int lane = threadIdx.x & 31, half = threadIdx.x >> 7;
  b = half ? 30 + lane : lane - 1;
  active = b < W / 8;
  store = active && lane > 0;
}

// First stored block of this warp's half (lane 1): half 0 block 0, half 1
// block 31.
__device__ __forceinline__ int first_stored_block() { return (threadIdx.x >> 7) ? 31 : 0; }

// Pass A's group 2 for S stages: stores the 8 rows of this lane's block.
// Row e of `out` is row group (32 >> S) R + (e >> GS) at angle 2^GS L1 +
// (e mod 2^GS); inter_q = the quadrant's intermediate [g (32)][a (2^S)][CS].
// S = 1: group 1 did the only stage and its angle l1 = 2 pair + p, so row e
// (quad h = e) is row group 16 R + 2 e + (L1 >> 1) at angle L1 & 1.
template <int L1, int S>
__device__ __forceinline__ void group2_passA(const float *xs, float *inter_q, int R, int c0) {
  using P = PassA<S>;
  if (c0 + 8 * first_stored_block() >= P::CS) return;  // nothing this half stores
  int b;
  bool active, store;
  group2_lane(b, active, store);
  float out[8][8];
  group2_compute<L1, 0, P::GS>(xs, b, active, out);
  const int d0 = c0 + 8 * b;
  if (store && d0 < P::CS) {
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int g = S == 1 ? 16 * R + 2 * e + (L1 >> 1) : (R << (3 - P::GS)) + (e >> P::GS);
      const int a = S == 1 ? L1 & 1 : (L1 << P::GS) + (e & ((1 << P::GS) - 1));
      st8(inter_q + ((size_t)g * (1 << S) + a) * P::CS + d0, out[e]);
    }
  }
}

// Pass B output staging: the CTA's tile (W offsets x 32 angles, 128-byte
// rows) goes through shared memory so that the (4, 2n-1, n) output is written
// with whole 128-byte row segments.  Group-2 lanes own rows 8 apart (block b
// = rows 8b..8b+7), so the 16-byte chunk index is XOR-swizzled with
// (row >> 3) & 7: the eight lanes of a quarter-warp then hit eight different
// bank groups when writing, and a row's eight chunks are distinct when read.

// Pass B's group 2: compute (per-L1 code), then, after the caller's barrier,
// stage the outputs (L1 only enters the addresses).  The barrier stays out of
// the per-L1 branches: inside them, a persistent loop around this code keeps
// 64 outputs live across four barrier paths and spills.
__device__ __forceinline__ void group2_passB_compute(const float *xs, int live, float (&out)[8][8]) {
  // A half whose first stored offset is at or past `live` computes nothing:
  // the store loop writes +0 for those rows.
  if (8 * first_stored_block() >= live) return;
  int b;
  bool active, store;
  group2_lane(b, active, store);
  switch ((threadIdx.x >> 5) & 3) {
    case 0: group2_compute<0, 0>(xs, b, active, out); break;
    case 1: group2_compute<1, 0>(xs, b, active, out); break;
    case 2: group2_compute<2, 0>(xs, b, active, out); break;
    default: group2_compute<3, 0>(xs, b, active, out); break;
  }
}

__device__ __forceinline__ void group2_passB_stage(float *ost, int live, const float (&out)[8][8]) {
  int b;
  bool active, store;
  group2_lane(b, active, store);
  if (!store || 8 * first_stored_block() >= live) return;
  const int L1 = (threadIdx.x >> 5) & 3;
  // Rows 8b..8b+7 share the swizzle term b & 7: fixed offsets from one base.
  const int sw = b & 7;
  float *p0 = ost + 8 * b * 32 + 4 * ((2 * L1) ^ sw);
  float *p1 = ost + 8 * b * 32 + 4 * ((2 * L1 + 1) ^ sw);
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    *reinterpret_cast<float4 *>(p0 + 32 * k) = make_float4(out[0][k], out[1][k], out[2][k], out[3][k]);
    *reinterpret_cast<float4 *>(p1 + 32 * k) = make_float4(out[4][k], out[5][k], out[6][k], out[7][k]);
  }
}

// Writes the staged tile: quarter-warps store one 128-byte row each.  Thread
// t handles chunk t & 7 of rows (t >> 3) + 32 i, i < W / 32; the row's swizzle
// term ((row >> 3) & 7) then only alternates between two values.  All shared
// loads are issued before the global stores.  Rows at or past `live` are +0
// (offsets beyond every angle's support) and are not read from the staging.
__device__ __forceinline__ void passB_store_tile(const float *ost, float *dst_q, int ap, int c0, int n, int live) {
  constexpr int IT = W / 32;  // 15
  static_assert(W % 32 == 0, "tile rows must split into 32-row steps");
  const int r0 = threadIdx.x >> 3, c = threadIdx.x & 7;
  const int sw0 = ((r0 >> 3) & 7), sw1 = (((r0 + 32) >> 3) & 7);
  const float *s0 = ost + r0 * 32 + 4 * (c ^ sw0);
  const float *s1 = ost + (r0 + 32) * 32 + 4 * (c ^ sw1);
  float4 v[IT];
#pragma unroll
  for (int i = 0; i < IT; ++i)
    v[i] = r0 + 32 * i < live ? *reinterpret_cast<const float4 *>((i & 1 ? s1 : s0) + (i >> 1) * 64 * 32)
                              : make_float4(0.f, 0.f, 0.f, 0.f);
  const int rows = min(W, 2 * n - 1 - c0);
  float *d = dst_q + (size_t)(c0 + r0) * n + ap * 32 + 4 * c;
  const size_t step = (size_t)32 * n;
#pragma unroll
  for (int i = 0; i < IT; ++i)
    if (r0 + 32 * i < rows) __stcs(reinterpret_cast<float4 *>(d + i * step), v[i]);
}


// One pass-A tile (n = 32 * 2^S): quadrant q, rows (or columns) 32 R ..
// 32 R + 31, column tile ct of one image; inter_img = that image's
// intermediate [q][g (32)][a (2^S)][CS].  NIT: the row-quadrant sweep length
// when the caller fixes it at compile time (a persistent loop around a sweep
// of run-time length spills), at least the tile's own (`pass_a_nit`);
// 0: full tiles sweep all four iterations, others their own run-time count.
template <int S, int NIT = 0, class Hook = NoHook>
__device__ __forceinline__ void pass_a_tile(const float *img, float *inter_img, int q, int R, int ct, float *xs,
                                            const Hook &hook = Hook()) {
  using P = PassA<S>;
  const int c0 = ct * W, tbase = c0 - HALO;
  const int pos = needed_positions(min(W, P::CS - c0));
  if (q == 0 || q == 3) {
    if constexpr (NIT > 0) group1_passA_rows<P::n, NIT>(img, q, R, tbase, pos, xs);
    else if (pos == TW) group1_passA_rows<P::n, NCH / 32>(img, q, R, tbase, pos, xs);
    else group1_passA_rows<P::n>(img, q, R, tbase, pos, xs);
  } else {
    group1_passA_cols<P::n>(img, q, R, tbase, pos, xs);
  }
  hook();
  __syncthreads();
  float *inter_q = inter_img + (size_t)q * P::n * P::CS;
  switch ((threadIdx.x >> 5) & 3) {
    case 0: group2_passA<0, S>(xs, inter_q, R, c0); break;
    case 1: group2_passA<1, S>(xs, inter_q, R, c0); break;
    case 2: group2_passA<2, S>(xs, inter_q, R, c0); break;
    default: group2_passA<3, S>(xs, inter_q, R, c0); break;
  }
}

// One pass-B tile (any n in [64, 1024]): quadrant q, input angle a' = ap,
// column tile ct of one image; inter_img = its intermediate [q][g (32)]
// [a (n/32)][cs], out_img = its (4, 2n-1, n) output.  LD: cache mode of the
// intermediate's loads.  FULL_SWEEP: every tile sweeps all positions (a
// persistent loop around a sweep of run-time length spills); the live rows
// are stored either way.
template <int LD, bool FULL_SWEEP = false, class Hook = NoHook>
__device__ __forceinline__ void pass_b_tile(const float *inter_img, float *out_img, int n, int cs, int q, int ap,
                                            int ct, float *xs, const Hook &hook = Hook()) {
  const int a_in = n / 32;
  const int c0 = ct * W, tbase = c0 - HALO;
  float *dst_q = out_img + (size_t)q * (2 * n - 1) * n;
  // Every final angle of this tile is below 32 a' + 32, and at angle a the
  // output is +0 at offsets >= n + a (beyond the support of every digital
  // line); offsets from `lim` on are +0 at all 32 angles.  Tiles past it only
  // store zeros; a tile that reaches it computes only the live rows.
  const int lim = min(2 * n - 1, n + 32 * ap + 31);
  const int live = min(W, lim - c0);
  if (live <= 0) {
    hook();
    passB_store_tile(xs, dst_q, ap, c0, n, 0);
    return;
  }
  // member j row: inter[q][j][ap][*]
  const size_t mstride = (size_t)a_in * cs;
  const float *src = inter_img + ((size_t)q * 32 * a_in + ap) * cs;
  const int pos = needed_positions(live);
  if (FULL_SWEEP || pos == TW) {  // full tile: the sweep length is a compile-time constant
    switch (ap & 3) {
      case 0: group1_passB<0, NCH / 32, LD>(src, ap, tbase, pos, xs, mstride, cs); break;
      case 1: group1_passB<1, NCH / 32, LD>(src, ap, tbase, pos, xs, mstride, cs); break;
      case 2: group1_passB<2, NCH / 32, LD>(src, ap, tbase, pos, xs, mstride, cs); break;
      default: group1_passB<3, NCH / 32, LD>(src, ap, tbase, pos, xs, mstride, cs); break;
    }
  } else {
    switch (ap & 3) {
      case 0: group1_passB<0, 0, LD>(src, ap, tbase, pos, xs, mstride, cs); break;
      case 1: group1_passB<1, 0, LD>(src, ap, tbase, pos, xs, mstride, cs); break;
      case 2: group1_passB<2, 0, LD>(src, ap, tbase, pos, xs, mstride, cs); break;
      default: group1_passB<3, 0, LD>(src, ap, tbase, pos, xs, mstride, cs); break;
    }
  }
  hook();
  __syncthreads();
  float out[8][8];
  group2_passB_compute(xs, live, out);
  __syncthreads();  // every warp is done reading the exchange rows
  // The output tile is staged over the exchange rows.
  group2_passB_stage(xs, live, out);
  __syncthreads();
  passB_store_tile(xs, dst_q, ap, c0, n, live);
}

// Pass-B column tiles of one (quadrant, input angle): W offsets each.
__host__ __device__ inline int pass_b_col_tiles(int n) { return (2 * n - 1 + W - 1) / W; }

}  // namespace fast
}  // namespace adrtg
