// Fast forward ADRT for float32 (two passes of five stages): the pass
// kernels and their host side (chunking, workspace, launches).  The device
// code, and the description of the decomposition, is in fwd_fast.cuh.
#include <mutex>

#include "fwd_fast.cuh"
#include "tune.cuh"

namespace adrtg {
namespace fast {

// The first S stages for n = 32 * 2^S.  inter layout: [image][q][row group g
// (32)][angle a (2^S)][CS]; grid (column tile, 32-row block R, quadrant,
// image), column tile fastest.
template <int S>
__global__ void __launch_bounds__(NT, 2) pass_a_kernel(const float *__restrict__ in,
                                                       float *__restrict__ inter) {
  using P = PassA<S>;
  extern __shared__ __align__(16) float xs[];
  unsigned t = blockIdx.x;
  const int ct = (int)(t % (unsigned)P::TILES); t /= (unsigned)P::TILES;
  const int R = (int)(t % (unsigned)(P::n / 32)); t /= (unsigned)(P::n / 32);
  const int q = (int)(t & 3u);
  const size_t bimg = t >> 2;
  pass_a_tile<S>(in + bimg * P::n * P::n, inter + bimg * 4 * P::n * P::CS, q, R, ct, xs);
}

template <int S>
static int launch_pass_a(const float *in, float *inter, int nb, cudaStream_t st) {
  using P = PassA<S>;
  static std::atomic<unsigned long long> configured{0};
  if (const int rc = smem_limit_once((const void *)pass_a_kernel<S>, SMEM, configured)) return rc;
  const unsigned grid = (unsigned)nb * 4u * (unsigned)(P::n / 32) * (unsigned)P::TILES;
  pass_a_kernel<S><<<grid, NT, SMEM, st>>>(in, inter);
  return launch_status();
}

// Pass B for any n >= 64: the last five stages.  inter layout per image:
// [q][g (32)][a (n/32)][cs]; out: (4, 2n-1, n).  (Staging the member rows in
// shared memory with bulk copies measured slower than these register loads:
// 34.2k vs 37.7k images/s at n = 1024.)  `err` is the device error word,
// reserved for kernels with bounded waits.
__global__ void __launch_bounds__(NT, 2) pass_b_kernel(const float *__restrict__ inter,
                                                       float *__restrict__ out, int n, int cs,
                                                       int col_tiles, unsigned *err) {
  extern __shared__ __align__(16) float xs[];
  // Grid (column tile + col_tiles * quadrant, image, input angle a'): the
  // input angle is the slowest launch dimension, so the CTAs resident on an
  // SM at a time mostly share a' mod 4 and run the same group-1 code
  // (measured 4 % faster than a' second-fastest, through fewer
  // instruction-cache misses).
  const int ct = (int)(blockIdx.x % (unsigned)col_tiles), q = (int)(blockIdx.x / (unsigned)col_tiles);
  const int bimg = (int)blockIdx.y, ap = (int)blockIdx.z;
  (void)err;
  pass_b_tile<LD_CS>(inter + (size_t)bimg * 4 * n * cs, out + (size_t)bimg * 4 * (2 * n - 1) * n, n, cs, q, ap, ct,
                     xs);
}

}  // namespace fast

// Row stride of the fast path's intermediate: the rows' support.  After the
// first L-5 stages a row group's values are +0 at offsets >= n + n/32 - 1
// (angles below n/32, each digital line rising by at most its angle), so the
// rows end there, rounded up to 8 floats (32 bytes: every row start is 256-bit
// aligned); pass B reads anything past the row end as +0.  n = 1024: 1056.
static int fast_cs(i64 n) { return (int)((n + n / 32 - 1 + 7) / 8 * 8); }
static_assert(fast::CS == (fast::N + fast::N / 32 - 1 + 7) / 8 * 8, "row stride at n = 1024");
static_assert(fast::PassA<5>::CS == fast::CS && fast::PassA<4>::CS == 528 && fast::PassA<3>::CS == 264 &&
                  fast::PassA<2>::CS == 136 && fast::PassA<1>::CS == 72,
              "pass A row strides equal the intermediate's");

int fast_inter_cs(i64 n) { return fast_cs(n); }

// Bytes of intermediate per image: [q][32][n/32][cs] float32.
size_t fast_inter_bytes(i64 n) { return sizeof(float) * 4 * (size_t)n * fast_cs(n); }

bool fast_forward_eligible(i64 n, size_t elem) { return elem == 4 && n >= 64 && n <= fast::N; }

// Images per chunk (pass A then pass B per chunk).  Larger launches measured
// faster than chunks whose intermediate stays in L2 (n = 1024, 256 images:
// 52.1k img/s with one launch pair, 46.9k with 5-image chunks): the launch
// tails cost more than the intermediate's round trip through HBM, which has
// bandwidth to spare here.  Built-in budget 4 GB of intermediate (248 images
// at n = 1024), or the tuned one; chunks are balanced so the last one is not
// a small tail.
static i64 fast_chunk(i64 batch, i64 n) {
  const int mb = tune_lookup(ADRT_GB300_OP_ADRT, ADRT_GB300_F32, n).chunk_mb;
  i64 k = (i64)(((size_t)(mb > 0 ? mb : 4096) << 20) / fast_inter_bytes(n));
  if (k < 1) k = 1;
  if (k > 65535) k = 65535;  // images are pass B's grid y dimension
  if (batch <= k) return batch;
  const i64 nchunks = (batch + k - 1) / k;
  return (batch + nchunks - 1) / nchunks;
}

size_t fast_workspace_bytes(i64 batch, i64 n) { return fast_inter_bytes(n) * (size_t)fast_chunk(batch, n); }

// Device-side error word of the fast kernels (raised when a bounded wait for
// bulk copies expires); read and cleared by adrt_gb300_device_status.
static __device__ unsigned g_fast_err;
static unsigned *g_fast_err_ptr[64];
static std::mutex g_fast_err_mu;

unsigned *fast_error_word() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lock(g_fast_err_mu);
  if (!g_fast_err_ptr[dev]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_fast_err) != cudaSuccess) return nullptr;
    g_fast_err_ptr[dev] = static_cast<unsigned *>(p);
  }
  return g_fast_err_ptr[dev];
}

int adrt_forward_fast(const float *in, float *out, i64 batch, i64 n, void *ws, size_t ws_bytes,
                      cudaStream_t st) {
  const i64 per = (i64)fast_inter_bytes(n);
  if (ws == nullptr || (i64)ws_bytes < per) return ADRT_GB300_ERR_WORKSPACE;
  unsigned *err = fast_error_word();
  if (!err) return ADRT_GB300_ERR_CUDA;
  static std::atomic<unsigned long long> configured_b{0};
  if (const int rc = smem_limit_once((const void *)fast::pass_b_kernel, fast::SMEM, configured_b)) return rc;
  i64 chunk = fast_chunk(batch, n);
  if ((i64)ws_bytes < per * chunk) chunk = (i64)ws_bytes / per;
  float *inter = static_cast<float *>(ws);
  const int cs = fast_cs(n);
  const int col_tiles = (int)((2 * n - 1 + fast::W - 1) / fast::W);
  const int L = num_iters(n);
  for (i64 b0 = 0; b0 < batch; b0 += chunk) {
    const int nb = (int)((batch - b0) < chunk ? (batch - b0) : chunk);
    int rc;
    // First L-5 stages: the register pass.
    const float *src = in + b0 * n * n;
    switch (L) {
      case 10: rc = fast::launch_pass_a<5>(src, inter, nb, st); break;
      case 9: rc = fast::launch_pass_a<4>(src, inter, nb, st); break;
      case 8: rc = fast::launch_pass_a<3>(src, inter, nb, st); break;
      case 7: rc = fast::launch_pass_a<2>(src, inter, nb, st); break;
      default: rc = fast::launch_pass_a<1>(src, inter, nb, st); break;
    }
    if (rc) return rc;
    const dim3 gridb((unsigned)(col_tiles * 4), (unsigned)nb, (unsigned)(n / 32));
    fast::pass_b_kernel<<<gridb, fast::NT, fast::SMEM, st>>>(inter, out + b0 * 4 * (2 * n - 1) * n, (int)n, cs,
                                                             col_tiles, err);
    rc = launch_status();
    if (rc) return rc;
  }
  return ADRT_GB300_OK;
}

}  // namespace adrtg
