// interp_to_cart: resample an ADRT output (batch, 4, 2n-1, n) onto the regular
// Cartesian Radon grid (batch, n, 4n).  Reference:
// src/adrt/adrt_cdefs_interp_adrtcart.hpp:62-114, bound with a float index
// type at src/adrt/adrt_cdefs_py.cpp:621-682.
//
// Which ADRT entry (quadrant, height, slope) and which scale factor each
// output point takes depends only on n and the output position, not on the
// data.  The host evaluates that index arithmetic once per (device, n) with
// exactly the reference's float operations and the same C math library calls
// (tanf, cosf, roundf, floorf, sqrt), so the selection is identical; the table
// lives on the device and the kernel is a gather and one multiply per output.
// The host code is built without floating-point contraction, as the
// reference's own build.
#include <cmath>
#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "common.cuh"

namespace adrtg {

namespace {

struct InterpTable {
  int *idx = nullptr;      // [n][4n]: q*(2n-1)*n + hi*n + si, or -1
  float *fac32 = nullptr;  // [4n] factor for float32 data
  double *fac64 = nullptr; // [4n] factor for float64 data
};

std::mutex g_interp_mu;
std::map<std::pair<int, long long>, InterpTable> g_interp;

// float constants of the reference (std::numbers::*_v<float> / 2, 4, 8).
constexpr float kPi = 3.14159265358979323846f;
constexpr float kSqrt2 = 1.41421356237309504880f;

// The selection for every output (o, a) and the per-angle factors, on the host.
void compute_table(long long n, int *idx, float *f32, double *f64) {
  const float pi_2 = kPi / 2.0f, pi_4 = kPi / 4.0f, pi_8 = kPi / 8.0f, sqrt2_2 = kSqrt2 / 2.0f;
  const long long rows = n, cols = 4 * n;
  const float t_left = sqrt2_2 - (sqrt2_2 / static_cast<float>(n));
  const float th_left = pi_2 - (pi_8 / static_cast<float>(n));
  std::vector<float> tvals((size_t)rows);
  for (long long o = 0; o < rows; ++o) {
    const float fr = static_cast<float>(o) / static_cast<float>(rows - 1);
    // std::lerp(-1, 1, fr) for endpoints of opposite sign: t*b + (1-t)*a.
    const float l = fr * 1.0f + (1.0f - fr) * -1.0f;
    tvals[(size_t)o] = t_left * l;
  }
  for (long long a = 0; a < cols; ++a) {
    const float fr = static_cast<float>(a) / static_cast<float>(cols - 1);
    const float l = fr * -1.0f + (1.0f - fr) * 1.0f;  // std::lerp(1, -1, fr)
    const float th = th_left * l;
    float cq = -th / pi_4;
    cq = cq < -2.0f ? -2.0f : (1.0f < cq ? 1.0f : cq);
    const int q = static_cast<int>(std::floor(cq)) + 2;
    const int sgn = q % 2 == 0 ? 1 : -1;
    const float th0 = pi_4 - std::fabs(std::fabs(th) - pi_4);
    float tan_theta = std::tan(th0);
    tan_theta = tan_theta < 0.0f ? 0.0f : (1.0f < tan_theta ? 1.0f : tan_theta);
    const float si = std::round(tan_theta * static_cast<float>(n - 1));
    {
      const float sa = si / static_cast<float>(n - 1);
      f32[a] = std::sqrt(sa * sa + 1.0f);
      const double sd = static_cast<double>(si) / static_cast<double>(n - 1);
      f64[a] = std::sqrt(sd * sd + 1.0);
    }
    const float cth = std::cos(th0);
    for (long long o = 0; o < rows; ++o) {
      const float t = tvals[(size_t)o];
      const float h0 = (0.5f + (tan_theta / 2.0f)) + ((sgn >= 0 ? t : -t) / cth);
      const float hi = (std::round(h0 * static_cast<float>(2 * n)) - 1.0f) / 2.0f;
      int v = -1;
      if (hi >= 0.0f && hi < static_cast<float>(2 * n - 1)) {
        const long long h = static_cast<long long>(hi), s = static_cast<long long>(si);
        v = (int)((q * (2 * n - 1) + h) * n + s);
      }
      idx[o * cols + a] = v;
    }
  }
}

// Builds the selection table on the host and uploads it.  The table is kept
// per (device, n) until the process exits (4 n^2 ints: 4 MiB at n = 1024).
// The upload is a synchronous copy, so the first call for each n on a device
// must come before any stream capture.  On failure nothing stays allocated.
int build_table(long long n, InterpTable *out) {
  std::vector<int> idx((size_t)(4 * n * n));
  std::vector<float> f32((size_t)(4 * n));
  std::vector<double> f64((size_t)(4 * n));
  compute_table(n, idx.data(), f32.data(), f64.data());
  InterpTable t{};
  const bool ok =
      cudaMalloc(&t.idx, sizeof(int) * idx.size()) == cudaSuccess &&
      cudaMalloc(&t.fac32, sizeof(float) * f32.size()) == cudaSuccess &&
      cudaMalloc(&t.fac64, sizeof(double) * f64.size()) == cudaSuccess &&
      cudaMemcpy(t.idx, idx.data(), sizeof(int) * idx.size(), cudaMemcpyHostToDevice) == cudaSuccess &&
      cudaMemcpy(t.fac32, f32.data(), sizeof(float) * f32.size(), cudaMemcpyHostToDevice) == cudaSuccess &&
      cudaMemcpy(t.fac64, f64.data(), sizeof(double) * f64.size(), cudaMemcpyHostToDevice) == cudaSuccess;
  if (!ok) {
    // cudaFree(nullptr) is a no-op, so a partial allocation is released whole.
    cudaFree(t.idx);
    cudaFree(t.fac32);
    cudaFree(t.fac64);
    return ADRT_GB300_ERR_CUDA;
  }
  *out = t;
  return ADRT_GB300_OK;
}

int table_for(long long n, InterpTable *t) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return ADRT_GB300_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_interp_mu);
  auto key = std::make_pair(dev, n);
  auto it = g_interp.find(key);
  if (it == g_interp.end()) {
    InterpTable tab;
    const int rc = build_table(n, &tab);
    if (rc) return rc;
    it = g_interp.emplace(key, tab).first;
  }
  *t = it->second;
  return ADRT_GB300_OK;
}

}  // namespace

// out[b][o][a] = factor[a] * in[b][idx[o][a]] (or 0 where idx < 0).  Grid:
// x over one image's 4 n^2 outputs (32-bit indices), y over images; the
// angle index a = k mod 4n is a mask (4n is a power of two).
template <typename T>
__global__ void interp_kernel(const T *__restrict__ in, T *__restrict__ out, const int *__restrict__ idx,
                              const T *__restrict__ fac, unsigned n) {
  const unsigned per_out = 4 * n * n, per_in = 4 * (2 * n - 1) * n, amask = 4 * n - 1;
  const T *src = in + (size_t)blockIdx.y * per_in;
  T *dst = out + (size_t)blockIdx.y * per_out;
  for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < per_out; k += gridDim.x * blockDim.x) {
    const int s = __ldg(idx + k);
    dst[k] = s >= 0 ? mul_rn(__ldg(fac + (k & amask)), src[s]) : T(0);
  }
}

int interp_to_cart_launch(const void *in, void *out, long long batch, long long n, int dtype, cudaStream_t st) {
  InterpTable tab;
  int rc = table_for(n, &tab);
  if (rc) return rc;
  const long long per_out = 4 * n * n;
  long long bx = (per_out + 255) / 256;
  if (bx > 2048) bx = 2048;
  const size_t es = dtype == ADRT_GB300_F32 ? 4 : 8;
  for (long long b0 = 0; b0 < batch; b0 += 65535) {
    const unsigned nb = (unsigned)(batch - b0 < 65535 ? batch - b0 : 65535);
    const dim3 grid((unsigned)bx, nb);
    const char *ib = static_cast<const char *>(in) + (size_t)b0 * 4 * (2 * n - 1) * n * es;
    char *ob = static_cast<char *>(out) + (size_t)b0 * per_out * es;
    if (dtype == ADRT_GB300_F32)
      interp_kernel<float><<<grid, 256, 0, st>>>(reinterpret_cast<const float *>(ib), reinterpret_cast<float *>(ob),
                                                 tab.idx, tab.fac32, (unsigned)n);
    else
      interp_kernel<double><<<grid, 256, 0, st>>>(reinterpret_cast<const double *>(ib),
                                                  reinterpret_cast<double *>(ob), tab.idx, tab.fac64, (unsigned)n);
    rc = launch_status();
    if (rc) return rc;
  }
  return ADRT_GB300_OK;
}

}  // namespace adrtg

extern "C" int adrt_gb300_interp_to_cart(const void *in, void *out, int64_t batch, int64_t n, int dtype,
                                         void *stream) {
  if (!in || !out) return ADRT_GB300_ERR_NULL;
  if (dtype != ADRT_GB300_F32 && dtype != ADRT_GB300_F64) return ADRT_GB300_ERR_DTYPE;
  if (batch < 1 || n < 2 || !adrtg::is_pow2(n)) return ADRT_GB300_ERR_SHAPE;
  // The reference's float index type represents 4n consecutive integers.
  if (n > (1ll << 24) / 4) return ADRT_GB300_ERR_TOO_LARGE;
  if (4 * n * n > 0x7FFFFFFFll) return ADRT_GB300_ERR_TOO_LARGE;
  return adrtg::interp_to_cart_launch(in, out, batch, n, dtype, static_cast<cudaStream_t>(stream));
}

// Host-only: the selection table of interp_to_cart for size n into caller
// buffers idx[n * 4n] (entry q*(2n-1)*n + h*n + s of an image's ADRT array,
// or -1 for zero), fac32[4n], fac64[4n] (factor per output angle for
// float32 / float64 data).  No device work; for checks and host tooling.
extern "C" int adrt_gb300_interp_table(int64_t n, int32_t *idx, float *fac32, double *fac64) {
  if (!idx || !fac32 || !fac64) return ADRT_GB300_ERR_NULL;
  if (n < 2 || !adrtg::is_pow2(n)) return ADRT_GB300_ERR_SHAPE;
  if (n > (1ll << 24) / 4 || 4 * n * n > 0x7FFFFFFFll) return ADRT_GB300_ERR_TOO_LARGE;
  adrtg::compute_table(n, idx, fac32, fac64);
  return ADRT_GB300_OK;
}
