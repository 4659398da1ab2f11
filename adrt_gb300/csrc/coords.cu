// Coordinate maps between the ADRT domain and the continuous Radon domain:
// coord_adrt (src/adrt/utils.py:250-332) and coord_cart_to_adrt
// (src/adrt/utils.py:335-435).  The reference evaluates them with NumPy; here
// they are element-wise kernels that follow NumPy's evaluation order and
// dtypes step by step (linspace as i*step + start, remainder via fmod,
// round-half-to-even, floor division).  Elementary operations are IEEE
// correctly rounded on both sides; arctan, sin, cos and tan come from the
// CUDA math library and can differ from NumPy's in the last place, so the
// float outputs agree to an ulp-level tolerance and the integer outputs
// except where such a difference crosses a rounding tie.
#include <cstdint>

#include "common.cuh"

namespace adrtg {

constexpr double kPiD = 3.14159265358979323846;

// offset (4, 2n-1, n) and angle (4, 1, n), float64.
__global__ void coord_adrt_kernel(long long n, double *__restrict__ offset, double *__restrict__ angle) {
  const long long C = 2 * n - 1;
  const double stop = (1.0 - (double)n) / (double)n;        // (1 - n) / n
  const double step = __dsub_rn(stop, 1.0) / (double)C;      // linspace(1, stop, 2n-1, endpoint=False)
  const double half_step = step / 2.0;
  const double ns_step = 1.0 / (double)(n - 1);              // linspace(0, 1, n)
  const double c = (double)(2 * n - 1) / (double)(2 * n);
  const long long total = C * n;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < total;
       k += (long long)gridDim.x * blockDim.x) {
    const long long i = k / n, j = k % n;
    const double hi = __dadd_rn(__dadd_rn(__dmul_rn((double)i, step), 1.0), half_step);
    const double ns = j == n - 1 ? 1.0 : __dadd_rn(__dmul_rn((double)j, ns_step), 0.0);
    const double th = atan(ns);
    const double num = __dadd_rn(hi, __dmul_rn(c, ns));
    const double h0 = __dmul_rn(__dsub_rn(num / __dadd_rn(1.0, ns), 0.5), __dadd_rn(cos(th), sin(th)));
    offset[k] = h0;
    offset[C * n + k] = -h0;
    offset[2 * C * n + k] = h0;
    offset[3 * C * n + k] = -h0;
    if (i == 0) {
      const double toff = __dsub_rn(th, kPiD / 2.0);
      angle[j] = toff;
      angle[n + j] = -th;
      angle[2 * n + j] = th;
      angle[3 * n + j] = -toff;
    }
  }
}

// NumPy's float remainder for a positive divisor: fmod, then shifted into
// [0, divisor).
template <typename T>
__device__ __forceinline__ T np_remainder(T a, T b) {
  T m = fmod(a, b);
  if (m != T(0) && ((b < T(0)) != (m < T(0)))) m = m + b;
  else if (m == T(0)) m = copysign(T(0), b);
  return m;
}

// NumPy promotes Python float constants to the array's dtype (weak scalars).
template <typename T>
__global__ void cart_to_adrt_kernel(const T *__restrict__ theta_in, const T *__restrict__ t_in, long long count,
                                    long long n, uint8_t *__restrict__ q_out, int64_t *__restrict__ h_out,
                                    uint64_t *__restrict__ s_out, double *__restrict__ f_out) {
  const T pi = (T)kPiD, pi_2 = (T)(kPiD / 2.0), pi_4 = (T)(kPiD / 4.0);
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < count;
       k += (long long)gridDim.x * blockDim.x) {
    T theta = theta_in[k];
    const T t = t_in[k];
    if (!(fabs(theta) <= pi_2)) theta = sub_rn(np_remainder(add_rn(theta, pi_2), pi), pi_2);
    T cl = div_rn(theta, pi_4);
    cl = cl < T(-2) ? T(-2) : (cl > T(1) ? T(1) : cl);
    const int q = (int)(int8_t)floor(cl) + 2;
    const T th0 = sub_rn(pi_4, fabs(sub_rn(fabs(theta), pi_4)));
    const T tn = tan(th0);
    const T sr = rint(mul_rn(tn, (T)(n - 1)));
    const uint64_t si = (uint64_t)sr;
    const double r = (double)si / (double)(n - 1);
    const double factor = sqrt(__dadd_rn(1.0, __dmul_rn(r, r)));
    const int sgn = 2 * (q % 2) - 1;
    const T a = mul_rn(T(0.5), add_rn(T(1), tn));
    const T b = div_rn(mul_rn((T)sgn, t), cos(th0));
    const T h = mul_rn(add_rn(a, b), (T)n);
    const int64_t r2 = (int64_t)rint(mul_rn(T(2), h));
    const int64_t d = r2 - 1;
    q_out[k] = (uint8_t)q;
    h_out[k] = d >= 0 ? d / 2 : -((-d + 1) / 2);  // floor division by 2
    s_out[k] = si;
    f_out[k] = factor;
  }
}

static unsigned grid_for(long long total) {
  long long g = (total + 255) / 256;
  if (g > 152 * 32) g = 152 * 32;
  return (unsigned)(g < 1 ? 1 : g);
}

}  // namespace adrtg

extern "C" int adrt_gb300_coord_adrt(int64_t n, double *offset, double *angle, void *stream) {
  if (!offset || !angle) return ADRT_GB300_ERR_NULL;
  if (n < 2 || !adrtg::is_pow2(n)) return ADRT_GB300_ERR_SHAPE;
  adrtg::coord_adrt_kernel<<<adrtg::grid_for((2 * n - 1) * n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      n, offset, angle);
  return adrtg::launch_status();
}

extern "C" int adrt_gb300_coord_cart_to_adrt(const void *theta, const void *t, int64_t count, int64_t n, int dtype,
                                             uint8_t *quadrant, int64_t *height, uint64_t *slope, double *factor,
                                             void *stream) {
  if (count < 0) return ADRT_GB300_ERR_SHAPE;
  if (n < 2 || !adrtg::is_pow2(n)) return ADRT_GB300_ERR_SHAPE;
  if (count == 0) return ADRT_GB300_OK;
  if (!theta || !t || !quadrant || !height || !slope || !factor) return ADRT_GB300_ERR_NULL;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == ADRT_GB300_F32)
    adrtg::cart_to_adrt_kernel<float><<<adrtg::grid_for(count), 256, 0, st>>>(
        static_cast<const float *>(theta), static_cast<const float *>(t), count, n, quadrant, height, slope, factor);
  else if (dtype == ADRT_GB300_F64)
    adrtg::cart_to_adrt_kernel<double><<<adrtg::grid_for(count), 256, 0, st>>>(
        static_cast<const double *>(theta), static_cast<const double *>(t), count, n, quadrant, height, slope,
        factor);
  else
    return ADRT_GB300_ERR_DTYPE;
  return adrtg::launch_status();
}
