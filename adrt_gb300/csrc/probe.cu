// Measurement kernel: the float64 add throughput of the current GPU, the roof
// that bounds the float64 transforms (their adds outnumber what HBM could
// deliver at GB300's FP64 rate).  Each thread runs 8 independent chains of
// x = x + c (round to nearest, as the transforms add); the sums are written
// so that nothing is optimised away.  No reference counterpart.
#include "common.cuh"

namespace {

__global__ void dadd_rate_kernel(double *__restrict__ out, int iters, double c) {
  double v[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = 1e-3 * threadIdx.x + i;
  for (int k = 0; k < iters; ++k) {
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = __dadd_rn(v[i], c);
  }
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < 8; ++i) s = __dadd_rn(s, v[i]);
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" int adrt_gb300_probe_dadd(double *out, int blocks, int threads, int iters, void *stream) {
  if (!out) return ADRT_GB300_ERR_NULL;
  if (blocks < 1 || threads < 32 || threads > 1024 || threads % 32 || iters < 1) return ADRT_GB300_ERR_SHAPE;
  dadd_rate_kernel<<<(unsigned)blocks, (unsigned)threads, 0, static_cast<cudaStream_t>(stream)>>>(out, iters, 1e-9);
  return adrtg::launch_status();
}
