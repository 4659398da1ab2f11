// Shared definitions for the adrt_gb300 CUDA library.
//
// Numerics: every kernel computes each output with the same operand pairing,
// operand order and copy-versus-add rule as the reference routine it replaces,
// so results are bit-identical.  The library is compiled with -fmad=false and
// without fast-math; adds that must not be reordered use __fadd_rn/__dadd_rn.
#pragma once

#include <atomic>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/adrt_gb300.h"

namespace adrtg {

using i64 = long long;

// ---- exact arithmetic helpers --------------------------------------------

__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float div_rn(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double div_rn(double a, double b) { return __ddiv_rn(a, b); }
// Two float32 adds in one packed instruction: d0 = a0 + b0, d1 = a1 + b1,
// each rounded to nearest like add_rn (add.rn.f32x2 rounds per element).
// Used where both operands of two neighbouring positions are adjacent in
// registers (butterfly shifts that are even).
__device__ __forceinline__ void add_rn2(float a0, float a1, float b0, float b1, float &d0, float &d1) {
  asm("{\n\t.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
      "add.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(d0), "=f"(d1)
      : "f"(a0), "f"(a1), "f"(b0), "f"(b1));
}

// Fused multiply-add, for kernels whose results are not compared bit for bit
// with the reference (the CG preconditioner).
__device__ __forceinline__ float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }

// ---- cache-hinted global access -------------------------------------------

// Streaming store for final outputs: written once, never re-read by us.
template <typename T>
__device__ __forceinline__ void st_stream(T *p, T v) { __stcs(p, v); }

// ---- host-side helpers ----------------------------------------------------

inline int num_iters(i64 n) {
  if (n <= 1) return 0;
  int bits = 0;
  for (i64 v = n; v; v >>= 1) ++bits;
  return bits - (((n & (n - 1)) == 0) ? 1 : 0);
}

inline bool is_pow2(i64 n) { return n > 0 && (n & (n - 1)) == 0; }

inline size_t dtype_size(int dtype) {
  return dtype == ADRT_GB300_F32 ? 4 : (dtype == ADRT_GB300_F64 ? 8 : 0);
}

inline int ceil_div_i(i64 a, i64 b) { return (int)((a + b - 1) / b); }

// The fast float32 kernels load and store 16- and 32-byte vectors: they run
// only on buffers that are 32-byte aligned (every cudaMalloc or torch
// allocation is); others take the generic kernels.
inline bool aligned32(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 31) == 0; }

// Count of kernel launches enqueued by this library (reported through
// adrt_gb300_launch_count); defined in capi.cu.
void count_launch();

// Map a CUDA error from a launch to the library status; every kernel launch
// in the library is followed by exactly one call.
inline int launch_status() {
  count_launch();
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? ADRT_GB300_OK : ADRT_GB300_ERR_CUDA;
}

// Raises a kernel's dynamic shared-memory limit on the current device.  The
// attribute belongs to the device, so it is set once per device: `done` is
// that kernel's bitmask of devices (0..63) already configured.  Two host
// threads may both set it the first time; setting it twice is harmless.
inline int smem_limit_once(const void *kern, size_t smem, std::atomic<unsigned long long> &done) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return ADRT_GB300_ERR_CUDA;
  const unsigned long long bit = 1ull << dev;
  if (done.load(std::memory_order_acquire) & bit) return ADRT_GB300_OK;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return ADRT_GB300_ERR_CUDA;
  done.fetch_or(bit, std::memory_order_acq_rel);
  return ADRT_GB300_OK;
}

}  // namespace adrtg
