// Forward ADRT that allocates nothing: its intermediate buffer is a static
// device array compiled into this library.
//
// Who needs it: hosts that hand the library only the input and output
// buffers and may not (or cannot) allocate device memory themselves -- for
// example a serving process that reserves its whole device memory budget at
// start-up and forbids allocation afterwards, a plugin running inside another
// framework that owns the memory pool, or a foreign-language caller with no
// binding to a device allocator.  The regular entry point asks such callers
// for a workspace; this one uses ADRT_GB300_NOALLOC_SCRATCH_BYTES of device
// memory that every GPU which loads the library holds until the process exits.
//
// The scratch is shared by every call on a device and keeps the last call's
// contents.  The forward transform overwrites every scratch element it later
// reads, so nothing needs clearing between calls.  Calls that overlap on the
// GPU (different streams, or host threads racing) use the same scratch and
// race; callers must order them.
//
// Set-up: the first call on each device looks up the scratch array's device
// address (cudaGetSymbolAddress, with that device current) and caches it, so
// that first call should come before any stream capture.  The cached address
// belongs to the device's primary context: a process that calls
// cudaDeviceReset must not use this entry point on that device afterwards.
#include <mutex>

#include "common.cuh"

namespace adrtg {
template <typename T>
int adrt_forward(const T *, T *, i64, i64, void *, size_t, cudaStream_t);
size_t fwd_workspace_bytes(i64, i64, size_t);
}  // namespace adrtg

using namespace adrtg;

namespace {

constexpr size_t kScratchBytes = ADRT_GB300_NOALLOC_SCRATCH_BYTES;
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
void *g_scratch_ptr[kMaxDevices] = {};
std::mutex g_scratch_mu;

// Device address of g_scratch on the current device.  In host code the name
// g_scratch is only a host-side stand-in, so the address is looked up once per
// device (with that device current) and cached.
int scratch_address(void **out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return ADRT_GB300_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (g_scratch_ptr[dev] == nullptr) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || p == nullptr)
      return ADRT_GB300_ERR_CUDA;
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return ADRT_GB300_OK;
}

}  // namespace

extern "C" int adrt_gb300_adrt_noalloc(const void *in, void *out, int64_t batch, int64_t n,
                                       int dtype, void *stream) {
  if (!in || !out) return ADRT_GB300_ERR_NULL;
  if (dtype != ADRT_GB300_F32 && dtype != ADRT_GB300_F64) return ADRT_GB300_ERR_DTYPE;
  if (batch < 1 || n < 1 || !is_pow2(n)) return ADRT_GB300_ERR_SHAPE;
  if (n > (i64(1) << 24)) return ADRT_GB300_ERR_TOO_LARGE;
  const size_t es = dtype_size(dtype);
  // One image's intermediate must fit; a batch runs in chunks of as many
  // images as fit in the scratch (at least one).
  if (fwd_workspace_bytes(1, n, es) > kScratchBytes) return ADRT_GB300_ERR_TOO_LARGE;
  void *scratch = nullptr;
  const int rc = scratch_address(&scratch);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == ADRT_GB300_F32)
    return adrt_forward<float>(static_cast<const float *>(in), static_cast<float *>(out), batch, n,
                               scratch, kScratchBytes, st);
  return adrt_forward<double>(static_cast<const double *>(in), static_cast<double *>(out), batch, n,
                              scratch, kScratchBytes, st);
}
