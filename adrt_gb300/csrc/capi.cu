// extern "C" entry points declared in include/adrt_gb300.h: argument checks,
// dtype dispatch and workspace accounting.  Shape rules follow the reference's
// src/adrt/adrt_cdefs_common.cpp:176-330.
#include "common.cuh"

namespace adrtg {
template <typename T> int adrt_forward(const T *, T *, i64, i64, void *, size_t, cudaStream_t);
template <typename T> int bdrt_forward(const T *, T *, i64, i64, void *, size_t, cudaStream_t, i64 rows_needed);
template <typename T> int adrt_step_launch(const T *, T *, i64, i64, int, cudaStream_t);
template <typename T> int bdrt_step_launch(const T *, T *, i64, i64, int, cudaStream_t);
template <typename T> int iadrt_launch(const T *, T *, i64, i64, void *, size_t, cudaStream_t);
template <typename T> int fmg_restriction_launch(const T *, T *, i64, i64, cudaStream_t);
template <typename T> int fmg_prolongation_launch(const T *, T *, i64, i64, i64, cudaStream_t);
template <typename T> int fmg_highpass_launch(const T *, T *, i64, i64, i64, cudaStream_t);
template <typename T> int quad_sum_launch(const T *, T *, i64, i64, cudaStream_t);
template <typename T> int fmg_correction_launch(const T *, T *, i64, i64, cudaStream_t);
template <typename T> int binary_launch(const T *, const T *, T *, i64, int, cudaStream_t);
template <typename T> int sumsq_launch(const T *, i64, double *, void *, cudaStream_t, i64);
size_t sumsq_workspace_bytes();
unsigned *fast_error_word();
size_t ragged_workspace_bytes(const int64_t *, i64, size_t, int *);
size_t ragged_error_offset(const int64_t *, i64, size_t);
template <typename T>
int adrt_ragged(const T *, T *, const int64_t *, i64, void *, size_t, unsigned long long, i64, cudaStream_t);
size_t cg_workspace_bytes(i64);
template <typename T> int batched_dot_launch(const T *, const T *, double *, i64, i64, void *, cudaStream_t);
template <typename T>
int cg_update_launch(T *, T *, const T *, const T *, const double *, const double *, const int *,
                     double *, i64, i64, void *, cudaStream_t);
template <typename T>
int cg_direction_launch(T *, const T *, const double *, double *, const int *, i64, i64, cudaStream_t);
template <typename T> int axpy_launch(double, const T *, T *, i64, cudaStream_t);
size_t fwd_workspace_bytes(i64, i64, size_t);
size_t bwd_workspace_bytes(i64, i64, size_t);
size_t iadrt_workspace_bytes(i64, i64, size_t);
int init_launch(const void *, void *, i64, i64, size_t, cudaStream_t);
int truncate_launch(const void *, void *, i64, i64, size_t, cudaStream_t);
int stitch_launch(const void *, void *, i64, i64, int, size_t, cudaStream_t);
int unstitch_launch(const void *in, void *out, i64 batch, i64 n, i64 vc, size_t es, cudaStream_t st);
}  // namespace adrtg

#include <atomic>

namespace adrtg {
static std::atomic<unsigned long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
}  // namespace adrtg

using namespace adrtg;

namespace {

// Largest n accepted: keeps 4 * n * (2n - 1) * 8 bytes and all index math in i64.
constexpr i64 kMaxN = i64(1) << 24;

int check_adrt_shape(i64 batch, i64 n) {
  if (batch < 1 || n < 1) return ADRT_GB300_ERR_SHAPE;
  if (!is_pow2(n)) return ADRT_GB300_ERR_SHAPE;
  if (n > kMaxN) return ADRT_GB300_ERR_TOO_LARGE;
  return ADRT_GB300_OK;
}

int check_dtype(int dtype) {
  return (dtype == ADRT_GB300_F32 || dtype == ADRT_GB300_F64) ? ADRT_GB300_OK : ADRT_GB300_ERR_DTYPE;
}

size_t adjoint_workspace(i64 batch, i64 n, size_t es) {
  return (size_t)batch * 4 * n * (2 * n - 1) * es + bwd_workspace_bytes(batch, n, es);
}

inline cudaStream_t S(void *s) { return static_cast<cudaStream_t>(s); }

}  // namespace

extern "C" {

const char *adrt_gb300_status_string(int status) {
  switch (status) {
    case ADRT_GB300_OK: return "ok";
    case ADRT_GB300_ERR_SHAPE: return "invalid shape";
    case ADRT_GB300_ERR_STEP: return "step out of range";
    case ADRT_GB300_ERR_DTYPE: return "unsupported dtype";
    case ADRT_GB300_ERR_WORKSPACE: return "workspace missing or too small";
    case ADRT_GB300_ERR_NULL: return "null pointer";
    case ADRT_GB300_ERR_CUDA: return "CUDA error";
    case ADRT_GB300_ERR_TIMEOUT: return "device wait timed out";
    case ADRT_GB300_ERR_TOO_LARGE: return "array is too big";
  }
  return "unknown status";
}

int adrt_gb300_num_iters(int64_t n) { return num_iters(n); }

uint64_t adrt_gb300_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

int adrt_gb300_workspace_size(int op, int64_t batch, int64_t n, int dtype, size_t *bytes) {
  if (!bytes) return ADRT_GB300_ERR_NULL;
  int rc = check_dtype(dtype);
  if (rc) return rc;
  if ((rc = check_adrt_shape(batch, n))) return rc;
  const size_t es = dtype_size(dtype);
  switch (op) {
    case ADRT_GB300_OP_ADRT: *bytes = fwd_workspace_bytes(batch, n, es); return ADRT_GB300_OK;
    case ADRT_GB300_OP_BDRT: *bytes = bwd_workspace_bytes(batch, n, es); return ADRT_GB300_OK;
    case ADRT_GB300_OP_IADRT: *bytes = iadrt_workspace_bytes(batch, n, es); return ADRT_GB300_OK;
    case ADRT_GB300_OP_ADJOINT: *bytes = adjoint_workspace(batch, n, es); return ADRT_GB300_OK;
  }
  return ADRT_GB300_ERR_SHAPE;
}

#define DISPATCH(dtype, CALL_F32, CALL_F64) \
  ((dtype) == ADRT_GB300_F32 ? (CALL_F32) : (CALL_F64))

int adrt_gb300_adrt(const void *in, void *out, int64_t batch, int64_t n, int dtype,
                    void *ws, size_t ws_bytes, void *stream) {
  int rc;
  if (!in || !out) return ADRT_GB300_ERR_NULL;
  if ((rc = check_dtype(dtype)) || (rc = check_adrt_shape(batch, n))) return rc;
  return DISPATCH(dtype,
                  adrt_forward<float>((const float *)in, (float *)out, batch, n, ws, ws_bytes, S(stream)),
                  adrt_forward<double>((const double *)in, (double *)out, batch, n, ws, ws_bytes, S(stream)));
}

int adrt_gb300_adrt_step(const void *in, void *out, int64_t batch, int64_t n, int step,
                         int dtype, void *stream) {
  int rc;
  if (!in || !out) return ADRT_GB300_ERR_NULL;
  if ((rc = check_dtype(dtype)) || (rc = check_adrt_shape(batch, n))) return rc;
  if (step < 0 || step >= num_iters(n)) return ADRT_GB300_ERR_STEP;
  return DISPATCH(dtype,
                  adrt_step_launch<float>((const float *)in, (float *)out, batch, n, step, S(stream)),
                  adrt_step_launch<double>((const double *)in, (double *)out, batch, n, step, S(stream)));
}

int adrt_gb300_bdrt(const void *in, void *out, int64_t batch, int64_t n, int dtype,
                    void *ws, size_t ws_bytes, void *stream) {
  int rc;
  if (!in || !out) return ADRT_GB300_ERR_NULL;
  if ((rc = check_dtype(dtype)) || (rc = check_adrt_shape(batch, n))) return rc;
  return DISPATCH(dtype,
                  bdrt_forward<float>((const float *)in, (float *)out, batch, n, ws, ws_bytes, S(stream), 2 * n - 1),
                  bdrt_forward<double>((const double *)in, (double *)out, batch, n, ws, ws_bytes, S(stream), 2 * n - 1));
}

int adrt_gb300_bdrt_step(const void *in, void *out, int64_t batch, int64_t n, int step,
                         int dtype, void *stream) {
  int rc;
  if (!in || !out) return ADRT_GB300_ERR_NULL;
  if ((rc = check_dtype(dtype)) || (rc = check_adrt_shape(batch, n))) return rc;
  if (step < 0 || step >= num_iters(n)) return ADRT_GB300_ERR_STEP;
  return DISPATCH(dtype,
                  bdrt_step_launch<float>((const float *)in, (float *)out, batch, n, step, S(stream)),
                  bdrt_step_launch<double>((const double *)in, (double *)out, batch, n, step, S(stream)));
}

int adrt_gb300_iadrt(const void *in, void *out, int64_t batch, int64_t n, int dtype,
                     void *ws, size_t ws_bytes, void *stream) {
  int rc;
  if (!in || !out) return ADRT_GB300_ERR_NULL;
  if ((rc = check_dtype(dtype)) || (rc = check_adrt_shape(batch, n))) return rc;
  return DISPATCH(dtype,
                  iadrt_launch<float>((const float *)in, (float *)out, batch, n, ws, ws_bytes, S(stream)),
                  iadrt_launch<double>((const double *)in, (double *)out, batch, n, ws, ws_bytes, S(stream)));
}

int adrt_gb300_adjoint(const void *in, void *out, int64_t batch, int64_t n, int dtype,
                       void *ws, size_t ws_bytes, void *stream) {
  int rc;
  if (!in || !out) return ADRT_GB300_ERR_NULL;
  if ((rc = check_dtype(dtype)) || (rc = check_adrt_shape(batch, n))) return rc;
  const size_t es = dtype_size(dtype);
  const size_t ybytes = (size_t)batch * 4 * n * (2 * n - 1) * es;
  if (!ws || ws_bytes < adjoint_workspace(batch, n, es)) return ADRT_GB300_ERR_WORKSPACE;
  void *y = ws;
  void *bws = static_cast<char *>(ws) + ybytes;
  const size_t bws_bytes = ws_bytes - ybytes;
  if (dtype == ADRT_GB300_F32) {
    // Only the top n offsets of each quadrant reach the quadrant sum.
    if ((rc = bdrt_forward<float>((const float *)in, (float *)y, batch, n, bws, bws_bytes, S(stream), n)))
      return rc;
    return quad_sum_launch<float>((const float *)y, (float *)out, batch, n, S(stream));
  }
  if ((rc = bdrt_forward<double>((const double *)in, (double *)y, batch, n, bws, bws_bytes, S(stream), n)))
    return rc;
  return quad_sum_launch<double>((const double *)y, (double *)out, batch, n, S(stream));
}

int adrt_gb300_adrt_init(const void *in, void *out, int64_t batch, int64_t n, size_t es,
                         void *stream) {
  int rc;
  if (!in || !out) return ADRT_GB300_ERR_NULL;
  if ((rc = check_adrt_shape(batch, n))) return rc;
  return init_launch(in, out, batch, n, es, S(stream));
}

int adrt_gb300_truncate(const void *in, void *out, int64_t batch, int64_t n, size_t es,
                        void *stream) {
  if (!in || !out) return ADRT_GB300_ERR_NULL;
  if (batch < 1 || n < 1) return ADRT_GB300_ERR_SHAPE;
  return truncate_launch(in, out, batch, n, es, S(stream));
}

int adrt_gb300_stitch(const void *in, void *out, int64_t batch, int64_t n, int remove_repeated,
                      size_t es, void *stream) {
  if (!in || !out) return ADRT_GB300_ERR_NULL;
  if (batch < 1 || n < 1) return ADRT_GB300_ERR_SHAPE;
  return stitch_launch(in, out, batch, n, remove_repeated ? 1 : 0, es, S(stream));
}

int adrt_gb300_unstitch(const void *in, void *out, int64_t batch, int64_t n, int remove_repeated,
                        size_t es, void *stream) {
  if (!in || !out) return ADRT_GB300_ERR_NULL;
  if (batch < 1 || n < 1) return ADRT_GB300_ERR_SHAPE;
  return unstitch_launch(in, out, batch, n, n - (remove_repeated ? 1 : 0), es, S(stream));
}

int adrt_gb300_fmg_restriction(const void *in, void *out, int64_t batch, int64_t n, int dtype,
                               void *stream) {
  int rc;
  if (!in || !out) return ADRT_GB300_ERR_NULL;
  if ((rc = check_dtype(dtype))) return rc;
  if (batch < 1 || n < 2 || (n % 2) != 0) return ADRT_GB300_ERR_SHAPE;
  return DISPATCH(dtype,
                  fmg_restriction_launch<float>((const float *)in, (float *)out, batch, n, S(stream)),
                  fmg_restriction_launch<double>((const double *)in, (double *)out, batch, n, S(stream)));
}

int adrt_gb300_fmg_prolongation(const void *in, void *out, int64_t batch, int64_t h, int64_t w,
                                int dtype, void *stream) {
  int rc;
  if (!in || !out) return ADRT_GB300_ERR_NULL;
  if ((rc = check_dtype(dtype))) return rc;
  if (batch < 1 || h < 1 || w < 1) return ADRT_GB300_ERR_SHAPE;
  return DISPATCH(dtype,
                  fmg_prolongation_launch<float>((const float *)in, (float *)out, batch, h, w, S(stream)),
                  fmg_prolongation_launch<double>((const double *)in, (double *)out, batch, h, w, S(stream)));
}

int adrt_gb300_fmg_highpass(const void *in, void *out, int64_t batch, int64_t h, int64_t w,
                            int dtype, void *stream) {
  int rc;
  if (!in || !out) return ADRT_GB300_ERR_NULL;
  if ((rc = check_dtype(dtype))) return rc;
  if (batch < 1 || h < 2 || w < 2) return ADRT_GB300_ERR_SHAPE;
  return DISPATCH(dtype,
                  fmg_highpass_launch<float>((const float *)in, (float *)out, batch, h, w, S(stream)),
                  fmg_highpass_launch<double>((const double *)in, (double *)out, batch, h, w, S(stream)));
}

int adrt_gb300_fmg_correction(const void *y, void *out, int64_t batch, int64_t n, int dtype,
                              void *stream) {
  int rc;
  if (!y || !out) return ADRT_GB300_ERR_NULL;
  if ((rc = check_dtype(dtype)) || (rc = check_adrt_shape(batch, n))) return rc;
  if (n < 2) return ADRT_GB300_ERR_SHAPE;
  return DISPATCH(dtype,
                  fmg_correction_launch<float>((const float *)y, (float *)out, batch, n, S(stream)),
                  fmg_correction_launch<double>((const double *)y, (double *)out, batch, n, S(stream)));
}

int adrt_gb300_elementwise(int op, const void *a, const void *b, void *out, int64_t count,
                           int dtype, void *stream) {
  int rc;
  if (!a || !b || !out) return ADRT_GB300_ERR_NULL;
  if ((rc = check_dtype(dtype))) return rc;
  if (count < 0 || (op != 0 && op != 1)) return ADRT_GB300_ERR_SHAPE;
  if (count == 0) return ADRT_GB300_OK;
  return DISPATCH(dtype,
                  binary_launch<float>((const float *)a, (const float *)b, (float *)out, count, op, S(stream)),
                  binary_launch<double>((const double *)a, (const double *)b, (double *)out, count, op, S(stream)));
}

size_t adrt_gb300_sumsq_workspace_size(void) { return sumsq_workspace_bytes(); }

int adrt_gb300_sumsq(const void *a, int64_t count, int dtype, double *out, void *ws,
                     void *stream) {
  int rc;
  if (!a || !out || !ws) return ADRT_GB300_ERR_NULL;
  if ((rc = check_dtype(dtype))) return rc;
  if (count < 0) return ADRT_GB300_ERR_SHAPE;
  return DISPATCH(dtype,
                  sumsq_launch<float>((const float *)a, count, out, ws, S(stream), 1),
                  sumsq_launch<double>((const double *)a, count, out, ws, S(stream), 1));
}

size_t adrt_gb300_sumsq_batched_workspace_size(int64_t batch) {
  return batch > 0 ? sumsq_workspace_bytes() * (size_t)batch : 0;
}

int adrt_gb300_sumsq_batched(const void *a, int64_t batch, int64_t count, int dtype, double *out, void *ws,
                             void *stream) {
  int rc;
  if (!a || !out || !ws) return ADRT_GB300_ERR_NULL;
  if ((rc = check_dtype(dtype))) return rc;
  if (count < 0 || batch < 1) return ADRT_GB300_ERR_SHAPE;
  if (batch > 65535) return ADRT_GB300_ERR_TOO_LARGE;
  return DISPATCH(dtype,
                  sumsq_launch<float>((const float *)a, count, out, ws, S(stream), batch),
                  sumsq_launch<double>((const double *)a, count, out, ws, S(stream), batch));
}

}  // extern "C"

extern "C" {

size_t adrt_gb300_cg_workspace_size(int64_t batch) { return batch > 0 ? cg_workspace_bytes(batch) : 0; }

int adrt_gb300_batched_dot(const void *a, const void *b, double *out, int64_t batch, int64_t per,
                           int dtype, void *ws, void *stream) {
  int rc;
  if (!a || !b || !out || !ws) return ADRT_GB300_ERR_NULL;
  if ((rc = check_dtype(dtype))) return rc;
  if (batch < 1 || batch > 65535 || per < 1) return ADRT_GB300_ERR_SHAPE;
  return DISPATCH(dtype,
                  batched_dot_launch<float>((const float *)a, (const float *)b, out, batch, per, ws, S(stream)),
                  batched_dot_launch<double>((const double *)a, (const double *)b, out, batch, per, ws, S(stream)));
}

int adrt_gb300_cg_update(void *x, void *r, const void *p, const void *Ap, const double *rs,
                         const double *pAp, const int *active, double *rs_new, int64_t batch,
                         int64_t per, int dtype, void *ws, void *stream) {
  int rc;
  if (!x || !r || !p || !Ap || !rs || !pAp || !active || !rs_new || !ws) return ADRT_GB300_ERR_NULL;
  if ((rc = check_dtype(dtype))) return rc;
  if (batch < 1 || batch > 65535 || per < 1) return ADRT_GB300_ERR_SHAPE;
  return DISPATCH(dtype,
                  cg_update_launch<float>((float *)x, (float *)r, (const float *)p, (const float *)Ap, rs, pAp,
                                          active, rs_new, batch, per, ws, S(stream)),
                  cg_update_launch<double>((double *)x, (double *)r, (const double *)p, (const double *)Ap, rs,
                                           pAp, active, rs_new, batch, per, ws, S(stream)));
}

int adrt_gb300_cg_direction(void *p, const void *r, const double *rs_new, double *rs,
                            const int *active, int64_t batch, int64_t per, int dtype, void *stream) {
  int rc;
  if (!p || !r || !rs_new || !rs || !active) return ADRT_GB300_ERR_NULL;
  if ((rc = check_dtype(dtype))) return rc;
  if (batch < 1 || batch > 65535 || per < 1) return ADRT_GB300_ERR_SHAPE;
  return DISPATCH(dtype,
                  cg_direction_launch<float>((float *)p, (const float *)r, rs_new, rs, active, batch, per, S(stream)),
                  cg_direction_launch<double>((double *)p, (const double *)r, rs_new, rs, active, batch, per, S(stream)));
}

int adrt_gb300_axpy(double alpha, const void *x, void *y, int64_t count, int dtype, void *stream) {
  int rc;
  if (!x || !y) return ADRT_GB300_ERR_NULL;
  if ((rc = check_dtype(dtype))) return rc;
  if (count < 0) return ADRT_GB300_ERR_SHAPE;
  if (count == 0) return ADRT_GB300_OK;
  return DISPATCH(dtype, axpy_launch<float>(alpha, (const float *)x, (float *)y, count, S(stream)),
                  axpy_launch<double>(alpha, (const double *)x, (double *)y, count, S(stream)));
}

}  // extern "C"

extern "C" {

int adrt_gb300_ragged_workspace_size(const int64_t *sizes, int64_t count, int dtype, size_t *bytes) {
  int rc;
  if (!sizes || !bytes) return ADRT_GB300_ERR_NULL;
  if ((rc = check_dtype(dtype))) return rc;
  if (count < 1) return ADRT_GB300_ERR_SHAPE;
  *bytes = ragged_workspace_bytes(sizes, count, dtype_size(dtype), &rc);
  return rc;
}

int adrt_gb300_adrt_ragged_ex(const void *in, void *out, const int64_t *sizes, int64_t count,
                              int dtype, void *ws, size_t ws_bytes, uint64_t wait_ns,
                              int64_t starve_image, void *stream) {
  int rc;
  if (!in || !out || !sizes) return ADRT_GB300_ERR_NULL;
  if ((rc = check_dtype(dtype))) return rc;
  if (count < 1) return ADRT_GB300_ERR_SHAPE;
  return DISPATCH(dtype,
                  adrt_ragged<float>((const float *)in, (float *)out, sizes, count, ws, ws_bytes, wait_ns,
                                     starve_image, S(stream)),
                  adrt_ragged<double>((const double *)in, (double *)out, sizes, count, ws, ws_bytes, wait_ns,
                                      starve_image, S(stream)));
}

int adrt_gb300_adrt_ragged(const void *in, void *out, const int64_t *sizes, int64_t count, int dtype,
                           void *ws, size_t ws_bytes, void *stream) {
  return adrt_gb300_adrt_ragged_ex(in, out, sizes, count, dtype, ws, ws_bytes, 0, -1, stream);
}

int adrt_gb300_ragged_status(const void *ws, const int64_t *sizes, int64_t count, int dtype,
                             void *stream) {
  int rc;
  if (!ws || !sizes) return ADRT_GB300_ERR_NULL;
  if ((rc = check_dtype(dtype))) return rc;
  if (count < 1) return ADRT_GB300_ERR_SHAPE;
  const size_t off = ragged_error_offset(sizes, count, dtype_size(dtype));
  if (off == 0) return ADRT_GB300_ERR_SHAPE;
  unsigned word = 0;
  if (cudaMemcpyAsync(&word, static_cast<const char *>(ws) + off, sizeof(word), cudaMemcpyDeviceToHost,
                      S(stream)) != cudaSuccess ||
      cudaStreamSynchronize(S(stream)) != cudaSuccess)
    return ADRT_GB300_ERR_CUDA;
  return word ? ADRT_GB300_ERR_TIMEOUT : ADRT_GB300_OK;
}

}  // extern "C"

extern "C" int adrt_gb300_device_status(void *stream) {
  unsigned *w = fast_error_word();
  if (!w) return ADRT_GB300_ERR_CUDA;
  unsigned word = 0;
  cudaStream_t st = S(stream);
  if (cudaMemcpyAsync(&word, w, sizeof(word), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return ADRT_GB300_ERR_CUDA;
  if (word) {
    const unsigned zero = 0;
    if (cudaMemcpyAsync(w, &zero, sizeof(zero), cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return ADRT_GB300_ERR_CUDA;
    return ADRT_GB300_ERR_TIMEOUT;
  }
  return ADRT_GB300_OK;
}
