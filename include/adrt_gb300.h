/*
 * adrt_gb300.h -- C ABI of the GB300 (sm_103a) ADRT library.
 *
 * Every entry point takes device pointers to C-contiguous arrays, plain sizes,
 * a dtype code and a CUDA stream (passed as void*, i.e. a cudaStream_t; NULL
 * is the legacy default stream).  Work is enqueued on that stream; the call
 * returns once it is enqueued.  No entry point allocates device memory: ops
 * that need a temporary take a caller-provided workspace whose size is given
 * by adrt_gb300_workspace_size().  Nothing throws across this boundary; each
 * call returns an adrt_gb300 status code.
 *
 * Shapes follow the reference package (karlotness/adrt):
 *   image      (batch, n, n)              n a power of two
 *   ADRT array (batch, 4, 2n-1, n)        quadrant, offset, angle
 * with a batch of 1 standing for the reference's unbatched arrays.
 *
 * Each declaration names the reference interface it replaces (file:line in
 * the reference repository).  In the reference those routines are reached
 * through the CPython module adrt._adrt_cdefs (src/adrt/adrt_cdefs_py.cpp:852-909),
 * whose argument checks and error messages the Python package adrt_gb300
 * reproduces before calling in here.
 */
#ifndef ADRT_GB300_H
#define ADRT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
enum {
  ADRT_GB300_OK = 0,
  ADRT_GB300_ERR_SHAPE = 1,     /* shape not valid for the op (reference: ValueError) */
  ADRT_GB300_ERR_STEP = 2,      /* step out of range (reference: ValueError) */
  ADRT_GB300_ERR_DTYPE = 3,     /* dtype not float32/float64 (reference: TypeError) */
  ADRT_GB300_ERR_WORKSPACE = 4, /* workspace missing or smaller than required */
  ADRT_GB300_ERR_NULL = 5,      /* a required pointer is NULL */
  ADRT_GB300_ERR_CUDA = 6,      /* the CUDA runtime reported an error */
  ADRT_GB300_ERR_TIMEOUT = 7,   /* a bounded device-side wait expired */
  ADRT_GB300_ERR_TOO_LARGE = 8  /* size arithmetic overflows (reference: ValueError) */
};

/* Dtype codes. */
enum { ADRT_GB300_F32 = 0, ADRT_GB300_F64 = 1 };

/* Ops that take a workspace. */
enum {
  ADRT_GB300_OP_ADRT = 0,
  ADRT_GB300_OP_BDRT = 1,
  ADRT_GB300_OP_IADRT = 2,
  ADRT_GB300_OP_ADJOINT = 3
};

/* Human-readable text for a status code (static storage). */
const char *adrt_gb300_status_string(int status);

/* ceil(log2(n)), 0 for n <= 1.
 * Replaces adrt::num_iters (src/adrt/adrt_cdefs_common.cpp:140-142). */
int adrt_gb300_num_iters(int64_t n);

/* Number of CUDA kernel launches this library has enqueued since it was
 * loaded (all threads, all devices).  For accounting; no reference counterpart. */
uint64_t adrt_gb300_launch_count(void);

/* Autotuner table (no reference counterpart; the reference has one CPU code
 * path).  Per (op in {ADRT_GB300_OP_ADRT, ADRT_GB300_OP_BDRT}, dtype, n a
 * power of two): width = forward tile width in offsets (0, 128 or 256),
 * max_fused = stages fused in shared memory per pass (0 = built-in 5, or
 * 1..5), chunk_mb = budget of one chunk's intermediate in MB, i.e. images
 * per launch (0 = built-in: 4096 for the float32 fast forward, 1024 for bdrt, 48
 * otherwise), use_fast = float32 fast forward kernels (-1 = when eligible,
 * 0 = off, 1 = on when eligible).  Results are bit-identical for every
 * setting; only speed changes.  Not synchronised with calls in flight on
 * other threads: set the table before launching work.  Workspace sizes
 * depend on it, so query them after setting it. */
int adrt_gb300_tune_set(int op, int dtype, int64_t n, int width, int max_fused, int chunk_mb, int use_fast);
int adrt_gb300_tune_get(int op, int dtype, int64_t n, int *width, int *max_fused, int *chunk_mb, int *use_fast);
void adrt_gb300_tune_reset(void);

/* Synchronises `stream`, then reports ADRT_GB300_ERR_TIMEOUT (and clears the
 * condition) if a kernel of this library on the current device gave up a
 * bounded wait for its bulk copies since the last call; ADRT_GB300_OK
 * otherwise.  No reference counterpart. */
int adrt_gb300_device_status(void *stream);

/* Measurement kernel (no reference counterpart): `blocks` x `threads`
 * threads each perform 8 x `iters` float64 adds (8 independent chains of
 * round-to-nearest adds) and write one double each to out (blocks x threads
 * doubles).  Timed by the caller, it gives the GPU's float64 add rate, the
 * roof of the float64 transforms. */
int adrt_gb300_probe_dadd(double *out, int blocks, int threads, int iters, void *stream);

/* Bytes of workspace that `op` needs for `batch` arrays of side n.  May be 0.
 * The reference allocates this temporary itself with PyMem_Malloc
 * (src/adrt/adrt_cdefs_py.cpp:301-307). */
int adrt_gb300_workspace_size(int op, int64_t batch, int64_t n, int dtype, size_t *bytes);

/* Forward ADRT: in (batch, n, n) -> out (batch, 4, 2n-1, n).
 * Replaces adrt::adrt_basic (src/adrt/adrt_cdefs_adrt.hpp:101-212),
 * bound as _adrt_cdefs.adrt (src/adrt/adrt_cdefs_py.cpp:275-341). */
int adrt_gb300_adrt(const void *in, void *out, int64_t batch, int64_t n, int dtype,
                    void *workspace, size_t workspace_bytes, void *stream);

/* Forward ADRT that allocates nothing and takes no workspace; no counterpart
 * in the reference.  For callers that are given input and output buffers but
 * may not allocate device memory (a fixed memory budget reserved at start-up,
 * a host framework that owns the pool, a binding without an allocator).  Its
 * intermediate is a static device array of ADRT_GB300_NOALLOC_SCRATCH_BYTES
 * that each GPU loading this library holds until exit; the first call on a
 * device looks up that array's address (make that first call before any
 * stream capture).  Sizes whose per-image intermediate exceeds the scratch
 * (float32 n >= 2048, float64 n >= 1024) return ADRT_GB300_ERR_TOO_LARGE.
 * All calls share the scratch: calls that overlap on the GPU race. */
#define ADRT_GB300_NOALLOC_SCRATCH_BYTES ((size_t)32 << 20)
int adrt_gb300_adrt_noalloc(const void *in, void *out, int64_t batch, int64_t n, int dtype,
                            void *stream);

/* ---- Ragged batches: `count` square images of power-of-two sides sizes[i]
 * (1 <= n <= 1024), packed back to back in `in` (image i after images 0..i-1),
 * transformed in one persistent launch into `out`, packed the same way
 * ((4, 2n-1, n) per image).  No counterpart in the reference, which
 * transforms one size per call; each image's result equals adrt_gb300_adrt's.
 * CTAs take (image, pass, tile) items from a device-side queue; second-pass
 * items wait, with a bounded device-side wait, for their image's first pass.
 * After the call, adrt_gb300_ragged_status synchronises the stream and
 * reports ADRT_GB300_ERR_TIMEOUT if any wait expired.  The call does not
 * wait for the GPU: its descriptors are uploaded from a pinned staging buffer
 * per device (allocated by the first call on that device, which therefore
 * must not be inside a stream capture), and one workspace serves one launch
 * at a time on one stream. */
int adrt_gb300_ragged_workspace_size(const int64_t *sizes, int64_t count, int dtype, size_t *bytes);
int adrt_gb300_adrt_ragged(const void *in, void *out, const int64_t *sizes, int64_t count, int dtype,
                           void *workspace, size_t workspace_bytes, void *stream);
int adrt_gb300_ragged_status(const void *workspace, const int64_t *sizes, int64_t count, int dtype,
                             void *stream);
/* As adrt_gb300_adrt_ragged with the wait limit in nanoseconds (0: default,
 * 4 s) and, for failure-detection tests, starve_image >= 0: that image's
 * second pass waits for a first-pass tile that does not exist, so its wait
 * expires and the status reports ADRT_GB300_ERR_TIMEOUT. */
int adrt_gb300_adrt_ragged_ex(const void *in, void *out, const int64_t *sizes, int64_t count,
                              int dtype, void *workspace, size_t workspace_bytes, uint64_t wait_ns,
                              int64_t starve_image, void *stream);

/* One forward stage in the output layout: (batch, 4, 2n-1, n) -> same.
 * Replaces adrt::adrt_step (src/adrt/adrt_cdefs_adrt.hpp:215-258),
 * bound as _adrt_cdefs.adrt_step (src/adrt/adrt_cdefs_py.cpp:343-412). */
int adrt_gb300_adrt_step(const void *in, void *out, int64_t batch, int64_t n, int step,
                         int dtype, void *stream);

/* Backprojection: (batch, 4, 2n-1, n) -> same.
 * Replaces adrt::bdrt_basic (src/adrt/adrt_cdefs_bdrt.hpp:121-187),
 * bound as _adrt_cdefs.bdrt (src/adrt/adrt_cdefs_py.cpp:482-548). */
int adrt_gb300_bdrt(const void *in, void *out, int64_t batch, int64_t n, int dtype,
                    void *workspace, size_t workspace_bytes, void *stream);

/* One backprojection stage: (batch, 4, 2n-1, n) -> same.
 * Replaces adrt::bdrt_step (src/adrt/adrt_cdefs_bdrt.hpp:190-244),
 * bound as _adrt_cdefs.bdrt_step (src/adrt/adrt_cdefs_py.cpp:550-619). */
int adrt_gb300_bdrt_step(const void *in, void *out, int64_t batch, int64_t n, int step,
                         int dtype, void *stream);

/* Exact inverse: (batch, 4, 2n-1, n) -> same.
 * Replaces adrt::iadrt_basic (src/adrt/adrt_cdefs_iadrt.hpp:110-176),
 * bound as _adrt_cdefs.iadrt (src/adrt/adrt_cdefs_py.cpp:414-480). */
int adrt_gb300_iadrt(const void *in, void *out, int64_t batch, int64_t n, int dtype,
                     void *workspace, size_t workspace_bytes, void *stream);

/* Transpose of the forward ADRT: (batch, 4, 2n-1, n) -> (batch, n, n), equal
 * to truncate(bdrt(a)) summed over quadrants in order ((q0+q1)+q2)+q3.
 * Replaces the user-level composition documented at src/adrt/_wrappers.py:283-284
 * (exactness test: tests/test_bdrt.py:310-325). */
int adrt_gb300_adjoint(const void *in, void *out, int64_t batch, int64_t n, int dtype,
                       void *workspace, size_t workspace_bytes, void *stream);

/* Quadrant initialisation: image (batch, n, n) -> (batch, 4, 2n-1, n), zeros
 * below the top n rows.  Any element type (elem_size 1, 2, 4 or 8 bytes).
 * Replaces adrt.core.adrt_init (src/adrt/core.py:123-176). */
int adrt_gb300_adrt_init(const void *in, void *out, int64_t batch, int64_t n,
                         size_t elem_size, void *stream);

/* Truncate: (batch, 4, 2n-1, n) -> (batch, 4, n, n), each quadrant un-rotated.
 * Any element type.  Replaces adrt.utils.truncate (src/adrt/utils.py:191-242). */
int adrt_gb300_truncate(const void *in, void *out, int64_t batch, int64_t n,
                        size_t elem_size, void *stream);

/* Stitch: (batch, 4, 2n-1, n) -> (batch, 3n-2, 4*(n - remove_repeated)).
 * Any element type.  Replaces adrt.utils.stitch_adrt (src/adrt/utils.py:65-134). */
int adrt_gb300_stitch(const void *in, void *out, int64_t batch, int64_t n,
                      int remove_repeated, size_t elem_size, void *stream);

/* Unstitch, the inverse of stitch: (batch, 3n-2, 4*(n - remove_repeated)) ->
 * (batch, 4, 2n-1, n); with remove_repeated each quadrant's last column is
 * taken from the next quadrant's first.  Any element type.  Replaces
 * adrt.utils.unstitch_adrt (src/adrt/utils.py:137-188). */
int adrt_gb300_unstitch(const void *in, void *out, int64_t batch, int64_t n,
                        int remove_repeated, size_t elem_size, void *stream);

/* interp_to_cart: (batch, 4, 2n-1, n) -> (batch, n, 4n), n a power of two
 * >= 2, float32/float64.  Replaces adrt::interp_adrtcart
 * (src/adrt/adrt_cdefs_interp_adrtcart.hpp:62-114), bound as
 * _adrt_cdefs.interp_to_cart with a float index type
 * (src/adrt/adrt_cdefs_py.cpp:621-682).  The first call for a given n on a
 * device builds and keeps that size's index table (host arithmetic and a
 * device allocation): do not make that first call inside CUDA-graph capture.
 * ADRT_GB300_ERR_TOO_LARGE when 4n exceeds the float index range. */
int adrt_gb300_interp_to_cart(const void *in, void *out, int64_t batch, int64_t n, int dtype, void *stream);

/* Host-only: the selection table behind interp_to_cart for size n, into
 * host buffers idx[n * 4n] (offset of the selected entry within one image's
 * (4, 2n-1, n) array, or -1 where the output is zero), fac32[4n] and
 * fac64[4n] (the scale factor per output column for float32 / float64 data).
 * out[b][o][a] = fac[a] * in[b][idx[o][a]].  No device work. */
int adrt_gb300_interp_table(int64_t n, int32_t *idx, float *fac32, double *fac64);

/* coord_adrt: the Radon offset (4, 2n-1, n) and angle (4, 1, n) of every
 * ADRT entry, float64, n a power of two >= 2.  Replaces adrt.utils.coord_adrt
 * (src/adrt/utils.py:250-332, NumPy code); arctan/sin/cos may differ from
 * NumPy's in the last place. */
int adrt_gb300_coord_adrt(int64_t n, double *offset, double *angle, void *stream);

/* coord_cart_to_adrt: for `count` points (theta, t) of dtype F32/F64, the
 * nearest ADRT entry (quadrant uint8, height int64, slope uint64) and its
 * scale factor (float64).  Replaces adrt.utils.coord_cart_to_adrt
 * (src/adrt/utils.py:335-435), following NumPy's dtypes and rounding. */
int adrt_gb300_coord_cart_to_adrt(const void *theta, const void *t, int64_t count, int64_t n, int dtype,
                                  uint8_t *quadrant, int64_t *height, uint64_t *slope, double *factor,
                                  void *stream);

/* Multigrid restriction: (batch, 4, 2n-1, n) -> (batch, 4, n-1, n/2), n even.
 * Replaces adrt::fmg_restriction (src/adrt/adrt_cdefs_fmg.hpp:53-73),
 * bound as _adrt_cdefs.press_fmg_restriction (src/adrt/adrt_cdefs_py.cpp:684-738). */
int adrt_gb300_fmg_restriction(const void *in, void *out, int64_t batch, int64_t n,
                               int dtype, void *stream);

/* Multigrid prolongation: (batch, h, w) -> (batch, 2h, 2w).
 * Replaces adrt::fmg_prolongation (src/adrt/adrt_cdefs_fmg.hpp:75-95),
 * bound as _adrt_cdefs.press_fmg_prolongation (src/adrt/adrt_cdefs_py.cpp:740-794). */
int adrt_gb300_fmg_prolongation(const void *in, void *out, int64_t batch, int64_t h,
                                int64_t w, int dtype, void *stream);

/* Multigrid high-pass filter: (batch, h, w) -> same, h, w >= 2.
 * Replaces adrt::fmg_highpass (src/adrt/adrt_cdefs_fmg.hpp:97-171),
 * bound as _adrt_cdefs.press_fmg_highpass (src/adrt/adrt_cdefs_py.cpp:796-850). */
int adrt_gb300_fmg_highpass(const void *in, void *out, int64_t batch, int64_t h,
                            int64_t w, int dtype, void *stream);

/* ---- Full-multigrid glue.  The reference evaluates these steps with NumPy
 * inside adrt.core.iadrt_fmg_step / iadrt_fmg_iter / adrt.iadrt_fmg; these
 * entry points compute the same values on the device. ------------------ */

/* out (batch, n, n) = mean over quadrants of truncate(y) / (n - 1), for
 * y (batch, 4, 2n-1, n): each term divided by (n-1), summed in quadrant order,
 * then divided by 4.  Replaces the NumPy expression at src/adrt/core.py:328-329. */
int adrt_gb300_fmg_correction(const void *y, void *out, int64_t batch, int64_t n, int dtype,
                              void *stream);

/* Elementwise out = a - b (op 0) or a + b (op 1) over `count` elements; out
 * may alias a.  Replaces the NumPy array arithmetic at src/adrt/core.py:327-330
 * and src/adrt/core.py:378. */
int adrt_gb300_elementwise(int op, const void *a, const void *b, void *out, int64_t count,
                           int dtype, void *stream);

/* Sum of squares of `count` elements accumulated in float64 with a fixed
 * (deterministic) order, written to the device double *out.  workspace must
 * hold adrt_gb300_sumsq_workspace_size() bytes.  Used for the residual norm
 * of the stopping rule at src/adrt/__init__.py:131-146. */
size_t adrt_gb300_sumsq_workspace_size(void);
int adrt_gb300_sumsq(const void *a, int64_t count, int dtype, double *out, void *workspace,
                     void *stream);

/* The same sum for each of `batch` consecutive arrays of `count` elements:
 * out[i] (device double[batch]) equals adrt_gb300_sumsq of array i bit for
 * bit.  workspace: adrt_gb300_sumsq_batched_workspace_size(batch) bytes.
 * Used by the batched full-multigrid inverse (per-image stopping rule). */
size_t adrt_gb300_sumsq_batched_workspace_size(int64_t batch);
int adrt_gb300_sumsq_batched(const void *a, int64_t batch, int64_t count, int dtype, double *out,
                             void *workspace, void *stream);

/* ---- Batched conjugate gradient on the normal equations A^T A x = A^T b.
 * The reference documents this solve as a SciPy recipe
 * (docs/examples.cginverse.md:40-67); these kernels run its vector algebra for
 * a whole batch on the device.  Per-image scalars are float64, accumulated in
 * a fixed order (deterministic).  `per` = elements per image.  Images whose
 * active[i] == 0 are left unchanged. ------------------------------------ */

/* Bytes of workspace the CG kernels need for `batch` images. */
size_t adrt_gb300_cg_workspace_size(int64_t batch);

/* out[i] = sum_k a[i,k] * b[i,k], returned in float64: per-thread partial
 * sums in the data type over a fixed strided slice, combined in float64 in a
 * fixed order (deterministic). */
int adrt_gb300_batched_dot(const void *a, const void *b, double *out, int64_t batch, int64_t per,
                           int dtype, void *workspace, void *stream);

/* alpha_i = rs[i] / pAp[i]; x += alpha p; r -= alpha Ap; rs_new[i] = <r, r>. */
int adrt_gb300_cg_update(void *x, void *r, const void *p, const void *Ap, const double *rs,
                         const double *pAp, const int *active, double *rs_new, int64_t batch,
                         int64_t per, int dtype, void *workspace, void *stream);

/* beta_i = rs_new[i] / rs[i]; p = r + beta p; rs[i] = rs_new[i]. */
int adrt_gb300_cg_direction(void *p, const void *r, const double *rs_new, double *rs,
                            const int *active, int64_t batch, int64_t per, int dtype, void *stream);

/* y += alpha * x elementwise (alpha rounded to the dtype; product and sum
 * rounded separately).  The ridge term of the regularised normal operator
 * (A^T A + lambda I) x of docs/examples.tomography.md:63-76. */
int adrt_gb300_axpy(double alpha, const void *x, void *y, int64_t count, int dtype, void *stream);

/* CG preconditioner (no reference counterpart): y = K * x per n x n image of
 * a batch, a "same"-size 2-D convolution with zero padding; K is
 * (2h+1) x (2h+1), 0 <= h <= 7, row-major, given as float64 values in HOST
 * memory (they are copied into the launch, so a captured CUDA graph keeps
 * them).  Point-symmetric K gives a symmetric operator; positive definite
 * when K's symbol is positive at every frequency.  x and y: device arrays of
 * batch * n * n elements of `dtype`, not overlapping; batch <= 65535,
 * n <= 32768. */
int adrt_gb300_precond_conv(const void *x, void *y, int64_t batch, int64_t n, const double *weights, int h,
                            int dtype, void *stream);

/* The same convolution y = K * x, fused with the per-image dot product
 * dot[i] = <x_i, y_i> (float64, device double[batch]; per-thread partial sums
 * in the data type, fixed-order float64 combination): preconditioned CG's
 * <r, M r>.  workspace: adrt_gb300_precond_dot_workspace_size(batch, n)
 * bytes of device memory. */
size_t adrt_gb300_precond_dot_workspace_size(int64_t batch, int64_t n);
int adrt_gb300_precond_conv_dot(const void *x, void *y, int64_t batch, int64_t n, const double *weights, int h,
                                int dtype, double *dot, void *workspace, size_t workspace_bytes, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* ADRT_GB300_H */
