// Elementwise and small-channel kernels of the learned CG preconditioner:
// the 1-channel input and output convolutions (too narrow for the tensor
// cores), 2x2 average pooling, nearest 2x upsampling, bias gradients, the
// training loss, and the fused Adam step that also refreshes the bf16 weight
// copies (forward layout and flipped/transposed input-gradient layout) the
// tensor-core convolutions read.
//
// Layouts: activations bf16 NHWC, images f32 (batch, h, w); first-layer
// weights f32 [9][32], last-layer weights f32 [9][32]; tap = 3 * dy + dx.

#include <cuda_bf16.h>

#include "../../include/adrt_gb300_net.h"
#include "common.cuh"

namespace adrtg {
namespace net {

using bf16 = __nv_bfloat16;
constexpr int kC0 = 32;  // channels at the network's first level

__device__ __forceinline__ float ld_bf(const bf16 *p) { return __bfloat162float(*p); }
__device__ __forceinline__ bool positive(bf16 v) {
  const unsigned short h = __bfloat16_as_ushort(v);
  return !(h & 0x8000u) && (h & 0x7FFFu);
}

// out[p][co] = relu(b[co] + sum_t w[t][co] * u[p + d_t]), u zero-padded.
__global__ void conv_in_kernel(const float *u, const float *w, const float *b, bf16 *out, int h, int wd,
                               long long npix) {
  __shared__ float sw[9 * kC0 + kC0];
  for (int i = threadIdx.x; i < 9 * kC0 + kC0; i += blockDim.x) sw[i] = i < 9 * kC0 ? w[i] : b[i - 9 * kC0];
  __syncthreads();
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npix) return;
  const long long hw = (long long)h * wd;
  const long long img = p / hw;
  const int y = (int)((p % hw) / wd), x = (int)(p % wd);
  float nb[9];
#pragma unroll
  for (int t = 0; t < 9; ++t) {
    const int yy = y + t / 3 - 1, xx = x + t % 3 - 1;
    nb[t] = (yy >= 0 && yy < h && xx >= 0 && xx < wd) ? u[img * hw + (long long)yy * wd + xx] : 0.0f;
  }
  unsigned packed[kC0 / 2];
#pragma unroll
  for (int c = 0; c < kC0; c += 2) {
    float v0 = sw[9 * kC0 + c], v1 = sw[9 * kC0 + c + 1];
#pragma unroll
    for (int t = 0; t < 9; ++t) {
      v0 += sw[t * kC0 + c] * nb[t];
      v1 += sw[t * kC0 + c + 1] * nb[t];
    }
    const unsigned lo = __bfloat16_as_ushort(__float2bfloat16_rn(fmaxf(v0, 0.0f)));
    const unsigned hi = __bfloat16_as_ushort(__float2bfloat16_rn(fmaxf(v1, 0.0f)));
    packed[c / 2] = lo | (hi << 16);
  }
  uint4 *dst = reinterpret_cast<uint4 *>(out + p * kC0);
#pragma unroll
  for (int q = 0; q < 4; ++q) dst[q] = make_uint4(packed[4 * q], packed[4 * q + 1], packed[4 * q + 2], packed[4 * q + 3]);
}

// dw[t][co] += sum_p g[p][co] * u[p + d_t];  db[co] += sum_p g[p][co].
// Block: 256 threads = 8 pixel lanes x 32 channels.
__global__ void conv_in_wgrad_kernel(const float *u, const bf16 *g, float *dw, float *db, int h, int wd,
                                     long long npix, int pix_per_block) {
  const int co = threadIdx.x & 31, pl = threadIdx.x >> 5;
  float acc[10];
#pragma unroll
  for (int i = 0; i < 10; ++i) acc[i] = 0.0f;
  const long long hw = (long long)h * wd;
  const long long p0 = (long long)blockIdx.x * pix_per_block;
  const long long p1 = min(p0 + pix_per_block, npix);
  for (long long p = p0 + pl; p < p1; p += 8) {
    const float gv = ld_bf(g + p * kC0 + co);
    const long long img = p / hw;
    const int y = (int)((p % hw) / wd), x = (int)(p % wd);
#pragma unroll
    for (int t = 0; t < 9; ++t) {
      const int yy = y + t / 3 - 1, xx = x + t % 3 - 1;
      const float uv = (yy >= 0 && yy < h && xx >= 0 && xx < wd) ? u[img * hw + (long long)yy * wd + xx] : 0.0f;
      acc[t] += gv * uv;
    }
    acc[9] += gv;
  }
  __shared__ float red[8][10][32];
#pragma unroll
  for (int i = 0; i < 10; ++i) red[pl][i][co] = acc[i];
  __syncthreads();
  for (int i = threadIdx.x; i < 10 * 32; i += blockDim.x) {
    const int k = i / 32, c = i % 32;
    float s = 0.0f;
    for (int l = 0; l < 8; ++l) s += red[l][k][c];
    if (k < 9)
      atomicAdd(dw + k * kC0 + c, s);
    else
      atomicAdd(db + c, s);
  }
}

// out[p] = b + sum_t sum_ci w[t][ci] * f[p + d_t][ci]  (f32 image).
__global__ void conv_out_kernel(const bf16 *f, const float *w, const float *b, float *out, int h, int wd,
                                long long npix) {
  __shared__ float sw[9 * kC0];
  for (int i = threadIdx.x; i < 9 * kC0; i += blockDim.x) sw[i] = w[i];
  __syncthreads();
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npix) return;
  const long long hw = (long long)h * wd;
  const long long img = p / hw;
  const int y = (int)((p % hw) / wd), x = (int)(p % wd);
  float v = b[0];
  for (int t = 0; t < 9; ++t) {
    const int yy = y + t / 3 - 1, xx = x + t % 3 - 1;
    if (yy < 0 || yy >= h || xx < 0 || xx >= wd) continue;
    const uint4 *src = reinterpret_cast<const uint4 *>(f + (img * hw + (long long)yy * wd + xx) * kC0);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const uint4 u4 = src[q];
      const unsigned e[4] = {u4.x, u4.y, u4.z, u4.w};
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        v += sw[t * kC0 + q * 8 + 2 * k] * __uint_as_float(e[k] << 16);
        v += sw[t * kC0 + q * 8 + 2 * k + 1] * __uint_as_float(e[k] & 0xFFFF0000u);
      }
    }
  }
  out[p] = v;
}

// Input gradient of the output convolution, masked by the ReLU of its input:
// dx[q][ci] = (f[q][ci] > 0) * sum_t w[t][ci] * g[q - d_t].
__global__ void conv_out_dgrad_kernel(const float *g, const float *w, const bf16 *f, bf16 *dx, int h, int wd,
                                      long long npix) {
  __shared__ float sw[9 * kC0];
  for (int i = threadIdx.x; i < 9 * kC0; i += blockDim.x) sw[i] = w[i];
  __syncthreads();
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= npix) return;
  const long long hw = (long long)h * wd;
  const long long img = q / hw;
  const int y = (int)((q % hw) / wd), x = (int)(q % wd);
  float gt[9];
#pragma unroll
  for (int t = 0; t < 9; ++t) {
    const int yy = y - (t / 3 - 1), xx = x - (t % 3 - 1);
    gt[t] = (yy >= 0 && yy < h && xx >= 0 && xx < wd) ? g[img * hw + (long long)yy * wd + xx] : 0.0f;
  }
  const bf16 *fm = f + q * kC0;
  unsigned packed[kC0 / 2];
#pragma unroll
  for (int c = 0; c < kC0; c += 2) {
    float v0 = 0.0f, v1 = 0.0f;
#pragma unroll
    for (int t = 0; t < 9; ++t) {
      v0 += sw[t * kC0 + c] * gt[t];
      v1 += sw[t * kC0 + c + 1] * gt[t];
    }
    if (!positive(fm[c])) v0 = 0.0f;
    if (!positive(fm[c + 1])) v1 = 0.0f;
    packed[c / 2] = (unsigned)__bfloat16_as_ushort(__float2bfloat16_rn(v0)) |
                    ((unsigned)__bfloat16_as_ushort(__float2bfloat16_rn(v1)) << 16);
  }
  uint4 *dst = reinterpret_cast<uint4 *>(dx + q * kC0);
#pragma unroll
  for (int k = 0; k < 4; ++k) dst[k] = make_uint4(packed[4 * k], packed[4 * k + 1], packed[4 * k + 2], packed[4 * k + 3]);
}

// dw[t][ci] += sum_p g[p] * f[p + d_t][ci];  db += sum_p g[p].
__global__ void conv_out_wgrad_kernel(const float *g, const bf16 *f, float *dw, float *db, int h, int wd,
                                      long long npix, int pix_per_block) {
  const int ci = threadIdx.x & 31, pl = threadIdx.x >> 5;
  float acc[10];
#pragma unroll
  for (int i = 0; i < 10; ++i) acc[i] = 0.0f;
  const long long hw = (long long)h * wd;
  const long long p0 = (long long)blockIdx.x * pix_per_block;
  const long long p1 = min(p0 + pix_per_block, npix);
  for (long long p = p0 + pl; p < p1; p += 8) {
    const float gv = g[p];
    const long long img = p / hw;
    const int y = (int)((p % hw) / wd), x = (int)(p % wd);
#pragma unroll
    for (int t = 0; t < 9; ++t) {
      const int yy = y + t / 3 - 1, xx = x + t % 3 - 1;
      const float fv =
          (yy >= 0 && yy < h && xx >= 0 && xx < wd) ? ld_bf(f + (img * hw + (long long)yy * wd + xx) * kC0 + ci) : 0.0f;
      acc[t] += gv * fv;
    }
    acc[9] += (ci == 0) ? gv : 0.0f;
  }
  __shared__ float red[8][10][32];
#pragma unroll
  for (int i = 0; i < 10; ++i) red[pl][i][ci] = acc[i];
  __syncthreads();
  for (int i = threadIdx.x; i < 10 * 32; i += blockDim.x) {
    const int k = i / 32, c = i % 32;
    float s = 0.0f;
    for (int l = 0; l < 8; ++l) s += red[l][k][c];
    if (k < 9)
      atomicAdd(dw + k * kC0 + c, s);
    else if (c == 0)
      atomicAdd(db, s);
  }
}

// 2x2 average pooling, NHWC, 8 channels per thread.
__global__ void pool2_kernel(const bf16 *x, bf16 *out, int h, int wd, int c, long long nout8) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nout8) return;
  const int c8 = c / 8;
  const int cc = (int)(i % c8) * 8;
  const long long po = i / c8;
  const int ho = h / 2, wo = wd / 2;
  const long long img = po / ((long long)ho * wo);
  const int yo = (int)((po / wo) % ho), xo = (int)(po % wo);
  float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const long long pi = (img * h + 2 * yo + k / 2) * wd + 2 * xo + k % 2;
    const uint4 u = *reinterpret_cast<const uint4 *>(x + pi * c + cc);
    const unsigned e[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      s[2 * j] += __uint_as_float(e[j] << 16);
      s[2 * j + 1] += __uint_as_float(e[j] & 0xFFFF0000u);
    }
  }
  unsigned o[4];
#pragma unroll
  for (int j = 0; j < 4; ++j)
    o[j] = (unsigned)__bfloat16_as_ushort(__float2bfloat16_rn(0.25f * s[2 * j])) |
           ((unsigned)__bfloat16_as_ushort(__float2bfloat16_rn(0.25f * s[2 * j + 1])) << 16);
  *reinterpret_cast<uint4 *>(out + po * c + cc) = make_uint4(o[0], o[1], o[2], o[3]);
}

// out[p] = (skip[p] + g_low[p / 2] / 4) * (mask[p] > 0); skip may be null.
__global__ void pool2_bwd_kernel(const bf16 *g_low, const bf16 *skip, const bf16 *mask, bf16 *out, int h, int wd,
                                 int c, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int ch = (int)(i % c);
  const long long p = i / c;
  const long long img = p / ((long long)h * wd);
  const int y = (int)((p / wd) % h), x = (int)(p % wd);
  const long long pl = (img * (h / 2) + y / 2) * (wd / 2) + x / 2;
  float v = 0.25f * ld_bf(g_low + pl * c + ch);
  if (skip) v += ld_bf(skip + i);
  if (mask && !positive(mask[i])) v = 0.0f;
  out[i] = __float2bfloat16_rn(v);
}

// Nearest-neighbour 2x upsampling, NHWC, 8 channels per thread.
__global__ void up2_kernel(const bf16 *x, bf16 *out, int h, int wd, int c, long long nout8) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nout8) return;
  const int c8 = c / 8;
  const int cc = (int)(i % c8) * 8;
  const long long po = i / c8;
  const int ho = 2 * h, wo = 2 * wd;
  const long long img = po / ((long long)ho * wo);
  const int yo = (int)((po / wo) % ho), xo = (int)(po % wo);
  const long long pi = (img * h + yo / 2) * wd + xo / 2;
  *reinterpret_cast<uint4 *>(out + po * c + cc) = *reinterpret_cast<const uint4 *>(x + pi * c + cc);
}

// g_low[q] = (sum of the 2x2 block of g_high) * (mask[q] > 0); (h, wd) low-res.
__global__ void up2_bwd_kernel(const bf16 *g_high, const bf16 *mask, bf16 *out, int h, int wd, int c, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int ch = (int)(i % c);
  const long long q = i / c;
  const long long img = q / ((long long)h * wd);
  const int y = (int)((q / wd) % h), x = (int)(q % wd);
  float s = 0.0f;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const long long ph = (img * 2 * h + 2 * y + k / 2) * (2 * wd) + 2 * x + k % 2;
    s += ld_bf(g_high + ph * c + ch);
  }
  if (mask && !positive(mask[i])) s = 0.0f;
  out[i] = __float2bfloat16_rn(s);
}

// db[c] += sum_p g[p][c]; block = 256 threads = 8 pixel lanes x 32 channels,
// channel group blockIdx.y.
__global__ void bias_grad_kernel(const bf16 *g, float *db, int c, long long npix, int pix_per_block) {
  const int cl = threadIdx.x & 31, pl = threadIdx.x >> 5;
  const int ch = blockIdx.y * 32 + cl;
  const long long p0 = (long long)blockIdx.x * pix_per_block;
  const long long p1 = min(p0 + pix_per_block, npix);
  float s = 0.0f;
  for (long long p = p0 + pl; p < p1; p += 8) s += ld_bf(g + p * c + ch);
  __shared__ float red[8][32];
  red[pl][cl] = s;
  __syncthreads();
  if (pl == 0) {
    float t = 0.0f;
    for (int l = 0; l < 8; ++l) t += red[l][cl];
    atomicAdd(db + ch, t);
  }
}

// d = scale * out - target.
__global__ void diff_kernel(const float *out, const float *target, float scale, float *d, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) d[i] = scale * out[i] - target[i];
}

// Loss (alpha * d.d + mu * d.e) / n added to *loss, and its gradient with
// respect to out, g = 2 * scale * (alpha * d + mu * e) / n, where e is a
// symmetric positive semi-definite operator applied to d (e may be null).
__global__ void loss_grad_kernel(const float *d, const float *e, float alpha, float mu, float scale, float *g,
                                 float *loss, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0.0f;
  if (i < n) {
    const float di = d[i];
    const float ei = e ? e[i] : 0.0f;
    g[i] = 2.0f * scale * (alpha * di + mu * ei) / (float)n;
    l = (alpha * di * di + mu * di * ei) / (float)n;
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) l += __shfl_xor_sync(0xFFFFFFFFu, l, o);
  if ((threadIdx.x & 31) == 0 && loss) atomicAdd(loss, l);
}

// Fused Adam over the flat f32 parameter vector; conv-weight segments also
// write the bf16 forward copy [9][co][ci] and the input-gradient copy
// wt[8 - t][ci][co].  With update == 0 only the bf16 copies are written.
__global__ void adam_kernel(float *p, const float *g, float *m, float *v, const AdrtnetSegment *segs, int nseg,
                            long long n, float lr, float b1, float b2, float eps, const long long *step, int update,
                            bf16 *wbuf) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float w = p[i];
  if (update) {
    const float k = (float)*step;
    const float c1 = 1.0f - powf(b1, k), c2 = 1.0f - powf(b2, k);
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    p[i] = w;
  }
  int s = 0;
  while (s + 1 < nseg && segs[s + 1].offset <= i) ++s;
  const AdrtnetSegment sg = segs[s];
  if (sg.kind != ADRTNET_SEG_CONV || i >= sg.offset + sg.count) return;
  const long long k = i - sg.offset;
  const int ci = (int)(k % sg.c_in);
  const int co = (int)((k / sg.c_in) % sg.c_out);
  const int t = (int)(k / ((long long)sg.c_in * sg.c_out));
  const bf16 wb = __float2bfloat16_rn(w);
  wbuf[sg.w_offset + k] = wb;
  wbuf[sg.wt_offset + ((long long)(8 - t) * sg.c_in + ci) * sg.c_out + co] = wb;
}

}  // namespace net
}  // namespace adrtg

using namespace adrtg;
using namespace adrtg::net;

namespace {
inline cudaStream_t S(void *s) { return static_cast<cudaStream_t>(s); }
inline unsigned blocks(long long n, int t) { return (unsigned)((n + t - 1) / t); }
inline bool img_ok(long long batch, long long h, long long w) {
  return batch >= 1 && h >= 1 && w >= 1 && batch * h * w < (1ll << 40);
}
}  // namespace

extern "C" {

int adrtnet_conv_in(const float *u, const float *w, const float *b, void *out, int64_t batch, int64_t h, int64_t wd,
                    void *stream) {
  if (!u || !w || !b || !out) return ADRT_GB300_ERR_NULL;
  if (!img_ok(batch, h, wd)) return ADRT_GB300_ERR_SHAPE;
  const long long n = batch * h * wd;
  conv_in_kernel<<<blocks(n, 256), 256, 0, S(stream)>>>(u, w, b, static_cast<bf16 *>(out), (int)h, (int)wd, n);
  return launch_status();
}

int adrtnet_conv_in_wgrad(const float *u, const void *g, float *dw, float *db, int64_t batch, int64_t h,
                          int64_t wd, void *stream) {
  if (!u || !g || !dw || !db) return ADRT_GB300_ERR_NULL;
  if (!img_ok(batch, h, wd)) return ADRT_GB300_ERR_SHAPE;
  const long long n = batch * h * wd;
  const int per = 2048;
  conv_in_wgrad_kernel<<<blocks(n, per), 256, 0, S(stream)>>>(u, static_cast<const bf16 *>(g), dw, db, (int)h,
                                                               (int)wd, n, per);
  return launch_status();
}

int adrtnet_conv_out(const void *f, const float *w, const float *b, float *out, int64_t batch, int64_t h,
                     int64_t wd, void *stream) {
  if (!f || !w || !b || !out) return ADRT_GB300_ERR_NULL;
  if (!img_ok(batch, h, wd)) return ADRT_GB300_ERR_SHAPE;
  const long long n = batch * h * wd;
  conv_out_kernel<<<blocks(n, 256), 256, 0, S(stream)>>>(static_cast<const bf16 *>(f), w, b, out, (int)h, (int)wd,
                                                         n);
  return launch_status();
}

int adrtnet_conv_out_bwd(const float *g, const float *w, const void *f, void *dx, float *dw, float *db,
                         int64_t batch, int64_t h, int64_t wd, void *stream) {
  if (!g || !w || !f || !dx || !dw || !db) return ADRT_GB300_ERR_NULL;
  if (!img_ok(batch, h, wd)) return ADRT_GB300_ERR_SHAPE;
  const long long n = batch * h * wd;
  conv_out_dgrad_kernel<<<blocks(n, 256), 256, 0, S(stream)>>>(g, w, static_cast<const bf16 *>(f),
                                                                static_cast<bf16 *>(dx), (int)h, (int)wd, n);
  int rc = launch_status();
  if (rc) return rc;
  const int per = 2048;
  conv_out_wgrad_kernel<<<blocks(n, per), 256, 0, S(stream)>>>(g, static_cast<const bf16 *>(f), dw, db, (int)h,
                                                                (int)wd, n, per);
  return launch_status();
}

int adrtnet_pool2(const void *x, void *out, int64_t batch, int64_t h, int64_t wd, int c, void *stream) {
  if (!x || !out) return ADRT_GB300_ERR_NULL;
  if (!img_ok(batch, h, wd) || h % 2 || wd % 2 || c % 8) return ADRT_GB300_ERR_SHAPE;
  const long long n8 = batch * (h / 2) * (wd / 2) * (c / 8);
  pool2_kernel<<<blocks(n8, 256), 256, 0, S(stream)>>>(static_cast<const bf16 *>(x), static_cast<bf16 *>(out),
                                                       (int)h, (int)wd, c, n8);
  return launch_status();
}

int adrtnet_pool2_bwd(const void *g_low, const void *skip, const void *mask, void *out, int64_t batch, int64_t h,
                      int64_t wd, int c, void *stream) {
  if (!g_low || !out) return ADRT_GB300_ERR_NULL;
  if (!img_ok(batch, h, wd) || h % 2 || wd % 2 || c < 1) return ADRT_GB300_ERR_SHAPE;
  const long long n = batch * h * wd * c;
  pool2_bwd_kernel<<<blocks(n, 256), 256, 0, S(stream)>>>(
      static_cast<const bf16 *>(g_low), static_cast<const bf16 *>(skip), static_cast<const bf16 *>(mask),
      static_cast<bf16 *>(out), (int)h, (int)wd, c, n);
  return launch_status();
}

int adrtnet_up2(const void *x, void *out, int64_t batch, int64_t h, int64_t wd, int c, void *stream) {
  if (!x || !out) return ADRT_GB300_ERR_NULL;
  if (!img_ok(batch, h, wd) || c % 8) return ADRT_GB300_ERR_SHAPE;
  const long long n8 = batch * 4 * h * wd * (c / 8);
  up2_kernel<<<blocks(n8, 256), 256, 0, S(stream)>>>(static_cast<const bf16 *>(x), static_cast<bf16 *>(out), (int)h,
                                                     (int)wd, c, n8);
  return launch_status();
}

int adrtnet_up2_bwd(const void *g_high, const void *mask, void *out, int64_t batch, int64_t h, int64_t wd, int c,
                    void *stream) {
  if (!g_high || !out) return ADRT_GB300_ERR_NULL;
  if (!img_ok(batch, h, wd) || c < 1) return ADRT_GB300_ERR_SHAPE;
  const long long n = batch * h * wd * c;
  up2_bwd_kernel<<<blocks(n, 256), 256, 0, S(stream)>>>(static_cast<const bf16 *>(g_high),
                                                         static_cast<const bf16 *>(mask), static_cast<bf16 *>(out),
                                                         (int)h, (int)wd, c, n);
  return launch_status();
}

int adrtnet_bias_grad(const void *g, float *db, int64_t npix, int c, void *stream) {
  if (!g || !db) return ADRT_GB300_ERR_NULL;
  if (npix < 1 || c % 32) return ADRT_GB300_ERR_SHAPE;
  const int per = 2048;
  const dim3 grid(blocks(npix, per), (unsigned)(c / 32));
  bias_grad_kernel<<<grid, 256, 0, S(stream)>>>(static_cast<const bf16 *>(g), db, c, npix, per);
  return launch_status();
}

int adrtnet_diff(const float *out, const float *target, float scale, float *d, int64_t n, void *stream) {
  if (!out || !target || !d) return ADRT_GB300_ERR_NULL;
  if (n < 1) return ADRT_GB300_ERR_SHAPE;
  diff_kernel<<<blocks(n, 256), 256, 0, S(stream)>>>(out, target, scale, d, n);
  return launch_status();
}

int adrtnet_loss_grad(const float *d, const float *e, float alpha, float mu, float scale, float *g, float *loss,
                      int64_t n, void *stream) {
  if (!d || !g) return ADRT_GB300_ERR_NULL;
  if (n < 1) return ADRT_GB300_ERR_SHAPE;
  loss_grad_kernel<<<blocks(n, 256), 256, 0, S(stream)>>>(d, e, alpha, mu, scale, g, loss, n);
  return launch_status();
}

int adrtnet_adam(float *p, const float *g, float *m, float *v, const AdrtnetSegment *segs, int nseg, int64_t n,
                 float lr, float beta1, float beta2, float eps, const int64_t *step, int update, void *wbuf,
                 void *stream) {
  if (!p || !segs || !wbuf || (update && (!g || !m || !v || !step))) return ADRT_GB300_ERR_NULL;
  if (n < 1 || nseg < 1) return ADRT_GB300_ERR_SHAPE;
  adam_kernel<<<blocks(n, 256), 256, 0, S(stream)>>>(p, g, m, v, segs, nseg, n, lr, beta1, beta2, eps,
                                                     reinterpret_cast<const long long *>(step), update,
                                                     static_cast<bf16 *>(wbuf));
  return launch_status();
}

}  // extern "C"
