// Elementwise operations of the StyleGAN2-shaped generator used by the MaterialGAN latent loop
// (src/materialgan.py:91-173 drives the reference's generator, src/higan_models/*).
//
//   gen_upsample2_fwd_kernel  2x up-sampling of NCHW FP32 maps: zero insertion followed by the
//                             [1,3,3,1] x [1,3,3,1] / 64 FIR with gain 4 and zero padding, in
//                             polyphase form: out[2m] = (x[m-1] + 3 x[m]) / 4 and
//                             out[2m+1] = (3 x[m] + x[m+1]) / 4 along each axis
//   gen_upsample2_bwd_kernel  its adjoint: gx[m] = (g[2m-1] + 3 g[2m] + 3 g[2m+1] + g[2m+2]) / 4
//                             along each axis, g zero outside
//   gen_scale_*               a modulated conv's input scaling x s[b, c] and its adjoint
//                             (input gradient and the per-plane style gradient)
//   gen_act_*                 a style layer's epilogue lrelu(y d[b, c] + ns noise[b] + bias[c]) gain
//                             and its adjoint (input, demodulation and noise gradients)
//
// Per-plane reductions run one block per plane in a fixed order, so the gradients are
// deterministic.
// All are HBM-bound. Each has a float4 form (used when rows and planes hold multiples of 4
// floats and the maps are 16-byte aligned, as every map of the generator is) and a scalar form
// for other shapes; planes lie on the grid's second axis or one block per plane.
#include <cuda_runtime.h>
#include <stdint.h>

#include "svbrdf_common.cuh"

namespace svb {
namespace gen {

// Taps of output index o along one axis of length n (input) -> (lo, hi, wlo, whi).
__device__ __forceinline__ void up_taps(int o, int n, int& lo, int& hi, float& wlo, float& whi) {
  const int m = o >> 1;
  if (o & 1) {
    lo = m; hi = m + 1; wlo = 0.75f; whi = 0.25f;
  } else {
    lo = m - 1; hi = m; wlo = 0.25f; whi = 0.75f;
  }
  if (lo < 0) wlo = 0.0f, lo = 0;
  if (hi >= n) whi = 0.0f, hi = n - 1;
}

// grid: (ceil(2h w / 256), planes); thread i of a plane computes output row Y = i / w,
// columns 2m and 2m+1 with m = i % w.
__global__ void __launch_bounds__(256) gen_upsample2_fwd_kernel(const float* __restrict__ x, float* __restrict__ y,
                                                                int h, int w) {
  const int H = 2 * h, W = 2 * w;
  const int i = blockIdx.x * 256 + threadIdx.x;
  if (i >= H * w) return;
  const int Y = i / w, m = i - Y * w;
  const long long p = blockIdx.y;
  int y0, y1;
  float wy0, wy1;
  up_taps(Y, h, y0, y1, wy0, wy1);
  const float* r0p = x + (p * h + y0) * w;
  const float* r1p = x + (p * h + y1) * w;
  float* yp = y + (p * H + Y) * W;
  // output columns X = 2m, 2m+1 share input column m: out[2m] = (x[m-1] + 3 x[m]) / 4,
  // out[2m+1] = (3 x[m] + x[m+1]) / 4 (zero outside)
  const float a0 = m > 0 ? __ldg(r0p + m - 1) : 0.0f, b0 = __ldg(r0p + m), c0 = m + 1 < w ? __ldg(r0p + m + 1) : 0.0f;
  const float a1 = m > 0 ? __ldg(r1p + m - 1) : 0.0f, b1 = __ldg(r1p + m), c1 = m + 1 < w ? __ldg(r1p + m + 1) : 0.0f;
  const float r0e = 0.25f * a0 + 0.75f * b0, r0o = 0.75f * b0 + 0.25f * c0;
  const float r1e = 0.25f * a1 + 0.75f * b1, r1o = 0.75f * b1 + 0.25f * c1;
  *reinterpret_cast<float2*>(yp + 2 * m) = make_float2(wy0 * r0e + wy1 * r1e, wy0 * r0o + wy1 * r1o);
}

// Adjoint taps of input index m along one axis (output length 2n): outputs 2m-1 .. 2m+2 with
// weights 1/4, 3/4, 3/4, 1/4, those outside [0, 2n) dropped.
// grid: (ceil(h w / 256), planes); one thread per input element.
__global__ void __launch_bounds__(256) gen_upsample2_bwd_kernel(const float* __restrict__ g, float* __restrict__ gx,
                                                                int h, int w) {
  const int H = 2 * h, W = 2 * w;
  const int i = blockIdx.x * 256 + threadIdx.x;
  if (i >= h * w) return;
  const int ym = i / w, xm = i - ym * w;
  const long long p = blockIdx.y;
  const float* gp = g + p * H * W;
  const float wt[4] = {0.25f, 0.75f, 0.75f, 0.25f};
  float acc = 0.0f;
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const int Y = 2 * ym - 1 + a;
    if (Y < 0 || Y >= H) continue;
    const float* row = gp + (size_t)Y * W;
    const float2 mid = *reinterpret_cast<const float2*>(row + 2 * xm);  // columns 2m, 2m+1
    float r = 0.75f * (mid.x + mid.y);
    if (xm > 0) r = fmaf(0.25f, __ldg(row + 2 * xm - 1), r);
    if (xm + 1 < w) r = fmaf(0.25f, __ldg(row + 2 * xm + 2), r);
    acc = fmaf(wt[a], r, acc);
  }
  gx[(p * h + ym) * w + xm] = acc;
}

// ---------------------------------------------------------------- style modulation
// y[p][i] = x[p][i] s[p] over planes p = b C + c (the input scaling of a modulated conv).
__global__ void gen_scale_fwd_kernel(const float* __restrict__ x, const float* __restrict__ s, float* __restrict__ y,
                                     int hw) {
  const long long p = blockIdx.y;
  const float sv = __ldg(s + p);
  const float* xp = x + p * hw;
  float* yp = y + p * hw;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < hw; i += gridDim.x * blockDim.x) yp[i] = xp[i] * sv;
}

__device__ __forceinline__ float block_sum256(float v, float* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  float t = 0.0f;
  if (threadIdx.x == 0)
    for (int w = 0; w < 8; ++w) t += red[w];
  return t;
}

// gx = g s[p]; gs[p] = sum_i g x (one block per plane: a fixed-order sum).
__global__ void __launch_bounds__(256) gen_scale_bwd_kernel(const float* __restrict__ g, const float* __restrict__ x,
                                                            const float* __restrict__ s, float* __restrict__ gx,
                                                            float* __restrict__ gs, int hw) {
  __shared__ float red[8];
  const long long p = blockIdx.x;
  const float sv = __ldg(s + p);
  const float* gp = g + p * hw;
  const float* xp = x + p * hw;
  float* gxp = gx + p * hw;
  float acc = 0.0f;
  for (int i = threadIdx.x; i < hw; i += 256) {
    const float gv = gp[i];
    gxp[i] = gv * sv;
    acc = fmaf(gv, __ldg(xp + i), acc);
  }
  const float t = block_sum256(acc, red);
  if (threadIdx.x == 0) gs[p] = t;
}

// ---------------------------------------------------------------- style-layer epilogue
// out = lrelu(y d[p] + ns noise[b][i] + bias[c], 0.2) gain, p = b C + c. d, noise nullable.
__device__ __forceinline__ float act_pre(float y, float dv, float nz, float bias) { return fmaf(y, dv, nz) + bias; }

__global__ void gen_act_fwd_kernel(const float* __restrict__ y, const float* __restrict__ d,
                                   const float* __restrict__ noise, const float* __restrict__ ns,
                                   const float* __restrict__ bias, float gain, float* __restrict__ out, int C, int hw) {
  const long long p = blockIdx.y;
  const int b = (int)(p / C), c = (int)(p % C);
  const float dv = d ? __ldg(d + p) : 1.0f;
  const float nsv = noise ? __ldg(ns) : 0.0f;
  const float bv = __ldg(bias + c);
  const float* yp = y + p * hw;
  const float* np = noise ? noise + (long long)b * hw : nullptr;
  float* op = out + p * hw;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < hw; i += gridDim.x * blockDim.x) {
    const float pre = act_pre(yp[i], dv, np ? nsv * __ldg(np + i) : 0.0f, bv);
    op[i] = (pre > 0.0f ? pre : 0.2f * pre) * gain;
  }
}

// gy = gpre d[p]; gd[p] = sum_i gpre y (one block per plane), gpre = gout gain slope(pre).
__global__ void __launch_bounds__(256) gen_act_bwd_kernel(const float* __restrict__ gout, const float* __restrict__ y,
                                                          const float* __restrict__ d, const float* __restrict__ noise,
                                                          const float* __restrict__ ns, const float* __restrict__ bias,
                                                          float gain, float* __restrict__ gy, float* __restrict__ gd,
                                                          int C, int hw) {
  __shared__ float red[8];
  const long long p = blockIdx.x;
  const int b = (int)(p / C), c = (int)(p % C);
  const float dv = d ? __ldg(d + p) : 1.0f;
  const float nsv = noise ? __ldg(ns) : 0.0f;
  const float bv = __ldg(bias + c);
  const float* yp = y + p * hw;
  const float* gp = gout + p * hw;
  const float* np = noise ? noise + (long long)b * hw : nullptr;
  float* gyp = gy + p * hw;
  float acc = 0.0f;
  for (int i = threadIdx.x; i < hw; i += 256) {
    const float yv = yp[i];
    const float pre = act_pre(yv, dv, np ? nsv * __ldg(np + i) : 0.0f, bv);
    const float gpre = gp[i] * gain * (pre > 0.0f ? 1.0f : 0.2f);
    gyp[i] = gpre * dv;
    acc = fmaf(gpre, yv, acc);
  }
  if (gd) {
    const float t = block_sum256(acc, red);
    if (threadIdx.x == 0) gd[p] = t;
  }
}

// gnoise[b][i] = ns sum_c gpre(b, c, i).
__global__ void gen_act_noise_bwd_kernel(const float* __restrict__ gout, const float* __restrict__ y,
                                         const float* __restrict__ d, const float* __restrict__ noise,
                                         const float* __restrict__ ns, const float* __restrict__ bias, float gain,
                                         float* __restrict__ gnoise, int C, int hw) {
  const int b = blockIdx.y;
  const float nsv = __ldg(ns);
  const float* np = noise + (long long)b * hw;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < hw; i += gridDim.x * blockDim.x) {
    const float nz = nsv * __ldg(np + i);
    float acc = 0.0f;
    for (int c = 0; c < C; ++c) {
      const long long p = (long long)b * C + c;
      const float dv = d ? __ldg(d + p) : 1.0f;
      const float pre = act_pre(y[p * hw + i], dv, nz, __ldg(bias + c));
      acc = fmaf(gout[p * hw + i] * gain, pre > 0.0f ? 1.0f : 0.2f, acc);
    }
    gnoise[(long long)b * hw + i] = acc * nsv;
  }
}

// ---------------------------------------------------------------- float4 forms
// Used when every row (w) or plane (hw) holds a multiple of 4 floats and the pointers are
// 16-byte aligned (every map of the generator: planes are r x r with r >= 4). Each thread keeps
// 64 B or more in flight, which is what an HBM-bound elementwise kernel needs to approach the
// copy bandwidth (the scalar forms above keep 4-8 B per thread and reach about a quarter).

__device__ __forceinline__ float4 f4(float a, float b, float c, float d) { return make_float4(a, b, c, d); }

// One input row's 4 columns 4q..4q+3 up-sampled along x: 8 outputs (zero outside the row).
struct Row8 {
  float v[8];
};
__device__ __forceinline__ Row8 up_row8(const float* __restrict__ row, int q, int w) {
  const float4 c = __ldg(reinterpret_cast<const float4*>(row) + q);
  const float l = q > 0 ? __ldg(row + 4 * q - 1) : 0.0f;
  const float r = 4 * q + 4 < w ? __ldg(row + 4 * q + 4) : 0.0f;
  const float x[6] = {l, c.x, c.y, c.z, c.w, r};
  Row8 o;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    o.v[2 * j] = 0.25f * x[j] + 0.75f * x[j + 1];
    o.v[2 * j + 1] = 0.75f * x[j + 1] + 0.25f * x[j + 2];
  }
  return o;
}

// grid: (ceil(h w/4 / 256), planes); thread (k, q) writes output rows 2k, 2k+1, columns
// 8q..8q+7 from input rows k-1, k, k+1. Optional s scales plane p by s[p] (the modulation of
// an up-sampling conv, which commutes with the up-sampling).
__global__ void __launch_bounds__(256) gen_upsample2_fwd4_kernel(const float* __restrict__ x,
                                                                 const float* __restrict__ s, float* __restrict__ y,
                                                                 int h, int w) {
  const int w4 = w >> 2;
  const int i = blockIdx.x * 256 + threadIdx.x;
  if (i >= h * w4) return;
  const int k = i / w4, q = i - k * w4;
  const long long p = blockIdx.y;
  const float sc = s ? __ldg(s + p) : 1.0f;
  const float* xp = x + p * h * w;
  Row8 zero;
#pragma unroll
  for (int j = 0; j < 8; ++j) zero.v[j] = 0.0f;
  const Row8 a = k > 0 ? up_row8(xp + (size_t)(k - 1) * w, q, w) : zero;
  const Row8 b = up_row8(xp + (size_t)k * w, q, w);
  const Row8 c = k + 1 < h ? up_row8(xp + (size_t)(k + 1) * w, q, w) : zero;
  float e[8], o[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    e[j] = (0.25f * a.v[j] + 0.75f * b.v[j]) * sc;
    o[j] = (0.75f * b.v[j] + 0.25f * c.v[j]) * sc;
  }
  float4* ye = reinterpret_cast<float4*>(y + (p * 2 * h + 2 * k) * 2 * w) + 2 * q;
  float4* yo = ye + (w >> 1);
  ye[0] = f4(e[0], e[1], e[2], e[3]);
  ye[1] = f4(e[4], e[5], e[6], e[7]);
  yo[0] = f4(o[0], o[1], o[2], o[3]);
  yo[1] = f4(o[4], o[5], o[6], o[7]);
}

// grid: (ceil(h w/4 / 256), planes); thread (ym, q) forms input columns 4q..4q+3 of input row
// ym from output rows 2ym-1 .. 2ym+2, columns 8q-1 .. 8q+8.
__global__ void __launch_bounds__(256) gen_upsample2_bwd4_kernel(const float* __restrict__ g, float* __restrict__ gx,
                                                                 int h, int w) {
  const int w4 = w >> 2, H = 2 * h, W = 2 * w;
  const int i = blockIdx.x * 256 + threadIdx.x;
  if (i >= h * w4) return;
  const int ym = i / w4, q = i - ym * w4;
  const long long p = blockIdx.y;
  const float* gp = g + p * H * W;
  const float wt[4] = {0.25f, 0.75f, 0.75f, 0.25f};
  float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const int Y = 2 * ym - 1 + a;
    if (Y < 0 || Y >= H) continue;
    const float* row = gp + (size_t)Y * W;
    const float4 c0 = __ldg(reinterpret_cast<const float4*>(row) + 2 * q);
    const float4 c1 = __ldg(reinterpret_cast<const float4*>(row) + 2 * q + 1);
    const float l = q > 0 ? __ldg(row + 8 * q - 1) : 0.0f;
    const float r = 8 * q + 8 < W ? __ldg(row + 8 * q + 8) : 0.0f;
    const float G[10] = {l, c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w, r};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const float v = 0.25f * G[2 * j] + 0.75f * (G[2 * j + 1] + G[2 * j + 2]) + 0.25f * G[2 * j + 3];
      acc[j] = fmaf(wt[a], v, acc[j]);
    }
  }
  reinterpret_cast<float4*>(gx + p * h * w)[i] = f4(acc[0], acc[1], acc[2], acc[3]);
}

constexpr int kU = 4;  // float4 per thread per pass of the streaming kernels

__global__ void __launch_bounds__(256) gen_scale_fwd4_kernel(const float4* __restrict__ x, const float* __restrict__ s,
                                                             float4* __restrict__ y, int hw4) {
  const long long p = blockIdx.y;
  const float sv = __ldg(s + p);
  const float4* xp = x + p * hw4;
  float4* yp = y + p * hw4;
  for (int i0 = blockIdx.x * 256 * kU + threadIdx.x; i0 < hw4; i0 += gridDim.x * 256 * kU) {
    float4 v[kU];
#pragma unroll
    for (int u = 0; u < kU; ++u)
      if (i0 + u * 256 < hw4) v[u] = __ldg(xp + i0 + u * 256);
#pragma unroll
    for (int u = 0; u < kU; ++u)
      if (i0 + u * 256 < hw4) yp[i0 + u * 256] = f4(v[u].x * sv, v[u].y * sv, v[u].z * sv, v[u].w * sv);
  }
}

__global__ void __launch_bounds__(256) gen_scale_bwd4_kernel(const float4* __restrict__ g, const float4* __restrict__ x,
                                                             const float* __restrict__ s, float4* __restrict__ gx,
                                                             float* __restrict__ gs, int hw4) {
  __shared__ float red[8];
  const long long p = blockIdx.x;
  const float sv = __ldg(s + p);
  const float4* gp = g + p * hw4;
  const float4* xp = x + p * hw4;
  float4* gxp = gx + p * hw4;
  float acc = 0.0f;
  for (int i0 = threadIdx.x; i0 < hw4; i0 += 256 * 2) {
    float4 gv[2], xv[2];
#pragma unroll
    for (int u = 0; u < 2; ++u)
      if (i0 + u * 256 < hw4) gv[u] = __ldg(gp + i0 + u * 256), xv[u] = __ldg(xp + i0 + u * 256);
#pragma unroll
    for (int u = 0; u < 2; ++u)
      if (i0 + u * 256 < hw4) {
        gxp[i0 + u * 256] = f4(gv[u].x * sv, gv[u].y * sv, gv[u].z * sv, gv[u].w * sv);
        acc = fmaf(gv[u].x, xv[u].x, acc);
        acc = fmaf(gv[u].y, xv[u].y, acc);
        acc = fmaf(gv[u].z, xv[u].z, acc);
        acc = fmaf(gv[u].w, xv[u].w, acc);
      }
  }
  const float t = block_sum256(acc, red);
  if (threadIdx.x == 0) gs[p] = t;
}

__device__ __forceinline__ float lrelu_gain(float pre, float gain) { return (pre > 0.0f ? pre : 0.2f * pre) * gain; }

__global__ void __launch_bounds__(256) gen_act_fwd4_kernel(const float4* __restrict__ y, const float* __restrict__ d,
                                                           const float4* __restrict__ noise,
                                                           const float* __restrict__ ns,
                                                           const float* __restrict__ bias, float gain,
                                                           float4* __restrict__ out, int C, int hw4) {
  const long long p = blockIdx.y;
  const int b = (int)(p / C), c = (int)(p % C);
  const float dv = d ? __ldg(d + p) : 1.0f;
  const float nsv = noise ? __ldg(ns) : 0.0f;
  const float bv = __ldg(bias + c);
  const float4* yp = y + p * hw4;
  const float4* np = noise ? noise + (long long)b * hw4 : nullptr;
  float4* op = out + p * hw4;
  for (int i0 = blockIdx.x * 256 * kU + threadIdx.x; i0 < hw4; i0 += gridDim.x * 256 * kU) {
    float4 v[kU], n[kU];
#pragma unroll
    for (int u = 0; u < kU; ++u)
      if (i0 + u * 256 < hw4) {
        v[u] = __ldg(yp + i0 + u * 256);
        n[u] = np ? __ldg(np + i0 + u * 256) : f4(0.0f, 0.0f, 0.0f, 0.0f);
      }
#pragma unroll
    for (int u = 0; u < kU; ++u)
      if (i0 + u * 256 < hw4)
        op[i0 + u * 256] = f4(lrelu_gain(act_pre(v[u].x, dv, nsv * n[u].x, bv), gain),
                              lrelu_gain(act_pre(v[u].y, dv, nsv * n[u].y, bv), gain),
                              lrelu_gain(act_pre(v[u].z, dv, nsv * n[u].z, bv), gain),
                              lrelu_gain(act_pre(v[u].w, dv, nsv * n[u].w, bv), gain));
  }
}

__device__ __forceinline__ float act_gpre(float go, float yv, float dv, float nz, float bv, float gain) {
  return go * gain * (act_pre(yv, dv, nz, bv) > 0.0f ? 1.0f : 0.2f);
}

__global__ void __launch_bounds__(256) gen_act_bwd4_kernel(const float4* __restrict__ gout, const float4* __restrict__ y,
                                                           const float* __restrict__ d,
                                                           const float4* __restrict__ noise,
                                                           const float* __restrict__ ns,
                                                           const float* __restrict__ bias, float gain,
                                                           float4* __restrict__ gy, float* __restrict__ gd, int C,
                                                           int hw4) {
  __shared__ float red[8];
  const long long p = blockIdx.x;
  const int b = (int)(p / C), c = (int)(p % C);
  const float dv = d ? __ldg(d + p) : 1.0f;
  const float nsv = noise ? __ldg(ns) : 0.0f;
  const float bv = __ldg(bias + c);
  const float4* yp = y + p * hw4;
  const float4* gp = gout + p * hw4;
  const float4* np = noise ? noise + (long long)b * hw4 : nullptr;
  float4* gyp = gy + p * hw4;
  float acc = 0.0f;
  for (int i0 = threadIdx.x; i0 < hw4; i0 += 256 * 2) {
    float4 gv[2], yv[2], nv[2];
#pragma unroll
    for (int u = 0; u < 2; ++u)
      if (i0 + u * 256 < hw4) {
        gv[u] = __ldg(gp + i0 + u * 256);
        yv[u] = __ldg(yp + i0 + u * 256);
        nv[u] = np ? __ldg(np + i0 + u * 256) : f4(0.0f, 0.0f, 0.0f, 0.0f);
      }
#pragma unroll
    for (int u = 0; u < 2; ++u)
      if (i0 + u * 256 < hw4) {
        const float a0 = act_gpre(gv[u].x, yv[u].x, dv, nsv * nv[u].x, bv, gain);
        const float a1 = act_gpre(gv[u].y, yv[u].y, dv, nsv * nv[u].y, bv, gain);
        const float a2 = act_gpre(gv[u].z, yv[u].z, dv, nsv * nv[u].z, bv, gain);
        const float a3 = act_gpre(gv[u].w, yv[u].w, dv, nsv * nv[u].w, bv, gain);
        gyp[i0 + u * 256] = f4(a0 * dv, a1 * dv, a2 * dv, a3 * dv);
        acc = fmaf(a0, yv[u].x, acc);
        acc = fmaf(a1, yv[u].y, acc);
        acc = fmaf(a2, yv[u].z, acc);
        acc = fmaf(a3, yv[u].w, acc);
      }
  }
  if (gd) {
    const float t = block_sum256(acc, red);
    if (threadIdx.x == 0) gd[p] = t;
  }
}

// grid: (ceil(hw4 / TX), B), 256 threads as TY = 256 / TX rows of TX columns: column tx owns
// float4 i = blockIdx.x TX + tx, row ty sums channels ty, ty + TY, ... (4 channels' loads in
// flight), and row 0 adds the rows' sums in order, so the sum is deterministic. TX = 32 for
// large maps; small maps (hw4 < 32) take TX = hw4 so their many channels spread over rows.
__global__ void __launch_bounds__(256) gen_act_noise_bwd4_kernel(const float4* __restrict__ gout,
                                                                 const float4* __restrict__ y,
                                                                 const float* __restrict__ d,
                                                                 const float4* __restrict__ noise,
                                                                 const float* __restrict__ ns,
                                                                 const float* __restrict__ bias, float gain,
                                                                 float4* __restrict__ gnoise, int C, int hw4, int TX) {
  __shared__ float4 red[256];
  const int TY = 256 / TX;
  const int t = threadIdx.x, tx = t % TX, ty = t / TX;
  const int b = blockIdx.y;
  const int i = blockIdx.x * TX + tx;
  const bool active = ty < TY && i < hw4;
  const float nsv = __ldg(ns);
  float4 acc = f4(0.0f, 0.0f, 0.0f, 0.0f);
  if (active) {
    const float4 nv = __ldg(noise + (long long)b * hw4 + i);
    const float n0 = nsv * nv.x, n1 = nsv * nv.y, n2 = nsv * nv.z, n3 = nsv * nv.w;
    const long long p0 = (long long)b * C;
    for (int c0 = ty; c0 < C; c0 += 4 * TY) {
      float4 gv[4], yv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int c = c0 + u * TY;
        if (c < C) gv[u] = __ldg(gout + (p0 + c) * hw4 + i), yv[u] = __ldg(y + (p0 + c) * hw4 + i);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int c = c0 + u * TY;
        if (c < C) {
          const float dv = d ? __ldg(d + p0 + c) : 1.0f, bv = __ldg(bias + c);
          acc.x += act_gpre(gv[u].x, yv[u].x, dv, n0, bv, gain);
          acc.y += act_gpre(gv[u].y, yv[u].y, dv, n1, bv, gain);
          acc.z += act_gpre(gv[u].z, yv[u].z, dv, n2, bv, gain);
          acc.w += act_gpre(gv[u].w, yv[u].w, dv, n3, bv, gain);
        }
      }
    }
  }
  red[t] = acc;
  __syncthreads();
  if (ty == 0 && i < hw4) {
    float4 sum = red[tx];
    for (int r = 1; r < TY; ++r) {
      const float4 v = red[r * TX + tx];
      sum.x += v.x, sum.y += v.y, sum.z += v.z, sum.w += v.w;
    }
    gnoise[(long long)b * hw4 + i] = f4(sum.x * nsv, sum.y * nsv, sum.z * nsv, sum.w * nsv);
  }
}

}  // namespace gen
}  // namespace svb

using namespace svb;

extern "C" {

static bool al16(const void* p) { return p == nullptr || (uintptr_t)p % 16 == 0; }

int svbrdf_gen_upsample2(const float* x, float* y, long long planes, int h, int w, void* stream) {
  return svbrdf_gen_upsample2_scaled(x, nullptr, y, planes, h, w, stream);
}

int svbrdf_gen_upsample2_scaled(const float* x, const float* s, float* y, long long planes, int h, int w,
                                void* stream) {
  if (!x || !y || planes < 1 || h < 1 || w < 1) return fail(SVBRDF_ERR_INVALID, "upsample2: bad arguments");
  if (planes > 65535 || 2LL * h * w > (1LL << 30)) return fail(SVBRDF_ERR_UNSUPPORTED, "upsample2: too large");
  cudaStream_t st = (cudaStream_t)stream;
  if (w % 4 == 0 && al16(x) && al16(y)) {
    dim3 grid((unsigned)(((long long)h * (w / 4) + 255) / 256), (unsigned)planes);
    gen::gen_upsample2_fwd4_kernel<<<grid, 256, 0, st>>>(x, s, y, h, w);
    return check_launch("gen_upsample2_fwd4_kernel");
  }
  if (s) return fail(SVBRDF_ERR_UNSUPPORTED, "upsample2: scaling needs w % 4 == 0 and 16-byte aligned maps");
  if ((uintptr_t)y % 8) return fail(SVBRDF_ERR_INVALID, "upsample2: y must be 8-byte aligned");
  dim3 grid((unsigned)((2LL * h * w + 255) / 256), (unsigned)planes);
  gen::gen_upsample2_fwd_kernel<<<grid, 256, 0, st>>>(x, y, h, w);
  return check_launch("gen_upsample2_fwd_kernel");
}

int svbrdf_gen_upsample2_bwd(const float* g, float* gx, long long planes, int h, int w, void* stream) {
  if (!g || !gx || planes < 1 || h < 1 || w < 1) return fail(SVBRDF_ERR_INVALID, "upsample2_bwd: bad arguments");
  if (planes > 65535 || (long long)h * w > (1LL << 30)) return fail(SVBRDF_ERR_UNSUPPORTED, "upsample2_bwd: too large");
  cudaStream_t st = (cudaStream_t)stream;
  if (w % 4 == 0 && al16(g) && al16(gx)) {
    dim3 grid((unsigned)(((long long)h * (w / 4) + 255) / 256), (unsigned)planes);
    gen::gen_upsample2_bwd4_kernel<<<grid, 256, 0, st>>>(g, gx, h, w);
    return check_launch("gen_upsample2_bwd4_kernel");
  }
  if ((uintptr_t)g % 8) return fail(SVBRDF_ERR_INVALID, "upsample2_bwd: g must be 8-byte aligned");
  dim3 grid((unsigned)(((long long)h * w + 255) / 256), (unsigned)planes);
  gen::gen_upsample2_bwd_kernel<<<grid, 256, 0, st>>>(g, gx, h, w);
  return check_launch("gen_upsample2_bwd_kernel");
}

static dim3 plane_grid(int n, long long planes, int per_block) {
  const int bx = (n + per_block - 1) / per_block;
  return dim3((unsigned)(bx < 64 ? bx : 64), (unsigned)planes);
}

int svbrdf_gen_scale(const float* x, const float* s, float* y, long long planes, int hw, void* stream) {
  if (!x || !s || !y || planes < 1 || planes > 65535 || hw < 1) return fail(SVBRDF_ERR_INVALID, "scale: bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  if (hw % 4 == 0 && al16(x) && al16(y)) {
    gen::gen_scale_fwd4_kernel<<<plane_grid(hw / 4, planes, 256 * gen::kU), 256, 0, st>>>(
        reinterpret_cast<const float4*>(x), s, reinterpret_cast<float4*>(y), hw / 4);
    return check_launch("gen_scale_fwd4_kernel");
  }
  gen::gen_scale_fwd_kernel<<<plane_grid(hw, planes, 256), 256, 0, st>>>(x, s, y, hw);
  return check_launch("gen_scale_fwd_kernel");
}

int svbrdf_gen_scale_bwd(const float* g, const float* x, const float* s, float* gx, float* gs, long long planes, int hw,
                         void* stream) {
  if (!g || !x || !s || !gx || !gs || planes < 1 || planes > 0x7fffffffLL || hw < 1)
    return fail(SVBRDF_ERR_INVALID, "scale_bwd: bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  if (hw % 4 == 0 && al16(g) && al16(x) && al16(gx)) {
    gen::gen_scale_bwd4_kernel<<<(unsigned)planes, 256, 0, st>>>(reinterpret_cast<const float4*>(g),
                                                                 reinterpret_cast<const float4*>(x), s,
                                                                 reinterpret_cast<float4*>(gx), gs, hw / 4);
    return check_launch("gen_scale_bwd4_kernel");
  }
  gen::gen_scale_bwd_kernel<<<(unsigned)planes, 256, 0, st>>>(g, x, s, gx, gs, hw);
  return check_launch("gen_scale_bwd_kernel");
}

int svbrdf_gen_act(const float* y, const float* d, const float* noise, const float* ns, const float* bias, float gain,
                   float* out, int b, int c, int hw, void* stream) {
  if (!y || !bias || !out || (noise && !ns) || b < 1 || c < 1 || hw < 1 || (long long)b * c > 65535)
    return fail(SVBRDF_ERR_INVALID, "act: bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  if (hw % 4 == 0 && al16(y) && al16(noise) && al16(out)) {
    gen::gen_act_fwd4_kernel<<<plane_grid(hw / 4, (long long)b * c, 256 * gen::kU), 256, 0, st>>>(
        reinterpret_cast<const float4*>(y), d, reinterpret_cast<const float4*>(noise), ns, bias, gain,
        reinterpret_cast<float4*>(out), c, hw / 4);
    return check_launch("gen_act_fwd4_kernel");
  }
  gen::gen_act_fwd_kernel<<<plane_grid(hw, (long long)b * c, 256), 256, 0, st>>>(y, d, noise, ns, bias, gain, out, c,
                                                                                 hw);
  return check_launch("gen_act_fwd_kernel");
}

int svbrdf_gen_act_bwd(const float* gout, const float* y, const float* d, const float* noise, const float* ns,
                       const float* bias, float gain, float* gy, float* gd, float* gnoise, int b, int c, int hw,
                       void* stream) {
  if (!gout || !y || !bias || !gy || (noise && !ns) || (gnoise && !noise) || b < 1 || c < 1 || hw < 1 ||
      b > 65535)
    return fail(SVBRDF_ERR_INVALID, "act_bwd: bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  const bool v4 = hw % 4 == 0 && al16(gout) && al16(y) && al16(noise) && al16(gy) && al16(gnoise);
  int rc;
  if (v4) {
    gen::gen_act_bwd4_kernel<<<(unsigned)((long long)b * c), 256, 0, st>>>(
        reinterpret_cast<const float4*>(gout), reinterpret_cast<const float4*>(y), d,
        reinterpret_cast<const float4*>(noise), ns, bias, gain, reinterpret_cast<float4*>(gy), gd, c, hw / 4);
    rc = check_launch("gen_act_bwd4_kernel");
  } else {
    gen::gen_act_bwd_kernel<<<(unsigned)((long long)b * c), 256, 0, st>>>(gout, y, d, noise, ns, bias, gain, gy, gd,
                                                                          c, hw);
    rc = check_launch("gen_act_bwd_kernel");
  }
  if (rc || !gnoise) return rc;
  if (v4) {
    const int hw4 = hw / 4, tx = hw4 < 32 ? hw4 : 32;
    dim3 grid((unsigned)((hw4 + tx - 1) / tx), (unsigned)b);
    gen::gen_act_noise_bwd4_kernel<<<grid, 256, 0, st>>>(
        reinterpret_cast<const float4*>(gout), reinterpret_cast<const float4*>(y), d,
        reinterpret_cast<const float4*>(noise), ns, bias, gain, reinterpret_cast<float4*>(gnoise), c, hw4, tx);
    return check_launch("gen_act_noise_bwd4_kernel");
  }
  const int bx = (hw + 255) / 256;
  gen::gen_act_noise_bwd_kernel<<<dim3((unsigned)(bx < 256 ? bx : 256), (unsigned)b), 256, 0, st>>>(
      gout, y, d, noise, ns, bias, gain, gnoise, c, hw);
  return check_launch("gen_act_noise_bwd_kernel");
}

}  // extern "C"
