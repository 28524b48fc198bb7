// Channels-last (NHWC) forms of the generator's elementwise work, so that the generator's
// activations stay in the layout cuDNN's convolutions run in and need no NCHW<->NHWC
// conversions around each convolution (src/materialgan.py:91-173 drives the reference's
// generator, src/higan_models/*). Maps are [B][H][W][C], C contiguous.
//
//   nhwc_up_fwd_kernel     2x up-sampling (zero insertion + [1,3,3,1]^2 / 64 FIR, gain 4, zero
//                          padding) of x, optionally times s[b][c]: out[2m] = (x[m-1] + 3 x[m]) / 4,
//                          out[2m+1] = (3 x[m] + x[m+1]) / 4 along each axis; with a halo of one,
//                          also the samples at -1 and 2n (x[0] / 4 and x[n-1] / 4), which a valid
//                          3x3 convolution of the result needs to equal the reference's transposed
//                          convolution followed by the filter (src/higan_models/
//                          stylegan2_generator_network.py:727-735)
//   nhwc_up_bwd_kernel     its adjoint: gx[m] = (g[2m-1] + 3 g[2m] + 3 g[2m+1] + g[2m+2]) / 4 per axis
//   nhwc_scale_fwd_kernel  y = x s[b][c]
//   nhwc_scale_bwd_kernel  gx = g s[b][c] and per-chunk column sums of g x (the style gradient)
//   nhwc_act_fwd_kernel    out = lrelu(y d[b][c] + ns noise[b][p] + bias[c], 0.2) gain
//   nhwc_act_bwd_kernel    gy = gpre d, per-chunk column sums of gpre y (the demodulation
//                          gradient) and gnoise[b][p] = ns sum_c gpre
//   nhwc_colsum_kernel     the column sums' second pass: chunks added in order
//
// VEC = 4 (float4 over channels) when C % 4 == 0 and the maps are 16-byte aligned, else 1.
// Grids put a map row or a batch entry on the second axis, so index math stays 32-bit; the
// streaming and column-sum kernels keep kU vectors per thread in flight. The column sums are
// two-pass with a fixed order, so the gradients are deterministic.
#include <cuda_runtime.h>
#include <stdint.h>

#include "svbrdf_common.cuh"

namespace svb {
namespace gen_nhwc {

constexpr int kMaxChunks = 64;  // column-sum chunks per batch entry (partials: B x 64 x C floats)

template <int VEC>
__device__ __forceinline__ void ldv(const float* p, float (&v)[VEC]) {
  if constexpr (VEC == 4) {
    const float4 t = __ldg(reinterpret_cast<const float4*>(p));
    v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
  } else {
    v[0] = __ldg(p);
  }
}

template <int VEC>
__device__ __forceinline__ void stv(float* p, const float (&v)[VEC]) {
  if constexpr (VEC == 4) {
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
  } else {
    p[0] = v[0];
  }
}

// Taps of output index o along an axis of input length n -> (lo, hi, wlo, whi).
__device__ __forceinline__ void taps(int o, int n, int& lo, int& hi, float& wlo, float& whi) {
  const int m = o >> 1;
  if (o & 1) {
    lo = m; hi = m + 1; wlo = 0.75f; whi = 0.25f;
  } else {
    lo = m - 1; hi = m; wlo = 0.25f; whi = 0.75f;
  }
  if (lo < 0) wlo = 0.0f, lo = 0;
  if (hi >= n) whi = 0.0f, hi = n - 1;
}

__device__ __forceinline__ float act_pre(float y, float dv, float nz, float bias) { return fmaf(y, dv, nz) + bias; }

// grid (min(ceil(W2 cv / 256), 8), B H2), W2 = 2w + 2 halo: block row (b, Y); thread t of the
// row is output vector (X, c) = (t / cv, t % cv), at up-sampled index X - halo, for t stepping
// by the row's threads. 32-bit index math within a row.
template <int VEC>
__global__ void __launch_bounds__(256) nhwc_up_fwd_kernel(const float* __restrict__ x, const float* __restrict__ s,
                                                          float* __restrict__ y, int h, int w, int C, int halo) {
  const int cv = C / VEC, W2 = 2 * w + 2 * halo, H2 = 2 * h + 2 * halo;
  const int Y = blockIdx.y % H2, b = blockIdx.y / H2;
  int y0, y1;
  float wy0, wy1;
  taps(Y - halo, h, y0, y1, wy0, wy1);
  const float* r0 = x + ((long long)b * h + y0) * w * C;
  const float* r1 = x + ((long long)b * h + y1) * w * C;
  const float* sb = s ? s + (long long)b * C : nullptr;
  float* out = y + (long long)blockIdx.y * W2 * C;
#pragma unroll 2
  for (int t = blockIdx.x * 256 + threadIdx.x; t < W2 * cv; t += gridDim.x * 256) {
    const int c = t % cv, X = t / cv;
    int x0, x1;
    float wx0, wx1;
    taps(X - halo, w, x0, x1, wx0, wx1);
    float a[VEC], bq[VEC], cq[VEC], d[VEC], o[VEC];
    ldv<VEC>(r0 + x0 * C + c * VEC, a);
    ldv<VEC>(r0 + x1 * C + c * VEC, bq);
    ldv<VEC>(r1 + x0 * C + c * VEC, cq);
    ldv<VEC>(r1 + x1 * C + c * VEC, d);
#pragma unroll
    for (int j = 0; j < VEC; ++j) o[j] = wy0 * (wx0 * a[j] + wx1 * bq[j]) + wy1 * (wx0 * cq[j] + wx1 * d[j]);
    if (sb) {
      float sv[VEC];
      ldv<VEC>(sb + c * VEC, sv);
#pragma unroll
      for (int j = 0; j < VEC; ++j) o[j] *= sv[j];
    }
    stv<VEC>(out + t * VEC, o);
  }
}

// grid (ceil(w cv / 256), B h): block row (b, ym); thread t is input vector (xm, c), summed
// from output rows 2ym-1 .. 2ym+2 and columns 2xm-1 .. 2xm+2 (up-sampled indices; g holds
// them from -halo on).
template <int VEC>
__global__ void __launch_bounds__(256) nhwc_up_bwd_kernel(const float* __restrict__ g, float* __restrict__ gx, int h,
                                                          int w, int C, int halo) {
  const int cv = C / VEC, H = 2 * h + 2 * halo, W = 2 * w + 2 * halo;
  const int ym = blockIdx.y % h, b = blockIdx.y / h;
  const float wt[4] = {0.25f, 0.75f, 0.75f, 0.25f};
  const float* gb = g + (long long)b * H * W * C;
  float* out = gx + (long long)blockIdx.y * w * C;
  for (int t = blockIdx.x * 256 + threadIdx.x; t < w * cv; t += gridDim.x * 256) {
    const int c = t % cv, xm = t / cv;
    float acc[VEC];
#pragma unroll
    for (int j = 0; j < VEC; ++j) acc[j] = 0.0f;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      const int Yr = 2 * ym - 1 + a + halo;
      if (Yr < 0 || Yr >= H) continue;
      const float* row = gb + (long long)Yr * W * C + c * VEC;
      float r[VEC];
#pragma unroll
      for (int j = 0; j < VEC; ++j) r[j] = 0.0f;
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int Xc = 2 * xm - 1 + e + halo;
        if (Xc < 0 || Xc >= W) continue;
        float tv[VEC];
        ldv<VEC>(row + Xc * C, tv);
#pragma unroll
        for (int j = 0; j < VEC; ++j) r[j] = fmaf(wt[e], tv[j], r[j]);
      }
#pragma unroll
      for (int j = 0; j < VEC; ++j) acc[j] = fmaf(wt[a], r[j], acc[j]);
    }
    stv<VEC>(out + t * VEC, acc);
  }
}

constexpr int kU = 4;  // vectors per thread per pass of the streaming kernels

// grid (ceil(HW cv / (256 kU)), B): block column b; vector t of entry b is (p, c) = (t / cv, t % cv).
template <int VEC>
__global__ void __launch_bounds__(256) nhwc_scale_fwd_kernel(const float* __restrict__ x, const float* __restrict__ s,
                                                             float* __restrict__ y, int HW, int C) {
  const int cv = C / VEC, n = HW * cv, b = blockIdx.y;
  const float* xb = x + (long long)b * HW * C;
  float* yb = y + (long long)b * HW * C;
  const float* sb = s + (long long)b * C;
  for (int t0 = blockIdx.x * 256 * kU + threadIdx.x; t0 < n; t0 += gridDim.x * 256 * kU) {
    float v[kU][VEC];
#pragma unroll
    for (int u = 0; u < kU; ++u)
      if (t0 + u * 256 < n) ldv<VEC>(xb + (t0 + u * 256) * VEC, v[u]);
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const int t = t0 + u * 256;
      if (t < n) {
        float sv[VEC];
        ldv<VEC>(sb + (t % cv) * VEC, sv);
#pragma unroll
        for (int j = 0; j < VEC; ++j) v[u][j] *= sv[j];
        stv<VEC>(yb + t * VEC, v[u]);
      }
    }
  }
}

// The block's column sums: thread (r, c) holds acc for channel vector c over its rows; row 0
// adds the rows in order and stores partial[b][chunk][c * VEC + j].
template <int VEC>
__device__ __forceinline__ void column_partials(const float (&acc)[VEC], float* red, int cv, int rows, float* part,
                                                int C, int nchunk) {
  const int tid = threadIdx.x;
#pragma unroll
  for (int j = 0; j < VEC; ++j) red[tid * VEC + j] = acc[j];
  __syncthreads();
  if (tid < cv) {
    float* out = part + ((long long)blockIdx.y * nchunk + blockIdx.x) * C + tid * VEC;
#pragma unroll
    for (int j = 0; j < VEC; ++j) {
      float sum = 0.0f;
      for (int r = 0; r < rows; ++r) sum += red[(r * cv + tid) * VEC + j];
      out[j] = sum;
    }
  }
}

// grid (nchunk, B), 256 threads as rows = 256 / cv rows of cv channel vectors; block
// (chunk, b) takes pixels [chunk * per, (chunk + 1) * per) of entry b, kU pixels per thread
// per step.
template <int VEC>
__global__ void __launch_bounds__(256) nhwc_scale_bwd_kernel(const float* __restrict__ g, const float* __restrict__ x,
                                                             const float* __restrict__ s, float* __restrict__ gx,
                                                             float* __restrict__ part, int HW, int C, int nchunk) {
  __shared__ float red[256 * VEC];
  const int cv = C / VEC, rows = 256 / cv;
  const int tid = threadIdx.x, c = tid % cv, r = tid / cv;
  const int b = blockIdx.y;
  const int per = (HW + nchunk - 1) / nchunk;
  const int p0 = blockIdx.x * per, p1 = min(HW, p0 + per);
  float acc[VEC];
#pragma unroll
  for (int j = 0; j < VEC; ++j) acc[j] = 0.0f;
  if (r < rows) {
    float sv[VEC];
    ldv<VEC>(s + (long long)b * C + c * VEC, sv);
    const float* gb = g + (long long)b * HW * C + c * VEC;
    const float* xb = x + (long long)b * HW * C + c * VEC;
    float* ob = gx + (long long)b * HW * C + c * VEC;
    for (int pb = p0 + r; pb < p1; pb += kU * rows) {
      float gv[kU][VEC], xv[kU][VEC];
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        const int p = pb + u * rows;
        if (p < p1) {
          ldv<VEC>(gb + (long long)p * C, gv[u]);
          ldv<VEC>(xb + (long long)p * C, xv[u]);
        }
      }
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        const int p = pb + u * rows;
        if (p < p1) {
          float o[VEC];
#pragma unroll
          for (int j = 0; j < VEC; ++j) {
            o[j] = gv[u][j] * sv[j];
            acc[j] = fmaf(gv[u][j], xv[u][j], acc[j]);
          }
          stv<VEC>(ob + (long long)p * C, o);
        }
      }
    }
  }
  column_partials<VEC>(acc, red, cv, rows, part, C, nchunk);
}

// grid (ceil(HW cv / (256 kU)), B) as nhwc_scale_fwd_kernel.
template <int VEC>
__global__ void __launch_bounds__(256) nhwc_act_fwd_kernel(const float* __restrict__ y, const float* __restrict__ d,
                                                           const float* __restrict__ noise,
                                                           const float* __restrict__ ns,
                                                           const float* __restrict__ bias, float gain,
                                                           const float* __restrict__ s2, float* __restrict__ out,
                                                           int HW, int C) {
  const int cv = C / VEC, n = HW * cv, b = blockIdx.y;
  const float nsv = noise ? __ldg(ns) : 0.0f;
  const float* yb = y + (long long)b * HW * C;
  float* ob = out + (long long)b * HW * C;
  const float* db = d ? d + (long long)b * C : nullptr;
  const float* nb = noise ? noise + (long long)b * HW : nullptr;
  for (int t0 = blockIdx.x * 256 * kU + threadIdx.x; t0 < n; t0 += gridDim.x * 256 * kU) {
    float v[kU][VEC];
#pragma unroll
    for (int u = 0; u < kU; ++u)
      if (t0 + u * 256 < n) ldv<VEC>(yb + (t0 + u * 256) * VEC, v[u]);
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const int t = t0 + u * 256;
      if (t < n) {
        const int c = t % cv, p = t / cv;
        float dv[VEC], bv[VEC];
        ldv<VEC>(bias + c * VEC, bv);
        if (db) {
          ldv<VEC>(db + c * VEC, dv);
        } else {
#pragma unroll
          for (int j = 0; j < VEC; ++j) dv[j] = 1.0f;
        }
        const float nz = nb ? nsv * __ldg(nb + p) : 0.0f;
        float sv[VEC];
        if (s2) {
          ldv<VEC>(s2 + (long long)b * C + c * VEC, sv);
        } else {
#pragma unroll
          for (int j = 0; j < VEC; ++j) sv[j] = 1.0f;
        }
#pragma unroll
        for (int j = 0; j < VEC; ++j) {
          const float pre = act_pre(v[u][j], dv[j], nz, bv[j]);
          v[u][j] = (pre > 0.0f ? pre : 0.2f * pre) * gain * sv[j];
        }
        stv<VEC>(ob + t * VEC, v[u]);
      }
    }
  }
}

// grid (nchunk, B) as nhwc_scale_bwd_kernel, kU pixels per thread per step. The noise
// gradient of pixel p is the sum of its gpre over the cv threads of its row: a shuffle
// butterfly within the row's lanes when cv is a power of two up to 32, else through shared
// memory.
template <int VEC, bool SCALE>
__global__ void __launch_bounds__(256, 3) nhwc_act_bwd_kernel(const float* __restrict__ gout,
                                                           const float* __restrict__ y, const float* __restrict__ d,
                                                           const float* __restrict__ noise,
                                                           const float* __restrict__ ns,
                                                           const float* __restrict__ bias, float gain,
                                                           const float* __restrict__ s2, float* __restrict__ gy,
                                                           float* __restrict__ part, float* __restrict__ part2,
                                                           float* __restrict__ gnoise, int HW, int C, int nchunk) {
  __shared__ float red[256 * VEC];
  __shared__ float rowbuf[kU][256];
  const int cv = C / VEC, rows = 256 / cv;
  const int tid = threadIdx.x, c = tid % cv, r = tid / cv;
  const int b = blockIdx.y;
  const int per = (HW + nchunk - 1) / nchunk;
  const int p0 = blockIdx.x * per, p1 = min(HW, p0 + per);
  const bool shfl = cv <= 32 && (cv & (cv - 1)) == 0;
  const float nsv = noise ? __ldg(ns) : 0.0f;
  const float* gb = gout + (long long)b * HW * C + c * VEC;
  const float* yb = y + (long long)b * HW * C + c * VEC;
  float* ob = gy + (long long)b * HW * C + c * VEC;
  const float* nb = noise ? noise + (long long)b * HW : nullptr;
  float dv[VEC], bv[VEC], sv[VEC], acc[VEC], acc2[VEC];
#pragma unroll
  for (int j = 0; j < VEC; ++j) acc[j] = 0.0f, acc2[j] = 0.0f, dv[j] = 1.0f, bv[j] = 0.0f, sv[j] = 1.0f;
  if (r < rows) {
    if (d) ldv<VEC>(d + (long long)b * C + c * VEC, dv);
    if (SCALE) ldv<VEC>(s2 + (long long)b * C + c * VEC, sv);
    ldv<VEC>(bias + c * VEC, bv);
  }
  // every thread runs the same number of steps (the shuffles and barriers are uniform)
  for (int pb = p0; pb < p1; pb += kU * rows) {
    float go[kU][VEC], yv[kU][VEC], nz[kU], rs[kU];
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const int p = pb + u * rows + r;
      rs[u] = 0.0f;
      nz[u] = 0.0f;
      if (r < rows && p < p1) {
        ldv<VEC>(gb + (long long)p * C, go[u]);
        ldv<VEC>(yb + (long long)p * C, yv[u]);
        if (nb) nz[u] = nsv * __ldg(nb + p);
      }
    }
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const int p = pb + u * rows + r;
      if (r < rows && p < p1) {
        float o[VEC];
#pragma unroll
        for (int j = 0; j < VEC; ++j) {
          const float pre = act_pre(yv[u][j], dv[j], nz[u], bv[j]);
          const float slope = pre > 0.0f ? 1.0f : 0.2f;
          // with s2 the output was scaled by the next layer's style: gout is dL/d(out s2)
          if (SCALE) acc2[j] = fmaf(go[u][j], pre * slope * gain, acc2[j]);
          const float gp = (SCALE ? go[u][j] * sv[j] : go[u][j]) * gain * slope;
          acc[j] = fmaf(gp, yv[u][j], acc[j]);
          rs[u] += gp;
          o[j] = gp * dv[j];
        }
        stv<VEC>(ob + (long long)p * C, o);
      }
    }
    if (gnoise) {
      if (shfl) {
        for (int o = cv >> 1; o > 0; o >>= 1) {
#pragma unroll
          for (int u = 0; u < kU; ++u) rs[u] += __shfl_xor_sync(0xffffffffu, rs[u], o);
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) {
          const int p = pb + u * rows + r;
          if (r < rows && p < p1 && c == 0) gnoise[(long long)b * HW + p] = rs[u] * nsv;
        }
      } else {
#pragma unroll
        for (int u = 0; u < kU; ++u) rowbuf[u][tid] = rs[u];
        __syncthreads();
#pragma unroll
        for (int u = 0; u < kU; ++u) {
          const int p = pb + u * rows + r;
          if (r < rows && p < p1 && c == 0) {
            float sum = 0.0f;
            for (int k = 0; k < cv; ++k) sum += rowbuf[u][r * cv + k];
            gnoise[(long long)b * HW + p] = sum * nsv;
          }
        }
        __syncthreads();
      }
    }
  }
  if (part) column_partials<VEC>(acc, red, cv, rows, part, C, nchunk);
  if (SCALE && part2) {
    __syncthreads();  // the first column pass has read red
    column_partials<VEC>(acc2, red, cv, rows, part2, C, nchunk);
  }
}

// out[b][c] = sum over chunks k (in order) of part[b][k][c].
__global__ void nhwc_colsum_kernel(const float* __restrict__ part, float* __restrict__ out, int B, int C,
                                   int nchunk) {
  const int i = blockIdx.x * 256 + threadIdx.x;
  if (i >= B * C) return;
  const int b = i / C, c = i % C;
  float sum = 0.0f;
  for (int k = 0; k < nchunk; ++k) sum += part[((long long)b * nchunk + k) * C + c];
  out[i] = sum;
}

// The toRGB layer's epilogue: its 1x1 convolution leaves a channels-last map with cp (>= c)
// channels per pixel; the image is written in NCHW (the layout of the textures the renderer
// reads) as img[b][ch][y][x] = yp[b][y][x][ch] + bias[ch] + up2(prev)[b][ch][y][x], prev the
// previous resolution's image (NCHW, nullable; up2 the [1, 3, 3, 1] up-sampling as
// nhwc_up_fwd_kernel computes it). grid (ceil(W / 256), B H): block row (b, y), thread x.
__global__ void __launch_bounds__(256) rgb_fwd_kernel(const float* __restrict__ yp, int cp,
                                                      const float* __restrict__ bias, const float* __restrict__ prev,
                                                      float* __restrict__ img, int C, int H, int W) {
  const int b = blockIdx.y / H, yy = blockIdx.y % H;
  const int x = blockIdx.x * 256 + threadIdx.x;
  if (x >= W) return;
  const float* row = yp + (((long long)b * H + yy) * W + x) * cp;
  int y0 = 0, y1 = 0, x0 = 0, x1 = 0;
  float wy0 = 0.f, wy1 = 0.f, wx0 = 0.f, wx1 = 0.f;
  if (prev) {
    taps(yy, H / 2, y0, y1, wy0, wy1);
    taps(x, W / 2, x0, x1, wx0, wx1);
  }
  const long long hw = (long long)H * W, hw2 = (long long)(H / 2) * (W / 2);
  for (int ch = 0; ch < C; ++ch) {
    float v = __ldg(row + ch) + __ldg(bias + ch);
    if (prev) {
      const float* pp = prev + ((long long)b * C + ch) * hw2;
      const int w2 = W / 2;
      v += wy0 * (wx0 * __ldg(pp + y0 * w2 + x0) + wx1 * __ldg(pp + y0 * w2 + x1)) +
           wy1 * (wx0 * __ldg(pp + y1 * w2 + x0) + wx1 * __ldg(pp + y1 * w2 + x1));
    }
    img[((long long)b * C + ch) * hw + (long long)yy * W + x] = v;
  }
}

// Its adjoint for the convolution: gyp[b][y][x][ch] = g[b][ch][y][x] for ch < C, 0 for the
// padding channels C .. cp - 1 (the skip image's gradient is the NCHW up-sampling adjoint of g).
template <int VEC>
__global__ void __launch_bounds__(256) rgb_bwd_kernel(const float* __restrict__ g, float* __restrict__ gyp, int cp,
                                                      int C, int H, int W) {
  const int b = blockIdx.y / H, yy = blockIdx.y % H;
  const int x = blockIdx.x * 256 + threadIdx.x;
  if (x >= W) return;
  float* row = gyp + (((long long)b * H + yy) * W + x) * cp;
  const long long hw = (long long)H * W;
  const float* gp = g + (long long)b * C * hw + (long long)yy * W + x;
  for (int ch = 0; ch < cp; ch += VEC) {  // VEC = 4: the pixel's row as 16-byte stores
    float v[VEC];
#pragma unroll
    for (int j = 0; j < VEC; ++j) v[j] = ch + j < C ? __ldg(gp + (long long)(ch + j) * hw) : 0.0f;
    stv<VEC>(row + ch, v);
  }
}

}  // namespace gen_nhwc
}  // namespace svb

using namespace svb;

namespace {

bool a16(const void* p) { return p == nullptr || (uintptr_t)p % 16 == 0; }

// Chunks per batch entry for the column sums: about 8 pixels per thread, at most 64.
int nchunks(int hw, int rows) {
  const long long n = ((long long)hw + 8LL * rows - 1) / (8LL * rows);
  return (int)(n < 1 ? 1 : n > gen_nhwc::kMaxChunks ? gen_nhwc::kMaxChunks : n);
}
// The same, reduced so that b x chunks blocks fill whole waves of a kernel that keeps
// `per_sm` blocks on each SM (the activation adjoint: 3, the scaling adjoint: 4), where they
// exceed one wave: on a 256^2 map of 16 entries, 57 chunks (2 full waves of the activation
// adjoint) instead of 64 (2.25).
int nchunks_waves(int hw, int rows, int b, int per_sm) {
  const int n0 = nchunks(hw, rows);
  const long long slots = (long long)(device_sm_count() > 0 ? device_sm_count() : 1) * per_sm;
  const long long waves = (long long)b * n0 / slots;
  if (waves < 1) return n0;
  const long long n = waves * slots / b;
  return (int)(n < 1 ? 1 : n < n0 ? n : n0);
}

}  // namespace

extern "C" {

int svbrdf_gen_nhwc_partial_floats(int b, int c) { return b * gen_nhwc::kMaxChunks * c; }

int svbrdf_gen_upsample2_nhwc(const float* x, const float* s, float* y, int b, int h, int w, int c, int halo,
                              void* stream) {
  if (!x || !y || b < 1 || h < 1 || w < 1 || c < 1) return fail(SVBRDF_ERR_INVALID, "upsample2_nhwc: bad arguments");
  if (halo != 0 && halo != 1) return fail(SVBRDF_ERR_INVALID, "upsample2_nhwc: halo must be 0 or 1 (got %d)", halo);
  if ((long long)b * (2 * h + 2 * halo) > 65535 || (2LL * w + 2 * halo) * c > (1LL << 30))
    return fail(SVBRDF_ERR_UNSUPPORTED, "upsample2_nhwc: too large");
  const bool v4 = c % 4 == 0 && a16(x) && a16(y) && a16(s);
  const int row = (2 * w + 2 * halo) * (v4 ? c / 4 : c);
  // at most 8 blocks per output row: each thread loops over several vectors of the row, so
  // the launch is a few tens of thousands of blocks rather than one per 256 vectors
  const int per_row = (row + 255) / 256;
  dim3 grid((unsigned)(per_row < 8 ? per_row : 8), (unsigned)(b * (2 * h + 2 * halo)));
  cudaStream_t st = (cudaStream_t)stream;
  if (v4) gen_nhwc::nhwc_up_fwd_kernel<4><<<grid, 256, 0, st>>>(x, s, y, h, w, c, halo);
  else gen_nhwc::nhwc_up_fwd_kernel<1><<<grid, 256, 0, st>>>(x, s, y, h, w, c, halo);
  return check_launch("nhwc_up_fwd_kernel");
}

int svbrdf_gen_upsample2_nhwc_bwd(const float* g, float* gx, int b, int h, int w, int c, int halo, void* stream) {
  if (!g || !gx || b < 1 || h < 1 || w < 1 || c < 1) return fail(SVBRDF_ERR_INVALID, "upsample2_nhwc_bwd: bad arguments");
  if (halo != 0 && halo != 1) return fail(SVBRDF_ERR_INVALID, "upsample2_nhwc_bwd: halo must be 0 or 1 (got %d)", halo);
  if ((long long)b * h > 65535 || (long long)w * c > (1LL << 30))
    return fail(SVBRDF_ERR_UNSUPPORTED, "upsample2_nhwc_bwd: too large");
  const bool v4 = c % 4 == 0 && a16(g) && a16(gx);
  const int row = w * (v4 ? c / 4 : c);
  dim3 grid((unsigned)((row + 255) / 256), (unsigned)(b * h));
  cudaStream_t st = (cudaStream_t)stream;
  if (v4) gen_nhwc::nhwc_up_bwd_kernel<4><<<grid, 256, 0, st>>>(g, gx, h, w, c, halo);
  else gen_nhwc::nhwc_up_bwd_kernel<1><<<grid, 256, 0, st>>>(g, gx, h, w, c, halo);
  return check_launch("nhwc_up_bwd_kernel");
}

static dim3 entry_grid(int hw, int cv, int b) {
  const long long blocks = ((long long)hw * cv + 256 * gen_nhwc::kU - 1) / (256 * gen_nhwc::kU);
  return dim3((unsigned)(blocks < 4096 ? blocks : 4096), (unsigned)b);
}

int svbrdf_gen_scale_nhwc(const float* x, const float* s, float* y, int b, int hw, int c, void* stream) {
  if (!x || !s || !y || b < 1 || b > 65535 || hw < 1 || c < 1) return fail(SVBRDF_ERR_INVALID, "scale_nhwc: bad arguments");
  if ((long long)hw * c > (1LL << 30)) return fail(SVBRDF_ERR_UNSUPPORTED, "scale_nhwc: too large");
  const bool v4 = c % 4 == 0 && a16(x) && a16(y) && a16(s);
  const int cv = v4 ? c / 4 : c;
  cudaStream_t st = (cudaStream_t)stream;
  if (v4) gen_nhwc::nhwc_scale_fwd_kernel<4><<<entry_grid(hw, cv, b), 256, 0, st>>>(x, s, y, hw, c);
  else gen_nhwc::nhwc_scale_fwd_kernel<1><<<entry_grid(hw, cv, b), 256, 0, st>>>(x, s, y, hw, c);
  return check_launch("nhwc_scale_fwd_kernel");
}

int svbrdf_gen_scale_nhwc_bwd(const float* g, const float* x, const float* s, float* gx, float* gs, float* part, int b,
                              int hw, int c, void* stream) {
  if (!g || !x || !s || !gx || !gs || !part || b < 1 || b > 65535 || hw < 1 || c < 1)
    return fail(SVBRDF_ERR_INVALID, "scale_nhwc_bwd: bad arguments");
  if ((long long)hw * c > (1LL << 30)) return fail(SVBRDF_ERR_UNSUPPORTED, "scale_nhwc_bwd: too large");
  const bool v4 = c % 4 == 0 && a16(g) && a16(x) && a16(gx) && a16(s);
  const int cv = v4 ? c / 4 : c;
  if (cv > 256) return fail(SVBRDF_ERR_UNSUPPORTED, "scale_nhwc_bwd: %d channels are more than one block's row", c);
  const int nc = nchunks_waves(hw, 256 / cv, b, 4);  // 64 registers: 4 blocks per SM
  cudaStream_t st = (cudaStream_t)stream;
  dim3 grid((unsigned)nc, (unsigned)b);
  if (v4) gen_nhwc::nhwc_scale_bwd_kernel<4><<<grid, 256, 0, st>>>(g, x, s, gx, part, hw, c, nc);
  else gen_nhwc::nhwc_scale_bwd_kernel<1><<<grid, 256, 0, st>>>(g, x, s, gx, part, hw, c, nc);
  int rc = check_launch("nhwc_scale_bwd_kernel");
  if (rc) return rc;
  gen_nhwc::nhwc_colsum_kernel<<<(unsigned)((b * c + 255) / 256), 256, 0, st>>>(part, gs, b, c, nc);
  return check_launch("nhwc_colsum_kernel");
}

int svbrdf_gen_act_nhwc(const float* y, const float* d, const float* noise, const float* ns, const float* bias,
                        float gain, float* out, int b, int hw, int c, void* stream) {
  if (!y || !bias || !out || (noise && !ns) || b < 1 || b > 65535 || hw < 1 || c < 1)
    return fail(SVBRDF_ERR_INVALID, "act_nhwc: bad arguments");
  if ((long long)hw * c > (1LL << 30)) return fail(SVBRDF_ERR_UNSUPPORTED, "act_nhwc: too large");
  const bool v4 = c % 4 == 0 && a16(y) && a16(d) && a16(bias) && a16(out);
  const int cv = v4 ? c / 4 : c;
  cudaStream_t st = (cudaStream_t)stream;
  if (v4)
    gen_nhwc::nhwc_act_fwd_kernel<4><<<entry_grid(hw, cv, b), 256, 0, st>>>(y, d, noise, ns, bias, gain, nullptr, out,
                                                                         hw, c);
  else
    gen_nhwc::nhwc_act_fwd_kernel<1><<<entry_grid(hw, cv, b), 256, 0, st>>>(y, d, noise, ns, bias, gain, nullptr, out,
                                                                         hw, c);
  return check_launch("nhwc_act_fwd_kernel");
}

int svbrdf_gen_act_scale_nhwc(const float* y, const float* d, const float* noise, const float* ns, const float* bias,
                              float gain, const float* s2, float* out, int b, int hw, int c, void* stream) {
  if (!y || !bias || !s2 || !out || (noise && !ns) || b < 1 || b > 65535 || hw < 1 || c < 1)
    return fail(SVBRDF_ERR_INVALID, "act_scale_nhwc: bad arguments");
  if ((long long)hw * c > (1LL << 30)) return fail(SVBRDF_ERR_UNSUPPORTED, "act_scale_nhwc: too large");
  const bool v4 = c % 4 == 0 && a16(y) && a16(d) && a16(bias) && a16(s2) && a16(out);
  const int cv = v4 ? c / 4 : c;
  cudaStream_t st = (cudaStream_t)stream;
  if (v4)
    gen_nhwc::nhwc_act_fwd_kernel<4><<<entry_grid(hw, cv, b), 256, 0, st>>>(y, d, noise, ns, bias, gain, s2, out, hw,
                                                                         c);
  else
    gen_nhwc::nhwc_act_fwd_kernel<1><<<entry_grid(hw, cv, b), 256, 0, st>>>(y, d, noise, ns, bias, gain, s2, out, hw,
                                                                         c);
  return check_launch("nhwc_act_fwd_kernel");
}

int svbrdf_gen_act_nhwc_bwd(const float* gout, const float* y, const float* d, const float* noise, const float* ns,
                            const float* bias, float gain, float* gy, float* gd, float* gnoise, float* part, int b,
                            int hw, int c, void* stream) {
  if (!gout || !y || !bias || !gy || (noise && !ns) || (gnoise && !noise) || (gd && !part) || b < 1 || b > 65535 ||
      hw < 1 || c < 1)
    return fail(SVBRDF_ERR_INVALID, "act_nhwc_bwd: bad arguments");
  if ((long long)hw * c > (1LL << 30)) return fail(SVBRDF_ERR_UNSUPPORTED, "act_nhwc_bwd: too large");
  const bool v4 = c % 4 == 0 && a16(gout) && a16(y) && a16(d) && a16(bias) && a16(gy);
  const int cv = v4 ? c / 4 : c;
  if (cv > 256) return fail(SVBRDF_ERR_UNSUPPORTED, "act_nhwc_bwd: %d channels are more than one block's row", c);
  const int nc = nchunks_waves(hw, 256 / cv, b, 3);
  cudaStream_t st = (cudaStream_t)stream;
  dim3 grid((unsigned)nc, (unsigned)b);
  float* pp = gd ? part : nullptr;
  if (v4)
    gen_nhwc::nhwc_act_bwd_kernel<4, false><<<grid, 256, 0, st>>>(gout, y, d, noise, ns, bias, gain, nullptr, gy, pp, nullptr,
                                                           gnoise, hw, c, nc);
  else
    gen_nhwc::nhwc_act_bwd_kernel<1, false><<<grid, 256, 0, st>>>(gout, y, d, noise, ns, bias, gain, nullptr, gy, pp, nullptr,
                                                           gnoise, hw, c, nc);
  int rc = check_launch("nhwc_act_bwd_kernel");
  if (rc || !gd) return rc;
  gen_nhwc::nhwc_colsum_kernel<<<(unsigned)((b * c + 255) / 256), 256, 0, st>>>(part, gd, b, c, nc);
  return check_launch("nhwc_colsum_kernel");
}

int svbrdf_gen_act_scale_nhwc_bwd(const float* gout, const float* y, const float* d, const float* noise, const float* ns,
                                  const float* bias, float gain, const float* s2, float* gy, float* gd, float* gs2,
                                  float* gnoise, float* part, float* part2, int b, int hw, int c, void* stream) {
  if (!gout || !y || !bias || !s2 || !gy || (noise && !ns) || (gnoise && !noise) || (gd && !part) ||
      (gs2 && !part2) || b < 1 || b > 65535 || hw < 1 || c < 1)
    return fail(SVBRDF_ERR_INVALID, "act_scale_nhwc_bwd: bad arguments");
  if ((long long)hw * c > (1LL << 30)) return fail(SVBRDF_ERR_UNSUPPORTED, "act_scale_nhwc_bwd: too large");
  const bool v4 = c % 4 == 0 && a16(gout) && a16(y) && a16(d) && a16(bias) && a16(s2) && a16(gy);
  const int cv = v4 ? c / 4 : c;
  if (cv > 256) return fail(SVBRDF_ERR_UNSUPPORTED, "act_scale_nhwc_bwd: %d channels are more than one block's row", c);
  const int nc = nchunks_waves(hw, 256 / cv, b, 3);
  cudaStream_t st = (cudaStream_t)stream;
  dim3 grid((unsigned)nc, (unsigned)b);
  float* pp = gd ? part : nullptr;
  float* pp2 = gs2 ? part2 : nullptr;
  if (v4)
    gen_nhwc::nhwc_act_bwd_kernel<4, true><<<grid, 256, 0, st>>>(gout, y, d, noise, ns, bias, gain, s2, gy, pp, pp2, gnoise,
                                                           hw, c, nc);
  else
    gen_nhwc::nhwc_act_bwd_kernel<1, true><<<grid, 256, 0, st>>>(gout, y, d, noise, ns, bias, gain, s2, gy, pp, pp2, gnoise,
                                                           hw, c, nc);
  int rc = check_launch("nhwc_act_bwd_kernel");
  if (rc) return rc;
  if (gd) {
    gen_nhwc::nhwc_colsum_kernel<<<(unsigned)((b * c + 255) / 256), 256, 0, st>>>(part, gd, b, c, nc);
    rc = check_launch("nhwc_colsum_kernel");
    if (rc) return rc;
  }
  if (gs2) {
    gen_nhwc::nhwc_colsum_kernel<<<(unsigned)((b * c + 255) / 256), 256, 0, st>>>(part2, gs2, b, c, nc);
    rc = check_launch("nhwc_colsum_kernel");
  }
  return rc;
}


int svbrdf_gen_rgb_nhwc(const float* yp, int cp, const float* bias, const float* prev, float* img, int b, int c, int h,
                        int w, void* stream) {
  if (!yp || !bias || !img || b < 1 || c < 1 || cp < c || h < 1 || w < 1)
    return fail(SVBRDF_ERR_INVALID, "rgb_nhwc: bad arguments");
  if (prev && (h % 2 || w % 2)) return fail(SVBRDF_ERR_INVALID, "rgb_nhwc: a skip image needs even H and W");
  if ((long long)b * h > 65535) return fail(SVBRDF_ERR_UNSUPPORTED, "rgb_nhwc: too large");
  dim3 grid((unsigned)((w + 255) / 256), (unsigned)(b * h));
  gen_nhwc::rgb_fwd_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(yp, cp, bias, prev, img, c, h, w);
  return check_launch("rgb_fwd_kernel");
}

int svbrdf_gen_rgb_nhwc_bwd(const float* g, float* gyp, int cp, int b, int c, int h, int w, void* stream) {
  if (!g || !gyp || b < 1 || c < 1 || cp < c || h < 1 || w < 1) return fail(SVBRDF_ERR_INVALID, "rgb_nhwc_bwd: bad arguments");
  if ((long long)b * h > 65535) return fail(SVBRDF_ERR_UNSUPPORTED, "rgb_nhwc_bwd: too large");
  dim3 grid((unsigned)((w + 255) / 256), (unsigned)(b * h));
  if (cp % 4 == 0 && a16(gyp))
    gen_nhwc::rgb_bwd_kernel<4><<<grid, 256, 0, (cudaStream_t)stream>>>(g, gyp, cp, c, h, w);
  else
    gen_nhwc::rgb_bwd_kernel<1><<<grid, 256, 0, (cudaStream_t)stream>>>(g, gyp, cp, c, h, w);
  return check_launch("rgb_bwd_kernel");
}

}  // extern "C"
