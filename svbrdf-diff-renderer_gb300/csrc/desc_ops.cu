// Fused operations of the descriptor loss around the tensor-core convolutions (conv_tc.cu).
//
// The descriptor (src/descriptor.py:7-79) normalises the renders with ImageNet statistics
// (mean 0.485/0.456/0.406, std 0.229/0.224/0.255, :65-75), runs VGG19 features and compares
// hooked ReLU outputs. Here the renders are first 2x2 box-downsampled, and the stack up to
// conv4_1 runs in NHWC BF16. These kernels replace the elementwise glue:
//
//   desc_conv1_fwd_kernel  2x2 box downsample + normalise + conv1_1 (3 -> 64) + bias + ReLU,
//                          FP32 and BF16 NHWC outputs (the FP32 copy feeds the relu1_1 hook)
//   desc_pool_fwd_kernel   2x2 max-pool (or average pool), NHWC BF16
//   desc_pool_bwd_kernel   its backward (max: the first maximum of each window takes the
//                          gradient, as ATen's pool; average: a quarter to each) + optional
//                          hook gradient + ReLU mask
//   desc_feat_loss_kernel  sum of (f - t)^2 as per-block partials (a fixed-order sum), and
//                          optionally g = coef (f - t) + gram_grad, masked by f > 0
//   desc_loss_sums_kernel  weighted sums of loss partials (fixed order)
//   desc_conv1_bwd_kernel  conv1_1 data gradient, back through the normalisation and the
//                          downsample to d/d render
//
// Each is HBM-bound elementwise or small-stencil work: one read and one write per element.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "svbrdf_common.cuh"

namespace svb {
namespace desc {

__constant__ float c_mean[3] = {0.485f, 0.456f, 0.406f};
__constant__ float c_std[3] = {0.229f, 0.224f, 0.255f};  // the reference's blue std is 0.255

constexpr int kTile = 16;

// ---------------------------------------------------------------- conv1_1 forward
// A block computes an 8-row x 16-column pixel tile, all 64 channels, with 128 threads. Thread t
// owns channels 4 (t % 16) .. +3 of the 16 pixels of tile row t / 16, so the 16 threads of a
// half-warp store one pixel's 64 channels as one contiguous 256-byte run (128 bytes in BF16).
// The products run as packed FP32 pair FMAs (channels 4k, 4k+1 and 4k+2, 4k+3), each lane
// rounded as a scalar FMA. Small blocks (several per SM) let one block's input staging overlap
// another's arithmetic and stores.
constexpr int kTileY = 8;
template <bool DOWN>
__global__ void __launch_bounds__(128) desc_conv1_fwd_kernel(const float* __restrict__ r, const float* __restrict__ w,
                                                             const float* __restrict__ b, float* __restrict__ out32,
                                                             __nv_bfloat16* __restrict__ out16, int H, int W) {
  __shared__ float s_in[3][kTileY + 2][kTile + 2];
  __shared__ __align__(16) float s_w[27][64];  // [ci*9 + ky*3 + kx][co]
  __shared__ __align__(16) float s_b[64];
  const int tid = threadIdx.x;
  const int v = blockIdx.z, y0 = blockIdx.y * kTileY, x0 = blockIdx.x * kTile;
  for (int i = tid; i < 64 * 27; i += 128) s_w[i % 27][i / 27] = w[i];  // w is [co][ci][ky][kx]
  if (tid < 64) s_b[tid] = b[tid];
  const int RH = DOWN ? 2 * H : H, RW = DOWN ? 2 * W : W;
  for (int i = tid; i < 3 * (kTileY + 2) * (kTile + 2); i += 128) {
    const int ci = i / ((kTileY + 2) * (kTile + 2)), rem = i % ((kTileY + 2) * (kTile + 2));
    const int ty = rem / (kTile + 2), tx = rem % (kTile + 2);
    const int gy = y0 + ty - 1, gx = x0 + tx - 1;
    float val = 0.0f;  // zero padding of the normalised image
    if (gy >= 0 && gy < H && gx >= 0 && gx < W) {
      const float* rp = r + ((size_t)v * 3 + ci) * RH * RW;
      float sv;
      if (DOWN) {
        const float* q = rp + (size_t)(2 * gy) * RW + 2 * gx;
        sv = (q[0] + q[1] + q[RW] + q[RW + 1]) * 0.25f;
      } else {
        sv = rp[(size_t)gy * RW + gx];
      }
      val = (sv - c_mean[ci]) / c_std[ci];
    }
    s_in[ci][ty][tx] = val;
  }
  __syncthreads();
  const int cg = tid & 15, row = tid >> 4;
  const int y = y0 + row;
  float2 acc[kTile][2];
  const float4 bias4 = reinterpret_cast<const float4*>(s_b)[cg];
#pragma unroll
  for (int px = 0; px < kTile; ++px) {
    acc[px][0] = make_float2(bias4.x, bias4.y);
    acc[px][1] = make_float2(bias4.z, bias4.w);
  }
#pragma unroll
  for (int ci = 0; ci < 3; ++ci)
#pragma unroll
    for (int ky = 0; ky < 3; ++ky) {
      // the 18 inputs of this channel and kernel row, read once for the three kx taps
      float xr[kTile + 2];
#pragma unroll
      for (int i = 0; i < kTile + 2; ++i) xr[i] = s_in[ci][row + ky][i];
#pragma unroll
      for (int kx = 0; kx < 3; ++kx) {
        const float4 w4 = reinterpret_cast<const float4*>(s_w[ci * 9 + ky * 3 + kx])[cg];
        const float2 w01 = make_float2(w4.x, w4.y), w23 = make_float2(w4.z, w4.w);
#pragma unroll
        for (int px = 0; px < kTile; ++px) {
          const float2 x2 = make_float2(xr[px + kx], xr[px + kx]);
          acc[px][0] = __ffma2_rn(w01, x2, acc[px][0]);
          acc[px][1] = __ffma2_rn(w23, x2, acc[px][1]);
        }
      }
    }
  if (y >= H) return;
#pragma unroll
  for (int px = 0; px < kTile; ++px) {
    const int x = x0 + px;
    if (x >= W) break;
    const float a0 = fmaxf(acc[px][0].x, 0.f), a1 = fmaxf(acc[px][0].y, 0.f), a2 = fmaxf(acc[px][1].x, 0.f),
                a3 = fmaxf(acc[px][1].y, 0.f);
    const size_t pix = ((size_t)v * H + y) * W + x;
    reinterpret_cast<float4*>(out32 + pix * 64)[cg] = make_float4(a0, a1, a2, a3);
    __nv_bfloat162 h0 = __floats2bfloat162_rn(a0, a1), h1 = __floats2bfloat162_rn(a2, a3);
    uint2 pk;
    pk.x = *reinterpret_cast<uint32_t*>(&h0);
    pk.y = *reinterpret_cast<uint32_t*>(&h1);
    reinterpret_cast<uint2*>(out16 + pix * 64)[cg] = pk;
  }
}

// ---------------------------------------------------------------- conv1_1 backward
// d render = conv1_1's data gradient (3 x 3, 64 -> 3 channels), through the normalisation
// and the 2x2 box downsample. A block takes a 16 x 16 tile of the 256-pixel side; each of its
// 128 threads computes 2 adjacent pixels of one row, so every weight pair and every input
// column read from shared memory serves up to 2 pixels (per channel pair and kernel row: 4
// input values and 9 weight pairs for 36 FMAs).
template <bool DOWN>
__global__ void __launch_bounds__(128) desc_conv1_bwd_kernel(const __nv_bfloat16* __restrict__ gz,
                                                            const float* __restrict__ w, float* __restrict__ gr,
                                                            int H, int W) {
  __shared__ __nv_bfloat162 s_g[32][kTile + 2][kTile + 2];  // gz tile, channel pairs outermost
  __shared__ __align__(8) float s_w[27][64];                 // [ci*9 + ky*3 + kx][co]
  const int tid = threadIdx.x;
  const int v = blockIdx.z, y0 = blockIdx.y * kTile, x0 = blockIdx.x * kTile;
  for (int i = tid; i < 64 * 27; i += 128) s_w[i % 27][i / 27] = w[i];
  // rows y0-1 .. y0+16 and columns x0-1 .. x0+16 of gz, 8 channels per step
  for (int i = tid; i < (kTile + 2) * (kTile + 2) * 8; i += 128) {
    const int p = i / 8, c8 = i % 8;
    const int ty = p / (kTile + 2), tx = p % (kTile + 2);
    const int gy = y0 + ty - 1, gx = x0 + tx - 1;
    uint4 val = make_uint4(0u, 0u, 0u, 0u);
    if (gy >= 0 && gy < H && gx >= 0 && gx < W)
      val = *reinterpret_cast<const uint4*>(gz + (((size_t)v * H + gy) * W + gx) * 64 + c8 * 8);
    const __nv_bfloat162* e = reinterpret_cast<const __nv_bfloat162*>(&val);
#pragma unroll
    for (int j = 0; j < 4; ++j) s_g[c8 * 4 + j][ty][tx] = e[j];
  }
  __syncthreads();
  const int ty = tid / 8, tx0 = 2 * (tid % 8);  // pixels (ty, tx0 .. tx0 + 1) of the tile
  float d[2][3];
#pragma unroll
  for (int q = 0; q < 2; ++q) d[q][0] = d[q][1] = d[q][2] = 0.f;
#pragma unroll 2
  for (int c2 = 0; c2 < 32; ++c2) {
#pragma unroll
    for (int ky = 0; ky < 3; ++ky) {
      // gz at output (y + 1 - ky, x + 1 - kx) = tile (ty + 2 - ky, tx + 2 - kx): columns tx0 .. tx0 + 3
      float2 g[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) g[j] = __bfloat1622float2(s_g[c2][ty + 2 - ky][tx0 + j]);
#pragma unroll
      for (int kx = 0; kx < 3; ++kx) {
#pragma unroll
        for (int ci = 0; ci < 3; ++ci) {
          const float2 wv = reinterpret_cast<const float2*>(s_w[ci * 9 + ky * 3 + kx])[c2];
#pragma unroll
          for (int q = 0; q < 2; ++q) d[q][ci] = fmaf(wv.y, g[q + 2 - kx].y, fmaf(wv.x, g[q + 2 - kx].x, d[q][ci]));
        }
      }
    }
  }
  const int y = y0 + ty, x = x0 + tx0;
  if (y >= H) return;
  const int RH = DOWN ? 2 * H : H, RW = DOWN ? 2 * W : W;
#pragma unroll
  for (int ci = 0; ci < 3; ++ci) {
    float* rp = gr + ((size_t)v * 3 + ci) * RH * RW;
    const float is = 1.0f / c_std[ci];
    float gq[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) gq[q] = d[q][ci] * is;
    if (DOWN) {
      if (x + 1 < W && RW % 4 == 0 && ((uintptr_t)rp & 15u) == 0) {  // 16-byte aligned rows
        const float4 a = make_float4(0.25f * gq[0], 0.25f * gq[0], 0.25f * gq[1], 0.25f * gq[1]);
        *reinterpret_cast<float4*>(rp + (size_t)(2 * y) * RW + 2 * x) = a;
        *reinterpret_cast<float4*>(rp + (size_t)(2 * y + 1) * RW + 2 * x) = a;
      } else {
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          if (x + q >= W) break;
          const float qv = 0.25f * gq[q];
          *reinterpret_cast<float2*>(rp + (size_t)(2 * y) * RW + 2 * (x + q)) = make_float2(qv, qv);
          *reinterpret_cast<float2*>(rp + (size_t)(2 * y + 1) * RW + 2 * (x + q)) = make_float2(qv, qv);
        }
      }
    } else {
#pragma unroll
      for (int q = 0; q < 2; ++q)
        if (x + q < W) rp[(size_t)y * RW + x + q] = gq[q];
    }
  }
}

// ---------------------------------------------------------------- 2x2 max-pool
__device__ __forceinline__ void bf8_load(const __nv_bfloat16* p, float f[8]) {
  const uint4 u = *reinterpret_cast<const uint4*>(p);
  const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const float2 t = __bfloat1622float2(h[j]);
    f[2 * j] = t.x;
    f[2 * j + 1] = t.y;
  }
}
__device__ __forceinline__ void bf8_store(__nv_bfloat16* p, const float f[8]) {
  uint4 u;
  uint32_t* w = reinterpret_cast<uint32_t*>(&u);
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    __nv_bfloat162 h = __floats2bfloat162_rn(f[2 * j], f[2 * j + 1]);
    w[j] = *reinterpret_cast<uint32_t*>(&h);
  }
  *reinterpret_cast<uint4*>(p) = u;
}

// x [V, H, W, C] -> y [V, H/2, W/2, C]; one thread per output pixel and 8 channels.
// AVG: the window's mean (the reference's VGGLoss swaps VGG19's max-pools for 2x2 average
// pools, src/descriptor.py:16-19), summed in row-major order in FP32 then halved twice.
template <bool AVG>
__global__ void desc_pool_fwd_kernel(const __nv_bfloat16* __restrict__ x, __nv_bfloat16* __restrict__ y, int V, int H,
                                     int W, int C) {
  // grid (ceil(Wo C8 / 256), V Ho): block row (v, yo); thread q of the row is (xo, c8)
  const int Ho = H / 2, Wo = W / 2, C8 = C / 8;
  const int v = blockIdx.y / Ho, yo = blockIdx.y % Ho;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < Wo * C8; q += gridDim.x * blockDim.x) {
    const int c8 = q % C8, xo = q / C8;
    const size_t p = ((size_t)v * Ho + yo) * Wo + xo;
    const __nv_bfloat16* base = x + (((size_t)v * H + 2 * yo) * W + 2 * xo) * C + c8 * 8;
    float m[8], t[8];
    bf8_load(base, m);
    const size_t offs[3] = {(size_t)C, (size_t)W * C, (size_t)W * C + C};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      bf8_load(base + offs[k], t);
#pragma unroll
      for (int j = 0; j < 8; ++j) m[j] = AVG ? m[j] + t[j] : (t[j] > m[j] ? t[j] : m[j]);
    }
    if (AVG) {
#pragma unroll
      for (int j = 0; j < 8; ++j) m[j] *= 0.25f;
    }
    bf8_store(y + p * C + c8 * 8, m);
  }
}

// gx = (pool-route(gy) + addend) * (x > 0). x is the pool's input, a ReLU output, so x > 0 is
// that ReLU's mask. Max-pool: the window's first maximum in row-major order takes the
// gradient. AVG: every element of the window takes gy / 4. Each thread issues all of its loads
// (the window's x, gy, the window's addend: nine 16-byte loads) before any arithmetic, keeping
// them as raw BF16 until use.
__device__ __forceinline__ float2 bf2f(const uint4& u, int e) {
  return __bfloat1622float2(reinterpret_cast<const __nv_bfloat162*>(&u)[e]);
}
template <bool AVG>
__global__ void __launch_bounds__(256) desc_pool_bwd_kernel(const __nv_bfloat16* __restrict__ gy,
                                                            const __nv_bfloat16* __restrict__ x,
                                                            const __nv_bfloat16* __restrict__ addend,
                                                            __nv_bfloat16* __restrict__ gx, int V, int H, int W,
                                                            int C) {
  // grid (ceil(Wo C8 / 256), V Ho): block row (v, yo); thread t of the row is (xo, c8)
  const int Ho = H / 2, Wo = W / 2, C8 = C / 8;
  const int v = blockIdx.y / Ho, yo = blockIdx.y % Ho;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < Wo * C8; t += gridDim.x * blockDim.x) {
    const int c8 = t % C8, xo = t / C8;
    const size_t p = ((size_t)v * Ho + yo) * Wo + xo;
    const size_t b0 = (((size_t)v * H + 2 * yo) * W + 2 * xo) * C + c8 * 8;
    const size_t offs[4] = {0, (size_t)C, (size_t)W * C, (size_t)W * C + C};
    uint4 xr[4], ar[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) xr[k] = __ldg(reinterpret_cast<const uint4*>(x + b0 + offs[k]));
    const uint4 gr = __ldg(reinterpret_cast<const uint4*>(gy + p * C + c8 * 8));
    if (addend) {
#pragma unroll
      for (int k = 0; k < 4; ++k) ar[k] = __ldg(reinterpret_cast<const uint4*>(addend + b0 + offs[k]));
    } else {
#pragma unroll
      for (int k = 0; k < 4; ++k) ar[k] = make_uint4(0u, 0u, 0u, 0u);  // BF16 zeros
    }
    uint4 o[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {  // channel pairs 2e, 2e + 1
      const float2 g = bf2f(gr, e);
      float2 xv[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) xv[k] = bf2f(xr[k], e);
      int amx = 0, amy = 0;
      if (!AVG) {
        float mx = xv[0].x, my = xv[0].y;
#pragma unroll
        for (int k = 1; k < 4; ++k) {
          if (xv[k].x > mx) { mx = xv[k].x; amx = k; }
          if (xv[k].y > my) { my = xv[k].y; amy = k; }
        }
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const float2 ad = bf2f(ar[k], e);
        float vx = AVG ? 0.25f * g.x : (amx == k ? g.x : 0.0f);
        float vy = AVG ? 0.25f * g.y : (amy == k ? g.y : 0.0f);
        vx += ad.x;
        vy += ad.y;
        const __nv_bfloat162 h = __floats2bfloat162_rn(xv[k].x > 0.0f ? vx : 0.0f, xv[k].y > 0.0f ? vy : 0.0f);
        reinterpret_cast<uint32_t*>(&o[k])[e] = *reinterpret_cast<const uint32_t*>(&h);
      }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) *reinterpret_cast<uint4*>(gx + b0 + offs[k]) = o[k];
  }
}

// ---------------------------------------------------------------- feature loss
constexpr int kLossThreads = 256;
constexpr int kLossBlocks = 1024;

template <typename TF>
__device__ __forceinline__ float ld(const TF* p, long long i);
template <>
__device__ __forceinline__ float ld<float>(const float* p, long long i) {
  return __ldg(p + i);
}
template <>
__device__ __forceinline__ float ld<__nv_bfloat16>(const __nv_bfloat16* p, long long i) {
  return __bfloat162float(p[i]);
}

// partial[b] = sum over block b's elements of (f - t)^2 (elements i = b*T + t, step B*T);
// if g: g = coef (f - t) + gram_grad, times (f > 0) when `mask`.
template <typename TF>
__global__ void __launch_bounds__(kLossThreads) desc_feat_loss_kernel(const TF* __restrict__ f,
                                                                      const float* __restrict__ t,
                                                                      const float* __restrict__ gram_grad, float coef,
                                                                      int mask, __nv_bfloat16* __restrict__ g,
                                                                      float* __restrict__ partial, long long n) {
  __shared__ float s_red[kLossThreads / 32];
  float acc = 0.0f;
  for (long long i = blockIdx.x * (long long)kLossThreads + threadIdx.x; i < n; i += (long long)kLossBlocks * kLossThreads) {
    const float fv = ld<TF>(f, i);
    const float d = fv - __ldg(t + i);
    acc = fmaf(d, d, acc);
    if (g) {
      float gv = coef * d;
      if (gram_grad) gv += __ldg(gram_grad + i);
      if (mask && !(fv > 0.0f)) gv = 0.0f;
      g[i] = __float2bfloat16_rn(gv);
    }
  }
  if (partial) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      float s = 0.0f;
      for (int w = 0; w < kLossThreads / 32; ++w) s += s_red[w];
      partial[blockIdx.x] = s;
    }
  }
}

// ---------------------------------------------------------------- loss sums
// out[j] = sum over segments s of group j of w_s x (sum of the segment's floats), added in a
// fixed order by one block: thread t adds elements t, t + 1024, ... of each segment in FP32
// (a few dozen terms), the weighted per-segment totals are kept in double, and the block's
// partials are added in thread order.
constexpr int kMaxLossSegs = 16;
constexpr int kLossSumThreads = 1024;
struct LossSegs {
  long long off[kMaxLossSegs];
  long long len[kMaxLossSegs];
  double w[kMaxLossSegs];
  int group[kMaxLossSegs];
  int n;
};
__global__ void __launch_bounds__(kLossSumThreads) desc_loss_sums_kernel(const float* __restrict__ buf, LossSegs segs,
                                                                          float* __restrict__ out) {
  __shared__ double red[2][kLossSumThreads / 32];
  double acc[2] = {0.0, 0.0};
  for (int k = 0; k < segs.n; ++k) {
    float sk = 0.0f;
    const float* p = buf + segs.off[k];
    const long long len = segs.len[k];
    // the thread's elements i, i + T, i + 2T, ... added in that order, eight loads in flight
    for (long long i = threadIdx.x; i < len; i += 8LL * kLossSumThreads) {
      float q[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const long long e = i + (long long)u * kLossSumThreads;
        q[u] = e < len ? __ldg(p + e) : 0.0f;
      }
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (i + (long long)u * kLossSumThreads < len) sk += q[u];
    }
    acc[segs.group[k]] += segs.w[k] * (double)sk;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    double v = acc[j];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[j][warp] = v;
  }
  __syncthreads();
  if (threadIdx.x < 2) {
    double t = 0.0;
    for (int w = 0; w < kLossSumThreads / 32; ++w) t += red[threadIdx.x][w];
    out[threadIdx.x] = (float)t;
  }
}

}  // namespace desc
}  // namespace svb

using namespace svb;
using namespace svb::desc;

template <bool AVG>
static int pool_fwd(const void* x, void* y, int v, int h, int w, int c, void* stream) {
  if (!x || !y) return fail(SVBRDF_ERR_INVALID, "null pointer");
  if (v < 1 || h < 2 || w < 2 || h % 2 || w % 2 || c < 8 || c % 8)
    return fail(SVBRDF_ERR_UNSUPPORTED, "pool: even H, W and C a multiple of 8 needed");
  if (((uintptr_t)x | (uintptr_t)y) % 16) return fail(SVBRDF_ERR_INVALID, "pool: 16-byte alignment needed");
  if ((long long)v * (h / 2) > 65535 || (long long)(w / 2) * (c / 8) >= (1LL << 30))
    return fail(SVBRDF_ERR_UNSUPPORTED, "pool: too large");
  const dim3 grid((unsigned)(((w / 2) * (c / 8) + 255) / 256), (unsigned)(v * (h / 2)));
  desc_pool_fwd_kernel<AVG><<<grid, 256, 0, (cudaStream_t)stream>>>(
      (const __nv_bfloat16*)x, (__nv_bfloat16*)y, v, h, w, c);
  return check_launch("desc_pool_fwd_kernel");
}

template <bool AVG>
static int pool_bwd(const void* gy, const void* x, const void* addend, void* gx, int v, int h, int w, int c,
                    void* stream) {
  if (!gy || !x || !gx) return fail(SVBRDF_ERR_INVALID, "null pointer");
  if (v < 1 || h < 2 || w < 2 || h % 2 || w % 2 || c < 8 || c % 8)
    return fail(SVBRDF_ERR_UNSUPPORTED, "pool: even H, W and C a multiple of 8 needed");
  if (((uintptr_t)gy | (uintptr_t)x | (uintptr_t)addend | (uintptr_t)gx) % 16)
    return fail(SVBRDF_ERR_INVALID, "pool: 16-byte alignment needed");
  if ((long long)v * (h / 2) > 65535 || (long long)(w / 2) * (c / 8) >= (1LL << 30))
    return fail(SVBRDF_ERR_UNSUPPORTED, "pool: too large");
  const dim3 grid((unsigned)(((w / 2) * (c / 8) + 255) / 256), (unsigned)(v * (h / 2)));
  desc_pool_bwd_kernel<AVG><<<grid, 256, 0, (cudaStream_t)stream>>>(
      (const __nv_bfloat16*)gy, (const __nv_bfloat16*)x, (const __nv_bfloat16*)addend, (__nv_bfloat16*)gx, v, h, w,
      c);
  return check_launch("desc_pool_bwd_kernel");
}

extern "C" {

int svbrdf_desc_partials() { return kLossBlocks; }

int svbrdf_desc_conv1_fwd(const float* renders, const float* weight, const float* bias, float* out_f32,
                          void* out_bf16, int v, int h, int w, int downsample, void* stream) {
  if (!renders || !weight || !bias || !out_f32 || !out_bf16) return fail(SVBRDF_ERR_INVALID, "null pointer");
  if (v < 1 || h < 1 || w < 1) return fail(SVBRDF_ERR_INVALID, "bad shape");
  if (((uintptr_t)out_f32 | (uintptr_t)out_bf16) % 16) return fail(SVBRDF_ERR_INVALID, "outputs must be 16-byte aligned");
  if (v > 65535 || (h + kTileY - 1) / kTileY > 65535) return fail(SVBRDF_ERR_UNSUPPORTED, "conv1_fwd: too large");
  dim3 grid((w + kTile - 1) / kTile, (h + kTileY - 1) / kTileY, v), block(128);
  cudaStream_t st = (cudaStream_t)stream;
  if (downsample)
    desc_conv1_fwd_kernel<true><<<grid, block, 0, st>>>(renders, weight, bias, out_f32, (__nv_bfloat16*)out_bf16, h, w);
  else
    desc_conv1_fwd_kernel<false><<<grid, block, 0, st>>>(renders, weight, bias, out_f32, (__nv_bfloat16*)out_bf16, h, w);
  return check_launch("desc_conv1_fwd_kernel");
}

int svbrdf_desc_conv1_bwd(const void* gz, const float* weight, float* grad_renders, int v, int h, int w, int downsample,
                          void* stream) {
  if (!gz || !weight || !grad_renders) return fail(SVBRDF_ERR_INVALID, "null pointer");
  if (v < 1 || h < 1 || w < 1) return fail(SVBRDF_ERR_INVALID, "bad shape");
  if ((uintptr_t)gz % 16 || (downsample && (uintptr_t)grad_renders % 8))
    return fail(SVBRDF_ERR_INVALID, "misaligned gz/grad_renders");
  dim3 grid((w + kTile - 1) / kTile, (h + kTile - 1) / kTile, v), block(128);
  cudaStream_t st = (cudaStream_t)stream;
  if (downsample)
    desc_conv1_bwd_kernel<true><<<grid, block, 0, st>>>((const __nv_bfloat16*)gz, weight, grad_renders, h, w);
  else
    desc_conv1_bwd_kernel<false><<<grid, block, 0, st>>>((const __nv_bfloat16*)gz, weight, grad_renders, h, w);
  return check_launch("desc_conv1_bwd_kernel");
}

int svbrdf_desc_pool_fwd(const void* x, void* y, int v, int h, int w, int c, void* stream) {
  return pool_fwd<false>(x, y, v, h, w, c, stream);
}

int svbrdf_desc_pool_bwd(const void* gy, const void* x, const void* addend, void* gx, int v, int h, int w, int c,
                         void* stream) {
  return pool_bwd<false>(gy, x, addend, gx, v, h, w, c, stream);
}

int svbrdf_desc_avgpool_fwd(const void* x, void* y, int v, int h, int w, int c, void* stream) {
  return pool_fwd<true>(x, y, v, h, w, c, stream);
}

int svbrdf_desc_avgpool_bwd(const void* gy, const void* x, const void* addend, void* gx, int v, int h, int w, int c,
                            void* stream) {
  return pool_bwd<true>(gy, x, addend, gx, v, h, w, c, stream);
}

int svbrdf_desc_feat_loss(const void* f, int f_is_bf16, const float* t, const float* gram_grad, float coef, int mask,
                          void* g, float* partial, long long n, void* stream) {
  if (!f || !t || n < 1) return fail(SVBRDF_ERR_INVALID, "null pointer or empty");
  cudaStream_t st = (cudaStream_t)stream;
  if (f_is_bf16)
    desc_feat_loss_kernel<__nv_bfloat16><<<kLossBlocks, kLossThreads, 0, st>>>(
        (const __nv_bfloat16*)f, t, gram_grad, coef, mask, (__nv_bfloat16*)g, partial, n);
  else
    desc_feat_loss_kernel<float><<<kLossBlocks, kLossThreads, 0, st>>>((const float*)f, t, gram_grad, coef, mask,
                                                                      (__nv_bfloat16*)g, partial, n);
  return check_launch("desc_feat_loss_kernel");
}

int svbrdf_desc_loss_sums(const float* buf, int n_segs, const long long* offsets, const long long* lengths,
                          const double* weights, const int* groups, float* out, void* stream) {
  if (!buf || !out || !offsets || !lengths || !weights || !groups) return fail(SVBRDF_ERR_INVALID, "null pointer");
  if (n_segs < 1 || n_segs > kMaxLossSegs)
    return fail(SVBRDF_ERR_UNSUPPORTED, "loss sums: 1 to %d segments (got %d)", kMaxLossSegs, n_segs);
  LossSegs segs;
  segs.n = n_segs;
  for (int k = 0; k < n_segs; ++k) {
    if (offsets[k] < 0 || lengths[k] < 0 || (groups[k] != 0 && groups[k] != 1))
      return fail(SVBRDF_ERR_INVALID, "loss sums: bad segment %d", k);
    segs.off[k] = offsets[k];
    segs.len[k] = lengths[k];
    segs.w[k] = weights[k];
    segs.group[k] = groups[k];
  }
  desc_loss_sums_kernel<<<1, kLossSumThreads, 0, (cudaStream_t)stream>>>(buf, segs, out);
  return check_launch("desc_loss_sums_kernel");
}

}  // extern "C"
