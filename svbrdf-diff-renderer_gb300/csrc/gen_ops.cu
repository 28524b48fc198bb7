// Elementwise operations of the StyleGAN2-shaped generator used by the MaterialGAN latent loop
// (src/materialgan.py:91-173 drives the reference's generator, src/higan_models/*).
//
//   gen_upsample2_fwd_kernel  2x up-sampling of NCHW FP32 maps: zero insertion followed by the
//                             [1,3,3,1] x [1,3,3,1] / 64 FIR with gain 4 and zero padding, in
//                             polyphase form: out[2m] = (x[m-1] + 3 x[m]) / 4 and
//                             out[2m+1] = (3 x[m] + x[m+1]) / 4 along each axis
//   gen_upsample2_bwd_kernel  its adjoint: gx[m] = (g[2m-1] + 3 g[2m] + 3 g[2m+1] + g[2m+2]) / 4
//                             along each axis, g zero outside
//
// One thread per two output columns (forward) or per input element (adjoint), planes on the
// grid's second axis; both are HBM-bound (the taps come through L1/L2, each output is
// written once).
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

}  // namespace gen
}  // namespace svb

using namespace svb;

extern "C" {

int svbrdf_gen_upsample2(const float* x, float* y, long long planes, int h, int w, void* stream) {
  if (!x || !y || planes < 1 || h < 1 || w < 1) return fail(SVBRDF_ERR_INVALID, "upsample2: bad arguments");
  if (planes > 65535 || 2LL * h * w > (1LL << 30)) return fail(SVBRDF_ERR_UNSUPPORTED, "upsample2: too large");
  if ((uintptr_t)y % 8) return fail(SVBRDF_ERR_INVALID, "upsample2: y must be 8-byte aligned");
  dim3 grid((unsigned)((2LL * h * w + 255) / 256), (unsigned)planes);
  gen::gen_upsample2_fwd_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(x, y, h, w);
  return check_launch("gen_upsample2_fwd_kernel");
}

int svbrdf_gen_upsample2_bwd(const float* g, float* gx, long long planes, int h, int w, void* stream) {
  if (!g || !gx || planes < 1 || h < 1 || w < 1) return fail(SVBRDF_ERR_INVALID, "upsample2_bwd: bad arguments");
  if (planes > 65535 || (long long)h * w > (1LL << 30)) return fail(SVBRDF_ERR_UNSUPPORTED, "upsample2_bwd: too large");
  if ((uintptr_t)g % 8) return fail(SVBRDF_ERR_INVALID, "upsample2_bwd: g must be 8-byte aligned");
  dim3 grid((unsigned)(((long long)h * w + 255) / 256), (unsigned)planes);
  gen::gen_upsample2_bwd_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(g, gx, h, w);
  return check_launch("gen_upsample2_bwd_kernel");
}

}  // extern "C"
