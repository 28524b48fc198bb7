// TF32 convolutions of the MaterialGAN generator on the 5th-generation tensor cores.
//
// The reference's generator (src/higan_models/stylegan2_generator_network.py:585-759) runs its
// modulated 3x3 convolutions through PyTorch, whose cuDNN path computes them in TF32 by default
// (FP32 data, TF32 products, FP32 accumulation). Here the generator's maps stay FP32 and
// channels-last ([B][H][W][C]); the style modulation and demodulation are applied around a
// shared-weight convolution (input channels scaled by the style before it, output channels by
// the demodulation after it, in the elementwise kernels of gen_nhwc.cu), so each layer's
// convolution is one implicit GEMM:
//   M = 128 output pixels: a TH x TW patch of NB images (16 x 8 of one image for maps of 16
//       and more columns; 8 x 8 x 2 images and 4 x 4 x 8 images for the 8^2 and 4^2 maps),
//   N = BN output channels, K = taps x Cin, consumed 32 channels (128 bytes of FP32) at a time.
// For each (tap, 32-channel chunk) the producer warp TMA-loads the shifted input patch (taps
// that fall outside the map read the TMA zero fill, which is the zero padding) and the
// BN x 32 weight slice, 128-byte swizzled, into a ring of shared-memory stages; one thread
// issues tcgen05.mma kind::tf32 (K = 8 per instruction) into a 128 x BN FP32 accumulator in
// TMEM; four epilogue warps read it with tcgen05.ld and store FP32 NHWC.
//
// `pad` is the input offset of the first tap: 1 for the same-padded 3x3 convolutions, 0 for
// the valid 3x3 convolution of the up-sampling layers (whose input is the up-sampled map with
// its one-sample halo), and, for data gradients, 2 - pad of the forward convolution: the data
// gradient of a 3x3 convolution is the same kernel run on dL/dY with the weights transposed
// (Cin <-> Cout) and flipped (tap -> 8 - tap). A 1x1 convolution (toRGB) is taps = 1, pad 0,
// with its 9 output channels padded to 32. Patches at the map's right and bottom edges may
// reach past it: those loads read the zero fill and the epilogue skips those pixels.
//
// Every mbarrier wait is bounded: on timeout the kernel records an error in `err`, stops
// issuing, drains its copies and MMAs (bounded), frees TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <atomic>

#include "tc_ptx.cuh"

namespace svb {
namespace tf32 {

using namespace svb::tc;

constexpr int BM = 128;
constexpr int BK = 32;          // FP32 channels per stage: one 128-byte swizzle row
constexpr int kThreads = 192;   // warp 0 TMA, warp 1 MMA + TMEM owner, warps 2..5 epilogue
enum ConvError : int { kErrTma = 31, kErrMma = 32, kErrEpi = 33 };

// Instruction descriptor, kind::tf32: FP32 accumulator, TF32 A and B, both K-major.
__host__ __device__ constexpr uint32_t idesc_tf32(int m, int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accum) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(accum)
      : "memory");
}

struct Geom {
  int B, Hin, Win, Cin, Ho, Wo, Cout;
  int TH, TW, NB;  // output patch of one CTA: NB images x TH rows x TW columns = 128 pixels
  int pad, taps;
};

template <int BN, int STAGES>
__global__ void __launch_bounds__(kThreads, 1)
conv_tf32_kernel(const __grid_constant__ CUtensorMap tmap_x, const __grid_constant__ CUtensorMap tmap_w,
                 float* __restrict__ y, Geom g, int* err) {
  constexpr int A_BYTES = BM * BK * 4;
  constexpr int B_BYTES = BN * BK * 4;
  constexpr int STAGE = A_BYTES + B_BYTES;
  extern __shared__ uint8_t dsmem[];
  __shared__ __align__(8) uint64_t full_bar[STAGES];
  __shared__ __align__(8) uint64_t empty_bar[STAGES];
  __shared__ __align__(8) uint64_t acc_bar;
  __shared__ uint32_t tmem_slot;

  const uint32_t base = (smem_u32(dsmem) + 1023u) & ~1023u;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tiles_x = (g.Wo + g.TW - 1) / g.TW, tiles_y = (g.Ho + g.TH - 1) / g.TH;
  const int tb = blockIdx.x / (tiles_x * tiles_y);
  const int trem = blockIdx.x % (tiles_x * tiles_y);
  const int b0 = tb * g.NB, y0 = (trem / tiles_x) * g.TH, x0 = (trem % tiles_x) * g.TW;
  const int n0 = blockIdx.y * BN;
  const int kchunks = g.Cin / BK;
  const int total = g.taps * kchunks;
  const int ks = g.taps == 9 ? 3 : 1;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(smem_u32(&full_bar[s]), 1);
      mbar_init(smem_u32(&empty_bar[s]), 1);
    }
    mbar_init(smem_u32(&acc_bar), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"((uint32_t)BN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      int issued = 0;
      for (int i = 0; i < total; ++i) {
        const int s = i % STAGES;
        const uint32_t ph = (uint32_t)(i / STAGES) & 1u;
        if (i >= STAGES && !mbar_wait(smem_u32(&empty_bar[s]), ph ^ 1u, err, kErrTma)) break;
        const int tap = i / kchunks, cc = i % kchunks;
        const int dy = tap / ks - g.pad, dx = tap % ks - g.pad;
        const uint32_t st = base + (uint32_t)(s * STAGE);
        const uint32_t fb = smem_u32(&full_bar[s]);
        mbar_expect_tx(fb, (uint32_t)STAGE);
        tma_4d(st, &tmap_x, cc * BK, x0 + dx, y0 + dy, b0, fb);
        tma_2d(st + A_BYTES, &tmap_w, tap * g.Cin + cc * BK, n0, fb);
        ++issued;
      }
      if (issued < total) {
        for (int i = issued > STAGES ? issued - STAGES : 0; i < issued; ++i) {
          uint32_t it = 0;
          while (!mbar_try(smem_u32(&full_bar[i % STAGES]), (uint32_t)(i / STAGES) & 1u) && ++it < kSpin) {
          }
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t id = idesc_tf32(BM, BN);
      for (int i = 0; i < total; ++i) {
        const int s = i % STAGES;
        const uint32_t ph = (uint32_t)(i / STAGES) & 1u;
        if (!mbar_wait(smem_u32(&full_bar[s]), ph, err, kErrMma)) break;
        fence_after();
        const uint32_t a = base + (uint32_t)(s * STAGE);
        const uint32_t b = a + A_BYTES;
#pragma unroll
        for (int k = 0; k < BK / 8; ++k)  // 8 TF32 channels = 32 bytes per MMA
          mma_tf32(tmem, sw128_desc(a + 32u * k), sw128_desc(b + 32u * k), id, (i > 0 || k > 0) ? 1u : 0u);
        mma_commit(smem_u32(&empty_bar[s]));
      }
      mma_commit(smem_u32(&acc_bar));  // also on abort, so TMEM is idle before it is freed
    }
  } else {
    const int q = warp & 3;
    const int m = q * 32 + lane;
    const int pb = b0 + m / (g.TH * g.TW);
    const int rem = m % (g.TH * g.TW);
    const int py = y0 + rem / g.TW, px = x0 + rem % g.TW;
    const bool inside = pb < g.B && py < g.Ho && px < g.Wo;
    const bool ok = __all_sync(0xffffffffu, mbar_wait(smem_u32(&acc_bar), 0u, err, kErrEpi)) &&
                    *(volatile int*)err == 0;
    fence_after();
    if (ok) {
      float* out = y + (((size_t)pb * g.Ho + py) * g.Wo + px) * g.Cout + n0;
#pragma unroll 1
      for (int c0 = 0; c0 < BN; c0 += 32) {
        uint32_t r[32];
        tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c0, r);
        if (inside) {
          float4* o4 = reinterpret_cast<float4*>(out + c0);
#pragma unroll
          for (int u = 0; u < 8; ++u)
            o4[u] = make_float4(__uint_as_float(r[4 * u]), __uint_as_float(r[4 * u + 1]),
                                __uint_as_float(r[4 * u + 2]), __uint_as_float(r[4 * u + 3]));
        }
      }
    }
  }
  fence_before();
  __syncthreads();
  if (warp == 1) {
    uint32_t it = 0;
    while (!mbar_try(smem_u32(&acc_bar), 0u) && ++it < kSpin) {
    }
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)BN) : "memory");
  }
}

template <int BN, int STAGES>
static int launch(const CUtensorMap& mx, const CUtensorMap& mw, float* y, const Geom& g, int* err, cudaStream_t st) {
  static std::atomic<size_t> have[64];
  const size_t smem = (size_t)STAGES * (BM * BK * 4 + BN * BK * 4) + 1024;
  auto kern = conv_tf32_kernel<BN, STAGES>;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return fail(SVBRDF_ERR_CUDA, "no usable device");
  if (have[dev].load() < smem) {
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
      return fail(SVBRDF_ERR_CUDA, "cudaFuncSetAttribute: %s", cudaGetErrorString(cudaGetLastError()));
    have[dev].store(smem);
  }
  const long long tiles = (long long)((g.B + g.NB - 1) / g.NB) * ((g.Ho + g.TH - 1) / g.TH) * ((g.Wo + g.TW - 1) / g.TW);
  dim3 grid((unsigned)tiles, (unsigned)(g.Cout / BN));
  kern<<<grid, kThreads, smem, st>>>(mx, mw, y, g, err);
  return check_launch("conv_tf32_kernel");
}

}  // namespace tf32
}  // namespace svb

using namespace svb;

extern "C" int svbrdf_gen_conv_tf32(const float* x, const float* weight, float* y, int b, int hin, int win, int cin,
                                    int cout, int ksize, int pad, int* err, void* stream) {
  using namespace svb::tf32;
  if (!x || !weight || !y || !err) return fail(SVBRDF_ERR_INVALID, "conv_tf32: null x/weight/y/err");
  if (ksize != 1 && ksize != 3) return fail(SVBRDF_ERR_INVALID, "conv_tf32: ksize must be 1 or 3");
  if (pad < 0 || pad > (ksize == 3 ? 2 : 0)) return fail(SVBRDF_ERR_INVALID, "conv_tf32: bad pad %d", pad);
  if (b < 1 || hin < 1 || win < 1 || cin < BK || cin % BK || cin > 8192)
    return fail(SVBRDF_ERR_UNSUPPORTED, "conv_tf32: Cin must be a multiple of %d (got %d)", BK, cin);
  if (cout < 32 || !(cout % 256 == 0 || cout == 128 || cout == 64 || cout == 32))
    return fail(SVBRDF_ERR_UNSUPPORTED, "conv_tf32: Cout must be 32, 64, 128 or a multiple of 256 (got %d)", cout);
  Geom g;
  g.B = b; g.Hin = hin; g.Win = win; g.Cin = cin; g.Cout = cout; g.pad = pad; g.taps = ksize * ksize;
  g.Ho = hin + 2 * pad - (ksize - 1);
  g.Wo = win + 2 * pad - (ksize - 1);
  if (g.Ho < 1 || g.Wo < 1) return fail(SVBRDF_ERR_INVALID, "conv_tf32: empty output");
  // output patch: 16 columns x 8 rows of one image, else whole small images stacked
  if (g.Wo >= 16) { g.TW = 16; g.TH = 8; g.NB = 1; }
  else if (g.Wo >= 8) { g.TW = 8; g.TH = 8; g.NB = 2; }
  else if (g.Wo >= 4) { g.TW = 4; g.TH = 4; g.NB = 8; }
  else return fail(SVBRDF_ERR_UNSUPPORTED, "conv_tf32: output narrower than 4");
  if ((long long)b * hin * win * cin >= (1LL << 40) || (long long)b * g.Ho * g.Wo >= (1LL << 31))
    return fail(SVBRDF_ERR_UNSUPPORTED, "conv_tf32: tensor too large");
  if (((uintptr_t)x | (uintptr_t)weight | (uintptr_t)y) % 16) return fail(SVBRDF_ERR_INVALID, "conv_tf32: 16-byte alignment");
  PFN_cuTensorMapEncodeTiled_v12000 enc = nullptr;
  int rc = get_tensor_map_encoder(&enc);
  if (rc) return rc;
  const int bn = cout >= 256 ? 256 : cout;
  CUtensorMap mx, mw;
  {
    const cuuint64_t dims[4] = {(cuuint64_t)cin, (cuuint64_t)win, (cuuint64_t)hin, (cuuint64_t)b};
    const cuuint64_t strides[3] = {(cuuint64_t)cin * 4, (cuuint64_t)win * cin * 4, (cuuint64_t)hin * win * cin * 4};
    const cuuint32_t box[4] = {(cuuint32_t)BK, (cuuint32_t)g.TW, (cuuint32_t)g.TH, (cuuint32_t)g.NB};
    const cuuint32_t es[4] = {1, 1, 1, 1};
    const CUresult r = enc(&mx, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<float*>(x), dims, strides, box, es,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(SVBRDF_ERR_CUDA, "cuTensorMapEncodeTiled(x) failed: %d", (int)r);
  }
  {
    const cuuint64_t dims[2] = {(cuuint64_t)g.taps * cin, (cuuint64_t)cout};
    const cuuint64_t strides[1] = {(cuuint64_t)g.taps * cin * 4};
    const cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)bn};
    const cuuint32_t es[2] = {1, 1};
    const CUresult r = enc(&mw, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(weight), dims, strides, box, es,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(SVBRDF_ERR_CUDA, "cuTensorMapEncodeTiled(weight) failed: %d", (int)r);
  }
  cudaStream_t st = (cudaStream_t)stream;
  switch (bn) {
    case 256: return launch<256, 4>(mx, mw, y, g, err, st);
    case 128: return launch<128, 5>(mx, mw, y, g, err, st);
    case 64: return launch<64, 6>(mx, mw, y, g, err, st);
    default: return launch<32, 6>(mx, mw, y, g, err, st);
  }
}
