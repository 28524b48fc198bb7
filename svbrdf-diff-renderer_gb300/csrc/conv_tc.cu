// BF16 3x3 convolutions (stride 1, zero padding 1) on the 5th-generation tensor cores.
//
// The descriptor loss of the reference (VGGLoss, src/descriptor.py:7-79) runs a VGG19
// feature stack over the renders. Here every 3x3 convolution with at least 64 input
// channels is an implicit GEMM on tcgen05:
//   M = 128 output pixels (an 8 x 16 patch of one image), N = BN output channels,
//   K = 9 taps x Cin, consumed 64 channels (128 bytes of BF16) at a time.
// For each (tap, 64-channel chunk) the producer warp TMA-loads the shifted 8x16x64 input
// patch from the NHWC activation tensor (out-of-image taps read the TMA zero fill, which
// is exactly the padding) and the BN x 64 weight slice, 128-byte swizzled, into a ring of
// shared-memory stages. One thread issues tcgen05.mma (kind::f16, BF16 in, FP32
// accumulate) into a 128 x BN TMEM accumulator; tcgen05.commit frees each stage and finally
// signals the epilogue. Four epilogue warps read TMEM with tcgen05.ld, apply the epilogue
// (bias + ReLU, or a ReLU-mask multiply for the backward pass) and store BF16 NHWC.
// The data gradient of a convolution is the same kernel run on dL/dY with the weights
// transposed (Cin <-> Cout) and flipped (tap -> 8 - tap).
//
// All mbarrier waits are bounded: on timeout the kernel writes an error code to `err`
// and finishes without further waits (TMEM is always released).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <atomic>

#include "tc_ptx.cuh"

namespace svb {
namespace tc {

constexpr int BM = 128;  // output pixels per CTA
constexpr int TH = 8, TW = 16;
constexpr int BK = 64;   // input channels per stage (one 128-byte swizzle row)
constexpr int kThreads = 192;  // warp 0 TMA, warp 1 MMA + TMEM owner, warps 2..5 epilogue

enum Epilogue : int { kEpiNone = 0, kEpiBiasRelu = 1, kEpiMask = 2, kEpiAddMask = 3 };
enum ConvError : int { kErrTma = 11, kErrMma = 12, kErrEpi = 13 };

template <int BN>
struct Shape {
  static constexpr int kABytes = BM * BK * 2;
  static constexpr int kBBytes = BN * BK * 2;
  static constexpr int kStage = kABytes + kBBytes;
};

template <int BN, int STAGES, int EPI>
__global__ void __launch_bounds__(kThreads, 2)
conv3x3_tc_kernel(const __grid_constant__ CUtensorMap tmap_x, const __grid_constant__ CUtensorMap tmap_w,
                  const float* __restrict__ bias, const __nv_bfloat16* __restrict__ mask,
                  const __nv_bfloat16* __restrict__ addend, __nv_bfloat16* __restrict__ y, int H, int W, int Cin,
                  int Cout, int* err) {
  using S = Shape<BN>;
  extern __shared__ uint8_t dsmem[];
  __shared__ __align__(8) uint64_t full_bar[STAGES];
  __shared__ __align__(8) uint64_t empty_bar[STAGES];
  __shared__ __align__(8) uint64_t acc_bar;
  __shared__ uint32_t tmem_slot;

  const uint32_t raw = smem_u32(dsmem);
  const uint32_t base = (raw + 1023u) & ~1023u;  // 128-byte swizzle atoms need 1024-byte alignment
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tiles_x = W / TW, tiles_y = H / TH;
  const int img = blockIdx.x / (tiles_x * tiles_y);
  const int trem = blockIdx.x % (tiles_x * tiles_y);
  const int y0 = (trem / tiles_x) * TH, x0 = (trem % tiles_x) * TW;
  const int n0 = blockIdx.y * BN;
  const int kchunks = Cin / BK;
  const int total = 9 * kchunks;

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
      // ---------------------------------------------------------------- TMA producer
      int issued = 0;
      for (int i = 0; i < total; ++i) {
        const int s = i % STAGES;
        const uint32_t ph = (uint32_t)(i / STAGES) & 1u;
        if (i >= STAGES && !mbar_wait(smem_u32(&empty_bar[s]), ph ^ 1u, err, kErrTma)) break;
        const int tap = i / kchunks, cc = i % kchunks;
        const int dy = tap / 3 - 1, dx = tap % 3 - 1;
        const uint32_t st = base + (uint32_t)(s * S::kStage);
        const uint32_t fb = smem_u32(&full_bar[s]);
        mbar_expect_tx(fb, (uint32_t)S::kStage);
        tma_4d(st, &tmap_x, cc * BK, x0 + dx, y0 + dy, img, fb);
        tma_2d(st + S::kABytes, &tmap_w, tap * Cin + cc * BK, n0, fb);
        ++issued;
      }
      if (issued < total) {
        // aborted: no load may still be writing shared memory when the CTA exits, so wait
        // (bounded) for the loads of the last min(issued, STAGES) stages to land
        for (int i = issued > STAGES ? issued - STAGES : 0; i < issued; ++i) {
          const uint32_t bar = smem_u32(&full_bar[i % STAGES]);
          const uint32_t ph = (uint32_t)(i / STAGES) & 1u;
          uint32_t it = 0;
          while (!mbar_try(bar, ph) && ++it < kSpin) {
          }
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---------------------------------------------------------------- MMA issuer
      constexpr uint32_t idesc = idesc_bf16(BM, BN);
      for (int i = 0; i < total; ++i) {
        const int s = i % STAGES;
        const uint32_t ph = (uint32_t)(i / STAGES) & 1u;
        if (!mbar_wait(smem_u32(&full_bar[s]), ph, err, kErrMma)) break;
        fence_after();
        const uint32_t a = base + (uint32_t)(s * S::kStage);
        const uint32_t b = a + S::kABytes;
#pragma unroll
        for (int k = 0; k < BK / 16; ++k)
          mma_bf16(tmem, sw128_desc(a + 32u * k), sw128_desc(b + 32u * k), idesc, (i > 0 || k > 0) ? 1u : 0u);
        mma_commit(smem_u32(&empty_bar[s]));
      }
      // Committed on the abort path too: acc_bar then completes once every MMA issued so far
      // has finished, so TMEM is not written after the CTA releases it. The epilogue skips
      // its stores when the error word is set.
      mma_commit(smem_u32(&acc_bar));
    }
  } else {
    // ---------------------------------------------------------------- epilogue (warps 2..5)
    const int q = warp & 3;  // TMEM lane quadrant this warp may read
    const int m = q * 32 + lane;
    const int py = y0 + m / TW, px = x0 + m % TW;
    const bool ok = __all_sync(0xffffffffu, mbar_wait(smem_u32(&acc_bar), 0u, err, kErrEpi)) &&
                    *(volatile int*)err == 0;
    fence_after();
    if (ok) {
      const size_t pix = ((size_t)img * H + py) * W + px;
      __nv_bfloat16* out = y + pix * Cout + n0;
#pragma unroll 1
      for (int c0 = 0; c0 < BN; c0 += 32) {
        uint32_t r[32];
        tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c0, r);
        float v[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
        if (EPI == kEpiBiasRelu) {
#pragma unroll
          for (int j = 0; j < 32; ++j) v[j] = fmaxf(v[j] + __ldg(bias + n0 + c0 + j), 0.0f);
        } else if (EPI == kEpiMask || EPI == kEpiAddMask) {
          if (EPI == kEpiAddMask) {  // + the hook's loss gradient at this activation
            const uint4* ap = reinterpret_cast<const uint4*>(addend + pix * Cout + n0 + c0);
#pragma unroll
            for (int u = 0; u < 4; ++u) {
              const uint4 av = __ldg(ap + u);
              const __nv_bfloat162* a2 = reinterpret_cast<const __nv_bfloat162*>(&av);
#pragma unroll
              for (int e = 0; e < 4; ++e) {
                const float2 f = __bfloat1622float2(a2[e]);
                v[u * 8 + 2 * e] += f.x;
                v[u * 8 + 2 * e + 1] += f.y;
              }
            }
          }
          const uint4* mp = reinterpret_cast<const uint4*>(mask + pix * Cout + n0 + c0);
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const uint4 mv = __ldg(mp + u);
            const __nv_bfloat162* m2 = reinterpret_cast<const __nv_bfloat162*>(&mv);
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              const float2 f = __bfloat1622float2(m2[e]);
              v[u * 8 + 2 * e] = f.x > 0.0f ? v[u * 8 + 2 * e] : 0.0f;
              v[u * 8 + 2 * e + 1] = f.y > 0.0f ? v[u * 8 + 2 * e + 1] : 0.0f;
            }
          }
        }
        uint4* op = reinterpret_cast<uint4*>(out + c0);
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          uint4 pk;
          __nv_bfloat162 h0 = __floats2bfloat162_rn(v[u * 8 + 0], v[u * 8 + 1]);
          __nv_bfloat162 h1 = __floats2bfloat162_rn(v[u * 8 + 2], v[u * 8 + 3]);
          __nv_bfloat162 h2 = __floats2bfloat162_rn(v[u * 8 + 4], v[u * 8 + 5]);
          __nv_bfloat162 h3 = __floats2bfloat162_rn(v[u * 8 + 6], v[u * 8 + 7]);
          pk.x = *reinterpret_cast<uint32_t*>(&h0);
          pk.y = *reinterpret_cast<uint32_t*>(&h1);
          pk.z = *reinterpret_cast<uint32_t*>(&h2);
          pk.w = *reinterpret_cast<uint32_t*>(&h3);
          op[u] = pk;
        }
      }
    }
  }
  fence_before();
  __syncthreads();
  if (warp == 1) {
    // The MMAs must be complete before TMEM is released. acc_bar has completed already
    // unless the epilogue's wait gave up; then wait again, bounded, for the issuer's commit.
    uint32_t it = 0;
    while (!mbar_try(smem_u32(&acc_bar), 0u) && ++it < kSpin) {
    }
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)BN) : "memory");
  }
}

// ---------------------------------------------------------------- host side
int get_tensor_map_encoder(PFN_cuTensorMapEncodeTiled_v12000* out) {
  static PFN_cuTensorMapEncodeTiled_v12000 fn_cached = nullptr;
  if (!fn_cached) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    const cudaError_t e =
        cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn)
      return fail(SVBRDF_ERR_CUDA, "cuTensorMapEncodeTiled is not available (%s)", cudaGetErrorString(e));
    fn_cached = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  }
  *out = fn_cached;
  return SVBRDF_OK;
}

template <int BN, int STAGES, int EPI>
static int launch(const CUtensorMap& mx, const CUtensorMap& mw, const float* bias, const void* mask,
                  const void* addend, void* y, int n, int h, int w, int cin, int cout, int* err, cudaStream_t st) {
  auto kern = conv3x3_tc_kernel<BN, STAGES, EPI>;
  const size_t smem = (size_t)STAGES * Shape<BN>::kStage + 1024;
  // cudaFuncSetAttribute applies to the current device only: remember it per device ordinal
  static std::atomic<bool> attr[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
    return fail(SVBRDF_ERR_CUDA, "conv3x3: no usable current device");
  if (!attr[dev].load()) {
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
      return fail(SVBRDF_ERR_CUDA, "cudaFuncSetAttribute: %s", cudaGetErrorString(cudaGetLastError()));
    attr[dev].store(true);
  }
  dim3 grid((unsigned)(n * (h / TH) * (w / TW)), (unsigned)(cout / BN));
  kern<<<grid, kThreads, smem, st>>>(mx, mw, bias, (const __nv_bfloat16*)mask, (const __nv_bfloat16*)addend,
                                     (__nv_bfloat16*)y, h, w, cin, cout, err);
  return check_launch("conv3x3_tc_kernel");
}

template <int BN>
static int dispatch_epi(int epi, const CUtensorMap& mx, const CUtensorMap& mw, const float* bias, const void* mask,
                        const void* addend, void* y, int n, int h, int w, int cin, int cout, int* err,
                        cudaStream_t st) {
  // 96 KB of stages per CTA: two CTAs share an SM (and its 512 TMEM columns), so one
  // CTA's epilogue overlaps the other's main loop
  constexpr int STAGES = BN == 256 ? 2 : (BN == 128 ? 3 : 4);
  switch (epi) {
    case kEpiNone: return launch<BN, STAGES, kEpiNone>(mx, mw, bias, mask, addend, y, n, h, w, cin, cout, err, st);
    case kEpiBiasRelu:
      return launch<BN, STAGES, kEpiBiasRelu>(mx, mw, bias, mask, addend, y, n, h, w, cin, cout, err, st);
    case kEpiMask: return launch<BN, STAGES, kEpiMask>(mx, mw, bias, mask, addend, y, n, h, w, cin, cout, err, st);
    default: return launch<BN, STAGES, kEpiAddMask>(mx, mw, bias, mask, addend, y, n, h, w, cin, cout, err, st);
  }
}

}  // namespace tc
}  // namespace svb

using namespace svb;

extern "C" int svbrdf_conv3x3_bf16_ex(const void* x, const void* weight, const float* bias, const void* mask,
                                      const void* addend, void* y, int n, int h, int w, int cin, int cout, int epilogue,
                                      int* err, void* stream) {
  using namespace svb::tc;
  if (!x || !weight || !y || !err) return fail(SVBRDF_ERR_INVALID, "null x/weight/y/err");
  if (n < 1 || h < TH || w < TW || h % TH || w % TW)
    return fail(SVBRDF_ERR_UNSUPPORTED, "conv3x3: H must be a multiple of %d and W of %d (got %dx%d)", TH, TW, h, w);
  if (cin < BK || cin % BK || cout < 64 || cout % 64 || cin > 4096 || cout > 4096)
    return fail(SVBRDF_ERR_UNSUPPORTED, "conv3x3: channels must be multiples of 64 (got %d -> %d)", cin, cout);
  if (epilogue < kEpiNone || epilogue > kEpiAddMask) return fail(SVBRDF_ERR_INVALID, "bad epilogue %d", epilogue);
  if (epilogue == kEpiBiasRelu && !bias) return fail(SVBRDF_ERR_INVALID, "bias+relu epilogue needs bias");
  if ((epilogue == kEpiMask || epilogue == kEpiAddMask) && !mask)
    return fail(SVBRDF_ERR_INVALID, "mask epilogue needs mask");
  if (epilogue == kEpiAddMask && !addend) return fail(SVBRDF_ERR_INVALID, "add+mask epilogue needs addend");
  if (((uintptr_t)x | (uintptr_t)weight | (uintptr_t)y | (uintptr_t)mask | (uintptr_t)addend) % 16)
    return fail(SVBRDF_ERR_INVALID, "conv3x3: tensors must be 16-byte aligned");
  if ((long long)n * h * w * cin >= (1LL << 40)) return fail(SVBRDF_ERR_UNSUPPORTED, "conv3x3: tensor too large");
  PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
  int rc = get_tensor_map_encoder(&g_encode);
  if (rc) return rc;
  const int bn = (cout % 256 == 0) ? 256 : (cout % 128 == 0 ? 128 : 64);
  CUtensorMap mx, mw;
  {
    const cuuint64_t dims[4] = {(cuuint64_t)cin, (cuuint64_t)w, (cuuint64_t)h, (cuuint64_t)n};
    const cuuint64_t strides[3] = {(cuuint64_t)cin * 2, (cuuint64_t)w * cin * 2, (cuuint64_t)h * w * cin * 2};
    const cuuint32_t box[4] = {(cuuint32_t)BK, (cuuint32_t)TW, (cuuint32_t)TH, 1};
    const cuuint32_t es[4] = {1, 1, 1, 1};
    const CUresult r = g_encode(&mx, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(x), dims, strides, box, es,
                                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(SVBRDF_ERR_CUDA, "cuTensorMapEncodeTiled(x) failed: %d", (int)r);
  }
  {
    const cuuint64_t dims[2] = {(cuuint64_t)9 * cin, (cuuint64_t)cout};
    const cuuint64_t strides[1] = {(cuuint64_t)9 * cin * 2};
    const cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)bn};
    const cuuint32_t es[2] = {1, 1};
    const CUresult r = g_encode(&mw, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(weight), dims, strides, box,
                                es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(SVBRDF_ERR_CUDA, "cuTensorMapEncodeTiled(weight) failed: %d", (int)r);
  }
  cudaStream_t st = (cudaStream_t)stream;
  switch (bn) {
    case 256: return dispatch_epi<256>(epilogue, mx, mw, bias, mask, addend, y, n, h, w, cin, cout, err, st);
    case 128: return dispatch_epi<128>(epilogue, mx, mw, bias, mask, addend, y, n, h, w, cin, cout, err, st);
    default: return dispatch_epi<64>(epilogue, mx, mw, bias, mask, addend, y, n, h, w, cin, cout, err, st);
  }
}

extern "C" int svbrdf_conv3x3_bf16(const void* x, const void* weight, const float* bias, const void* mask, void* y,
                                   int n, int h, int w, int cin, int cout, int epilogue, int* err, void* stream) {
  if (epilogue == svb::tc::kEpiAddMask) return fail(SVBRDF_ERR_INVALID, "add+mask epilogue needs svbrdf_conv3x3_bf16_ex");
  return svbrdf_conv3x3_bf16_ex(x, weight, bias, mask, nullptr, y, n, h, w, cin, cout, epilogue, err, stream);
}
