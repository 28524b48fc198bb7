// BF16 3x3 convolutions (stride 1, zero padding 1) on the 5th-generation tensor cores.
//
// The descriptor loss of the reference (VGGLoss, src/descriptor.py:7-79) runs a VGG19
// feature stack over the renders. Here every 3x3 convolution with at least 64 input
// channels is an implicit GEMM on tcgen05:
//   M = 128 output pixels per M-tile (an 8 x 16 patch of one image; a tile stacks MT = 2 of
//   them along y where Cout <= 128, so one weight slice feeds 256 pixels), N = BN output
//   channels, K = 9 taps x Cin, consumed 64 channels (128 bytes of BF16) at a time.
// The kernel is persistent: one CTA per SM walks the tiles i, i + grid, ... For each (tap,
// 64-channel chunk) the producer warp TMA-loads the shifted 8x16x64 input patches from the
// NHWC activation tensor (out-of-image taps read the TMA zero fill, which is exactly the
// padding) and the BN x 64 weight slice, 128-byte swizzled, into a ring of shared-memory
// stages that runs on across tiles. One thread issues tcgen05.mma (kind::f16, BF16 in, FP32
// accumulate) into MT 128 x BN TMEM accumulators, double-buffered; tcgen05.commit frees each
// stage and signals the epilogue per tile. Four epilogue warps read TMEM with tcgen05.ld,
// apply the epilogue (bias + ReLU, or a ReLU-mask multiply for the backward pass) and store
// BF16 NHWC while the MMAs of the next tile run.
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

constexpr int BM = 128;  // output pixels per M-tile
constexpr int TH = 8, TW = 16;
constexpr int BK = 64;   // input channels per stage (one 128-byte swizzle row)
constexpr int kThreads = 192;  // warp 0 TMA, warp 1 MMA + TMEM owner, warps 2..5 epilogue

enum Epilogue : int { kEpiNone = 0, kEpiBiasRelu = 1, kEpiMask = 2, kEpiAddMask = 3 };
enum ConvError : int { kErrTma = 11, kErrMma = 12, kErrEpi = 13 };

// One accumulator row (an output pixel) of 32 channels through the epilogue, stored as BF16.
template <int EPI>
__device__ __forceinline__ void epilogue_store32(const uint32_t (&r)[32], const float* __restrict__ bias,
                                                 const __nv_bfloat16* __restrict__ mask,
                                                 const __nv_bfloat16* __restrict__ addend, __nv_bfloat16* out,
                                                 size_t off, int nc) {
  float v[32];
#pragma unroll
  for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
  if (EPI == kEpiBiasRelu) {
#pragma unroll
    for (int j = 0; j < 32; ++j) v[j] = fmaxf(v[j] + __ldg(bias + nc + j), 0.0f);
  } else if (EPI == kEpiMask || EPI == kEpiAddMask) {
    if (EPI == kEpiAddMask) {  // + the hook's loss gradient at this activation
      const uint4* ap = reinterpret_cast<const uint4*>(addend + off);
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
    const uint4* mp = reinterpret_cast<const uint4*>(mask + off);
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
  uint4* op = reinterpret_cast<uint4*>(out + off);
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

// Persistent: grid = min(tiles, SMs), CTA i runs tiles i, i + grid, ... A tile is MT stacked
// 8 x 16 patches of one image (MT x 128 output pixels) x BN output channels; tiles sharing a
// patch are consecutive, so their input loads meet in L2. The producer's ring runs on across
// tiles and the MT accumulators are double-buffered in TMEM, so the epilogue of tile j
// overlaps the MMAs of tile j + 1.
template <int BN, int MT, int STAGES, int EPI>
__global__ void __launch_bounds__(kThreads, 1)
conv3x3_tc_kernel(const __grid_constant__ CUtensorMap tmap_x, const __grid_constant__ CUtensorMap tmap_w,
                  const float* __restrict__ bias, const __nv_bfloat16* __restrict__ mask,
                  const __nv_bfloat16* __restrict__ addend, __nv_bfloat16* __restrict__ y, int N, int H, int W,
                  int Cin, int Cout, int* err) {
  constexpr int A_BYTES = BM * BK * 2;
  constexpr int B_BYTES = BN * BK * 2;
  constexpr int STAGE = MT * A_BYTES + B_BYTES;
  constexpr uint32_t ACC_COLS = MT * BN;
  constexpr uint32_t TMEM_COLS = 2 * ACC_COLS;
  static_assert(TMEM_COLS >= 32 && TMEM_COLS <= 512 && (TMEM_COLS & (TMEM_COLS - 1)) == 0, "TMEM columns");
  extern __shared__ uint8_t dsmem[];
  __shared__ __align__(8) uint64_t full_bar[STAGES];
  __shared__ __align__(8) uint64_t empty_bar[STAGES];
  __shared__ __align__(8) uint64_t tfull_bar[2];   // accumulator buffer ready (MMA commit)
  __shared__ __align__(8) uint64_t tempty_bar[2];  // accumulator buffer drained (4 epilogue warps)
  __shared__ __align__(8) uint64_t done_bar;       // every MMA of this CTA complete
  __shared__ uint32_t tmem_slot;

  const uint32_t base = (smem_u32(dsmem) + 1023u) & ~1023u;  // 128-byte swizzle atoms need 1024-byte alignment
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tiles_x = W / TW, tiles_y = H / (TH * MT), tiles_n = Cout / BN;
  const int n_tiles = N * tiles_y * tiles_x * tiles_n;
  const int kchunks = Cin / BK;
  const int total = 9 * kchunks;
  auto coord = [&](int t, int& img, int& y0, int& x0, int& n0) {
    n0 = (t % tiles_n) * BN;
    int r = t / tiles_n;
    x0 = (r % tiles_x) * TW;
    r /= tiles_x;
    y0 = (r % tiles_y) * (TH * MT);
    img = r / tiles_y;
  };

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(smem_u32(&full_bar[s]), 1);
      mbar_init(smem_u32(&empty_bar[s]), 1);
    }
    for (int a = 0; a < 2; ++a) {
      mbar_init(smem_u32(&tfull_bar[a]), 1);
      mbar_init(smem_u32(&tempty_bar[a]), 4);
    }
    mbar_init(smem_u32(&done_bar), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(TMEM_COLS)
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
      int q = 0;  // stages issued by this CTA
      bool bad = false;
      for (int t = blockIdx.x; t < n_tiles && !bad; t += gridDim.x) {
        int img, y0, x0, n0;
        coord(t, img, y0, x0, n0);
        for (int i = 0; i < total; ++i) {
          const int s = q % STAGES;
          const uint32_t ph = (uint32_t)(q / STAGES) & 1u;
          if (q >= STAGES && !mbar_wait(smem_u32(&empty_bar[s]), ph ^ 1u, err, kErrTma)) {
            bad = true;
            break;
          }
          const int tap = i / kchunks, cc = i % kchunks;
          const int dy = tap / 3 - 1, dx = tap % 3 - 1;
          const uint32_t st = base + (uint32_t)(s * STAGE);
          const uint32_t fb = smem_u32(&full_bar[s]);
          mbar_expect_tx(fb, (uint32_t)STAGE);
#pragma unroll
          for (int mt = 0; mt < MT; ++mt)
            tma_4d(st + (uint32_t)(mt * A_BYTES), &tmap_x, cc * BK, x0 + dx, y0 + mt * TH + dy, img, fb);
          tma_2d(st + (uint32_t)(MT * A_BYTES), &tmap_w, tap * Cin + cc * BK, n0, fb);
          ++q;
        }
      }
      if (bad) {
        // aborted: no load may still be writing shared memory when the CTA exits, so wait
        // (bounded) for the loads of the last min(q, STAGES) stages to land
        for (int i = q > STAGES ? q - STAGES : 0; i < q; ++i) {
          uint32_t it = 0;
          while (!mbar_try(smem_u32(&full_bar[i % STAGES]), (uint32_t)(i / STAGES) & 1u) && ++it < kSpin) {
          }
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---------------------------------------------------------------- MMA issuer
      constexpr uint32_t idesc = idesc_bf16(BM, BN);
      int q = 0, j = 0;
      bool bad = false;
      for (int t = blockIdx.x; t < n_tiles && !bad; t += gridDim.x, ++j) {
        const int a = j & 1;
        // the epilogue must have drained this buffer's previous tile (j - 2)
        if (j >= 2 && !mbar_wait(smem_u32(&tempty_bar[a]), ((uint32_t)(j >> 1) & 1u) ^ 1u, err, kErrMma)) break;
        fence_after();
        const uint32_t acc = tmem + (uint32_t)a * ACC_COLS;
        for (int i = 0; i < total; ++i, ++q) {
          const int s = q % STAGES;
          const uint32_t ph = (uint32_t)(q / STAGES) & 1u;
          if (!mbar_wait(smem_u32(&full_bar[s]), ph, err, kErrMma)) {
            bad = true;
            break;
          }
          fence_after();
          const uint32_t sa = base + (uint32_t)(s * STAGE);
          const uint32_t sb = sa + (uint32_t)(MT * A_BYTES);
#pragma unroll
          for (int k = 0; k < BK / 16; ++k) {
#pragma unroll
            for (int mt = 0; mt < MT; ++mt)
              mma_bf16(acc + (uint32_t)(mt * BN), sw128_desc(sa + (uint32_t)(mt * A_BYTES) + 32u * k),
                       sw128_desc(sb + 32u * k), idesc, (i > 0 || k > 0) ? 1u : 0u);
          }
          mma_commit(smem_u32(&empty_bar[s]));
        }
        if (!bad) mma_commit(smem_u32(&tfull_bar[a]));
      }
      // Committed on the abort path too: done_bar completes once every MMA issued so far has
      // finished, so TMEM is not written after the CTA releases it.
      mma_commit(smem_u32(&done_bar));
    }
  } else {
    // ---------------------------------------------------------------- epilogue (warps 2..5)
    const int qw = warp & 3;  // TMEM lane quadrant this warp may read
    const int m = qw * 32 + lane;
    int j = 0;
    for (int t = blockIdx.x; t < n_tiles; t += gridDim.x, ++j) {
      const int a = j & 1;
      const bool ok = __all_sync(0xffffffffu, mbar_wait(smem_u32(&tfull_bar[a]), (uint32_t)(j >> 1) & 1u, err,
                                                        kErrEpi)) &&
                      *(volatile int*)err == 0;
      fence_after();
      if (!ok) break;  // the error word is set; no store of this tile happens
      int img, y0, x0, n0;
      coord(t, img, y0, x0, n0);
#pragma unroll
      for (int mt = 0; mt < MT; ++mt) {
        const size_t pix = ((size_t)img * H + y0 + mt * TH + m / TW) * W + x0 + m % TW;
#pragma unroll 1
        for (int c0 = 0; c0 < BN; c0 += 32) {
          uint32_t r[32];
          tmem_ld32(tmem + ((uint32_t)(qw * 32) << 16) + (uint32_t)(a * ACC_COLS + mt * BN + c0), r);
          epilogue_store32<EPI>(r, bias, mask, addend, y, pix * Cout + n0 + c0, n0 + c0);
        }
      }
      fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_u32(&tempty_bar[a]));
    }
  }
  fence_before();
  __syncthreads();
  if (warp == 1) {
    // every MMA must be complete before TMEM is released (bounded wait for the final commit)
    uint32_t it = 0;
    while (!mbar_try(smem_u32(&done_bar), 0u) && ++it < kSpin) {
    }
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
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

constexpr size_t kStageBudget = 200 * 1024;  // ring bytes per CTA (one CTA per SM)

template <int BN, int MT>
constexpr int conv_stages() {
  return (int)(kStageBudget / (size_t)(MT * BM * BK * 2 + BN * BK * 2)) < 8
             ? (int)(kStageBudget / (size_t)(MT * BM * BK * 2 + BN * BK * 2))
             : 8;
}

template <int BN, int MT, int EPI>
static int launch(const CUtensorMap& mx, const CUtensorMap& mw, const float* bias, const void* mask,
                  const void* addend, void* y, int n, int h, int w, int cin, int cout, int* err, cudaStream_t st) {
  constexpr int STAGES = conv_stages<BN, MT>();
  static_assert(STAGES >= 3, "ring too shallow");
  auto kern = conv3x3_tc_kernel<BN, MT, STAGES, EPI>;
  const size_t smem = (size_t)STAGES * (MT * BM * BK * 2 + BN * BK * 2) + 1024;
  // cudaFuncSetAttribute applies to the current device only: remember it per device ordinal
  static std::atomic<bool> attr[64];
  static std::atomic<int> sms[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
    return fail(SVBRDF_ERR_CUDA, "conv3x3: no usable current device");
  if (!attr[dev].load()) {
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
      return fail(SVBRDF_ERR_CUDA, "cudaFuncSetAttribute: %s", cudaGetErrorString(cudaGetLastError()));
    attr[dev].store(true);
  }
  if (sms[dev].load() == 0) {
    int c = 0;
    if (cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || c < 1)
      return fail(SVBRDF_ERR_CUDA, "conv3x3: no SM count");
    sms[dev].store(c);
  }
  const long long tiles = (long long)n * (h / (TH * MT)) * (w / TW) * (cout / BN);
  if (tiles >= (1LL << 31)) return fail(SVBRDF_ERR_UNSUPPORTED, "conv3x3: too many tiles");
  const int grid = (int)(tiles < sms[dev].load() ? tiles : sms[dev].load());
  kern<<<grid, kThreads, smem, st>>>(mx, mw, bias, (const __nv_bfloat16*)mask, (const __nv_bfloat16*)addend,
                                     (__nv_bfloat16*)y, n, h, w, cin, cout, err);
  return check_launch("conv3x3_tc_kernel");
}

template <int BN, int MT>
static int dispatch_epi(int epi, const CUtensorMap& mx, const CUtensorMap& mw, const float* bias, const void* mask,
                        const void* addend, void* y, int n, int h, int w, int cin, int cout, int* err,
                        cudaStream_t st) {
  switch (epi) {
    case kEpiNone: return launch<BN, MT, kEpiNone>(mx, mw, bias, mask, addend, y, n, h, w, cin, cout, err, st);
    case kEpiBiasRelu:
      return launch<BN, MT, kEpiBiasRelu>(mx, mw, bias, mask, addend, y, n, h, w, cin, cout, err, st);
    case kEpiMask: return launch<BN, MT, kEpiMask>(mx, mw, bias, mask, addend, y, n, h, w, cin, cout, err, st);
    default: return launch<BN, MT, kEpiAddMask>(mx, mw, bias, mask, addend, y, n, h, w, cin, cout, err, st);
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
  // two stacked 8 x 16 patches per tile (each weight slice feeds 256 pixels) where H allows and
  // Cout fits two double-buffered pairs of accumulators in TMEM
  const bool two = h % (2 * TH) == 0 && bn <= 128;
  switch (bn) {
    case 256: return dispatch_epi<256, 1>(epilogue, mx, mw, bias, mask, addend, y, n, h, w, cin, cout, err, st);
    case 128:
      return two ? dispatch_epi<128, 2>(epilogue, mx, mw, bias, mask, addend, y, n, h, w, cin, cout, err, st)
                 : dispatch_epi<128, 1>(epilogue, mx, mw, bias, mask, addend, y, n, h, w, cin, cout, err, st);
    default:
      return two ? dispatch_epi<64, 2>(epilogue, mx, mw, bias, mask, addend, y, n, h, w, cin, cout, err, st)
                 : dispatch_epi<64, 1>(epilogue, mx, mw, bias, mask, addend, y, n, h, w, cin, cout, err, st);
  }
}

extern "C" int svbrdf_conv3x3_bf16(const void* x, const void* weight, const float* bias, const void* mask, void* y,
                                   int n, int h, int w, int cin, int cout, int epilogue, int* err, void* stream) {
  if (epilogue == svb::tc::kEpiAddMask) return fail(SVBRDF_ERR_INVALID, "add+mask epilogue needs svbrdf_conv3x3_bf16_ex");
  return svbrdf_conv3x3_bf16_ex(x, weight, bias, mask, nullptr, y, n, h, w, cin, cout, epilogue, err, stream);
}
