// BF16 3x3 convolutions (stride 1, zero padding 1) on the 5th-generation tensor cores.
//
// The descriptor loss of the reference (VGGLoss, src/descriptor.py:7-79) runs a VGG19
// feature stack over the renders. Here every 3x3 convolution with at least 64 input
// channels is an implicit GEMM on tcgen05:
//   M = 128 output pixels per M-tile (a 16-row x 8-column patch of one image; a tile stacks
//   MT = 2 of them along y where Cout <= 128, so one weight slice feeds 256 pixels), N = BN
//   output channels, K = 9 taps x Cin, consumed 64 channels (128 bytes of BF16) at a time.
// The kernel is persistent: one CTA per SM walks the tiles i, i + grid, ... For each 64-channel
// chunk the producer warp TMA-loads the tile's input patch once, with its one-pixel halo
// (out-of-image pixels read the TMA zero fill, which is exactly the padding), and the 9 taps'
// BN x 64 weight slices, all 128-byte swizzled, into two rings of shared-memory stages that run
// on across tiles; the 9 taps read the one patch through shifted descriptors (the halo form
// below). One thread issues tcgen05.mma (kind::f16, BF16 in, FP32 accumulate) into MT
// 128 x BN TMEM accumulators, double-buffered; tcgen05.commit frees each stage and signals the
// epilogue per tile. A commit group of MMAs costs at least about 560 cycles on this part (an
// M=128, N=64, K=16 MMA issues every 48 cycles, N=128 every 64), so where BN <= 128 a weight
// stage holds a whole kernel row (3 taps, 24 MMAs per commit) instead of one tap. Eight epilogue warps (two per TMEM lane quadrant, each with half the
// columns) read TMEM with tcgen05.ld, apply the epilogue (bias + ReLU, or a ReLU-mask multiply
// for the backward pass) and store BF16 NHWC while the MMAs of the next tile run.
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
constexpr int TH = 8, TW = 16;  // the entry point's shape granularity (H % 8, W % 16)
constexpr int BK = 64;   // input channels per chunk (one 128-byte weight row)
constexpr int kThreads = 320;  // warp 0 TMA, warp 1 MMA + TMEM owner, warps 2..9 epilogue
constexpr int kEpiWarps = 8;  // two per TMEM lane quadrant, each draining half the columns

// kEpiUnpoolMax / kEpiUnpoolAvg: the convolution's output is the gradient at a 2x2 pool's
// output; the epilogue routes it back to the pool's input (the window's first maximum, or a
// quarter to each element), adds the addend there and applies the ReLU mask of the pool's input.
// `mask` is the pool's input and `y` the gradient at it, both [N, 2H, 2W, Cout].
// kEpiRenderDown / kEpiRender (BN = 16, the data gradient of the descriptor's first layer,
// 64 -> 3 channels padded to 16): channel c < 3 of the accumulator times scale[c] (`bias`) is the
// gradient at the normalised render, written FP32 NCHW to `y` [N][3][2H][2W] through the 2x2
// box downsample's adjoint (each of the window's 4 pixels takes the value; the 1/4 is in scale)
// or [N][3][H][W] without it.
enum Epilogue : int { kEpiNone = 0, kEpiBiasRelu = 1, kEpiMask = 2, kEpiAddMask = 3, kEpiUnpoolMax = 4,
                      kEpiUnpoolAvg = 5, kEpiRenderDown = 6, kEpiRender = 7 };
enum ConvError : int { kErrTma = 11, kErrMma = 12, kErrEpi = 13 };

// One accumulator row (an output pixel) of 32 channels through the epilogue, stored as BF16;
// `mv` and `av` hold the row's 32 mask and addend values (BF16, 4 x 16 bytes each).
template <int EPI>
__device__ __forceinline__ void epilogue_values32(const uint32_t (&r)[32], const float* __restrict__ bias,
                                                  const uint4 (&mv)[4], const uint4 (&av)[4], int nc, uint4 (&pk)[4]) {
  float v[32];
#pragma unroll
  for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
  if (EPI == kEpiBiasRelu) {
#pragma unroll
    for (int j = 0; j < 32; ++j) v[j] = fmaxf(v[j] + __ldg(bias + nc + j), 0.0f);
  } else if (EPI == kEpiMask || EPI == kEpiAddMask) {
    if (EPI == kEpiAddMask) {  // + the hook's loss gradient at this activation
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const __nv_bfloat162* a2 = reinterpret_cast<const __nv_bfloat162*>(&av[u]);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const float2 f = __bfloat1622float2(a2[e]);
          v[u * 8 + 2 * e] += f.x;
          v[u * 8 + 2 * e + 1] += f.y;
        }
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const __nv_bfloat162* m2 = reinterpret_cast<const __nv_bfloat162*>(&mv[u]);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const float2 f = __bfloat1622float2(m2[e]);
        v[u * 8 + 2 * e] = f.x > 0.0f ? v[u * 8 + 2 * e] : 0.0f;
        v[u * 8 + 2 * e + 1] = f.y > 0.0f ? v[u * 8 + 2 * e + 1] : 0.0f;
      }
    }
  }
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    __nv_bfloat162 h0 = __floats2bfloat162_rn(v[u * 8 + 0], v[u * 8 + 1]);
    __nv_bfloat162 h1 = __floats2bfloat162_rn(v[u * 8 + 2], v[u * 8 + 3]);
    __nv_bfloat162 h2 = __floats2bfloat162_rn(v[u * 8 + 4], v[u * 8 + 5]);
    __nv_bfloat162 h3 = __floats2bfloat162_rn(v[u * 8 + 6], v[u * 8 + 7]);
    pk[u].x = *reinterpret_cast<uint32_t*>(&h0);
    pk[u].y = *reinterpret_cast<uint32_t*>(&h1);
    pk[u].z = *reinterpret_cast<uint32_t*>(&h2);
    pk[u].w = *reinterpret_cast<uint32_t*>(&h3);
  }
}
template <int EPI>
__device__ __forceinline__ void epilogue_apply32(const uint32_t (&r)[32], const float* __restrict__ bias,
                                                 const uint4 (&mv)[4], const uint4 (&av)[4], __nv_bfloat16* out,
                                                 size_t off, int nc) {
  uint4 pk[4];
  epilogue_values32<EPI>(r, bias, mv, av, nc, pk);
  uint4* op = reinterpret_cast<uint4*>(out + off);
#pragma unroll
  for (int u = 0; u < 4; ++u) op[u] = pk[u];
}

// The row's mask (and addend) values, 4 x 16 bytes each, for epilogue_apply32.
template <int EPI>
__device__ __forceinline__ void epilogue_load32(const __nv_bfloat16* __restrict__ mask,
                                                const __nv_bfloat16* __restrict__ addend, size_t off, uint4 (&mv)[4],
                                                uint4 (&av)[4]) {
  if (EPI == kEpiMask || EPI == kEpiAddMask) {
#pragma unroll
    for (int u = 0; u < 4; ++u) mv[u] = __ldg(reinterpret_cast<const uint4*>(mask + off) + u);
  }
  if (EPI == kEpiAddMask) {
#pragma unroll
    for (int u = 0; u < 4; ++u) av[u] = __ldg(reinterpret_cast<const uint4*>(addend + off) + u);
  }
}

// One accumulator row (the gradient at pool-output pixel (py, px), 32 channels) routed back
// through a 2x2 pool: `base` is element (2 py, 2 px, channel) of the [.., 2H, 2W, Cout] maps,
// `rs` their row stride in elements. Window order (0,0), (0,1), (1,0), (1,1); a max-pool's
// gradient goes to the first maximum (strictly greater replaces).
template <bool AVG>
__device__ __forceinline__ void epilogue_unpool32(const uint32_t (&r)[32], const __nv_bfloat16* __restrict__ x,
                                                  const __nv_bfloat16* __restrict__ addend, __nv_bfloat16* out,
                                                  size_t base, size_t rs, int cout) {
  const size_t offs[4] = {base, base + cout, base + rs, base + rs + cout};
#pragma unroll
  for (int u = 0; u < 4; ++u) {  // 8 channels at a time
    uint4 xv[4], av[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) xv[k] = __ldg(reinterpret_cast<const uint4*>(x + offs[k]) + u);
    if (addend) {
#pragma unroll
      for (int k = 0; k < 4; ++k) av[k] = __ldg(reinterpret_cast<const uint4*>(addend + offs[k]) + u);
    }
    float xf[4][8], o[4][8];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&xv[k]);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const float2 f = __bfloat1622float2(h[e]);
        xf[k][2 * e] = f.x;
        xf[k][2 * e + 1] = f.y;
      }
    }
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const float g = __uint_as_float(r[u * 8 + c]);
      int am = 0;
      if (!AVG) {
        float m = xf[0][c];
#pragma unroll
        for (int k = 1; k < 4; ++k)
          if (xf[k][c] > m) {
            m = xf[k][c];
            am = k;
          }
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) o[k][c] = AVG ? 0.25f * g : (am == k ? g : 0.0f);
    }
    if (addend) {
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&av[k]);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const float2 f = __bfloat1622float2(h[e]);
          o[k][2 * e] += f.x;
          o[k][2 * e + 1] += f.y;
        }
      }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      uint4 pk;
      uint32_t* pw = reinterpret_cast<uint32_t*>(&pk);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const float a0 = xf[k][2 * e] > 0.0f ? o[k][2 * e] : 0.0f;
        const float a1 = xf[k][2 * e + 1] > 0.0f ? o[k][2 * e + 1] : 0.0f;
        __nv_bfloat162 hh = __floats2bfloat162_rn(a0, a1);
        pw[e] = *reinterpret_cast<uint32_t*>(&hh);
      }
      reinterpret_cast<uint4*>(out + offs[k])[u] = pk;
    }
  }
}

// ---------------------------------------------------------------- halo form
// Each input patch is loaded once per 64-channel chunk, halo included, and shared by the 9
// taps. A tile is MT stacked 16-row x 8-column patches of one image; its input is the
// (16 MT + 2) x 10 halo patch, one TMA box of 128-byte pixel rows (64 BF16 channels), 128-byte
// swizzled, pixels row-major (10 per patch row) from a 1024-byte boundary. The 128 accumulator
// rows of M-tile mt are the patch's 16 rows of 8 pixels: 8-row group r of tap (ky, kx) starts at
// patch pixel (16 mt + r + ky) x 10 + kx, so a tap is the patch's descriptor moved by
// (10 ky + kx) pixels, with 8-row groups 10 pixels (1280 bytes) apart (SBO). The weight slices
// [BN][64] stream through their own ring, TPS taps per stage; with RESB (one 64-channel chunk,
// one Cout block: conv1_2 and its data gradient) all 9 slices are one stage, loaded once per
// CTA and never released. Per chunk the tile loads (16 MT + 2) x 10 x 128 bytes of input instead
// of 9 x MT x 16 KB.
// TST (BN = 64, MT = 2, epilogues 0..3): each epilogue warp writes its 32 pixels x 64 channels,
// BF16, into its own 4 KB block of shared memory (128-byte rows, 128-byte swizzled) and one lane
// stores the block with a TMA tensor store (`tmap_y`, box 64 x 8 x 4), instead of 2048 16-byte
// stores per tile spread over 128-byte strides.
template <int MT>
struct Halo {
  static constexpr int kRows = 16 * MT + 2, kCols = 10;
  static constexpr int kABytes = ((kRows * kCols * 128 + 1023) / 1024) * 1024;  // one 64-channel chunk
};

template <int BN, int MT, int AST, int BST, int EPI, int TPS, bool RESB, bool TST>
__global__ void __launch_bounds__(kThreads, 1)
conv3x3_halo_kernel(const __grid_constant__ CUtensorMap tmap_x, const __grid_constant__ CUtensorMap tmap_w,
                    const __grid_constant__ CUtensorMap tmap_y, const float* __restrict__ bias,
                    const __nv_bfloat16* __restrict__ mask, const __nv_bfloat16* __restrict__ addend,
                    __nv_bfloat16* __restrict__ y, int N, int H, int W, int Cin, int Cout, int* err) {
  using HP = Halo<MT>;
  constexpr int B_BYTES = BN * BK * 2;  // one tap's weight slice
  constexpr int S_BYTES = TPS * B_BYTES;  // one weight stage
  constexpr int GROUPS = 9 / TPS;
  static_assert(TPS == 1 || TPS == 3 || TPS == 9, "a weight stage holds one tap, a kernel row or all 9");
  static_assert(!RESB || (TPS == 9 && BST == 1), "resident weights: one stage of all 9 taps");
  static_assert(!TST || (BN == 64 && MT == 2 && EPI <= kEpiAddMask), "TMA-store epilogue: BN 64, MT 2, epilogues 0..3");
  constexpr uint32_t ACC_COLS = MT * BN;
  constexpr uint32_t TMEM_COLS = 2 * ACC_COLS;
  static_assert(TMEM_COLS >= 32 && TMEM_COLS <= 512 && (TMEM_COLS & (TMEM_COLS - 1)) == 0, "TMEM columns");
  static_assert(B_BYTES % 1024 == 0, "weight slices keep the 1024-byte swizzle alignment");
  extern __shared__ uint8_t dsmem[];
  __shared__ __align__(8) uint64_t afull[AST], aempty[AST], bfull[BST], bempty[BST];
  __shared__ __align__(8) uint64_t tfull_bar[2], tempty_bar[2], done_bar;
  __shared__ uint32_t tmem_slot;

  const uint32_t bbase = (smem_u32(dsmem) + 1023u) & ~1023u;  // weight ring, then the halo ring
  const uint32_t abase = bbase + (uint32_t)(BST * S_BYTES);
  const uint32_t sbase = abase + (uint32_t)(AST * HP::kABytes);  // TST: 8 x 4 KB output blocks
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tiles_x = W / 8, tiles_y = (H + 16 * MT - 1) / (16 * MT), tiles_n = Cout / BN;
  const int n_tiles = N * tiles_y * tiles_x * tiles_n;
  const int kchunks = Cin / BK;
  auto coord = [&](int t, int& img, int& y0, int& x0, int& n0) {
    n0 = (t % tiles_n) * BN;
    int r = t / tiles_n;
    x0 = (r % tiles_x) * 8;
    r /= tiles_x;
    y0 = (r % tiles_y) * (16 * MT);
    img = r / tiles_y;
  };

  if (threadIdx.x == 0) {
    for (int s = 0; s < AST; ++s) {
      mbar_init(smem_u32(&afull[s]), 1);
      mbar_init(smem_u32(&aempty[s]), 1);
    }
    for (int s = 0; s < BST; ++s) {
      mbar_init(smem_u32(&bfull[s]), 1);
      mbar_init(smem_u32(&bempty[s]), 1);
    }
    for (int a = 0; a < 2; ++a) {
      mbar_init(smem_u32(&tfull_bar[a]), 1);
      mbar_init(smem_u32(&tempty_bar[a]), kEpiWarps);
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
      int qa = 0, qb = 0;
      bool bad = false;
      for (int t = blockIdx.x; t < n_tiles && !bad; t += gridDim.x) {
        int img, y0, x0, n0;
        coord(t, img, y0, x0, n0);
        for (int cc = 0; cc < kchunks && !bad; ++cc) {
          const int sa = qa % AST;
          if (qa >= AST && !mbar_wait(smem_u32(&aempty[sa]), ((uint32_t)(qa / AST) & 1u) ^ 1u, err, kErrTma)) {
            bad = true;
            break;
          }
          const uint32_t fa = smem_u32(&afull[sa]);
          mbar_expect_tx(fa, (uint32_t)(HP::kRows * HP::kCols * 128));
          tma_4d(abase + (uint32_t)(sa * HP::kABytes), &tmap_x, cc * BK, x0 - 1, y0 - 1, img, fa);
          ++qa;
          for (int grp = 0; grp < GROUPS && (!RESB || qb == 0); ++grp) {
            const int sb = qb % BST;
            if (qb >= BST && !mbar_wait(smem_u32(&bempty[sb]), ((uint32_t)(qb / BST) & 1u) ^ 1u, err, kErrTma)) {
              bad = true;
              break;
            }
            const uint32_t fb = smem_u32(&bfull[sb]);
            mbar_expect_tx(fb, (uint32_t)S_BYTES);
            for (int u = 0; u < TPS; ++u)
              tma_2d(bbase + (uint32_t)(sb * S_BYTES + u * B_BYTES), &tmap_w, (grp * TPS + u) * Cin + cc * BK, n0, fb);
            ++qb;
          }
        }
      }
      if (bad) {
        // aborted: no load may still be writing shared memory when the CTA exits
        for (int i = qa > AST ? qa - AST : 0; i < qa; ++i) {
          uint32_t it = 0;
          while (!mbar_try(smem_u32(&afull[i % AST]), (uint32_t)(i / AST) & 1u) && ++it < kSpin) {
          }
        }
        for (int i = qb > BST ? qb - BST : 0; i < qb; ++i) {
          uint32_t it = 0;
          while (!mbar_try(smem_u32(&bfull[i % BST]), (uint32_t)(i / BST) & 1u) && ++it < kSpin) {
          }
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---------------------------------------------------------------- MMA issuer
      constexpr uint32_t idesc = idesc_bf16(BM, BN);
      int qa = 0, qb = 0, j = 0;
      bool bad = false;
      for (int t = blockIdx.x; t < n_tiles && !bad; t += gridDim.x, ++j) {
        const int a = j & 1;
        if (j >= 2 && !mbar_wait(smem_u32(&tempty_bar[a]), ((uint32_t)(j >> 1) & 1u) ^ 1u, err, kErrMma)) break;
        fence_after();
        const uint32_t acc = tmem + (uint32_t)a * ACC_COLS;
        for (int cc = 0; cc < kchunks && !bad; ++cc) {
          const int sa = qa % AST;
          if (!mbar_wait(smem_u32(&afull[sa]), (uint32_t)(qa / AST) & 1u, err, kErrMma)) {
            bad = true;
            break;
          }
          const uint32_t achunk = abase + (uint32_t)(sa * HP::kABytes);
          for (int grp = 0; grp < GROUPS; ++grp) {
            const int sb = qb % BST;
            if ((!RESB || qb == 0) && !mbar_wait(smem_u32(&bfull[sb]), (uint32_t)(qb / BST) & 1u, err, kErrMma)) {
              bad = true;
              break;
            }
            fence_after();
#pragma unroll
            for (int u = 0; u < TPS; ++u) {
              const int tap = grp * TPS + u;
              const uint32_t atap = achunk + (uint32_t)(((tap / 3) * HP::kCols + tap % 3) * 128);
              const uint32_t bs = bbase + (uint32_t)(sb * S_BYTES + u * B_BYTES);
#pragma unroll
              for (int k = 0; k < BK / 16; ++k) {  // 16 channels (32 bytes) per MMA
#pragma unroll
                for (int mt = 0; mt < MT; ++mt)
                  mma_bf16(acc + (uint32_t)(mt * BN),
                           sw128_desc_sbo(atap + (uint32_t)(mt * 16 * HP::kCols * 128 + 32 * k),
                                          (uint32_t)(HP::kCols * 128)),
                           sw128_desc(bs + 32u * k), idesc, (cc > 0 || tap > 0 || k > 0) ? 1u : 0u);
              }
            }
            if (!RESB) {
              mma_commit(smem_u32(&bempty[sb]));
              ++qb;
            } else {
              qb = 1;
            }
          }
          if (bad) break;
          mma_commit(smem_u32(&aempty[sa]));
          ++qa;
        }
        if (!bad) mma_commit(smem_u32(&tfull_bar[a]));
      }
      mma_commit(smem_u32(&done_bar));  // also on abort, so TMEM is idle before it is freed
    }
  } else {
    // ---------------------------------------------------------------- epilogue (warps 2..9)
    // Each thread owns accumulator row m (one output pixel) and drains NCH 32-column chunks: of
    // every M-tile, its half of the columns; or, where BN = 64 and MT = 2, all 64 columns of
    // M-tile `half`, so that each thread moves its pixel's whole 128-byte row. The mask / addend
    // values of the first PF chunks depend only on the tile's coordinates, so they are loaded
    // before the wait for the accumulator.
    constexpr bool BYTILE = BN == 64 && MT == 2;
    constexpr int CPH = BYTILE ? 2 : (BN >= 64 ? BN / 64 : 1);  // 32-column chunks per M-tile drained
    constexpr int NCH = BN >= 64 ? (BYTILE ? 1 : MT) * CPH : 0;  // BN = 16 (the render epilogues) drains below
    constexpr int PF = EPI == kEpiMask ? (NCH < 4 ? NCH : 4) : EPI == kEpiAddMask ? (NCH < 2 ? NCH : 2) : 0;
    const int qw = warp & 3;        // the TMEM lane quadrant this warp may read
    const int half = (warp - 2) >> 2;  // which half of the columns (or which M-tile) it drains
    const int m = qw * 32 + lane;  // accumulator row: patch row m / 8, column m % 8
    const int mt0 = BYTILE ? half : 0, cbase = BYTILE ? 0 : half * (BN / 2);
    int j = 0;
    for (int t = blockIdx.x; t < n_tiles; t += gridDim.x, ++j) {
      const int a = j & 1;
      int img, y0, x0, n0;
      coord(t, img, y0, x0, n0);
      uint4 pm[PF > 0 ? PF : 1][4], pa[PF > 0 ? PF : 1][4];
#pragma unroll
      for (int q = 0; q < PF; ++q) {
        const int mt = mt0 + q / CPH, c0 = cbase + (q % CPH) * 32;
        const int py = y0 + 16 * mt + m / 8, px = x0 + m % 8;
#pragma unroll
        for (int u = 0; u < 4; ++u) pm[q][u] = pa[q][u] = make_uint4(0u, 0u, 0u, 0u);
        if (py < H) epilogue_load32<EPI>(mask, addend, (((size_t)img * H + py) * W + px) * Cout + n0 + c0, pm[q], pa[q]);
      }
      const bool ok = __all_sync(0xffffffffu, mbar_wait(smem_u32(&tfull_bar[a]), (uint32_t)(j >> 1) & 1u, err,
                                                        kErrEpi)) &&
                      *(volatile int*)err == 0;
      fence_after();
      if (!ok) break;
      if (TST && j > 0) {  // the previous tile's store has read this warp's block
        if (lane == 0) bulk_wait_read0();
        __syncwarp();
      }
#pragma unroll
      for (int q = 0; q < NCH; ++q) {
        const int mt = mt0 + q / CPH, c0 = cbase + (q % CPH) * 32;
        const int py = y0 + 16 * mt + m / 8, px = x0 + m % 8;
        const size_t off = (((size_t)img * H + py) * W + px) * Cout + n0 + c0;
        uint32_t r[32];
        tmem_ld32(tmem + ((uint32_t)(qw * 32) << 16) + (uint32_t)(a * ACC_COLS + mt * BN + c0), r);
        if (TST) {
          // row `lane` of this warp's block, 16-byte chunk c0 / 8 + u at its swizzled position
          uint4 pk[4], mv[4], av[4];
          if (q < PF) {
            epilogue_values32<EPI>(r, bias, pm[q < PF ? q : 0], pa[q < PF ? q : 0], n0 + c0, pk);
          } else {
#pragma unroll
            for (int u = 0; u < 4; ++u) mv[u] = av[u] = make_uint4(0u, 0u, 0u, 0u);
            if (py < H) epilogue_load32<EPI>(mask, addend, off, mv, av);
            epilogue_values32<EPI>(r, bias, mv, av, n0 + c0, pk);
          }
          const uint32_t row = sbase + (uint32_t)((warp - 2) * 4096 + lane * 128);
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const uint32_t a16 = row + (uint32_t)((((c0 >> 3) + u) ^ (lane & 7)) * 16);
            asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(a16), "r"(pk[u].x), "r"(pk[u].y),
                         "r"(pk[u].z), "r"(pk[u].w)
                         : "memory");
          }
        } else if (EPI == kEpiUnpoolMax || EPI == kEpiUnpoolAvg) {
          if (py < H) {
            const size_t rs = (size_t)2 * W * Cout;
            const size_t base = ((size_t)img * 2 * H + 2 * py) * rs + (size_t)2 * px * Cout + n0 + c0;
            epilogue_unpool32<EPI == kEpiUnpoolAvg>(r, mask, addend, y, base, rs, Cout);
          }
        } else if (py < H) {
          if (q < PF) {
            epilogue_apply32<EPI>(r, bias, pm[q < PF ? q : 0], pa[q < PF ? q : 0], y, off, n0 + c0);
          } else {
            uint4 mv[4], av[4];
            epilogue_load32<EPI>(mask, addend, off, mv, av);
            epilogue_apply32<EPI>(r, bias, mv, av, y, off, n0 + c0);
          }
        }
      }
      if (TST) {  // the warp's 4 patch rows x 8 pixels x 64 channels, one tensor store
        fence_async_smem();
        __syncwarp();
        if (lane == 0) {
          tma_store_4d(&tmap_y, sbase + (uint32_t)((warp - 2) * 4096), n0, x0, y0 + 16 * mt0 + 4 * qw, img);
          bulk_commit();
        }
      }
      if ((EPI == kEpiRenderDown || EPI == kEpiRender) && half == 0) {
        float* dr = reinterpret_cast<float*>(y);
        const int px = x0 + m % 8;
#pragma unroll
        for (int mt = 0; mt < MT; ++mt) {
          const int py = y0 + 16 * mt + m / 8;
          uint32_t r[4];
          tmem_ld4(tmem + ((uint32_t)(qw * 32) << 16) + (uint32_t)(a * ACC_COLS + mt * BN), r);
          if (py < H) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              const float val = __uint_as_float(r[c]) * __ldg(bias + c);
              if (EPI == kEpiRenderDown) {
                float* row = dr + (((size_t)img * 3 + c) * 2 * H + 2 * py) * (size_t)(2 * W) + 2 * px;
                *reinterpret_cast<float2*>(row) = make_float2(val, val);
                *reinterpret_cast<float2*>(row + 2 * W) = make_float2(val, val);
              } else {
                dr[(((size_t)img * 3 + c) * H + py) * (size_t)W + px] = val;
              }
            }
          }
        }
      }
      fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_u32(&tempty_bar[a]));
    }
    if (TST && lane == 0) bulk_wait0();  // the stores have finished with shared memory
  }
  fence_before();
  __syncthreads();
  if (warp == 1) {
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

constexpr size_t kStageBudget = 216 * 1024;  // ring bytes per CTA (one CTA per SM)

// Taps per weight stage: a kernel row where the MMAs are narrow (BN <= 128), else one tap.
template <int BN>
constexpr int halo_tps() {
  return BN <= 128 ? 3 : 1;
}
constexpr size_t kStagingBytes = (size_t)kEpiWarps * 4096;  // TST: one 4 KB output block per epilogue warp
// Weight-ring depth: as many stages as fit beside two input slots (and the TST output blocks),
// up to 16 taps in flight.
template <int BN, int MT, bool TST>
constexpr int halo_bstages() {
  constexpr size_t stage = (size_t)halo_tps<BN>() * BN * BK * 2;
  constexpr int fit = (int)((kStageBudget - 2 * (size_t)Halo<MT>::kABytes - (TST ? kStagingBytes : 0)) / stage);
  constexpr int cap = 16 / halo_tps<BN>();
  return fit < cap ? fit : cap;
}

template <int BN, int MT, int EPI, bool RESB, bool TST>
static int launch_variant(const CUtensorMap& mx, const CUtensorMap& mw, const CUtensorMap& my, const float* bias,
                          const void* mask, const void* addend, void* y, int n, int h, int w, int cin, int cout,
                          int* err, cudaStream_t st) {
  constexpr int TPS = RESB ? 9 : halo_tps<BN>();
  constexpr int BST = RESB ? 1 : halo_bstages<BN, MT, TST>();
  static_assert(RESB || (BST >= 2 && BST * TPS >= 5), "weight ring too shallow");
  auto kern = conv3x3_halo_kernel<BN, MT, 2, BST, EPI, TPS, RESB, TST>;
  const size_t smem = (size_t)BST * TPS * BN * BK * 2 + 2 * (size_t)Halo<MT>::kABytes + (TST ? kStagingBytes : 0) +
                      1024;
  static_assert((size_t)BST * TPS * BN * BK * 2 + 2 * (size_t)Halo<MT>::kABytes + (TST ? kStagingBytes : 0) + 1024 <=
                    227 * 1024,
                "shared memory");
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
  const long long tiles = (long long)n * ((h + 16 * MT - 1) / (16 * MT)) * (w / 8) * (cout / BN);
  if (tiles >= (1LL << 31)) return fail(SVBRDF_ERR_UNSUPPORTED, "conv3x3: too many tiles");
  const int grid = (int)(tiles < sms[dev].load() ? tiles : sms[dev].load());
  kern<<<grid, kThreads, smem, st>>>(mx, mw, my, bias, (const __nv_bfloat16*)mask, (const __nv_bfloat16*)addend,
                                     (__nv_bfloat16*)y, n, h, w, cin, cout, err);
  return check_launch("conv3x3_halo_kernel");
}

// `my`: the output's tensor map for the TMA-store epilogue (BN = 64, MT = 2, epilogues 0..3), or
// null; weights stay resident where the layer is one 64-channel chunk and one Cout block.
template <int BN, int MT, int EPI>
static int launch_halo(const CUtensorMap& mx, const CUtensorMap& mw, const CUtensorMap* my, const float* bias,
                       const void* mask, const void* addend, void* y, int n, int h, int w, int cin, int cout, int* err,
                       cudaStream_t st) {
  if constexpr (BN == 64 && MT == 2 && EPI <= kEpiAddMask) {
    if (my) {
      if (cin == BK && cout == BN)
        return launch_variant<BN, MT, EPI, true, true>(mx, mw, *my, bias, mask, addend, y, n, h, w, cin, cout, err, st);
      return launch_variant<BN, MT, EPI, false, true>(mx, mw, *my, bias, mask, addend, y, n, h, w, cin, cout, err, st);
    }
  }
  return launch_variant<BN, MT, EPI, false, false>(mx, mw, mx, bias, mask, addend, y, n, h, w, cin, cout, err, st);
}

template <int BN, int MT>
static int dispatch_halo(int epi, const CUtensorMap& mx, const CUtensorMap& mw, const CUtensorMap* my,
                         const float* bias, const void* mask, const void* addend, void* y, int n, int h, int w, int cin,
                         int cout, int* err, cudaStream_t st) {
  switch (epi) {
    case kEpiNone: return launch_halo<BN, MT, kEpiNone>(mx, mw, my, bias, mask, addend, y, n, h, w, cin, cout, err, st);
    case kEpiBiasRelu:
      return launch_halo<BN, MT, kEpiBiasRelu>(mx, mw, my, bias, mask, addend, y, n, h, w, cin, cout, err, st);
    case kEpiMask: return launch_halo<BN, MT, kEpiMask>(mx, mw, my, bias, mask, addend, y, n, h, w, cin, cout, err, st);
    case kEpiAddMask:
      return launch_halo<BN, MT, kEpiAddMask>(mx, mw, my, bias, mask, addend, y, n, h, w, cin, cout, err, st);
    case kEpiUnpoolMax:
      return launch_halo<BN, MT, kEpiUnpoolMax>(mx, mw, my, bias, mask, addend, y, n, h, w, cin, cout, err, st);
    default: return launch_halo<BN, MT, kEpiUnpoolAvg>(mx, mw, my, bias, mask, addend, y, n, h, w, cin, cout, err, st);
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
  if (epilogue < kEpiNone || epilogue > kEpiUnpoolAvg) return fail(SVBRDF_ERR_INVALID, "bad epilogue %d", epilogue);
  if (epilogue == kEpiBiasRelu && !bias) return fail(SVBRDF_ERR_INVALID, "bias+relu epilogue needs bias");
  if ((epilogue == kEpiMask || epilogue == kEpiAddMask || epilogue >= kEpiUnpoolMax) && !mask)
    return fail(SVBRDF_ERR_INVALID, "mask epilogue needs mask");
  if (epilogue == kEpiAddMask && !addend) return fail(SVBRDF_ERR_INVALID, "add+mask epilogue needs addend");
  if (((uintptr_t)x | (uintptr_t)weight | (uintptr_t)y | (uintptr_t)mask | (uintptr_t)addend) % 16)
    return fail(SVBRDF_ERR_INVALID, "conv3x3: tensors must be 16-byte aligned");
  if ((long long)n * h * w * cin >= (1LL << 40)) return fail(SVBRDF_ERR_UNSUPPORTED, "conv3x3: tensor too large");
  PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
  int rc = get_tensor_map_encoder(&g_encode);
  if (rc) return rc;
  // BN = 256 (one M-tile) only on maps under 32 rows: elsewhere BN = 128 with two M-tiles has
  // the same MMA time per tap (N = 128 issues at 98 % of the N = 256 rate) and streams half the
  // weight bytes per output, which is what limits a 128 x 256 tile
  const int bn = (cout % 256 == 0 && h < 32) ? 256 : (cout % 128 == 0 ? 128 : 64);
  CUtensorMap mw;
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
  {
    // the (16 MT + 2) x 10 input patch of each 64-channel chunk, loaded once: one 128-byte
    // swizzled row per pixel; two stacked patches per tile where the map has 32+ rows and Cout
    // fits two double-buffered pairs of accumulators in TMEM
    const int mt = (bn <= 128 && h >= 32) ? 2 : 1;
    CUtensorMap mh;
    const cuuint64_t dims[4] = {(cuuint64_t)cin, (cuuint64_t)w, (cuuint64_t)h, (cuuint64_t)n};
    const cuuint64_t strides[3] = {(cuuint64_t)cin * 2, (cuuint64_t)w * cin * 2, (cuuint64_t)h * w * cin * 2};
    const cuuint32_t box[4] = {(cuuint32_t)BK, 10u, (cuuint32_t)(16 * mt + 2), 1u};
    const cuuint32_t es[4] = {1, 1, 1, 1};
    const CUresult r = g_encode(&mh, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(x), dims, strides, box, es,
                                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(SVBRDF_ERR_CUDA, "cuTensorMapEncodeTiled(halo x) failed: %d", (int)r);
    // the output as 64-channel x 8 x 4 boxes for the TMA-store epilogue (BN 64, MT 2)
    CUtensorMap my;
    const CUtensorMap* pmy = nullptr;
    if (bn == 64 && mt == 2 && epilogue <= kEpiAddMask) {
      const cuuint64_t ydims[4] = {(cuuint64_t)cout, (cuuint64_t)w, (cuuint64_t)h, (cuuint64_t)n};
      const cuuint64_t ystrides[3] = {(cuuint64_t)cout * 2, (cuuint64_t)w * cout * 2, (cuuint64_t)h * w * cout * 2};
      const cuuint32_t ybox[4] = {64u, 8u, 4u, 1u};
      const CUresult ry = g_encode(&my, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, y, ydims, ystrides, ybox, es,
                                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                   CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
      if (ry != CUDA_SUCCESS) return fail(SVBRDF_ERR_CUDA, "cuTensorMapEncodeTiled(y) failed: %d", (int)ry);
      pmy = &my;
    }
    switch (bn) {
      case 256: return dispatch_halo<256, 1>(epilogue, mh, mw, pmy, bias, mask, addend, y, n, h, w, cin, cout, err, st);
      case 128:
        return mt == 2 ? dispatch_halo<128, 2>(epilogue, mh, mw, pmy, bias, mask, addend, y, n, h, w, cin, cout, err, st)
                       : dispatch_halo<128, 1>(epilogue, mh, mw, pmy, bias, mask, addend, y, n, h, w, cin, cout, err, st);
      default:
        return mt == 2 ? dispatch_halo<64, 2>(epilogue, mh, mw, pmy, bias, mask, addend, y, n, h, w, cin, cout, err, st)
                       : dispatch_halo<64, 1>(epilogue, mh, mw, pmy, bias, mask, addend, y, n, h, w, cin, cout, err, st);
    }
  }
}

extern "C" int svbrdf_desc_conv1_bwd_tc(const void* gz, const void* w16, const float* scale, float* dr, int n, int h,
                                        int w, int down, int* err, void* stream) {
  using namespace svb::tc;
  if (!gz || !w16 || !scale || !dr || !err) return fail(SVBRDF_ERR_INVALID, "conv1_bwd_tc: null argument");
  if (n < 1 || n > 65535 || h < TH || w < TW || h % TH || w % TW)
    return fail(SVBRDF_ERR_UNSUPPORTED, "conv1_bwd_tc: H must be a multiple of %d and W of %d (got %dx%d)", TH, TW, h,
                w);
  if (((uintptr_t)gz | (uintptr_t)w16) % 16 || (uintptr_t)dr % 8)
    return fail(SVBRDF_ERR_INVALID, "conv1_bwd_tc: gz / w16 must be 16-byte aligned, dr 8-byte aligned");
  if ((long long)n * h * w * 64 >= (1LL << 40)) return fail(SVBRDF_ERR_UNSUPPORTED, "conv1_bwd_tc: tensor too large");
  PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
  int rc = get_tensor_map_encoder(&g_encode);
  if (rc) return rc;
  CUtensorMap mw, mh;
  {
    const cuuint64_t dims[2] = {(cuuint64_t)9 * 64, 16};
    const cuuint64_t strides[1] = {(cuuint64_t)9 * 64 * 2};
    const cuuint32_t box[2] = {(cuuint32_t)BK, 16u};
    const cuuint32_t es[2] = {1, 1};
    const CUresult r = g_encode(&mw, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(w16), dims, strides, box,
                                es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(SVBRDF_ERR_CUDA, "cuTensorMapEncodeTiled(w16) failed: %d", (int)r);
  }
  const int mt = h >= 32 ? 2 : 1;
  {
    const cuuint64_t dims[4] = {64, (cuuint64_t)w, (cuuint64_t)h, (cuuint64_t)n};
    const cuuint64_t strides[3] = {64 * 2, (cuuint64_t)w * 64 * 2, (cuuint64_t)h * w * 64 * 2};
    const cuuint32_t box[4] = {(cuuint32_t)BK, 10u, (cuuint32_t)(16 * mt + 2), 1u};
    const cuuint32_t es[4] = {1, 1, 1, 1};
    const CUresult r = g_encode(&mh, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(gz), dims, strides, box,
                                es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(SVBRDF_ERR_CUDA, "cuTensorMapEncodeTiled(gz) failed: %d", (int)r);
  }
  cudaStream_t st = (cudaStream_t)stream;
  void* y = dr;
  if (down)
    return mt == 2 ? launch_halo<16, 2, kEpiRenderDown>(mh, mw, nullptr, scale, nullptr, nullptr, y, n, h, w, 64, 16, err, st)
                   : launch_halo<16, 1, kEpiRenderDown>(mh, mw, nullptr, scale, nullptr, nullptr, y, n, h, w, 64, 16, err, st);
  return mt == 2 ? launch_halo<16, 2, kEpiRender>(mh, mw, nullptr, scale, nullptr, nullptr, y, n, h, w, 64, 16, err, st)
                 : launch_halo<16, 1, kEpiRender>(mh, mw, nullptr, scale, nullptr, nullptr, y, n, h, w, 64, 16, err, st);
}

extern "C" int svbrdf_conv3x3_bf16(const void* x, const void* weight, const float* bias, const void* mask, void* y,
                                   int n, int h, int w, int cin, int cout, int epilogue, int* err, void* stream) {
  if (epilogue == svb::tc::kEpiAddMask) return fail(SVBRDF_ERR_INVALID, "add+mask epilogue needs svbrdf_conv3x3_bf16_ex");
  return svbrdf_conv3x3_bf16_ex(x, weight, bias, mask, nullptr, y, n, h, w, cin, cout, epilogue, err, stream);
}
