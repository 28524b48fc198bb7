// TF32 convolutions of the MaterialGAN generator on the 5th-generation tensor cores.
//
// The reference's generator (src/higan_models/stylegan2_generator_network.py:585-759) runs its
// modulated 3x3 convolutions through PyTorch, whose cuDNN path computes them in TF32 by default
// (FP32 data, TF32 products, FP32 accumulation). Here the generator's maps stay FP32 and
// channels-last ([B][H][W][C]); the style modulation and demodulation are applied around a
// shared-weight convolution (input channels scaled by the style before it, output channels by
// the demodulation after it, in the elementwise kernels of gen_nhwc.cu), so each layer's
// convolution is one implicit GEMM:
//   M = 128 output pixels per M-tile: a TH x TW patch of NB images (16 x 8 of one image for
//       maps of 16 and more columns; 8 x 8 x 2 images and 4 x 4 x 8 images for the 8^2 and
//       4^2 maps); a CTA tile stacks MT = 2 M-tiles along y where Cout <= 128 and the map has
//       16+ rows, so each weight slice staged in shared memory feeds 256 pixels,
//   N = BN output channels, K = taps x Cin, consumed 32 channels (128 bytes of FP32) at a time.
// The kernel is persistent (one CTA per SM walking the tiles i, i + grid, ...). For each
// (tap, 32-channel chunk) the producer warp TMA-loads the MT shifted input patches (taps that
// fall outside the map read the TMA zero fill, which is the zero padding) and the BN x 32
// weight slice, 128-byte swizzled, into a ring of shared-memory stages that runs on across
// tiles; one thread issues tcgen05.mma kind::tf32 (K = 8 per instruction) into MT 128 x BN
// FP32 accumulators in TMEM, double-buffered, so four epilogue warps drain tile j (tcgen05.ld,
// FP32 NHWC stores) while the MMAs of tile j + 1 run.
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
  int TH, TW, NB;  // one M-tile: NB images x TH rows x TW columns = 128 output pixels
  int pad, taps;
  int tiles_x, tiles_y, tiles_b, tiles_n;  // CTA tiles along x, y (TH * MT rows), images, Cout / BN
  int splits, kper;  // K split into `splits` ranges of kper (tap, chunk) steps; 1 = no split
};

// One CTA tile: MT M-tiles stacked along y (MT * TH rows) x BN output channels.
struct TileCoord {
  int b0, y0, x0, n0;
};
template <int BN, int MT>
__device__ __forceinline__ TileCoord tile_coord(const Geom& g, int t) {
  TileCoord c;
  const int nb = t % g.tiles_n;
  int r = t / g.tiles_n;  // consecutive tiles share the input patch (one per Cout block)
  c.x0 = (r % g.tiles_x) * g.TW;
  r /= g.tiles_x;
  c.y0 = (r % g.tiles_y) * (g.TH * MT);
  c.b0 = (r / g.tiles_y) * g.NB;
  c.n0 = nb * BN;
  return c;
}

// Persistent: grid = min(tiles, SMs); CTA i runs tiles i, i + grid, ... The producer's ring
// runs across tile boundaries, and the accumulator is double-buffered in TMEM (2 x MT x BN
// columns), so the epilogue of tile j overlaps the MMAs of tile j + 1.
template <int BN, int MT, int STAGES>
__global__ void __launch_bounds__(kThreads, 1)
conv_tf32_kernel(const __grid_constant__ CUtensorMap tmap_x, const __grid_constant__ CUtensorMap tmap_w,
                 float* __restrict__ y, float* __restrict__ ws, Geom g, int* err) {
  constexpr int A_BYTES = BM * BK * 4;
  constexpr int B_BYTES = BN * BK * 4;
  constexpr int STAGE = MT * A_BYTES + B_BYTES;
  constexpr uint32_t ACC_COLS = MT * BN;          // one tile's accumulators
  constexpr uint32_t TMEM_COLS = 2 * ACC_COLS;    // double-buffered
  static_assert(TMEM_COLS >= 32 && TMEM_COLS <= 512 && (TMEM_COLS & (TMEM_COLS - 1)) == 0, "TMEM columns");
  extern __shared__ uint8_t dsmem[];
  __shared__ __align__(8) uint64_t full_bar[STAGES];
  __shared__ __align__(8) uint64_t empty_bar[STAGES];
  __shared__ __align__(8) uint64_t tfull_bar[2];   // accumulator buffer ready (MMA commit)
  __shared__ __align__(8) uint64_t tempty_bar[2];  // accumulator buffer drained (4 epilogue warps)
  __shared__ __align__(8) uint64_t done_bar;       // every MMA of this CTA complete
  __shared__ uint32_t tmem_slot;

  const uint32_t base = (smem_u32(dsmem) + 1023u) & ~1023u;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // work items: (tile, K range); with splits > 1 each writes an FP32 partial plane of ws
  const int n_items = g.tiles_b * g.tiles_y * g.tiles_x * g.tiles_n * g.splits;
  const int kchunks = g.Cin / BK;
  const int total = g.taps * kchunks;
  const int ks = g.taps == 9 ? 3 : 1;

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
      int q = 0;  // stages issued by this CTA
      bool bad = false;
      for (int w = blockIdx.x; w < n_items && !bad; w += gridDim.x) {
        const TileCoord c = tile_coord<BN, MT>(g, w / g.splits);
        const int k_lo = (w % g.splits) * g.kper, k_hi = min(total, k_lo + g.kper);
        for (int i = k_lo; i < k_hi; ++i) {
          const int s = q % STAGES;
          const uint32_t ph = (uint32_t)(q / STAGES) & 1u;
          if (q >= STAGES && !mbar_wait(smem_u32(&empty_bar[s]), ph ^ 1u, err, kErrTma)) {
            bad = true;
            break;
          }
          const int tap = i / kchunks, cc = i % kchunks;
          const int dy = tap / ks - g.pad, dx = tap % ks - g.pad;
          const uint32_t st = base + (uint32_t)(s * STAGE);
          const uint32_t fb = smem_u32(&full_bar[s]);
          mbar_expect_tx(fb, (uint32_t)STAGE);
#pragma unroll
          for (int mt = 0; mt < MT; ++mt)
            tma_4d(st + (uint32_t)(mt * A_BYTES), &tmap_x, cc * BK, c.x0 + dx, c.y0 + mt * g.TH + dy, c.b0, fb);
          tma_2d(st + (uint32_t)(MT * A_BYTES), &tmap_w, tap * g.Cin + cc * BK, c.n0, fb);
          ++q;
        }
      }
      if (bad) {  // let the copies in flight land before the CTA can exit
        for (int i = q > STAGES ? q - STAGES : 0; i < q; ++i) {
          uint32_t it = 0;
          while (!mbar_try(smem_u32(&full_bar[i % STAGES]), (uint32_t)(i / STAGES) & 1u) && ++it < kSpin) {
          }
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t id = idesc_tf32(BM, BN);
      int q = 0, j = 0;
      bool bad = false;
      for (int w = blockIdx.x; w < n_items && !bad; w += gridDim.x, ++j) {
        const int k_lo = (w % g.splits) * g.kper, k_hi = min(total, k_lo + g.kper);
        const int a = j & 1;
        // the epilogue must have drained this buffer's previous tile (j - 2)
        if (j >= 2 && !mbar_wait(smem_u32(&tempty_bar[a]), ((uint32_t)(j >> 1) & 1u) ^ 1u, err, kErrMma)) break;
        fence_after();
        const uint32_t acc = tmem + (uint32_t)a * ACC_COLS;
        for (int i = k_lo; i < k_hi; ++i, ++q) {
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
          for (int k = 0; k < BK / 8; ++k) {  // 8 TF32 channels = 32 bytes per MMA
#pragma unroll
            for (int mt = 0; mt < MT; ++mt)
              mma_tf32(acc + (uint32_t)(mt * BN), sw128_desc(sa + (uint32_t)(mt * A_BYTES) + 32u * k),
                       sw128_desc(sb + 32u * k), id, (i > k_lo || k > 0) ? 1u : 0u);
          }
          mma_commit(smem_u32(&empty_bar[s]));
        }
        if (!bad) mma_commit(smem_u32(&tfull_bar[a]));
      }
      mma_commit(smem_u32(&done_bar));  // also on abort, so TMEM is idle before it is freed
    }
  } else {
    const int qw = warp & 3;  // TMEM lanes 32 qw .. 32 qw + 31
    const int m = qw * 32 + lane;
    int j = 0;
    for (int w = blockIdx.x; w < n_items; w += gridDim.x, ++j) {
      const int a = j & 1;
      const bool ok = __all_sync(0xffffffffu, mbar_wait(smem_u32(&tfull_bar[a]), (uint32_t)(j >> 1) & 1u, err,
                                                        kErrEpi)) &&
                      *(volatile int*)err == 0;
      fence_after();
      if (!ok) break;
      const TileCoord c = tile_coord<BN, MT>(g, w / g.splits);
      float* dst = g.splits > 1 ? ws + (size_t)(w % g.splits) * ((size_t)g.B * g.Ho * g.Wo * g.Cout) : y;
      const int pb = c.b0 + m / (g.TH * g.TW);
      const int rem = m % (g.TH * g.TW);
      const int px = c.x0 + rem % g.TW;
#pragma unroll
      for (int mt = 0; mt < MT; ++mt) {
        const int py = c.y0 + mt * g.TH + rem / g.TW;
        const bool inside = pb < g.B && py < g.Ho && px < g.Wo;
        float* out = dst + (((size_t)pb * g.Ho + py) * g.Wo + px) * g.Cout + c.n0;
#pragma unroll 1
        for (int c0 = 0; c0 < BN; c0 += 32) {
          uint32_t r[32];
          tmem_ld32(tmem + ((uint32_t)(qw * 32) << 16) + (uint32_t)(a * ACC_COLS + mt * BN + c0), r);
          if (inside) {
            float4* o4 = reinterpret_cast<float4*>(out + c0);
#pragma unroll
            for (int u = 0; u < 8; ++u)
              o4[u] = make_float4(__uint_as_float(r[4 * u]), __uint_as_float(r[4 * u + 1]),
                                  __uint_as_float(r[4 * u + 2]), __uint_as_float(r[4 * u + 3]));
          }
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
    uint32_t it = 0;
    while (!mbar_try(smem_u32(&done_bar), 0u) && ++it < kSpin) {
    }
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
}

// ---------------------------------------------------------------- halo form
// Maps of 16+ rows and 8+ columns load each input patch once per 32-channel chunk, halo
// included, and share it between the taps. A tile is MT stacked 16-row x 8-column output
// patches of one image; its input is the (16 MT + KS - 1) x (8 + KS - 1) patch starting at
// (y0 - pad, x0 - pad), one TMA box of 128-byte pixel rows (32 TF32 channels), 128-byte
// swizzled, row-major from a 1024-byte boundary. Accumulator row r of M-tile mt is output pixel
// (16 mt + r / 8, r % 8), so tap (ky, kx) reads the patch's descriptor moved by ky kCols + kx
// pixels, with 8-row groups kCols pixels (kCols x 128 bytes) apart (SBO); the swizzle follows
// the address, so any pixel offset is a valid start. The taps' BN x 32 weight slices stream
// through their own ring (128-byte swizzle), TPS taps per stage: a whole kernel row where the
// MMAs are narrow (BN <= 128), as a group of MMAs between two commits costs at least about 560
// cycles. Per chunk a tile loads about 1.4 x MT x 16 KB of input instead of taps x MT x 16 KB.
// A work item is (tile, range of chunks); with splits > 1 its partial goes to plane `split` of ws.
template <int MT, int KS>
struct HaloT {
  static constexpr int kRows = 16 * MT + KS - 1, kCols = 8 + KS - 1;
  static constexpr int kABytes = ((kRows * kCols * 128 + 1023) / 1024) * 1024;  // 32 channels
};

constexpr int kHaloThreads = 320;  // warp 0 TMA, warp 1 MMA + TMEM owner, warps 2..9 epilogue (two per
                                   // TMEM lane quadrant, each draining half the columns)

template <int BN, int MT, int KS, int AST, int BST, int NBUF, int TPS>
__global__ void __launch_bounds__(kHaloThreads, 1)
conv_tf32_halo_kernel(const __grid_constant__ CUtensorMap tmap_x, const __grid_constant__ CUtensorMap tmap_w,
                      float* __restrict__ y, float* __restrict__ ws, Geom g, int* err) {
  using HP = HaloT<MT, KS>;
  constexpr int B_BYTES = BN * BK * 4;  // one tap's weight slice
  constexpr int TAPS = KS * KS;
  constexpr int S_BYTES = TPS * B_BYTES;  // one weight stage
  constexpr int GROUPS = TAPS / TPS;
  static_assert(TAPS % TPS == 0, "a weight stage holds whole taps of one chunk");
  constexpr uint32_t ACC_COLS = MT * BN;
  constexpr uint32_t TMEM_COLS = NBUF * ACC_COLS;  // NBUF = 2: double-buffered accumulators
  static_assert(TMEM_COLS >= 32 && TMEM_COLS <= 512 && (TMEM_COLS & (TMEM_COLS - 1)) == 0, "TMEM columns");
  static_assert(B_BYTES % 1024 == 0, "weight slices keep the 1024-byte swizzle alignment");
  extern __shared__ uint8_t dsmem[];
  __shared__ __align__(8) uint64_t afull[AST], aempty[AST], bfull[BST], bempty[BST];
  __shared__ __align__(8) uint64_t tfull_bar[2], tempty_bar[2], done_bar;
  __shared__ uint32_t tmem_slot;

  const uint32_t bbase = (smem_u32(dsmem) + 1023u) & ~1023u;
  const uint32_t abase = bbase + (uint32_t)(BST * S_BYTES);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n_items = g.tiles_b * g.tiles_y * g.tiles_x * g.tiles_n * g.splits;
  const int kchunks = g.Cin / BK;
  auto coord = [&](int t, int& img, int& y0, int& x0, int& n0) {
    n0 = (t % g.tiles_n) * BN;
    int r = t / g.tiles_n;
    x0 = (r % g.tiles_x) * 8;
    r /= g.tiles_x;
    y0 = (r % g.tiles_y) * (16 * MT);
    img = r / g.tiles_y;
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
      mbar_init(smem_u32(&tempty_bar[a]), 8);
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
      int qa = 0, qb = 0;
      bool bad = false;
      for (int w = blockIdx.x; w < n_items && !bad; w += gridDim.x) {
        int img, y0, x0, n0;
        coord(w / g.splits, img, y0, x0, n0);
        const int c_lo = (w % g.splits) * g.kper, c_hi = min(kchunks, c_lo + g.kper);
        for (int cc = c_lo; cc < c_hi && !bad; ++cc) {
          const int sa = qa % AST;
          if (qa >= AST && !mbar_wait(smem_u32(&aempty[sa]), ((uint32_t)(qa / AST) & 1u) ^ 1u, err, kErrTma)) {
            bad = true;
            break;
          }
          const uint32_t fa = smem_u32(&afull[sa]);
          mbar_expect_tx(fa, (uint32_t)(HP::kRows * HP::kCols * 128));
          tma_4d(abase + (uint32_t)(sa * HP::kABytes), &tmap_x, cc * BK, x0 - g.pad, y0 - g.pad, img, fa);
          ++qa;
          for (int grp = 0; grp < GROUPS; ++grp) {
            const int sb = qb % BST;
            if (qb >= BST && !mbar_wait(smem_u32(&bempty[sb]), ((uint32_t)(qb / BST) & 1u) ^ 1u, err, kErrTma)) {
              bad = true;
              break;
            }
            const uint32_t fb = smem_u32(&bfull[sb]);
            mbar_expect_tx(fb, (uint32_t)S_BYTES);
            for (int u = 0; u < TPS; ++u)
              tma_2d(bbase + (uint32_t)(sb * S_BYTES + u * B_BYTES), &tmap_w, (grp * TPS + u) * g.Cin + cc * BK, n0,
                     fb);
            ++qb;
          }
        }
      }
      if (bad) {  // let the copies in flight land before the CTA can exit
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
      constexpr uint32_t id = idesc_tf32(BM, BN);
      int qa = 0, qb = 0, j = 0;
      bool bad = false;
      for (int w = blockIdx.x; w < n_items && !bad; w += gridDim.x, ++j) {
        const int a = j % NBUF;
        // the epilogue must have drained this buffer's previous tile (j - NBUF)
        if (j >= NBUF && !mbar_wait(smem_u32(&tempty_bar[a]), ((uint32_t)(j / NBUF) & 1u) ^ 1u, err, kErrMma)) break;
        fence_after();
        const uint32_t acc = tmem + (uint32_t)a * ACC_COLS;
        const int c_lo = (w % g.splits) * g.kper, c_hi = min(kchunks, c_lo + g.kper);
        for (int cc = c_lo; cc < c_hi && !bad; ++cc) {
          const int sa = qa % AST;
          if (!mbar_wait(smem_u32(&afull[sa]), (uint32_t)(qa / AST) & 1u, err, kErrMma)) {
            bad = true;
            break;
          }
          const uint32_t achunk = abase + (uint32_t)(sa * HP::kABytes);
          for (int grp = 0; grp < GROUPS; ++grp) {
            const int sb = qb % BST;
            if (!mbar_wait(smem_u32(&bfull[sb]), (uint32_t)(qb / BST) & 1u, err, kErrMma)) {
              bad = true;
              break;
            }
            fence_after();
#pragma unroll
            for (int u = 0; u < TPS; ++u) {
              const int tap = grp * TPS + u;
              const uint32_t atap = achunk + (uint32_t)(((tap / KS) * HP::kCols + tap % KS) * 128);
              const uint32_t bs = bbase + (uint32_t)(sb * S_BYTES + u * B_BYTES);
#pragma unroll
              for (int k = 0; k < BK / 8; ++k) {  // 8 TF32 channels (32 bytes) per MMA
#pragma unroll
                for (int mt = 0; mt < MT; ++mt)
                  mma_tf32(acc + (uint32_t)(mt * BN),
                           sw128_desc_sbo(atap + (uint32_t)(mt * 16 * HP::kCols * 128 + 32 * k),
                                          (uint32_t)(HP::kCols * 128)),
                           sw128_desc(bs + 32u * k), id, (cc > c_lo || tap > 0 || k > 0) ? 1u : 0u);
              }
            }
            mma_commit(smem_u32(&bempty[sb]));
            ++qb;
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
    const int qw = warp & 3;        // the TMEM lane quadrant this warp may read
    const int half = (warp - 2) >> 2;  // which half of the columns it drains (BN = 32: half 0 only)
    constexpr int HCOLS = BN >= 64 ? BN / 2 : BN;
    const int m = qw * 32 + lane;  // accumulator row: patch row m / 8, column m % 8
    int j = 0;
    for (int w = blockIdx.x; w < n_items; w += gridDim.x, ++j) {
      const int a = j % NBUF;
      const bool ok = __all_sync(0xffffffffu, mbar_wait(smem_u32(&tfull_bar[a]), (uint32_t)(j / NBUF) & 1u, err,
                                                        kErrEpi)) &&
                      *(volatile int*)err == 0;
      fence_after();
      if (!ok) break;
      int img, y0, x0, n0;
      coord(w / g.splits, img, y0, x0, n0);
      float* dst = g.splits > 1 ? ws + (size_t)(w % g.splits) * ((size_t)g.B * g.Ho * g.Wo * g.Cout) : y;
      const int px = x0 + m % 8;
#pragma unroll
      for (int mt = 0; mt < MT; ++mt) {
        const int py = y0 + 16 * mt + m / 8;
        const bool inside = py < g.Ho && px < g.Wo;
        float* out = dst + (((size_t)img * g.Ho + py) * g.Wo + px) * g.Cout + n0;
#pragma unroll 1
        for (int c0 = half * HCOLS; c0 < BN && c0 < (half + 1) * HCOLS; c0 += 32) {
          uint32_t r[32];
          tmem_ld32(tmem + ((uint32_t)(qw * 32) << 16) + (uint32_t)(a * ACC_COLS + mt * BN + c0), r);
          if (inside) {
            float4* o4 = reinterpret_cast<float4*>(out + c0);
#pragma unroll
            for (int u = 0; u < 8; ++u)
              o4[u] = make_float4(__uint_as_float(r[4 * u]), __uint_as_float(r[4 * u + 1]),
                                  __uint_as_float(r[4 * u + 2]), __uint_as_float(r[4 * u + 3]));
          }
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
    uint32_t it = 0;
    while (!mbar_try(smem_u32(&done_bar), 0u) && ++it < kSpin) {
    }
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
}

constexpr size_t kStageBudget = 200 * 1024;  // ring bytes per CTA (one CTA per SM)

template <int BN, int MT>
constexpr int stages_for() {
  return (int)(kStageBudget / (size_t)(MT * BM * BK * 4 + BN * BK * 4)) < 8
             ? (int)(kStageBudget / (size_t)(MT * BM * BK * 4 + BN * BK * 4))
             : 8;
}

// K-split partial planes summed in split order: y[i] = sum_s ws[s][i] (float4 over i).
__global__ void __launch_bounds__(256) conv_tf32_split_sum_kernel(const float4* __restrict__ ws, float4* __restrict__ y,
                                                                   long long n4, int splits) {
  for (long long i = blockIdx.x * 256LL + threadIdx.x; i < n4; i += (long long)gridDim.x * 256) {
    float4 a = __ldg(ws + i);
    for (int s = 1; s < splits; ++s) {
      const float4 b = __ldg(ws + (long long)s * n4 + i);
      a.x += b.x;
      a.y += b.y;
      a.z += b.z;
      a.w += b.w;
    }
    y[i] = a;
  }
}

static int sm_count(int* out) {
  static std::atomic<int> sms[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return fail(SVBRDF_ERR_CUDA, "no usable device");
  if (sms[dev].load() == 0) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1)
      return fail(SVBRDF_ERR_CUDA, "no SM count");
    sms[dev].store(n);
  }
  *out = sms[dev].load();
  return SVBRDF_OK;
}

// The convolution's shape, patch, CTA tiling and K split. Maps with fewer CTA tiles than half
// the SMs split K (taps x channel chunks, at least 4 steps a split) so that about one CTA per
// SM has work; the splits then need a workspace of splits x B x Ho x Wo x Cout floats.
struct Plan {
  Geom g;
  int bn, mt;
  int halo, ks;  // the halo form (maps of 16+ rows, 8+ columns) and the kernel size
};
static int plan_conv(int b, int hin, int win, int cin, int cout, int ksize, int pad, int sms, Plan* pl) {
  if (ksize != 1 && ksize != 3) return fail(SVBRDF_ERR_INVALID, "conv_tf32: ksize must be 1 or 3");
  if (pad < 0 || pad > (ksize == 3 ? 2 : 0)) return fail(SVBRDF_ERR_INVALID, "conv_tf32: bad pad %d", pad);
  if (b < 1 || hin < 1 || win < 1 || cin < BK || cin % BK || cin > 8192)
    return fail(SVBRDF_ERR_UNSUPPORTED, "conv_tf32: Cin must be a multiple of %d (got %d)", BK, cin);
  if (cout < 32 || !(cout % 256 == 0 || cout == 128 || cout == 64 || cout == 32))
    return fail(SVBRDF_ERR_UNSUPPORTED, "conv_tf32: Cout must be 32, 64, 128 or a multiple of 256 (got %d)", cout);
  Geom& g = pl->g;
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
  pl->bn = cout >= 256 ? 256 : cout;
  pl->ks = ksize;
  pl->halo = (g.Wo >= 8 && g.Ho >= 16) ? 1 : 0;
  if (pl->halo) {
    // 16-row x 8-column patches, two stacked where the map has 32+ rows and Cout fits two
    // double-buffered accumulators in TMEM (BN <= 128; a 256 x 256 tile would fill TMEM with
    // one accumulator, and the exposed epilogue then costs more than the halved weight
    // traffic saves: measured 5-35 % slower on the generator's 32^2-128^2 layers). Wide
    // layers (Cout >= 256) on such maps take BN = 128 with two M-tiles rather than BN = 256
    // with one: the same MMA time per tap (an N = 128 MMA issues at 98 % of the N = 256 rate)
    // for half the weight bytes per output, which a 128 x 256 tile streams from L2 at about
    // 90 GB/s per SM, its limit. K splits count 32-channel chunks (all taps each).
    g.TW = 8; g.TH = 16; g.NB = 1;
    if (pl->bn == 256 && g.Ho >= 32) pl->bn = 128;
    pl->mt = (g.Ho >= 32 && pl->bn <= 128) ? 2 : 1;
    g.tiles_x = (g.Wo + 7) / 8;
    g.tiles_y = (g.Ho + 16 * pl->mt - 1) / (16 * pl->mt);
    g.tiles_b = g.B;
    g.tiles_n = g.Cout / pl->bn;
    const long long tiles = (long long)g.tiles_b * g.tiles_y * g.tiles_x * g.tiles_n;
    if (tiles >= (1LL << 30)) return fail(SVBRDF_ERR_UNSUPPORTED, "conv_tf32: too many tiles");
    const int chunks = cin / BK;
    int splits = 1;
    if (2 * tiles < sms) {
      splits = (int)(sms / tiles);
      if (splits > chunks / 2) splits = chunks / 2;
      if (splits < 1) splits = 1;
    }
    g.kper = (chunks + splits - 1) / splits;
    g.splits = (chunks + g.kper - 1) / g.kper;
    return SVBRDF_OK;
  }
  // two M-tiles per CTA tile (one weight slice feeds 256 output pixels) where the map has 16+
  // rows and Cout fits two double-buffered accumulators in TMEM
  pl->mt = (g.NB == 1 && g.Ho >= 16 && pl->bn <= 128) ? 2 : 1;
  g.tiles_x = (g.Wo + g.TW - 1) / g.TW;
  g.tiles_y = (g.Ho + g.TH * pl->mt - 1) / (g.TH * pl->mt);
  g.tiles_b = (g.B + g.NB - 1) / g.NB;
  g.tiles_n = g.Cout / pl->bn;
  const long long tiles = (long long)g.tiles_b * g.tiles_y * g.tiles_x * g.tiles_n;
  if (tiles >= (1LL << 30)) return fail(SVBRDF_ERR_UNSUPPORTED, "conv_tf32: too many tiles");
  const int total = g.taps * (cin / BK);
  int splits = 1;
  if (2 * tiles < sms) {
    splits = (int)(sms / tiles);
    if (splits > total / 4) splits = total / 4;
    if (splits < 1) splits = 1;
  }
  g.kper = (total + splits - 1) / splits;
  g.splits = (total + g.kper - 1) / g.kper;  // no empty split
  return SVBRDF_OK;
}

static long long split_ws_floats(const Geom& g) {
  return g.splits > 1 ? (long long)g.splits * g.B * g.Ho * g.Wo * g.Cout : 0;
}

template <int BN, int MT>
static int launch(const CUtensorMap& mx, const CUtensorMap& mw, float* y, float* ws, const Geom& g, int sms, int* err,
                  cudaStream_t st) {
  constexpr int STAGES = stages_for<BN, MT>();
  static_assert(STAGES >= 3, "ring too shallow");
  static std::atomic<size_t> have[64];
  const size_t smem = (size_t)STAGES * (MT * BM * BK * 4 + BN * BK * 4) + 1024;
  auto kern = conv_tf32_kernel<BN, MT, STAGES>;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return fail(SVBRDF_ERR_CUDA, "no usable device");
  if (have[dev].load() < smem) {
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
      return fail(SVBRDF_ERR_CUDA, "cudaFuncSetAttribute: %s", cudaGetErrorString(cudaGetLastError()));
    have[dev].store(smem);
  }
  const long long items = (long long)g.tiles_b * g.tiles_y * g.tiles_x * g.tiles_n * g.splits;
  const int grid = (int)(items < sms ? items : sms);
  kern<<<grid, kThreads, smem, st>>>(mx, mw, y, ws, g, err);
  int rc = check_launch("conv_tf32_kernel");
  if (rc || g.splits == 1) return rc;
  const long long n4 = (long long)g.B * g.Ho * g.Wo * g.Cout / 4;
  const long long blocks = (n4 + 255) / 256;
  conv_tf32_split_sum_kernel<<<(unsigned)(blocks < 4 * sms ? blocks : 4 * sms), 256, 0, st>>>(
      reinterpret_cast<const float4*>(ws), reinterpret_cast<float4*>(y), n4, g.splits);
  return check_launch("conv_tf32_split_sum_kernel");
}

// Taps per weight stage: a kernel row of a 3x3 convolution where the MMAs are narrow.
template <int BN, int KS>
constexpr int halo_tps() {
  return (KS == 3 && BN <= 128) ? 3 : 1;
}
// Weight-ring depth: as many stages as fit beside two input slots, up to 16 taps in flight.
template <int BN, int MT, int KS>
constexpr int halo_bstages() {
  constexpr size_t stage = (size_t)halo_tps<BN, KS>() * BN * BK * 4;
  constexpr int fit = (int)((kStageBudget - 2 * (size_t)HaloT<MT, KS>::kABytes) / stage);
  constexpr int cap = 16 / halo_tps<BN, KS>();
  return fit < cap ? fit : cap;
}

template <int BN, int MT, int KS>
static int launch_halo(const CUtensorMap& mx, const CUtensorMap& mw, float* y, float* ws, const Geom& g, int sms,
                       int* err, cudaStream_t st) {
  constexpr int TPS = halo_tps<BN, KS>();
  constexpr int BST = halo_bstages<BN, MT, KS>();
  static_assert(BST >= 2 && BST * TPS >= 4, "weight ring too shallow");
  // 512 TMEM columns hold two MT x BN accumulators up to MT x BN = 256, else one
  constexpr int NBUF = MT * BN <= 256 ? 2 : 1;
  static std::atomic<size_t> have[64];
  const size_t smem = (size_t)BST * TPS * BN * BK * 4 + 2 * (size_t)HaloT<MT, KS>::kABytes + 1024;
  auto kern = conv_tf32_halo_kernel<BN, MT, KS, 2, BST, NBUF, TPS>;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return fail(SVBRDF_ERR_CUDA, "no usable device");
  if (have[dev].load() < smem) {
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
      return fail(SVBRDF_ERR_CUDA, "cudaFuncSetAttribute: %s", cudaGetErrorString(cudaGetLastError()));
    have[dev].store(smem);
  }
  const long long items = (long long)g.tiles_b * g.tiles_y * g.tiles_x * g.tiles_n * g.splits;
  const int grid = (int)(items < sms ? items : sms);
  kern<<<grid, kHaloThreads, smem, st>>>(mx, mw, y, ws, g, err);
  int rc = check_launch("conv_tf32_halo_kernel");
  if (rc || g.splits == 1) return rc;
  const long long n4 = (long long)g.B * g.Ho * g.Wo * g.Cout / 4;
  const long long blocks = (n4 + 255) / 256;
  conv_tf32_split_sum_kernel<<<(unsigned)(blocks < 4 * sms ? blocks : 4 * sms), 256, 0, st>>>(
      reinterpret_cast<const float4*>(ws), reinterpret_cast<float4*>(y), n4, g.splits);
  return check_launch("conv_tf32_split_sum_kernel");
}

template <int KS>
static int dispatch_halo(int bn, int mt, const CUtensorMap& mx, const CUtensorMap& mw, float* y, float* ws,
                         const Geom& g, int sms, int* err, cudaStream_t st) {
  switch (bn) {
    case 256: return launch_halo<256, 1, KS>(mx, mw, y, ws, g, sms, err, st);
    case 128: return mt == 2 ? launch_halo<128, 2, KS>(mx, mw, y, ws, g, sms, err, st)
                             : launch_halo<128, 1, KS>(mx, mw, y, ws, g, sms, err, st);
    case 64: return mt == 2 ? launch_halo<64, 2, KS>(mx, mw, y, ws, g, sms, err, st)
                            : launch_halo<64, 1, KS>(mx, mw, y, ws, g, sms, err, st);
    default: return mt == 2 ? launch_halo<32, 2, KS>(mx, mw, y, ws, g, sms, err, st)
                            : launch_halo<32, 1, KS>(mx, mw, y, ws, g, sms, err, st);
  }
}

}  // namespace tf32
}  // namespace svb

using namespace svb;

extern "C" long long svbrdf_gen_conv_tf32_ws_bytes(int b, int hin, int win, int cin, int cout, int ksize, int pad) {
  using namespace svb::tf32;
  int sms = 0;
  tf32::Plan pl;
  if (sm_count(&sms) || plan_conv(b, hin, win, cin, cout, ksize, pad, sms, &pl)) return -1;
  return 4 * split_ws_floats(pl.g);
}

extern "C" int svbrdf_gen_conv_tf32_ex(const float* x, const float* weight, float* y, void* ws, long long ws_bytes,
                                       int b, int hin, int win, int cin, int cout, int ksize, int pad, int* err,
                                       void* stream) {
  using namespace svb::tf32;
  if (!x || !weight || !y || !err) return fail(SVBRDF_ERR_INVALID, "conv_tf32: null x/weight/y/err");
  int sms = 0;
  const int src = sm_count(&sms);
  tf32::Plan pl;
  int rc = plan_conv(b, hin, win, cin, cout, ksize, pad, src == SVBRDF_OK ? sms : 0, &pl);  // shape errors first
  if (rc) return rc;
  if (src) return src;
  Geom& g = pl.g;
  if (g.splits > 1 && (!ws || ws_bytes < 4 * split_ws_floats(g))) {  // no room: one K range per tile
    const int total = g.taps * (cin / BK);
    g.splits = 1;
    g.kper = total;
  }
  if (((uintptr_t)x | (uintptr_t)weight | (uintptr_t)y | (uintptr_t)(g.splits > 1 ? ws : nullptr)) % 16)
    return fail(SVBRDF_ERR_INVALID, "conv_tf32: 16-byte alignment");
  PFN_cuTensorMapEncodeTiled_v12000 enc = nullptr;
  rc = get_tensor_map_encoder(&enc);
  if (rc) return rc;
  const int bn = pl.bn;
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
  float* wsf = g.splits > 1 ? static_cast<float*>(ws) : nullptr;
  if (pl.halo) {
    // the (16 MT + k - 1) x (8 + k - 1) input patch of a 32-channel chunk, one 128-byte
    // swizzled row per pixel
    CUtensorMap mh;
    const int rows = 16 * pl.mt + ksize - 1, cols = 8 + ksize - 1;
    const cuuint64_t dims[4] = {(cuuint64_t)cin, (cuuint64_t)win, (cuuint64_t)hin, (cuuint64_t)b};
    const cuuint64_t strides[3] = {(cuuint64_t)cin * 4, (cuuint64_t)win * cin * 4, (cuuint64_t)hin * win * cin * 4};
    const cuuint32_t box[4] = {(cuuint32_t)BK, (cuuint32_t)cols, (cuuint32_t)rows, 1u};
    const cuuint32_t es[4] = {1, 1, 1, 1};
    const CUresult r = enc(&mh, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<float*>(x), dims, strides, box, es,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(SVBRDF_ERR_CUDA, "cuTensorMapEncodeTiled(halo x) failed: %d", (int)r);
    return ksize == 3 ? dispatch_halo<3>(bn, pl.mt, mh, mw, y, wsf, g, sms, err, st)
                      : dispatch_halo<1>(bn, pl.mt, mh, mw, y, wsf, g, sms, err, st);
  }
  const bool two = pl.mt == 2;
  switch (bn) {
    case 256: return launch<256, 1>(mx, mw, y, wsf, g, sms, err, st);
    case 128: return two ? launch<128, 2>(mx, mw, y, wsf, g, sms, err, st) : launch<128, 1>(mx, mw, y, wsf, g, sms, err, st);
    case 64: return two ? launch<64, 2>(mx, mw, y, wsf, g, sms, err, st) : launch<64, 1>(mx, mw, y, wsf, g, sms, err, st);
    default: return two ? launch<32, 2>(mx, mw, y, wsf, g, sms, err, st) : launch<32, 1>(mx, mw, y, wsf, g, sms, err, st);
  }
}

extern "C" int svbrdf_gen_conv_tf32(const float* x, const float* weight, float* y, int b, int hin, int win, int cin,
                                    int cout, int ksize, int pad, int* err, void* stream) {
  return svbrdf_gen_conv_tf32_ex(x, weight, y, nullptr, 0, b, hin, win, cin, cout, ksize, pad, err, stream);
}
