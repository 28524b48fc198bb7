// Gram products of the descriptor's Gram term on the 5th-generation tensor cores.
//
// The reference's Gram branch is G = F F^T / S of a [C, S] feature matrix
// (VGGLoss.compute_feature_vector, src/descriptor.py:50-56). Features here are NHWC BF16
// maps [V][S][C] (S pixels), so per view G = F^T F / S, and the loss gradient flows back as
// dF = F (dG + dG^T) / S. Three kernels:
//
//   gram_kernel        partial[v][split][i][j] = sum over one split of the pixels of
//                      F[p][i] F[p][j]. An implicit GEMM with M = 128 channels (i), N = BN
//                      channels (j), K = pixels: both operands are MN-major (channels are
//                      contiguous), loaded straight from the feature map as 64-channel x
//                      64-pixel boxes with 128-byte swizzle (a box past the last channel is
//                      the TMA zero fill, so C = 64 runs as M = 128 with half the rows zero).
//                      One thread issues tcgen05.mma (kind::f16, BF16 in, FP32 accumulate into
//                      TMEM); four epilogue warps read TMEM (tcgen05.ld) and store the partial.
//   gram_finish_kernel G = sum of the splits' partials in a fixed order / S, minus the target
//                      Gram; each row's squared difference summed in a fixed order (the loss),
//                      and coef (G - Gt) rounded to BF16 (the scaled, symmetric dG).
//   gemm_nt_kernel     out[b][m][n] = sum_k A[b][m][k] B[b][n][k] with both operands K-major
//                      (BF16, FP32 accumulate, FP32 out): dF = F dG for the backward pass.
//
// Every mbarrier wait is bounded: on timeout the kernel records an error code in `err`, stops
// issuing, drains its copies and MMAs (bounded), frees its TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <atomic>

#include "tc_ptx.cuh"

namespace svb {
namespace gram {

using namespace svb::tc;

constexpr int kThreads = 192;  // warp 0 TMA, warp 1 MMA + TMEM owner, warps 2..5 epilogue
constexpr int KP = 64;         // pixels per stage of the Gram product
constexpr int kAtom = 64 * 64 * 2;  // one 64-channel x 64-row BF16 box: 8 KB
enum GramError : int { kErrTma = 21, kErrMma = 22, kErrEpi = 23 };

// Instruction descriptor, kind::f16, BF16 x BF16 -> FP32; `mn_major` sets both operands MN-major.
__host__ __device__ constexpr uint32_t idesc(int m, int n, bool mn_major) {
  return idesc_bf16(m, n) | (mn_major ? ((1u << 15) | (1u << 16)) : 0u);
}

// Shared teardown: wait (bounded) for the final commit so no MMA writes TMEM after it is freed.
__device__ __forceinline__ void release_tmem(uint64_t* acc_bar, uint32_t tmem, uint32_t cols) {
  uint32_t it = 0;
  while (!mbar_try(smem_u32(acc_bar), 0u) && ++it < kSpin) {
  }
  fence_after();
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(cols) : "memory");
}

// Aborted producer: wait (bounded) for the loads of the last min(issued, stages) stages to land.
__device__ __forceinline__ void drain_loads(uint64_t* full_bar, int issued, int stages) {
  for (int i = issued > stages ? issued - stages : 0; i < issued; ++i) {
    uint32_t it = 0;
    while (!mbar_try(smem_u32(&full_bar[i % stages]), (uint32_t)(i / stages) & 1u) && ++it < kSpin) {
    }
  }
}

// grid (tiles_i * tiles_j, splits, V). Rows of the partial at or beyond C are not stored.
// Z64 (C = 64): a stage is the one 64-channel box, which is B and A's first atom; A's second
// atom (rows 64..127, never stored) is a zero atom written once per CTA, reached through A's
// leading byte offset. One 8 KB load per 64-pixel step instead of three.
template <int BN, int STAGES, bool Z64>
__global__ void __launch_bounds__(kThreads)
gram_kernel(const __grid_constant__ CUtensorMap tmap_f, float* __restrict__ partial, int S, int C, int splits,
            int pix_per_split, int* err) {
  static_assert(!Z64 || BN == 64, "Z64 is the 64-channel form");
  constexpr int A_BYTES = Z64 ? 0 : 2 * kAtom;  // M = 128 channels: two 64-channel atoms
  constexpr int B_BYTES = (BN / 64) * kAtom;
  constexpr int STAGE = A_BYTES + B_BYTES;
  extern __shared__ uint8_t dsmem[];
  __shared__ __align__(8) uint64_t full_bar[STAGES];
  __shared__ __align__(8) uint64_t empty_bar[STAGES];
  __shared__ __align__(8) uint64_t acc_bar;
  __shared__ uint32_t tmem_slot;

  const uint32_t base = (smem_u32(dsmem) + 1023u) & ~1023u;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tiles_j = C / BN;
  const int i0 = (blockIdx.x / tiles_j) * 128, j0 = (blockIdx.x % tiles_j) * BN;
  const int split = blockIdx.y, v = blockIdx.z;
  const int p0 = split * pix_per_split;
  const int p1 = min(S, p0 + pix_per_split);
  const int steps = p1 > p0 ? (p1 - p0) / KP : 0;
  const int row0 = v * S + p0;
  const uint32_t zbase = base + (uint32_t)(STAGES * STAGE);  // Z64: the zero atom
  if (Z64) {
    for (int i = threadIdx.x; i < kAtom / 16; i += blockDim.x)
      asm volatile("st.shared.v4.b32 [%0], {%1, %1, %1, %1};" ::"r"(zbase + 16u * i), "r"(0u) : "memory");
    fence_async_smem();  // the zeros are read by the MMAs (async proxy); the barrier below orders them
  }

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
      for (int i = 0; i < steps; ++i) {
        const int s = i % STAGES;
        const uint32_t ph = (uint32_t)(i / STAGES) & 1u;
        if (i >= STAGES && !mbar_wait(smem_u32(&empty_bar[s]), ph ^ 1u, err, kErrTma)) break;
        const uint32_t st = base + (uint32_t)(s * STAGE);
        const uint32_t fb = smem_u32(&full_bar[s]);
        const int row = row0 + i * KP;
        mbar_expect_tx(fb, (uint32_t)STAGE);
        if (!Z64) {
          tma_2d(st, &tmap_f, i0, row, fb);
          tma_2d(st + kAtom, &tmap_f, i0 + 64, row, fb);  // past C: zero fill
        }
#pragma unroll
        for (int b = 0; b < BN / 64; ++b) tma_2d(st + A_BYTES + b * kAtom, &tmap_f, j0 + 64 * b, row, fb);
        ++issued;
      }
      if (issued < steps) drain_loads(full_bar, issued, STAGES);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t id = idesc(128, BN, true);
      for (int i = 0; i < steps; ++i) {
        const int s = i % STAGES;
        const uint32_t ph = (uint32_t)(i / STAGES) & 1u;
        if (!mbar_wait(smem_u32(&full_bar[s]), ph, err, kErrMma)) break;
        fence_after();
        const uint32_t a = base + (uint32_t)(s * STAGE);
        const uint32_t b = a + A_BYTES;
        // Z64: A's atoms are the stage's box and the zero atom (zbase - a bytes on)
        const uint32_t a_lbo = Z64 ? zbase - a : (uint32_t)kAtom;
#pragma unroll
        for (int k = 0; k < KP / 16; ++k)  // 16 pixels = two 8-row groups per MMA
          mma_bf16(tmem, sw128_desc_mn(a + 2048u * k, a_lbo, 1024), sw128_desc_mn(b + 2048u * k, kAtom, 1024), id,
                   (i > 0 || k > 0) ? 1u : 0u);
        mma_commit(smem_u32(&empty_bar[s]));
      }
      mma_commit(smem_u32(&acc_bar));  // also on abort, so TMEM is idle before it is freed
    }
  } else {
    const int q = warp & 3;
    const int i = i0 + q * 32 + lane;
    const bool ok = __all_sync(0xffffffffu, mbar_wait(smem_u32(&acc_bar), 0u, err, kErrEpi)) &&
                    *(volatile int*)err == 0;
    fence_after();
    if (ok) {
      float* out = partial + (((size_t)v * splits + split) * C + i) * C + j0;
#pragma unroll 1
      for (int c0 = 0; c0 < BN; c0 += 32) {
        uint32_t r[32];
        tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c0, r);
        if (i < C) {
          float4* o4 = reinterpret_cast<float4*>(out + c0);
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const float4 val = steps > 0 ? make_float4(__uint_as_float(r[4 * u]), __uint_as_float(r[4 * u + 1]),
                                                       __uint_as_float(r[4 * u + 2]), __uint_as_float(r[4 * u + 3]))
                                         : make_float4(0.f, 0.f, 0.f, 0.f);
            o4[u] = val;
          }
        }
      }
    }
  }
  fence_before();
  __syncthreads();
  if (warp == 1) release_tmem(&acc_bar, tmem, (uint32_t)BN);
}

// grid (ceil(C / rows), V), 256 threads: `rows` = 256 / cw rows of view v per block, cw threads
// per row (cw = C rounded up to a power of two, 32 to 256). The splits' partials of an element
// are loaded up to eight at a time (all of them for the usual 2 to 8 splits) and added in split
// order.
__global__ void __launch_bounds__(256)
gram_finish_kernel(const float* __restrict__ partial, int splits, int C, int cw, float inv_s,
                   const float* __restrict__ gt, float coef, float* __restrict__ gram_out,
                   __nv_bfloat16* __restrict__ dgram, float* __restrict__ loss_part) {
  const int rows = 256 / cw, r = threadIdx.x / cw, j0 = threadIdx.x % cw;
  const int i = blockIdx.x * rows + r, v = blockIdx.y;
  __shared__ double red[8];
  float acc = 0.0f;  // this thread's squared differences (one to C / 256 of them)
  const size_t stride = (size_t)C * C;
  if (i < C) {
    for (int j = j0; j < C; j += cw) {
      const float* pp = partial + ((size_t)v * splits * C + i) * C + j;
      float g = 0.f;
      for (int sp = 0; sp < splits; sp += 8) {  // up to 8 loads in flight, summed in split order
        float q[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) q[u] = sp + u < splits ? __ldg(pp + (size_t)(sp + u) * stride) : 0.0f;
#pragma unroll
        for (int u = 0; u < 8; ++u)
          if (sp + u < splits) g += q[u];
      }
      g *= inv_s;
      const size_t o = ((size_t)v * C + i) * C + j;
      if (gram_out) gram_out[o] = g;
      const float d = gt ? g - __ldg(gt + o) : g;
      acc = fmaf(d, d, acc);
      if (dgram) dgram[o] = __float2bfloat16_rn(coef * d);
    }
  }
  // FP32 within a warp (a fixed xor tree), FP64 across the row's warps: FP64 arithmetic is
  // scarce on this part, and the row sum is stored as FP32
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = (double)acc;
  __syncthreads();
  if (j0 == 0 && i < C && loss_part) {  // the row's warps, in order
    double t = 0.0;
    for (int w = 0; w < cw / 32; ++w) t += red[r * (cw / 32) + w];
    loss_part[(size_t)v * C + i] = (float)t;
  }
}

// The feature term fused into the Gram gradient's epilogue (FUSE): per element of row r,
// channel n of the [batch * m, n] maps, d = f - t, g = coef d + (F dG)[r][n], times (f > 0)
// if `mask`, stored BF16; each epilogue warp's sum of d^2 goes to partial[cta * 4 + warp].
struct FeatEpi {
  const void* f;  // the hook's features, BF16 or FP32
  int f_bf16;
  const void* t;  // target features, BF16 or FP32
  int t_bf16;
  float coef;
  int mask;
  __nv_bfloat16* g;  // the loss gradient at the hook
  float* partial;
};

// out[b][m][n] = sum_k A[b][m][k] B[b][n][k]; grid (batch * m / 128, n / BN). A: rows
// b * m + r of a [batch * m, k] map; B: rows b * n + r of a [batch * n, k] map.
template <int BN, int STAGES, bool FUSE>
__global__ void __launch_bounds__(kThreads, 1)
gemm_nt_kernel(const __grid_constant__ CUtensorMap tmap_a, const __grid_constant__ CUtensorMap tmap_b,
               float* __restrict__ out, int M, int Nn, int K, int* err, FeatEpi fe) {
  constexpr int A_BYTES = 128 * 64 * 2;
  constexpr int B_BYTES = BN * 64 * 2;
  constexpr int STAGE = A_BYTES + B_BYTES;
  extern __shared__ uint8_t dsmem[];
  __shared__ __align__(8) uint64_t full_bar[STAGES];
  __shared__ __align__(8) uint64_t empty_bar[STAGES];
  __shared__ __align__(8) uint64_t acc_bar;
  __shared__ uint32_t tmem_slot;
  __shared__ __align__(16) float s_tr[FUSE ? 4 : 1][32][36];  // per epilogue warp: a 32 x 32 chunk, rows padded

  const uint32_t base = (smem_u32(dsmem) + 1023u) & ~1023u;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int mtiles = M / 128;
  const int b = blockIdx.x / mtiles, m0 = (blockIdx.x % mtiles) * 128;
  const int n0 = blockIdx.y * BN;
  const int steps = K / 64;

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
      for (int i = 0; i < steps; ++i) {
        const int s = i % STAGES;
        const uint32_t ph = (uint32_t)(i / STAGES) & 1u;
        if (i >= STAGES && !mbar_wait(smem_u32(&empty_bar[s]), ph ^ 1u, err, kErrTma)) break;
        const uint32_t st = base + (uint32_t)(s * STAGE);
        const uint32_t fb = smem_u32(&full_bar[s]);
        mbar_expect_tx(fb, (uint32_t)STAGE);
        tma_2d(st, &tmap_a, i * 64, b * M + m0, fb);
        tma_2d(st + A_BYTES, &tmap_b, i * 64, b * Nn + n0, fb);
        ++issued;
      }
      if (issued < steps) drain_loads(full_bar, issued, STAGES);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t id = idesc(128, BN, false);
      for (int i = 0; i < steps; ++i) {
        const int s = i % STAGES;
        const uint32_t ph = (uint32_t)(i / STAGES) & 1u;
        if (!mbar_wait(smem_u32(&full_bar[s]), ph, err, kErrMma)) break;
        fence_after();
        const uint32_t a = base + (uint32_t)(s * STAGE);
        const uint32_t bb = a + A_BYTES;
#pragma unroll
        for (int k = 0; k < 4; ++k)
          mma_bf16(tmem, sw128_desc(a + 32u * k), sw128_desc(bb + 32u * k), id, (i > 0 || k > 0) ? 1u : 0u);
        mma_commit(smem_u32(&empty_bar[s]));
      }
      mma_commit(smem_u32(&acc_bar));
    }
  } else {
    const int q = warp & 3;
    const int m = m0 + q * 32 + lane;
    const bool ok = __all_sync(0xffffffffu, mbar_wait(smem_u32(&acc_bar), 0u, err, kErrEpi)) &&
                    *(volatile int*)err == 0;
    fence_after();
    if (FUSE) {
      // This warp's 32 rows: each 32-column chunk of F dG goes through a shared-memory tile so
      // that f, t and g are read and written a row at a time (8 lanes x 4 channels per row,
      // four rows per instruction) instead of one row per lane.
      float(*tr)[36] = s_tr[q];
      const size_t row0 = (size_t)b * M + m0 + q * 32;
      const int rg = lane >> 3, qd = lane & 7;
      float acc = 0.0f;
      if (ok) {
#pragma unroll 1
        for (int c0 = 0; c0 < BN; c0 += 32) {
          uint32_t r[32];
          tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c0, r);
#pragma unroll
          for (int k = 0; k < 8; ++k)
            *reinterpret_cast<float4*>(&tr[lane][4 * k]) =
                make_float4(__uint_as_float(r[4 * k]), __uint_as_float(r[4 * k + 1]), __uint_as_float(r[4 * k + 2]),
                            __uint_as_float(r[4 * k + 3]));
          __syncwarp();
          // four rows' f and t first (8 loads in flight per lane), then their arithmetic
#pragma unroll 1
          for (int h = 0; h < 8; h += 4) {
          float fv[4][4], tv[4][4];
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const size_t off = (row0 + 4 * (h + i) + rg) * Nn + n0 + c0 + 4 * qd;
            if (fe.f_bf16) {
              const uint2 raw = __ldg(reinterpret_cast<const uint2*>(reinterpret_cast<const __nv_bfloat16*>(fe.f) + off));
              const float2 a = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&raw.x));
              const float2 c = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&raw.y));
              fv[i][0] = a.x; fv[i][1] = a.y; fv[i][2] = c.x; fv[i][3] = c.y;
            } else {
              const float4 v4 = __ldg(reinterpret_cast<const float4*>(reinterpret_cast<const float*>(fe.f) + off));
              fv[i][0] = v4.x; fv[i][1] = v4.y; fv[i][2] = v4.z; fv[i][3] = v4.w;
            }
            if (fe.t_bf16) {
              const uint2 raw = __ldg(reinterpret_cast<const uint2*>(reinterpret_cast<const __nv_bfloat16*>(fe.t) + off));
              const float2 a = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&raw.x));
              const float2 c = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&raw.y));
              tv[i][0] = a.x; tv[i][1] = a.y; tv[i][2] = c.x; tv[i][3] = c.y;
            } else {
              const float4 t4 = __ldg(reinterpret_cast<const float4*>(reinterpret_cast<const float*>(fe.t) + off));
              tv[i][0] = t4.x; tv[i][1] = t4.y; tv[i][2] = t4.z; tv[i][3] = t4.w;
            }
          }
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int rr = 4 * (h + i) + rg;
            const size_t off = (row0 + rr) * Nn + n0 + c0 + 4 * qd;
            const float4 gd = *reinterpret_cast<const float4*>(&tr[rr][4 * qd]);
            const float gg[4] = {gd.x, gd.y, gd.z, gd.w};
            float gv[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              const float d = fv[i][e] - tv[i][e];
              acc = fmaf(d, d, acc);
              gv[e] = fe.mask && !(fv[i][e] > 0.0f) ? 0.0f : fmaf(fe.coef, d, gg[e]);
            }
            __nv_bfloat162 h0 = __floats2bfloat162_rn(gv[0], gv[1]);
            __nv_bfloat162 h1 = __floats2bfloat162_rn(gv[2], gv[3]);
            *reinterpret_cast<uint2*>(fe.g + off) = make_uint2(*reinterpret_cast<uint32_t*>(&h0),
                                                               *reinterpret_cast<uint32_t*>(&h1));
          }
          }
          __syncwarp();  // the tile is rewritten by the next chunk
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if (lane == 0) fe.partial[((size_t)blockIdx.y * gridDim.x + blockIdx.x) * 4 + q] = acc;
    } else if (ok) {
      float* o = out + ((size_t)b * M + m) * Nn + n0;
#pragma unroll 1
      for (int c0 = 0; c0 < BN; c0 += 32) {
        uint32_t r[32];
        tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c0, r);
        float4* o4 = reinterpret_cast<float4*>(o + c0);
#pragma unroll
        for (int u = 0; u < 8; ++u)
          o4[u] = make_float4(__uint_as_float(r[4 * u]), __uint_as_float(r[4 * u + 1]), __uint_as_float(r[4 * u + 2]),
                              __uint_as_float(r[4 * u + 3]));
      }
    }
  }
  fence_before();
  __syncthreads();
  if (warp == 1) release_tmem(&acc_bar, tmem, (uint32_t)BN);
}

// ---------------------------------------------------------------- host side
static int encode_2d(CUtensorMap* map, const void* ptr, uint64_t inner, uint64_t outer, uint32_t box_inner,
                     uint32_t box_outer) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = nullptr;
  int rc = get_tensor_map_encoder(&enc);
  if (rc) return rc;
  const cuuint64_t dims[2] = {(cuuint64_t)inner, (cuuint64_t)outer};
  const cuuint64_t strides[1] = {(cuuint64_t)inner * 2};
  const cuuint32_t box[2] = {box_inner, box_outer};
  const cuuint32_t es[2] = {1, 1};
  const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box, es,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(SVBRDF_ERR_CUDA, "cuTensorMapEncodeTiled failed: %d", (int)r);
  return SVBRDF_OK;
}

// Dynamic shared memory for `need` bytes on the current device, once per instantiation.
template <typename K>
static int allow(K kern, size_t need, std::atomic<size_t>* have) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return fail(SVBRDF_ERR_CUDA, "no usable device");
  if (have[dev].load() < need) {
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need) != cudaSuccess)
      return fail(SVBRDF_ERR_CUDA, "cudaFuncSetAttribute: %s", cudaGetErrorString(cudaGetLastError()));
    have[dev].store(need);
  }
  return SVBRDF_OK;
}

template <int BN, int STAGES, bool Z64>
static int launch_gram(const CUtensorMap& m, float* partial, int v, int s, int c, int splits, int pps, int* err,
                       cudaStream_t st) {
  static std::atomic<size_t> have[64];
  const size_t smem = (size_t)STAGES * ((Z64 ? 0 : 2 * kAtom) + (BN / 64) * kAtom) + (Z64 ? kAtom : 0) + 1024;
  auto kern = gram_kernel<BN, STAGES, Z64>;
  int rc = allow(kern, smem, have);
  if (rc) return rc;
  dim3 grid((unsigned)(((c + 127) / 128) * (c / BN)), (unsigned)splits, (unsigned)v);
  kern<<<grid, kThreads, smem, st>>>(m, partial, s, c, splits, pps, err);
  return check_launch("gram_kernel");
}

template <int BN, int STAGES, bool FUSE>
static int launch_gemm(const CUtensorMap& ma, const CUtensorMap& mb, float* out, int batch, int m, int n, int k,
                       int* err, const FeatEpi& fe, cudaStream_t st) {
  static std::atomic<size_t> have[64];
  const size_t smem = (size_t)STAGES * (128 * 64 * 2 + BN * 64 * 2) + 1024;
  auto kern = gemm_nt_kernel<BN, STAGES, FUSE>;
  int rc = allow(kern, smem, have);
  if (rc) return rc;
  dim3 grid((unsigned)(batch * (m / 128)), (unsigned)(n / BN));
  kern<<<grid, kThreads, smem, st>>>(ma, mb, out, m, n, k, err, fe);
  return check_launch("gemm_nt_kernel");
}

// Shared by svbrdf_desc_gemm_nt (FUSE false, out) and svbrdf_desc_gemm_nt_feat (FUSE true, fe).
template <bool FUSE>
static int gemm_nt_entry(const void* a, const void* b, float* out, int batch, int m, int n, int k, int* err,
                         const FeatEpi& fe, void* stream) {
  if (!a || !b || !err || (!FUSE && !out)) return fail(SVBRDF_ERR_INVALID, "gemm_nt: null a/b/out/err");
  if (FUSE && (!fe.f || !fe.t || !fe.g || !fe.partial)) return fail(SVBRDF_ERR_INVALID, "gemm_nt_feat: null f/t/g/partial");
  if (batch < 1 || m < 128 || m % 128 || k < 64 || k % 64 || (n != 64 && n != 128 && n % 256))
    return fail(SVBRDF_ERR_UNSUPPORTED, "gemm_nt: m %% 128, k %% 64 and n in {64, 128, 256 x j} needed");
  if ((long long)batch * m >= (1LL << 31) || (long long)batch * n >= (1LL << 31) || k > 65536)
    return fail(SVBRDF_ERR_UNSUPPORTED, "gemm_nt: too large");
  if ((long long)batch * (m / 128) > 0x7fffffffLL || n / (n >= 256 ? 256 : n) > 65535)
    return fail(SVBRDF_ERR_UNSUPPORTED, "gemm_nt: grid too large");
  if (((uintptr_t)a | (uintptr_t)b | (uintptr_t)out | (uintptr_t)fe.f | (uintptr_t)fe.t | (uintptr_t)fe.g) % 16)
    return fail(SVBRDF_ERR_INVALID, "gemm_nt: 16-byte alignment");
  CUtensorMap ma, mb;
  const int bn = n >= 256 ? 256 : n;
  int rc = encode_2d(&ma, a, (uint64_t)k, (uint64_t)batch * m, 64, 128);
  if (rc) return rc;
  rc = encode_2d(&mb, b, (uint64_t)k, (uint64_t)batch * n, 64, (uint32_t)bn);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  if (k <= 64 && bn == 64) {
    // one k-step per tile: a single stage keeps the CTA at about 42 KB, five to an SM, so that
    // more tiles' epilogues (the fused feature term, memory-latency bound) run at once
    return launch_gemm<64, 1, FUSE>(ma, mb, out, batch, m, n, k, err, fe, st);
  }
  if (k <= 128) {
    // one or two k-steps per tile: a 2-stage ring keeps the CTA small (49-97 KB), so several
    // CTAs share an SM and one's set-up and epilogue overlap another's loads and MMAs
    if (bn == 64) return launch_gemm<64, 2, FUSE>(ma, mb, out, batch, m, n, k, err, fe, st);
    if (bn == 128) return launch_gemm<128, 2, FUSE>(ma, mb, out, batch, m, n, k, err, fe, st);
    return launch_gemm<256, 2, FUSE>(ma, mb, out, batch, m, n, k, err, fe, st);
  }
  if (bn == 64) return launch_gemm<64, 6, FUSE>(ma, mb, out, batch, m, n, k, err, fe, st);
  if (bn == 128) return launch_gemm<128, 5, FUSE>(ma, mb, out, batch, m, n, k, err, fe, st);
  return launch_gemm<256, 4, FUSE>(ma, mb, out, batch, m, n, k, err, fe, st);
}

}  // namespace gram
}  // namespace svb

using namespace svb;

extern "C" {

int svbrdf_desc_gram_splits(int v, int s, int c) {
  if (v < 1 || s < gram::KP || c < 64) return 0;
  // The product's K (pixels) is split so that the tiles of all views make about one wave of
  // 152 CTAs where C >= 128 (each split's [c][c] partial is read back by the finishing sum)
  // and two waves where C = 64 (small partials, and the product per split is short: measured
  // 27 us against 34 with one wave on 9 views of 256^2); every split gets the same whole
  // number of 64-pixel steps (none is empty).
  const int tiles = ((c + 127) / 128) * (c / (c >= 256 ? 256 : c));
  const int steps = s / gram::KP;
  const int target = c <= 64 ? 304 : 152;
  int splits = target / (tiles * v);  // rounded down: all CTAs in the intended waves
  if (splits < 1) splits = 1;
  if (splits > steps) splits = steps;
  const int per = (steps + splits - 1) / splits;
  return (steps + per - 1) / per;
}

int svbrdf_desc_gram(const void* features, float* partial, int v, int s, int c, int splits, int* err, void* stream) {
  using namespace svb::gram;
  if (!features || !partial || !err) return fail(SVBRDF_ERR_INVALID, "gram: null features/partial/err");
  if (v < 1 || v > 65535 || s < KP || s % KP) return fail(SVBRDF_ERR_UNSUPPORTED, "gram: S must be a multiple of 64");
  if (c != 64 && c != 128 && c % 256) return fail(SVBRDF_ERR_UNSUPPORTED, "gram: C must be 64, 128 or a multiple of 256");
  if (c > 4096) return fail(SVBRDF_ERR_UNSUPPORTED, "gram: C above 4096");
  if (splits < 1 || splits > s / KP || splits > 65535) return fail(SVBRDF_ERR_INVALID, "gram: bad split count %d", splits);
  if ((long long)v * s >= (1LL << 31)) return fail(SVBRDF_ERR_UNSUPPORTED, "gram: too many pixels");
  if ((uintptr_t)features % 16 || (uintptr_t)partial % 16) return fail(SVBRDF_ERR_INVALID, "gram: 16-byte alignment");
  const int steps = s / KP;
  const int pps = ((steps + splits - 1) / splits) * KP;
  CUtensorMap m;
  int rc = encode_2d(&m, features, (uint64_t)c, (uint64_t)v * s, 64, 64);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  if (c == 64) return launch_gram<64, 8, true>(m, partial, v, s, c, splits, pps, err, st);  // 73 KB: 3 CTAs per SM
  if (c == 128) return launch_gram<128, 5, false>(m, partial, v, s, c, splits, pps, err, st);
  return launch_gram<256, 4, false>(m, partial, v, s, c, splits, pps, err, st);
}

int svbrdf_desc_gram_finish(const float* partial, int splits, int v, int c, int s, const float* gram_target,
                            float coef, float* gram_out, void* dgram, float* loss_part, void* stream) {
  if (!partial || splits < 1 || v < 1 || v > 65535 || c < 1 || c > 65535 || s < 1)
    return fail(SVBRDF_ERR_INVALID, "gram_finish: bad arguments");
  int cw = 32;
  while (cw < c && cw < 256) cw *= 2;
  const int rows = 256 / cw;
  dim3 grid((unsigned)((c + rows - 1) / rows), (unsigned)v);
  gram::gram_finish_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(partial, splits, c, cw, 1.0f / (float)s, gram_target,
                                                                   coef, gram_out, (__nv_bfloat16*)dgram, loss_part);
  return check_launch("gram_finish_kernel");
}

int svbrdf_desc_gemm_nt(const void* a, const void* b, float* out, int batch, int m, int n, int k, int* err,
                        void* stream) {
  const gram::FeatEpi none{};
  return gram::gemm_nt_entry<false>(a, b, out, batch, m, n, k, err, none, stream);
}

long long svbrdf_desc_gemm_nt_feat_partials(int batch, int m, int n) {
  if (batch < 1 || m < 128 || n < 64) return 0;
  return (long long)batch * (m / 128) * (n / (n >= 256 ? 256 : n)) * 4;
}

int svbrdf_desc_gemm_nt_feat(const void* a, const void* b, const void* f, int dtypes, const void* t, float coef,
                             int mask, void* g, float* partial, int batch, int m, int n, int k, int* err,
                             void* stream) {
  if (dtypes < 0 || dtypes > 3) return fail(SVBRDF_ERR_INVALID, "gemm_nt_feat: dtypes must be 0..3");
  const gram::FeatEpi fe{f, dtypes & 1, t, (dtypes >> 1) & 1, coef, mask ? 1 : 0, (__nv_bfloat16*)g, partial};
  return gram::gemm_nt_entry<true>(a, b, nullptr, batch, m, n, k, err, fe, stream);
}

}  // extern "C"
