// Fused render + loss + adjoint + Adam: one pass per optimiser iteration.
//
// Replaces the loop body of SvbrdfOptim.optim (src/svbrdf.py:56-71):
//   rendereds = eval(textures.clamp(-1, 1)); loss = MSE(rendereds, targets);
//   zero_grad(); loss.backward(); optimizer.step()
// Each texel's 9 parameters, its Adam moments and its V targets are read once, every
// per-view term is recomputed in registers, and the parameters and moments are written
// back. Per-iteration HBM traffic: 108 B read + 108 B written + 12*V B of targets per texel
// (variants 3 and 4 move that once per launch of up to 32 iterations).
//
// Kernels:
//   fused_step_kernel     one material, grid-stride, direct loads (drop-in SvbrdfOptim)
//   batched_step_kernel   many materials, persistent, direct loads           (variant 0)
//   batched_tma_kernel    many materials, persistent, warp-specialised bulk-copy
//                         (TMA) pipeline through a shared-memory ring         (variant 1)
//   batched_pair_kernel   the variant 1 pipeline with two texels per thread in
//                         FP32x2                                              (variant 2)
//   batched_fuse_kernel   variant 2's arithmetic, up to 32 iterations per launch on
//                         each tile's state held in shared memory             (variant 3)
//   batched_fuse2_kernel  variant 3 without the producer warp: the last warp to
//                         finish with a buffer refills it                     (variant 4)
#include <math.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <numeric>
#include <vector>

#include "svbrdf_common.cuh"
#include "svbrdf_plan.cuh"

namespace svb {

int check_common(const float* tex, const float* cam, const float* lit, const float* lpow, int V, int H, int W,
                 float size);

// Most iterations one launch of the resident-state kernels runs (svbrdf_batched_steps splits
// longer runs evenly); the workspace holds loss partials for that many.
constexpr int kFuseMax = 32;
int grid_for(long long T, int threads, int occupancy_blocks);

AdamScalars make_adam(int step, float lr, float beta1, float beta2, float eps) {
  // torch.optim.Adam computes the bias corrections as Python floats (double) and hands
  // them to FP32 kernels.
  const double bc1 = 1.0 - pow((double)beta1, (double)step);
  const double bc2 = 1.0 - pow((double)beta2, (double)step);
  AdamScalars s;
  s.one_minus_b1 = (float)(1.0 - (double)beta1);
  s.b2 = beta2;
  s.one_minus_b2 = (float)(1.0 - (double)beta2);
  s.inv_bc2_sqrt = (float)(1.0 / sqrt(bc2));
  s.eps = eps;
  s.neg_step_size = (float)(-(double)lr / bc1);
  return s;
}

__device__ __forceinline__ AdamScalars device_adam(const AdamHyper& h, int step) {
  const double bc1 = 1.0 - pow((double)h.beta1, (double)step);
  const double bc2 = 1.0 - pow((double)h.beta2, (double)step);
  AdamScalars s;
  s.one_minus_b1 = (float)(1.0 - (double)h.beta1);
  s.b2 = h.beta2;
  s.one_minus_b2 = (float)(1.0 - (double)h.beta2);
  s.inv_bc2_sqrt = (float)(1.0 / sqrt(bc2));
  s.eps = h.eps;
  s.neg_step_size = (float)(-(double)h.lr / bc1);
  return s;
}

// Render, loss and adjoint of one texel over its V views, from already-loaded inputs.
// `raw` are the stored parameters (the optimiser clamps them to [-1, 1] before eval,
// src/svbrdf.py:60); targets come from `tgt_at(v, c)`. Returns the summed squared error
// and the parameter gradient scaled by `scale`, zero outside [-1, 1].
template <int LOSS, bool GRAD_POW, bool ALL_COLOC, typename TgtFn>
__device__ __forceinline__ float texel_fused_grad(const float raw[9], float px, float py, int V, const View* s_views,
                                                  const float* s_pow, float scale, TgtFn tgt_at, float g[9],
                                                  float gp[3]) {
  float t[9];
#pragma unroll
  for (int c = 0; c < 9; ++c) t[c] = fminf(fmaxf(raw[c], -1.0f), 1.0f);
  if (ALL_COLOC) {
    const float loss = coloc_texel<LOSS, GRAD_POW>(t, px, py, V, s_views, s_pow, scale, tgt_at, g, gp);
#pragma unroll
    for (int c = 0; c < 9; ++c) g[c] = (raw[c] >= -1.0f && raw[c] <= 1.0f) ? g[c] : 0.0f;
    return loss;
  }
  Maps m;
  decode(t, m);
  Adj a;
  adj_zero(a);
  float loss = 0.f;
  for (int v = 0; v < V; ++v) {
    float io[3];
    tgt_at(v, io);
    if (s_views[v].coloc != 0.f)
      texel_view<kModeFused, LOSS, GRAD_POW, true>(m, px, py, s_views[v], s_pow, io, loss, a);
    else
      texel_view<kModeFused, LOSS, GRAD_POW, false>(m, px, py, s_views[v], s_pow, io, loss, a);
  }
  adj_to_params(t, m, a, scale, g);
#pragma unroll
  for (int c = 0; c < 9; ++c) g[c] = (raw[c] >= -1.0f && raw[c] <= 1.0f) ? g[c] : 0.0f;
  if (GRAD_POW) {
    gp[0] += a.gp[0] * scale;
    gp[1] += a.gp[1] * scale;
    gp[2] += a.gp[2] * scale;
  }
  return loss;
}

// One texel of one fused iteration with direct global loads. Returns the squared error.
template <int LOSS, bool GRAD_POW, bool ALL_COLOC>
__device__ __forceinline__ float fused_texel(float* __restrict__ tex, float* __restrict__ mom1,
                                             float* __restrict__ mom2, const float* __restrict__ tgt, long long T,
                                             long long idx, float px, float py, int V, const View* s_views,
                                             const float* s_pow, float scale, const AdamScalars& adam,
                                             float gp[3]) {
  float raw[9];
#pragma unroll
  for (int c = 0; c < 9; ++c) raw[c] = tex[(size_t)c * T + idx];
  const float* tp = tgt + idx;
  auto tgt_at = [&](int v, float io[3]) {
    const float* p = tp + (size_t)(3 * v) * T;
    io[0] = __ldcs(p);
    io[1] = __ldcs(p + T);
    io[2] = __ldcs(p + 2 * (size_t)T);
  };
  float g[9];
  const float loss =
      texel_fused_grad<LOSS, GRAD_POW, ALL_COLOC>(raw, px, py, V, s_views, s_pow, scale, tgt_at, g, gp);
#pragma unroll
  for (int c = 0; c < 9; ++c) {
    float p = raw[c];
    float m1 = mom1[(size_t)c * T + idx];
    float m2 = mom2[(size_t)c * T + idx];
    adam_update(p, m1, m2, g[c], adam);
    tex[(size_t)c * T + idx] = p;
    mom1[(size_t)c * T + idx] = m1;
    mom2[(size_t)c * T + idx] = m2;
  }
  return loss;
}

constexpr int kFusedThreads = 256;

template <int LOSS, bool GRAD_POW>
__global__ void __launch_bounds__(kFusedThreads)
fused_step_kernel(float* __restrict__ tex, float* __restrict__ mom1, float* __restrict__ mom2,
                  const float* __restrict__ tgt, const float* __restrict__ cam, const float* __restrict__ lit,
                  float* __restrict__ lpow, float* __restrict__ lstate, int V, int H, int W, float size,
                  float scale, double inv_n, AdamScalars adam, float* loss_out, float4* partials,
                  unsigned* counter) {
  __shared__ View s_views[kMaxViews];
  __shared__ float s_pow[3];
  __shared__ float s_red[kFusedThreads / 32];
  __shared__ double s_dred[4 * kFusedThreads / 32];
  __shared__ int s_flag;
  stage_views(s_views, cam, lit, V);
  if (threadIdx.x < 3) s_pow[threadIdx.x] = lpow[threadIdx.x];
  __syncthreads();

  // 64-bit texel index: the grid-stride step cannot wrap for any H*W the host accepts
  const long long T = (long long)H * W;
  const long long stride = (long long)gridDim.x * blockDim.x;
  float loss = 0.f;
  float gp[3] = {0.f, 0.f, 0.f};
  bool allc = true;
  for (int v = 0; v < V; ++v) allc = allc && (s_views[v].coloc != 0.f);
  if (allc) {
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < T; idx += stride) {
      float px, py;
      texel_pos((int)(idx / W), (int)(idx % W), W, H, size, px, py);
      loss += fused_texel<LOSS, GRAD_POW, true>(tex, mom1, mom2, tgt, T, idx, px, py, V, s_views, s_pow, scale,
                                                adam, gp);
    }
  } else {
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < T; idx += stride) {
      float px, py;
      texel_pos((int)(idx / W), (int)(idx % W), W, H, size, px, py);
      loss += fused_texel<LOSS, GRAD_POW, false>(tex, mom1, mom2, tgt, T, idx, px, py, V, s_views, s_pow, scale,
                                                 adam, gp);
    }
  }

  const float bl = block_sum<kFusedThreads>(loss, s_red);
  float b0 = 0.f, b1 = 0.f, b2 = 0.f;
  if (GRAD_POW) {
    b0 = block_sum<kFusedThreads>(gp[0], s_red);
    b1 = block_sum<kFusedThreads>(gp[1], s_red);
    b2 = block_sum<kFusedThreads>(gp[2], s_red);
  }
  if (publish_partial_and_check_last(partials, counter, make_float4(bl, b0, b1, b2), &s_flag)) {
    double tot[4];
    sum_partials<kFusedThreads>(partials, gridDim.x, tot, s_dred);
    if (threadIdx.x == 0) {
      *loss_out = (float)(tot[0] * inv_n);
      if (GRAD_POW) {
        // Adam on the learnable light power, same hyper-parameters and step as the maps
        // (one optimiser over [textures, light_pow], src/svbrdf.py:50).
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          float p = s_pow[c], m1 = lstate[c], m2 = lstate[3 + c];
          adam_update(p, m1, m2, (float)tot[1 + c], adam);
          lpow[c] = p;
          lstate[c] = m1;
          lstate[3 + c] = m2;
        }
      }
      *counter = 0u;
    }
  }
}

template <typename K>
int occupancy_of(K kernel, int threads, size_t smem = 0) {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, smem) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return n;
}

// ---- row/column of a texel index without integer division: exact for T < 2^24 ----
__device__ __forceinline__ void texel_rc(int idx, const MatDesc& md, int& i, int& j) {
  i = (int)((float)idx * md.inv_w);
  j = idx - i * md.W;
  if (j < 0) { --i; j += md.W; }
  else if (j >= md.W) { ++i; j -= md.W; }
}

// End of a batched launch, in every CTA: the warps' partial losses (`per_tile` per tile and
// iteration; and with a learnable light, the light-gradient partials) of this CTA's own tiles
// are summed per (iteration, tile) in warp order into the tile totals that follow the partials
// in the workspace. The last CTA to finish then forms each material's mean loss from its
// tiles' totals in tile order (a launch that ran `iters` iterations, steps step - iters + 1 ..
// step, fills one loss_hist row per iteration), runs Adam on the learnable light powers, stores
// the step counter and resets the completion counter. Both levels have a fixed order, so the
// losses are deterministic; the last CTA reads one value per tile and iteration instead of
// one per warp (15x fewer), in parallel across its warps.
template <int NT>
__device__ __forceinline__ void batched_finish(const char* plan, const PlanHeader* hdr, const MatDesc* mats,
                                               const float* partial, int per_tile, float* loss_hist, int hist_len,
                                               int step, int* step_counter, unsigned* counter, int* s_flag,
                                               int nwarps, int iters = 1, const float* lpart = nullptr,
                                               const AdamScalars* light_adam = nullptr) {
  const int n_tiles = hdr->n_tiles;
  const size_t slots = (size_t)n_tiles * per_tile;
  float* tile_tot = const_cast<float*>(partial) + slots * (hdr->variant >= 3 ? kFuseMax : 1) + (hdr->light ? 3 * slots : 0);
  __syncthreads();  // every warp of this CTA has written its partials
  {
    const int* cta_off = (const int*)(plan + hdr->off_cta);
    const int* order = (const int*)(plan + hdr->off_order);
    const int k0 = cta_off[blockIdx.x], nk = cta_off[blockIdx.x + 1] - k0;
    for (int e = threadIdx.x; e < iters * nk; e += blockDim.x) {
      const int i = e / nk, tile = order[k0 + e % nk];
      const float* p = partial + ((size_t)i * n_tiles + tile) * per_tile;
      float t = 0.f;
      for (int q = 0; q < per_tile; ++q) t += __ldcg(p + q);
      tile_tot[(size_t)i * n_tiles + tile] = t;
    }
    if (lpart) {
      for (int e = threadIdx.x; e < 3 * nk; e += blockDim.x) {
        const int c = e / nk, tile = order[k0 + e % nk];
        const float* p = lpart + 3 * (size_t)tile * per_tile + c;  // (tile, warp, channel)
        float t = 0.f;
        for (int q = 0; q < per_tile; ++q) t += __ldcg(p + 3 * q);
        tile_tot[(size_t)(kFuseMax + c) * n_tiles + tile] = t;
      }
    }
    __threadfence();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned prev = atomicAdd(counter, 1u);
    *s_flag = (prev == gridDim.x - 1) ? 1 : 0;
  }
  __syncthreads();
  if (!*s_flag) return;
  __threadfence();
  const int* mat_tiles = (const int*)(plan + hdr->off_mat_tiles);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  // one warp per (iteration, material)
  for (int e = w; e < iters * hdr->n_mat; e += nw) {
    const int i = e / hdr->n_mat, mi = e % hdr->n_mat;
    const float* tt = tile_tot + (size_t)i * n_tiles;
    double acc = 0.0;
    for (int t = mat_tiles[mi] + lane; t < mat_tiles[mi + 1]; t += 32) acc += (double)__ldcg(tt + t);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) loss_hist[(size_t)((step - iters + i) % hist_len) * hdr->n_mat + mi] = (float)(acc * mats[mi].inv_n);
  }
  if (lpart) {
    // Learnable light (one-iteration launches): per material, the light-power gradient summed
    // over its tiles in a fixed order, then Adam on the light with the maps' hyper-parameters
    // and step (one optimiser over [textures, light_pow], src/svbrdf.py:50).
    const AdamScalars ad = *light_adam;
    for (int mi = w; mi < hdr->n_mat; mi += nw) {
      const MatDesc& md = mats[mi];
      if (!md.lstate) continue;
      double g[3] = {0.0, 0.0, 0.0};
      for (int t = mat_tiles[mi] + lane; t < mat_tiles[mi + 1]; t += 32) {
#pragma unroll
        for (int c = 0; c < 3; ++c) g[c] += (double)__ldcg(tile_tot + (size_t)(kFuseMax + c) * n_tiles + t);
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) g[c] += __shfl_xor_sync(0xffffffffu, g[c], o);
      }
      if (lane == 0) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          float p = md.lpow[c], m1 = md.lstate[c], m2 = md.lstate[3 + c];
          adam_update(p, m1, m2, (float)g[c], ad);
          md.lpow[c] = p;
          md.lstate[c] = m1;
          md.lstate[3 + c] = m2;
        }
      }
    }
  }
  if (threadIdx.x == 0) {
    *step_counter = step;
    *counter = 0u;
  }
}

// Light-power gradient partial of one warp's texels of one tile: lanes' values summed in a
// fixed order, written by lane 0 to slot (tile, warp).
__device__ __forceinline__ void write_light_partial(float* lpart, int tile, int nwarps, float s0, float s1, float s2) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    s0 += __shfl_xor_sync(0xffffffffu, s0, o);
    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  }
  if ((threadIdx.x & 31) == 0) {
    float* p = lpart + 3 * ((size_t)tile * nwarps + (threadIdx.x >> 5));
    p[0] = s0;
    p[1] = s1;
    p[2] = s2;
  }
}

// ============================================================== variant 0: direct loads
template <int LOSS, int NT>
__global__ void __launch_bounds__(NT)
batched_step_kernel(const char* __restrict__ plan, AdamHyper hyper, int* __restrict__ step_counter,
                    float* __restrict__ loss_hist, int hist_len, float* __restrict__ tile_loss, unsigned* ws) {
  __shared__ View s_views[kMaxViews];
  __shared__ float s_pow[3];
  __shared__ float s_red[NT / 32];
  __shared__ AdamScalars s_adam;
  __shared__ int s_step;
  if (threadIdx.x == 0) {
    s_step = *step_counter + 1;  // 1-based step of this launch
    s_adam = device_adam(hyper, s_step);
  }
  __syncthreads();
  const AdamScalars adam = s_adam;
  const PlanHeader* hdr = (const PlanHeader*)plan;
  const MatDesc* mats = (const MatDesc*)(plan + hdr->off_mats);
  const View* views = (const View*)(plan + hdr->off_views);
  const int* cta_off = (const int*)(plan + hdr->off_cta);
  const int* order = (const int*)(plan + hdr->off_order);
  const int2* tiles = (const int2*)(plan + hdr->off_tiles);
  const float* coords = (const float*)(plan + hdr->off_coords);
  const int tile_texels = hdr->tile_texels;

  int cur = -1;
  MatDesc md;
  float gp_unused[3];
  const int k0 = cta_off[blockIdx.x], k1 = cta_off[blockIdx.x + 1];
  for (int k = k0; k < k1; ++k) {
    const int tid = order[k];
    const int2 tl = tiles[tid];
    if (tl.x != cur) {
      __syncthreads();
      cur = tl.x;
      md = mats[cur];
      for (int v = threadIdx.x; v < md.V; v += NT) s_views[v] = views[md.view_off + v];
      if (threadIdx.x < 3) s_pow[threadIdx.x] = md.lpow[threadIdx.x];
      __syncthreads();
    }
    const int T = md.H * md.W;
    const int end = min(tl.y + tile_texels, T);
    float loss = 0.f;
    for (int idx = tl.y + threadIdx.x; idx < end; idx += NT) {
      int i, j;
      texel_rc(idx, md, i, j);
      const float px = __ldg(coords + md.coord_off + j), py = __ldg(coords + md.coord_off + md.W + i);
      if (md.all_coloc)
        loss += fused_texel<LOSS, false, true>(md.tex, md.m1, md.m2, md.tgt, T, idx, px, py, md.V, s_views, s_pow,
                                               md.scale, adam, gp_unused);
      else
        loss += fused_texel<LOSS, false, false>(md.tex, md.m1, md.m2, md.tgt, T, idx, px, py, md.V, s_views, s_pow,
                                                md.scale, adam, gp_unused);
    }
    const float bl = block_sum<NT>(loss, s_red);
    if (threadIdx.x == 0) tile_loss[tid] = bl;
  }
  __shared__ int s_last;
  batched_finish<NT>(plan, hdr, mats, tile_loss, 1, loss_hist, hist_len, s_step, step_counter,
                     ws + kWsCounter, &s_last, NT / 32);
}

// ============================================================== variant 1: TMA pipeline
//
// One producer warp streams, per tile of NT = 32*NCW texels, the chunks
//   P  = the 9 parameter planes,
//   Tc = target planes of views 4c .. 4c+3 (3 planes per view),  c = 0 .. ceil(V/4)-1,
//   M  = the 9 exp_avg planes,  S = the 9 exp_avg_sq planes
// into a ring of shared-memory slots of 12 planes x NT floats with cp.async.bulk (the
// non-tensor TMA path). Each slot has an mbarrier signalling "full" (transaction bytes)
// and one signalling "empty" (one arrival per consumer warp). The NCW consumer warps own
// one texel per thread and read everything from shared memory, so the bytes in flight
// are bounded by the ring, not by registers. Updated parameters and moments go back with
// coalesced stores. Every wait is bounded: on timeout the kernel records an error in the
// workspace, stops issuing, drains its in-flight copies and returns.

constexpr int kMaxRing = 64;
constexpr int kSlotPlanes = 12;  // 9 parameter/moment planes, or 4 views x 3 target planes
constexpr uint32_t kSpinLimit = 1u << 22;
constexpr size_t kRingBudget = 200 * 1024;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}
__device__ __forceinline__ void named_sync(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// Bounded wait on an mbarrier phase. Gives up (and records `code`) after `limit` polls, or
// early once another warp has recorded an error.
__device__ __forceinline__ bool wait_phase_n(uint32_t bar, uint32_t parity, int* err, int code, uint32_t limit) {
  uint32_t it = 0;
  while (!mbar_try_wait(bar, parity)) {
    if (++it >= limit) {
      atomicCAS(err, 0, code);
      return false;
    }
    if ((it & 255u) == 0 && *(volatile int*)err != 0) return false;
  }
  return true;
}

__device__ __forceinline__ bool wait_phase(uint32_t bar, uint32_t parity, int* err, int code) {
  return wait_phase_n(bar, parity, err, code, kSpinLimit);
}

// Consumer-side ring cursor.
struct RingCursor {
  int slot;
  uint32_t phase;
  bool ok;
};

template <int NT>
__device__ __forceinline__ const float* ring_acquire(RingCursor& rc, const float* ring, uint64_t* full_bar, int* err) {
  if (rc.ok) rc.ok = __all_sync(0xffffffffu, wait_phase(smem_u32(&full_bar[rc.slot]), rc.phase, err, kDevTimeoutFull));
  return ring + (size_t)rc.slot * (kSlotPlanes * NT);
}

__device__ __forceinline__ void ring_release(RingCursor& rc, uint64_t* empty_bar, int R) {
  __syncwarp();
  if ((threadIdx.x & 31) == 0 && rc.ok) mbar_arrive(smem_u32(&empty_bar[rc.slot]));
  if (++rc.slot == R) { rc.slot = 0; rc.phase ^= 1u; }
}

// Step past the current slot without freeing it (released later with ring_release_slot).
__device__ __forceinline__ int ring_hold(RingCursor& rc, int R) {
  const int held = rc.slot;
  if (++rc.slot == R) { rc.slot = 0; rc.phase ^= 1u; }
  return held;
}

__device__ __forceinline__ void ring_release_slot(const RingCursor& rc, int slot, uint64_t* empty_bar) {
  __syncwarp();
  if ((threadIdx.x & 31) == 0 && rc.ok) mbar_arrive(smem_u32(&empty_bar[slot]));
}

template <int LOSS, int NCW>
__global__ void __launch_bounds__((NCW + 1) * 32, 1)
batched_tma_kernel(const char* __restrict__ plan, AdamHyper hyper, int* __restrict__ step_counter,
                   float* __restrict__ loss_hist, int hist_len, float* __restrict__ warp_loss, unsigned* ws) {
  constexpr int NT = NCW * 32;
  constexpr int SLOT = kSlotPlanes * NT;  // floats per ring slot
  extern __shared__ __align__(128) float ring[];
  __shared__ __align__(8) uint64_t full_bar[kMaxRing];
  __shared__ __align__(8) uint64_t empty_bar[kMaxRing];
  __shared__ View s_views[kMaxViews];
  __shared__ __align__(8) float s_cx[kMaxViews + 2], s_cy[kMaxViews + 2], s_cz[kMaxViews + 2];
  __shared__ MatDesc s_md;
  __shared__ float s_pow[3];
  __shared__ AdamScalars s_adam;
  __shared__ int s_step;
  __shared__ int s_last;

  const PlanHeader* hdr = (const PlanHeader*)plan;
  const MatDesc* mats = (const MatDesc*)(plan + hdr->off_mats);
  const View* views = (const View*)(plan + hdr->off_views);
  const int* cta_off = (const int*)(plan + hdr->off_cta);
  const int* order = (const int*)(plan + hdr->off_order);
  const int2* tiles = (const int2*)(plan + hdr->off_tiles);
  const float* coords = (const float*)(plan + hdr->off_coords);
  const int R = hdr->ring_slots;
  int* err = (int*)(ws + kWsError);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < R; ++s) {
      mbar_init(smem_u32(&full_bar[s]), 1);
      mbar_init(smem_u32(&empty_bar[s]), NCW);
    }
    fence_mbar_init();
    s_step = *step_counter + 1;
    s_adam = device_adam(hyper, s_step);
  }
  __syncthreads();
  const int k0 = cta_off[blockIdx.x], k1 = cta_off[blockIdx.x + 1];
  const uint32_t ring_base = smem_u32(ring);

  if (warp == NCW) {
    // ------------------------------------------------------------ producer
    if (lane == 0) {
      int slot = 0;
      uint32_t phase = 0;
      long long issued = 0;
      bool ok = true;
      for (int k = k0; k < k1 && ok; ++k) {
        const int2 tl = tiles[order[k]];
        const MatDesc md = mats[tl.x];
        const int T = md.H * md.W, V = md.V;
        const uint32_t bytes = (uint32_t)min(NT, T - tl.y) * 4u;
        const int nt = (V + 3) / 4;
        for (int q = 0; q < nt + 3; ++q) {
          if (issued >= R && !wait_phase(smem_u32(&empty_bar[slot]), phase ^ 1u, err, kDevTimeoutEmpty)) {
            ok = false;
            break;
          }
          const float* base;
          int plane0, nplanes;
          if (q == 0) { base = md.tex; plane0 = 0; nplanes = 9; }
          else if (q <= nt) { base = md.tgt; plane0 = 12 * (q - 1); nplanes = min(12, 3 * V - plane0); }
          else if (q == nt + 1) { base = md.m1; plane0 = 0; nplanes = 9; }
          else { base = md.m2; plane0 = 0; nplanes = 9; }
          const uint32_t fb = smem_u32(&full_bar[slot]);
          mbar_arrive_expect_tx(fb, (uint32_t)nplanes * bytes);
          const float* src = base + (size_t)plane0 * T + tl.y;
          for (int p = 0; p < nplanes; ++p)
            bulk_g2s(ring_base + (uint32_t)(slot * SLOT + p * NT) * 4u, src + (size_t)p * T, bytes, fb);
          ++issued;
          if (++slot == R) { slot = 0; phase ^= 1u; }
        }
      }
      if (!ok) {
        // drain: wait for the copies of the last min(R, issued) chunks to land
        const long long n = issued < R ? issued : R;
        int s = slot;
        uint32_t ph = phase;
        for (long long i = 0; i < n; ++i) {
          if (--s < 0) { s = R - 1; ph ^= 1u; }
          uint32_t it = 0;
          while (!mbar_try_wait(smem_u32(&full_bar[s]), ph)) {
            if (++it >= kSpinLimit) { atomicCAS(err, 0, kDevTimeoutDrain); break; }
          }
        }
      }
    }
  } else {
    // ------------------------------------------------------------ consumers
    const int tid = threadIdx.x;
    RingCursor rc{0, 0u, true};
    int cur = -1;
    for (int k = k0; k < k1; ++k) {
      const int tile = order[k];
      const int2 tl = tiles[tile];
      if (tl.x != cur) {  // uniform over the consumer warps
        named_sync(1, NT);
        cur = tl.x;
        if (tid == 0) s_md = mats[cur];
        const int vo = mats[cur].view_off, nv = mats[cur].V;
        for (int v = tid; v < nv; v += NT) {
          const View w = views[vo + v];
          s_views[v] = w;
          s_cx[v] = w.cx;
          s_cy[v] = w.cy;
          s_cz[v] = w.cz;
        }
        if (tid < 3) s_pow[tid] = mats[cur].lpow[tid];
        named_sync(1, NT);
      }
      const int T = s_md.H * s_md.W, V = s_md.V;
      const bool active = tid < T - tl.y;
      const int idx = tl.y + tid;
      const float scale = s_md.scale;
      float px = 0.f, py = 0.f;
      if (active) {
        int i, j;
        texel_rc(idx, s_md, i, j);
        px = __ldg(coords + s_md.coord_off + j);
        py = __ldg(coords + s_md.coord_off + s_md.W + i);
      }
      // ---- parameters: the slot stays held until the update, so the 9 values are read
      // again there instead of being kept in registers through the view loop
      const float* psl = ring_acquire<NT>(rc, ring, full_bar, err);
      const int pslot = ring_hold(rc, R);
      float g[9], gp[3];
      float loss;
      if (s_md.all_coloc) {
        TexelC2 tp;
        {
          float t9[9];
#pragma unroll
          for (int c = 0; c < 9; ++c) t9[c] = fminf(fmaxf(psl[c * NT + tid], -1.0f), 1.0f);
          TexelC tc;
          coloc_prepare(t9, px, py, tc);
          pack_texel(tc, tp);
        }
        AccC2 ap;
        acc2_zero(ap);
        const float2 PP[3] = {bc2(s_pow[0]), bc2(s_pow[1]), bc2(s_pow[2])};
        for (int v0 = 0; v0 < V; v0 += 4) {
          const float* sl = ring_acquire<NT>(rc, ring, full_bar, err);
          const int nv = min(4, V - v0);
#pragma unroll
          for (int j = 0; j < 4; j += 2) {
            if (j + 1 < nv) {
              float2 tg[3];
#pragma unroll
              for (int c = 0; c < 3; ++c) tg[c] = make_float2(sl[(3 * j + c) * NT + tid], sl[(3 * j + 3 + c) * NT + tid]);
              const float2 cx = *reinterpret_cast<const float2*>(&s_cx[v0 + j]);
              const float2 cy = *reinterpret_cast<const float2*>(&s_cy[v0 + j]);
              const float2 cz = *reinterpret_cast<const float2*>(&s_cz[v0 + j]);
              coloc_view2<LOSS>(tp, cx, cy, cz, PP, tg, ap);
            }
          }
          if (nv & 1) {  // odd last view of the material: lane x only
            const int j = nv - 1;
            float2 tg[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              const float t = sl[(3 * j + c) * NT + tid];
              tg[c] = make_float2(t, t);
            }
            coloc_view2<LOSS, true>(tp, bc2(s_cx[v0 + j]), bc2(s_cy[v0 + j]), bc2(s_cz[v0 + j]), PP, tg, ap);
          }
          ring_release(rc, empty_bar, R);
        }
        AccC a;
        acc_zero(a);
        acc2_fold(ap, a);
        TexelC tc;
        tc.n0 = tp.n0.x; tc.n1 = tp.n1.x; tc.n2 = tp.n2.x;
        float t9[9];
#pragma unroll
        for (int c = 0; c < 9; ++c) t9[c] = fminf(fmaxf(psl[c * NT + tid], -1.0f), 1.0f);
        loss = coloc_finish<LOSS, false>(t9, tc, a, scale, g, gp);
      } else {
        float t9[9];
#pragma unroll
        for (int c = 0; c < 9; ++c) t9[c] = fminf(fmaxf(psl[c * NT + tid], -1.0f), 1.0f);
        Maps m;
        decode(t9, m);
        Adj a;
        adj_zero(a);
        loss = 0.f;
        for (int v0 = 0; v0 < V; v0 += 4) {
          const float* sl = ring_acquire<NT>(rc, ring, full_bar, err);
          const int nv = min(4, V - v0);
          for (int j = 0; j < nv; ++j) {
            float io[3];
            io[0] = sl[(3 * j + 0) * NT + tid];
            io[1] = sl[(3 * j + 1) * NT + tid];
            io[2] = sl[(3 * j + 2) * NT + tid];
            const View& w = s_views[v0 + j];
            if (w.coloc != 0.f) texel_view<kModeFused, LOSS, false, true>(m, px, py, w, s_pow, io, loss, a);
            else texel_view<kModeFused, LOSS, false, false>(m, px, py, w, s_pow, io, loss, a);
          }
          ring_release(rc, empty_bar, R);
        }
        adj_to_params(t9, m, a, scale, g);
      }
      // ---- Adam moments, update, write back
      float m1[9], m2[9];
      {
        const float* sl = ring_acquire<NT>(rc, ring, full_bar, err);
#pragma unroll
        for (int p = 0; p < 9; ++p) m1[p] = sl[p * NT + tid];
        ring_release(rc, empty_bar, R);
      }
      {
        const float* sl = ring_acquire<NT>(rc, ring, full_bar, err);
#pragma unroll
        for (int p = 0; p < 9; ++p) m2[p] = sl[p * NT + tid];
        ring_release(rc, empty_bar, R);
      }
      if (active && rc.ok) {
        float* tex = s_md.tex + idx;
        float* gm1 = s_md.m1 + idx;
        float* gm2 = s_md.m2 + idx;
        const AdamScalars ad = s_adam;
        float pv[9];
#pragma unroll
        for (int c = 0; c < 9; ++c) {
          pv[c] = psl[c * NT + tid];
          g[c] = (pv[c] >= -1.0f && pv[c] <= 1.0f) ? g[c] : 0.0f;  // textures.clamp(-1, 1)
        }
#pragma unroll
        for (int c = 0; c < 8; c += 2) {
          float2 p2 = make_float2(pv[c], pv[c + 1]), a2 = make_float2(m1[c], m1[c + 1]);
          float2 b2 = make_float2(m2[c], m2[c + 1]);
          adam_update2(p2, a2, b2, make_float2(g[c], g[c + 1]), ad);
          pv[c] = p2.x; pv[c + 1] = p2.y; m1[c] = a2.x; m1[c + 1] = a2.y; m2[c] = b2.x; m2[c + 1] = b2.y;
        }
        adam_update(pv[8], m1[8], m2[8], g[8], ad);
#pragma unroll
        for (int c = 0; c < 9; ++c) {
          const int off = c * T;
          tex[off] = pv[c];
          gm1[off] = m1[c];
          gm2[off] = m2[c];
        }
      } else {
        loss = 0.f;
      }
      ring_release_slot(rc, pslot, empty_bar);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, o);
      if (lane == 0) warp_loss[(size_t)tile * NCW + warp] = loss;
    }
  }
  batched_finish<NT + 32>(plan, hdr, mats, warp_loss, NCW, loss_hist, hist_len, s_step, step_counter,
                          ws + kWsCounter, &s_last, NCW);
}

// ============================================================== variant 2: texel pairs
//
// The pipeline of variant 1 with two adjacent texels per consumer thread, so a tile is
// TT = 2 x 32 x NCW texels. Lane x of every FP32x2 value is texel 2i of the tile, lane y
// texel 2i+1: the per-texel set-up, the map-back to the parameters and Adam run packed,
// shared and global accesses are 64-bit, and the co-located view loop steps one view at
// a time for both texels (no odd-view tail). Slots hold 9 planes of TT floats; per tile
// the producer streams
//   P = the 9 parameter planes, Tc = targets of views 3c .. 3c+2, P again, M = exp_avg,
//   S = exp_avg_sq.
// The second copy of P (an L2 hit: the tile's parameters were read a few chunks earlier)
// feeds the map-back and the update, so every slot is released as soon as it has been
// read and the ring never deadlocks, whatever the view count and ring depth.
// Waits, error recording and draining follow variant 1. GEN instantiations also carry the
// general (light off the camera) path; plans whose views are all co-located launch the
// instantiation without it, which keeps its registers for the co-located loop.
constexpr int kPairSlotPlanes = 9;
constexpr int kPairChunkViews = 3;
constexpr size_t kPairRingBudget = 216 * 1024;
// Shapes with at most this many consumer warps run two CTAs per SM, each with half the
// shared memory: two independent pipelines whose phases (MUFU-heavy set-up and map-back,
// FMA-heavy view loop, stores) drift apart and overlap.
constexpr int kPairTwoCtaNcw = 7;
constexpr size_t kPairRingBudgetTwoCta = 104 * 1024;

// ((k + 0.5) / n - 0.5) * size, each operation IEEE round-to-nearest: the pixel-centre grid
// of src/microfacet.py:16-19 exactly as the planner's FP32 coordinate table holds it.
__device__ __forceinline__ float pixel_centre(int k, float n, float size) {
  return __fmul_rn(__fsub_rn(__fdiv_rn(__fadd_rn((float)k, 0.5f), n), 0.5f), size);
}

// Wait (bounded, warp-uniform) for the cursor's slot and return it as float2 pairs.
template <int SLOT>
__device__ __forceinline__ const float2* pair_acquire(RingCursor& rc, const float* ring, uint64_t* full_bar, int* err) {
  if (rc.ok) rc.ok = __all_sync(0xffffffffu, wait_phase(smem_u32(&full_bar[rc.slot]), rc.phase, err, kDevTimeoutFull));
  return reinterpret_cast<const float2*>(ring + (size_t)rc.slot * SLOT);
}

// Record the producer publishes in each ring slot next to its planes (behind the ring in
// dynamic shared memory). P chunks carry the tile and its material, target chunks the views
// of the chunk, so consumers read everything a tile needs from shared memory and never wait
// on one another.
struct __align__(16) PairSlotRec {
  float4 cxy[kPairChunkViews];  // target chunks: (cx, cx, cy, cy) of views 3c .. 3c+2
  float4 czz[kPairChunkViews];  // (cz, cz, 0, 0)
  View view[kPairChunkViews];   // the full views, for the general path
  float* tex;                   // P chunks: the tile's material ...
  float* m1;
  float* m2;
  float* unused;
  int tile, first, W, H;        // ... tile id and first texel
  int V, all_coloc, pad0, pad1;
  float scale, size, inv_w, pad2;
  float P[4];                   // light power
};

template <int LOSS, int NCW, bool GEN>
__global__ void __launch_bounds__((NCW + 1) * 32, NCW <= kPairTwoCtaNcw ? 2 : 1)
batched_pair_kernel(const char* __restrict__ plan, AdamHyper hyper, int* __restrict__ step_counter,
                    float* __restrict__ loss_hist, int hist_len, float* __restrict__ warp_loss, unsigned* ws,
                    float* __restrict__ lpart) {
  constexpr int NT = NCW * 32;
  constexpr int TT = 2 * NT;                  // texels per tile
  constexpr int SLOT = kPairSlotPlanes * TT;  // floats per ring slot
  extern __shared__ __align__(128) float ring[];
  __shared__ __align__(8) uint64_t full_bar[kMaxRing];
  __shared__ __align__(8) uint64_t empty_bar[kMaxRing];
  __shared__ MatDesc s_prod_md;            // the producer's current material ...
  __shared__ View s_prod_views[kMaxViews];  // ... its views
  __shared__ float s_prod_pow[4];           // ... and light power
  __shared__ AdamScalars s_adam;
  __shared__ int s_step;
  __shared__ int s_last;

  const PlanHeader* hdr = (const PlanHeader*)plan;
  const MatDesc* mats = (const MatDesc*)(plan + hdr->off_mats);
  const View* views = (const View*)(plan + hdr->off_views);
  const int* cta_off = (const int*)(plan + hdr->off_cta);
  const int R = hdr->ring_slots;
  PairSlotRec* recs = reinterpret_cast<PairSlotRec*>(ring + (size_t)R * SLOT);
  int* err = (int*)(ws + kWsError);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < R; ++s) {
      mbar_init(smem_u32(&full_bar[s]), 1);
      mbar_init(smem_u32(&empty_bar[s]), NCW);
    }
    fence_mbar_init();
    s_step = *step_counter + 1;
    s_adam = device_adam(hyper, s_step);
  }
  __syncthreads();
  const int k0 = cta_off[blockIdx.x], k1 = cta_off[blockIdx.x + 1];
  const uint32_t ring_base = smem_u32(ring);

  if (warp == NCW) {
    // ------------------------------------------------------------ producer (the whole warp)
    // Lane 0 fills the slot's record and posts the chunk's bytes on its full barrier (a
    // release that publishes the record); lanes 0 .. nplanes-1 then issue one plane copy
    // each. The next tile's entry is loaded one tile ahead and a material's fields and
    // views only when the material changes.
    const int4* seq = (const int4*)(plan + hdr->off_seq);
    int slot = 0;
    uint32_t phase = 0;
    long long issued = 0;
    bool ok = true;
    int4 sq_next = k0 < k1 ? seq[k0] : make_int4(0, 0, 0, 0);
    int cur = -1;
    for (int k = k0; k < k1 && ok; ++k) {
      const int4 sq = sq_next;
      if (k + 1 < k1) sq_next = seq[k + 1];
      if (sq.y != cur) {
        cur = sq.y;
        __syncwarp();
        const MatDesc& m = mats[cur];
        if (lane == 0) s_prod_md = m;
        if (lane < 3) s_prod_pow[lane] = m.lpow[lane];
        for (int v = lane; v < m.V; v += 32) s_prod_views[v] = views[m.view_off + v];
        __syncwarp();
      }
      const MatDesc& md = s_prod_md;
      const int T = md.H * md.W, V = md.V;
      const int first = sq.z;
      const uint32_t bytes = (uint32_t)min(TT, T - first) * 4u;
      const int nt = (V + kPairChunkViews - 1) / kPairChunkViews;
      for (int q = 0; q < nt + 4; ++q) {
        if (issued >= R) {
          ok = __all_sync(0xffffffffu, wait_phase(smem_u32(&empty_bar[slot]), phase ^ 1u, err, kDevTimeoutEmpty));
          if (!ok) break;
        }
        const float* base;
        int plane0, nplanes;
        if (q == 0 || q == nt + 1) { base = md.tex; plane0 = 0; nplanes = 9; }
        else if (q <= nt) {
          base = md.tgt;
          plane0 = 3 * kPairChunkViews * (q - 1);
          nplanes = min(3 * kPairChunkViews, 3 * V - plane0);
        }
        else if (q == nt + 2) { base = md.m1; plane0 = 0; nplanes = 9; }
        else { base = md.m2; plane0 = 0; nplanes = 9; }
        const uint32_t fb = smem_u32(&full_bar[slot]);
        if (lane == 0) {
          PairSlotRec& r = recs[slot];
          if (q == 0 || q >= nt + 1) {  // P, P', M and S chunks carry the tile record
            r.tex = md.tex; r.m1 = md.m1; r.m2 = md.m2;
            r.tile = sq.x; r.first = first; r.W = md.W; r.H = md.H;
            r.V = V; r.all_coloc = md.all_coloc;
            r.scale = md.scale; r.size = md.size; r.inv_w = md.inv_w;
            r.P[0] = s_prod_pow[0]; r.P[1] = s_prod_pow[1]; r.P[2] = s_prod_pow[2];
          } else if (q <= nt) {
            for (int j = 0; j < kPairChunkViews && kPairChunkViews * (q - 1) + j < V; ++j) {
              const View& w = s_prod_views[kPairChunkViews * (q - 1) + j];
              r.cxy[j] = make_float4(w.cx, w.cx, w.cy, w.cy);
              r.czz[j] = make_float4(w.cz, w.cz, 0.f, 0.f);
              r.view[j] = w;
            }
          }
          mbar_arrive_expect_tx(fb, (uint32_t)nplanes * bytes);
        }
        __syncwarp();
        if (lane < nplanes)
          bulk_g2s(ring_base + (uint32_t)(slot * SLOT + lane * TT) * 4u, base + (size_t)(plane0 + lane) * T + first,
                   bytes, fb);
        ++issued;
        if (++slot == R) { slot = 0; phase ^= 1u; }
      }
    }
    if (!ok && lane == 0) {
      // drain: wait for the copies of the last min(R, issued) chunks to land
      const long long n = issued < R ? issued : R;
      int s = slot;
      uint32_t ph = phase;
      for (long long i = 0; i < n; ++i) {
        if (--s < 0) { s = R - 1; ph ^= 1u; }
        uint32_t it = 0;
        while (!mbar_try_wait(smem_u32(&full_bar[s]), ph)) {
          if (++it >= kSpinLimit) { atomicCAS(err, 0, kDevTimeoutDrain); break; }
        }
      }
    }
    __syncwarp();
  } else {
    // ------------------------------------------------------------ consumers
    // A warp whose wait gave up (the error word is set) stops: no barrier among the
    // consumer warps depends on it, and the launch's results are marked invalid.
    const int tid = threadIdx.x;
    RingCursor rc{0, 0u, true};
    for (int k = k0; k < k1; ++k) {
      const float2* pp = pair_acquire<SLOT>(rc, ring, full_bar, err) + tid;
      if (!rc.ok) break;
      const PairSlotRec& r0 = recs[rc.slot];
      const int first = r0.first, W = r0.W, V = r0.V;
      const int T = W * r0.H;
      // T is a multiple of 4 and tiles start at multiples of TT: both texels of a pair
      // are in range or neither is
      const bool active = 2 * tid < T - first;
      const int idx = first + 2 * tid;
      float2 px = make_float2(0.f, 0.f), py = make_float2(0.f, 0.f);
      if (active) {
        int i = (int)((float)idx * r0.inv_w);
        int j = idx - i * W;
        if (j < 0) { --i; j += W; }
        else if (j >= W) { ++i; j -= W; }
        int i1 = i, j1 = j + 1;
        if (j1 == W) { j1 = 0; ++i1; }
        // the planner's coordinate table, recomputed with the same IEEE operations
        const float size = r0.size, fw = (float)W, fh = (float)r0.H;
        px = make_float2(pixel_centre(j, fw, size), pixel_centre(j1, fw, size));
        const float yi = -pixel_centre(i, fh, size);
        py = make_float2(yi, i1 == i ? yi : -pixel_centre(i1, fh, size));
      }
      float2 g[9];
      float2 pv[9];  // raw parameters of the second P copy
      float2 loss2;
      float2 gpl[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};  // dL/d light
      bool live = true;
      if (!GEN || r0.all_coloc) {
        TexelPair u;
        {
          const float P[3] = {r0.P[0], r0.P[1], r0.P[2]};
          float2 t9[9];
#pragma unroll
          for (int c = 0; c < 9; ++c) t9[c] = clamp2(pp[c * NT]);
          ring_release(rc, empty_bar, R);
          coloc_prepare_pair(t9, px, py, P, u);
        }
        AccC2 a;
        acc2_zero(a);
        for (int v0 = 0; v0 < V; v0 += kPairChunkViews) {
          const float2* tp = pair_acquire<SLOT>(rc, ring, full_bar, err) + tid;
          if (!rc.ok) { live = false; break; }
          const PairSlotRec& rv = recs[rc.slot];
          const int nv = min(kPairChunkViews, V - v0);
#pragma unroll
          for (int j = 0; j < kPairChunkViews; ++j) {
            if (j < nv) {
              const float2 tg[3] = {tp[(3 * j) * NT], tp[(3 * j + 1) * NT], tp[(3 * j + 2) * NT]};
              const float4 cxy = rv.cxy[j];
              const float4 czz = rv.czz[j];
              coloc_view_pair<LOSS>(u, make_float2(cxy.x, cxy.y), make_float2(cxy.z, cxy.w),
                                    make_float2(czz.x, czz.y), tg, a);
            }
          }
          ring_release(rc, empty_bar, R);
        }
        if (!live) break;
        const float2* pq = pair_acquire<SLOT>(rc, ring, full_bar, err) + tid;
        if (!rc.ok) break;
        const PairSlotRec& r1 = recs[rc.slot];
        const float P[3] = {r1.P[0], r1.P[1], r1.P[2]};
        const float scale = r1.scale;
#pragma unroll
        for (int c = 0; c < 9; ++c) pv[c] = pq[c * NT];
        ring_release(rc, empty_bar, R);
        float2 t9[9];
#pragma unroll
        for (int c = 0; c < 9; ++c) t9[c] = clamp2(pv[c]);
        loss2 = coloc_finish_pair<LOSS>(t9, u, a, P, scale, g);
        if (lpart) coloc_light_grad_pair<LOSS>(t9, a, scale, gpl);
      } else {
        // general views: the two texels one after the other through each chunk
        const float P[3] = {r0.P[0], r0.P[1], r0.P[2]};
        Maps ma, mb;
        Adj aa, ab;
        {
          float ta[9], tb[9];
#pragma unroll
          for (int c = 0; c < 9; ++c) {
            const float2 t = clamp2(pp[c * NT]);
            ta[c] = t.x;
            tb[c] = t.y;
          }
          ring_release(rc, empty_bar, R);
          decode(ta, ma);
          decode(tb, mb);
        }
        adj_zero(aa);
        adj_zero(ab);
        float la = 0.f, lb = 0.f;
        for (int v0 = 0; v0 < V; v0 += kPairChunkViews) {
          const float2* tp = pair_acquire<SLOT>(rc, ring, full_bar, err) + tid;
          if (!rc.ok) { live = false; break; }
          const PairSlotRec& rv = recs[rc.slot];
          const int nv = min(kPairChunkViews, V - v0);
          for (int j = 0; j < nv; ++j) {
            const float2 t0 = tp[(3 * j) * NT], t1 = tp[(3 * j + 1) * NT], t2 = tp[(3 * j + 2) * NT];
            const View& w = rv.view[j];
            float ia[3] = {t0.x, t1.x, t2.x}, ib[3] = {t0.y, t1.y, t2.y};
            if (w.coloc != 0.f) {
              texel_view<kModeFused, LOSS, true, true>(ma, px.x, py.x, w, P, ia, la, aa);
              texel_view<kModeFused, LOSS, true, true>(mb, px.y, py.y, w, P, ib, lb, ab);
            } else {
              texel_view<kModeFused, LOSS, true, false>(ma, px.x, py.x, w, P, ia, la, aa);
              texel_view<kModeFused, LOSS, true, false>(mb, px.y, py.y, w, P, ib, lb, ab);
            }
          }
          ring_release(rc, empty_bar, R);
        }
        if (!live) break;
        const float2* pq = pair_acquire<SLOT>(rc, ring, full_bar, err) + tid;
        if (!rc.ok) break;
        const float scale = recs[rc.slot].scale;
#pragma unroll
        for (int c = 0; c < 3; ++c) gpl[c] = make_float2(aa.gp[c] * scale, ab.gp[c] * scale);
#pragma unroll
        for (int c = 0; c < 9; ++c) pv[c] = pq[c * NT];
        ring_release(rc, empty_bar, R);
        float ta[9], tb[9], ga[9], gb[9];
#pragma unroll
        for (int c = 0; c < 9; ++c) {
          const float2 t = clamp2(pv[c]);
          ta[c] = t.x;
          tb[c] = t.y;
        }
        adj_to_params(ta, ma, aa, scale, ga);
        adj_to_params(tb, mb, ab, scale, gb);
#pragma unroll
        for (int c = 0; c < 9; ++c) g[c] = make_float2(ga[c], gb[c]);
        loss2 = make_float2(la, lb);
      }
      // ---- Adam moments, update, write back (the destination comes from the S record)
      float2 m1[9], m2[9];
      {
        const float2* sp = pair_acquire<SLOT>(rc, ring, full_bar, err) + tid;
        if (!rc.ok) break;
#pragma unroll
        for (int c = 0; c < 9; ++c) m1[c] = sp[c * NT];
        ring_release(rc, empty_bar, R);
      }
      const float2* sp2 = pair_acquire<SLOT>(rc, ring, full_bar, err) + tid;
      if (!rc.ok) break;
      const PairSlotRec& r3 = recs[rc.slot];
      float* tex = r3.tex + idx;
      float* gm1 = r3.m1 + idx;
      float* gm2 = r3.m2 + idx;
      const int tile = r3.tile;
#pragma unroll
      for (int c = 0; c < 9; ++c) m2[c] = sp2[c * NT];
      ring_release(rc, empty_bar, R);
      float loss = 0.f;
      if (active) {
        const AdamScalars ad = s_adam;
#pragma unroll
        for (int c = 0; c < 9; ++c) {
          float2 p = pv[c];
          // textures.clamp(-1, 1): no gradient outside the range (nor for NaN)
          const float2 gc = make_float2(fabsf(p.x) <= 1.0f ? g[c].x : 0.0f, fabsf(p.y) <= 1.0f ? g[c].y : 0.0f);
          adam_update2(p, m1[c], m2[c], gc, ad);
          const size_t off = (size_t)c * T;
          *reinterpret_cast<float2*>(tex + off) = p;
          *reinterpret_cast<float2*>(gm1 + off) = m1[c];
          *reinterpret_cast<float2*>(gm2 + off) = m2[c];
        }
        loss = loss2.x + loss2.y;
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, o);
      if (lane == 0) warp_loss[(size_t)tile * NCW + warp] = loss;
      if (lpart)
        write_light_partial(lpart, tile, NCW, active ? gpl[0].x + gpl[0].y : 0.f, active ? gpl[1].x + gpl[1].y : 0.f,
                            active ? gpl[2].x + gpl[2].y : 0.f);
    }
  }
  batched_finish<NT + 32>(plan, hdr, mats, warp_loss, NCW, loss_hist, hist_len, s_step, step_counter,
                          ws + kWsCounter, &s_last, NCW, 1, lpart, &s_adam);
}

// ============================================================== variant 3: resident state
//
// Texels are independent across the whole optimisation: a texel's gradient depends only on
// its own parameters and targets, and Adam is elementwise. So one launch can run several
// iterations on a tile before moving on, keeping the tile's parameters and both moments in
// shared memory in between. Per tile the producer copies
//   state = P, M, S (27 planes of TT floats) into a dedicated shared-memory area, then
//   K times: Tc = targets of views 3c .. 3c+2 through the ring (as variant 2),
// and the consumers run K iterations (render, adjoint, Adam) on the resident state, writing
// parameters and moments back to global memory after the last. HBM then carries a tile's
// state and targets once per launch instead of once per iteration; the targets of
// iterations 2 .. K are L2 hits (a tile's targets are at most 16 x 3 x 4 x TT bytes, and
// 152 CTAs keep well under L2 in flight). Per-iteration losses go to per-(iteration, tile,
// warp) partials, so the loss history equals K separate launches'. The state area is
// single-buffered: the producer reloads it once every consumer warp has signalled it done
// with the tile (state_empty), after a proxy fence orders their shared-memory writes before
// the bulk copies. Waits, error recording and draining follow variant 2.
constexpr int kStatePlanes = 27;
constexpr size_t kFuseBudget = 220 * 1024;
constexpr size_t kFuseBudgetTwoCta = 100 * 1024;

// The tile the state area currently holds (written by the producer before it posts the
// state's bytes, read by the consumers after the state barrier completes).
struct __align__(16) FuseStateRec {
  float* tex;
  float* m1;
  float* m2;
  float* unused;
  int tile, first, W, H;
  int V, all_coloc, pad0, pad1;
  float scale, size, inv_w, pad2;
  float P[4];
};

// Pixel centres of consumer thread tid's texel pair (first + 2 tid, first + 2 tid + 1), as
// variant 2 computes them.
__device__ __forceinline__ void pair_coords(const FuseStateRec& r, int tid, float2& px, float2& py) {
  const int W = r.W, idx = r.first + 2 * tid;
  int i = (int)((float)idx * r.inv_w);
  int j = idx - i * W;
  if (j < 0) { --i; j += W; }
  else if (j >= W) { ++i; j -= W; }
  int i1 = i, j1 = j + 1;
  if (j1 == W) { j1 = 0; ++i1; }
  const float size = r.size, fw = (float)W, fh = (float)r.H;
  px = make_float2(pixel_centre(j, fw, size), pixel_centre(j1, fw, size));
  const float yi = -pixel_centre(i, fh, size);
  py = make_float2(yi, i1 == i ? yi : -pixel_centre(i1, fh, size));
}

__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

template <int LOSS, int NCW, bool GEN>
__global__ void __launch_bounds__((NCW + 1) * 32, NCW <= kPairTwoCtaNcw ? 2 : 1)
batched_fuse_kernel(const char* __restrict__ plan, AdamHyper hyper, int* __restrict__ step_counter,
                    float* __restrict__ loss_hist, int hist_len, int iters, float* __restrict__ warp_loss,
                    unsigned* ws, float* __restrict__ lpart) {
  constexpr int NT = NCW * 32;
  constexpr int TT = 2 * NT;                  // texels per tile
  constexpr int SLOT = kPairSlotPlanes * TT;  // floats per ring slot
  constexpr int STATE = kStatePlanes * TT;    // floats of the state area
  extern __shared__ __align__(128) float smem[];
  float* state = smem;
  float* ring = smem + STATE;
  __shared__ __align__(8) uint64_t full_bar[kMaxRing];
  __shared__ __align__(8) uint64_t empty_bar[kMaxRing];
  __shared__ __align__(8) uint64_t state_full;
  __shared__ __align__(8) uint64_t state_empty;
  __shared__ FuseStateRec s_rec;
  __shared__ MatDesc s_prod_md;
  __shared__ View s_prod_views[kMaxViews];
  __shared__ float s_prod_pow[4];
  __shared__ AdamScalars s_adam[kFuseMax];
  __shared__ int s_step;
  __shared__ int s_last;

  const PlanHeader* hdr = (const PlanHeader*)plan;
  const MatDesc* mats = (const MatDesc*)(plan + hdr->off_mats);
  const View* views = (const View*)(plan + hdr->off_views);
  const int* cta_off = (const int*)(plan + hdr->off_cta);
  const int R = hdr->ring_slots;
  const int n_tiles = hdr->n_tiles;
  PairSlotRec* recs = reinterpret_cast<PairSlotRec*>(ring + (size_t)R * SLOT);
  int* err = (int*)(ws + kWsError);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  const int step0 = *step_counter;  // steps step0 + 1 .. step0 + iters
  if (threadIdx.x == 0) {
    for (int s = 0; s < R; ++s) {
      mbar_init(smem_u32(&full_bar[s]), 1);
      mbar_init(smem_u32(&empty_bar[s]), NCW);
    }
    mbar_init(smem_u32(&state_full), 1);
    mbar_init(smem_u32(&state_empty), NCW);
    fence_mbar_init();
    s_step = step0 + iters;
  }
  for (int i = threadIdx.x; i < iters; i += blockDim.x) s_adam[i] = device_adam(hyper, step0 + 1 + i);
  __syncthreads();
  const int k0 = cta_off[blockIdx.x], k1 = cta_off[blockIdx.x + 1];

  if (warp == NCW) {
    // ------------------------------------------------------------ producer (the whole warp)
    const uint32_t ring_base = smem_u32(ring), state_base = smem_u32(state);
    const uint32_t sfull = smem_u32(&state_full), sempty = smem_u32(&state_empty);
    const int4* seq = (const int4*)(plan + hdr->off_seq);
    int slot = 0;
    uint32_t phase = 0, sphase = 0;
    long long issued = 0, states = 0;
    bool ok = true;
    int4 sq_next = k0 < k1 ? seq[k0] : make_int4(0, 0, 0, 0);
    int cur = -1;
    for (int k = k0; k < k1 && ok; ++k) {
      const int4 sq = sq_next;
      if (k + 1 < k1) sq_next = seq[k + 1];
      if (sq.y != cur) {
        cur = sq.y;
        __syncwarp();
        const MatDesc& m = mats[cur];
        if (lane == 0) s_prod_md = m;
        if (lane < 3) s_prod_pow[lane] = m.lpow[lane];
        for (int v = lane; v < m.V; v += 32) s_prod_views[v] = views[m.view_off + v];
        __syncwarp();
      }
      const MatDesc& md = s_prod_md;
      const int T = md.H * md.W, V = md.V;
      const int first = sq.z;
      const uint32_t bytes = (uint32_t)min(TT, T - first) * 4u;
      const int nt = (V + kPairChunkViews - 1) / kPairChunkViews;
      // the state area is free once every consumer warp is done with the previous tile
      if (k > k0) {
        ok = __all_sync(0xffffffffu, wait_phase(sempty, sphase, err, kDevTimeoutEmpty));
        sphase ^= 1u;
        if (!ok) break;
      }
      if (lane == 0) {
        FuseStateRec& r = s_rec;
        r.tex = md.tex; r.m1 = md.m1; r.m2 = md.m2;
        r.tile = sq.x; r.first = first; r.W = md.W; r.H = md.H;
        r.V = V; r.all_coloc = md.all_coloc;
        r.scale = md.scale; r.size = md.size; r.inv_w = md.inv_w;
        r.P[0] = s_prod_pow[0]; r.P[1] = s_prod_pow[1]; r.P[2] = s_prod_pow[2];
        mbar_arrive_expect_tx(sfull, (uint32_t)kStatePlanes * bytes);
      }
      __syncwarp();
      if (lane < kStatePlanes) {
        const float* base = lane < 9 ? md.tex : lane < 18 ? md.m1 : md.m2;
        bulk_g2s(state_base + (uint32_t)(lane * TT) * 4u, base + (size_t)(lane % 9) * T + first, bytes, sfull);
      }
      ++states;
      for (int it = 0; it < iters && ok; ++it) {
        for (int q = 0; q < nt; ++q) {
          if (issued >= R) {
            ok = __all_sync(0xffffffffu, wait_phase(smem_u32(&empty_bar[slot]), phase ^ 1u, err, kDevTimeoutEmpty));
            if (!ok) break;
          }
          const int plane0 = 3 * kPairChunkViews * q;
          const int nplanes = min(3 * kPairChunkViews, 3 * V - plane0);
          const uint32_t fb = smem_u32(&full_bar[slot]);
          if (lane == 0) {
            PairSlotRec& r = recs[slot];
            for (int j = 0; j < kPairChunkViews && kPairChunkViews * q + j < V; ++j) {
              const View& w = s_prod_views[kPairChunkViews * q + j];
              r.cxy[j] = make_float4(w.cx, w.cx, w.cy, w.cy);
              r.czz[j] = make_float4(w.cz, w.cz, 0.f, 0.f);
              r.view[j] = w;
            }
            mbar_arrive_expect_tx(fb, (uint32_t)nplanes * bytes);
          }
          __syncwarp();
          if (lane < nplanes)
            bulk_g2s(ring_base + (uint32_t)(slot * SLOT + lane * TT) * 4u,
                     md.tgt + (size_t)(plane0 + lane) * T + first, bytes, fb);
          ++issued;
          if (++slot == R) { slot = 0; phase ^= 1u; }
        }
      }
    }
    if (!ok && lane == 0) {
      // drain: the last min(R, issued) ring chunks and the last state copy must land
      const long long n = issued < R ? issued : R;
      int s = slot;
      uint32_t ph = phase;
      for (long long i = 0; i < n; ++i) {
        if (--s < 0) { s = R - 1; ph ^= 1u; }
        uint32_t it = 0;
        while (!mbar_try_wait(smem_u32(&full_bar[s]), ph)) {
          if (++it >= kSpinLimit) { atomicCAS(err, 0, kDevTimeoutDrain); break; }
        }
      }
      if (states > 0) {
        uint32_t it = 0;
        while (!mbar_try_wait(sfull, (uint32_t)((states - 1) & 1))) {
          if (++it >= kSpinLimit) { atomicCAS(err, 0, kDevTimeoutDrain); break; }
        }
      }
    }
    __syncwarp();
  } else {
    // ------------------------------------------------------------ consumers
    const int tid = threadIdx.x;
    float2* sw = reinterpret_cast<float2*>(state) + tid;  // plane c at sw[c * NT]
    const float2* sp = sw;
    RingCursor rc{0, 0u, true};
    uint32_t sfp = 0;
    for (int k = k0; k < k1; ++k) {
      if (rc.ok) rc.ok = __all_sync(0xffffffffu, wait_phase(smem_u32(&state_full), sfp, err, kDevTimeoutFull));
      sfp ^= 1u;
      if (!rc.ok) break;
      // The tile's fields are read from the shared record where they are used (it stays put
      // until this warp signals state_empty), which keeps them out of registers in the loop.
      const FuseStateRec& r0 = s_rec;
      const int V = r0.V;
      const bool coloc = !GEN || r0.all_coloc;
      const bool active = 2 * tid < r0.W * r0.H - r0.first;
      bool live = true;
      // the pair's pixel centres, once per tile (they do not change across its iterations)
      float2 px = make_float2(0.f, 0.f), py = make_float2(0.f, 0.f);
      if (active) pair_coords(r0, tid, px, py);
      for (int it = 0; it < iters; ++it) {
        float2 g[9];
        float2 loss2;
        float2 gpl[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};  // dL/d light
        if (coloc) {
          TexelPair u;
          {
            const float P[3] = {r0.P[0], r0.P[1], r0.P[2]};
            float2 t9[9];
#pragma unroll
            for (int c = 0; c < 9; ++c) t9[c] = clamp2(sp[c * NT]);
            coloc_prepare_pair(t9, px, py, P, u);
          }
          AccC2 a;
          acc2_zero(a);
          for (int v0 = 0; v0 < V; v0 += kPairChunkViews) {
            const float2* tp = pair_acquire<SLOT>(rc, ring, full_bar, err) + tid;
            if (!rc.ok) { live = false; break; }
            const PairSlotRec& rv = recs[rc.slot];
            const int nv = min(kPairChunkViews, V - v0);
#pragma unroll
            for (int j = 0; j < kPairChunkViews; ++j) {
              if (j < nv) {
                const float2 tg[3] = {tp[(3 * j) * NT], tp[(3 * j + 1) * NT], tp[(3 * j + 2) * NT]};
                const float4 cxy = rv.cxy[j];
                const float4 czz = rv.czz[j];
                coloc_view_pair<LOSS>(u, make_float2(cxy.x, cxy.y), make_float2(cxy.z, cxy.w),
                                      make_float2(czz.x, czz.y), tg, a);
              }
            }
            ring_release(rc, empty_bar, R);
          }
          if (!live) break;
          float2 t9[9];
#pragma unroll
          for (int c = 0; c < 9; ++c) t9[c] = clamp2(sp[c * NT]);
          const float P[3] = {r0.P[0], r0.P[1], r0.P[2]};
          loss2 = coloc_finish_pair<LOSS>(t9, u, a, P, r0.scale, g);
          if (lpart) coloc_light_grad_pair<LOSS>(t9, a, r0.scale, gpl);
        } else {
          // general views: the two texels one after the other through each chunk
          const float P[3] = {r0.P[0], r0.P[1], r0.P[2]};
          Maps ma, mb;
          Adj aa, ab;
          {
            float ta[9], tb[9];
#pragma unroll
            for (int c = 0; c < 9; ++c) {
              const float2 t = clamp2(sp[c * NT]);
              ta[c] = t.x;
              tb[c] = t.y;
            }
            decode(ta, ma);
            decode(tb, mb);
          }
          adj_zero(aa);
          adj_zero(ab);
          float la = 0.f, lb = 0.f;
          for (int v0 = 0; v0 < V; v0 += kPairChunkViews) {
            const float2* tp = pair_acquire<SLOT>(rc, ring, full_bar, err) + tid;
            if (!rc.ok) { live = false; break; }
            const PairSlotRec& rv = recs[rc.slot];
            const int nv = min(kPairChunkViews, V - v0);
            for (int j = 0; j < nv; ++j) {
              const float2 t0 = tp[(3 * j) * NT], t1 = tp[(3 * j + 1) * NT], t2 = tp[(3 * j + 2) * NT];
              const View& w = rv.view[j];
              float ia[3] = {t0.x, t1.x, t2.x}, ib[3] = {t0.y, t1.y, t2.y};
              if (w.coloc != 0.f) {
                texel_view<kModeFused, LOSS, true, true>(ma, px.x, py.x, w, P, ia, la, aa);
                texel_view<kModeFused, LOSS, true, true>(mb, px.y, py.y, w, P, ib, lb, ab);
              } else {
                texel_view<kModeFused, LOSS, true, false>(ma, px.x, py.x, w, P, ia, la, aa);
                texel_view<kModeFused, LOSS, true, false>(mb, px.y, py.y, w, P, ib, lb, ab);
              }
            }
            ring_release(rc, empty_bar, R);
          }
          if (!live) break;
#pragma unroll
          for (int c = 0; c < 3; ++c) gpl[c] = make_float2(aa.gp[c] * r0.scale, ab.gp[c] * r0.scale);
          float ta[9], tb[9], ga[9], gb[9];
#pragma unroll
          for (int c = 0; c < 9; ++c) {
            const float2 t = clamp2(sp[c * NT]);
            ta[c] = t.x;
            tb[c] = t.y;
          }
          adj_to_params(ta, ma, aa, r0.scale, ga);
          adj_to_params(tb, mb, ab, r0.scale, gb);
#pragma unroll
          for (int c = 0; c < 9; ++c) g[c] = make_float2(ga[c], gb[c]);
          loss2 = make_float2(la, lb);
        }
        // ---- Adam on the resident state; the last iteration writes to global memory
        float loss = 0.f;
        if (active) {
          const AdamScalars ad = s_adam[it];
          const bool last = it + 1 == iters;
          const int T = r0.W * r0.H, idx = r0.first + 2 * tid;
          float* tex = r0.tex;
          float* gm1 = r0.m1;
          float* gm2 = r0.m2;
#pragma unroll
          for (int c = 0; c < 9; ++c) {
            float2 p = sp[c * NT], m1 = sp[(9 + c) * NT], m2 = sp[(18 + c) * NT];
            // textures.clamp(-1, 1): no gradient outside the range (nor for NaN)
            const float2 gc = make_float2(fabsf(p.x) <= 1.0f ? g[c].x : 0.0f, fabsf(p.y) <= 1.0f ? g[c].y : 0.0f);
            adam_update2(p, m1, m2, gc, ad);
            if (last) {
              const size_t off = (size_t)c * T + idx;
              *reinterpret_cast<float2*>(tex + off) = p;
              *reinterpret_cast<float2*>(gm1 + off) = m1;
              *reinterpret_cast<float2*>(gm2 + off) = m2;
            } else {
              sw[c * NT] = p;
              sw[(9 + c) * NT] = m1;
              sw[(18 + c) * NT] = m2;
            }
          }
          loss = loss2.x + loss2.y;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, o);
        if (lane == 0) warp_loss[((size_t)it * n_tiles + r0.tile) * NCW + warp] = loss;
        if (lpart)  // plans with a learnable light run one iteration per launch
          write_light_partial(lpart, r0.tile, NCW, active ? gpl[0].x + gpl[0].y : 0.f,
                              active ? gpl[1].x + gpl[1].y : 0.f, active ? gpl[2].x + gpl[2].y : 0.f);
      }
      if (!live) break;
      // this warp's shared-memory writes come before the next tile's bulk copies into the area
      fence_proxy_async_smem();
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_u32(&state_empty));
    }
  }
  batched_finish<NT + 32>(plan, hdr, mats, warp_loss, NCW, loss_hist, hist_len, s_step, step_counter,
                          ws + kWsCounter, &s_last, NCW, iters, lpart, &s_adam[0]);
}

// ============================================================== variant 4: resident state, no producer
//
// Variant 3's schedule without a producer warp: every warp computes, and the copies are
// issued by whichever warp finishes with a buffer last.
//   * Ring: a warp that has read a target chunk counts itself out of its slot with a
//     shared-memory atomic; the last of the NCW warps refills the slot with the chunk R
//     positions later in the CTA's chunk sequence (tile by tile: K iterations x
//     ceil(V/3) chunks), found by walking the tile list forward from its own position.
//   * State: the last warp to finish a tile copies the next tile's state and record.
// Warp 0 issues the first tile's state and the first R chunks. Sixteen compute warps fill
// the four sub-partitions evenly (variant 3 has fifteen beside the producer), and the
// 256-thread shape runs two independent CTAs per SM. Each warp orders its shared-memory
// reads (and its state writes) before the copies that overwrite them with a CTA fence before
// its count and, in the refilling warp, an async-proxy fence before the copy. Waits are
// bounded as in the other variants; a CTA whose warps gave up drains every copy it issued
// before returning.
constexpr int kFuse2TwoCtaNcw = 8;
constexpr size_t kFuse2Budget = 220 * 1024;
constexpr size_t kFuse2BudgetTwoCta = 100 * 1024;

// Position `steps` chunks after local chunk l of CTA tile k (tiles k .. k1-1 in schedule
// order, iters x ceil(V/3) chunks each). False past the CTA's last chunk.
__device__ __forceinline__ bool fuse_walk(const int4* seq, const MatDesc* mats, int k, int l, int steps, int k1,
                                          int iters, int& kout, int& lout) {
  int rem = l + steps;
  while (k < k1) {
    const int n = iters * ((mats[seq[k].y].V + kPairChunkViews - 1) / kPairChunkViews);
    if (rem < n) {
      kout = k;
      lout = rem;
      return true;
    }
    rem -= n;
    ++k;
  }
  return false;
}

// Whole warp: target chunk l of CTA tile k into ring slot `slot`.
template <int TT>
__device__ __forceinline__ void fuse_issue_chunk(const int4* seq, const MatDesc* mats, const View* views, int k, int l,
                                                 int slot, uint32_t ring_base, PairSlotRec* recs, uint64_t* full_bar,
                                                 int* issue_cnt) {
  constexpr int SLOT = kPairSlotPlanes * TT;
  const int lane = threadIdx.x & 31;
  const int4 sq = seq[k];
  const MatDesc& md = mats[sq.y];
  const int V = md.V, T = md.H * md.W, first = sq.z;
  const int nt = (V + kPairChunkViews - 1) / kPairChunkViews;
  const int q = l % nt;
  const uint32_t bytes = (uint32_t)min(TT, T - first) * 4u;
  const int plane0 = 3 * kPairChunkViews * q;
  const int nplanes = min(3 * kPairChunkViews, 3 * V - plane0);
  const uint32_t fb = smem_u32(&full_bar[slot]);
  if (lane == 0) {
    PairSlotRec& r = recs[slot];
    for (int j = 0; j < kPairChunkViews && kPairChunkViews * q + j < V; ++j) {
      const View w = views[md.view_off + kPairChunkViews * q + j];
      r.cxy[j] = make_float4(w.cx, w.cx, w.cy, w.cy);
      r.czz[j] = make_float4(w.cz, w.cz, 0.f, 0.f);
      r.view[j] = w;
    }
    ++issue_cnt[slot];
    mbar_arrive_expect_tx(fb, (uint32_t)nplanes * bytes);
  }
  __syncwarp();
  if (lane < nplanes)
    bulk_g2s(ring_base + (uint32_t)(slot * SLOT + lane * TT) * 4u, md.tgt + (size_t)(plane0 + lane) * T + first,
             bytes, fb);
}

// Whole warp: the state (parameters, exp_avg, exp_avg_sq) and record of CTA tile k.
template <int TT>
__device__ __forceinline__ void fuse_issue_state(const int4* seq, const MatDesc* mats, int k, uint32_t state_base,
                                                 FuseStateRec* rec, uint64_t* state_full, int* state_cnt) {
  const int lane = threadIdx.x & 31;
  const int4 sq = seq[k];
  const MatDesc& md = mats[sq.y];
  const int T = md.H * md.W, first = sq.z;
  const uint32_t bytes = (uint32_t)min(TT, T - first) * 4u;
  const uint32_t sfull = smem_u32(state_full);
  if (lane == 0) {
    rec->tex = md.tex; rec->m1 = md.m1; rec->m2 = md.m2;
    rec->tile = sq.x; rec->first = first; rec->W = md.W; rec->H = md.H;
    rec->V = md.V; rec->all_coloc = md.all_coloc;
    rec->scale = md.scale; rec->size = md.size; rec->inv_w = md.inv_w;
    rec->P[0] = md.lpow[0]; rec->P[1] = md.lpow[1]; rec->P[2] = md.lpow[2];
    ++*state_cnt;
    mbar_arrive_expect_tx(sfull, (uint32_t)kStatePlanes * bytes);
  }
  __syncwarp();
  if (lane < kStatePlanes) {
    const float* base = lane < 9 ? md.tex : lane < 18 ? md.m1 : md.m2;
    bulk_g2s(state_base + (uint32_t)(lane * TT) * 4u, base + (size_t)(lane % 9) * T + first, bytes, sfull);
  }
}

// Whole warp: count this warp out of a buffer; true in the one warp that counted last
// (the counter is reset for the buffer's next use). The CTA fence orders the warp's reads
// and writes of the buffer before its count.
__device__ __forceinline__ bool fuse_count_out(int* cnt, int nwarps) {
  __syncwarp();
  int old = 0;
  if ((threadIdx.x & 31) == 0) {
    __threadfence_block();
    old = atomicAdd(cnt, 1);
    if (old == nwarps - 1) {
      __threadfence_block();  // with the other warps' fence-then-count: their accesses happen before ours
      *cnt = 0;
    }
  }
  old = __shfl_sync(0xffffffffu, old, 0);
  return old == nwarps - 1;
}

template <int LOSS, int NCW, bool GEN>
__global__ void __launch_bounds__(NCW * 32, NCW <= kFuse2TwoCtaNcw ? 2 : 1)
batched_fuse2_kernel(const char* __restrict__ plan, AdamHyper hyper, int* __restrict__ step_counter,
                     float* __restrict__ loss_hist, int hist_len, int iters, float* __restrict__ warp_loss,
                     unsigned* ws) {
  constexpr int NT = NCW * 32;
  constexpr int TT = 2 * NT;                  // texels per tile
  constexpr int SLOT = kPairSlotPlanes * TT;  // floats per ring slot
  constexpr int STATE = kStatePlanes * TT;    // floats of the state area
  extern __shared__ __align__(128) float smem[];
  float* state = smem;
  float* ring = smem + STATE;
  __shared__ __align__(8) uint64_t full_bar[kMaxRing];
  __shared__ __align__(8) uint64_t state_full;
  __shared__ int rel_cnt[kMaxRing];
  __shared__ int issue_cnt[kMaxRing];
  __shared__ int st_rel;
  __shared__ int st_issued;
  __shared__ FuseStateRec s_rec;
  __shared__ AdamScalars s_adam[kFuseMax];
  __shared__ int s_step;
  __shared__ int s_last;

  const PlanHeader* hdr = (const PlanHeader*)plan;
  const MatDesc* mats = (const MatDesc*)(plan + hdr->off_mats);
  const View* views = (const View*)(plan + hdr->off_views);
  const int* cta_off = (const int*)(plan + hdr->off_cta);
  const int4* seq = (const int4*)(plan + hdr->off_seq);
  const int R = hdr->ring_slots;
  const int n_tiles = hdr->n_tiles;
  PairSlotRec* recs = reinterpret_cast<PairSlotRec*>(ring + (size_t)R * SLOT);
  int* err = (int*)(ws + kWsError);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, tid = threadIdx.x;
  const uint32_t ring_base = smem_u32(ring), state_base = smem_u32(state);

  const int step0 = *step_counter;  // steps step0 + 1 .. step0 + iters
  if (threadIdx.x == 0) {
    for (int s = 0; s < R; ++s) {
      mbar_init(smem_u32(&full_bar[s]), 1);
      rel_cnt[s] = 0;
      issue_cnt[s] = 0;
    }
    mbar_init(smem_u32(&state_full), 1);
    st_rel = 0;
    st_issued = 0;
    fence_mbar_init();
    s_step = step0 + iters;
  }
  for (int i = threadIdx.x; i < iters; i += blockDim.x) s_adam[i] = device_adam(hyper, step0 + 1 + i);
  __syncthreads();
  const int k0 = cta_off[blockIdx.x], k1 = cta_off[blockIdx.x + 1];
  if (warp == 0 && k0 < k1) {
    fuse_issue_state<TT>(seq, mats, k0, state_base, &s_rec, &state_full, &st_issued);
    for (int c = 0; c < R; ++c) {
      int kk, ll;
      if (!fuse_walk(seq, mats, k0, 0, c, k1, iters, kk, ll)) break;
      fuse_issue_chunk<TT>(seq, mats, views, kk, ll, c, ring_base, recs, full_bar, issue_cnt);
    }
  }

  const float2* sp = reinterpret_cast<const float2*>(state) + tid;  // plane c at sp[c * NT]
  float2* sw = reinterpret_cast<float2*>(state) + tid;
  RingCursor rc{0, 0u, true};
  uint32_t sfp = 0;
  for (int k = k0; k < k1; ++k) {
    if (rc.ok) rc.ok = __all_sync(0xffffffffu, wait_phase(smem_u32(&state_full), sfp, err, kDevTimeoutFull));
    sfp ^= 1u;
    if (!rc.ok) break;
    const FuseStateRec& r0 = s_rec;
    const int V = r0.V;
    const int nt = (V + kPairChunkViews - 1) / kPairChunkViews;
    const bool coloc = !GEN || r0.all_coloc;
    const bool active = 2 * tid < r0.W * r0.H - r0.first;
    bool live = true;
    for (int it = 0; it < iters; ++it) {
      float2 g[9];
      float2 loss2;
      float2 px = make_float2(0.f, 0.f), py = make_float2(0.f, 0.f);
      if (active) pair_coords(r0, tid, px, py);
      if (coloc) {
        TexelPair u;
        {
          const float P[3] = {r0.P[0], r0.P[1], r0.P[2]};
          float2 t9[9];
#pragma unroll
          for (int c = 0; c < 9; ++c) t9[c] = clamp2(sp[c * NT]);
          coloc_prepare_pair(t9, px, py, P, u);
        }
        AccC2 a;
        acc2_zero(a);
        for (int qq = 0; qq < nt; ++qq) {
          const float2* tp = pair_acquire<SLOT>(rc, ring, full_bar, err) + tid;
          if (!rc.ok) { live = false; break; }
          const PairSlotRec& rv = recs[rc.slot];
          const int nv = min(kPairChunkViews, V - kPairChunkViews * qq);
#pragma unroll
          for (int j = 0; j < kPairChunkViews; ++j) {
            if (j < nv) {
              const float2 tg[3] = {tp[(3 * j) * NT], tp[(3 * j + 1) * NT], tp[(3 * j + 2) * NT]};
              const float4 cxy = rv.cxy[j];
              const float4 czz = rv.czz[j];
              coloc_view_pair<LOSS>(u, make_float2(cxy.x, cxy.y), make_float2(cxy.z, cxy.w),
                                    make_float2(czz.x, czz.y), tg, a);
            }
          }
          if (fuse_count_out(&rel_cnt[rc.slot], NCW)) {
            int kk, ll;
            if (fuse_walk(seq, mats, k, it * nt + qq, R, k1, iters, kk, ll)) {
              fence_proxy_async_smem();
              fuse_issue_chunk<TT>(seq, mats, views, kk, ll, rc.slot, ring_base, recs, full_bar, issue_cnt);
            }
          }
          if (++rc.slot == R) { rc.slot = 0; rc.phase ^= 1u; }
        }
        if (!live) break;
        float2 t9[9];
#pragma unroll
        for (int c = 0; c < 9; ++c) t9[c] = clamp2(sp[c * NT]);
        const float P[3] = {r0.P[0], r0.P[1], r0.P[2]};
        loss2 = coloc_finish_pair<LOSS>(t9, u, a, P, r0.scale, g);
      } else {
        const float P[3] = {r0.P[0], r0.P[1], r0.P[2]};
        Maps ma, mb;
        Adj aa, ab;
        {
          float ta[9], tb[9];
#pragma unroll
          for (int c = 0; c < 9; ++c) {
            const float2 t = clamp2(sp[c * NT]);
            ta[c] = t.x;
            tb[c] = t.y;
          }
          decode(ta, ma);
          decode(tb, mb);
        }
        adj_zero(aa);
        adj_zero(ab);
        float la = 0.f, lb = 0.f;
        for (int qq = 0; qq < nt; ++qq) {
          const float2* tp = pair_acquire<SLOT>(rc, ring, full_bar, err) + tid;
          if (!rc.ok) { live = false; break; }
          const PairSlotRec& rv = recs[rc.slot];
          const int nv = min(kPairChunkViews, V - kPairChunkViews * qq);
          for (int j = 0; j < nv; ++j) {
            const float2 t0 = tp[(3 * j) * NT], t1 = tp[(3 * j + 1) * NT], t2 = tp[(3 * j + 2) * NT];
            const View& w = rv.view[j];
            float ia[3] = {t0.x, t1.x, t2.x}, ib[3] = {t0.y, t1.y, t2.y};
            if (w.coloc != 0.f) {
              texel_view<kModeFused, LOSS, false, true>(ma, px.x, py.x, w, P, ia, la, aa);
              texel_view<kModeFused, LOSS, false, true>(mb, px.y, py.y, w, P, ib, lb, ab);
            } else {
              texel_view<kModeFused, LOSS, false, false>(ma, px.x, py.x, w, P, ia, la, aa);
              texel_view<kModeFused, LOSS, false, false>(mb, px.y, py.y, w, P, ib, lb, ab);
            }
          }
          if (fuse_count_out(&rel_cnt[rc.slot], NCW)) {
            int kk, ll;
            if (fuse_walk(seq, mats, k, it * nt + qq, R, k1, iters, kk, ll)) {
              fence_proxy_async_smem();
              fuse_issue_chunk<TT>(seq, mats, views, kk, ll, rc.slot, ring_base, recs, full_bar, issue_cnt);
            }
          }
          if (++rc.slot == R) { rc.slot = 0; rc.phase ^= 1u; }
        }
        if (!live) break;
        float ta[9], tb[9], ga[9], gb[9];
#pragma unroll
        for (int c = 0; c < 9; ++c) {
          const float2 t = clamp2(sp[c * NT]);
          ta[c] = t.x;
          tb[c] = t.y;
        }
        adj_to_params(ta, ma, aa, r0.scale, ga);
        adj_to_params(tb, mb, ab, r0.scale, gb);
#pragma unroll
        for (int c = 0; c < 9; ++c) g[c] = make_float2(ga[c], gb[c]);
        loss2 = make_float2(la, lb);
      }
      float loss = 0.f;
      if (active) {
        const AdamScalars ad = s_adam[it];
        const bool last = it + 1 == iters;
        const int T = r0.W * r0.H, idx = r0.first + 2 * tid;
        float* tex = r0.tex;
        float* gm1 = r0.m1;
        float* gm2 = r0.m2;
#pragma unroll
        for (int c = 0; c < 9; ++c) {
          float2 p = sp[c * NT], m1 = sp[(9 + c) * NT], m2 = sp[(18 + c) * NT];
          const float2 gc = make_float2(fabsf(p.x) <= 1.0f ? g[c].x : 0.0f, fabsf(p.y) <= 1.0f ? g[c].y : 0.0f);
          adam_update2(p, m1, m2, gc, ad);
          if (last) {
            const size_t off = (size_t)c * T + idx;
            *reinterpret_cast<float2*>(tex + off) = p;
            *reinterpret_cast<float2*>(gm1 + off) = m1;
            *reinterpret_cast<float2*>(gm2 + off) = m2;
          } else {
            sw[c * NT] = p;
            sw[(9 + c) * NT] = m1;
            sw[(18 + c) * NT] = m2;
          }
        }
        loss = loss2.x + loss2.y;
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, o);
      if (lane == 0) warp_loss[((size_t)it * n_tiles + r0.tile) * NCW + warp] = loss;
    }
    if (!live) break;
    // this warp's state writes come before the next tile's bulk copies into the area
    fence_proxy_async_smem();
    if (fuse_count_out(&st_rel, NCW) && k + 1 < k1) {
      fence_proxy_async_smem();
      fuse_issue_state<TT>(seq, mats, k + 1, state_base, &s_rec, &state_full, &st_issued);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && *(volatile int*)err != 0) {
    // drain: every copy this CTA issued must land before the CTA's shared memory goes away
    for (int s = 0; s < R; ++s) {
      if (issue_cnt[s] == 0) continue;
      uint32_t it = 0;
      while (!mbar_try_wait(smem_u32(&full_bar[s]), (uint32_t)((issue_cnt[s] - 1) & 1))) {
        if (++it >= kSpinLimit) { atomicCAS(err, 0, kDevTimeoutDrain); break; }
      }
    }
    if (st_issued > 0) {
      uint32_t it = 0;
      while (!mbar_try_wait(smem_u32(&state_full), (uint32_t)((st_issued - 1) & 1))) {
        if (++it >= kSpinLimit) { atomicCAS(err, 0, kDevTimeoutDrain); break; }
      }
    }
  }
  batched_finish<NT>(plan, hdr, mats, warp_loss, NCW, loss_hist, hist_len, s_step, step_counter,
                     ws + kWsCounter, &s_last, NCW, iters);
}

// ============================================================== wait self-test
// The failure path of every bounded wait, exercised on purpose: one warp waits on a barrier
// phase that its own arrival completes (the healthy path), then on a barrier that nothing
// ever arrives on, giving up after `limit` polls. It records kDevTimeoutFull in the error
// word and returns; no copy is in flight, so the context stays usable. ws[2] and ws[3] report
// the two waits' outcomes (1 = completed).
__global__ void __launch_bounds__(32) wait_selftest_kernel(unsigned* ws, uint32_t limit) {
  __shared__ __align__(8) uint64_t bar_done, bar_never;
  if (threadIdx.x == 0) {
    mbar_init(smem_u32(&bar_done), 1);
    mbar_init(smem_u32(&bar_never), 1);
    fence_mbar_init();
  }
  __syncwarp();
  int* err = (int*)(ws + kWsError);
  if (threadIdx.x == 0) mbar_arrive(smem_u32(&bar_done));
  __syncwarp();
  const bool done = __all_sync(0xffffffffu, wait_phase_n(smem_u32(&bar_done), 0u, err, kDevTimeoutFull, limit));
  const bool never = __all_sync(0xffffffffu, wait_phase_n(smem_u32(&bar_never), 0u, err, kDevTimeoutFull, limit));
  if (threadIdx.x == 0) {
    ws[2] = done ? 1u : 0u;
    ws[3] = never ? 1u : 0u;
  }
}

// ============================================================== planner
static size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

struct PlanLayout {
  size_t off_mats, off_views, off_cta, off_order, off_tiles, off_mat_tiles, off_coords, off_seq, total;
  int n_tiles, n_ctas, total_views, ring;
  long long coord_floats;
};

int resident_ctas(int variant, int threads);

static int slot_bytes(int threads) { return kSlotPlanes * threads * 4; }
static int pair_slot_bytes(int threads) { return kPairSlotPlanes * 2 * threads * 4 + (int)sizeof(PairSlotRec); }
static size_t pair_ring_budget(int threads) {
  return threads / 32 <= kPairTwoCtaNcw ? kPairRingBudgetTwoCta : kPairRingBudget;
}
// variant 3: the state area (27 planes of the tile) comes out of the budget first
static size_t fuse_state_bytes(int threads) { return (size_t)kStatePlanes * 2 * threads * 4; }
static int fuse_ring(int threads, int variant) {
  const bool two = variant == 4 ? threads / 32 <= kFuse2TwoCtaNcw : threads / 32 <= kPairTwoCtaNcw;
  const size_t budget = variant == 4 ? (two ? kFuse2BudgetTwoCta : kFuse2Budget) : (two ? kFuseBudgetTwoCta : kFuseBudget);
  const size_t state = fuse_state_bytes(threads);
  if (state >= budget) return 0;
  return (int)std::min<size_t>(kMaxRing, (budget - state) / pair_slot_bytes(threads));
}

static int plan_layout(const svbrdf_material* mats, int n, const svbrdf_batch_config* cfg, PlanLayout& L) {
  if (!mats || n <= 0) return fail(SVBRDF_ERR_INVALID, "no materials");
  if (!cfg) return fail(SVBRDF_ERR_INVALID, "null config");
  const int variant = cfg->variant;
  if (variant < 0 || variant > 4) return fail(SVBRDF_ERR_INVALID, "variant must be 0 .. 4 (got %d)", variant);
  if (variant == 0) {
    if (cfg->threads != 128 && cfg->threads != 256 && cfg->threads != 512)
      return fail(SVBRDF_ERR_UNSUPPORTED, "threads must be 128, 256 or 512 (got %d)", cfg->threads);
    if (cfg->tile_texels <= 0 || cfg->tile_texels % cfg->threads)
      return fail(SVBRDF_ERR_INVALID, "tile_texels must be a positive multiple of threads");
  } else {
    if (variant == 1 && cfg->threads != 256 && cfg->threads != 384 && cfg->threads != 480 && cfg->threads != 608)
      return fail(SVBRDF_ERR_UNSUPPORTED, "pipelined variant: threads must be 256, 384, 480 or 608 (got %d)",
                  cfg->threads);
    if (variant == 1 && cfg->tile_texels != cfg->threads)
      return fail(SVBRDF_ERR_INVALID, "pipelined variant: tile_texels must equal threads");
    if (variant == 2 && cfg->threads != 224 && cfg->threads != 256 && cfg->threads != 384 && cfg->threads != 480 &&
        cfg->threads != 608)
      return fail(SVBRDF_ERR_UNSUPPORTED, "texel-pair variant: threads must be 224, 256, 384, 480 or 608 (got %d)",
                  cfg->threads);
    if (variant == 2 && cfg->tile_texels != 2 * cfg->threads)
      return fail(SVBRDF_ERR_INVALID, "texel-pair variant: tile_texels must be twice threads");
    if (variant == 3 && cfg->threads != 224 && cfg->threads != 256 && cfg->threads != 384 && cfg->threads != 480)
      return fail(SVBRDF_ERR_UNSUPPORTED, "resident-state variant: threads must be 224, 256, 384 or 480 (got %d)",
                  cfg->threads);
    if (variant == 3 && cfg->tile_texels != 2 * cfg->threads)
      return fail(SVBRDF_ERR_INVALID, "resident-state variant: tile_texels must be twice threads");
    if (variant == 4 && cfg->threads != 256 && cfg->threads != 512)
      return fail(SVBRDF_ERR_UNSUPPORTED, "producer-less resident-state variant: threads must be 256 or 512 (got %d)",
                  cfg->threads);
    if (variant == 4 && cfg->tile_texels != 2 * cfg->threads)
      return fail(SVBRDF_ERR_INVALID, "producer-less resident-state variant: tile_texels must be twice threads");
  }
  long long tiles = 0, coords = 0;
  int views = 0, max_views = 0;
  for (int i = 0; i < n; ++i) {
    const svbrdf_material& m = mats[i];
    if (!m.textures || !m.exp_avg || !m.exp_avg_sq || !m.targets || !m.light_pow || !m.camera_pos || !m.light_pos)
      return fail(SVBRDF_ERR_INVALID, "material %d has a null pointer", i);
    if (m.n_views <= 0 || m.height <= 0 || m.width <= 0 || !(m.size > 0.f))
      return fail(SVBRDF_ERR_INVALID, "material %d has a bad shape", i);
    if (m.n_views > kMaxViews) return fail(SVBRDF_ERR_UNSUPPORTED, "material %d: too many views", i);
    if (m.light_adam_state && variant != 2 && variant != 3)
      return fail(SVBRDF_ERR_UNSUPPORTED, "material %d: a learnable light power needs variant 2 or 3 (got %d)", i,
                  variant);
    const long long T = (long long)m.height * m.width;
    if (T >= (1LL << 24)) return fail(SVBRDF_ERR_UNSUPPORTED, "material %d: more than 2^24 texels", i);
    if (variant >= 1) {
      if (T % 4) return fail(SVBRDF_ERR_UNSUPPORTED, "pipelined variant: material %d H*W must be a multiple of 4", i);
      const void* ptrs[4] = {m.textures, m.exp_avg, m.exp_avg_sq, m.targets};
      for (const void* p : ptrs)
        if ((uintptr_t)p % 16) return fail(SVBRDF_ERR_UNSUPPORTED, "pipelined variant: material %d not 16-byte aligned", i);
    }
    tiles += (T + cfg->tile_texels - 1) / cfg->tile_texels;
    views += m.n_views;
    max_views = std::max(max_views, m.n_views);
    coords += m.width + m.height;
  }
  if (tiles > (1LL << 30)) return fail(SVBRDF_ERR_UNSUPPORTED, "too many tiles");
  int ctas = cfg->ctas > 0 ? cfg->ctas : resident_ctas(variant, cfg->threads);
  if (ctas <= 0) return fail(SVBRDF_ERR_CUDA, "could not query the device");
  if (ctas > tiles) ctas = (int)tiles;
  L.n_tiles = (int)tiles;
  L.n_ctas = ctas;
  L.total_views = views;
  L.coord_floats = coords;
  L.ring = variant == 1   ? (int)std::min<size_t>(kMaxRing, kRingBudget / slot_bytes(cfg->threads))
           : variant == 2 ? (int)std::min<size_t>(kMaxRing, pair_ring_budget(cfg->threads) / pair_slot_bytes(cfg->threads))
           : variant >= 3 ? fuse_ring(cfg->threads, variant)
                          : 0;
  if (variant >= 3 && L.ring < 2)
    return fail(SVBRDF_ERR_UNSUPPORTED, "resident-state variant: %d threads leave room for %d ring slots", cfg->threads,
                L.ring);
  // variant 1 holds a tile's parameter slot until its last chunk (S) has been read, so
  // all 3 + ceil(V/4) chunks of a tile must fit in the ring at once
  if (variant == 1 && 3 + (max_views + 3) / 4 > L.ring)
    return fail(SVBRDF_ERR_UNSUPPORTED, "pipelined variant: %d views need %d ring slots; %d threads leave room for %d",
                max_views, 3 + (max_views + 3) / 4, cfg->threads, L.ring);
  size_t o = align_up(sizeof(PlanHeader), 16);
  L.off_mats = o; o += sizeof(MatDesc) * n; o = align_up(o, 16);
  L.off_views = o; o += sizeof(View) * views; o = align_up(o, 16);
  L.off_cta = o; o += sizeof(int) * (ctas + 1); o = align_up(o, 16);
  L.off_order = o; o += sizeof(int) * tiles; o = align_up(o, 16);
  L.off_tiles = o; o += sizeof(int2) * tiles; o = align_up(o, 16);
  L.off_mat_tiles = o; o += sizeof(int) * (n + 1); o = align_up(o, 16);
  L.off_coords = o; o += sizeof(float) * coords; o = align_up(o, 16);
  L.off_seq = o; o += sizeof(int4) * tiles; o = align_up(o, 16);
  L.total = o;
  if (L.total > (size_t)0x7fffffff) return fail(SVBRDF_ERR_UNSUPPORTED, "plan too large");
  return SVBRDF_OK;
}

}  // namespace svb

using namespace svb;

namespace svb {
template <int NCW>
static size_t tma_smem(int ring) {
  return (size_t)ring * kSlotPlanes * NCW * 32 * 4;
}

template <int NCW>
static size_t pair_smem(int ring) {
  return (size_t)ring * (kPairSlotPlanes * 2 * NCW * 32 * 4 + sizeof(PairSlotRec));
}

// Dynamic shared memory already allowed for one kernel instantiation, per device ordinal:
// cudaFuncSetAttribute applies to the current device only.
struct SmemAllowance {
  std::mutex mu;
  size_t have[64] = {};
};

// Once per kernel instantiation and device: allow the ring's dynamic shared memory.
template <typename Kernel>
static int allow_smem(Kernel kernel, size_t need, SmemAllowance& a) {
  int dev = 0;
  const cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(SVBRDF_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= 64) return fail(SVBRDF_ERR_UNSUPPORTED, "device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lock(a.mu);
  if (need > a.have[dev]) {
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need) != cudaSuccess)
      return fail(SVBRDF_ERR_CUDA, "cudaFuncSetAttribute: %s", cudaGetErrorString(cudaGetLastError()));
    a.have[dev] = need;
  }
  return SVBRDF_OK;
}

template <int LOSS, int NCW>
static int tma_prepare(int ring) {
  static SmemAllowance a;
  return allow_smem(batched_tma_kernel<LOSS, NCW>, tma_smem<NCW>(ring), a);
}

template <int NCW>
static size_t fuse_smem(int ring) {
  return (size_t)kStatePlanes * 2 * NCW * 32 * 4 + pair_smem<NCW>(ring);
}

template <int LOSS, int NCW, bool GEN>
static int fuse2_prepare(int ring) {
  static SmemAllowance a;
  return allow_smem(batched_fuse2_kernel<LOSS, NCW, GEN>, fuse_smem<NCW>(ring), a);
}

template <int LOSS, int NCW, bool GEN>
static int fuse_prepare(int ring) {
  static SmemAllowance a;
  return allow_smem(batched_fuse_kernel<LOSS, NCW, GEN>, fuse_smem<NCW>(ring), a);
}

template <int LOSS, int NCW, bool GEN>
static int pair_prepare(int ring) {
  static SmemAllowance a;
  return allow_smem(batched_pair_kernel<LOSS, NCW, GEN>, pair_smem<NCW>(ring), a);
}

int resident_ctas(int variant, int threads) {
  const int sms = device_sm_count();
  if (sms <= 0) return 0;
  // one pipelined CTA per SM (its ring takes the shared memory); two for the small texel-pair shape
  if (variant == 4) return threads / 32 <= kFuse2TwoCtaNcw ? 2 * sms : sms;
  if (variant >= 2 && threads / 32 <= kPairTwoCtaNcw) return 2 * sms;
  if (variant >= 1) return sms;
  int occ = 1;
  switch (threads) {
    case 128: occ = occupancy_of(batched_step_kernel<0, 128>, 128); break;
    case 256: occ = occupancy_of(batched_step_kernel<0, 256>, 256); break;
    default: occ = occupancy_of(batched_step_kernel<0, 512>, 512); break;
  }
  return sms * std::max(occ, 1);
}
}  // namespace svb

extern "C" {

int svbrdf_fused_step(float* textures, float* exp_avg, float* exp_avg_sq, const float* targets,
                      const float* camera_pos, const float* light_pos, float* light_pow, float* light_adam_state,
                      int n_views, int height, int width, float size, int loss_kind, int step, float lr,
                      float beta1, float beta2, float eps, float* loss_out, void* workspace,
                      size_t workspace_bytes, void* stream) {
  int rc = check_common(textures, camera_pos, light_pos, light_pow, n_views, height, width, size);
  if (rc) return rc;
  if (!exp_avg || !exp_avg_sq || !targets || !loss_out)
    return fail(SVBRDF_ERR_INVALID, "null exp_avg/exp_avg_sq/targets/loss_out");
  if (loss_kind < SVBRDF_LOSS_MSE || loss_kind > SVBRDF_LOSS_LOG1P_PRE)
    return fail(SVBRDF_ERR_INVALID, "bad loss_kind %d", loss_kind);
  if (step < 1) return fail(SVBRDF_ERR_INVALID, "step must be >= 1");
  if (!workspace || workspace_bytes < kWorkspaceBytes)
    return fail(SVBRDF_ERR_WORKSPACE, "workspace of %zu bytes needed", kWorkspaceBytes);
  const long long T = (long long)height * width;
  const double N = 3.0 * n_views * (double)T;
  const float scale = (float)(2.0 / N);
  const AdamScalars adam = make_adam(step, lr, beta1, beta2, eps);
  unsigned* counter = (unsigned*)workspace;
  float4* partials = (float4*)((char*)workspace + 16);
  cudaStream_t st = (cudaStream_t)stream;
  const bool gp = light_adam_state != nullptr;
#define SVB_FUSED(L, G)                                                                                        \
  {                                                                                                            \
    static int occ = occupancy_of(fused_step_kernel<L, G>, kFusedThreads);                                     \
    const int grid = grid_for(T, kFusedThreads, occ);                                                          \
    fused_step_kernel<L, G><<<grid, kFusedThreads, 0, st>>>(textures, exp_avg, exp_avg_sq, targets, camera_pos, \
                                                            light_pos, light_pow, light_adam_state, n_views,    \
                                                            height, width, size, scale, 1.0 / N, adam,          \
                                                            loss_out, partials, counter);                       \
  }
  if (gp) {
    if (loss_kind == SVBRDF_LOSS_MSE) SVB_FUSED(0, true)
    else if (loss_kind == SVBRDF_LOSS_LOG1P) SVB_FUSED(1, true)
    else SVB_FUSED(2, true)
  } else {
    if (loss_kind == SVBRDF_LOSS_MSE) SVB_FUSED(0, false)
    else if (loss_kind == SVBRDF_LOSS_LOG1P) SVB_FUSED(1, false)
    else SVB_FUSED(2, false)
  }
#undef SVB_FUSED
  return check_launch("fused_step_kernel");
}

}  // extern "C"

// ---------------------------------------------------------------- no-allocation variant
// svbrdf_fused_step_noalloc runs the same fused_step_kernel as svbrdf_fused_step, but its
// scratch (the completion counter and one float4 of partial sums per CTA) lives in this
// file-scope device array instead of a caller workspace. Every GPU that loads the library
// holds these 32 KB until the process exits.
namespace svb {
constexpr int kNoAllocMaxBlocks = 2048;
constexpr size_t kNoAllocScratchBytes = 16 + (size_t)kNoAllocMaxBlocks * sizeof(float4);
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Device address of g_noalloc_scratch on the current device. Host code cannot use the
// symbol's name as a pointer, so it is resolved once per device (with that device
// current) through cudaGetSymbolAddress and cached.
static int noalloc_scratch(void** out) {
  static std::mutex mu;
  static void* cache[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(SVBRDF_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= 64) return fail(SVBRDF_ERR_UNSUPPORTED, "device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lock(mu);
  if (!cache[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return fail(SVBRDF_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
    }
    cache[dev] = p;
  }
  *out = cache[dev];
  return SVBRDF_OK;
}
}  // namespace svb

extern "C" {

int svbrdf_fused_step_noalloc(float* textures, float* exp_avg, float* exp_avg_sq, const float* targets,
                              const float* camera_pos, const float* light_pos, float* light_pow,
                              float* light_adam_state, int n_views, int height, int width, float size,
                              int loss_kind, int step, float lr, float beta1, float beta2, float eps,
                              float* loss_out, void* stream) {
  int rc = check_common(textures, camera_pos, light_pos, light_pow, n_views, height, width, size);
  if (rc) return rc;
  if (!exp_avg || !exp_avg_sq || !targets || !loss_out)
    return fail(SVBRDF_ERR_INVALID, "null exp_avg/exp_avg_sq/targets/loss_out");
  if (loss_kind < SVBRDF_LOSS_MSE || loss_kind > SVBRDF_LOSS_LOG1P_PRE)
    return fail(SVBRDF_ERR_INVALID, "bad loss_kind %d", loss_kind);
  if (step < 1) return fail(SVBRDF_ERR_INVALID, "step must be >= 1");
  const long long T = (long long)height * width;
  const bool gp = light_adam_state != nullptr;
  // The grid is fixed (and checked against the scratch) before anything is enqueued, so a
  // rejected call leaves no work on the stream and no node in a capture.
  int grid = 0;
#define SVB_GRID_NA(L, G)                                                    \
  {                                                                          \
    static int occ = occupancy_of(fused_step_kernel<L, G>, kFusedThreads);   \
    grid = grid_for(T, kFusedThreads, occ);                                  \
  }
  if (gp) {
    if (loss_kind == SVBRDF_LOSS_MSE) SVB_GRID_NA(0, true)
    else if (loss_kind == SVBRDF_LOSS_LOG1P) SVB_GRID_NA(1, true)
    else SVB_GRID_NA(2, true)
  } else {
    if (loss_kind == SVBRDF_LOSS_MSE) SVB_GRID_NA(0, false)
    else if (loss_kind == SVBRDF_LOSS_LOG1P) SVB_GRID_NA(1, false)
    else SVB_GRID_NA(2, false)
  }
#undef SVB_GRID_NA
  if (grid > kNoAllocMaxBlocks)
    return fail(SVBRDF_ERR_UNSUPPORTED, "no-allocation step needs %d CTAs of scratch; the static array holds %d", grid,
                kNoAllocMaxBlocks);
  void* scratch = nullptr;
  rc = noalloc_scratch(&scratch);
  if (rc) return rc;
  const double N = 3.0 * n_views * (double)T;
  const float scale = (float)(2.0 / N);
  const AdamScalars adam = make_adam(step, lr, beta1, beta2, eps);
  unsigned* counter = (unsigned*)scratch;
  float4* partials = (float4*)((char*)scratch + 16);
  cudaStream_t st = (cudaStream_t)stream;
  // the counter must start at zero; the array keeps whatever the previous call left
  cudaError_t e = cudaMemsetAsync(counter, 0, 16, st);
  if (e != cudaSuccess) return fail(SVBRDF_ERR_CUDA, "cudaMemsetAsync(scratch counter): %s", cudaGetErrorString(e));
#define SVB_FUSED_NA(L, G)                                                                                     \
  fused_step_kernel<L, G><<<grid, kFusedThreads, 0, st>>>(textures, exp_avg, exp_avg_sq, targets, camera_pos, \
                                                          light_pos, light_pow, light_adam_state, n_views,    \
                                                          height, width, size, scale, 1.0 / N, adam,          \
                                                          loss_out, partials, counter);
  if (gp) {
    if (loss_kind == SVBRDF_LOSS_MSE) SVB_FUSED_NA(0, true)
    else if (loss_kind == SVBRDF_LOSS_LOG1P) SVB_FUSED_NA(1, true)
    else SVB_FUSED_NA(2, true)
  } else {
    if (loss_kind == SVBRDF_LOSS_MSE) SVB_FUSED_NA(0, false)
    else if (loss_kind == SVBRDF_LOSS_LOG1P) SVB_FUSED_NA(1, false)
    else SVB_FUSED_NA(2, false)
  }
#undef SVB_FUSED_NA
  return check_launch("fused_step_kernel (no-allocation)");
}

}  // extern "C"

namespace svb {
// (tile, warp) partial slots of one iteration, and the loss-partial floats of a launch
// (every iteration of a resident-state launch keeps its own).
static size_t ws_slots(const PlanHeader* h) {
  return (size_t)h->n_tiles * (h->variant >= 1 ? (size_t)(h->threads / 32) : 1);
}
static size_t ws_loss_floats(const PlanHeader* h) { return ws_slots(h) * (h->variant >= 3 ? (size_t)kFuseMax : 1); }
}  // namespace svb

extern "C" {

size_t svbrdf_batched_plan_bytes(const svbrdf_material* materials, int n_materials,
                                 const svbrdf_batch_config* config) {
  PlanLayout L;
  if (plan_layout(materials, n_materials, config, L)) return 0;
  return L.total;
}

int svbrdf_batched_plan(const svbrdf_material* materials, int n_materials, const svbrdf_batch_config* config,
                        void* host_plan, size_t plan_bytes) {
  PlanLayout L;
  int rc = plan_layout(materials, n_materials, config, L);
  if (rc) return rc;
  if (!host_plan || plan_bytes < L.total) return fail(SVBRDF_ERR_INVALID, "plan buffer of %zu bytes needed", L.total);
  char* base = (char*)host_plan;
  memset(base, 0, L.total);
  PlanHeader* h = (PlanHeader*)base;
  h->magic = kPlanMagic;
  h->n_mat = n_materials;
  h->n_tiles = L.n_tiles;
  h->n_ctas = L.n_ctas;
  h->threads = config->threads;
  h->tile_texels = config->tile_texels;
  h->off_mats = (int)L.off_mats;
  h->off_views = (int)L.off_views;
  h->off_cta = (int)L.off_cta;
  h->off_order = (int)L.off_order;
  h->off_tiles = (int)L.off_tiles;
  h->off_mat_tiles = (int)L.off_mat_tiles;
  h->off_coords = (int)L.off_coords;
  h->off_seq = (int)L.off_seq;
  h->variant = config->variant;
  h->ring_slots = L.ring;
  h->total_bytes = (long long)L.total;
  MatDesc* md = (MatDesc*)(base + L.off_mats);
  View* vw = (View*)(base + L.off_views);
  int* cta_off = (int*)(base + L.off_cta);
  int* order = (int*)(base + L.off_order);
  int2* tiles = (int2*)(base + L.off_tiles);
  int* mat_tiles = (int*)(base + L.off_mat_tiles);
  float* coords = (float*)(base + L.off_coords);
  std::vector<double> cost(L.n_tiles);
  int voff = 0, t = 0;
  long long coff = 0;
  double total = 0;
  for (int i = 0; i < n_materials; ++i) {
    const svbrdf_material& m = materials[i];
    const long long T = (long long)m.height * m.width;
    const double N = 3.0 * m.n_views * (double)T;
    md[i].tex = m.textures;
    md[i].m1 = m.exp_avg;
    md[i].m2 = m.exp_avg_sq;
    md[i].tgt = m.targets;
    md[i].lpow = m.light_pow;
    md[i].lstate = m.light_adam_state;
    if (m.light_adam_state) h->light = 1;
    md[i].H = m.height;
    md[i].W = m.width;
    md[i].V = m.n_views;
    md[i].view_off = voff;
    md[i].size = m.size;
    md[i].scale = (float)(2.0 / N);
    md[i].inv_w = 1.0f / (float)m.width;
    md[i].coord_off = (int)coff;
    md[i].inv_n = 1.0 / N;
    // pixel-centre grid of src/microfacet.py:16-19, FP32 with IEEE division: x[j], -y[i]
    for (int j = 0; j < m.width; ++j)
      coords[coff + j] = (((float)j + 0.5f) / (float)m.width - 0.5f) * m.size;
    for (int r = 0; r < m.height; ++r)
      coords[coff + m.width + r] = -((((float)r + 0.5f) / (float)m.height - 0.5f) * m.size);
    coff += m.width + m.height;
    int allc = 1;
    for (int v = 0; v < m.n_views; ++v) {
      View& w = vw[voff + v];
      w.cx = m.camera_pos[3 * v]; w.cy = m.camera_pos[3 * v + 1]; w.cz = m.camera_pos[3 * v + 2];
      w.lx = m.light_pos[3 * v]; w.ly = m.light_pos[3 * v + 1]; w.lz = m.light_pos[3 * v + 2];
      w.coloc = (w.cx == w.lx && w.cy == w.ly && w.cz == w.lz) ? 1.f : 0.f;
      allc = allc && w.coloc != 0.f;
    }
    md[i].all_coloc = allc;
    if (!allc) h->general = 1;
    voff += m.n_views;
    mat_tiles[i] = t;
    for (long long x = 0; x < T; x += config->tile_texels) {
      tiles[t] = make_int2(i, (int)x);
      const long long cnt = std::min<long long>(config->tile_texels, T - x);
      // cost model: per-texel fixed work (set-up, map-back, Adam, parameter and moment
      // traffic) ~ 5 views
      cost[t] = (double)cnt * (m.n_views + 5.0);
      total += cost[t];
      ++t;
    }
  }
  mat_tiles[n_materials] = t;
  h->total_cost = total;
  // Contiguous split: CTA c takes the run of tiles (in material order) whose cost midpoints
  // fall in its share [c, c+1) * total / n_ctas. Every CTA's load is within one tile of the
  // mean, and a CTA crosses few material boundaries, so its consumers rarely re-stage a
  // material's views and its producer rarely reloads a material.
  int kk = 0;
  double acc = 0.0;
  for (int c = 0; c < L.n_ctas; ++c) {
    cta_off[c] = kk;
    const double target = total * (double)(c + 1) / (double)L.n_ctas;
    while (kk < L.n_tiles && (c == L.n_ctas - 1 || acc + 0.5 * cost[kk] <= target)) {
      acc += cost[kk];
      order[kk] = kk;
      ++kk;
    }
  }
  cta_off[L.n_ctas] = L.n_tiles;
  int4* seq = (int4*)(base + L.off_seq);
  for (int k = 0; k < L.n_tiles; ++k) seq[k] = make_int4(order[k], tiles[order[k]].x, tiles[order[k]].y, 0);
  return SVBRDF_OK;
}

size_t svbrdf_batched_workspace_bytes(const void* host_plan) {
  if (!host_plan) return 0;
  const PlanHeader* h = (const PlanHeader*)host_plan;
  if (h->magic != kPlanMagic) return 0;
  // loss partials, light partials, then the per-(iteration, tile) totals (kFuseMax rows) and
  // the per-tile light totals (3 rows)
  return kWsLossOffset + sizeof(float) * ws_loss_floats(h) + (h->light ? sizeof(float) * 3 * ws_slots(h) : 0) +
         sizeof(float) * (size_t)h->n_tiles * (kFuseMax + 3);
}

int svbrdf_selftest_wait_timeout(void* workspace, size_t workspace_bytes, int limit, void* stream) {
  if (!workspace || workspace_bytes < 16) return fail(SVBRDF_ERR_WORKSPACE, "self-test: 16 bytes of workspace needed");
  if (limit < 1 || limit > (1 << 24)) return fail(SVBRDF_ERR_INVALID, "self-test: limit must be in [1, 2^24]");
  wait_selftest_kernel<<<1, 32, 0, (cudaStream_t)stream>>>((unsigned*)workspace, (uint32_t)limit);
  return check_launch("wait_selftest_kernel");
}

int svbrdf_batched_step(const void* device_plan, const void* host_plan, int loss_kind, int* step_counter, float lr,
                        float beta1, float beta2, float eps, float* loss_hist, int hist_len, void* workspace,
                        size_t workspace_bytes, void* stream) {
  return svbrdf_batched_steps(device_plan, host_plan, loss_kind, step_counter, lr, beta1, beta2, eps, loss_hist,
                              hist_len, 1, workspace, workspace_bytes, stream);
}

// One launch of the single-iteration variants (0, 1, 2).
static int batched_launch_one(const PlanHeader* h, const char* plan, int loss_kind, int* step_counter,
                              AdamHyper hyper, float* loss_hist, int hist_len, unsigned* ws, float* part,
                              float* lpart, cudaStream_t st);

int svbrdf_batched_steps(const void* device_plan, const void* host_plan, int loss_kind, int* step_counter, float lr,
                         float beta1, float beta2, float eps, float* loss_hist, int hist_len, int iters,
                         void* workspace, size_t workspace_bytes, void* stream) {
  if (!device_plan || !host_plan || !loss_hist || !step_counter)
    return fail(SVBRDF_ERR_INVALID, "null plan/step_counter/loss_hist");
  const PlanHeader* h = (const PlanHeader*)host_plan;
  if (h->magic != kPlanMagic) return fail(SVBRDF_ERR_INVALID, "host_plan is not a plan");
  if (loss_kind < SVBRDF_LOSS_MSE || loss_kind > SVBRDF_LOSS_LOG1P_PRE)
    return fail(SVBRDF_ERR_INVALID, "bad loss_kind %d", loss_kind);
  if (hist_len < 1) return fail(SVBRDF_ERR_INVALID, "hist_len must be >= 1");
  if (iters < 0) return fail(SVBRDF_ERR_INVALID, "iters must be >= 0");
  const size_t need = svbrdf_batched_workspace_bytes(host_plan);
  if (!workspace || workspace_bytes < need) return fail(SVBRDF_ERR_WORKSPACE, "workspace of %zu bytes needed", need);
  unsigned* ws = (unsigned*)workspace;
  float* part = (float*)((char*)workspace + kWsLossOffset);
  float* lpart = h->light ? part + ws_loss_floats(h) : nullptr;
  AdamHyper hyper;
  hyper.lr = lr;
  hyper.beta1 = beta1;
  hyper.beta2 = beta2;
  hyper.eps = eps;
  cudaStream_t st = (cudaStream_t)stream;
  const char* plan = (const char*)device_plan;
  if (h->variant < 3) {
    for (int i = 0; i < iters; ++i) {
      const int rc =
          batched_launch_one(h, plan, loss_kind, step_counter, hyper, loss_hist, hist_len, ws, part, lpart, st);
      if (rc) return rc;
    }
    return SVBRDF_OK;
  }
  const int ring = h->ring_slots;
  if (ring < 2 || ring > kMaxRing) return fail(SVBRDF_ERR_INVALID, "bad ring depth %d", ring);
  // iters split evenly over ceil(iters / kFuseMax) launches; a learnable light couples every
  // texel of a material once per iteration, so such plans run one iteration per launch
  const int launches = h->light ? iters : (iters + kFuseMax - 1) / kFuseMax;
  for (int l = 0; l < launches; ++l) {
    const int k = iters / launches + (l < iters % launches ? 1 : 0);
#define SVB_F(L, NCW, G)                                                                                       {                                                                                                              int prc = fuse_prepare<L, NCW, G>(ring);                                                                     if (prc) return prc;                                                                                         batched_fuse_kernel<L, NCW, G><<<h->n_ctas, (NCW + 1) * 32, fuse_smem<NCW>(ring), st>>>(                         plan, hyper, step_counter, loss_hist, hist_len, k, part, ws, lpart);                                   }
#define SVB_FG(L, NCW)                  if (h->general) SVB_F(L, NCW, true)   else SVB_F(L, NCW, false)
#define SVB_FL(NCW)                                         if (loss_kind == SVBRDF_LOSS_MSE) SVB_FG(0, NCW)          else if (loss_kind == SVBRDF_LOSS_LOG1P) SVB_FG(1, NCW)   else SVB_FG(2, NCW)
    if (h->variant == 3) {
      switch (h->threads) {
        case 224: SVB_FL(7) break;
        case 256: SVB_FL(8) break;
        case 384: SVB_FL(12) break;
        default: SVB_FL(15) break;
      }
    }
#undef SVB_FL
#undef SVB_FG
#undef SVB_F
#define SVB_F2(L, NCW, G)                                                                                      {                                                                                                              int prc = fuse2_prepare<L, NCW, G>(ring);                                                                    if (prc) return prc;                                                                                         batched_fuse2_kernel<L, NCW, G><<<h->n_ctas, NCW * 32, fuse_smem<NCW>(ring), st>>>(                              plan, hyper, step_counter, loss_hist, hist_len, k, part, ws);                                          }
#define SVB_F2G(L, NCW)                  if (h->general) SVB_F2(L, NCW, true)   else SVB_F2(L, NCW, false)
#define SVB_F2L(NCW)                                         if (loss_kind == SVBRDF_LOSS_MSE) SVB_F2G(0, NCW)          else if (loss_kind == SVBRDF_LOSS_LOG1P) SVB_F2G(1, NCW)   else SVB_F2G(2, NCW)
    if (h->variant == 4) {
      if (h->threads == 256) SVB_F2L(8)
      else SVB_F2L(16)
    }
#undef SVB_F2L
#undef SVB_F2G
#undef SVB_F2
    const int rc = check_launch(h->variant == 3 ? "batched_fuse_kernel" : "batched_fuse2_kernel");
    if (rc) return rc;
  }
  return SVBRDF_OK;
}

static int batched_launch_one(const PlanHeader* h, const char* plan, int loss_kind, int* step_counter,
                              AdamHyper hyper, float* loss_hist, int hist_len, unsigned* ws, float* part,
                              float* lpart, cudaStream_t st) {
  if (h->variant == 0) {
#define SVB_B(L, NT) \
  batched_step_kernel<L, NT><<<h->n_ctas, NT, 0, st>>>(plan, hyper, step_counter, loss_hist, hist_len, part, ws)
#define SVB_BL(NT)                                       \
  if (loss_kind == SVBRDF_LOSS_MSE) SVB_B(0, NT);        \
  else if (loss_kind == SVBRDF_LOSS_LOG1P) SVB_B(1, NT); \
  else SVB_B(2, NT);
    switch (h->threads) {
      case 128: SVB_BL(128) break;
      case 256: SVB_BL(256) break;
      default: SVB_BL(512) break;
    }
#undef SVB_BL
#undef SVB_B
    return check_launch("batched_step_kernel");
  }
  const int ring = h->ring_slots;
  if (ring < 2 || ring > kMaxRing) return fail(SVBRDF_ERR_INVALID, "bad ring depth %d", ring);
  if (h->variant == 2) {
#define SVB_P(L, NCW, G)                                                                                     \
  {                                                                                                          \
    int prc = pair_prepare<L, NCW, G>(ring);                                                                 \
    if (prc) return prc;                                                                                     \
    batched_pair_kernel<L, NCW, G><<<h->n_ctas, (NCW + 1) * 32, pair_smem<NCW>(ring), st>>>(                 \
        plan, hyper, step_counter, loss_hist, hist_len, part, ws, lpart);                                    \
  }
#define SVB_PG(L, NCW)         \
  if (h->general) SVB_P(L, NCW, true) \
  else SVB_P(L, NCW, false)
#define SVB_PL(NCW)                                       \
  if (loss_kind == SVBRDF_LOSS_MSE) SVB_PG(0, NCW)        \
  else if (loss_kind == SVBRDF_LOSS_LOG1P) SVB_PG(1, NCW) \
  else SVB_PG(2, NCW)
    switch (h->threads) {
      case 224: SVB_PL(7) break;
      case 256: SVB_PL(8) break;
      case 384: SVB_PL(12) break;
      case 480: SVB_PL(15) break;
      default: SVB_PL(19) break;
    }
#undef SVB_PG
#undef SVB_PL
#undef SVB_P
    return check_launch("batched_pair_kernel");
  }
#define SVB_T(L, NCW)                                                                                        \
  {                                                                                                          \
    int prc = tma_prepare<L, NCW>(ring);                                                                     \
    if (prc) return prc;                                                                                     \
    batched_tma_kernel<L, NCW><<<h->n_ctas, (NCW + 1) * 32, tma_smem<NCW>(ring), st>>>(                      \
        plan, hyper, step_counter, loss_hist, hist_len, part, ws);                                           \
  }
#define SVB_TL(NCW)                                       \
  if (loss_kind == SVBRDF_LOSS_MSE) SVB_T(0, NCW)         \
  else if (loss_kind == SVBRDF_LOSS_LOG1P) SVB_T(1, NCW)  \
  else SVB_T(2, NCW)
  switch (h->threads) {
    case 256: SVB_TL(8) break;
    case 384: SVB_TL(12) break;
    case 480: SVB_TL(15) break;
    default: SVB_TL(19) break;
  }
#undef SVB_TL
#undef SVB_T
  return check_launch("batched_tma_kernel");
}

}  // extern "C"
