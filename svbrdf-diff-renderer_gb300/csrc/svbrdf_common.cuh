// Shared host/device plumbing of the C-ABI library: error state, argument checks,
// block reductions and the last-block-done grid reduction.
#pragma once

#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>

#include "svbrdf_gb300.h"
#include "svbrdf_math.cuh"

namespace svb {

// ---- error reporting: a per-host-thread message behind svbrdf_last_error() ----
void set_error(const char* fmt, ...);
int fail(int code, const char* fmt, ...);
int check_launch(const char* what);

int device_sm_count();  // cached per device

// Largest grid any single-material kernel uses; sizes the reduction workspace.
constexpr int kMaxGrid = 4096;
// Workspace layout: [0..15] counter + pad, then kMaxGrid float4 partials.
constexpr size_t kWorkspaceBytes = 16 + (size_t)kMaxGrid * 16;

// ---- device reductions ----
template <int NT>
__device__ __forceinline__ float block_sum(float v, float* smem /* >= NT/32 floats */) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) smem[w] = v;
  __syncthreads();
  float r = 0.f;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int i = 0; i < NT / 32; ++i) r += smem[i];
  }
  return r;  // valid in thread 0
}

// Writes this block's 4 partial sums and returns true in every thread of the block that
// finished last (the classic threadfence reduction: no waiting, no spin).
__device__ __forceinline__ bool publish_partial_and_check_last(float4* partials, unsigned* counter, float4 mine,
                                                               int* s_flag) {
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = mine;
    __threadfence();
    const unsigned prev = atomicAdd(counter, 1u);
    *s_flag = (prev == gridDim.x - 1) ? 1 : 0;
  }
  __syncthreads();
  const bool last = *s_flag != 0;
  if (last) __threadfence();
  return last;
}

// Sums the grid's partials in a fixed order (deterministic) in double; thread 0 gets it.
template <int NT>
__device__ __forceinline__ void sum_partials(const float4* partials, int n, double out[4], double* smem /* 4*NT/32 */) {
  double a[4] = {0.0, 0.0, 0.0, 0.0};
  for (int i = threadIdx.x; i < n; i += NT) {
    const float4 p = __ldcg(partials + i);
    a[0] += p.x; a[1] += p.y; a[2] += p.z; a[3] += p.w;
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a[q] += __shfl_xor_sync(0xffffffffu, a[q], o);
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < 4; ++q) smem[w * 4 + q] = a[q];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      double t = 0.0;
      for (int i = 0; i < NT / 32; ++i) t += smem[i * 4 + q];
      out[q] = t;
    }
  }
}

// Stage V views (camera, light) into shared memory and flag the co-located ones.
__device__ __forceinline__ void stage_views(View* s_views, const float* cam, const float* lit, int V) {
  for (int v = threadIdx.x; v < V; v += blockDim.x) {
    View w;
    w.cx = cam[3 * v + 0]; w.cy = cam[3 * v + 1]; w.cz = cam[3 * v + 2];
    w.lx = lit[3 * v + 0]; w.ly = lit[3 * v + 1]; w.lz = lit[3 * v + 2];
    w.coloc = (w.cx == w.lx && w.cy == w.ly && w.cz == w.lz) ? 1.0f : 0.0f;
    w.pad = 0.f;
    s_views[v] = w;
  }
}

}  // namespace svb
