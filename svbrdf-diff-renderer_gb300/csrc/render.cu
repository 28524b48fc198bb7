// Forward render (+ optional loss) and its standalone adjoint: the two halves of the
// drop-in Microfacet.eval with a hand-written backward (src/microfacet.py:84-120).
#include <string>

#include "svbrdf_common.cuh"

namespace svb {

// ------------------------------------------------------------------ error state
static thread_local std::string g_last_error;

void set_error(const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
}

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

int check_launch(const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(SVBRDF_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  return SVBRDF_OK;
}

int device_sm_count() {
  static int cache[64] = {0};
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (dev >= 0 && dev < 64 && cache[dev] > 0) return cache[dev];
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  if (dev >= 0 && dev < 64) cache[dev] = n;
  return n;
}

// ------------------------------------------------------------------ kernels
constexpr int kRenderThreads = 256;

template <int LOSS>
__global__ void __launch_bounds__(kRenderThreads)
render_fwd_kernel(const float* __restrict__ tex, const float* __restrict__ cam, const float* __restrict__ lit,
                  const float* __restrict__ lpow, int V, int H, int W, float size, float* __restrict__ out,
                  const float* __restrict__ targets, float4* partials, unsigned* counter, float* loss_out,
                  double inv_n, int B) {
  __shared__ View s_views[kMaxViews];
  __shared__ float s_pow[3];
  __shared__ float s_red[kRenderThreads / 32];
  __shared__ double s_dred[4 * kRenderThreads / 32];
  __shared__ int s_flag;
  stage_views(s_views, cam, lit, V);
  if (threadIdx.x < 3) s_pow[threadIdx.x] = lpow[threadIdx.x];
  __syncthreads();

  const long long T = (long long)H * W;
  float loss = 0.f;
  Adj dummy;
  // texel gi of the batch: material b = gi / T, texel idx = gi % T; material b's maps start at
  // 9 T b, its renders (and targets) at 3 V T b
  for (long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x; gi < T * B;
       gi += (long long)gridDim.x * blockDim.x) {
    const long long b = gi / T, idx = gi - b * T;
    const float* texb = tex + 9 * T * b;
    float t[9];
#pragma unroll
    for (int c = 0; c < 9; ++c) t[c] = texb[c * T + idx];
    Maps m;
    decode(t, m);
    float px, py;
    texel_pos((int)(idx / W), (int)(idx % W), W, H, size, px, py);
    const long long vb = 3LL * V * T * b;
    for (int v = 0; v < V; ++v) {
      float io[3];
      if (LOSS >= 0) {
#pragma unroll
        for (int c = 0; c < 3; ++c) io[c] = targets[vb + (3LL * v + c) * T + idx];
      }
      if (s_views[v].coloc != 0.f)
        texel_view<kModeFwd, LOSS, false, true>(m, px, py, s_views[v], s_pow, io, loss, dummy);
      else
        texel_view<kModeFwd, LOSS, false, false>(m, px, py, s_views[v], s_pow, io, loss, dummy);
      if (out) {
#pragma unroll
        for (int c = 0; c < 3; ++c) out[vb + (3LL * v + c) * T + idx] = io[c];
      }
    }
  }
  if (LOSS >= 0) {
    const float bl = block_sum<kRenderThreads>(loss, s_red);
    if (publish_partial_and_check_last(partials, counter, make_float4(bl, 0.f, 0.f, 0.f), &s_flag)) {
      double tot[4];
      sum_partials<kRenderThreads>(partials, gridDim.x, tot, s_dred);
      if (threadIdx.x == 0) {
        *loss_out = (float)(tot[0] * inv_n);
        *counter = 0u;
      }
    }
  }
}

template <bool GRAD_POW>
__global__ void __launch_bounds__(kRenderThreads)
render_bwd_kernel(const float* __restrict__ tex, const float* __restrict__ cam, const float* __restrict__ lit,
                  const float* __restrict__ lpow, int V, int H, int W, float size,
                  const float* __restrict__ gout, float* __restrict__ gtex, float* __restrict__ gpow,
                  float4* partials, unsigned* counter, int B) {
  __shared__ View s_views[kMaxViews];
  __shared__ float s_pow[3];
  __shared__ float s_red[kRenderThreads / 32];
  __shared__ double s_dred[4 * kRenderThreads / 32];
  __shared__ int s_flag;
  stage_views(s_views, cam, lit, V);
  if (threadIdx.x < 3) s_pow[threadIdx.x] = lpow[threadIdx.x];
  __syncthreads();

  const long long T = (long long)H * W;
  float gp0 = 0.f, gp1 = 0.f, gp2 = 0.f, unused = 0.f;
  for (long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x; gi < T * B;
       gi += (long long)gridDim.x * blockDim.x) {
    const long long b = gi / T, idx = gi - b * T;
    const float* texb = tex + 9 * T * b;
    float t[9];
#pragma unroll
    for (int c = 0; c < 9; ++c) t[c] = texb[c * T + idx];
    Maps m;
    decode(t, m);
    float px, py;
    texel_pos((int)(idx / W), (int)(idx % W), W, H, size, px, py);
    Adj a;
    adj_zero(a);
    const long long vb = 3LL * V * T * b;
    for (int v = 0; v < V; ++v) {
      float io[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) io[c] = gout[vb + (3LL * v + c) * T + idx];
      if (s_views[v].coloc != 0.f)
        texel_view<kModeBwd, kLossMSE, GRAD_POW, true>(m, px, py, s_views[v], s_pow, io, unused, a);
      else
        texel_view<kModeBwd, kLossMSE, GRAD_POW, false>(m, px, py, s_views[v], s_pow, io, unused, a);
    }
    float g[9];
    adj_to_params(t, m, a, 1.0f, g);
#pragma unroll
    for (int c = 0; c < 9; ++c) gtex[9 * T * b + c * T + idx] = g[c];
    if (GRAD_POW) { gp0 += a.gp[0]; gp1 += a.gp[1]; gp2 += a.gp[2]; }
  }
  if (GRAD_POW) {
    const float b0 = block_sum<kRenderThreads>(gp0, s_red);
    const float b1 = block_sum<kRenderThreads>(gp1, s_red);
    const float b2 = block_sum<kRenderThreads>(gp2, s_red);
    if (publish_partial_and_check_last(partials, counter, make_float4(0.f, b0, b1, b2), &s_flag)) {
      double tot[4];
      sum_partials<kRenderThreads>(partials, gridDim.x, tot, s_dred);
      if (threadIdx.x == 0) {
        gpow[0] = (float)tot[1];
        gpow[1] = (float)tot[2];
        gpow[2] = (float)tot[3];
        *counter = 0u;
      }
    }
  }
}

// ------------------------------------------------------------------ launch helpers
int check_common(const float* tex, const float* cam, const float* lit, const float* lpow, int V, int H, int W,
                 float size) {
  if (!tex || !cam || !lit || !lpow) return fail(SVBRDF_ERR_INVALID, "null textures/camera_pos/light_pos/light_pow");
  if (V <= 0 || H <= 0 || W <= 0) return fail(SVBRDF_ERR_INVALID, "bad shape V=%d H=%d W=%d", V, H, W);
  if (V > kMaxViews) return fail(SVBRDF_ERR_UNSUPPORTED, "n_views=%d exceeds the maximum %d", V, kMaxViews);
  if (!(size > 0.0f)) return fail(SVBRDF_ERR_INVALID, "size must be > 0");
  // every kernel indexes texels in 64 bits; row and column indices stay 32-bit
  if ((long long)H * W >= (1LL << 31)) return fail(SVBRDF_ERR_UNSUPPORTED, "H*W = %lld is not below 2^31", (long long)H * W);
  return SVBRDF_OK;
}

int grid_for(long long T, int threads, int occupancy_blocks) {
  const int sms = device_sm_count();
  long long need = (T + threads - 1) / threads;
  long long cap = (long long)(sms > 0 ? sms : 1) * (occupancy_blocks > 0 ? occupancy_blocks : 1);
  if (cap > kMaxGrid) cap = kMaxGrid;
  if (need > cap) need = cap;
  return (int)(need < 1 ? 1 : need);
}

template <typename K>
int occupancy(K kernel, int threads) {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, 0) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return n;
}

}  // namespace svb

using namespace svb;

extern "C" {

const char* svbrdf_last_error(void) { return g_last_error.c_str(); }
int svbrdf_abi_version(void) { return SVBRDF_ABI_VERSION; }
int svbrdf_max_views(void) { return kMaxViews; }
size_t svbrdf_workspace_bytes(void) { return kWorkspaceBytes; }

int svbrdf_render_fwd_batch(const float* textures, const float* camera_pos, const float* light_pos,
                            const float* light_pow, int n_views, int height, int width, float size, int batch,
                            float* out, const float* targets, int loss_kind, float* loss_out, void* workspace,
                            size_t workspace_bytes, void* stream) {
  int rc = check_common(textures, camera_pos, light_pos, light_pow, n_views, height, width, size);
  if (rc) return rc;
  if (batch < 1 || (long long)batch * height * width >= (1LL << 40))
    return fail(SVBRDF_ERR_INVALID, "bad batch %d", batch);
  if (loss_kind < SVBRDF_LOSS_NONE || loss_kind > SVBRDF_LOSS_LOG1P_PRE)
    return fail(SVBRDF_ERR_INVALID, "bad loss_kind %d", loss_kind);
  if (loss_kind == SVBRDF_LOSS_NONE && !out) return fail(SVBRDF_ERR_INVALID, "out is NULL and no loss requested");
  if (loss_kind != SVBRDF_LOSS_NONE) {
    if (!targets || !loss_out) return fail(SVBRDF_ERR_INVALID, "loss requested without targets/loss_out");
    if (!workspace || workspace_bytes < kWorkspaceBytes)
      return fail(SVBRDF_ERR_WORKSPACE, "workspace of %zu bytes needed", kWorkspaceBytes);
  }
  const long long T = (long long)height * width;
  const double inv_n = 1.0 / (3.0 * n_views * (double)T * batch);
  unsigned* counter = (unsigned*)workspace;
  float4* partials = workspace ? (float4*)((char*)workspace + 16) : nullptr;
  cudaStream_t st = (cudaStream_t)stream;
  switch (loss_kind) {
#define SVB_FWD(L)                                                                                          \
  {                                                                                                         \
    static int occ = occupancy(render_fwd_kernel<L>, kRenderThreads);                                       \
    const int grid = grid_for(T * batch, kRenderThreads, occ);                                              \
    render_fwd_kernel<L><<<grid, kRenderThreads, 0, st>>>(textures, camera_pos, light_pos, light_pow,      \
                                                          n_views, height, width, size, out, targets,       \
                                                          partials, counter, loss_out, inv_n, batch);       \
    break;                                                                                                  \
  }
    case SVBRDF_LOSS_NONE: SVB_FWD(-1)
    case SVBRDF_LOSS_MSE: SVB_FWD(0)
    case SVBRDF_LOSS_LOG1P: SVB_FWD(1)
    default: SVB_FWD(2)
#undef SVB_FWD
  }
  return check_launch("render_fwd_kernel");
}

int svbrdf_render_fwd(const float* textures, const float* camera_pos, const float* light_pos,
                      const float* light_pow, int n_views, int height, int width, float size, float* out,
                      const float* targets, int loss_kind, float* loss_out, void* workspace,
                      size_t workspace_bytes, void* stream) {
  return svbrdf_render_fwd_batch(textures, camera_pos, light_pos, light_pow, n_views, height, width, size, 1, out,
                                 targets, loss_kind, loss_out, workspace, workspace_bytes, stream);
}

int svbrdf_render_bwd_batch(const float* textures, const float* camera_pos, const float* light_pos,
                            const float* light_pow, int n_views, int height, int width, float size, int batch,
                            const float* grad_out, float* grad_textures, float* grad_light_pow, void* workspace,
                            size_t workspace_bytes, void* stream) {
  int rc = check_common(textures, camera_pos, light_pos, light_pow, n_views, height, width, size);
  if (rc) return rc;
  if (batch < 1 || (long long)batch * height * width >= (1LL << 40))
    return fail(SVBRDF_ERR_INVALID, "bad batch %d", batch);
  if (!grad_out || !grad_textures) return fail(SVBRDF_ERR_INVALID, "null grad_out/grad_textures");
  if (grad_light_pow && (!workspace || workspace_bytes < kWorkspaceBytes))
    return fail(SVBRDF_ERR_WORKSPACE, "workspace of %zu bytes needed", kWorkspaceBytes);
  const long long T = (long long)height * width;
  unsigned* counter = (unsigned*)workspace;
  float4* partials = workspace ? (float4*)((char*)workspace + 16) : nullptr;
  cudaStream_t st = (cudaStream_t)stream;
  if (grad_light_pow) {
    static int occ = occupancy(render_bwd_kernel<true>, kRenderThreads);
    const int grid = grid_for(T * batch, kRenderThreads, occ);
    render_bwd_kernel<true><<<grid, kRenderThreads, 0, st>>>(textures, camera_pos, light_pos, light_pow, n_views,
                                                             height, width, size, grad_out, grad_textures,
                                                             grad_light_pow, partials, counter, batch);
  } else {
    static int occ = occupancy(render_bwd_kernel<false>, kRenderThreads);
    const int grid = grid_for(T * batch, kRenderThreads, occ);
    render_bwd_kernel<false><<<grid, kRenderThreads, 0, st>>>(textures, camera_pos, light_pos, light_pow, n_views,
                                                              height, width, size, grad_out, grad_textures,
                                                              nullptr, partials, counter, batch);
  }
  return check_launch("render_bwd_kernel");
}

int svbrdf_render_bwd(const float* textures, const float* camera_pos, const float* light_pos,
                      const float* light_pow, int n_views, int height, int width, float size,
                      const float* grad_out, float* grad_textures, float* grad_light_pow, void* workspace,
                      size_t workspace_bytes, void* stream) {
  return svbrdf_render_bwd_batch(textures, camera_pos, light_pos, light_pow, n_views, height, width, size, 1, grad_out,
                                 grad_textures, grad_light_pow, workspace, workspace_bytes, stream);
}

}  // extern "C"
