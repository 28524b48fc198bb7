// Fused render + loss + adjoint + Adam: one pass per optimiser iteration.
//
// Replaces the loop body of SvbrdfOptim.optim (src/svbrdf.py:56-71):
//   rendereds = eval(textures.clamp(-1, 1)); loss = MSE(rendereds, targets);
//   zero_grad(); loss.backward(); optimizer.step()
// Each thread owns a texel: it reads the 9 parameters, the Adam moments and the V
// targets once, recomputes every per-view term in registers, and writes the 9
// parameters and the two moments back. Per-iteration HBM traffic is therefore
// (36 + 36 + 36) read + (36 + 36 + 36) write + 12*V target bytes per texel.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "svbrdf_common.cuh"

namespace svb {

int check_common(const float* tex, const float* cam, const float* lit, const float* lpow, int V, int H, int W,
                 float size);
int grid_for(long long T, int threads, int occupancy_blocks);

AdamScalars make_adam(int step, float lr, float beta1, float beta2, float eps) {
  // torch.optim.Adam (single-tensor and foreach paths) computes the bias corrections as
  // Python floats and hands them to FP32 kernels.
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

// One texel of one fused iteration. Returns the texel's summed squared error.
template <int LOSS, bool GRAD_POW>
__device__ __forceinline__ float fused_texel(float* __restrict__ tex, float* __restrict__ mom1,
                                             float* __restrict__ mom2, const float* __restrict__ tgt,
                                             long long T, long long idx, int W, int H, float size, int V,
                                             const View* s_views, const float* s_pow, float scale,
                                             const AdamScalars& adam, float gp[3]) {
  float raw[9], t[9];
#pragma unroll
  for (int c = 0; c < 9; ++c) {
    raw[c] = tex[c * T + idx];
    t[c] = fminf(fmaxf(raw[c], -1.0f), 1.0f);  // textures.clamp(-1, 1), src/svbrdf.py:60
  }
  Maps m;
  decode(t, m);
  float px, py;
  texel_pos((int)(idx / W), (int)(idx % W), W, H, size, px, py);
  Adj a;
  adj_zero(a);
  float loss = 0.f;
  for (int v = 0; v < V; ++v) {
    float io[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) io[c] = __ldcs(tgt + (3LL * v + c) * T + idx);
    if (s_views[v].coloc != 0.f)
      texel_view<kModeFused, LOSS, GRAD_POW, true>(m, px, py, s_views[v], s_pow, io, loss, a);
    else
      texel_view<kModeFused, LOSS, GRAD_POW, false>(m, px, py, s_views[v], s_pow, io, loss, a);
  }
  float g[9];
  adj_to_params(t, m, a, scale, g);
#pragma unroll
  for (int c = 0; c < 9; ++c) {
    const float gc = (raw[c] >= -1.0f && raw[c] <= 1.0f) ? g[c] : 0.0f;
    float p = raw[c];
    float m1 = mom1[c * T + idx];
    float m2 = mom2[c * T + idx];
    adam_update(p, m1, m2, gc, adam);
    tex[c * T + idx] = p;
    mom1[c * T + idx] = m1;
    mom2[c * T + idx] = m2;
  }
  if (GRAD_POW) {
    gp[0] += a.gp[0] * scale;
    gp[1] += a.gp[1] * scale;
    gp[2] += a.gp[2] * scale;
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

  const long long T = (long long)H * W;
  float loss = 0.f;
  float gp[3] = {0.f, 0.f, 0.f};
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < T;
       idx += (long long)gridDim.x * blockDim.x)
    loss += fused_texel<LOSS, GRAD_POW>(tex, mom1, mom2, tgt, T, idx, W, H, size, V, s_views, s_pow, scale, adam,
                                        gp);

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
int occupancy_of(K kernel, int threads) {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, 0) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return n;
}

// ============================================================== batched, persistent
//
// Plan (one contiguous buffer, identical on host and device):
//   PlanHeader | MatDesc[n_mat] | View[total views] | int cta_off[n_ctas+1]
//   | int2 tiles[n_tiles] (material, first texel) | int mat_tile_off[n_mat+1]
// Tiles of one material are contiguous in tile-index order (mat_tile_off), so the
// per-material loss is a fixed-order sum over a tile range. cta_off[c]..cta_off[c+1]
// indexes `order`, a permutation of tile ids balanced across CTAs by the planner.

struct PlanHeader {
  int magic;
  int n_mat;
  int n_tiles;
  int n_ctas;
  int threads;
  int tile_texels;
  int off_mats;      // byte offsets from the plan base
  int off_views;
  int off_cta;
  int off_order;
  int off_tiles;
  int off_mat_tiles;
  long long total_bytes;
  double total_cost;  // texel*views
};

struct __align__(16) MatDesc {
  float* tex;
  float* m1;
  float* m2;
  const float* tgt;
  const float* lpow;
  int H, W, V, view_off;
  float size, scale;
  double inv_n;
};

constexpr int kPlanMagic = 0x53564231;  // "SVB1"

// Adam hyper-parameters of a batched launch; the step itself lives on the device so
// one captured graph can be replayed indefinitely.
struct AdamHyper {
  float lr, beta1, beta2, eps;
};

__device__ __forceinline__ AdamScalars device_adam(const AdamHyper& h, int step) {
  // same double-precision bias corrections as make_adam() / torch.optim.Adam
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

template <int LOSS, int NT>
__global__ void __launch_bounds__(NT)
batched_step_kernel(const char* __restrict__ plan, AdamHyper hyper, int* __restrict__ step_counter,
                    float* __restrict__ loss_hist, int hist_len, float* __restrict__ tile_loss, unsigned* counter) {
  __shared__ View s_views[kMaxViews];
  __shared__ float s_pow[3];
  __shared__ float s_red[NT / 32];
  __shared__ int s_flag;
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
    const long long T = (long long)md.H * md.W;
    const long long end = min((long long)tl.y + tile_texels, T);
    float loss = 0.f;
    for (long long idx = tl.y + threadIdx.x; idx < end; idx += NT)
      loss += fused_texel<LOSS, false>(md.tex, md.m1, md.m2, md.tgt, T, idx, md.W, md.H, md.size, md.V, s_views,
                                       s_pow, md.scale, adam, gp_unused);
    const float bl = block_sum<NT>(loss, s_red);
    if (threadIdx.x == 0) tile_loss[tid] = bl;
  }

  // last CTA: per-material loss, one warp per material, fixed order
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned prev = atomicAdd(counter, 1u);
    s_flag = (prev == gridDim.x - 1) ? 1 : 0;
  }
  __syncthreads();
  if (!s_flag) return;
  __threadfence();
  const int* mat_tiles = (const int*)(plan + hdr->off_mat_tiles);
  float* loss_out = loss_hist + (size_t)((s_step - 1) % hist_len) * hdr->n_mat;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int mi = w; mi < hdr->n_mat; mi += NT / 32) {
    double acc = 0.0;
    for (int t = mat_tiles[mi] + lane; t < mat_tiles[mi + 1]; t += 32) acc += (double)__ldcg(tile_loss + t);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) loss_out[mi] = (float)(acc * mats[mi].inv_n);
  }
  if (threadIdx.x == 0) {
    *step_counter = s_step;
    *counter = 0u;
  }
}

static size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

struct PlanLayout {
  size_t off_mats, off_views, off_cta, off_order, off_tiles, off_mat_tiles, total;
  int n_tiles, n_ctas, total_views;
};

int resident_ctas(int threads);

static int plan_layout(const svbrdf_material* mats, int n, const svbrdf_batch_config* cfg, PlanLayout& L) {
  if (!mats || n <= 0) return fail(SVBRDF_ERR_INVALID, "no materials");
  if (!cfg) return fail(SVBRDF_ERR_INVALID, "null config");
  if (cfg->threads != 128 && cfg->threads != 256 && cfg->threads != 512)
    return fail(SVBRDF_ERR_UNSUPPORTED, "threads must be 128, 256 or 512 (got %d)", cfg->threads);
  if (cfg->tile_texels <= 0 || cfg->tile_texels % cfg->threads)
    return fail(SVBRDF_ERR_INVALID, "tile_texels must be a positive multiple of threads");
  long long tiles = 0;
  int views = 0;
  for (int i = 0; i < n; ++i) {
    const svbrdf_material& m = mats[i];
    if (!m.textures || !m.exp_avg || !m.exp_avg_sq || !m.targets || !m.light_pow || !m.camera_pos || !m.light_pos)
      return fail(SVBRDF_ERR_INVALID, "material %d has a null pointer", i);
    if (m.n_views <= 0 || m.height <= 0 || m.width <= 0 || !(m.size > 0.f))
      return fail(SVBRDF_ERR_INVALID, "material %d has a bad shape", i);
    if (m.n_views > kMaxViews) return fail(SVBRDF_ERR_UNSUPPORTED, "material %d: too many views", i);
    const long long T = (long long)m.height * m.width;
    if (T > (1LL << 30)) return fail(SVBRDF_ERR_UNSUPPORTED, "material %d too large", i);
    tiles += (T + cfg->tile_texels - 1) / cfg->tile_texels;
    views += m.n_views;
  }
  if (tiles > (1LL << 30)) return fail(SVBRDF_ERR_UNSUPPORTED, "too many tiles");
  int ctas = cfg->ctas > 0 ? cfg->ctas : resident_ctas(cfg->threads);
  if (ctas <= 0) return fail(SVBRDF_ERR_CUDA, "could not query the device");
  if (ctas > tiles) ctas = (int)tiles;
  L.n_tiles = (int)tiles;
  L.n_ctas = ctas;
  L.total_views = views;
  size_t o = align_up(sizeof(PlanHeader), 16);
  L.off_mats = o; o += sizeof(MatDesc) * n; o = align_up(o, 16);
  L.off_views = o; o += sizeof(View) * views; o = align_up(o, 16);
  L.off_cta = o; o += sizeof(int) * (ctas + 1); o = align_up(o, 16);
  L.off_order = o; o += sizeof(int) * tiles; o = align_up(o, 16);
  L.off_tiles = o; o += sizeof(int2) * tiles; o = align_up(o, 16);
  L.off_mat_tiles = o; o += sizeof(int) * (n + 1); o = align_up(o, 16);
  L.total = o;
  return SVBRDF_OK;
}

}  // namespace svb

using namespace svb;

namespace svb {
int resident_ctas(int threads) {
  const int sms = device_sm_count();
  if (sms <= 0) return 0;
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
  h->total_bytes = (long long)L.total;
  MatDesc* md = (MatDesc*)(base + L.off_mats);
  View* vw = (View*)(base + L.off_views);
  int* cta_off = (int*)(base + L.off_cta);
  int* order = (int*)(base + L.off_order);
  int2* tiles = (int2*)(base + L.off_tiles);
  int* mat_tiles = (int*)(base + L.off_mat_tiles);
  std::vector<double> cost(L.n_tiles);
  int voff = 0, t = 0;
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
    md[i].H = m.height;
    md[i].W = m.width;
    md[i].V = m.n_views;
    md[i].view_off = voff;
    md[i].size = m.size;
    md[i].scale = (float)(2.0 / N);
    md[i].inv_n = 1.0 / N;
    for (int v = 0; v < m.n_views; ++v) {
      View& w = vw[voff + v];
      w.cx = m.camera_pos[3 * v]; w.cy = m.camera_pos[3 * v + 1]; w.cz = m.camera_pos[3 * v + 2];
      w.lx = m.light_pos[3 * v]; w.ly = m.light_pos[3 * v + 1]; w.lz = m.light_pos[3 * v + 2];
      w.coloc = (w.cx == w.lx && w.cy == w.ly && w.cz == w.lz) ? 1.f : 0.f;
    }
    voff += m.n_views;
    mat_tiles[i] = t;
    for (long long x = 0; x < T; x += config->tile_texels) {
      tiles[t] = make_int2(i, (int)x);
      const long long cnt = std::min<long long>(config->tile_texels, T - x);
      // cost model: per-texel fixed work (decode, adjoint map-back, Adam) ~ 3 views
      cost[t] = (double)cnt * (m.n_views + 3.0);
      total += cost[t];
      ++t;
    }
  }
  mat_tiles[n_materials] = t;
  h->total_cost = total;
  // Longest-processing-time-first assignment to CTAs, then each CTA's tiles sorted by
  // id so consecutive tiles share a material (fewer view re-stages).
  std::vector<int> idx(L.n_tiles);
  std::iota(idx.begin(), idx.end(), 0);
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return cost[a] > cost[b]; });
  std::vector<double> load(L.n_ctas, 0.0);
  std::vector<std::vector<int>> per(L.n_ctas);
  // min-heap over (load, cta)
  std::vector<std::pair<double, int>> heap;
  heap.reserve(L.n_ctas);
  for (int c = 0; c < L.n_ctas; ++c) heap.push_back({0.0, c});
  auto cmp = [](const std::pair<double, int>& a, const std::pair<double, int>& b) {
    return a.first > b.first || (a.first == b.first && a.second > b.second);
  };
  std::make_heap(heap.begin(), heap.end(), cmp);
  for (int ti : idx) {
    std::pop_heap(heap.begin(), heap.end(), cmp);
    auto top = heap.back();
    heap.pop_back();
    per[top.second].push_back(ti);
    top.first += cost[ti];
    heap.push_back(top);
    std::push_heap(heap.begin(), heap.end(), cmp);
  }
  int k = 0;
  for (int c = 0; c < L.n_ctas; ++c) {
    cta_off[c] = k;
    std::sort(per[c].begin(), per[c].end());
    for (int ti : per[c]) order[k++] = ti;
  }
  cta_off[L.n_ctas] = k;
  return SVBRDF_OK;
}

size_t svbrdf_batched_workspace_bytes(const void* host_plan) {
  if (!host_plan) return 0;
  const PlanHeader* h = (const PlanHeader*)host_plan;
  if (h->magic != kPlanMagic) return 0;
  return 256 + sizeof(float) * (size_t)h->n_tiles;
}

int svbrdf_batched_step(const void* device_plan, const void* host_plan, int loss_kind, int* step_counter,
                        float lr, float beta1, float beta2, float eps, float* loss_hist, int hist_len,
                        void* workspace, size_t workspace_bytes, void* stream) {
  if (!device_plan || !host_plan || !loss_hist || !step_counter)
    return fail(SVBRDF_ERR_INVALID, "null plan/step_counter/loss_hist");
  const PlanHeader* h = (const PlanHeader*)host_plan;
  if (h->magic != kPlanMagic) return fail(SVBRDF_ERR_INVALID, "host_plan is not a plan");
  if (loss_kind < SVBRDF_LOSS_MSE || loss_kind > SVBRDF_LOSS_LOG1P_PRE)
    return fail(SVBRDF_ERR_INVALID, "bad loss_kind %d", loss_kind);
  if (hist_len < 1) return fail(SVBRDF_ERR_INVALID, "hist_len must be >= 1");
  const size_t need = svbrdf_batched_workspace_bytes(host_plan);
  if (!workspace || workspace_bytes < need) return fail(SVBRDF_ERR_WORKSPACE, "workspace of %zu bytes needed", need);
  unsigned* counter = (unsigned*)workspace;
  float* tile_loss = (float*)((char*)workspace + 256);
  AdamHyper hyper;
  hyper.lr = lr;
  hyper.beta1 = beta1;
  hyper.beta2 = beta2;
  hyper.eps = eps;
  cudaStream_t st = (cudaStream_t)stream;
  const char* plan = (const char*)device_plan;
#define SVB_B(L, NT) \
  batched_step_kernel<L, NT><<<h->n_ctas, NT, 0, st>>>(plan, hyper, step_counter, loss_hist, hist_len, tile_loss, counter)
#define SVB_BL(NT)                                    \
  if (loss_kind == SVBRDF_LOSS_MSE) SVB_B(0, NT);     \
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

}  // extern "C"
