// Batched work plan shared by the host planner and the persistent kernels.
//
// One contiguous buffer, identical on host and device:
//   PlanHeader | MatDesc[n_mat] | View[total views] | int cta_off[n_ctas+1]
//   | int order[n_tiles] | int2 tiles[n_tiles] (material, first texel)
//   | int mat_tile_off[n_mat+1] | float coord tables (per material: x[W], then y[H])
//   | int4 seq[n_tiles] (order[k]'s tile, material and first texel, in CTA order)
// Tiles of one material are contiguous in tile-index order (mat_tile_off), so each
// material's loss is a fixed-order sum over a tile range. cta_off[c]..cta_off[c+1]
// indexes `order`, the planner's balanced permutation of tile ids for CTA c.
#pragma once

#include "svbrdf_math.cuh"

namespace svb {

struct PlanHeader {
  int magic;
  int n_mat;
  int n_tiles;
  int n_ctas;
  int threads;      // consumer threads per CTA
  int tile_texels;
  int off_mats;     // byte offsets from the plan base
  int off_views;
  int off_cta;
  int off_order;
  int off_tiles;
  int off_mat_tiles;
  int off_coords;
  int variant;      // 0: direct loads, 1: bulk-copy (TMA) pipeline, 2: the pipeline on texel pairs
  int ring_slots;   // variants 1 and 2: shared-memory ring depth
  int general;      // 1 when some material has a view whose light is not at the camera
  int off_seq;      // int4 (tile, material, first texel, 0) per entry of `order`
  int light;        // 1 when some material's light power is learnable (MatDesc::lstate)
  long long total_bytes;
  double total_cost;
};

struct __align__(16) MatDesc {
  float* tex;
  float* m1;
  float* m2;
  const float* tgt;
  float* lpow;
  float* lstate;      // light power Adam state [6] (exp_avg, exp_avg_sq), or null: light fixed
  int H, W, V, view_off;
  float size, scale;  // scale = 2 / (3 V H W), the loss-gradient normaliser
  float inv_w;        // 1 / W for the row/column split of a texel index
  int coord_off;      // float index of this material's x table (y follows at +W)
  int all_coloc;      // 1 when every view has the light at the camera
  int pad;
  double inv_n;       // 1 / (3 V H W)
};

constexpr int kPlanMagic = 0x53564232;  // "SVB2"

// Adam hyper-parameters of a batched launch; the step itself lives on the device so
// one captured graph can be replayed indefinitely.
struct AdamHyper {
  float lr, beta1, beta2, eps;
};

// Workspace of a batched launch: [0] completion counter, [1] error word, then from byte
// 256 the per-(tile, warp) partial losses, then (plans with a learnable light) the
// per-(tile, warp) partial light-power gradients, 3 floats each.
constexpr int kWsCounter = 0;
constexpr int kWsError = 1;
constexpr size_t kWsLossOffset = 256;

// Error codes written to the workspace error word by a kernel that gave up waiting.
enum DeviceError : int {
  kDevOk = 0,
  kDevTimeoutFull = 1,   // a consumer waited too long for a bulk copy
  kDevTimeoutEmpty = 2,  // the producer waited too long for consumers to free a slot
  kDevTimeoutDrain = 3,  // in-flight copies did not land while shutting down
};

}  // namespace svb
