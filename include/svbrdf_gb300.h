/*
 * svbrdf_gb300.h - C ABI of the GB300 (sm_103a) differentiable SVBRDF renderer.
 *
 * Drop-in kernels for the per-pixel hot path of tflsguoyu/svbrdf-diff-renderer:
 * the flash-lit GGX/Cook-Torrance renderer Microfacet.eval (src/microfacet.py:84-120),
 * its autograd backward, and the per-pixel Adam loop SvbrdfOptim.optim
 * (src/svbrdf.py:44-83). The reference is pure Python and has no FFI; these entry
 * points are what its Python classes call through ctypes.
 *
 * Conventions shared by every entry point:
 *  - All tensor pointers are DEVICE pointers to contiguous FP32 data unless marked HOST.
 *    textures are planar [9][H][W] (channels 0:3 diffuse, 3:5 normal xy, 5 roughness,
 *    6:9 specular; the reference's [1,9,H,W], src/microfacet.py:72-77); renders, targets
 *    and render gradients are planar [V][3][H][W]; camera_pos/light_pos are [V][3] in cm;
 *    light_pow is [3].
 *  - `stream` is a cudaStream_t (NULL = the legacy default stream). Every call is
 *    asynchronous and stream-ordered; no call synchronises the device or allocates memory.
 *  - Scratch memory ("workspace") is caller-owned. It must be zero-filled once before
 *    its first use; the library leaves it ready for the next call. Calls that share one
 *    workspace must be ordered on the same stream.
 *  - Return value: SVBRDF_OK (0) or a negative SVBRDF_ERR_* code; svbrdf_last_error()
 *    then returns a message for the calling host thread. The reference instead asserts
 *    (src/microfacet.py:85-86) or prints and exits (src/svbrdf.py:91-92).
 */
#ifndef SVBRDF_GB300_H
#define SVBRDF_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SVBRDF_ABI_VERSION 4

enum {
  SVBRDF_OK = 0,
  SVBRDF_ERR_INVALID = -1,     /* null pointer, bad size, bad enum value */
  SVBRDF_ERR_UNSUPPORTED = -2, /* e.g. more views than svbrdf_max_views() */
  SVBRDF_ERR_CUDA = -3,        /* a CUDA runtime call or kernel launch failed */
  SVBRDF_ERR_WORKSPACE = -4    /* workspace missing or too small */
};

/* Image loss. MSE is the reference's nn.MSELoss on the gamma-encoded renders
 * (src/optimization.py:14,28-29). LOG1P is mean((log1p(render)-log1p(target))^2);
 * LOG1P_PRE is the same with the targets already passed as log1p(target). */
enum {
  SVBRDF_LOSS_NONE = -1,
  SVBRDF_LOSS_MSE = 0,
  SVBRDF_LOSS_LOG1P = 1,
  SVBRDF_LOSS_LOG1P_PRE = 2
};

/* Message for the last failed call on this host thread ("" if none). */
const char* svbrdf_last_error(void);
int svbrdf_abi_version(void);
/* Largest view count a single material may have. */
int svbrdf_max_views(void);
/* Workspace bytes for svbrdf_render_fwd / svbrdf_render_bwd / svbrdf_fused_step. */
size_t svbrdf_workspace_bytes(void);

/* Forward render: out = Microfacet(res, V, size, cl).eval(textures).
 * Replaces Microfacet.eval, src/microfacet.py:84-120 (construction :10-26 folds into the
 * arguments). `out` may be NULL when only the loss is wanted. With loss_kind != NONE,
 * `targets` [V][3][H][W] and `loss_out` (one device float) are required and the mean loss
 * is written to *loss_out (src/optimization.py:28-29). */
int svbrdf_render_fwd(const float* textures, const float* camera_pos, const float* light_pos,
                      const float* light_pow, int n_views, int height, int width, float size,
                      float* out, const float* targets, int loss_kind, float* loss_out,
                      void* workspace, size_t workspace_bytes, void* stream);

/* Adjoint of svbrdf_render_fwd: given dL/d(render) `grad_out` [V][3][H][W], writes
 * dL/d(textures) to `grad_textures` [9][H][W] (overwritten) and, when `grad_light_pow`
 * is not NULL, dL/d(light_pow) [3] (overwritten). Replaces the autograd graph of
 * Microfacet.eval (src/microfacet.py:84-120, backward through src/svbrdf.py:70). The
 * forward terms are recomputed, nothing is saved between the two calls. */
int svbrdf_render_bwd(const float* textures, const float* camera_pos, const float* light_pos,
                      const float* light_pow, int n_views, int height, int width, float size,
                      const float* grad_out, float* grad_textures, float* grad_light_pow,
                      void* workspace, size_t workspace_bytes, void* stream);

/* The same two calls over a leading batch of `batch` materials of one shape, all under the same
 * views and light (the reference's Microfacet.eval on textures [B, 9, H, W], which renders to
 * [B * n_views, 3, H, W], src/microfacet.py:84-120): textures [batch][9][H][W], out / targets /
 * grad_out [batch][n_views][3][H][W], grad_textures [batch][9][H][W]; the loss is the mean over
 * the whole batch and grad_light_pow sums over it. One launch each. */
int svbrdf_render_fwd_batch(const float* textures, const float* camera_pos, const float* light_pos,
                            const float* light_pow, int n_views, int height, int width, float size, int batch,
                            float* out, const float* targets, int loss_kind, float* loss_out, void* workspace,
                            size_t workspace_bytes, void* stream);
int svbrdf_render_bwd_batch(const float* textures, const float* camera_pos, const float* light_pos,
                            const float* light_pow, int n_views, int height, int width, float size, int batch,
                            const float* grad_out, float* grad_textures, float* grad_light_pow, void* workspace,
                            size_t workspace_bytes, void* stream);

/* One fused iteration of SvbrdfOptim.optim (src/svbrdf.py:56-71): render of
 * clamp(textures, -1, 1), image loss, adjoint and torch.optim.Adam update
 * (betas beta1/beta2, eps, no weight decay, 1-based `step` after this update), in one
 * pass over the texels. textures, exp_avg and exp_avg_sq are updated in place; the mean
 * loss of the pre-update textures goes to *loss_out. With `light_adam_state` non-NULL the
 * light power is learnable (src/svbrdf.py:48-50, 58-59): light_pow [3] is then updated in
 * place by Adam with state light_adam_state [6] = {exp_avg[3], exp_avg_sq[3]}. */
int svbrdf_fused_step(float* textures, float* exp_avg, float* exp_avg_sq, const float* targets,
                      const float* camera_pos, const float* light_pos, float* light_pow,
                      float* light_adam_state, int n_views, int height, int width, float size,
                      int loss_kind, int step, float lr, float beta1, float beta2, float eps,
                      float* loss_out, void* workspace, size_t workspace_bytes, void* stream);

/* svbrdf_fused_step without a workspace argument. This entry point has no counterpart in
 * the reference; it exists for callers that cannot allocate device memory at the point
 * where they step the optimiser: for example a host application that hands this library
 * only the tensors it already owns from its own memory pool, or that calls it from code
 * where cudaMalloc is not allowed. Arguments and results are those of svbrdf_fused_step.
 * The scratch it needs (a completion counter and one 16-byte partial sum per CTA) lives in
 * a static device array of 16 + 2048*16 bytes inside the library, so a step may use at
 * most 2048 CTAs (a GB300 uses about 300); a call that would need more returns
 * SVBRDF_ERR_UNSUPPORTED. The call itself allocates nothing: no cudaMalloc, no cudaFree.
 * The first call on each device looks the array up with cudaGetSymbolAddress, with that
 * device current; make that first call before any stream capture. Every call clears the
 * counter with cudaMemsetAsync on `stream` before its launch. All calls share the one
 * array, so calls whose kernels overlap on the GPU (different streams, no ordering between
 * them) race on it and give wrong losses; order them on one stream. */
int svbrdf_fused_step_noalloc(float* textures, float* exp_avg, float* exp_avg_sq, const float* targets,
                              const float* camera_pos, const float* light_pos, float* light_pow,
                              float* light_adam_state, int n_views, int height, int width, float size,
                              int loss_kind, int step, float lr, float beta1, float beta2, float eps,
                              float* loss_out, void* stream);

/* ---- batched: many materials of uneven resolution and view count in one launch ---- */

/* One material of a batch. Device pointers except camera_pos/light_pos (HOST, read by the
 * planner only). Each material is what one SvbrdfOptim instance owns.
 * With light_adam_state non-NULL the material's light power is learnable, as with
 * SvbrdfOptim.optim(..., optim_light=True) (src/svbrdf.py:48-50, 58-59): light_pow is then
 * updated in place each iteration by the same Adam as the maps (one optimiser over
 * [textures, light_pow], src/svbrdf.py:50), with state light_adam_state [6] =
 * {exp_avg[3], exp_avg_sq[3]} (zeroed by the caller before the first step). The light is
 * shared by every texel, so its gradient is a reduction over the whole material each
 * iteration: such plans need variant 2 or 3, and variant 3 then runs one iteration per
 * launch. Without it light_pow is only read. */
typedef struct svbrdf_material {
  float* textures;         /* [9][H][W], updated in place */
  float* exp_avg;          /* [9][H][W] Adam first moment */
  float* exp_avg_sq;       /* [9][H][W] Adam second moment */
  const float* targets;    /* [V][3][H][W] */
  float* light_pow;        /* [3]; written only when light_adam_state is non-NULL */
  const float* camera_pos; /* HOST [V][3] */
  const float* light_pos;  /* HOST [V][3] */
  int n_views;
  int height;
  int width;
  float size;
  float* light_adam_state; /* [6] or NULL (light power fixed) */
} svbrdf_material;

/* Launch shape of the persistent batched kernel (chosen by the autotuner).
 * variant 0 (direct loads): threads 128, 256 or 512; tile_texels a multiple of threads.
 * variant 1 (bulk-copy pipeline: one producer warp streams planes into a shared-memory
 *   ring with cp.async.bulk, `threads` consumer threads compute from it): threads 256,
 *   384, 480 or 608, tile_texels == threads; every material needs H*W % 4 == 0 and 16-byte
 *   aligned textures/exp_avg/exp_avg_sq/targets.
 * variant 2 (the variant 1 pipeline with two adjacent texels per consumer thread, every
 *   per-texel stage in FP32x2): threads 224, 256, 384 or 480, tile_texels == 2 * threads,
 *   the material requirements of variant 1. threads 224 runs two CTAs per SM.
 * variant 3 (resident state: the variant 2 arithmetic, but a launch runs up to 32
 *   iterations on each tile, keeping the tile's parameters and Adam moments in shared
 *   memory between them, so HBM carries them once per launch; only the targets stream per
 *   iteration, from L2 after the first): threads 224, 256, 384 or 480, tile_texels ==
 *   2 * threads, the material requirements of variant 1. Use svbrdf_batched_steps.
 * variant 4 (variant 3 without the producer warp: the last warp to finish with a ring slot
 *   or the state refills it, so all warps compute): threads 256 (two CTAs per SM) or 512,
 *   tile_texels == 2 * threads, the material requirements of variant 1.
 * ctas: persistent CTAs (0 = SM count x resident CTAs per SM). */
typedef struct svbrdf_batch_config {
  int threads;
  int tile_texels;
  int ctas;
  int variant;
} svbrdf_batch_config;

/* Workspace of svbrdf_batched_step: the int32 at byte offset 4 is a device error word,
 * 0 while healthy. A pipelined launch that waited too long for its copies or consumers
 * stores a non-zero code there (1: copy never landed, 2: consumers stalled, 3: drain
 * timeout), skips the rest of its work and returns; the caller reads the word after
 * synchronising and treats non-zero as a failed step. */
#define SVBRDF_WORKSPACE_ERROR_OFFSET 4

/* Self-test of the batched kernels' failure path: a one-warp kernel waits on an mbarrier
 * phase that nothing completes, gives up after `limit` polls (at most 2^24), stores 1 (the
 * "copy never landed" code) in the error word at byte SVBRDF_WORKSPACE_ERROR_OFFSET, and
 * returns with the context usable. Bytes 8 and 12 receive 1 and 0: a wait its own arrival
 * completed, and the one that ran out. The workspace must start zeroed (16 bytes). */
int svbrdf_selftest_wait_timeout(void* workspace, size_t workspace_bytes, int limit, void* stream);

/* Bytes of the plan for this batch (0 on error). */
size_t svbrdf_batched_plan_bytes(const svbrdf_material* materials, int n_materials,
                                 const svbrdf_batch_config* config);
/* Build the plan (material table, views, work list balanced across CTAs) into a HOST
 * buffer. The caller copies it verbatim into a device buffer of the same size. */
int svbrdf_batched_plan(const svbrdf_material* materials, int n_materials,
                        const svbrdf_batch_config* config, void* host_plan, size_t plan_bytes);
/* Workspace bytes for svbrdf_batched_step with this plan. */
size_t svbrdf_batched_workspace_bytes(const void* host_plan);
/* One fused render+adjoint+Adam iteration for every material of the plan, in one
 * persistent launch (the loop body of src/svbrdf.py:56-71 for each material). All
 * materials share the Adam hyper-parameters. The step count lives on the device:
 * `step_counter` (one int, 0 before the first iteration) is read by the launch, which
 * uses step = *step_counter + 1 and stores it back when done, so a CUDA graph of these
 * launches can be replayed any number of times. The mean loss of material m for that
 * step goes to loss_hist[((step - 1) % hist_len) * n_materials + m]. */
int svbrdf_batched_step(const void* device_plan, const void* host_plan, int loss_kind, int* step_counter,
                        float lr, float beta1, float beta2, float eps, float* loss_hist, int hist_len,
                        void* workspace, size_t workspace_bytes, void* stream);
/* `iters` iterations of svbrdf_batched_step (the whole `for epoch in range(epochs)` loop of
 * src/svbrdf.py:56-71 for every material). Variants 0-2 launch once per iteration; variants
 * 3 and 4 run ceil(iters / 32) launches of up to 32 iterations each. The parameters, moments, step
 * counter and loss history afterwards equal those of `iters` svbrdf_batched_step calls. */
int svbrdf_batched_steps(const void* device_plan, const void* host_plan, int loss_kind, int* step_counter,
                         float lr, float beta1, float beta2, float eps, float* loss_hist, int hist_len, int iters,
                         void* workspace, size_t workspace_bytes, void* stream);

/* ---- descriptor loss: BF16 3x3 convolutions on the tensor cores ---- */

/* y = epilogue(conv3x3(x, weight)), stride 1, zero padding 1, for the VGG-feature loss of
 * VGGLoss (src/descriptor.py:7-79; the reference runs torchvision's VGG19, :13, 43).
 * x: BF16 NHWC [n][h][w][cin]; weight: BF16 [cout][9][cin] (tap = 3*ky + kx); y: BF16 NHWC
 * [n][h][w][cout]. h % 8 == 0, w % 16 == 0, cin and cout multiples of 64; 16-byte aligned.
 * epilogue 0: none; 1: bias [cout] (FP32) then ReLU; 2: multiply by (mask > 0), mask BF16
 * NHWC like y (a ReLU mask for the backward pass). The data gradient dL/dx of a convolution
 * is this call on dL/d(pre-activation) with weight'[cin][8 - tap][cout] = weight[cout][tap][cin].
 * FP32 accumulation in tensor memory. `err` (one device int, zeroed by the caller) receives a
 * non-zero code if a launch gave up waiting on its pipeline. */
int svbrdf_conv3x3_bf16(const void* x, const void* weight, const float* bias, const void* mask, void* y, int n,
                        int h, int w, int cin, int cout, int epilogue, int* err, void* stream);

/* As svbrdf_conv3x3_bf16, plus epilogue 3: (acc + addend) * (mask > 0), addend BF16 NHWC like
 * y. In the descriptor's backward pass this adds a hooked layer's loss gradient to the data
 * gradient arriving from the layer above and applies that hooked ReLU's mask, in one pass
 * (the autograd graph of src/descriptor.py:77-79 does the add, the mask and the next
 * convolution as separate kernels).
 * Epilogues 4 and 5 fold the backward pass of a 2x2 pool (stride 2) that precedes this
 * convolution in the forward pass: the result (the gradient at the pool's output, h x w) is
 * routed to the pool's input, mask BF16 NHWC [n][2h][2w][cout] -- to the first maximum of each
 * window in row-major order (4, a max-pool, as ATen routes it) or a quarter to each element
 * (5, an average pool) -- plus addend (BF16 like mask, or null) there, times (mask > 0) (the
 * ReLU below the pool), written to y [n][2h][2w][cout]. One pass replaces the pool's backward
 * kernel and the round trip of the pooled gradient through memory. */
int svbrdf_conv3x3_bf16_ex(const void* x, const void* weight, const float* bias, const void* mask,
                           const void* addend, void* y, int n, int h, int w, int cin, int cout, int epilogue,
                           int* err, void* stream);

/* ---- descriptor loss: fused glue around the convolutions (no counterpart kernels in the
 * reference, whose VGGLoss runs torchvision modules and autograd, src/descriptor.py:7-79) ---- */

/* Number of per-block partial sums svbrdf_desc_feat_loss writes. */
int svbrdf_desc_partials(void);

/* The loss scalars from their partial sums in one launch: out[j] = sum over the segments k with
 * groups[k] == j (j = 0, 1) of weights[k] x (sum of the lengths[k] floats at buf + offsets[k]),
 * added in a fixed order (FP32 within a thread's share of a segment, double across them; 1 to 16
 * segments; host arrays). For the
 * descriptor: group 0 the feature terms' partials (weights w_k^2 / n_features), group 1 the
 * Gram terms' loss rows (weights w_k^2 / n_gram), as VGGLoss.forward weights them
 * (src/descriptor.py:77-79). */
int svbrdf_desc_loss_sums(const float* buf, int n_segs, const long long* offsets, const long long* lengths,
                          const double* weights, const int* groups, float* out, void* stream);

/* 2x2 box downsample (if `downsample`) of renders [v][3][2h][2w] FP32, ImageNet normalisation
 * with the reference's statistics (src/descriptor.py:65-75), conv1_1 (weight [64][3][3][3],
 * bias [64], FP32, zero padding 1) and ReLU. Writes NHWC [v][h][w][64] in FP32 (out_f32) and
 * BF16 (out_bf16). */
int svbrdf_desc_conv1_fwd(const float* renders, const float* weight, const float* bias, float* out_f32,
                          void* out_bf16, int v, int h, int w, int downsample, void* stream);

/* Data gradient of svbrdf_desc_conv1_fwd before its ReLU: gz BF16 NHWC [v][h][w][64] (the
 * masked gradient at conv1_1's output) -> grad_renders FP32 [v][3][2h][2w] (or [v][3][h][w]
 * without `downsample`), overwritten. */
int svbrdf_desc_conv1_bwd(const void* gz, const float* weight, float* grad_renders, int v, int h, int w,
                          int downsample, void* stream);

/* The same data gradient on the tensor cores: the 64 -> 3 channel 3x3 convolution as a BF16
 * tcgen05 implicit GEMM (N = 16: weight rows 3..15 zero), FP32 accumulation. w16: BF16
 * [16][9][64], row c, tap 3 ky + kx, channel k = conv1_1's weight[k][c][2 - ky][2 - kx] for
 * c < 3. scale[c] (FP32, 3 values) multiplies channel c: 1 / std[c] of the normalisation, times
 * 1/4 with `downsample` (the box filter's adjoint gives each of the window's 4 render pixels
 * the scaled value). h % 8 == 0, w % 16 == 0; gz and w16 16-byte aligned, grad_renders
 * 8-byte aligned. `err` as in svbrdf_conv3x3_bf16. */
int svbrdf_desc_conv1_bwd_tc(const void* gz, const void* w16, const float* scale, float* grad_renders, int v, int h,
                             int w, int downsample, int* err, void* stream);

/* 2x2 max-pool, BF16 NHWC [v][h][w][c] -> [v][h/2][w/2][c]; h, w even, c % 8 == 0. */
int svbrdf_desc_pool_fwd(const void* x, void* y, int v, int h, int w, int c, void* stream);

/* Max-pool backward fused with a hook gradient and a ReLU mask: gx = (route(gy) + addend) *
 * (x > 0), where x [v][h][w][c] is the pool's input (a ReLU output), gy [v][h/2][w/2][c] the
 * gradient at its output, addend (nullable) like x. The first maximum of each 2x2 window in
 * row-major order takes the gradient, as ATen's max-pool does. BF16 throughout. */
int svbrdf_desc_pool_bwd(const void* gy, const void* x, const void* addend, void* gx, int v, int h, int w, int c,
                         void* stream);

/* The same pair with 2x2 average pools (the reference's VGGLoss replaces VGG19's max-pools
 * with average pools, src/descriptor.py:16-19): each window element takes gy / 4. */
int svbrdf_desc_avgpool_fwd(const void* x, void* y, int v, int h, int w, int c, void* stream);
int svbrdf_desc_avgpool_bwd(const void* gy, const void* x, const void* addend, void* gx, int v, int h, int w, int c,
                            void* stream);

/* Feature term of one hook: partial[b] (b < svbrdf_desc_partials(), if partial) = block b's
 * share of sum (f - t)^2, a fixed-order split; if g: g = coef (f - t) + gram_grad (nullable),
 * times (f > 0) if `mask`, stored BF16. f is BF16 (f_is_bf16) or FP32, t and gram_grad FP32,
 * all n elements. */
int svbrdf_desc_feat_loss(const void* f, int f_is_bf16, const float* t, const float* gram_grad, float coef, int mask,
                          void* g, float* partial, long long n, void* stream);

/* ---- descriptor loss: the Gram term on the tensor cores (the reference's Gram branch
 * G = F F^T / S, src/descriptor.py:50-56, for NHWC features F [V][S][C]) ---- */

/* Split count (over the pixels) that svbrdf_desc_gram should use for v views of s pixels and
 * c channels (0 for unsupported sizes). */
int svbrdf_desc_gram_splits(int v, int s, int c);

/* partial[v][split][c][c] = sum over split `split` of the pixels of F[v][p][i] F[v][p][j]: BF16
 * features [v][s][c] (s % 64 == 0; c 64, 128 or a multiple of 256; 16-byte aligned), FP32
 * partial products (tcgen05, FP32 accumulation). `err` as in svbrdf_conv3x3_bf16. */
int svbrdf_desc_gram(const void* features, float* partial, int v, int s, int c, int splits, int* err, void* stream);

/* G[v][i][j] = (sum over splits of partial, in split order) / s; with gram_target (FP32
 * [v][c][c], nullable) d = G - target, else d = G. Writes, each when non-NULL: gram_out = G
 * (FP32), dgram = coef d (BF16), loss_part[v][i] = sum_j d^2 (FP32, fixed order). */
int svbrdf_desc_gram_finish(const float* partial, int splits, int v, int c, int s, const float* gram_target,
                            float coef, float* gram_out, void* dgram, float* loss_part, void* stream);

/* out[b][m][n] = sum_k A[b][m][k] B[b][n][k] (FP32), A BF16 [batch][m][k], B BF16 [batch][n][k]:
 * m % 128 == 0, k % 64 == 0, n 64, 128 or a multiple of 256, 16-byte aligned. For the Gram term's
 * gradient dF = F dG (dG symmetric, so B = dG). */
int svbrdf_desc_gemm_nt(const void* a, const void* b, float* out, int batch, int m, int n, int k, int* err,
                        void* stream);

/* The Gram gradient dF = F dG with the feature term of the same hook in its epilogue (the
 * reference's feature + Gram loss of one hooked layer, src/descriptor.py:39-60, 77-79): per
 * element of the [batch * m, n] maps, d = f - t, g = coef d + dF, times (f > 0) if `mask`,
 * stored BF16 (as svbrdf_desc_feat_loss with gram_grad = dF, which then never reaches memory);
 * partial[i] (i < svbrdf_desc_gemm_nt_feat_partials(batch, m, n)) = a fixed-order share of
 * sum d^2. a = the hook's BF16 features [batch][m][k = n], b = dG BF16 [batch][n][n]; f is the
 * same map as a or its FP32 original, t BF16 or FP32: `dtypes` bit 0 set = f is BF16, bit 1 set
 * = t is BF16 (a BF16 hook's target features lose nothing in BF16 and cost 2 bytes fewer per
 * element). Shapes as svbrdf_desc_gemm_nt. */
long long svbrdf_desc_gemm_nt_feat_partials(int batch, int m, int n);
int svbrdf_desc_gemm_nt_feat(const void* a, const void* b, const void* f, int dtypes, const void* t, float coef,
                             int mask, void* g, float* partial, int batch, int m, int n, int k, int* err,
                             void* stream);

/* ---- MaterialGAN generator: 2x up-sampling of its feature maps and skip images (the
 * reference's generator, src/higan_models/*, up-samples by zero insertion and a [1,3,3,1]
 * FIR; src/materialgan.py:91-173 runs it in the latent loop) ---- */

/* y [planes][2h][2w] = zero insertion of x [planes][h][w], then the separable [1,3,3,1]^2 / 64
 * FIR with gain 4 and zero padding: along each axis out[2m] = (x[m-1] + 3 x[m]) / 4 and
 * out[2m+1] = (3 x[m] + x[m+1]) / 4. FP32, contiguous planes. */
int svbrdf_gen_upsample2(const float* x, float* y, long long planes, int h, int w, void* stream);

/* svbrdf_gen_upsample2 of x[p] s[p] (a modulated up-sampling conv's input scaling, which
 * commutes with the up-sampling), s nullable. Needs w % 4 == 0 and 16-byte aligned x, y. */
int svbrdf_gen_upsample2_scaled(const float* x, const float* s, float* y, long long planes, int h, int w,
                                void* stream);

/* The adjoint of svbrdf_gen_upsample2: gx [planes][h][w] from g [planes][2h][2w]. */
int svbrdf_gen_upsample2_bwd(const float* g, float* gx, long long planes, int h, int w, void* stream);

/* ---- MaterialGAN generator: a style layer's elementwise work around its modulated conv (the
 * reference's StyleGAN2 layer in src/higan_models/*: input channels scaled by the style, output
 * channels by the demodulation, then per-layer noise, bias and leaky ReLU x sqrt 2) ---- */

/* y[p][i] = x[p][i] s[p] over planes p = b C + c (planes <= 65535), hw elements per plane. */
int svbrdf_gen_scale(const float* x, const float* s, float* y, long long planes, int hw, void* stream);

/* Adjoint of svbrdf_gen_scale: gx = g s[p] and gs[p] = sum_i g[p][i] x[p][i] (fixed order). */
int svbrdf_gen_scale_bwd(const float* g, const float* x, const float* s, float* gx, float* gs, long long planes,
                         int hw, void* stream);

/* out[b][c][i] = lrelu(y[b][c][i] d[b][c] + ns noise[b][i] + bias[c], 0.2) gain. d nullable
 * (taken as 1), noise nullable (no noise term); ns points at the device scalar noise strength. */
int svbrdf_gen_act(const float* y, const float* d, const float* noise, const float* ns, const float* bias, float gain,
                   float* out, int b, int c, int hw, void* stream);

/* Adjoint of svbrdf_gen_act with respect to y, d and noise: gy = gpre d, gd[b][c] = sum_i gpre y
 * (gd nullable), gnoise[b][i] = ns sum_c gpre (gnoise nullable), gpre = gout gain slope. */
int svbrdf_gen_act_bwd(const float* gout, const float* y, const float* d, const float* noise, const float* ns,
                       const float* bias, float gain, float* gy, float* gd, float* gnoise, int b, int c, int hw,
                       void* stream);

/* ---- the same generator work on channels-last maps [b][h][w][c] (the layout cuDNN's
 * convolutions run in, so the generator needs no NCHW<->NHWC conversions). float4 over channels
 * when c % 4 == 0 and the maps are 16-byte aligned. The backward calls with column sums take a
 * scratch `part` of svbrdf_gen_nhwc_partial_floats(b, c) floats and are deterministic. ---- */

/* Floats of the `part` scratch the *_nhwc_bwd calls need. */
int svbrdf_gen_nhwc_partial_floats(int b, int c);

/* y [b][2h+2 halo][2w+2 halo][c] = 2x up-sampling (as svbrdf_gen_upsample2) of x [b][h][w][c],
 * times s[b][c] when s is not null. halo 0 or 1: with 1 the map also holds the up-sampled
 * samples at -1 and 2h (2w), x[0] / 4 and x[h-1] / 4 along each axis. A valid (unpadded) 3x3
 * convolution of that map is the reference's up-sampling convolution: a stride-2 transposed
 * convolution followed by the [1,3,3,1] filter (src/higan_models/stylegan2_generator_network.py:
 * 727-735); a zero-padded convolution of the halo-free map differs from it on the border. */
int svbrdf_gen_upsample2_nhwc(const float* x, const float* s, float* y, int b, int h, int w, int c, int halo,
                              void* stream);

/* Adjoint of the up-sampling: gx [b][h][w][c] from g [b][2h+2 halo][2w+2 halo][c]. */
int svbrdf_gen_upsample2_nhwc_bwd(const float* g, float* gx, int b, int h, int w, int c, int halo, void* stream);

/* The toRGB layer's epilogue (the reference's ToRGB output plus the up-sampled skip image,
 * src/higan_models/stylegan2_generator_network.py): img [b][c][h][w] (NCHW) = yp[b][y][x][ch]
 * (channels-last, cp >= c channels per pixel: the 1x1 convolution's padded output) + bias[ch]
 * + up2(prev) (prev NCHW [b][c][h/2][w/2], nullable; the 2x up-sampling of
 * svbrdf_gen_upsample2). The adjoint writes gyp = g for ch < c and 0 for the padding channels;
 * prev's gradient is svbrdf_gen_upsample2_bwd of g. */
int svbrdf_gen_rgb_nhwc(const float* yp, int cp, const float* bias, const float* prev, float* img, int b, int c, int h,
                        int w, void* stream);
int svbrdf_gen_rgb_nhwc_bwd(const float* g, float* gyp, int cp, int b, int c, int h, int w, void* stream);

/* y[b][p][c] = x[b][p][c] s[b][c], hw pixels. */
int svbrdf_gen_scale_nhwc(const float* x, const float* s, float* y, int b, int hw, int c, void* stream);

/* gx = g s[b][c]; gs[b][c] = sum_p g x. c / 4 (c % 4 == 0) or c at most 256. */
int svbrdf_gen_scale_nhwc_bwd(const float* g, const float* x, const float* s, float* gx, float* gs, float* part, int b,
                              int hw, int c, void* stream);

/* out = lrelu(y d[b][c] + ns noise[b][p] + bias[c], 0.2) gain; d and noise nullable. */
int svbrdf_gen_act_nhwc(const float* y, const float* d, const float* noise, const float* ns, const float* bias,
                        float gain, float* out, int b, int hw, int c, void* stream);

/* Adjoint of svbrdf_gen_act_nhwc: gy, gd[b][c] = sum_p gpre y (nullable), gnoise[b][p] =
 * ns sum_c gpre (nullable). */
int svbrdf_gen_act_nhwc_bwd(const float* gout, const float* y, const float* d, const float* noise, const float* ns,
                            const float* bias, float gain, float* gy, float* gd, float* gnoise, float* part, int b,
                            int hw, int c, void* stream);

/* A style layer's epilogue fused with the next layer's input scaling, for an output whose only
 * consumer is that layer (the generator's up-sampling layers feed only the convolution after
 * them): out = lrelu(y d + ns noise + bias, 0.2) gain s2[b][c] is written, the unscaled map is
 * not. The adjoint takes dL/d out and gives gy, gd, gnoise as svbrdf_gen_act_nhwc_bwd and
 * gs2[b][c] = sum over the pixels of dL/d out x (the unscaled output), with a second scratch of
 * svbrdf_gen_nhwc_partial_floats(b, c) floats for its column sums. */
int svbrdf_gen_act_scale_nhwc(const float* y, const float* d, const float* noise, const float* ns, const float* bias,
                              float gain, const float* s2, float* out, int b, int hw, int c, void* stream);
int svbrdf_gen_act_scale_nhwc_bwd(const float* gout, const float* y, const float* d, const float* noise, const float* ns,
                                  const float* bias, float gain, const float* s2, float* gy, float* gd, float* gs2,
                                  float* gnoise, float* part, float* part2, int b, int hw, int c, void* stream);

/* ---- MaterialGAN generator: its convolutions in TF32 on the tensor cores (the reference's
 * modulated convolutions, src/higan_models/stylegan2_generator_network.py:585-759, computed as a
 * shared-weight convolution between the modulation and demodulation kernels above) ---- */

/* y [b][ho][wo][cout] = k x k convolution (ksize 3 or 1) of x [b][hin][win][cin] with weight
 * [cout][ksize*ksize][cin] (tap = 3 ky + kx), zero padding `pad` (0..2 for 3x3, 0 for 1x1):
 * ho = hin + 2 pad - (ksize - 1). FP32 data, TF32 products, FP32 accumulation in tensor memory.
 * cin % 32 == 0; cout 32, 64, 128 or a multiple of 256; wo >= 4; 16-byte aligned. The data
 * gradient of a convolution is this call on dL/dY with weight'[cin][8 - tap][cout] =
 * weight[cout][tap][cin] and pad' = ksize - 1 - pad. `err` as in svbrdf_conv3x3_bf16. */
int svbrdf_gen_conv_tf32(const float* x, const float* weight, float* y, int b, int hin, int win, int cin, int cout,
                         int ksize, int pad, int* err, void* stream);

/* The same convolution with a caller-owned workspace: a map with fewer output tiles than half
 * the SMs (the generator's 4^2 to 16^2 layers) splits K over the tiles' CTAs, each split writing
 * an FP32 partial of y into ws, then sums the partials in split order (deterministic).
 * svbrdf_gen_conv_tf32_ws_bytes gives the bytes such a call uses (0: no split; -1: an
 * unsupported shape); with a smaller or NULL ws the call runs unsplit, as svbrdf_gen_conv_tf32. */
long long svbrdf_gen_conv_tf32_ws_bytes(int b, int hin, int win, int cin, int cout, int ksize, int pad);
int svbrdf_gen_conv_tf32_ex(const float* x, const float* weight, float* y, void* ws, long long ws_bytes, int b,
                            int hin, int win, int cin, int cout, int ksize, int pad, int* err, void* stream);

/* ---- novel-view rendering under an environment map (the reference's MitsubaRender,
 * src/mitsubarender.py:7-105, for the video of src/scripts.py:44-59) ---- */

/* image [res][res][3] (clipped to [0, 1], raised to 1/2.2) of the material textures
 * [9][h][w] (parameters in [-1, 1]) on the reference's rectangle, turned Ry(angle_deg)
 * Rx(-15) Rz(-5) and scaled by 0.3, seen by a 50-degree camera at (0, 0, 1), lit by the
 * lat-long environment env [he][we][3] (linear radiance, times `intensity`). Direct
 * illumination, spp samples per pixel, each one environment sample (row_cdf [he+1], row_pdf
 * [he], col_cdf [he][we+1], col_pdf [he][we]: luminance x sin(theta) tables) and one BSDF
 * sample, power-heuristic weights; random numbers hashed from (seed, pixel, sample, dim). */
int svbrdf_envmap_render(const float* textures, int h, int w, const float* env, int he, int we, const float* row_cdf,
                         const float* row_pdf, const float* col_cdf, const float* col_pdf, float* image, int res,
                         float angle_deg, float intensity, int spp, unsigned seed, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SVBRDF_GB300_H */
