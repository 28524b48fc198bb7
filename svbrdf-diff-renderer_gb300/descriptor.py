"""Descriptor (VGG-feature) loss with BF16 tensor-core convolutions.

The reference's ``VGGLoss`` (src/descriptor.py:7-79) normalises the renders with ImageNet
statistics (mean 0.485/0.456/0.406, std 0.229/0.224/0.255, :65-75), runs torchvision's VGG19
``.features``, hooks four ReLU outputs (:26-27) and takes the MSE of the weighted, flattened
features against the targets' (:39-60, 77-79); a Gram-matrix branch exists but is off (:50-56).

Here the stack is VGG19-shaped up to conv4_1 (conv1_1..conv4_1, 3x3 kernels, ReLU, 2x2
max-pool) with seeded He-normal weights (pretrained ImageNet weights are not available
offline), the renders are 2x2 box-downsampled first, and both terms are on:

* feature L2: mean over the concatenated weighted features of (w F - w F_t)^2, as in
  ``compute_feature_vector`` + ``MSELoss``;
* Gram: the same over the weighted Gram matrices G = F F^T / S (S = H W of the layer).

Hooks: relu1_1, relu1_2, relu3_2, relu4_1 (the reference hooks relu4_2, which lies past
conv4_1), weights [1, 1, 1, 1] / 4 (the reference's default).

``mode="reference"`` runs the reference's own semantics instead: VGG19 to relu4_2 with
average pools, hooks relu1_1, relu1_2, relu3_2, relu4_2, no downsample, no Gram term.

Every 3x3 convolution with 64 or more input channels runs as a tcgen05 implicit GEMM
(``svbrdf_conv3x3_bf16``: BF16 operands, FP32 accumulation in TMEM, bias + ReLU fused).
Its data gradient is the same kernel on the transposed, flipped weights. The glue around
them is fused into a few kernels of the same library:

* conv1_1 (3 input channels, under 1% of the FLOPs) with the downsample and the
  normalisation in front of it, FP32;
* NHWC max-pools;
* the feature term with its gradient.

The backward pass is a hand-written chain, not autograd. Each data-gradient convolution's
epilogue adds the next hook's loss gradient and applies the ReLU mask below, and the
max-pool backward does the same. The Gram products run on tcgen05 too (gram_tc.cu): G = F^T F
straight from the NHWC feature map (MN-major operands, split over the pixels, partials summed
in a fixed order by a finish kernel that also forms the loss rows and the BF16 dG), and the
gradient F dG as a K-major BF16 GEMM; BF16 operands, FP32 accumulation.
"""
from __future__ import annotations

import ctypes
import math
from typing import List, Optional, Sequence

import torch

from . import _native as N

MEAN = (0.485, 0.456, 0.406)
STD = (0.229, 0.224, 0.255)  # the reference's std for blue is 0.255 (src/descriptor.py:69)
# (name, cin, cout) in order; "pool" = 2x2 max-pool
VGG19_TO_CONV4_1 = [("conv1_1", 3, 64), ("conv1_2", 64, 64), "pool", ("conv2_1", 64, 128), ("conv2_2", 128, 128),
                    "pool", ("conv3_1", 128, 256), ("conv3_2", 256, 256), ("conv3_3", 256, 256),
                    ("conv3_4", 256, 256), "pool", ("conv4_1", 256, 512)]
HOOKS = ("conv1_1", "conv1_2", "conv3_2", "conv4_1")  # their ReLU outputs
# The reference's own stack: VGG19 up to relu4_2 (src/descriptor.py:26-27 hooks features
# 1, 3, 13, 22 = relu1_1, relu1_2, relu3_2, relu4_2), its max-pools swapped for average pools
# (:16-19), full-resolution renders and the feature term alone (is_gram off, :77-79).
VGG19_TO_CONV4_2 = VGG19_TO_CONV4_1 + [("conv4_2", 512, 512)]
REF_HOOKS = ("conv1_1", "conv1_2", "conv3_2", "conv4_2")

EPI_NONE, EPI_BIAS_RELU, EPI_MASK, EPI_ADD_MASK, EPI_UNPOOL_MAX, EPI_UNPOOL_AVG = 0, 1, 2, 3, 4, 5


def conv3x3_bf16(x: torch.Tensor, w: torch.Tensor, bias: Optional[torch.Tensor], epilogue: int,
                 err: torch.Tensor, mask: Optional[torch.Tensor] = None) -> torch.Tensor:
    """NHWC BF16 3x3 conv on the tensor cores. ``w`` is [Cout, 9, Cin] BF16."""
    L = N.lib()
    n, h, wd, cin = x.shape
    cout = w.shape[0]
    y = torch.empty(n, h, wd, cout, device=x.device, dtype=torch.bfloat16)
    N.check(L.svbrdf_conv3x3_bf16(x.data_ptr(), w.data_ptr(), N.ptr(bias), N.ptr(mask), y.data_ptr(), n, h, wd, cin,
                                  cout, epilogue, err.data_ptr(), N.stream_handle(x.device)))
    return y


def gram_bf16(f: torch.Tensor, err: torch.Tensor, target: Optional[torch.Tensor] = None, coef: float = 0.0,
              want_dgram: bool = False, rows_out: Optional[torch.Tensor] = None):
    """The Gram term of NHWC BF16 features f [V, H, W, C] on the tensor cores
    (svbrdf_desc_gram + svbrdf_desc_gram_finish): G = F^T F / S per view (FP32 [V, C, C]). With
    ``target``: (None, loss rows [V, C] = sum_j (G - target)^2, BF16 coef (G - target) if
    ``want_dgram``), the rows written into ``rows_out`` when given (a contiguous FP32 [V, C]
    view); without: (G, None, None)."""
    L = N.lib()
    st = N.stream_handle(f.device)
    v, h, w, c = f.shape
    s = h * w
    f = f.contiguous()
    splits = L.svbrdf_desc_gram_splits(v, s, c)
    if splits <= 0:
        raise N.SvbrdfError(-2, f"gram: unsupported shape {tuple(f.shape)}")
    part = torch.empty(v, splits, c, c, device=f.device, dtype=torch.float32)
    N.check(L.svbrdf_desc_gram(f.data_ptr(), part.data_ptr(), v, s, c, splits, err.data_ptr(), st))
    if target is None:
        g = torch.empty(v, c, c, device=f.device, dtype=torch.float32)
        N.check(L.svbrdf_desc_gram_finish(part.data_ptr(), splits, v, c, s, None, 0.0, g.data_ptr(), None, None, st))
        return g, None, None
    rows = rows_out if rows_out is not None else torch.empty(v, c, device=f.device, dtype=torch.float32)
    dg = torch.empty(v, c, c, device=f.device, dtype=torch.bfloat16) if want_dgram else None
    N.check(L.svbrdf_desc_gram_finish(part.data_ptr(), splits, v, c, s, target.data_ptr(), float(coef), None,
                                      N.ptr(dg), rows.data_ptr(), st))
    return None, rows, dg


def gemm_nt_bf16(a: torch.Tensor, b: torch.Tensor, err: torch.Tensor) -> torch.Tensor:
    """out[b, m, n] = sum_k a[b, m, k] b[b, n, k] (BF16 operands, FP32 out) on the tensor cores."""
    L = N.lib()
    bt, m, k = a.shape
    n = b.shape[1]
    out = torch.empty(bt, m, n, device=a.device, dtype=torch.float32)
    N.check(L.svbrdf_desc_gemm_nt(a.contiguous().data_ptr(), b.contiguous().data_ptr(), out.data_ptr(), bt, m, n, k,
                                  err.data_ptr(), N.stream_handle(a.device)))
    return out


def he_normal_weights(seed: int, layers=VGG19_TO_CONV4_1):
    """Seeded He-normal (std sqrt(2 / (9 Cin))) weights, zero biases, torch layout [Cout, Cin, 3, 3]."""
    g = torch.Generator().manual_seed(seed)
    out = {}
    for item in layers:
        if item == "pool":
            continue
        name, cin, cout = item
        std = math.sqrt(2.0 / (9 * cin))
        out[name] = (torch.randn(cout, cin, 3, 3, generator=g) * std, torch.zeros(cout))
    return out


class VGGDescriptor:
    """Feature + Gram descriptor loss over renders, BF16 tensor-core convolutions.

    ``load(targets)`` caches the target features (like ``VGGLoss.load``, src/descriptor.py:62-63);
    ``loss(renders)`` returns (feature_loss, gram_loss) as 0-d tensors, differentiable w.r.t.
    ``renders [V, 3, H, W]`` (H, W multiples of 16 after the 2x2 downsample).
    ``fuse_pool`` (default False): True runs each pool's backward pass in the epilogue of the
    data gradient of the convolution above it instead of its own kernel. The fused epilogue
    reads the pool's input and the hook gradient at four window positions per lane (16 bytes
    each, 256 bytes apart) and measured slower than the separate kernels at the descriptor's
    sizes.
    """

    def __init__(self, device="cuda", seed: int = 0, weights: Sequence[float] = (0.25, 0.25, 0.25, 0.25),
                 downsample: Optional[bool] = None, mode: str = "config"):
        if mode not in ("config", "reference"):
            raise ValueError(f"mode must be 'config' or 'reference', not {mode!r}")
        self.device = torch.device(device)
        self.mode = mode
        ref = mode == "reference"
        self.layers = VGG19_TO_CONV4_2 if ref else VGG19_TO_CONV4_1
        self.hooks = REF_HOOKS if ref else HOOKS
        self.avg_pool = ref
        self.gram = not ref
        self.hook_weights = list(weights)
        self.downsample = (not ref) if downsample is None else downsample
        self.fuse_pool = False
        self.err = torch.zeros(1, dtype=torch.int32, device=self.device)
        raw = he_normal_weights(seed, self.layers)
        self.params = {}
        for name, (w, b) in raw.items():
            wb = w.to(torch.bfloat16)  # the weights the tensor cores see
            cout, cin = wb.shape[:2]
            entry = {"w32": wb.float().to(self.device), "b": b.to(self.device)}
            if cin >= 64:
                # forward: [Cout, tap, Cin]; data gradient: [Cin, tap, Cout] with the taps flipped
                entry["w_fwd"] = wb.permute(0, 2, 3, 1).reshape(cout, 9, cin).contiguous().to(self.device)
                entry["w_dg"] = wb.flip(2, 3).permute(1, 2, 3, 0).reshape(cin, 9, cout).contiguous().to(self.device)
            else:
                # conv1_1's data gradient on the tensor cores: [16, tap, 64], rows 3..15 zero
                w16 = torch.zeros(16, 9, cout, dtype=torch.bfloat16)
                w16[:cin] = wb.flip(2, 3).permute(1, 2, 3, 0).reshape(cin, 9, cout)
                entry["w_dg16"] = w16.contiguous().to(self.device)
                sc = torch.tensor([1.0 / s for s in STD], dtype=torch.float32)
                entry["dg_scale"] = (sc * (0.25 if self.downsample else 1.0)).to(self.device)
            self.params[name] = entry
        self.target = None
        self.target16 = None  # BF16 copies of the BF16 hooks' targets (load)

    def bf16_weights(self):
        """{name: (weight [Cout, Cin, 3, 3] as the kernels use it, bias)} in FP32."""
        return {k: (v["w32"].cpu(), v["b"].cpu()) for k, v in self.params.items()}

    # ---- forward -----------------------------------------------------------------------
    def _forward(self, renders: torch.Tensor):
        """Run the stack. Returns (acts, hooks): acts[i] is the output of layer i of
        self.layers (NHWC BF16); hooks maps each hooked layer to its feature (relu1_1 in
        FP32, the others BF16)."""
        L = N.lib()
        st = N.stream_handle(self.device)
        x = renders.detach().float().contiguous()
        v, _, rh, rw = x.shape
        h, w = (rh // 2, rw // 2) if self.downsample else (rh, rw)
        p = self.params["conv1_1"]
        y32 = torch.empty(v, h, w, 64, device=self.device, dtype=torch.float32)
        y16 = torch.empty(v, h, w, 64, device=self.device, dtype=torch.bfloat16)
        N.check(L.svbrdf_desc_conv1_fwd(x.data_ptr(), p["w32"].data_ptr(), p["b"].data_ptr(), y32.data_ptr(),
                                        y16.data_ptr(), v, h, w, int(self.downsample), st))
        acts, hooks = [y16], {"conv1_1": y32}
        pool_fwd = L.svbrdf_desc_avgpool_fwd if self.avg_pool else L.svbrdf_desc_pool_fwd
        for item in self.layers[1:]:
            prev = acts[-1]
            if item == "pool":
                n_, hh, ww, c = prev.shape
                y = torch.empty(n_, hh // 2, ww // 2, c, device=self.device, dtype=torch.bfloat16)
                N.check(pool_fwd(prev.data_ptr(), y.data_ptr(), n_, hh, ww, c, st))
                acts.append(y)
                continue
            name, cin, cout = item
            q = self.params[name]
            y = conv3x3_bf16(prev, q["w_fwd"], q["b"], EPI_BIAS_RELU, self.err)
            acts.append(y)
            if name in self.hooks:
                hooks[name] = y
        return acts, hooks

    # ---- loss terms --------------------------------------------------------------------
    def _terms(self, hooks, cf: Optional[float], cg: Optional[float], hooks16=None):
        """Feature and Gram losses (0-d FP32 tensors). With cf/cg given, also the loss
        gradient at each hooked activation, cf d(feature)/df + cg d(gram)/df, as BF16 NHWC; the
        last layer's gradient is masked by its ReLU (it starts the backward chain). Every term's
        partial sums land in one buffer, and one launch (svbrdf_desc_loss_sums) adds them with
        the hook weights in a fixed order."""
        L = N.lib()
        st = N.stream_handle(self.device)
        tf, tg = self.target
        if hooks16 is None:
            hooks16 = {n: (f if f.dtype == torch.bfloat16 else f.to(torch.bfloat16)) for n, f in hooks.items()}
        nf = sum(f.numel() for f in hooks.values())
        ng = sum(g.numel() for g in tg)
        nparts = L.svbrdf_desc_partials()
        fused = cf is not None and self.gram
        # segments: each hook's feature partials, then each hook's Gram loss rows
        lens, weights, groups = [], [], []
        for name, wt in zip(self.hooks, self.hook_weights):
            v, h, w, c = hooks[name].shape
            lens.append(int(L.svbrdf_desc_gemm_nt_feat_partials(v, h * w, c)) if fused else nparts)
            weights.append(wt * wt / nf)
            groups.append(0)
        if self.gram:
            for name, wt in zip(self.hooks, self.hook_weights):
                v, h, w, c = hooks[name].shape
                lens.append(v * c)
                weights.append(wt * wt / ng)
                groups.append(1)
        offs = [0]
        for n in lens[:-1]:
            offs.append(offs[-1] + n)
        buf = torch.empty(offs[-1] + lens[-1], device=self.device, dtype=torch.float32)
        nh = len(self.hooks)
        grads = {}
        last = [it for it in self.layers if it != "pool"][-1][0]
        for k, (name, wt) in enumerate(zip(self.hooks, self.hook_weights)):
            f = hooks[name]
            v, h, w, c = f.shape
            s = h * w
            part = buf[offs[k]:offs[k] + lens[k]]
            g = None
            if self.gram:
                # the BF16 feature map (relu1_1's hook is FP32; its BF16 copy feeds conv1_2)
                ff = hooks16[name]
                # d/dF of w^2 sum (G - Gt)^2 / ng with G = F^T F / s: F (2 dG) / s, dG = 2 w^2 (G - Gt) / ng
                coef_g = (4.0 * wt * wt * cg / (ng * s)) if cf is not None else 0.0
                rows = buf[offs[nh + k]:offs[nh + k] + lens[nh + k]].view(v, c)
                _, _, dgram = gram_bf16(ff, self.err, tg[k], coef_g, want_dgram=cf is not None, rows_out=rows)
            coef = (2.0 * wt * wt * cf / nf) if cf is not None else 0.0
            if cf is not None:
                g = torch.empty(v, h, w, c, device=self.device, dtype=torch.bfloat16)
                grads[name] = g
            if fused:
                # the Gram gradient F dG with this hook's feature term in its epilogue; a BF16
                # hook's targets are read in BF16 (exact: they are BF16 values)
                t16 = self.target16[k] if getattr(self, "target16", None) else None
                dtypes = int(f.dtype == torch.bfloat16) | (2 if t16 is not None else 0)
                N.check(L.svbrdf_desc_gemm_nt_feat(ff.data_ptr(), dgram.data_ptr(), f.data_ptr(), dtypes,
                                                   (t16 if t16 is not None else tf[k]).data_ptr(), coef,
                                                   int(name == last), g.data_ptr(), part.data_ptr(), v, s, c, c,
                                                   self.err.data_ptr(), st))
            else:
                N.check(L.svbrdf_desc_feat_loss(f.data_ptr(), int(f.dtype == torch.bfloat16), tf[k].data_ptr(),
                                                None, coef, int(name == last), N.ptr(g), part.data_ptr(),
                                                f.numel(), st))
        out = torch.empty(2, device=self.device, dtype=torch.float32)
        ns = len(lens)
        a_off = (ctypes.c_longlong * ns)(*offs)
        a_len = (ctypes.c_longlong * ns)(*lens)
        a_w = (ctypes.c_double * ns)(*weights)
        a_g = (ctypes.c_int * ns)(*groups)
        N.check(L.svbrdf_desc_loss_sums(buf.data_ptr(), ns, ctypes.addressof(a_off), ctypes.addressof(a_len),
                                        ctypes.addressof(a_w), ctypes.addressof(a_g), out.data_ptr(), st))
        fl = out[0]
        gl = out[1] if self.gram else torch.zeros((), device=self.device)
        return fl, gl, grads

    # ---- backward chain ----------------------------------------------------------------
    def _backward(self, acts, grads, render_shape):
        """d(loss)/d renders from the hook gradients, layer by layer in reverse:
        data-gradient convolutions whose epilogue adds the next hook's gradient and applies
        the ReLU mask below; each pool's backward (routing, the hook gradient of the convolution
        under it, that ReLU's mask) as its own kernel, or with ``fuse_pool`` in the epilogue of
        the data gradient of the convolution above it, which then writes the gradient at the
        pool's input; then conv1_1's data gradient (tensor cores) back through the
        normalisation and the downsample."""
        L = N.lib()
        st = N.stream_handle(self.device)
        items = self.layers
        pool_bwd = L.svbrdf_desc_avgpool_bwd if self.avg_pool else L.svbrdf_desc_pool_bwd
        g = grads[items[-1][0]]  # masked gradient at the last ReLU
        i = len(items) - 1
        while i > 0:
            item, below = items[i], items[i - 1]
            x = acts[i - 1]  # the input of layer i: a ReLU output, or a pool output
            n_, h, w, c = x.shape
            if item == "pool":
                # below is a convolution: route, add its hook gradient, mask by its ReLU
                gx = torch.empty_like(x)
                add = grads.get(below[0])
                N.check(pool_bwd(g.data_ptr(), x.data_ptr(), N.ptr(add), gx.data_ptr(), n_, h, w, c, st))
                g = gx
                i -= 1
                continue
            q = self.params[item[0]]
            step = 1
            if below == "pool" and self.fuse_pool:
                xp = acts[i - 2]  # the pool's input, a ReLU output
                gx = torch.empty_like(xp)
                add = grads.get(items[i - 2][0])
                epi, mask = (EPI_UNPOOL_AVG if self.avg_pool else EPI_UNPOOL_MAX), xp
                step = 2
            elif below == "pool":
                gx = torch.empty(n_, h, w, c, device=self.device, dtype=torch.bfloat16)
                epi, mask, add = EPI_NONE, None, None
            else:
                gx = torch.empty(n_, h, w, c, device=self.device, dtype=torch.bfloat16)
                add = grads.get(below[0])
                epi, mask = (EPI_ADD_MASK if add is not None else EPI_MASK), x
            N.check(L.svbrdf_conv3x3_bf16_ex(g.data_ptr(), q["w_dg"].data_ptr(), None, N.ptr(mask), N.ptr(add),
                                             gx.data_ptr(), n_, h, w, item[2], item[1], epi, self.err.data_ptr(), st))
            g = gx
            i -= step
        v, h, w, _ = g.shape
        dr = torch.empty(render_shape, device=self.device, dtype=torch.float32)
        p = self.params["conv1_1"]
        N.check(L.svbrdf_desc_conv1_bwd_tc(g.data_ptr(), p["w_dg16"].data_ptr(), p["dg_scale"].data_ptr(),
                                           dr.data_ptr(), v, h, w, int(self.downsample), self.err.data_ptr(), st))
        return dr

    def features(self, renders: torch.Tensor) -> List[torch.Tensor]:
        """Hooked ReLU outputs, each NHWC [V, H, W, C] (BF16, except relu1_1 in FP32)."""
        _, hooks = self._forward(renders)
        return [hooks[n] for n in self.hooks]

    def load(self, targets: torch.Tensor):
        self._graph = None  # a captured graph holds the previous targets' features
        with torch.no_grad():
            acts, hooks = self._forward(targets)
            feats = [hooks[n] for n in self.hooks]
            grams = ([gram_bf16(self._bf16_hooks(acts, hooks)[n], self.err)[0] for n in self.hooks]
                     if self.gram else [])
            self.target = ([f.float().contiguous() for f in feats], grams)
            self.target16 = [f.contiguous() if f.dtype == torch.bfloat16 else None for f in feats]

    @staticmethod
    def _bf16_hooks(acts, hooks):
        """The hooked features as BF16 NHWC maps: relu1_1's BF16 copy is the first activation."""
        return {n: (acts[0] if n == "conv1_1" else f) for n, f in hooks.items()}

    def loss(self, renders: torch.Tensor):
        """(feature_loss, gram_loss) as 0-d tensors, differentiable w.r.t. ``renders``."""
        if self.target is None:
            raise RuntimeError("call load(targets) first")
        return _DescriptorLoss.apply(renders, self)

    def device_error(self) -> int:
        return int(self.err.item())

    # ---- CUDA-graph replay of forward + backward -------------------------------------
    # One pass issues a few dozen kernels; replaying them as one graph removes the host
    # dispatch cost, which otherwise exceeds the GPU time of the whole stack.
    def _capture(self, shape):
        static_r = torch.zeros(shape, device=self.device)
        side = torch.cuda.Stream(self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(side):
            for _ in range(2):
                self._loss_and_grad_eager(static_r)
        torch.cuda.current_stream(self.device).wait_stream(side)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            fl, gl, dr = self._loss_and_grad_eager(static_r)
        self._graph = (tuple(shape), graph, static_r, fl, gl, dr)

    def _loss_and_grad_eager(self, renders):
        acts, hooks = self._forward(renders)
        fl, gl, grads = self._terms(hooks, 1.0, 1.0, self._bf16_hooks(acts, hooks))
        return fl, gl, self._backward(acts, grads, renders.shape)

    def loss_and_grad(self, renders: torch.Tensor):
        """(feature_loss, gram_loss, d(feature + gram)/d renders) by one graph replay. The
        returned tensors are reused by the next call."""
        if self.target is None:
            raise RuntimeError("call load(targets) first")
        if getattr(self, "_graph", None) is None or self._graph[0] != tuple(renders.shape):
            self._capture(renders.shape)
        _, graph, static_r, fl, gl, dr = self._graph
        with torch.no_grad():
            static_r.copy_(renders)
        graph.replay()
        return fl, gl, dr


def reference_descriptors(device="cuda", seed: int = 0):
    """The reference latent loop's two feature losses (src/materialgan.py:28-34): the VGG in
    the reference's own semantics, hook weights [1, 1, 4, 8] / 14 for latent epochs and
    [8, 8, 2, 1] / 19 for noise epochs, the same network weights. The pair is
    MaterialGANOptim's ``descriptor``."""
    large = VGGDescriptor(device, seed=seed, weights=[w / 14 for w in (1, 1, 4, 8)], mode="reference")
    small = VGGDescriptor(device, seed=seed, weights=[w / 19 for w in (8, 8, 2, 1)], mode="reference")
    return large, small


class _DescriptorLoss(torch.autograd.Function):
    """(feature, Gram) losses with the hand-written backward chain of VGGDescriptor."""

    @staticmethod
    def forward(ctx, renders, desc):
        acts, hooks = desc._forward(renders)
        fl, gl, _ = desc._terms(hooks, None, None, desc._bf16_hooks(acts, hooks))
        ctx.desc = desc
        ctx.shape = renders.shape
        ctx.acts, ctx.hooks = acts, hooks
        return fl, gl

    @staticmethod
    def backward(ctx, gfl, ggl):
        desc = ctx.desc
        _, _, grads = desc._terms(ctx.hooks, float(gfl), float(ggl), desc._bf16_hooks(ctx.acts, ctx.hooks))
        dr = desc._backward(ctx.acts, grads, ctx.shape)
        ctx.acts = ctx.hooks = None
        return dr, None


class _DescriptorTerm(torch.autograd.Function):
    """feature + Gram loss of ``renders`` with its gradient from one graph replay."""

    @staticmethod
    def forward(ctx, renders, desc):
        fl, gl, g = desc.loss_and_grad(renders.detach())
        ctx.save_for_backward(g.clone())
        return (fl + gl).detach().clone()

    @staticmethod
    def backward(ctx, gout):
        (g,) = ctx.saved_tensors
        return gout * g, None


def descriptor_term(renders: torch.Tensor, desc: VGGDescriptor) -> torch.Tensor:
    """Differentiable feature + Gram descriptor loss of ``renders`` (graph-replayed)."""
    return _DescriptorTerm.apply(renders, desc)
