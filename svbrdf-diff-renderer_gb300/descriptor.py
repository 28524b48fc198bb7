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

Every 3x3 convolution with 64 or more input channels runs as a tcgen05 implicit GEMM
(``svbrdf_conv3x3_bf16``: BF16 operands, FP32 accumulation in TMEM, bias + ReLU fused).
Its data gradient is the same kernel on the transposed, flipped weights. conv1_1 (3 input
channels, under 1% of the FLOPs), the pools and the normalisation use torch; the Gram
products are plain batched BF16 GEMMs (cuBLAS tensor cores, FP32 accumulation).
"""
from __future__ import annotations

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

EPI_NONE, EPI_BIAS_RELU, EPI_MASK = 0, 1, 2


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


class _ConvReLU(torch.autograd.Function):
    """relu(conv3x3(x) + b) with frozen weights; backward gives dL/dx only."""

    @staticmethod
    def forward(ctx, x, w_fwd, w_dgrad, bias, err):
        x = x.to(torch.bfloat16).contiguous()
        y = conv3x3_bf16(x, w_fwd, bias, EPI_BIAS_RELU, err)
        ctx.save_for_backward(y, w_dgrad, err)
        return y

    @staticmethod
    def backward(ctx, gy):
        y, w_dgrad, err = ctx.saved_tensors
        gz = (gy.to(torch.bfloat16) * (y > 0)).contiguous()
        gx = conv3x3_bf16(gz, w_dgrad, None, EPI_NONE, err)
        return gx, None, None, None, None


_BMM_F32_OUT = {}


def _bmm_f32out(a: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    """Batched BF16 x BF16 product on the tensor cores, FP32 accumulation, FP32 result when
    torch exposes bmm's out_dtype (checked once per device), else a BF16 result widened."""
    key = a.device
    if key not in _BMM_F32_OUT:
        try:
            z = torch.zeros(1, 2, 2, device=a.device, dtype=torch.bfloat16)
            _BMM_F32_OUT[key] = torch.bmm(z, z, out_dtype=torch.float32).dtype == torch.float32
        except (TypeError, RuntimeError):
            _BMM_F32_OUT[key] = False
    if _BMM_F32_OUT[key]:
        return torch.bmm(a, b, out_dtype=torch.float32)
    return torch.bmm(a, b).float()


class _Gram(torch.autograd.Function):
    """G = F^T F / S for NHWC features F [V, H, W, C] (BF16); gradient F (dG + dG^T) / S."""

    @staticmethod
    def forward(ctx, f):
        v, h, w, c = f.shape
        ff = f.reshape(v, h * w, c).to(torch.bfloat16)
        ctx.save_for_backward(ff)
        ctx.shape = f.shape
        return _bmm_f32out(ff.transpose(1, 2), ff) / (h * w)

    @staticmethod
    def backward(ctx, g):
        (ff,) = ctx.saved_tensors
        v, h, w, c = ctx.shape
        gs = ((g + g.transpose(1, 2)) / (h * w)).to(torch.bfloat16)
        return torch.bmm(ff, gs).reshape(v, h, w, c)


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
    """

    def __init__(self, device="cuda", seed: int = 0, weights: Sequence[float] = (0.25, 0.25, 0.25, 0.25),
                 downsample: bool = True):
        self.device = torch.device(device)
        self.hook_weights = list(weights)
        self.downsample = downsample
        self.err = torch.zeros(1, dtype=torch.int32, device=self.device)
        raw = he_normal_weights(seed)
        self.params = {}
        for name, (w, b) in raw.items():
            wb = w.to(torch.bfloat16)  # the weights the tensor cores see
            cout, cin = wb.shape[:2]
            entry = {"w32": wb.float().to(self.device), "b": b.to(self.device)}
            if cin >= 64:
                # forward: [Cout, tap, Cin]; data gradient: [Cin, tap, Cout] with the taps flipped
                entry["w_fwd"] = wb.permute(0, 2, 3, 1).reshape(cout, 9, cin).contiguous().to(self.device)
                entry["w_dg"] = wb.flip(2, 3).permute(1, 2, 3, 0).reshape(cin, 9, cout).contiguous().to(self.device)
            self.params[name] = entry
        self.mean = torch.tensor(MEAN, device=self.device).view(1, 3, 1, 1)
        self.std = torch.tensor(STD, device=self.device).view(1, 3, 1, 1)
        self.target = None

    def bf16_weights(self):
        """{name: (weight [Cout, Cin, 3, 3] as the kernels use it, bias)} in FP32."""
        return {k: (v["w32"].cpu(), v["b"].cpu()) for k, v in self.params.items()}

    def prepare(self, renders: torch.Tensor) -> torch.Tensor:
        x = renders
        if self.downsample:
            x = torch.nn.functional.avg_pool2d(x, 2)
        return (x - self.mean) / self.std

    def features(self, renders: torch.Tensor) -> List[torch.Tensor]:
        """Hooked ReLU outputs, each NHWC [V, H, W, C] (BF16, except relu1_1 in FP32)."""
        x = self.prepare(renders)
        feats = []
        act = None
        for item in VGG19_TO_CONV4_1:
            if item == "pool":
                act = torch.nn.functional.max_pool2d(act.permute(0, 3, 1, 2), 2).permute(0, 2, 3, 1).contiguous()
                continue
            name, cin, cout = item
            p = self.params[name]
            if cin < 64:
                y = torch.relu(torch.nn.functional.conv2d(x, p["w32"], p["b"], padding=1))
                act = y.permute(0, 2, 3, 1).contiguous()
            else:
                act = _ConvReLU.apply(act, p["w_fwd"], p["w_dg"], p["b"], self.err)
            if name in HOOKS:
                feats.append(act)
        return feats

    @staticmethod
    def _gram(f: torch.Tensor) -> torch.Tensor:
        return _Gram.apply(f)

    def load(self, targets: torch.Tensor):
        self._graph = None  # a captured graph holds the previous targets' features
        with torch.no_grad():
            feats = self.features(targets)
            self.target = ([f.float() for f in feats], [self._gram(f) for f in feats])

    def loss(self, renders: torch.Tensor):
        if self.target is None:
            raise RuntimeError("call load(targets) first")
        feats = self.features(renders)
        tf, tg = self.target
        fl, gl, nf, ng = 0.0, 0.0, 0, 0
        for w, f, t, gt in zip(self.hook_weights, feats, tf, tg):
            fl = fl + (w * w) * torch.nn.functional.mse_loss(f.float(), t, reduction="sum")
            nf += f.numel()
            g = self._gram(f)
            gl = gl + (w * w) * torch.nn.functional.mse_loss(g, gt, reduction="sum")
            ng += g.numel()
        return fl / nf, gl / ng

    def device_error(self) -> int:
        return int(self.err.item())

    # ---- CUDA-graph replay of forward + backward -------------------------------------
    # One eager pass issues a few hundred small kernels; replaying them as one graph removes
    # the host dispatch cost, which otherwise exceeds the GPU time of the whole stack.
    @torch.enable_grad()
    def _capture(self, shape):
        static_r = torch.zeros(shape, device=self.device, requires_grad=True)
        side = torch.cuda.Stream(self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(side):
            for _ in range(2):
                static_r.grad = None
                fl, gl = self.loss(static_r)
                (fl + gl).backward()
        torch.cuda.current_stream(self.device).wait_stream(side)
        static_r.grad = None
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            fl, gl = self.loss(static_r)
            (fl + gl).backward()
        self._graph = (tuple(shape), graph, static_r, fl, gl)

    def loss_and_grad(self, renders: torch.Tensor):
        """(feature_loss, gram_loss, d(feature + gram)/d renders) by one graph replay. The
        returned tensors are reused by the next call."""
        if getattr(self, "_graph", None) is None or self._graph[0] != tuple(renders.shape):
            self._capture(renders.shape)
        _, graph, static_r, fl, gl = self._graph
        with torch.no_grad():
            static_r.copy_(renders)
        graph.replay()
        return fl, gl, static_r.grad


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
