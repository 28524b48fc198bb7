"""FP64 CPU oracle of the descriptor loss.

Parity is pinned for mode="reference": tests/golden/make_golden_nets.py runs the reference's
own VGGLoss (src/descriptor.py:7-79) in FP64 with torchvision's vgg19 replaced by VGG19's
layer list carrying seeded weights (the pretrained ImageNet weights cannot be downloaded),
and tests/test_descriptor_oracle.py checks this module's features, Gram branch, loss and
gradient against that fixture. The configs mode (max-pool, downsample, Gram term, hooks to
relu4_1) shares every building block with the pinned mode.

TEST INFRASTRUCTURE ONLY (tests and bench's CPU legs). Restates the VGG-feature loss of
src/descriptor.py:7-79 with the stack the GPU module uses: 2x2 box downsample, ImageNet
normalisation with the reference's std (0.229, 0.224, 0.255; src/descriptor.py:65-75),
conv1_1..conv4_1 (3x3, padding 1, ReLU, 2x2 max-pool), hooks at relu1_1, relu1_2, relu3_2,
relu4_1, and the weighted feature-L2 (src/descriptor.py:39-60, 77-79) and Gram (:50-56)
terms. Runs in FP64 on the exact weights the BF16 kernels use, so the difference to the GPU
measures the BF16 activations and FP32 tensor-core accumulation alone.

mode="reference" restates the reference's own VGGLoss instead: full-resolution renders,
VGG19 to relu4_2 with its max-pools replaced by 2x2 average pools (src/descriptor.py:16-19),
hooks at features 1, 3, 13, 22 = relu1_1, relu1_2, relu3_2, relu4_2 (:26-27), and the
feature MSE alone (:77-79).
"""
from __future__ import annotations

import torch

MEAN = (0.485, 0.456, 0.406)
STD = (0.229, 0.224, 0.255)
LAYERS = [("conv1_1", 3, 64), ("conv1_2", 64, 64), "pool", ("conv2_1", 64, 128), ("conv2_2", 128, 128), "pool",
          ("conv3_1", 128, 256), ("conv3_2", 256, 256), ("conv3_3", 256, 256), ("conv3_4", 256, 256), "pool",
          ("conv4_1", 256, 512)]
HOOKS = ("conv1_1", "conv1_2", "conv3_2", "conv4_1")
REF_LAYERS = LAYERS + [("conv4_2", 512, 512)]
REF_HOOKS = ("conv1_1", "conv1_2", "conv3_2", "conv4_2")


def _bf16(x):
    """x rounded to BF16 (nearest even) in the forward pass, the identity in the backward."""
    return x + (x.to(torch.bfloat16).to(x.dtype) - x).detach()


def features(renders, weights, downsample=True, mode="config", bf16=False, gram_inputs=None):
    """Hooked ReLU outputs. With ``bf16`` every convolution's output is rounded to BF16 after
    its ReLU (straight through in the backward pass), as the tensor-core stack stores its
    activations, except the relu1_1 hook itself, which that stack keeps in FP32 for the feature
    term while feeding the rounded copy on; ``gram_inputs`` (a list) then receives the features
    the Gram term reads (the rounded copies)."""
    ref = mode == "reference"
    layers, hooks = (REF_LAYERS, REF_HOOKS) if ref else (LAYERS, HOOKS)
    x = renders.double()
    if downsample:
        x = torch.nn.functional.avg_pool2d(x, 2)
    mean = torch.tensor(MEAN, dtype=torch.float64).view(1, 3, 1, 1)
    std = torch.tensor(STD, dtype=torch.float64).view(1, 3, 1, 1)
    x = (x - mean) / std
    out = []
    for item in layers:
        if item == "pool":
            x = torch.nn.functional.avg_pool2d(x, 2) if ref else torch.nn.functional.max_pool2d(x, 2)
            continue
        name = item[0]
        w, b = weights[name]
        y = torch.relu(torch.nn.functional.conv2d(x, w.double(), b.double(), padding=1))
        x = _bf16(y) if bf16 else y
        if name in hooks:
            out.append(y if (bf16 and name == "conv1_1") else x)
            if gram_inputs is not None:
                gram_inputs.append(x)
    return out


def feature_vector(renders, weights, hook_weights=(0.25, 0.25, 0.25, 0.25), downsample=False, mode="reference"):
    """The concatenated weighted feature vector of ``VGGLoss.compute_feature_vector``
    (src/descriptor.py:39-60): per hook, the whole batch's features flattened (N, C, H, W
    order) times the hook's weight, hooks in order."""
    feats = features(renders, weights, downsample, mode)
    return torch.cat([f.flatten() * w for f, w in zip(feats, hook_weights)])


def gram_vector(render, weights, hook_weights=(0.25, 0.25, 0.25, 0.25), downsample=False, mode="reference"):
    """``compute_feature_vector(x, is_gram=True)`` of one render (src/descriptor.py:50-56):
    per hook G = F F^T / S of the [C, S] feature matrix, flattened, times the hook's weight."""
    feats = features(render.unsqueeze(0) if render.dim() == 3 else render, weights, downsample, mode)
    return torch.cat([gram(f).flatten() * w for f, w in zip(feats, hook_weights)])


def gram(f):
    v, c, h, w = f.shape
    ff = f.reshape(v, c, h * w)
    return torch.bmm(ff, ff.transpose(1, 2)) / (h * w)


def loss_terms(renders, targets, weights, hook_weights=(0.25, 0.25, 0.25, 0.25), downsample=None, mode="config",
               bf16=False, views_total=None):
    """(feature_loss, gram_loss, d(feature+gram)/d renders) in FP64. In reference mode the
    Gram loss is 0 and the renders are not downsampled. ``bf16`` rounds the activations as the
    tensor-core stack does (see ``features``). Both terms are sums over the views, so a subset
    of the views of a larger batch gives that batch's per-view terms: ``views_total`` is the
    batch's view count, whose element counts normalise the means."""
    ref = mode == "reference"
    downsample = (not ref) if downsample is None else downsample
    r = renders.detach().double().clone().requires_grad_(True)
    with torch.no_grad():
        tgi = []
        tf = features(targets, weights, downsample, mode, bf16, tgi)
        tg = [gram(f) for f in (tgi if bf16 else tf)]
    gi = []
    feats = features(r, weights, downsample, mode, bf16, gi)
    scale = (views_total / renders.shape[0]) if views_total else 1.0
    fl, gl, nf, ng = 0.0, 0.0, 0, 0
    for k, (w, f, t, g_t) in enumerate(zip(hook_weights, feats, tf, tg)):
        # the reference's MSE of the concatenated weighted features (src/descriptor.py:39-60)
        fl = fl + (w * w) * ((f - t) ** 2).sum()
        nf += f.numel()
        if not ref:
            g = gram(gi[k] if bf16 else f)
            gl = gl + (w * w) * ((g - g_t) ** 2).sum()
            ng += g.numel()
    fl = fl / (nf * scale)
    gl = gl / (ng * scale) if not ref else torch.zeros((), dtype=torch.float64)
    (fl + gl).backward()
    return float(fl.detach()), float(gl.detach()), r.grad.detach()
