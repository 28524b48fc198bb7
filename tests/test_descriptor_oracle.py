"""The FP64 descriptor oracle on the CPU: its two modes follow the stacks they restate."""
import math

import torch

from oracle import descriptor_ref as DR


def _weights(seed=0, layers=DR.REF_LAYERS):
    g = torch.Generator().manual_seed(seed)
    out = {}
    for item in layers:
        if item == "pool":
            continue
        name, cin, cout = item
        out[name] = (torch.randn(cout, cin, 3, 3, generator=g) * math.sqrt(2.0 / (9 * cin)), torch.zeros(cout))
    return out


def test_reference_mode_hooks_and_shapes():
    """Reference mode: full resolution, average pools, hooks relu1_1, relu1_2, relu3_2 and
    relu4_2 (VGG19 features 1, 3, 13, 22)."""
    w = _weights()
    r = torch.rand(2, 3, 32, 32, generator=torch.Generator().manual_seed(1))
    feats = DR.features(r, w, downsample=False, mode="reference")
    assert [tuple(f.shape) for f in feats] == [(2, 64, 32, 32), (2, 64, 32, 32), (2, 256, 8, 8), (2, 512, 4, 4)]
    cfg = DR.features(r, w, downsample=True, mode="config")
    assert [tuple(f.shape) for f in cfg] == [(2, 64, 16, 16), (2, 64, 16, 16), (2, 256, 4, 4), (2, 512, 2, 2)]
    # the pools differ: the same renders give different relu3_2 features in the two stacks
    mx = DR.features(r, w, downsample=False, mode="config")
    assert not torch.allclose(feats[2], mx[2])


def test_reference_mode_loss_is_feature_mse_only():
    w = _weights(3)
    g = torch.Generator().manual_seed(2)
    tgt = torch.rand(2, 3, 32, 32, generator=g)
    cur = (tgt + 0.05 * torch.randn(2, 3, 32, 32, generator=g)).clamp(0, 1)
    fl, gl, grad = DR.loss_terms(cur, tgt, w, mode="reference")
    assert gl == 0.0 and fl > 0.0
    # the feature MSE of the concatenated weighted hooks (src/descriptor.py:39-60, 77-79)
    f = DR.features(cur, w, downsample=False, mode="reference")
    t = DR.features(tgt, w, downsample=False, mode="reference")
    vec = torch.cat([(0.25 * a).flatten() for a in f])
    tvec = torch.cat([(0.25 * b).flatten() for b in t])
    assert abs(fl - float(((vec - tvec) ** 2).mean())) <= 1e-12 * fl
    assert grad.shape == cur.shape and torch.isfinite(grad).all()
    # identical inputs: zero loss and gradient
    fl0, _, g0 = DR.loss_terms(tgt, tgt, w, mode="reference")
    assert fl0 == 0.0 and float(g0.abs().max()) == 0.0
