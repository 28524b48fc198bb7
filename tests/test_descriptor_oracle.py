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


def _golden_nets():
    import importlib
    import sys

    from conftest import GOLDEN
    if str(GOLDEN) not in sys.path:
        sys.path.insert(0, str(GOLDEN))
    return importlib.import_module("make_golden_nets")


def fixture_descriptor_weights(d):
    """The fixture's VGG19 weights (numpy-seeded, so the same on every platform), conv1_1 ..
    conv4_2 by name."""
    MG = _golden_nets()
    ws = MG.descriptor_weights(int(d["seed_weights"]))
    names = [item[0] for item in DR.REF_LAYERS if item != "pool"]
    return {n: (torch.from_numpy(w), torch.from_numpy(b)) for n, (w, b) in zip(names, ws)}


def test_reference_mode_matches_reference_vggloss(golden):
    """Pinned to the reference's own VGGLoss (src/descriptor.py:7-79) run in FP64 on the same
    weights and inputs (tests/golden/descriptor_ref_128.npz): the weighted feature vector
    (hooks relu1_1, relu1_2, relu3_2, relu4_2 after average pools), the Gram branch, the loss
    and its gradient with respect to the renders, all within 1e-10."""
    d = golden("descriptor_ref_128.npz")
    MG = _golden_nets()
    w = fixture_descriptor_weights(d)
    x_np, y_np = MG.descriptor_inputs(int(d["seed_inputs"]))
    x, y = torch.from_numpy(x_np), torch.from_numpy(y_np)
    assert abs(float(x.sum()) - float(d["x_sum"])) <= 1e-9 and abs(float(y.sum()) - float(d["y_sum"])) <= 1e-9
    hw = tuple(float(v) for v in d["weights_hook"])
    fv = DR.feature_vector(x, w, hw, downsample=False, mode="reference")
    assert fv.numel() == int(d["feat_len"])
    assert torch.allclose(fv[d["feat_idx"].long()], d["feat_val"], rtol=1e-10, atol=1e-12)
    segs = torch.cumsum(torch.cat((torch.zeros(1, dtype=torch.long), d["feat_segments"].long())), 0)
    for i in range(4):
        assert abs(float(fv[segs[i]:segs[i + 1]].norm()) - float(d["feat_norm"][i])) <= 1e-10 * float(d["feat_norm"][i])
    gv = DR.gram_vector(x[0], w, hw, downsample=False, mode="reference")
    assert gv.numel() == int(d["gram_len"])
    assert torch.allclose(gv[d["gram_idx"].long()], d["gram_val"], rtol=1e-10, atol=1e-12)
    fl, gl, grad = DR.loss_terms(x, y, w, hw, downsample=False, mode="reference")
    assert gl == 0.0
    assert abs(fl - float(d["loss"])) <= 1e-10 * float(d["loss"])
    g = grad.reshape(-1)
    assert torch.allclose(g[d["grad_idx"].long()], d["grad_val"], rtol=1e-9, atol=1e-15)
    assert abs(float(grad.norm()) - float(d["grad_norm"])) <= 1e-10 * float(d["grad_norm"])
