"""Golden fixtures for the descriptor loss and the generator, made by running the reference.

Run from the repository root in a container that holds the reference checkout:

    python tests/golden/make_golden_nets.py --ref /path/to/svbrdf-diff-renderer

* ``descriptor_ref_128.npz``: the reference's ``VGGLoss`` (src/descriptor.py:7-79) in FP64
  on two 128^2 renders against two targets: the loss, its gradient with respect to the
  renders, samples of the weighted feature vector and its per-hook norms, and the Gram
  branch (``compute_feature_vector(..., is_gram=True)``, :50-56) of the first render.
  ``torchvision`` is not installed and its pretrained VGG19 cannot be downloaded, so
  ``torchvision.models.vgg19`` is replaced by a module that returns VGG19's ``features``
  layer list (conv/ReLU/max-pool, 37 layers; the reference swaps the max-pools for average
  pools itself) with weights drawn from numpy, and ``torchvision.transforms.Normalize`` by
  the per-channel (x - mean) / std it computes.
* ``generator_ref_256.npz``: the reference's ``StyleGAN2GeneratorNet`` (src/higan_models/
  stylegan2_generator_network.py:36) as MaterialGAN builds it (256^2, 9 channels, fused
  modulation, truncation psi 1; src/higan_models/stylegan2_generator.py:31-44,
  base_generator.py:89-92) in FP64 with every parameter drawn from numpy: ``synthesis(wp)``
  output samples and per-channel sums and norms, the gradient of sum(out * R) (R drawn from
  numpy) with respect to W+ and to the 13 global noise maps (src/globalvar.py:50-86), and the
  mapping network's w for one z.

Weights and inputs come from ``numpy.random.default_rng`` seeds stored in the fixtures, so the
tests regenerate them on any platform; ``descriptor_weights`` and ``generator_state`` below are
imported by the tests for that.
"""
from __future__ import annotations

import argparse
import importlib
import pathlib
import sys
import types

import numpy as np
import torch

HERE = pathlib.Path(__file__).resolve().parent

# VGG19 `features` layer list: (kind, cin, cout) for convs, then ReLU; "M" = max-pool.
VGG19_CFG = [64, 64, "M", 128, 128, "M", 256, 256, 256, 256, "M", 512, 512, 512, 512, "M", 512, 512, 512, 512, "M"]
DESC_SEED, DESC_INPUT_SEED = 5, 6
GEN_SEED, GEN_INPUT_SEED = 7, 8


def vgg19_convs():
    """(index in `features`, cin, cout) of VGG19's 16 convolutions."""
    out, idx, cin = [], 0, 3
    for v in VGG19_CFG:
        if v == "M":
            idx += 1
            continue
        out.append((idx, cin, v))
        cin = v
        idx += 2
    return out


def descriptor_weights(seed=DESC_SEED):
    """He-normal weights (std sqrt(2 / (9 cin))) and small biases of VGG19's convolutions,
    float64 numpy, in `features` order."""
    rng = np.random.default_rng(seed)
    ws = []
    for _, cin, cout in vgg19_convs():
        w = rng.standard_normal((cout, cin, 3, 3)) * np.sqrt(2.0 / (9 * cin))
        b = rng.standard_normal(cout) * 0.01
        ws.append((w, b))
    return ws


def descriptor_inputs(seed=DESC_INPUT_SEED, n=2, res=128):
    rng = np.random.default_rng(seed)
    return rng.uniform(0.0, 1.0, (n, 3, res, res)), rng.uniform(0.0, 1.0, (n, 3, res, res))


def generator_state(keys_shapes, seed=GEN_SEED):
    """numpy values for the reference generator's parameters, drawn in the order given:
    standard normal for weights and the constant input, 0.1 x standard normal for biases,
    style biases, noise strengths and w_avg."""
    rng = np.random.default_rng(seed)
    out = {}
    for k, shape in keys_shapes:
        scale = 1.0 if (k.endswith(".weight") or k.endswith(".const")) else 0.1
        out[k] = np.asarray(rng.standard_normal(shape) * scale)
    return out


def fixture_key_shapes(keys, key_shapes):
    """(key, shape) pairs from a fixture's keys and -1-padded shapes."""
    return [(str(k), tuple(int(x) for x in sh if x >= 0)) for k, sh in zip(keys, key_shapes)]


def generator_inputs(num_ws=14, seed=GEN_INPUT_SEED, res=256, channels=9):
    rng = np.random.default_rng(seed)
    wp = rng.standard_normal((1, num_ws, 512))
    noises = [rng.standard_normal((1, 1, r, r)) for r in [4] + [2 ** l for l in range(3, 9) for _ in (0, 1)]]
    R = rng.standard_normal((1, channels, res, res))
    z = rng.standard_normal((1, 512))
    return wp, noises, R, z


def _stub_torchvision(weights):
    tv = types.ModuleType("torchvision")
    models = types.ModuleType("torchvision.models")
    transforms = types.ModuleType("torchvision.transforms")

    class _VGG:
        def __init__(self):
            layers, it = [], iter(weights)
            cin = 3
            for v in VGG19_CFG:
                if v == "M":
                    layers.append(torch.nn.MaxPool2d(kernel_size=2, stride=2))
                    continue
                conv = torch.nn.Conv2d(cin, v, kernel_size=3, padding=1)
                w, b = next(it)
                with torch.no_grad():
                    conv.weight.copy_(torch.from_numpy(w))
                    conv.bias.copy_(torch.from_numpy(b))
                layers += [conv, torch.nn.ReLU(inplace=True)]
                cin = v
            self.features = torch.nn.Sequential(*layers).double()

    def vgg19(weights=None):
        return _VGG()

    class Normalize:
        def __init__(self, mean, std):
            self.mean, self.std = mean, std

        def __call__(self, x):
            m = torch.as_tensor(self.mean, dtype=x.dtype).view(-1, 1, 1)
            s = torch.as_tensor(self.std, dtype=x.dtype).view(-1, 1, 1)
            return (x - m) / s

    models.vgg19 = vgg19
    transforms.Normalize = Normalize
    tv.models, tv.transforms = models, transforms
    sys.modules["torchvision"] = tv
    sys.modules["torchvision.models"] = models
    sys.modules["torchvision.transforms"] = transforms


def _stub_other():
    class _Any(types.ModuleType):
        def __getattr__(self, name):
            if name.startswith("__"):
                raise AttributeError(name)
            return lambda *a, **k: None

    for name in ("cv2", "PIL", "PIL.Image", "matplotlib", "matplotlib.pyplot", "tqdm", "requests"):
        sys.modules.setdefault(name, _Any(name))


def case_descriptor(ref_root):
    ws = descriptor_weights()
    _stub_torchvision(ws)
    sys.path.insert(0, str(ref_root))
    D = importlib.import_module("src.descriptor")
    loss_mod = D.VGGLoss("cpu")
    x_np, y_np = descriptor_inputs()
    x = torch.from_numpy(x_np).requires_grad_(True)
    y = torch.from_numpy(y_np)
    loss_mod.load(y)
    loss = loss_mod(x)
    loss.backward()
    with torch.no_grad():
        fv = loss_mod.compute_feature_vector(loss_mod.normalize(x.detach()))
        seg = [o.numel() for o in _hook_outputs(loss_mod, x.detach())]
        gv = loss_mod.compute_feature_vector(loss_mod.normalize(x.detach()[0:1]), is_gram=True)
    rng = np.random.default_rng(99)
    fidx = np.sort(rng.choice(fv.numel(), 8192, replace=False))
    gidx = np.sort(rng.choice(gv.numel(), 4096, replace=False))
    bounds = np.cumsum([0] + seg)
    fnorm = [float(fv[bounds[i]:bounds[i + 1]].norm()) for i in range(len(seg))]
    gsizes = [c * c for c in (64, 64, 256, 512)]
    gb = np.cumsum([0] + gsizes)
    gnorm = [float(gv[gb[i]:gb[i + 1]].norm()) for i in range(4)]
    grad = x.grad.detach().numpy()
    gsel = np.sort(rng.choice(grad.size, 4096, replace=False))
    return {"seed_weights": DESC_SEED, "seed_inputs": DESC_INPUT_SEED, "loss": float(loss),
            "weights_hook": np.asarray(loss_mod.weights, dtype=np.float64),
            "feat_len": fv.numel(), "feat_segments": np.asarray(seg), "feat_idx": fidx, "feat_val": fv.numpy()[fidx],
            "feat_norm": np.asarray(fnorm), "gram_len": gv.numel(), "gram_idx": gidx, "gram_val": gv.numpy()[gidx],
            "gram_norm": np.asarray(gnorm), "grad_idx": gsel, "grad_val": grad.reshape(-1)[gsel],
            "grad_norm": float(np.linalg.norm(grad)), "x_sum": float(x_np.sum()), "y_sum": float(y_np.sum())}


def _hook_outputs(loss_mod, x):
    loss_mod.outputs = []
    loss_mod.net(loss_mod.normalize(x))
    return list(loss_mod.outputs)


def generator_keys(net):
    """(key, shape) of every parameter of the reference network plus truncation.w_avg."""
    ks = [(k, tuple(p.shape)) for k, p in net.named_parameters()]
    ks.append(("truncation.w_avg", tuple(net.truncation.w_avg.shape)))
    return sorted(ks)


def case_generator(ref_root):
    sys.path.insert(0, str(ref_root))
    G = importlib.import_module("src.higan_models.stylegan2_generator_network")
    gv = importlib.import_module("src.globalvar")
    net = G.StyleGAN2GeneratorNet(resolution=256, image_channels=9, fused_modulate=True, truncation_psi=1.0,
                                  truncation_layers=18, randomize_noise=False).double()
    keys = generator_keys(net)
    vals = generator_state(keys)
    sd = net.state_dict()
    for k, v in vals.items():
        sd[k] = torch.from_numpy(v)
    net.load_state_dict(sd)
    wp_np, noises_np, R_np, z_np = generator_inputs()
    wp = torch.from_numpy(wp_np).requires_grad_(True)
    gv.noises = [torch.from_numpy(n).requires_grad_(True) for n in noises_np]
    gv.noise_idx = 0
    out = net.synthesis(wp)
    loss = (out * torch.from_numpy(R_np)).sum()
    loss.backward()
    with torch.no_grad():
        w = net.truncation(net.mapping(torch.from_numpy(z_np)))
    o = out.detach().numpy()
    rng = np.random.default_rng(98)
    oidx = np.sort(rng.choice(o.size, 8192, replace=False))
    res = {"seed_weights": GEN_SEED, "seed_inputs": GEN_INPUT_SEED, "loss": float(loss),
           "keys": np.asarray([k for k, _ in keys]),
           "key_shapes": np.asarray([list(sh) + [-1] * (4 - len(sh)) for _, sh in keys]),
           "out_idx": oidx, "out_val": o.reshape(-1)[oidx],
           "out_sum": o.sum(axis=(0, 2, 3)), "out_norm": np.sqrt((o ** 2).sum(axis=(0, 2, 3))),
           "grad_wp": wp.grad.detach().numpy(), "w_mapped": w.detach().numpy()[0, 0]}
    for i, n in enumerate(gv.noises):
        g = n.grad.detach().numpy().reshape(-1)
        res[f"noise{i}_norm"] = float(np.linalg.norm(g))
        k = min(g.size, 1024)
        sel = np.sort(rng.choice(g.size, k, replace=False))
        res[f"noise{i}_idx"] = sel
        res[f"noise{i}_val"] = g[sel]
    return res


def save(name, d):
    np.savez_compressed(HERE / name, **{k: np.asarray(v) for k, v in d.items()})
    print("wrote", name)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="root of a checkout of the reference repository")
    a = ap.parse_args()
    torch.set_default_dtype(torch.float64)
    _stub_other()
    save("descriptor_ref_128.npz", case_descriptor(pathlib.Path(a.ref)))
    save("generator_ref_256.npz", case_generator(pathlib.Path(a.ref)))


if __name__ == "__main__":
    main()
