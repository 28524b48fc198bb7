"""Generate the golden fixtures by running the reference implementation itself.

Run from the repository root in a container that holds the reference checkout:

    python tests/golden/make_golden.py [--ref /path/to/svbrdf-diff-renderer]

It imports the reference's ``src/microfacet.py`` (numpy + torch only) and
``src/svbrdf.py:SvbrdfOptim`` (with its image/plot modules ``cv2``, ``PIL`` and
``matplotlib`` replaced by no-op stubs, because only the optimiser loop is used) and
records, on small seeded scenes:

* ``render_coloc_20.npz``: ``Microfacet.eval`` renders (FP32, and FP64 with the grid and
  lights cast), MSE loss and its autograd gradient for a co-located 3x3 grid;
* ``render_general_24.npz``: separate light and camera positions, unequal light power,
  edge-case maps (normal xy outside the unit disc, values at exactly -1 and 1, zero
  roughness), gradients of the MSE and log1p losses and of the light power;
* ``optim_traj_16.npz`` / ``optim_traj_light_16.npz``: 20 epochs of the reference's own
  ``SvbrdfOptim.optim`` loop (src/svbrdf.py:44-83) from ``init_from_const``, without and
  with the learnable light power.

The fixtures are small (a few hundred KB) and committed; the reference checkout is not
needed to run the tests.
"""
from __future__ import annotations

import argparse
import importlib
import importlib.util
import pathlib
import sys
import tempfile
import types

import numpy as np
import torch

HERE = pathlib.Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO))


def _stub_modules():
    class _Any(types.ModuleType):
        def __getattr__(self, name):
            if name.startswith("__"):
                raise AttributeError(name)
            return lambda *a, **k: None

    for name in ("cv2", "PIL", "PIL.Image", "matplotlib", "matplotlib.pyplot"):
        sys.modules.setdefault(name, _Any(name))
    sys.modules["PIL"].Image = sys.modules["PIL.Image"]
    sys.modules["matplotlib"].pyplot = sys.modules["matplotlib.pyplot"]


def load_reference(ref_root: pathlib.Path):
    _stub_modules()
    sys.path.insert(0, str(ref_root))
    micro = importlib.import_module("src.microfacet")
    svb = importlib.import_module("src.svbrdf")
    return micro, svb


def ref_render(micro, textures, cam, lit, lpow, size, dtype):
    res = textures.shape[2]
    cl = [cam.to(dtype), lit.to(dtype), lpow.to(dtype)]
    r = micro.Microfacet(res, cam.shape[0], size, cl, "cpu")
    if dtype == torch.float64:
        r.pos = r.pos.double()
    return r, r.eval(textures.to(dtype))


def ref_loss_grad(micro, textures, targets, cam, lit, lpow, size, dtype, kind):
    tex = textures.detach().to(dtype).clone().requires_grad_(True)
    lp = lpow.detach().to(dtype).clone().requires_grad_(True)
    res = textures.shape[2]
    r = micro.Microfacet(res, cam.shape[0], size, [cam.to(dtype), lit.to(dtype), lp], "cpu")
    if dtype == torch.float64:
        r.pos = r.pos.double()
    r.update_light(lp)
    out = r.eval(tex)
    tg = targets.to(dtype)
    if kind == "mse":
        loss = torch.nn.functional.mse_loss(out, tg)
    else:
        loss = torch.nn.functional.mse_loss(torch.log1p(out), torch.log1p(tg))
    loss.backward()
    return out.detach(), float(loss.item()), tex.grad.detach(), lp.grad.detach()


def case_coloc(micro, scenes):
    sc = scenes.single_scene(res=20, seed=1000)
    _, gt32 = ref_render(micro, sc.gt, sc.camera_pos, sc.light_pos, sc.light_pow, sc.size, torch.float32)
    g = torch.Generator().manual_seed(11)
    targets = (gt32 + 0.01 * torch.randn(gt32.shape, generator=g)).clamp(0, 1)
    # a mid-optimisation state: blend of the constant init and the ground truth
    state = (0.5 * sc.gt + 0.5 * scenes.const_init(20)).contiguous()
    out = {"textures_gt": sc.gt, "textures": state, "camera_pos": sc.camera_pos, "light_pos": sc.light_pos,
           "light_pow": sc.light_pow, "size": torch.tensor(sc.size), "targets": targets,
           "render_gt32": gt32}
    _, r64 = ref_render(micro, sc.gt, sc.camera_pos, sc.light_pos, sc.light_pow, sc.size, torch.float64)
    out["render_gt64"] = r64
    for dt, tag in ((torch.float32, "32"), (torch.float64, "64")):
        o, l, gt_, gl = ref_loss_grad(micro, state, targets, sc.camera_pos, sc.light_pos, sc.light_pow,
                                      sc.size, dt, "mse")
        out["render" + tag] = o
        out["loss_mse" + tag] = torch.tensor(l, dtype=torch.float64)
        out["grad_mse" + tag] = gt_
        out["gradpow_mse" + tag] = gl
    return out


def case_general(micro, scenes):
    res, n = 24, 5
    g = torch.Generator().manual_seed(21)
    cam = torch.cat(((torch.rand(n, 2, generator=g) * 2 - 1) * 8, 25 + 10 * torch.rand(n, 1, generator=g)), 1)
    lit = torch.cat(((torch.rand(n, 2, generator=g) * 2 - 1) * 8, 25 + 10 * torch.rand(n, 1, generator=g)), 1)
    lpow = torch.tensor([1200.0, 1500.0, 1800.0])
    tex = scenes.make_material(res, 1001)
    # normal xy beyond the unit disc (and beyond [-1, 1]) on some texels
    tex[0, 3, 0:4, :] = torch.linspace(-1.3, 1.3, res)
    tex[0, 4, 0:4, :] = 0.9
    # exact bounds
    tex[0, 0:3, 5, :] = -1.0
    tex[0, 6:9, 6, :] = 1.0
    tex[0, 5, 7, :] = -1.0   # zero roughness
    tex[0, 5, 8, :] = 1.0
    tex[0, 3:5, 9, :] = 0.0
    _, ref32 = ref_render(micro, scenes.make_material(res, 1002), cam, lit, lpow, 17.0, torch.float32)
    gg = torch.Generator().manual_seed(22)
    targets = (ref32 + 0.01 * torch.randn(ref32.shape, generator=gg)).clamp(0, 1)
    out = {"textures": tex, "camera_pos": cam, "light_pos": lit, "light_pow": lpow,
           "size": torch.tensor(17.0), "targets": targets}
    for kind in ("mse", "log1p"):
        for dt, tag in ((torch.float32, "32"), (torch.float64, "64")):
            o, l, gt_, gl = ref_loss_grad(micro, tex, targets, cam, lit, lpow, 17.0, dt, kind)
            out["render" + tag] = o
            out[f"loss_{kind}{tag}"] = torch.tensor(l, dtype=torch.float64)
            out[f"grad_{kind}{tag}"] = gt_
            out[f"gradpow_{kind}{tag}"] = gl
    return out


class _SvbrdfObjStub:
    """The slice of ``SvbrdfIO`` that ``SvbrdfOptim.optim`` touches (src/svbrdf.py:44-83)."""

    def __init__(self, cl, tmp):
        self.cl = cl
        self.optimize_dir = pathlib.Path(tmp)

    def save_textures_th(self, *a, **k):
        pass

    def save_images_th(self, *a, **k):
        pass


def case_traj(micro, svb, scenes, optim_light):
    res, epochs, lr = 16, 20, 0.01
    sc = scenes.single_scene(res=res, seed=1003)
    _, gt32 = ref_render(micro, sc.gt, sc.camera_pos, sc.light_pos, sc.light_pow, sc.size, torch.float32)
    g = torch.Generator().manual_seed(31)
    targets = (gt32 + 0.01 * torch.randn(gt32.shape, generator=g)).clamp(0, 1)
    lpow0 = torch.tensor([1300.0, 1400.0, 1500.0]) if optim_light else sc.light_pow.clone()
    cl = [sc.camera_pos.clone(), sc.light_pos.clone(), lpow0.clone()]
    renderer = micro.Microfacet(res, sc.n_views, sc.size, cl, "cpu")
    opt = svb.SvbrdfOptim("cpu", renderer)
    opt.load_targets(targets)
    opt.init_from_const()
    init = opt.textures.detach().clone()
    with tempfile.TemporaryDirectory() as tmp:
        obj = _SvbrdfObjStub(cl, tmp)
        losses = []
        orig = opt.compute_image_loss

        def rec(pred):
            loss = orig(pred)
            losses.append(float(loss.item()))
            return loss

        opt.compute_image_loss = rec
        opt.optim(epochs, lr, obj, optim_light)
    st = opt.optimizer.state[opt.textures]
    out = {"init": init, "camera_pos": sc.camera_pos, "light_pos": sc.light_pos, "light_pow0": lpow0,
           "size": torch.tensor(sc.size), "targets": targets, "epochs": torch.tensor(epochs),
           "lr": torch.tensor(lr), "textures": opt.textures.detach(), "exp_avg": st["exp_avg"],
           "exp_avg_sq": st["exp_avg_sq"], "loss": torch.tensor(losses[:epochs], dtype=torch.float64)}
    if optim_light:
        out["light_pow"] = obj.cl[2].detach()
    return out


def save(name, d):
    arrs = {k: (v.detach().cpu().numpy() if torch.is_tensor(v) else np.asarray(v)) for k, v in d.items()}
    np.savez_compressed(HERE / name, **arrs)
    print("wrote", name, sum(a.nbytes for a in arrs.values()), "bytes raw")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="root of a checkout of the reference repository")
    a = ap.parse_args()
    torch.manual_seed(0)
    micro, svb = load_reference(pathlib.Path(a.ref))
    scenes = importlib.import_module("svbrdf-diff-renderer_gb300.scenes")
    save("render_coloc_20.npz", case_coloc(micro, scenes))
    save("render_general_24.npz", case_general(micro, scenes))
    save("optim_traj_16.npz", case_traj(micro, svb, scenes, False))
    save("optim_traj_light_16.npz", case_traj(micro, svb, scenes, True))


if __name__ == "__main__":
    main()
