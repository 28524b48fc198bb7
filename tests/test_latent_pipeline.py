"""The latent-loop script and light optimisation on the CPU: the renderer is the oracle's
differentiable torch render behind Microfacet's interface, the generator a small seeded one,
so the host logic (initialisation modes, light handling, files) runs without a GPU. The CUDA
paths of the same loop are tested in test_materialgan.py."""
import json
import types

import pytest
import torch

from oracle import microfacet_ref as R


class TorchRenderer:
    """Microfacet's interface (.res, .n_of_imgs, .update_light, .eval) on the oracle."""

    def __init__(self, res, n, size, cl, device="cpu"):
        self.res, self.n_of_imgs, self.size = res, n, float(size)
        self.cam, self.lit = torch.as_tensor(cl[0]).float(), torch.as_tensor(cl[1]).float()
        self.light_pow = torch.as_tensor(cl[2]).float()

    def update_light(self, light_pow):
        self.light_pow = light_pow

    def eval(self, textures):
        return R.render(textures, self.cam, self.lit, self.light_pow, self.size, torch.float32)


def _setup(svb, res=16):
    sc = svb.scenes.single_scene(res=res, seed=1016)
    tg = R.render(sc.gt, sc.camera_pos, sc.light_pos, sc.light_pow * 1.3, sc.size, torch.float32)
    gen = svb.materialgan.StyleGAN2Generator(resolution=res, fmap_max=16, w_dim=32, seed=1, channels_last=False)
    return sc, tg, gen


def test_latent_loop_optimises_the_light(svb):
    sc, tg, gen = _setup(svb)
    r = TorchRenderer(16, 9, sc.size, sc.cl)
    o = svb.materialgan.MaterialGANOptim("cpu", r, gen)
    o.load_targets(tg)
    o.init_from(batch=1, seed=2)
    scene = types.SimpleNamespace(cl=[sc.camera_pos, sc.light_pos, sc.light_pow.clone()])
    o.optim([8, 2, 2], 0.05, scene, optim_light=True)
    light = scene.cl[2]
    assert light.requires_grad and light.is_leaf and r.light_pow is light
    assert not torch.allclose(light.detach(), sc.light_pow)  # the light moved
    assert len(o.loss_image_list) == 8 and all(x == x for x in o.loss_image_list)
    with pytest.raises(ValueError):
        o.optim([1, 1, 1], 0.05, None, optim_light=True)


def _scene_dir(svb, tmp_path, sc):
    cams = sc.camera_pos.tolist()
    cfg = {"reference_dir": "ref", "target_dir": "target", "optimize_dir": "optim", "rerender_dir": "rerender",
           "im_size": sc.size, "idx": list(range(9)), "camera_pos": cams, "light_pos": cams,
           "light_pow": sc.light_pow.tolist()}
    j = tmp_path / "scene.json"
    j.write_text(json.dumps(cfg))
    io = svb.SvbrdfIO(j, "cpu")
    io.save_images_th(R.render(sc.gt, sc.camera_pos, sc.light_pos, sc.light_pow, sc.size, torch.float32),
                      io.target_dir)
    return j


@pytest.mark.parametrize("init", ["none", "latent", "latent+noise"])
def test_optim_ganlatent_script(svb, tmp_path, monkeypatch, init):
    """optim_ganlatent (src/scripts.py:100-143): the three tex_init forms, the output files."""
    sc, _, gen = _setup(svb)
    j = _scene_dir(svb, tmp_path, sc)
    monkeypatch.setattr(svb.scripts, "Microfacet", TorchRenderer)
    tex_init = []
    if init != "none":
        seed_opt = svb.materialgan.MaterialGANOptim("cpu", TorchRenderer(16, 9, sc.size, sc.cl), gen)
        seed_opt.init_from(batch=1, seed=7, noise="random")
        seed_opt.save_latent(tmp_path / "optim_latent.pt", tmp_path / "optim_noise.pt")
        tex_init = [tmp_path / "optim_latent.pt"] + ([tmp_path / "optim_noise.pt"] if init == "latent+noise" else [])
    start = {}
    real_optim = svb.materialgan.MaterialGANOptim.optim

    def spy(self, *a, **k):  # the state the optimisation starts from
        start["latent"] = self.latent.detach().clone()
        start["noises"] = [n.detach().clone() for n in self.noises]
        return real_optim(self, *a, **k)

    monkeypatch.setattr(svb.materialgan.MaterialGANOptim, "optim", spy)
    opt = svb.optim_ganlatent(j, 16, 0.02, [4, 2, 1], tex_init, device="cpu", generator=gen)
    assert len(opt.loss_image_list) == 4
    for name in ("nom.png", "dif.png", "spe.png", "rgh.png"):
        assert (tmp_path / "optim" / name).exists()
    assert (tmp_path / "rerender" / "08.png").exists()
    if init != "none":
        assert torch.equal(start["latent"], torch.load(tmp_path / "optim_latent.pt"))
    if init == "latent":  # a latent alone starts from the reference's average (zero) noise
        assert all(float(n.abs().max()) == 0.0 for n in start["noises"])
    if init == "latent+noise":
        saved = torch.load(tmp_path / "optim_noise.pt")
        assert all(torch.equal(a, b) for a, b in zip(start["noises"], saved))
    if init == "none":  # random noise, as init_from([]) draws
        assert any(float(n.abs().max()) > 0.0 for n in start["noises"])
    with pytest.raises(ValueError):
        svb.optim_ganlatent(j, 16, 0.02, [1, 1, 1], "auto", device="cpu", generator=gen)


def test_gen_textures_from_materialgan(svb, tmp_path):
    """src/scripts.py:18-28: a random material's maps written to reference_dir."""
    sc, _, gen = _setup(svb)
    j = _scene_dir(svb, tmp_path, sc)
    t = svb.gen_textures_from_materialgan(j, device="cpu", generator=gen, seed=4)
    assert t.shape == (1, 9, 16, 16) and float(t.abs().max()) <= 1.0
    for name in ("nom.png", "dif.png", "spe.png", "rgh.png"):
        assert (tmp_path / "ref" / name).exists()
    back = svb.SvbrdfIO(j, "cpu").load_textures_th(tmp_path / "ref", 16)
    assert float((back[:, 0:3] - t[:, 0:3]).abs().max()) <= 2.0 / 255 + 1e-6  # 8-bit PNG round trip


class FakeDescriptor:
    """loss_and_grad of a feature loss (0.5 |r - t|^2 mean), recording when it is used."""

    def __init__(self, name, log):
        self.name, self.log = name, log

    def load(self, targets):
        self.t = targets.detach().clone()

    def loss_and_grad(self, renders):
        self.log.append(self.name)
        d = renders - self.t
        return (0.5 * (d * d).mean()), torch.zeros(()), d / d.numel()


def test_latent_loop_picks_the_phase_feature_loss(svb):
    """A (latent-phase, noise-phase) descriptor pair: latent epochs use the first, noise
    epochs the second, as the reference's "L" and "N" losses; both load the targets."""
    sc, tg, gen = _setup(svb)
    log = []
    pair = (FakeDescriptor("L", log), FakeDescriptor("N", log))
    o = svb.materialgan.MaterialGANOptim("cpu", TorchRenderer(16, 9, sc.size, sc.cl), gen, descriptor=pair)
    o.load_targets(tg)
    assert torch.equal(pair[0].t, tg) and torch.equal(pair[1].t, tg)
    o.init_from(batch=1, seed=2)
    o.optim([7, 2, 1], 0.02)
    assert log == ["L", "L", "N", "L", "L", "N", "L"]
    assert len(o.loss_feature_list) == 7


def test_reference_helpers_of_the_latent_optimiser(svb):
    sc, tg, gen = _setup(svb)
    log = []
    pair = (FakeDescriptor("L", log), FakeDescriptor("N", log))
    o = svb.materialgan.MaterialGANOptim("cpu", TorchRenderer(16, 9, sc.size, sc.cl), gen, descriptor=pair)
    o.load_targets(tg)
    r = tg + 0.1
    assert torch.allclose(o.compute_image_loss(r), torch.tensor(0.01), atol=1e-6)
    assert float(o.compute_feature_loss(r, "N")) > 0 and log == ["N"]
    with pytest.raises(ValueError):
        o.compute_feature_loss(r, "X")
    leaves = o.gradient([torch.zeros(2), torch.ones(3)])
    assert all(t.requires_grad and t.is_leaf for t in leaves)
    bare = svb.materialgan.MaterialGANOptim("cpu", None, gen)
    bare.load_targets(tg)
    assert float(bare.compute_feature_loss(r, "L")) == 0.0
