"""Pin the CPU oracle to the reference: fixtures made by running the reference's own
src/microfacet.py and src/svbrdf.py (tests/golden/make_golden.py)."""
import pytest
import torch

from conftest import rel_l2


def _scene(d):
    return d["camera_pos"], d["light_pos"], d["light_pow"], float(d["size"])


def test_render_coloc_matches_reference(golden, oracle):
    d = golden("render_coloc_20.npz")
    cam, lit, lp, size = _scene(d)
    o32 = oracle.render(d["textures_gt"], cam, lit, lp, size, torch.float32)
    o64 = oracle.render(d["textures_gt"], cam, lit, lp, size, torch.float64)
    # same op sequence in the same precision: bit-identical on this host
    assert torch.equal(o32, d["render_gt32"])
    assert rel_l2(o64, d["render_gt64"]) < 1e-14
    # the reference's own FP32 noise against FP64, which every FP32 result inherits
    assert rel_l2(d["render_gt32"], d["render_gt64"]) < 1e-5


@pytest.mark.parametrize("kind", ["mse", "log1p"])
def test_grad_general_matches_reference(golden, oracle, kind):
    d = golden("render_general_24.npz")
    cam, lit, lp, size = _scene(d)
    for dt, tag, tol in ((torch.float32, "32", 1e-6), (torch.float64, "64", 1e-12)):
        loss, g, gp = oracle.loss_and_grad(d["textures"], d["targets"], cam, lit, lp, size, kind, dt, grad_light=True)
        assert abs(loss - float(d[f"loss_{kind}{tag}"])) <= tol * abs(loss) + 1e-12
        assert rel_l2(g, d[f"grad_{kind}{tag}"]) < tol
        assert rel_l2(gp, d[f"gradpow_{kind}{tag}"]) < tol


def test_grad_coloc_matches_reference(golden, oracle):
    d = golden("render_coloc_20.npz")
    cam, lit, lp, size = _scene(d)
    loss, g, _ = oracle.loss_and_grad(d["textures"], d["targets"], cam, lit, lp, size, "mse", torch.float64)
    assert rel_l2(g, d["grad_mse64"]) < 1e-12
    # The reference's own FP32 autograd sits ~1.4e-4 (relative L2) from FP64 here: the
    # normal and roughness terms lose digits to 1 - cos^2 cancellation near highlights.
    # The GPU tests hold the kernels to 1e-4 or to this level, whichever is larger.
    assert rel_l2(d["grad_mse32"], d["grad_mse64"]) < 5e-4


@pytest.mark.parametrize("name,light", [("optim_traj_16.npz", False), ("optim_traj_light_16.npz", True)])
def test_optim_loop_matches_reference(golden, oracle, name, light):
    d = golden(name)
    cam, lit, _, size = _scene({**d, "light_pow": d["light_pow0"]})
    r = oracle.optim_loop(d["init"], d["targets"], cam, lit, d["light_pow0"], size, int(d["epochs"]),
                          float(d["lr"]), "mse", light, torch.float32)
    assert rel_l2(r["textures"], d["textures"]) < 1e-6
    assert rel_l2(r["exp_avg"], d["exp_avg"]) < 1e-5
    assert max(abs(a - b) / b for a, b in zip(r["loss"], d["loss"].tolist())) < 1e-5
    if light:
        assert rel_l2(r["light_pow"], d["light_pow"]) < 1e-7


def test_fd_matches_fp64_autograd(golden, oracle):
    d = golden("render_general_24.npz")
    cam, lit, lp, size = _scene(d)
    texels = [(12, 3), (15, 20), (20, 11)]
    fd = oracle.fd_gradient(d["textures"], d["targets"], cam, lit, lp, size, texels, "mse", h=1e-6)
    g = d["grad_mse64"]
    ad = torch.stack([g[0, :, i, j] for i, j in texels])
    assert rel_l2(fd, ad) < 1e-6
