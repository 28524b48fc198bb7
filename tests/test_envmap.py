"""Novel-view rendering under an environment map (the reference's MitsubaRender video,
src/mitsubarender.py:7-105, src/scripts.py:44-59): the CPU oracle's own checks, and the CUDA
kernel against the oracle on the same random numbers."""
import math

import numpy as np
import pytest
import torch

from conftest import rel_l2


def _white_furnace_textures(h=8, w=8):
    tex = np.zeros((9, h, w))
    tex[0:3] = 1.0   # diffuse albedo 1 (stored value 1 -> PNG 1 -> linear 1)
    tex[6:9] = -1.0  # specular reflectance 0
    tex[3:5] = 0.0   # flat normal
    tex[5] = 0.0     # roughness 0.5 in storage
    return tex


def test_env_distribution_is_normalised(svb):
    env = svb.envmap.synthetic_envmap(16, 32, seed=2)
    rc, rp, cc, cp = svb.envmap.env_distribution(env)
    assert rc.shape == (17,) and cc.shape == (16, 33) and rp.shape == (16,) and cp.shape == (16, 32)
    assert rc[0] == 0.0 and rc[-1] == 1.0 and np.all(np.diff(rc) >= 0)
    assert np.all(cc[:, 0] == 0.0) and np.all(cc[:, -1] == 1.0) and np.all(np.diff(cc, axis=1) >= 0)
    assert abs(float((rp[:, None] * cp).sum()) - 1.0) < 1e-5
    # the solid-angle pdf integrates to one over the sphere
    from oracle import envmap_ref as E
    g = np.random.default_rng(0)
    d = g.normal(size=(200000, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    _, pdf = E._env_eval(env, rp, cp, d, 1.0)
    assert abs(float(pdf.mean()) * 4 * math.pi - 1.0) < 0.02


def test_oracle_white_furnace(svb):
    """A white diffuse (albedo 1, no specular) blend under a constant unit environment
    reflects 0.5 (the blend weight); pixels that miss the rectangle see the environment."""
    from oracle import envmap_ref as E
    env = np.ones((8, 16, 3), np.float32)
    tables = svb.envmap.env_distribution(env)
    img = E.render(_white_furnace_textures(), env, tables, 8, 0.0, 1.0, spp=512, seed=3)
    rad = img ** 2.2
    assert np.allclose(rad[0, 0], 1.0)  # a corner misses the rectangle
    centre = rad[3:5, 3:5]
    assert np.all(np.abs(centre - 0.5) < 0.03), centre


def test_video_angles_and_validation(svb):
    a = svb.envmap.video_angles()
    assert a.shape == (59,) and a[0] == pytest.approx(-40.0) and a[-1] == pytest.approx(40.0) and a[29] == pytest.approx(0.0, abs=1e-9)
    with pytest.raises(ValueError):
        svb.envmap.env_distribution(np.zeros((4, 8, 3), np.float32))


@pytest.mark.gpu
@pytest.mark.parametrize("angle", [-40.0, 0.0, 23.0])
def test_kernel_matches_oracle(svb, cuda, angle):
    """The CUDA renderer against the FP64 oracle: same scene, same random numbers. FP32
    against FP64 rounding may flip a rare discrete choice (a rectangle edge, an environment
    texel boundary), so the images are compared in relative L2."""
    from oracle import envmap_ref as E
    mat = svb.scenes.make_material(24, 4321)[0].numpy()  # [9, 24, 24] parameters
    env = svb.envmap.synthetic_envmap(16, 32, seed=5)
    r = svb.EnvmapRenderer([32, 32], env, torch.from_numpy(mat), device=cuda, spp=16, seed=11)
    got = r.render(angle, 0.5)
    want = E.render(mat, env, r.tables_np, 32, angle, 0.5, spp=16, seed=11)
    assert got.shape == (32, 32, 3) and np.isfinite(got).all()
    # a flipped environment-texel choice moves one sample of one pixel by up to the contrast
    # of the map's bright lobes, so the image-wide bound is loose and the per-pixel one tight
    assert rel_l2(torch.from_numpy(got), torch.from_numpy(want)) <= 1e-2
    assert np.mean(np.abs(got - want) < 2e-3) >= 0.95


@pytest.mark.gpu
def test_kernel_white_furnace_and_video(svb, cuda):
    env = np.ones((8, 16, 3), np.float32)
    tex = torch.from_numpy(_white_furnace_textures()).float()
    r = svb.EnvmapRenderer([16, 16], env, tex, device=cuda, spp=1024, seed=7)
    rad = r.render(0.0, 1.0) ** 2.2
    assert np.allclose(rad[0, 0], 1.0, atol=1e-6)
    assert np.all(np.abs(rad[7:9, 7:9] - 0.5) < 0.02), rad[7:9, 7:9]
    r.spp = 4
    frames = r.render_video(n=5, light_intensity=0.5)
    assert len(frames) == 5 + 3 and all(f.shape == (16, 16, 3) for f in frames)
    assert np.array_equal(frames[5], frames[3]) and np.array_equal(frames[7], frames[1])
