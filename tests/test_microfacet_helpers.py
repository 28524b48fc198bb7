"""The reference's tensor helpers on Microfacet (src/microfacet.py:16-20, 54-79), run on the
CPU: the renderer object is made without its CUDA set-up, since the helpers need none."""
import torch

from oracle import microfacet_ref as R


def _renderer(svb, res=8, n=2, size=17.0):
    r = object.__new__(svb.Microfacet)
    r.res, r.n_of_imgs, r.size, r.eps, r.device = res, n, size, 1e-6, torch.device("cpu")
    return r


def test_pixel_grid_and_directions(svb):
    r = _renderer(svb)
    pos = r.pos
    assert pos.shape == (2, 3, 8, 8)
    assert torch.equal(pos[0], R.pixel_positions(8, 17.0, torch.float32))
    cam = torch.tensor([[1.0, -2.0, 30.0], [0.0, 0.0, 25.0]])
    d, dist2 = r.get_dir(cam)
    vec = cam[:, :, None, None] - pos
    assert torch.allclose(dist2[:, 0], (vec * vec).sum(1))
    assert torch.allclose(d, vec / vec.norm(dim=1, keepdim=True))
    assert torch.equal(r.dot(vec, vec)[:, 1], r.dot(vec, vec)[:, 2])  # expanded to 3 channels


def test_tex2map_matches_the_oracle_decode(svb):
    r = _renderer(svb, res=16, n=3)
    t = svb.scenes.make_material(16, 77)
    normal, diffuse, specular, roughness = r.tex2map(t)
    assert normal.shape == diffuse.shape == specular.shape == roughness.shape == (3, 3, 16, 16)
    assert torch.allclose(diffuse[0], ((t[0, 0:3] + 1) / 2) ** 2.2)
    assert torch.allclose(roughness[1, 2], ((t[0, 5] + 1) / 2) ** 2.2)
    assert torch.allclose(specular[2], ((t[0, 6:9] + 1) / 2) ** 2.2)
    assert torch.allclose(normal[0:1], R._reconstruct_normal(t[:, 3:5]), atol=1e-6)
    assert torch.allclose(normal.norm(dim=1), torch.ones(3, 16, 16), atol=1e-6)
