"""optim_perpixel / render drop-ins (src/scripts.py:31-41, 67-97) end to end on a scene
folder written with the package's own image I/O."""
import json

import pytest
import torch

pytestmark = pytest.mark.gpu


def _scene_dir(svb, tmp_path, res=32):
    sc = svb.scenes.single_scene(res=res, seed=1007)
    cams = sc.camera_pos.tolist()
    cfg = {"reference_dir": "ref", "target_dir": "target", "optimize_dir": "optim", "rerender_dir": "rerender",
           "im_size": sc.size, "idx": list(range(9)), "camera_pos": cams, "light_pos": cams,
           "light_pow": sc.light_pow.tolist()}
    j = tmp_path / "scene.json"
    j.write_text(json.dumps(cfg))
    io = svb.SvbrdfIO(j, "cpu")
    io.save_textures_th(sc.gt, io.reference_dir)
    return j, sc


def test_render_then_optim_perpixel(svb, cuda, tmp_path):
    j, sc = _scene_dir(svb, tmp_path)
    out = svb.render(j, 32, device=cuda)
    assert out.shape == (9, 3, 32, 32)
    assert (tmp_path / "target" / "08.png").exists()
    opt = svb.optim_perpixel(j, 32, 0.02, 30, "const", device=cuda)
    assert len(opt.loss_image_list) == 30
    assert opt.loss_image_list[-1] < 0.5 * opt.loss_image_list[0]
    for name in ("nom.png", "dif.png", "spe.png", "rgh.png"):
        assert (tmp_path / "optim" / name).exists()
    assert (tmp_path / "rerender" / "00.png").exists()


def test_optim_perpixel_textures_init_and_light(svb, cuda, tmp_path):
    j, sc = _scene_dir(svb, tmp_path)
    svb.render(j, 32, device=cuda)
    opt = svb.optim_perpixel(j, 32, 0.01, 5, "textures", optim_light=True, device=cuda)
    # starting from the maps that rendered the targets, the loss is only 8-bit noise
    assert opt.loss_image_list[0] < 1e-3
    assert torch.isfinite(opt.light_pow).all()
    with pytest.raises(ValueError):
        svb.optim_perpixel(j, 32, 0.01, 1, "bogus", device=cuda)
