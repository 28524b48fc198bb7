"""Failure detection without a GPU fault, and checkpoint/resume.

* A bounded wait that nothing completes gives up, records its code in the workspace error
  word and returns; the host reads the word and raises; the context stays usable.
* Optimiser state saved to disk and loaded into a new optimiser continues bit-identically.
* Each SvbrdfOptim.optim call starts a fresh Adam, as the reference's does."""
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _mats(svb, n=3):
    from oracle import microfacet_ref as R
    return svb.scenes.batched_scenes(n=n, resolutions=(16, 32), vmin=3, vmax=7,
                                     render_fn=lambda *a: R.render(*a, dtype=torch.float32))


def test_bounded_wait_times_out_and_reports(svb, cuda):
    N = svb._native
    L = N.lib()
    ws = torch.zeros(16, dtype=torch.uint8, device=cuda)
    N.check(L.svbrdf_selftest_wait_timeout(ws.data_ptr(), ws.numel(), 2000, N.stream_handle(cuda)))
    torch.cuda.synchronize()
    w = ws.view(torch.int32).cpu().tolist()
    assert w[1] == 1  # "copy never landed"
    assert w[2] == 1 and w[3] == 0  # the completed wait, the one that ran out
    # the context is still usable: a batched run afterwards is healthy
    b = svb.BatchedOptim(_mats(svb, 2), device=cuda, config=svb.BatchConfig(480, 960, 0, 3))
    b.run(3)
    b.check()
    assert b.device_error() == 0


def test_host_turns_the_error_word_into_an_exception(svb, cuda):
    """The word a timed-out launch leaves (set here from the host) fails the next check."""
    N = svb._native
    b = svb.BatchedOptim(_mats(svb, 2), device=cuda, config=svb.BatchConfig(480, 960, 0, 2))
    b.run(2)
    b.check()
    off = N.WORKSPACE_ERROR_OFFSET
    b.ws[off:off + 4].view(torch.int32).fill_(2)
    assert b.device_error() == 2
    with pytest.raises(svb.SvbrdfError):
        b.check()


@pytest.mark.parametrize("variant", [2, 3])
def test_batched_checkpoint_resume_is_exact(svb, cuda, tmp_path, variant):
    mats = _mats(svb)
    cfg = svb.BatchConfig(480, 960, 0, variant)
    a = svb.BatchedOptim(mats, device=cuda, config=cfg, hist_len=20)
    a.run(5)
    a.save(tmp_path / "ck.pt")
    a.run(7)
    b = svb.BatchedOptim(mats, device=cuda, config=cfg, hist_len=20)
    b.load(tmp_path / "ck.pt")
    b.run(7)
    for i in range(len(mats)):
        assert torch.equal(a.tex[i], b.tex[i])
        assert torch.equal(a.m1[i], b.m1[i]) and torch.equal(a.m2[i], b.m2[i])
    assert torch.equal(a.loss_hist, b.loss_hist)
    assert int(b.step_dev.item()) == 12 and b.step_count == 12
    other = svb.BatchedOptim(_mats(svb, 2), device=cuda, config=cfg, hist_len=20)
    with pytest.raises(ValueError):
        other.load(tmp_path / "ck.pt")


def test_fused_optim_calls_start_fresh_adam_and_checkpoint(svb, cuda, tmp_path):
    """Two optim calls follow the reference's two loops, each with a new Adam; the maps
    saved after them load into a new optimiser unchanged."""
    from oracle import microfacet_ref as R
    sc = svb.scenes.single_scene(res=64, seed=1014)
    svb.scenes.add_targets(sc, lambda *a: R.render(*a, dtype=torch.float32))
    r = svb.Microfacet(64, 9, sc.size, [t.to(cuda) for t in sc.cl], cuda)
    o = svb.SvbrdfOptim(cuda, r, loss="log1p")
    o.load_targets(sc.targets.to(cuda))
    o.init_from_tex(sc.init.to(cuda))
    o.optim(3, 0.01, None, False)
    o.optim(4, 0.01, None, False)
    ref = R.optim_loop(sc.init, sc.targets, sc.camera_pos, sc.light_pos, sc.light_pow, sc.size, 3, 0.01, "log1p",
                       False, torch.float64)
    ref = R.optim_loop(ref["textures"], sc.targets, sc.camera_pos, sc.light_pos, sc.light_pow, sc.size, 4, 0.01,
                       "log1p", False, torch.float64)
    assert rel_l2(o.textures.detach(), ref["textures"]) <= 2e-5
    assert rel_l2(o.exp_avg_sq, ref["exp_avg_sq"]) <= 1e-4
    o.save(tmp_path / "perpixel.pt")
    o2 = svb.SvbrdfOptim(cuda, r, loss="log1p")
    o2.load(tmp_path / "perpixel.pt")
    assert torch.equal(o2.textures.detach(), o.textures.detach())
    assert o2._step == 4 and o2.loss_image_list == o.loss_image_list


def test_latent_save_and_resume(svb, cuda, tmp_path):
    gen = svb.materialgan.StyleGAN2Generator(resolution=32, fmap_max=32, seed=0)
    sc = svb.scenes.single_scene(res=32, seed=1015)
    r = svb.Microfacet(32, 9, sc.size, [t.to(cuda) for t in sc.cl], cuda)
    o = svb.materialgan.MaterialGANOptim(cuda, r, gen)
    o.load_targets(torch.rand(9, 3, 32, 32).to(cuda))
    o.init_from(batch=1, seed=3, noise="random")
    o.save_latent(tmp_path / "optim_latent.pt", tmp_path / "optim_noise.pt")
    t0 = o.latent_to_textures().detach()
    o2 = svb.materialgan.MaterialGANOptim(cuda, r, gen)
    o2.load_targets(torch.rand(9, 3, 32, 32).to(cuda))
    o2.init_from(batch=1, seed=99)
    o2.load_latent(tmp_path / "optim_latent.pt", tmp_path / "optim_noise.pt")
    assert torch.equal(o2.latent_to_textures().detach(), t0)
