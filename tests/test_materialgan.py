"""StyleGAN2-shaped generator (CPU) and the latent loop through the GPU renderer."""
import pytest
import torch


def _small_gen(svb, res=32, seed=0):
    return svb.materialgan.StyleGAN2Generator(resolution=res, w_dim=64, fmap_base=512, fmap_max=64, seed=seed,
                                              mapping_layers=2)


def test_generator_shapes_and_gradients(svb):
    gen = _small_gen(svb)
    assert gen.num_ws == 2 * 5 - 2
    assert gen.noise_res == [4, 8, 8, 16, 16, 32, 32]
    g = torch.Generator().manual_seed(1)
    wp = torch.randn(2, gen.num_ws, 64, generator=g).requires_grad_(True)
    noises = [n.requires_grad_(True) for n in gen.make_noises("random", 2)]
    t = svb.materialgan.latent_to_textures(gen, wp, noises)
    assert t.shape == (2, 9, 32, 32)
    assert t[:, 5].abs().max() <= 0.5 and t.abs().max() <= 1.0
    t.square().mean().backward()
    assert wp.grad is not None and wp.grad.abs().sum() > 0
    assert all(n.grad is not None for n in noises)


def test_generator_is_seeded(svb):
    a, b = _small_gen(svb, seed=3), _small_gen(svb, seed=3)
    wp = torch.zeros(1, a.num_ws, 64)
    assert torch.equal(a.synthesis(wp), b.synthesis(wp))
    c = _small_gen(svb, seed=4)
    assert not torch.equal(a.synthesis(wp), c.synthesis(wp))


def test_full_size_architecture(svb):
    gen = svb.materialgan.StyleGAN2Generator(resolution=256, seed=0)
    assert gen.num_ws == 14 and len(gen.noise_res) == 13
    assert gen.const.shape == (1, 512, 4, 4)
    assert gen.rgbs[-1].conv.weight.shape[0] == 9  # 9 texture channels
    assert gen.convs[-1].conv.weight.shape[0] == 128  # 128 channels at 256^2


def test_upsample_textures(svb):
    t = svb.scenes.make_material(16, 1000)
    up = svb.materialgan.upsample_textures(t, 32)
    assert up.shape == (1, 9, 32, 32)
    assert up.abs().max() <= 1.0
    assert (up[:, 3:5].pow(2).sum(1) <= 1.0 + 1e-5).all()


@pytest.mark.gpu
def test_latent_loop_through_gpu_renderer(svb, cuda):
    from oracle import microfacet_ref as R

    gen = svb.materialgan.StyleGAN2Generator(resolution=256, fmap_max=64, seed=0)
    sc = svb.scenes.single_scene(res=256, seed=1011)
    tg = torch.cat([R.render(svb.scenes.make_material(256, 1011 + i), sc.camera_pos, sc.light_pos, sc.light_pow,
                             sc.size, torch.float32) for i in range(2)])
    r = svb.Microfacet(256, 9, sc.size, [t.to(cuda) for t in sc.cl], cuda)
    o = svb.materialgan.MaterialGANOptim(cuda, r, gen)
    o.load_targets(tg.to(cuda))
    o.init_from(batch=2, seed=5)
    tex = o.optim([12, 4, 2], 0.02)
    assert tex.shape == (2, 9, 256, 256)
    assert len(o.loss_image_list) == 12
    assert min(o.loss_image_list[-4:]) < o.loss_image_list[0]


@pytest.mark.gpu
def test_refinement_handoff(svb, cuda):
    """Generator maps at 256 -> Lanczos 512 -> batched fused per-pixel refinement."""
    from oracle import microfacet_ref as R

    sc = svb.scenes.single_scene(res=512, seed=1012, render_fn=lambda *a: R.render(*a, dtype=torch.float32))
    coarse = svb.scenes.make_material(256, 1012)
    init = svb.materialgan.upsample_textures(coarse, 512)
    sc.init = init
    b = svb.BatchedOptim([sc], lr=0.01, loss="mse", device=cuda, config=svb.BatchConfig(384, 384, 0, 1))
    b.run(20)
    losses = b.loss_hist[:20, 0].tolist()
    assert losses[-1] < losses[0]
