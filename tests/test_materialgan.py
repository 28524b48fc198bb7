"""StyleGAN2-shaped generator (CPU) and the latent loop through the GPU renderer."""
import pytest
import torch

from conftest import rel_l2


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
    # a second call continues from the current latent and appends its losses, on both the
    # graph path and the eager one
    o.optim([3, 2, 1], 0.02)
    o.optim([2, 1, 1], 0.02, graph=False)
    assert len(o.loss_image_list) == 17 and all(isinstance(x, float) for x in o.loss_image_list)


@pytest.mark.gpu
def test_latent_graph_matches_eager(svb, cuda):
    """The CUDA-graph epochs follow the eager loop (fresh torch Adam each epoch).

    A fresh Adam's step is lr g / (|g| + eps): every element moves by about lr whatever its
    gradient's size, so rounding-level differences in near-zero gradients flip steps and the
    two trajectories part after a step or two. The first loss (no step yet) and the second
    (one step) agree to rounding. After that, both runs only have to descend alike: by 30% or
    more, ending within 30% of each other (how far apart they end depends on where the
    rounding of the reductions first flips a step, so a tighter bound is a coin toss). TF32 is
    off for both runs, since the convolution algorithms picked under capture and eagerly
    may round differently."""
    from oracle import microfacet_ref as R

    tf32 = torch.backends.cudnn.allow_tf32, torch.backends.cuda.matmul.allow_tf32
    torch.backends.cudnn.allow_tf32 = torch.backends.cuda.matmul.allow_tf32 = False

    gen = svb.materialgan.StyleGAN2Generator(resolution=256, fmap_max=64, seed=0)
    sc = svb.scenes.single_scene(res=256, seed=1012)
    tg = torch.cat([R.render(svb.scenes.make_material(256, 1012 + i), sc.camera_pos, sc.light_pos, sc.light_pow,
                             sc.size, torch.float32) for i in range(2)])
    r = svb.Microfacet(256, 9, sc.size, [t.to(cuda) for t in sc.cl], cuda)
    runs = []
    for graph in (False, True):
        o = svb.materialgan.MaterialGANOptim(cuda, r, gen)
        o.load_targets(tg.to(cuda))
        o.init_from(batch=2, seed=6)
        tex = o.optim([9, 3, 2], 0.02, graph=graph)
        runs.append((tex.clone(), list(o.loss_image_list), o.latent.detach().clone()))
    torch.backends.cudnn.allow_tf32, torch.backends.cuda.matmul.allow_tf32 = tf32
    (t0, l0, w0), (t1, l1, w1) = runs
    assert len(l1) == 9
    assert abs(l1[0] - l0[0]) <= 1e-6 * l0[0]
    assert abs(l1[1] - l0[1]) <= 1e-5 * l0[1]
    assert l0[-1] < 0.7 * l0[0] and l1[-1] < 0.7 * l1[0]
    assert abs(l1[-1] - l0[-1]) <= 0.3 * l0[-1]
    assert torch.isfinite(t1).all() and t1.shape == t0.shape


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


def test_upsample_polyphase_matches_fir(svb):
    """The separable polyphase 2x up-sampling equals zero insertion + the 4x4 FIR."""
    MG = svb.materialgan
    x = torch.randn(2, 5, 7, 9, dtype=torch.float64, generator=torch.Generator().manual_seed(3))
    assert torch.allclose(MG._upsample2(x), MG._upsample2_fir(x), rtol=0, atol=1e-14)


def test_unfused_modulated_conv_matches_per_sample_weights(svb):
    """Input scaling + shared-weight conv + output demodulation equals the convolution with
    per-sample modulated, demodulated weights."""
    MG = svb.materialgan
    g = torch.Generator().manual_seed(4)
    conv = MG._ModConv(8, 6, 3, 16, g).double()
    x = torch.randn(3, 8, 10, 10, dtype=torch.float64, generator=g)
    w = torch.randn(3, 16, dtype=torch.float64, generator=g)
    s = conv.affine(w)
    wt = conv.weight[None] * conv.scale * s[:, None, :, None, None]
    wt = wt * torch.rsqrt(wt.pow(2).sum(dim=(2, 3, 4), keepdim=True) + 1e-8)
    ref = torch.nn.functional.conv2d(x.reshape(1, 24, 10, 10), wt.reshape(18, 8, 3, 3), padding=1, groups=3)
    assert torch.allclose(conv(x, w), ref.reshape(3, 6, 10, 10), rtol=1e-12, atol=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("channels_last", [False, True])
@pytest.mark.parametrize("shape", [(2, 5, 7, 9), (2, 5, 4, 8), (1, 3, 12, 4), (2, 8, 5, 3)])
def test_upsample_kernel_matches_fir(svb, cuda, shape, channels_last):
    """The CUDA up-sampling and its adjoint against the FIR form (FP64 on the CPU): scalar
    kernels for odd widths (NCHW) or channel counts (NHWC), float4 kernels otherwise."""
    MG = svb.materialgan
    g = torch.Generator().manual_seed(7)
    x = torch.randn(*shape, generator=g)
    ref = MG._upsample2_fir(x.double())
    xd = x.to(cuda)
    if channels_last:
        xd = xd.contiguous(memory_format=torch.channels_last)
    xc = xd.requires_grad_(True)
    y = MG._upsample2(xc)
    assert torch.allclose(y.double().cpu(), ref, rtol=0, atol=1e-5)
    go = torch.randn(shape[0], shape[1], 2 * shape[2], 2 * shape[3], generator=g)
    y.backward(go.to(cuda))
    xr = x.double().requires_grad_(True)
    MG._upsample2_fir(xr).backward(go.double())
    assert torch.allclose(xc.grad.double().cpu(), xr.grad, rtol=0, atol=1e-5)


@pytest.mark.gpu
@pytest.mark.parametrize("channels_last", [False, True])
@pytest.mark.parametrize("with_noise,hw", [(True, (9, 7)), (False, (9, 7)), (True, (8, 12)), (False, (4, 4))])
def test_style_layer_kernels_match_torch(svb, cuda, with_noise, hw, channels_last):
    """A style layer through the modulation and epilogue kernels against the same layer in
    FP64 torch on the CPU: the output and the gradients of the input, the style vector and the
    noise map (the latent loop's only gradients)."""
    MG = svb.materialgan
    g = torch.Generator().manual_seed(11)
    layer = MG._StyleLayer(12, 10, 16, g, up=True)
    with torch.no_grad():
        layer.bias.copy_(torch.randn(10, generator=g) * 0.3)
        layer.noise_strength.fill_(0.7)
    for p in layer.parameters():
        p.requires_grad_(False)
    h, wd = hw  # (9, 7) runs the scalar kernels, multiples of 4 the float4 ones
    x = torch.randn(3, 12, h, wd, generator=g)
    w = torch.randn(3, 16, generator=g)
    nz = torch.randn(3, 1, 2 * h, 2 * wd, generator=g) if with_noise else None
    go = torch.randn(3, 10, 2 * h, 2 * wd, generator=g)

    ref = MG._StyleLayer(12, 10, 16, torch.Generator().manual_seed(0), up=True).double()
    ref.load_state_dict({k: v.double() for k, v in layer.state_dict().items()})
    for p in ref.parameters():
        p.requires_grad_(False)
    xr, wr = x.double().requires_grad_(True), w.double().requires_grad_(True)
    nr = nz.double().requires_grad_(True) if with_noise else None
    yr = ref(xr, wr, nr)
    yr.backward(go.double())

    lc = layer.to(cuda)
    xd = x.to(cuda)
    if channels_last:  # the NHWC kernels (12 input and 10 output channels: both vector widths)
        xd = xd.contiguous(memory_format=torch.channels_last)
    xc, wc = xd.requires_grad_(True), w.to(cuda).requires_grad_(True)
    nc = nz.to(cuda).requires_grad_(True) if with_noise else None
    torch.backends.cudnn.allow_tf32 = False
    try:
        yc = lc(xc, wc, nc)
        yc.backward(go.to(cuda))
    finally:
        torch.backends.cudnn.allow_tf32 = True
    assert yc.is_contiguous(memory_format=torch.channels_last) == channels_last
    assert rel_l2(yc.detach(), yr.detach()) < 1e-5
    assert rel_l2(xc.grad.double().cpu(), xr.grad) < 1e-5
    assert rel_l2(wc.grad.double().cpu(), wr.grad) < 1e-5
    if with_noise:
        assert rel_l2(nc.grad.double().cpu(), nr.grad) < 1e-5


@pytest.mark.gpu
def test_generator_channels_last_matches_nchw(svb, cuda):
    """The whole generator with channels-last feature maps (the NHWC kernels, cuDNN without
    layout conversions) against the same weights run NCHW: textures, and the gradients of
    the latent and of every noise map, in FP32 with TF32 off."""
    MG = svb.materialgan
    outs = []
    torch.backends.cudnn.allow_tf32 = False
    try:
        for cl in (False, True):
            gen = MG.StyleGAN2Generator(resolution=64, fmap_max=64, seed=3, channels_last=cl).to(cuda)
            for p in gen.parameters():
                p.requires_grad_(False)
            with torch.no_grad():
                for m in gen.modules():
                    if isinstance(m, MG._StyleLayer):
                        m.noise_strength.fill_(0.3)
                        m.bias.normal_(0.0, 0.2, generator=torch.Generator(device=cuda).manual_seed(1))
            gz = torch.Generator().manual_seed(9)
            wp = (torch.randn(2, gen.num_ws, gen.w_dim, generator=gz) * 0.5).to(cuda).requires_grad_(True)
            noises = [n.requires_grad_(True) for n in gen.make_noises("random", 2, cuda, seed=4)]
            t = gen.synthesis(wp, noises)
            go = torch.randn(t.shape, generator=torch.Generator().manual_seed(5)).to(cuda)
            (t * go).sum().backward()
            outs.append((t.detach().contiguous(), wp.grad.clone(), [n.grad.clone() for n in noises]))
    finally:
        torch.backends.cudnn.allow_tf32 = True
    (t0, g0, n0), (t1, g1, n1) = outs
    assert rel_l2(t1, t0) < 1e-5
    assert rel_l2(g1, g0) < 1e-4
    for a, b in zip(n1, n0):
        assert rel_l2(a, b) < 1e-4


def _reference_generator(svb, device="cpu", dtype=torch.float64):
    """Our generator carrying the weights of tests/golden/generator_ref_256.npz (drawn from
    numpy, loaded through load_reference_state_dict), plus the fixture and its inputs."""
    import importlib
    import sys

    import numpy as np

    from conftest import GOLDEN
    if str(GOLDEN) not in sys.path:
        sys.path.insert(0, str(GOLDEN))
    MG = importlib.import_module("make_golden_nets")
    d = dict(np.load(GOLDEN / "generator_ref_256.npz"))
    vals = MG.generator_state(MG.fixture_key_shapes(d["keys"], d["key_shapes"]), int(d["seed_weights"]))
    gen = svb.materialgan.StyleGAN2Generator(256, out_channels=9, seed=0, channels_last=True).to(device, dtype)
    gen.load_reference_state_dict({k: torch.from_numpy(v) for k, v in vals.items()})
    wp, noises, R, z = MG.generator_inputs(seed=int(d["seed_inputs"]))
    return gen, d, wp, noises, R, z


def test_generator_matches_reference_network(svb):
    """Pinned to the reference's own StyleGAN2GeneratorNet (src/higan_models/
    stylegan2_generator_network.py:36) as MaterialGAN builds it, run in FP64 on numpy-drawn
    weights (tests/golden/generator_ref_256.npz): synthesis(W+) output, its gradient with
    respect to W+ and the 13 noise maps, and the mapping network, all within 1e-9. This ties
    channel counts, W+ indices, noise order, the up-sampling convolutions, toRGB skips and the
    style/demodulation arithmetic to the reference."""
    gen, d, wp_np, noises_np, R_np, z_np = _reference_generator(svb)
    wp = torch.from_numpy(wp_np).requires_grad_(True)
    noises = [torch.from_numpy(n).requires_grad_(True) for n in noises_np]
    out = gen.synthesis(wp, noises)
    loss = (out * torch.from_numpy(R_np)).sum()
    loss.backward()
    o = out.detach().reshape(-1)
    assert abs(float(loss.detach()) - float(d["loss"])) <= 1e-9 * abs(float(d["loss"]))
    assert torch.allclose(o[torch.from_numpy(d["out_idx"])], torch.from_numpy(d["out_val"]), rtol=1e-9, atol=1e-12)
    on = out.detach().pow(2).sum((0, 2, 3)).sqrt()
    assert torch.allclose(on, torch.from_numpy(d["out_norm"]), rtol=1e-10)
    assert rel_l2(wp.grad, torch.from_numpy(d["grad_wp"])) <= 1e-9
    for i, n in enumerate(noises):
        g = n.grad.reshape(-1)
        assert abs(float(g.norm()) - float(d[f"noise{i}_norm"])) <= 1e-9 * float(d[f"noise{i}_norm"])
        assert torch.allclose(g[torch.from_numpy(d[f"noise{i}_idx"])], torch.from_numpy(d[f"noise{i}_val"]),
                              rtol=1e-8, atol=1e-10)
    with torch.no_grad():
        w = gen.truncate(gen.map(torch.from_numpy(z_np)))
    assert rel_l2(w[0], torch.from_numpy(d["w_mapped"])) <= 1e-12


@pytest.mark.gpu
def test_gpu_generator_matches_reference_network(svb, cuda):
    """The GPU generator (channels-last maps, the NHWC kernels with the up-sampling halo,
    cuDNN convolutions in FP32 with TF32 off) on the reference network's fixture
    (tests/golden/generator_ref_256.npz): output, W+ gradient and noise gradients within
    FP32 accuracy of the reference's FP64 run: the output within 1e-5, the gradients within
    three times the error of the same network run in FP32 on the CPU (at least 1e-4)."""
    gen, d, wp_np, noises_np, R_np, _ = _reference_generator(svb, cuda, torch.float32)
    for p in gen.parameters():
        p.requires_grad_(False)
    torch.backends.cudnn.allow_tf32 = False
    try:
        wp = torch.from_numpy(wp_np).float().to(cuda).requires_grad_(True)
        noises = [torch.from_numpy(n).float().to(cuda).requires_grad_(True) for n in noises_np]
        out = gen.synthesis(wp, noises)
        loss = (out * torch.from_numpy(R_np).float().to(cuda)).sum()
        loss.backward()
    finally:
        torch.backends.cudnn.allow_tf32 = True
    o = out.detach().double().cpu()
    # the same network in FP32 on the CPU (torch ops) sets the FP32 error floor of the gradients
    gc, _, _, _, _, _ = _reference_generator(svb, "cpu", torch.float32)
    wc = torch.from_numpy(wp_np).float().requires_grad_(True)
    nc = [torch.from_numpy(n).float().requires_grad_(True) for n in noises_np]
    (gc.synthesis(wc, nc) * torch.from_numpy(R_np).float()).sum().backward()
    e32_wp = rel_l2(wc.grad, torch.from_numpy(d["grad_wp"]))
    e32_n = max(abs(float(n.grad.double().norm()) - float(d[f"noise{i}_norm"])) / float(d[f"noise{i}_norm"])
                for i, n in enumerate(nc))
    e_wp = rel_l2(wp.grad, torch.from_numpy(d["grad_wp"]))
    e_n = max(abs(float(n.grad.double().norm()) - float(d[f"noise{i}_norm"])) / float(d[f"noise{i}_norm"])
              for i, n in enumerate(noises))
    print(f"FP32 generator vs reference FP64: W+ gradient GPU {e_wp:.2e} (CPU FP32 {e32_wp:.2e}), "
          f"noise-gradient norms GPU {e_n:.2e} (CPU FP32 {e32_n:.2e})")
    assert abs(float(loss.detach()) - float(d["loss"])) <= 1e-4 * abs(float(d["loss"]))
    ov = o.reshape(-1)[torch.from_numpy(d["out_idx"])]
    assert rel_l2(ov, torch.from_numpy(d["out_val"])) <= 1e-5
    assert rel_l2(o.pow(2).sum((0, 2, 3)).sqrt(), torch.from_numpy(d["out_norm"])) <= 1e-5
    assert e_wp <= max(1e-4, 3 * e32_wp)
    assert e_n <= max(1e-4, 3 * e32_n)


@pytest.mark.gpu
@pytest.mark.parametrize("b,h,cin,cout,k,pad", [(16, 4, 512, 512, 3, 1), (3, 8, 512, 512, 3, 1), (2, 10, 512, 256, 3, 0),
                                                 (2, 18, 256, 128, 3, 0), (1, 32, 128, 128, 3, 1),
                                                 (2, 16, 128, 9, 1, 0), (2, 20, 128, 64, 3, 1),
                                                 (16, 64, 64, 64, 3, 1), (24, 64, 64, 256, 3, 1),
                                                 (16, 66, 128, 128, 3, 0), (2, 32, 256, 256, 3, 1),
                                                 (4, 40, 512, 256, 3, 0), (3, 64, 256, 512, 3, 1),
                                                 (16, 64, 256, 256, 3, 1)])
def test_conv_tf32_matches_torch(svb, cuda, b, h, cin, cout, k, pad):
    """The TF32 tensor-core convolution (forward and data gradient through _ConvTF32) against
    torch's FP32 convolution of the same channels-last maps: relative L2 <= 2e-3 (TF32 rounds
    both operands to 10 mantissa bits; FP32 accumulation). The shapes cover the 4^2 and 8^2
    patches, two M-tiles per CTA tile (with a partial second one at 20 rows), maps with more
    tiles than SMs, where each persistent CTA runs several tiles through both TMEM accumulator
    buffers, and deep 256- and 512-channel maps (a partial tile at 38 rows, several tiles per
    CTA)."""
    MG = svb.materialgan
    g = torch.Generator().manual_seed(b * h + cin)
    x = torch.randn(b, cin, h, h, generator=g).to(cuda).contiguous(memory_format=torch.channels_last)
    w = (torch.randn(cout, cin, k, k, generator=g) / (cin * k * k) ** 0.5).to(cuda)
    conv = MG._ModConv(cin, cout, k, 512, torch.Generator().manual_seed(0)).to(cuda)
    conv.requires_grad_(False)
    with torch.no_grad():
        conv.weight.copy_(w / conv.scale)
    w_fwd, w_dg = conv._tf32_weights(conv.weight * conv.scale)
    xr = x.clone().requires_grad_(True)
    y = MG._ConvTF32.apply(xr, w_fwd, w_dg, cout, k, pad)
    gy = torch.randn(y.shape, generator=g).to(cuda)
    (y * gy).sum().backward()
    torch.backends.cudnn.allow_tf32 = False
    try:
        x2 = x.clone().requires_grad_(True)
        ref = torch.nn.functional.conv2d(x2, w, padding=pad)
        (ref * gy).sum().backward()
    finally:
        torch.backends.cudnn.allow_tf32 = True
    torch.cuda.synchronize()
    assert MG.generator_device_error(cuda) == 0
    assert y.shape == ref.shape
    assert rel_l2(y, ref) <= 2e-3
    assert rel_l2(xr.grad, x2.grad) <= 2e-3


def _tf32_generator_errors(svb, cuda, gen, d, wp_np, noises_np, R_np):
    """Errors of one GPU synthesis + backward against the reference network's FP64 fixture:
    (output at the fixture's indices, W+ gradient, worst noise-gradient norm), relative."""
    wp = torch.from_numpy(wp_np).float().to(cuda).requires_grad_(True)
    noises = [torch.from_numpy(n).float().to(cuda).requires_grad_(True) for n in noises_np]
    out = gen.synthesis(wp, noises)
    (out * torch.from_numpy(R_np).float().to(cuda)).sum().backward()
    torch.cuda.synchronize()
    assert svb.materialgan.generator_device_error(cuda) == 0
    o = out.detach().double().cpu()
    e_out = rel_l2(o.reshape(-1)[torch.from_numpy(d["out_idx"])], torch.from_numpy(d["out_val"]))
    e_wp = rel_l2(wp.grad, torch.from_numpy(d["grad_wp"]))
    e_n = max(abs(float(n.grad.double().norm()) - float(d[f"noise{i}_norm"])) / float(d[f"noise{i}_norm"])
              for i, n in enumerate(noises))
    return e_out, e_wp, e_n


@pytest.mark.gpu
@pytest.mark.parametrize("b,h,cin,cout,k,pad", [(16, 4, 512, 512, 3, 1), (16, 8, 512, 512, 3, 1),
                                                 (16, 16, 512, 512, 3, 1), (16, 6, 512, 512, 3, 2),
                                                 (16, 8, 512, 32, 1, 0)])
def test_conv_tf32_split_k_matches_unsplit(svb, cuda, b, h, cin, cout, k, pad):
    """The generator's small maps (4^2 to 16^2, 512 channels) split K over a workspace
    (svbrdf_gen_conv_tf32_ex): the summed partials equal the unsplit kernel's result up to FP32
    summation order, and torch's FP32 convolution within TF32 accuracy."""
    N = svb._native
    L = N.lib()
    g = torch.Generator().manual_seed(b * h + cout)
    x = torch.randn(b, h, h, cin, generator=g).to(cuda)
    w = (torch.randn(cout, k * k, cin, generator=g) / (cin * k * k) ** 0.5).to(cuda)
    ho = h + 2 * pad - (k - 1)
    nb = int(L.svbrdf_gen_conv_tf32_ws_bytes(b, h, h, cin, cout, k, pad))
    assert nb > 0  # these maps have fewer tiles than half the SMs
    ws = torch.empty(nb, device=cuda, dtype=torch.uint8)
    err = torch.zeros(1, dtype=torch.int32, device=cuda)
    st = N.stream_handle(cuda)
    y_split = torch.empty(b, ho, ho, cout, device=cuda)
    y_one = torch.empty_like(y_split)
    for _ in range(2):  # the workspace is reused
        N.check(L.svbrdf_gen_conv_tf32_ex(x.data_ptr(), w.data_ptr(), y_split.data_ptr(), ws.data_ptr(), nb, b, h, h,
                                          cin, cout, k, pad, err.data_ptr(), st))
    N.check(L.svbrdf_gen_conv_tf32(x.data_ptr(), w.data_ptr(), y_one.data_ptr(), b, h, h, cin, cout, k, pad,
                                   err.data_ptr(), st))
    torch.backends.cudnn.allow_tf32 = False
    try:
        ref = torch.nn.functional.conv2d(x.permute(0, 3, 1, 2), w.reshape(cout, k, k, cin).permute(0, 3, 1, 2),
                                         padding=pad).permute(0, 2, 3, 1)
    finally:
        torch.backends.cudnn.allow_tf32 = True
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    assert rel_l2(y_split, y_one) <= 1e-5
    assert rel_l2(y_split, ref) <= 2e-3


@pytest.mark.gpu
@pytest.mark.parametrize("b,h,c,noise", [(4, 16, 128, True), (2, 8, 512, False), (16, 64, 256, True), (3, 8, 6, True)])
def test_act_scale_matches_composition(svb, cuda, b, h, c, noise):
    """The style layer's epilogue fused with the next layer's input scaling (_ActScaleNHWC)
    against _ActNHWC followed by the scaling, forward and all four gradients (y, d, noise,
    the next style)."""
    MG = svb.materialgan
    g = torch.Generator().manual_seed(b * c + h)
    y = torch.randn(b, c, h, h, generator=g).to(cuda).contiguous(memory_format=torch.channels_last)
    d = (torch.rand(b, c, generator=g) + 0.5).to(cuda)
    nz = torch.randn(b, 1, h, h, generator=g).to(cuda) if noise else None
    ns = torch.tensor(0.3, device=cuda)
    bias = torch.randn(c, generator=g).to(cuda)
    s2 = (torch.randn(b, c, generator=g) * 0.5 + 1.0).to(cuda)
    gout = torch.randn(b, c, h, h, generator=g).to(cuda).contiguous(memory_format=torch.channels_last)

    def run(fused):
        yy, dd, s22 = y.clone().requires_grad_(True), d.clone().requires_grad_(True), s2.clone().requires_grad_(True)
        nn_ = nz.clone().requires_grad_(True) if noise else None
        if fused:
            out = MG._ActScaleNHWC.apply(yy, dd, nn_, ns, bias, MG.LRELU_GAIN, s22)
        else:
            out = MG._ActNHWC.apply(yy, dd, nn_, ns, bias, MG.LRELU_GAIN) * s22[:, :, None, None]
        (out * gout).sum().backward()
        return out.detach(), yy.grad, dd.grad, s22.grad, (nn_.grad if noise else None)

    a, r = run(True), run(False)
    torch.cuda.synchronize()
    for x1, x2 in zip(a, r):
        if x1 is not None:
            assert rel_l2(x1, x2) <= 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("b,h,cp,c,skip", [(3, 16, 32, 9, True), (2, 4, 32, 9, False), (16, 64, 32, 9, True)])
def test_rgb_epilogue_matches_torch(svb, cuda, b, h, cp, c, skip):
    """The toRGB epilogue kernel (padded channels-last conv output + bias + up-sampled skip
    image, written NCHW) and its adjoint against the same composition in torch ops."""
    MG = svb.materialgan
    g = torch.Generator().manual_seed(b * h + cp)
    yp = torch.randn(b, cp, h, h, generator=g).to(cuda).contiguous(memory_format=torch.channels_last)
    bias = torch.randn(c, generator=g).to(cuda)
    prev = torch.randn(b, c, h // 2, h // 2, generator=g).to(cuda) if skip else None
    y1 = yp.clone().requires_grad_(True)
    p1 = prev.clone().requires_grad_(True) if skip else None
    out = MG._RgbNHWC.apply(y1, bias, p1, c)
    assert out.is_contiguous() and out.shape == (b, c, h, h)
    y2 = yp.clone().requires_grad_(True)
    p2 = prev.clone().requires_grad_(True) if skip else None
    ref = y2[:, :c] + bias.view(1, -1, 1, 1)
    if skip:
        ref = ref + MG._up1d(MG._up1d(p2, -1), -2)
    gout = torch.randn(out.shape, generator=g).to(cuda)
    (out * gout).sum().backward()
    (ref * gout).sum().backward()
    torch.cuda.synchronize()
    assert rel_l2(out, ref) <= 1e-6
    assert rel_l2(y1.grad, y2.grad) <= 1e-6
    assert float(y1.grad[:, c:].abs().max()) == 0.0
    if skip:
        assert rel_l2(p1.grad, p2.grad) <= 1e-6


@pytest.mark.gpu
def test_gpu_generator_tf32_matches_reference_network(svb, cuda):
    """The generator as it runs by default on the GPU (channels-last maps, the TF32 tensor-core
    convolutions, the NHWC kernels) on the reference network's fixture
    (tests/golden/generator_ref_256.npz, the reference's FP64 run). The reference's own GPU path
    runs these convolutions in TF32 too (PyTorch's cuDNN default), so the bound is that path's
    error: the same generator with its convolutions on cuDNN in TF32 (convolution weights
    marked trainable, which keeps a layer off the frozen-weight kernels). Output within
    max(1e-2, twice cuDNN's error), W+ and noise gradients within max(3e-2, twice cuDNN's)."""
    MG = svb.materialgan
    gen, d, wp_np, noises_np, R_np, _ = _reference_generator(svb, cuda, torch.float32)
    for p in gen.parameters():
        p.requires_grad_(False)
    assert torch.backends.cudnn.allow_tf32
    ours = _tf32_generator_errors(svb, cuda, gen, d, wp_np, noises_np, R_np)
    convs = [m for m in gen.modules() if isinstance(m, MG._ModConv)]
    assert convs and all(getattr(m, "_tf32_key", None) is not None for m in convs)  # the TF32 kernels ran
    for m in convs:
        m.weight.requires_grad_(True)
    lib = _tf32_generator_errors(svb, cuda, gen, d, wp_np, noises_np, R_np)
    print("TF32 generator vs reference FP64 (output, W+ gradient, noise-gradient norms): tcgen05 kernels "
          + ", ".join(f"{e:.2e}" for e in ours) + "; cuDNN TF32 " + ", ".join(f"{e:.2e}" for e in lib))
    for e, e_lib, floor in zip(ours, lib, (1e-2, 3e-2, 3e-2)):
        assert e <= max(floor, 2 * e_lib)
