"""BF16 tensor-core 3x3 convolution and the descriptor loss.

The convolution is checked against torch's FP32 conv2d on the same BF16 inputs (relative
L2 <= 1e-2: the output is rounded to BF16, 2^-8 relative). The descriptor loss is checked
per term against the FP64 CPU oracle on the same weights: feature and Gram losses within
1e-3 relative (measured ~3e-5). The gradient w.r.t. the renders is held to relative L2
<= 0.3 and cosine >= 0.95: rounding the activations to BF16 moves ReLU kinks and max-pool
winners, and the FP64 oracle with its activations rounded to BF16 the same way is itself
0.18 (relative L2) from the unrounded FP64 gradient."""
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _ref_conv(x_nhwc, w_cout_tap_cin, bias=None):
    cout, _, cin = w_cout_tap_cin.shape
    w = w_cout_tap_cin.float().reshape(cout, 3, 3, cin).permute(0, 3, 1, 2)
    y = torch.nn.functional.conv2d(x_nhwc.float().permute(0, 3, 1, 2), w, bias, padding=1)
    return y.permute(0, 2, 3, 1)


@pytest.mark.parametrize("n,h,w,cin,cout", [(1, 8, 16, 64, 64), (2, 16, 32, 64, 128), (1, 24, 48, 128, 256),
                                            (2, 32, 32, 256, 512), (1, 8, 16, 192, 64)])
def test_conv3x3_tc_matches_torch(svb, cuda, n, h, w, cin, cout):
    D = svb.descriptor
    g = torch.Generator().manual_seed(n * 1000 + cin)
    x = torch.randn(n, h, w, cin, generator=g).to(cuda, torch.bfloat16)
    wt = (torch.randn(cout, 9, cin, generator=g) * (2.0 / (9 * cin)) ** 0.5).to(cuda, torch.bfloat16)
    b = (torch.randn(cout, generator=g) * 0.1).to(cuda)
    err = torch.zeros(1, dtype=torch.int32, device=cuda)
    y0 = D.conv3x3_bf16(x, wt, None, D.EPI_NONE, err)
    y1 = D.conv3x3_bf16(x, wt, b, D.EPI_BIAS_RELU, err)
    mask = torch.randn(n, h, w, cout, generator=g).to(cuda, torch.bfloat16)
    y2 = D.conv3x3_bf16(x, wt, None, D.EPI_MASK, err, mask=mask)
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    ref = _ref_conv(x, wt)
    assert rel_l2(y0.float(), ref) <= 1e-2
    assert rel_l2(y1.float(), torch.relu(ref + b)) <= 1e-2
    assert rel_l2(y2.float(), ref * (mask.float() > 0)) <= 1e-2


def test_conv3x3_tc_data_gradient(svb, cuda):
    D = svb.descriptor
    g = torch.Generator().manual_seed(7)
    n, h, w, cin, cout = 2, 16, 32, 64, 128
    wt = torch.randn(cout, cin, 3, 3, generator=g) * 0.05
    wb = wt.to(torch.bfloat16)
    w_dg = wb.flip(2, 3).permute(1, 2, 3, 0).reshape(cin, 9, cout).contiguous().to(cuda)
    gy = torch.randn(n, h, w, cout, generator=g).to(cuda, torch.bfloat16)
    err = torch.zeros(1, dtype=torch.int32, device=cuda)
    gx = D.conv3x3_bf16(gy, w_dg, None, D.EPI_NONE, err)
    ref = torch.nn.grad.conv2d_input((n, cin, h, w), wb.float().to(cuda), gy.float().permute(0, 3, 1, 2), padding=1)
    assert rel_l2(gx.float(), ref.permute(0, 2, 3, 1)) <= 1e-2


def test_conv3x3_rejects_bad_shapes(svb, cuda):
    D = svb.descriptor
    err = torch.zeros(1, dtype=torch.int32, device=cuda)
    x = torch.zeros(1, 8, 20, 64, device=cuda, dtype=torch.bfloat16)  # W not a multiple of 16
    wt = torch.zeros(64, 9, 64, device=cuda, dtype=torch.bfloat16)
    with pytest.raises(svb.SvbrdfError):
        D.conv3x3_bf16(x, wt, None, D.EPI_NONE, err)
    x = torch.zeros(1, 8, 16, 32, device=cuda, dtype=torch.bfloat16)  # Cin not a multiple of 64
    with pytest.raises(svb.SvbrdfError):
        D.conv3x3_bf16(x, torch.zeros(64, 9, 32, device=cuda, dtype=torch.bfloat16), None, D.EPI_NONE, err)


def test_descriptor_loss_vs_fp64_oracle(svb, cuda):
    from oracle import descriptor_ref as DR
    from oracle import microfacet_ref as R

    # 256^2 renders: 128^2 after the 2x2 downsample, 16^2 at conv4_1 (the 8x16 tile minimum)
    sc = svb.scenes.single_scene(res=256, seed=1008)
    tgt = R.render(sc.gt, sc.camera_pos[:2], sc.light_pos[:2], sc.light_pow, sc.size, torch.float32)
    cur = R.render((0.5 * sc.gt + 0.5 * sc.init), sc.camera_pos[:2], sc.light_pos[:2], sc.light_pow, sc.size,
                   torch.float32)
    d = svb.descriptor.VGGDescriptor(cuda, seed=3)
    d.load(tgt.to(cuda))
    r = cur.to(cuda).requires_grad_(True)
    fl, gl = d.loss(r)
    (fl + gl).backward()
    torch.cuda.synchronize()
    assert d.device_error() == 0
    rfl, rgl, rgrad = DR.loss_terms(cur, tgt, d.bf16_weights())
    e_f = abs(float(fl.detach()) - rfl) / rfl
    e_g = abs(float(gl.detach()) - rgl) / rgl
    e_d = rel_l2(r.grad, rgrad)
    a, b = r.grad.double().cpu().flatten(), rgrad.double().flatten()
    cos = float(a @ b / (a.norm() * b.norm()))
    print(f"descriptor vs FP64: feature {e_f:.2e}, gram {e_g:.2e}, d/drender rel-L2 {e_d:.2e}, cosine {cos:.4f}")
    assert e_f <= 1e-3 and e_g <= 1e-3
    assert e_d <= 0.3 and cos >= 0.95


def test_perpixel_with_descriptor_loss(svb, cuda):
    """The descriptor-augmented per-pixel loop (BF16 tensor-core features) lowers the loss."""
    from oracle import microfacet_ref as R

    sc = svb.scenes.single_scene(res=256, seed=1009)
    svb.scenes.add_targets(sc, lambda *a: R.render(*a, dtype=torch.float32))
    r = svb.Microfacet(256, 9, sc.size, [t.to(cuda) for t in sc.cl], cuda)
    d = svb.descriptor.VGGDescriptor(cuda, seed=0)
    o = svb.SvbrdfOptim(cuda, r, loss="log1p", descriptor=d, descriptor_weight=0.1)
    o.load_targets(sc.targets.to(cuda))
    o.init_from_tex(sc.init.to(cuda))
    o.optim(8, 0.02, None, False)
    assert d.device_error() == 0
    assert o.loss_image_list[-1] < o.loss_image_list[0]


def test_graph_replay_matches_eager(svb, cuda):
    from oracle import microfacet_ref as R

    sc = svb.scenes.single_scene(res=256, seed=1010)
    tgt = R.render(sc.gt, sc.camera_pos[:3], sc.light_pos[:3], sc.light_pow, sc.size, torch.float32).to(cuda)
    cur = R.render(sc.init, sc.camera_pos[:3], sc.light_pos[:3], sc.light_pow, sc.size, torch.float32).to(cuda)
    d = svb.descriptor.VGGDescriptor(cuda, seed=1)
    d.load(tgt)
    r = cur.clone().requires_grad_(True)
    fl, gl = d.loss(r)
    (fl + gl).backward()
    for _ in range(2):  # capture, then a second replay
        gfl, ggl, gg = d.loss_and_grad(cur)
    torch.cuda.synchronize()
    assert abs(float(gfl) - float(fl.detach())) <= 1e-6 * float(fl.detach())
    assert abs(float(ggl) - float(gl.detach())) <= 1e-6 * float(gl.detach())
    assert rel_l2(gg, r.grad) <= 1e-6


def test_descriptor_reference_mode_vs_fp64_oracle(svb, cuda):
    """mode="reference": the reference's own VGGLoss semantics (average pools, hooks relu1_1,
    relu1_2, relu3_2, relu4_2, full resolution, feature term only) against the FP64 oracle's
    restatement of it, with the same weights."""
    from oracle import descriptor_ref as DR
    from oracle import microfacet_ref as R

    sc = svb.scenes.single_scene(res=128, seed=1013)
    tgt = R.render(sc.gt, sc.camera_pos[:2], sc.light_pos[:2], sc.light_pow, sc.size, torch.float32)
    cur = R.render((0.5 * sc.gt + 0.5 * sc.init), sc.camera_pos[:2], sc.light_pos[:2], sc.light_pow, sc.size,
                   torch.float32)
    d = svb.descriptor.VGGDescriptor(cuda, seed=4, mode="reference")
    assert not d.downsample and d.avg_pool and not d.gram
    d.load(tgt.to(cuda))
    r = cur.to(cuda).requires_grad_(True)
    fl, gl = d.loss(r)
    (fl + gl).backward()
    torch.cuda.synchronize()
    assert d.device_error() == 0 and float(gl.detach()) == 0.0
    rfl, rgl, rgrad = DR.loss_terms(cur, tgt, d.bf16_weights(), mode="reference")
    assert rgl == 0.0
    e_f = abs(float(fl.detach()) - rfl) / rfl
    e_d = rel_l2(r.grad, rgrad)
    a, b = r.grad.double().cpu().flatten(), rgrad.double().flatten()
    cos = float(a @ b / (a.norm() * b.norm()))
    print(f"reference-mode descriptor vs FP64: feature {e_f:.2e}, d/drender rel-L2 {e_d:.2e}, cosine {cos:.4f}")
    assert e_f <= 1e-3
    assert e_d <= 0.3 and cos >= 0.95
    # the graph-replayed forward + backward gives the same loss and gradient
    gfl, ggl, gdr = d.loss_and_grad(cur.to(cuda))
    assert abs(float(gfl) - float(fl.detach())) <= 1e-6 * float(fl.detach())
    assert rel_l2(gdr, r.grad) <= 1e-6


def test_avgpool_kernels_match_torch(svb, cuda):
    """svbrdf_desc_avgpool_fwd/_bwd against torch's average pool on the same BF16 values, the
    backward with its hook gradient and ReLU mask."""
    N = svb._native
    L = N.lib()
    g = torch.Generator().manual_seed(21)
    x = torch.relu(torch.randn(2, 8, 12, 16, generator=g)).to(cuda, torch.bfloat16)  # NHWC
    y = torch.empty(2, 4, 6, 16, device=cuda, dtype=torch.bfloat16)
    st = N.stream_handle(cuda)
    N.check(L.svbrdf_desc_avgpool_fwd(x.data_ptr(), y.data_ptr(), 2, 8, 12, 16, st))
    ref = torch.nn.functional.avg_pool2d(x.float().permute(0, 3, 1, 2), 2).permute(0, 2, 3, 1)
    assert (y.float() - ref).abs().max() <= 1e-2 * ref.abs().max()
    gy = torch.randn(2, 4, 6, 16, generator=g).to(cuda, torch.bfloat16)
    add = torch.randn(2, 8, 12, 16, generator=g).to(cuda, torch.bfloat16)
    gx = torch.empty_like(x)
    N.check(L.svbrdf_desc_avgpool_bwd(gy.data_ptr(), x.data_ptr(), add.data_ptr(), gx.data_ptr(), 2, 8, 12, 16, st))
    up = gy.float().repeat_interleave(2, dim=1).repeat_interleave(2, dim=2) * 0.25
    want = (up + add.float()) * (x.float() > 0)
    assert (gx.float() - want).abs().max() <= 2e-2 * want.abs().max()
