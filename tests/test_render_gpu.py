"""Forward render and hand-written adjoint on the GPU against the reference fixtures
(made by running the reference itself) and the FP64 oracle.

Tolerances (written here, measured on the reference itself):
* renders: relative L2 <= 1e-5 against the reference's FP32 render and against FP64;
  the reference's own FP32 render is 5e-6 from FP64, up to 2e-4 on single highlight
  pixels (1 - cos^2 cancellation), hence max-abs 1e-3 per element;
* gradients: relative L2 <= max(1e-4, 2 x the reference's own FP32-vs-FP64 error).
"""
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _renderer(svb, d, res, cuda):
    cl = [d["camera_pos"].to(cuda), d["light_pos"].to(cuda), d["light_pow"].to(cuda)]
    return svb.Microfacet(res, d["camera_pos"].shape[0], float(d["size"]), cl, cuda)


@pytest.mark.parametrize("case,key,tex_key", [("render_coloc_20.npz", "render_gt", "textures_gt"),
                                              ("render_general_24.npz", "render", "textures")])
def test_forward_matches_reference(svb, golden, cuda, case, key, tex_key):
    d = golden(case)
    res = d[tex_key].shape[-1]
    r = _renderer(svb, d, res, cuda)
    out = r.eval(d[tex_key].to(cuda)).cpu()
    assert out.shape == d[key + "32"].shape
    # the reference's own FP32 render is 0.7e-5 (co-located) / 1.1e-5 (general) from FP64
    tol = max(1e-5, rel_l2(d[key + "32"], d[key + "64"]))
    assert rel_l2(out, d[key + "32"]) <= tol
    assert rel_l2(out, d[key + "64"]) <= tol
    assert float((out.double() - d[key + "64"]).abs().max()) <= 1e-3


@pytest.mark.parametrize("kind", ["mse", "log1p"])
def test_adjoint_general_matches_reference(svb, golden, cuda, kind):
    d = golden("render_general_24.npz")
    r = _renderer(svb, d, 24, cuda)
    tex = d["textures"].to(cuda).requires_grad_(True)
    lp = d["light_pow"].to(cuda).requires_grad_(True)
    r.update_light(lp)
    out = r.eval(tex)
    tg = d["targets"].to(cuda)
    if kind == "mse":
        loss = torch.nn.functional.mse_loss(out, tg)
    else:
        loss = torch.nn.functional.mse_loss(torch.log1p(out), torch.log1p(tg))
    loss.backward()
    g64, g32 = d[f"grad_{kind}64"], d[f"grad_{kind}32"]
    tol = max(1e-4, 2 * rel_l2(g32, g64))
    assert rel_l2(tex.grad, g64) <= tol
    assert rel_l2(tex.grad, g32) <= tol
    assert rel_l2(lp.grad, d[f"gradpow_{kind}64"]) <= 1e-4
    assert abs(float(loss.detach()) - float(d[f"loss_{kind}64"])) <= 1e-5 * float(d[f"loss_{kind}64"])


def test_adjoint_coloc_matches_reference(svb, golden, cuda):
    d = golden("render_coloc_20.npz")
    r = _renderer(svb, d, 20, cuda)
    tex = d["textures"].to(cuda).requires_grad_(True)
    loss = torch.nn.functional.mse_loss(r.eval(tex), d["targets"].to(cuda))
    loss.backward()
    g64, g32 = d["grad_mse64"], d["grad_mse32"]
    assert rel_l2(tex.grad, g64) <= max(1e-4, 2 * rel_l2(g32, g64))
    for c in range(9):  # per channel group too
        assert rel_l2(tex.grad[0, c], g64[0, c]) <= max(1e-4, 2 * rel_l2(g32[0, c], g64[0, c]))


def test_render_loss_kernel(svb, golden, cuda):
    d = golden("render_general_24.npz")
    r = _renderer(svb, d, 24, cuda)
    for kind in ("mse", "log1p"):
        l = r.render_loss(d["textures"].to(cuda), d["targets"].to(cuda), kind)
        ref = float(d[f"loss_{kind}64"])
        assert abs(float(l) - ref) <= 1e-5 * ref


def test_adjoint_vs_fp64_finite_differences_1024(svb, oracle, cuda):
    """64 random texels of the 1024^2, 9-view scene, FP64 central differences, h=1e-6."""
    sc = svb.scenes.single_scene(res=1024, device=cuda)
    svb.scenes.add_targets(sc, lambda *a: svb.Microfacet(1024, 9, a[4], [a[1], a[2], a[3]], cuda).eval(a[0]))
    state = (0.5 * sc.gt + 0.5 * sc.init).contiguous()
    r = svb.Microfacet(1024, 9, sc.size, sc.cl, cuda)
    tex = state.clone().requires_grad_(True)
    out = r.eval(tex)
    loss = torch.nn.functional.mse_loss(torch.log1p(out), torch.log1p(sc.targets))
    loss.backward()
    g = torch.Generator().manual_seed(5)
    cand = torch.randint(0, 1024, (256, 2), generator=g).tolist()
    od = out.detach()
    ok = [(i, j) for i, j in cand if 2e-3 < float(od[:, :, i, j].min()) and float(od[:, :, i, j].max()) < 0.999][:64]
    assert len(ok) == 64
    fd = oracle.fd_gradient(state.cpu(), sc.targets.cpu(), sc.camera_pos.cpu(), sc.light_pos.cpu(),
                            sc.light_pow.cpu(), sc.size, ok, "log1p", h=1e-6)
    ad = torch.stack([tex.grad[0, :, i, j].cpu() for i, j in ok])
    assert rel_l2(ad, fd) <= 1e-4


def test_eval_rejects_wrong_resolution(svb, golden, cuda):
    d = golden("render_coloc_20.npz")
    r = _renderer(svb, d, 20, cuda)
    with pytest.raises(AssertionError):
        r.eval(torch.zeros(1, 9, 16, 16, device=cuda))


def test_many_views_and_non_square_budget(svb, cuda):
    # V = max views, res not a multiple of the block size
    V = svb._native.load().svbrdf_max_views()
    g = torch.Generator().manual_seed(3)
    cam = torch.cat(((torch.rand(V, 2, generator=g) * 2 - 1) * 8, 25 + 10 * torch.rand(V, 1, generator=g)), 1)
    tex = svb.scenes.make_material(37, 1010)
    r = svb.Microfacet(37, V, 17.0, [cam.to(cuda), cam.to(cuda), torch.full((3,), 1500.0, device=cuda)], cuda)
    out = r.eval(tex.to(cuda)).cpu()
    from oracle import microfacet_ref as R
    ref = R.render(tex, cam, cam, torch.full((3,), 1500.0), 17.0, torch.float64)
    assert rel_l2(out, ref) <= 1e-5


def test_batched_eval_matches_per_material(svb, golden, cuda):
    """A leading batch of materials (the reference's eval on [B, 9, H, W] -> [B * n, 3, H, W])
    renders and differentiates in one launch each (svbrdf_render_fwd_batch / _bwd_batch): the
    same renders and texture gradients as one call per material, and a light-power gradient
    equal to their sum (one fixed-order reduction over the batch, so equal up to summation
    order)."""
    d = golden("render_general_24.npz")
    res = d["textures"].shape[-1]
    r = _renderer(svb, d, res, cuda)
    g = torch.Generator().manual_seed(5)
    tex = (d["textures"].float() + 0.3 * torch.randn(3, 9, res, res, generator=g)).clamp(-1, 1).to(cuda)
    n = r.n_of_imgs
    wts = torch.randn(3 * n, 3, res, res, generator=g).to(cuda)
    lp = r.light_pow.detach().clone().requires_grad_(True)
    r.update_light(lp)
    tb = tex.clone().requires_grad_(True)
    out = r.eval(tb)
    assert out.shape == (3 * n, 3, res, res)
    (out * wts).sum().backward()
    g_batch = lp.grad.clone()
    g_sum = torch.zeros_like(g_batch)
    for b in range(3):
        lp.grad = None
        t1 = tex[b:b + 1].clone().requires_grad_(True)
        o1 = r.eval(t1)
        (o1 * wts[b * n:(b + 1) * n]).sum().backward()
        assert torch.equal(out[b * n:(b + 1) * n].detach(), o1.detach())
        assert torch.equal(tb.grad[b:b + 1], t1.grad)
        g_sum += lp.grad
    assert rel_l2(g_batch, g_sum) <= 1e-6
