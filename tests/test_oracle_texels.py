"""The oracle's gathered-texel forms against its whole-image forms (CPU).

The bench-shaped parity tests check the GPU kernels on a sample of texels per material,
because the oracle cannot afford whole 1024^2 materials for 100 iterations. These tests
show that the sample forms are the whole-image oracle restricted to those texels: the
strip render equals the grid render to the last bit or two in FP32 (torch's CPU kernels
vectorise a 1 x n strip differently from an H x W grid) and to 1e-14 in FP64, and the
per-texel trajectories equal the whole-material loop's at the same texels."""
import torch

from conftest import rel_l2


def _scene(svb, R, res=12, seed=1004, views=5):
    sc = svb.scenes.batched_scenes(n=1, resolutions=(res,), vmin=views, vmax=views)[0]
    svb.scenes.add_targets(sc, lambda *a: R.render(*a, dtype=torch.float32))
    sc.init = (0.5 * sc.gt + 0.5 * sc.init).contiguous()
    return sc


def test_texel_positions_match_grid(oracle):
    pos = oracle.pixel_positions(16, 17.0, torch.float32)
    idx = torch.arange(256)
    px, py = oracle.texel_positions(idx, 16, 16, 17.0)
    assert torch.equal(px, pos[0].reshape(-1))
    assert torch.equal(py, pos[1].reshape(-1))


def test_render_texels_equals_render(svb, oracle):
    sc = _scene(svb, oracle)
    idx = torch.tensor([0, 5, 17, 63, 100, 143])
    px, py = oracle.texel_positions(idx, sc.res, sc.res, sc.size)
    t9 = sc.init.reshape(9, -1)[:, idx]
    for dtype, tol in ((torch.float32, 2.5e-7), (torch.float64, 1e-14)):
        full = oracle.render(sc.init, sc.camera_pos, sc.light_pos, sc.light_pow, sc.size, dtype)
        strip = oracle.render_texels(t9, px, py, sc.camera_pos, sc.light_pos, sc.light_pow, dtype)
        ref = full.reshape(full.shape[0], 3, -1)[:, :, idx]
        assert float(((strip - ref).abs() / ref.abs()).max()) <= tol


def test_optim_texels_equals_optim_loop(svb, oracle):
    sc = _scene(svb, oracle)
    for kind in ("mse", "log1p"):
        ref = oracle.optim_loop(sc.init, sc.targets, sc.camera_pos, sc.light_pos, sc.light_pow, sc.size, 6, 0.01,
                                kind, False, torch.float64)
        T = sc.res * sc.res
        idx = torch.tensor([3, 40, 77, 141])
        px, py = oracle.texel_positions(idx, sc.res, sc.res, sc.size)
        tg = sc.targets.reshape(sc.n_views, 3, -1)[:, :, idx]
        out = oracle.optim_texels(sc.init.reshape(9, -1)[:, idx], px, py, tg, sc.camera_pos, sc.light_pos,
                                  sc.light_pow, sc.n_views * 3 * T, 6, 0.01, kind)
        for k in ("textures", "exp_avg", "exp_avg_sq"):
            assert rel_l2(out[k], ref[k].reshape(9, -1)[:, idx]) <= 1e-12, k
        # the whole-material loss of epoch 0 from every texel's squared error
        allidx = torch.arange(T)
        ax, ay = oracle.texel_positions(allidx, sc.res, sc.res, sc.size)
        full = oracle.optim_texels(sc.init.reshape(9, -1), ax, ay, sc.targets.reshape(sc.n_views, 3, -1),
                                   sc.camera_pos, sc.light_pos, sc.light_pow, sc.n_views * 3 * T, 6, 0.01, kind)
        losses = full["sq_err"].sum(1) / (sc.n_views * 3 * T)
        for e in range(6):
            assert abs(float(losses[e]) - ref["loss"][e]) <= 1e-12 * ref["loss"][e]
        e1 = oracle.loss_texels(sc.init.reshape(9, -1), ax, ay, sc.targets.reshape(sc.n_views, 3, -1), sc.camera_pos,
                                sc.light_pos, sc.light_pow, kind) / (sc.n_views * 3 * T)
        assert abs(e1 - ref["loss"][0]) <= 1e-12 * ref["loss"][0]


def test_optim_texels_many_materials_in_one_call(svb, oracle):
    """Texels of materials with different view counts in one call (views padded and masked,
    per-texel loss normaliser) follow the trajectories of one call per material."""
    mats = svb.scenes.batched_scenes(n=3, resolutions=(24, 32), vmin=3, vmax=7)
    for m in mats:
        svb.scenes.add_targets(m, lambda *a: oracle.render(*a, dtype=torch.float32))
    vmax = max(m.n_views for m in mats)
    parts, sep = [], []
    for m in mats:
        T = m.res * m.res
        idx = torch.tensor([0, T // 3, T - 1])
        px, py = oracle.texel_positions(idx, m.res, m.res, m.size)
        tg = m.targets.reshape(m.n_views, 3, -1)[:, :, idx]
        t9 = (0.3 * m.gt + 0.7 * m.init).reshape(9, -1)[:, idx]
        n_full = m.n_views * 3 * T
        sep.append(oracle.optim_texels(t9, px, py, tg, m.camera_pos, m.light_pos, m.light_pow, n_full, 5, 0.01,
                                       "log1p"))
        pad = vmax - m.n_views
        cam = torch.cat((m.camera_pos, m.camera_pos[:1].expand(pad, 3)), 0).unsqueeze(2).expand(-1, -1, 3)
        lit = torch.cat((m.light_pos, m.light_pos[:1].expand(pad, 3)), 0).unsqueeze(2).expand(-1, -1, 3)
        tgp = torch.cat((tg, torch.zeros(pad, 3, 3)), 0)
        mask = torch.cat((torch.ones(m.n_views, 3), torch.zeros(pad, 3)), 0)
        parts.append((t9, px, py, tgp, cam, lit, m.light_pow.view(3, 1).expand(3, 3), torch.full((3,), n_full), mask))
    cat = [torch.cat([p[k] for p in parts], -1) for k in range(9)]
    out = oracle.optim_texels(cat[0], cat[1], cat[2], cat[3], cat[4], cat[5], cat[6], cat[7].double(), 5, 0.01,
                              "log1p", view_mask=cat[8])
    for i, s in enumerate(sep):
        for k in ("textures", "exp_avg", "exp_avg_sq"):
            assert rel_l2(out[k][:, 3 * i:3 * i + 3], s[k]) <= 1e-12, k
        assert rel_l2(out["sq_err"][:, 3 * i:3 * i + 3], s["sq_err"]) <= 1e-12
