"""Batched persistent kernel: each material must follow the trajectory the
single-material fused kernel gives it, on an uneven batch. Both kernels inline the same
per-texel code, but they are separate kernels (ptxas may contract and schedule them
differently), so the comparison allows last-bit differences."""
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _batch(svb, cuda, n=6, general=True):
    from oracle import microfacet_ref as R
    mats = svb.scenes.batched_scenes(n=n, resolutions=(16, 32, 48), vmin=3, vmax=12,
                                     render_fn=lambda *a: R.render(*a, dtype=torch.float32))
    if general:
        mats[1].light_pos = mats[1].light_pos + torch.tensor([1.0, -2.0, 3.0])  # one non-co-located material
    return mats


@pytest.mark.parametrize("variant,threads,tile,general", [
    (0, 128, 128, True), (0, 256, 512, True), (0, 512, 2048, True),
    (1, 256, 256, True), (1, 384, 384, True), (1, 480, 480, True), (1, 608, 608, True),
    (2, 256, 512, True), (2, 384, 768, True), (2, 480, 960, True),
    (2, 480, 960, False), (2, 256, 512, False), (2, 224, 448, True), (2, 224, 448, False),
    (3, 480, 960, True), (3, 480, 960, False), (3, 224, 448, True), (3, 384, 768, False),
    (4, 512, 1024, True), (4, 512, 1024, False), (4, 256, 512, True), (4, 256, 512, False)])
def test_batched_equals_single(svb, cuda, variant, threads, tile, general):
    """`general` puts one material's light off the camera; without it every view is
    co-located and the texel-pair variant launches its instantiation without the general
    path."""
    mats = _batch(svb, cuda, general=general)
    cfg = svb.BatchConfig(threads=threads, tile_texels=tile, ctas=5, variant=variant)
    b = svb.BatchedOptim(mats, lr=0.01, loss="log1p", device=cuda, config=cfg)
    losses = []
    for _ in range(7):
        b.step()
        losses.append(b.loss_out.clone())
    for i, m in enumerate(mats):
        r = svb.Microfacet(m.res, m.n_views, m.size, [t.to(cuda) for t in m.cl], cuda)
        o = svb.SvbrdfOptim(cuda, r, loss="log1p")
        o.load_targets(m.targets.to(cuda))
        o.init_from_tex(m.init.to(cuda))
        o.optim(7, 0.01, None, False)
        assert rel_l2(b.tex[i], o.textures.detach()) <= 1e-6
        assert rel_l2(b.m1[i], o.exp_avg) <= 1e-5
        assert rel_l2(b.m2[i], o.exp_avg_sq) <= 1e-5
        for k in range(7):
            assert abs(float(losses[k][i]) - o.loss_image_list[k]) <= 1e-6 * o.loss_image_list[k]
    assert b.device_error() == 0


@pytest.mark.parametrize("general", [False, True])
def test_pair_many_views_equals_single(svb, cuda, general):
    """40 views: 14 target chunks per tile go through a 6-slot ring."""
    from oracle import microfacet_ref as R
    mats = svb.scenes.batched_scenes(n=2, resolutions=(32,), vmin=40, vmax=40,
                                     render_fn=lambda *a: R.render(*a, dtype=torch.float32))
    if general:
        mats[0].light_pos = mats[0].light_pos + torch.tensor([0.5, 1.0, -2.0])
    b = svb.BatchedOptim(mats, lr=0.01, loss="log1p", device=cuda,
                         config=svb.BatchConfig(threads=480, tile_texels=960, ctas=2, variant=2))
    for _ in range(4):
        b.step()
    assert b.device_error() == 0
    for i, m in enumerate(mats):
        r = svb.Microfacet(m.res, m.n_views, m.size, [t.to(cuda) for t in m.cl], cuda)
        o = svb.SvbrdfOptim(cuda, r, loss="log1p")
        o.load_targets(m.targets.to(cuda))
        o.init_from_tex(m.init.to(cuda))
        o.optim(4, 0.01, None, False)
        assert rel_l2(b.tex[i], o.textures.detach()) <= 1e-6
        assert rel_l2(b.m2[i], o.exp_avg_sq) <= 1e-5


@pytest.mark.parametrize("variant,threads,tile", [(0, 256, 1024), (1, 384, 384), (2, 480, 960)])
def test_batched_graph_matches_eager(svb, cuda, variant, threads, tile):
    mats = _batch(svb, cuda)
    cfg = svb.BatchConfig(threads=threads, tile_texels=tile, ctas=0, variant=variant)
    a = svb.BatchedOptim(mats, device=cuda, config=cfg)
    for _ in range(5):
        a.step()
    b = svb.BatchedOptim(mats, device=cuda, config=cfg)
    b.run(2)
    b.run(3)  # re-captured for 3 iterations, continuing at step 3
    for i in range(len(mats)):
        assert torch.equal(a.tex[i], b.tex[i])
    assert torch.equal(a.loss_out, b.loss_out)
    assert torch.equal(a.loss_hist[:5], b.loss_hist[:5])
    # a replay of the same graph keeps advancing, identically to eager steps
    b.run(3)
    for _ in range(3):
        a.step()
    for i in range(len(mats)):
        assert torch.equal(a.tex[i], b.tex[i])
    # reset restarts from the initial state
    b.reset(inits=[m.init for m in mats], targets=[m.targets for m in mats])
    b.run(3)
    c = svb.BatchedOptim(mats, device=cuda, config=cfg)
    for _ in range(3):
        c.step()
    for i in range(len(mats)):
        assert torch.equal(c.tex[i], b.tex[i])


def test_autotune_picks_a_valid_config(svb, cuda, tmp_path, monkeypatch):
    monkeypatch.setattr(svb.batched, "CACHE_FILE", tmp_path / "tune.json")
    mats = _batch(svb, cuda, n=4)
    b = svb.BatchedOptim(mats, device=cuda)
    assert b.config.tile_texels % b.config.threads == 0
    assert len(b.tune_results if hasattr(b, "tune_results") else [1]) >= 1
    b.step()
    assert torch.isfinite(b.loss_out).all()


@pytest.mark.parametrize("variant", [2, 3, 4])
def test_pipeline_matches_sequential_batches(svb, cuda, variant):
    """BatchedPipeline (two buffers, copies on side streams) gives each batch exactly the
    maps and losses that a sequential reset + run of BatchedOptim gives it."""
    mats = _batch(svb, cuda, n=4, general=False)
    threads = 512 if variant == 4 else 480
    cfg = svb.BatchConfig(threads=threads, tile_texels=2 * threads, ctas=0, variant=variant)
    g = torch.Generator().manual_seed(5)
    batches = []
    for _ in range(3):
        inits = [(m.init + 0.05 * torch.randn(m.init.shape, generator=g)).clamp(-1, 1).pin_memory() for m in mats]
        tgts = [(m.targets * (1.0 + 0.1 * torch.rand(1, generator=g))).pin_memory() for m in mats]
        batches.append((inits, tgts))
    def copy(res):
        return [m.clone() for m in res[0]], res[1].clone()

    pipe = svb.BatchedPipeline(mats, iters=6, lr=0.01, loss="log1p", device=cuda, config=cfg)
    t0 = pipe.submit(*batches[0])
    t1 = pipe.submit(*batches[1])
    got = [copy(pipe.result(t0))]
    t2 = pipe.submit(*batches[2])  # reuses batch 0's buffer
    got += [copy(pipe.result(t1)), copy(pipe.result(t2))]
    assert pipe.device_error() == 0
    ref = svb.BatchedOptim(mats, lr=0.01, loss="log1p", device=cuda, config=cfg, hist_len=6)
    for (inits, tgts), (maps, losses) in zip(batches, got):
        ref.reset(inits=inits, targets=tgts)
        ref.run(6)
        torch.cuda.synchronize()
        for a, b in zip(maps, ref.tex):
            assert torch.equal(a, b.cpu())
        assert torch.equal(losses, ref.loss_hist.cpu())
    with pytest.raises(ValueError):
        pipe.result(t0)  # its buffer has been reused


def _single(svb, cuda, m, iters):
    r = svb.Microfacet(m.res, m.n_views, m.size, [t.to(cuda) for t in m.cl], cuda)
    o = svb.SvbrdfOptim(cuda, r, loss="log1p")
    o.load_targets(m.targets.to(cuda))
    o.init_from_tex(m.init.to(cuda))
    o.optim(iters, 0.01, None, False)
    return o


@pytest.mark.parametrize("variant,threads,general,iters", [
    (3, 480, False, 7), (3, 480, True, 7), (3, 224, False, 9), (3, 256, True, 5), (3, 384, False, 6),
    (3, 480, False, 45), (4, 512, False, 7), (4, 512, True, 7), (4, 256, False, 9), (4, 256, True, 5),
    (4, 512, False, 45), (4, 512, False, 1)])
def test_resident_state_equals_single(svb, cuda, variant, threads, general, iters):
    """Variants 3 and 4 run `iters` iterations per launch (45: two launches of 23 and 22) on
    the shared-memory state; every material's maps, moments and per-iteration losses must
    match the single-material optimiser's."""
    mats = _batch(svb, cuda, general=general)
    cfg = svb.BatchConfig(threads=threads, tile_texels=2 * threads, ctas=5, variant=variant)
    b = svb.BatchedOptim(mats, lr=0.01, loss="log1p", device=cuda, config=cfg, hist_len=iters)
    b.run(iters)
    assert b.device_error() == 0
    for i, m in enumerate(mats):
        o = _single(svb, cuda, m, iters)
        assert rel_l2(b.tex[i], o.textures.detach()) <= 1e-6
        assert rel_l2(b.m1[i], o.exp_avg) <= 1e-5
        assert rel_l2(b.m2[i], o.exp_avg_sq) <= 1e-5
        for k in range(iters):
            assert abs(float(b.loss_hist[k, i]) - o.loss_image_list[k]) <= 1e-6 * o.loss_image_list[k]


@pytest.mark.parametrize("variant,threads", [(3, 480), (4, 512), (4, 256)])
def test_resident_state_matches_pair_variant(svb, cuda, variant, threads):
    """Variants 3 and 4 against variant 2 (one launch per iteration) over 70 iterations:
    three launches of 24, 23 and 23 iterations, then single-iteration steps."""
    mats = _batch(svb, cuda, n=5, general=False)
    a = svb.BatchedOptim(mats, device=cuda, config=svb.BatchConfig(480, 960, 0, 2), hist_len=75)
    b = svb.BatchedOptim(mats, device=cuda, config=svb.BatchConfig(threads, 2 * threads, 0, variant), hist_len=75)
    a.run(70)
    b.run(70)
    for _ in range(5):
        a.step()
        b.step()
    assert b.device_error() == 0 and a.device_error() == 0
    for i in range(len(mats)):
        assert rel_l2(b.tex[i], a.tex[i]) <= 1e-6
        assert rel_l2(b.m2[i], a.m2[i]) <= 1e-5
    assert rel_l2(b.loss_hist, a.loss_hist) <= 1e-6
    assert int(b.step_dev.item()) == 75


@pytest.mark.parametrize("variant,threads", [(3, 480), (4, 512), (4, 256)])
@pytest.mark.parametrize("general", [False, True])
def test_resident_state_many_views(svb, cuda, general, variant, threads):
    """40 views: 14 target chunks per iteration through a 2- or 3-slot ring, 6 iterations
    per launch."""
    from oracle import microfacet_ref as R
    mats = svb.scenes.batched_scenes(n=2, resolutions=(32,), vmin=40, vmax=40,
                                     render_fn=lambda *a: R.render(*a, dtype=torch.float32))
    if general:
        mats[0].light_pos = mats[0].light_pos + torch.tensor([0.5, 1.0, -2.0])
    b = svb.BatchedOptim(mats, lr=0.01, loss="log1p", device=cuda,
                         config=svb.BatchConfig(threads=threads, tile_texels=2 * threads, ctas=2, variant=variant))
    b.run(6)
    assert b.device_error() == 0
    for i, m in enumerate(mats):
        o = _single(svb, cuda, m, 6)
        assert rel_l2(b.tex[i], o.textures.detach()) <= 1e-6
        assert rel_l2(b.m2[i], o.exp_avg_sq) <= 1e-5


@pytest.mark.parametrize("variant,threads,general", [(2, 480, False), (2, 480, True), (3, 480, False),
                                                      (3, 224, True), (2, 224, False), (3, 384, False)])
def test_batched_learnable_light_equals_single(svb, cuda, variant, threads, general):
    """optim_light on a batch: each material's light power and maps follow the trajectory the
    single-material kernel gives them (src/svbrdf.py:48-50, 58-59); the resident-state
    variant runs one iteration per launch then."""
    mats = _batch(svb, cuda, general=general)
    for k, m in enumerate(mats):  # distinct starting powers, off the targets' 1500
        m.light_pow = m.light_pow * (0.8 + 0.1 * k)
    cfg = svb.BatchConfig(threads=threads, tile_texels=2 * threads, ctas=5, variant=variant)
    b = svb.BatchedOptim(mats, lr=0.01, loss="log1p", device=cuda, config=cfg, optim_light=True, hist_len=7)
    assert b.launches(7) == 7
    b.run(7)
    assert b.device_error() == 0
    for i, m in enumerate(mats):
        r = svb.Microfacet(m.res, m.n_views, m.size, [t.to(cuda) for t in m.cl], cuda)
        o = svb.SvbrdfOptim(cuda, r, loss="log1p", kernel="single")
        o.load_targets(m.targets.to(cuda))
        o.init_from_tex(m.init.to(cuda))
        o.optim(7, 0.01, None, True)
        assert rel_l2(b.tex[i], o.textures.detach()) <= 1e-6
        assert rel_l2(b.m2[i], o.exp_avg_sq) <= 1e-5
        assert rel_l2(b.light_pow(i), o.light_pow) <= 1e-6
        for k in range(7):
            assert abs(float(b.loss_hist[k, i]) - o.loss_image_list[k]) <= 1e-6 * o.loss_image_list[k]


@pytest.mark.parametrize("variant", [2, 3])
def test_batched_learnable_light_matches_reference(svb, golden, cuda, variant):
    """The reference's own 20-epoch trajectory with a learnable light (optim_traj_light_16)."""
    d = golden("optim_traj_light_16.npz")
    sc = svb.scenes.Scene(res=d["init"].shape[-1], size=float(d["size"]), camera_pos=d["camera_pos"],
                          light_pos=d["light_pos"], light_pow=d["light_pow0"], gt=None, targets=d["targets"],
                          init=d["init"])
    b = svb.BatchedOptim([sc], lr=float(d["lr"]), loss="mse", device=cuda, optim_light=True,
                         config=svb.BatchConfig(480, 960, 0, variant), hist_len=int(d["epochs"]))
    b.run(int(d["epochs"]))
    assert rel_l2(b.tex[0], d["textures"]) <= 2e-5
    assert rel_l2(b.light_pow(0), d["light_pow"]) <= 1e-6
    ref = d["loss"].tolist()
    assert max(abs(float(b.loss_hist[k, 0]) - ref[k]) / ref[k] for k in range(len(ref))) <= 1e-5
