"""The seeded synthetic workload that stands in for captured datasets: the value ranges,
view layouts and seeding its docstrings state."""
import torch


def test_material_ranges_and_tilt(svb):
    t = svb.scenes.make_material(64, 1000)
    assert t.shape == (1, 9, 64, 64)
    stored = (t + 1) / 2  # parameter -> [0, 1] storage value
    dif, spe, rgh = stored[0, 0:3], stored[0, 6:9], stored[0, 5]
    assert float(dif.min()) >= 0.05 - 1e-6 and float(dif.max()) <= 0.9 + 1e-6
    assert float(spe.min()) >= 0.02 - 1e-6 and float(spe.max()) <= 0.5 + 1e-6
    assert float(rgh.min()) >= 0.1 - 1e-6 and float(rgh.max()) <= 0.9 + 1e-6
    nx, ny = t[0, 3], t[0, 4]
    tilt = torch.rad2deg(torch.asin(torch.sqrt(nx * nx + ny * ny).clamp(max=1.0)))
    assert float(tilt.max()) <= 30.0 + 1e-3 and float(tilt.max()) >= 29.0  # scaled to the stated maximum


def test_material_seeding(svb):
    a = svb.scenes.make_material(32, 1234)
    assert torch.equal(a, svb.scenes.make_material(32, 1234))
    assert not torch.equal(a, svb.scenes.make_material(32, 1235))


def test_grid_and_batched_views(svb):
    cam = svb.scenes.grid_views()
    assert cam.shape == (9, 3) and torch.all(cam[:, 2] == 30.0)
    assert sorted(set(cam[:, 0].tolist())) == [-6.0, 0.0, 6.0]
    scenes = svb.scenes.batched_scenes(n=40, resolutions=(16, 32), vmin=5, vmax=16)
    assert {s.res for s in scenes} == {16, 32}
    vs = [s.n_views for s in scenes]
    assert min(vs) >= 5 and max(vs) <= 16
    for s in scenes:
        c = s.camera_pos
        assert float(c[:, :2].abs().max()) <= 8.0 and float(c[:, 2].min()) >= 25.0 and float(c[:, 2].max()) <= 35.0
        assert torch.equal(s.light_pos, c)  # co-located flash
    again = svb.scenes.batched_scenes(n=40, resolutions=(16, 32), vmin=5, vmax=16)
    assert [(s.res, s.n_views) for s in again] == [(s.res, s.n_views) for s in scenes]


def test_targets_are_noisy_clamped_renders(svb):
    from oracle import microfacet_ref as R
    sc = svb.scenes.single_scene(res=16, seed=1001, render_fn=lambda *a: R.render(*a, dtype=torch.float32))
    clean = R.render(sc.gt, sc.camera_pos, sc.light_pos, sc.light_pow, sc.size, torch.float32)
    assert sc.targets.shape == clean.shape
    assert float(sc.targets.min()) >= 0.0 and float(sc.targets.max()) <= 1.0
    inside = (clean > 0.05) & (clean < 0.95)
    noise = (sc.targets - clean)[inside]
    assert abs(float(noise.std()) - 0.01) < 0.002 and abs(float(noise.mean())) < 0.002
