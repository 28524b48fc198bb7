"""The C-ABI library builds for sm_103a, loads without a GPU, exports every symbol the
header declares, and validates arguments on the host before touching the device."""
import ctypes
import re

import numpy as np
import pytest

from conftest import REPO


@pytest.fixture(scope="module")
def lib(svb):
    return svb._native.load()


def test_exports_match_header(svb, lib):
    hdr = (REPO / "include" / "svbrdf_gb300.h").read_text()
    declared = set(re.findall(r"\b(svbrdf_[a-z_0-9]+)\s*\(", hdr))
    assert declared == set(svb._native.EXPORTS)
    for name in declared:
        assert hasattr(lib, name), name


def test_constants(lib):
    assert lib.svbrdf_abi_version() == 4
    assert lib.svbrdf_max_views() >= 16
    assert lib.svbrdf_workspace_bytes() >= 16


def test_invalid_arguments_rejected_on_host(svb, lib):
    SV = svb._native
    # null textures
    rc = lib.svbrdf_render_fwd(None, None, None, None, 9, 8, 8, 17.0, None, None, -1, None, None, 0, None)
    assert rc == -1 and b"null" in lib.svbrdf_last_error()
    fake = ctypes.c_void_p(16)
    # too many views
    rc = lib.svbrdf_render_fwd(fake, fake, fake, fake, 10_000, 8, 8, 17.0, fake, None, -1, None, None, 0, None)
    assert rc == -2
    # bad loss kind
    rc = lib.svbrdf_render_fwd(fake, fake, fake, fake, 9, 8, 8, 17.0, fake, None, 7, None, None, 0, None)
    assert rc == -1
    # loss without workspace
    rc = lib.svbrdf_render_fwd(fake, fake, fake, fake, 9, 8, 8, 17.0, fake, fake, 0, fake, None, 0, None)
    assert rc == -4
    # fused step: step 0 and missing workspace
    args = [fake] * 8 + [9, 8, 8, 17.0, 0, 0, 0.01, 0.9, 0.999, 1e-8, fake, fake, 1 << 20, None]
    assert lib.svbrdf_fused_step(*args) == -1
    args[13] = 1
    args[20] = 0
    assert lib.svbrdf_fused_step(*args) == -4
    with pytest.raises(SV.SvbrdfError):
        SV.check(-4)


def _materials(SV, shapes):
    arrs = (SV.svbrdf_material * len(shapes))()
    keep = []
    for i, (h, w, v) in enumerate(shapes):
        cam = np.random.default_rng(i).uniform(-8, 8, (v, 3)).astype(np.float32)
        cam[:, 2] = 30
        keep.append(cam)
        arrs[i] = SV.svbrdf_material(16, 16, 16, 16, 16, cam.ctypes.data, cam.ctypes.data, v, h, w, 17.0)
    return arrs, keep


def test_batched_plan_host_logic(svb, lib):
    SV = svb._native
    shapes = [(256, 256, 9), (64, 64, 5), (128, 128, 16), (256, 256, 7), (32, 32, 12)]
    mats, keep = _materials(SV, shapes)
    cfg = SV.svbrdf_batch_config(256, 1024, 7, 0)
    nbytes = lib.svbrdf_batched_plan_bytes(mats, len(shapes), ctypes.byref(cfg))
    assert nbytes > 0
    buf = np.zeros(nbytes, np.uint8)
    assert lib.svbrdf_batched_plan(mats, len(shapes), ctypes.byref(cfg), buf.ctypes.data, nbytes) == 0
    hdr = np.frombuffer(buf[:48].tobytes(), np.int32)
    magic, n_mat, n_tiles, n_ctas, threads, tile = hdr[:6]
    off_mats, off_views, off_cta, off_order, off_tiles, off_mat_tiles = hdr[6:12]
    assert n_mat == 5 and n_ctas == 7 and threads == 256 and tile == 1024
    exp_tiles = sum(-(-h * w // 1024) for h, w, _ in shapes)
    assert n_tiles == exp_tiles
    cta = np.frombuffer(buf[off_cta:off_cta + 4 * (n_ctas + 1)].tobytes(), np.int32)
    order = np.frombuffer(buf[off_order:off_order + 4 * n_tiles].tobytes(), np.int32)
    tiles = np.frombuffer(buf[off_tiles:off_tiles + 8 * n_tiles].tobytes(), np.int32).reshape(-1, 2)
    mt = np.frombuffer(buf[off_mat_tiles:off_mat_tiles + 4 * (n_mat + 1)].tobytes(), np.int32)
    # every tile scheduled exactly once
    assert cta[0] == 0 and cta[-1] == n_tiles
    assert sorted(order.tolist()) == list(range(n_tiles))
    # tiles cover each material's texels exactly, contiguous per material
    for m, (h, w, v) in enumerate(shapes):
        t = tiles[mt[m]:mt[m + 1]]
        assert (t[:, 0] == m).all()
        assert t[:, 1].tolist() == list(range(0, h * w, 1024))
    # contiguous split: each CTA takes a run of tiles in material order and carries at most
    # the mean plus one tile
    assert order.tolist() == list(range(n_tiles))
    cost = np.array([min(1024, shapes[m][0] * shapes[m][1] - x) * (shapes[m][2] + 5) for m, x in tiles], float)
    loads = [cost[order[cta[c]:cta[c + 1]]].sum() for c in range(n_ctas)]
    assert max(loads) <= cost.sum() / n_ctas + cost.max() + 1e-6
    assert min(loads) >= cost.sum() / n_ctas - cost.max() - 1e-6
    ws = lib.svbrdf_batched_workspace_bytes(buf.ctypes.data)
    assert ws >= 4 * n_tiles


def test_batched_plan_rejects_bad_config(svb, lib):
    SV = svb._native
    mats, keep = _materials(SV, [(64, 64, 9)])
    for cfg in (SV.svbrdf_batch_config(100, 1000, 4, 0), SV.svbrdf_batch_config(256, 1000, 4, 0)):
        assert lib.svbrdf_batched_plan_bytes(mats, 1, ctypes.byref(cfg)) == 0
    mats[0].n_views = 1000
    assert lib.svbrdf_batched_plan_bytes(mats, 1, ctypes.byref(SV.svbrdf_batch_config(256, 1024, 4, 0))) == 0


def test_pipelined_plan_requirements(svb, lib):
    SV = svb._native
    ok_cfg = SV.svbrdf_batch_config(384, 384, 4, 1)
    mats, keep = _materials(SV, [(64, 64, 9), (32, 32, 5)])
    assert lib.svbrdf_batched_plan_bytes(mats, 2, ctypes.byref(ok_cfg)) > 0
    # tile must equal the consumer thread count
    assert lib.svbrdf_batched_plan_bytes(mats, 2, ctypes.byref(SV.svbrdf_batch_config(384, 768, 4, 1))) == 0
    # unsupported width
    assert lib.svbrdf_batched_plan_bytes(mats, 2, ctypes.byref(SV.svbrdf_batch_config(512, 512, 4, 1))) == 0
    # H*W not a multiple of 4
    odd, keep2 = _materials(SV, [(37, 37, 9)])
    assert lib.svbrdf_batched_plan_bytes(odd, 1, ctypes.byref(ok_cfg)) == 0
    assert b"multiple of 4" in lib.svbrdf_last_error()
    # misaligned pointer
    mats[0].textures = 20
    assert lib.svbrdf_batched_plan_bytes(mats, 2, ctypes.byref(ok_cfg)) == 0
    assert b"aligned" in lib.svbrdf_last_error()
    # bad variant
    assert lib.svbrdf_batched_plan_bytes(keep2 and odd, 1, ctypes.byref(SV.svbrdf_batch_config(256, 256, 4, 7))) == 0


def test_pipelined_plan_rejects_views_beyond_ring(svb, lib):
    """Variant 1 holds a tile's parameter slot through the tile: 3 + ceil(V/4) chunks must
    fit in the ring. The texel-pair variant streams the parameters twice and takes any V."""
    SV = svb._native
    mats, keep = _materials(SV, [(32, 32, 40)])
    assert lib.svbrdf_batched_plan_bytes(mats, 1, ctypes.byref(SV.svbrdf_batch_config(480, 480, 2, 1))) == 0
    assert b"ring slots" in lib.svbrdf_last_error()
    assert lib.svbrdf_batched_plan_bytes(mats, 1, ctypes.byref(SV.svbrdf_batch_config(480, 960, 2, 2))) > 0
    few, keep2 = _materials(SV, [(32, 32, 16)])
    assert lib.svbrdf_batched_plan_bytes(few, 1, ctypes.byref(SV.svbrdf_batch_config(608, 608, 2, 1))) > 0


def test_pair_plan_requirements_and_ring(svb, lib):
    SV = svb._native
    mats, keep = _materials(SV, [(64, 64, 9), (32, 32, 5)])
    cfg = SV.svbrdf_batch_config(480, 960, 3, 2)
    n = lib.svbrdf_batched_plan_bytes(mats, 2, ctypes.byref(cfg))
    assert n > 0
    # tile must be twice the consumer thread count; 512 threads is not offered
    assert lib.svbrdf_batched_plan_bytes(mats, 2, ctypes.byref(SV.svbrdf_batch_config(480, 480, 3, 2))) == 0
    assert b"twice" in lib.svbrdf_last_error()
    assert lib.svbrdf_batched_plan_bytes(mats, 2, ctypes.byref(SV.svbrdf_batch_config(512, 1024, 3, 2))) == 0
    buf = np.zeros(n, np.uint8)
    assert lib.svbrdf_batched_plan(mats, 2, ctypes.byref(cfg), buf.ctypes.data, n) == 0
    hdr = np.frombuffer(buf[:72].tobytes(), np.int32)
    n_tiles, variant, ring, general = hdr[2], hdr[13], hdr[14], hdr[15]
    assert variant == 2 and general == 0  # _materials gives co-located views
    assert n_tiles == -(-64 * 64 // 960) + -(-32 * 32 // 960)
    # slots of 9 planes x 960 floats plus a 288-byte record, within the 216 KB ring budget
    budget, slot = 216 * 1024, 9 * 960 * 4 + 288
    assert 2 <= ring <= 64 and ring * slot <= budget < (ring + 1) * slot
    # header, per-(tile, warp) loss partials (per iteration for the resident-state variant),
    # then per-tile totals of up to 32 iterations and 3 light-power sums (two-level reduction)
    assert lib.svbrdf_batched_workspace_bytes(buf.ctypes.data) == 256 + 4 * n_tiles * (480 // 32) + 4 * n_tiles * (32 + 3)
    # seq: (tile, material, first texel) for each entry of the CTA-ordered tile list
    off_order, off_tiles, off_seq = hdr[9], hdr[10], hdr[16]
    order = np.frombuffer(buf[off_order:off_order + 4 * n_tiles].tobytes(), np.int32)
    tiles = np.frombuffer(buf[off_tiles:off_tiles + 8 * n_tiles].tobytes(), np.int32).reshape(-1, 2)
    seq = np.frombuffer(buf[off_seq:off_seq + 16 * n_tiles].tobytes(), np.int32).reshape(-1, 4)
    assert np.array_equal(seq[:, 0], order) and np.array_equal(seq[:, 1:3], tiles[order]) and not seq[:, 3].any()
    # the 7-warp shape runs two CTAs per SM: half the shared memory for its ring
    cfg7 = SV.svbrdf_batch_config(224, 448, 3, 2)
    n7 = lib.svbrdf_batched_plan_bytes(mats, 2, ctypes.byref(cfg7))
    buf7 = np.zeros(n7, np.uint8)
    assert lib.svbrdf_batched_plan(mats, 2, ctypes.byref(cfg7), buf7.ctypes.data, n7) == 0
    ring7 = np.frombuffer(buf7[:64].tobytes(), np.int32)[14]
    budget7, slot7 = 104 * 1024, 9 * 448 * 4 + 288
    assert ring7 * slot7 <= budget7 < (ring7 + 1) * slot7


@pytest.mark.parametrize("variant,threads,budget,ring", [(3, 480, 220, 3), (3, 384, 220, 5), (3, 256, 220, 9),
                                                          (3, 224, 100, 3), (4, 512, 220, 3), (4, 256, 100, 2)])
def test_resident_state_plan_ring_and_workspace(svb, lib, variant, threads, budget, ring):
    """Variants 3 and 4: the 27-plane state area comes out of the shared-memory budget before
    the ring of 9-plane target slots; the workspace holds partials for 32 iterations."""
    SV = svb._native
    mats, keep = _materials(SV, [(64, 64, 9), (32, 32, 5)])
    tt = 2 * threads
    cfg = SV.svbrdf_batch_config(threads, tt, 3, variant)
    n = lib.svbrdf_batched_plan_bytes(mats, 2, ctypes.byref(cfg))
    assert n > 0
    buf = np.zeros(n, np.uint8)
    assert lib.svbrdf_batched_plan(mats, 2, ctypes.byref(cfg), buf.ctypes.data, n) == 0
    hdr = np.frombuffer(buf[:72].tobytes(), np.int32)
    n_tiles, got = hdr[2], hdr[14]
    assert hdr[13] == variant and got == ring
    state, slot = 27 * tt * 4, 9 * tt * 4 + 288
    assert state + ring * slot <= budget * 1024 < state + (ring + 1) * slot
    assert lib.svbrdf_batched_workspace_bytes(buf.ctypes.data) == 256 + 4 * n_tiles * (threads // 32) * 32 + 4 * n_tiles * (32 + 3)
    # 608 threads is not offered by the resident-state variant; tiles must be twice threads
    assert lib.svbrdf_batched_plan_bytes(mats, 2, ctypes.byref(SV.svbrdf_batch_config(608, 1216, 3, 3))) == 0
    assert lib.svbrdf_batched_plan_bytes(mats, 2, ctypes.byref(SV.svbrdf_batch_config(480, 480, 3, 3))) == 0


def test_pipelined_plan_ring_and_workspace(svb, lib):
    SV = svb._native
    mats, keep = _materials(SV, [(64, 64, 9), (32, 32, 5)])
    cfg = SV.svbrdf_batch_config(480, 480, 3, 1)
    n = lib.svbrdf_batched_plan_bytes(mats, 2, ctypes.byref(cfg))
    buf = np.zeros(n, np.uint8)
    assert lib.svbrdf_batched_plan(mats, 2, ctypes.byref(cfg), buf.ctypes.data, n) == 0
    hdr = np.frombuffer(buf[:64].tobytes(), np.int32)
    n_tiles, variant, ring = hdr[2], hdr[13], hdr[14]
    assert variant == 1
    assert 2 <= ring <= 64 and ring * 12 * 480 * 4 <= 200 * 1024
    # one partial loss per (tile, consumer warp) after the 256-byte header
    assert lib.svbrdf_batched_workspace_bytes(buf.ctypes.data) == 256 + 4 * n_tiles * (480 // 32) + 4 * n_tiles * (32 + 3)
    # coordinate tables: the reference's pixel-centre grid (src/microfacet.py:16-19)
    off_coords = hdr[12]
    xs = np.frombuffer(buf[off_coords:off_coords + 4 * 64].tobytes(), np.float32)
    ref = ((np.arange(64, dtype=np.float32) + np.float32(0.5)) / np.float32(64) - np.float32(0.5)) * np.float32(17.0)
    assert np.array_equal(xs, ref)


def test_new_entry_points_reject_bad_arguments_on_host(svb, lib):
    """The multi-iteration batched call, the generator, descriptor and environment-map
    kernels check their arguments on the host, before any device work."""
    SV = svb._native
    fake = ctypes.c_void_p(16)
    # svbrdf_batched_steps: negative iteration count, too small a workspace
    mats, keep = _materials(SV, [(64, 64, 9)])
    cfg = SV.svbrdf_batch_config(480, 960, 3, 3)
    n = lib.svbrdf_batched_plan_bytes(mats, 1, ctypes.byref(cfg))
    buf = np.zeros(n, np.uint8)
    assert lib.svbrdf_batched_plan(mats, 1, ctypes.byref(cfg), buf.ctypes.data, n) == 0
    need = lib.svbrdf_batched_workspace_bytes(buf.ctypes.data)
    step = [fake, buf.ctypes.data, 1, fake, 0.01, 0.9, 0.999, 1e-8, fake, 4]
    assert lib.svbrdf_batched_steps(*step, -1, fake, need, None) == -1
    assert lib.svbrdf_batched_steps(*step, 5, fake, need - 4, None) == -4
    assert lib.svbrdf_batched_steps(fake, buf.ctypes.data, 9, fake, 0.01, 0.9, 0.999, 1e-8, fake, 4, 5, fake, need,
                                    None) == -1  # bad loss kind
    assert lib.svbrdf_batched_steps(fake, buf.ctypes.data, 1, fake, 0.01, 0.9, 0.999, 1e-8, fake, 0, 5, fake, need,
                                    None) == -1  # no loss history rows
    # generator kernels
    assert lib.svbrdf_gen_upsample2(None, fake, 4, 8, 8, None) == -1
    assert lib.svbrdf_gen_upsample2_scaled(fake, fake, fake, 4, 8, 6, None) == -2  # scaling needs w % 4 == 0
    assert lib.svbrdf_gen_scale(fake, fake, fake, 70000, 64, None) == -1            # planes beyond a grid axis
    assert lib.svbrdf_gen_act_bwd(fake, fake, None, None, fake, fake, 1.0, fake, None, fake, 2, 4, 64, None) == -1
    assert lib.svbrdf_gen_scale_nhwc_bwd(fake, fake, fake, fake, fake, fake, 2, 64, 2048, None) == -2
    assert lib.svbrdf_gen_act_nhwc(fake, None, fake, None, fake, 1.0, fake, 2, 64, 8, None) == -1  # noise, no strength
    assert lib.svbrdf_gen_upsample2_nhwc(fake, None, fake, 40000, 2, 8, 8, 0, None) == -2        # B 2h beyond a grid axis
    assert lib.svbrdf_gen_upsample2_nhwc(fake, None, fake, 2, 2, 8, 8, 2, None) == -1            # halo 0 or 1
    assert lib.svbrdf_gen_upsample2_nhwc_bwd(fake, fake, 2, 2, 8, 8, -1, None) == -1
    assert lib.svbrdf_gen_nhwc_partial_floats(3, 128) == 3 * 64 * 128
    # descriptor average pool: odd size
    assert lib.svbrdf_desc_avgpool_fwd(fake, fake, 1, 7, 8, 64, None) == -2
    assert lib.svbrdf_desc_avgpool_bwd(None, fake, None, fake, 1, 8, 8, 64, None) == -1
    # environment map: null tables, bad sizes
    args = [fake, 8, 8, fake, 8, 16, fake, fake, fake, None, fake, 32, 0.0, 1.0, 16, 1, None]
    assert lib.svbrdf_envmap_render(*args) == -1
    args[9] = fake
    args[14] = 0  # no samples
    assert lib.svbrdf_envmap_render(*args) == -1
    assert b"envmap" in lib.svbrdf_last_error()


def test_corrupt_plan_is_rejected_on_host(svb, lib):
    """Host-side fault injection: a plan whose header was overwritten is refused before any
    launch."""
    SV = svb._native
    mats, keep = _materials(SV, [(64, 64, 9)])
    cfg = SV.svbrdf_batch_config(480, 960, 3, 3)
    n = lib.svbrdf_batched_plan_bytes(mats, 1, ctypes.byref(cfg))
    buf = np.zeros(n, np.uint8)
    assert lib.svbrdf_batched_plan(mats, 1, ctypes.byref(cfg), buf.ctypes.data, n) == 0
    need = lib.svbrdf_batched_workspace_bytes(buf.ctypes.data)
    buf[0:4] = 0  # the magic
    fake = ctypes.c_void_p(16)
    assert lib.svbrdf_batched_workspace_bytes(buf.ctypes.data) == 0
    assert lib.svbrdf_batched_steps(fake, buf.ctypes.data, 1, fake, 0.01, 0.9, 0.999, 1e-8, fake, 4, 3, fake, need,
                                    None) == -1
    assert b"not a plan" in lib.svbrdf_last_error()
    # the wait self-test needs its 16-byte workspace and a sane poll limit
    assert lib.svbrdf_selftest_wait_timeout(fake, 8, 100, None) == -4
    assert lib.svbrdf_selftest_wait_timeout(fake, 16, 0, None) == -1


def test_texel_count_limit_rejected_on_host(lib):
    """H*W must stay below 2^31 (the kernels index texels in 64 bits, rows and columns in 32):
    the host rejects larger shapes before touching the device. Nothing is launched here."""
    fake = ctypes.c_void_p(16)
    for h, w in ((32768, 65536), (46341, 46341), (65536, 65536)):  # 2^31 exactly, just above, 2^32
        rc = lib.svbrdf_render_fwd(fake, fake, fake, fake, 9, h, w, 17.0, fake, None, -1, None, None, 0, None)
        assert rc == -2 and b"2^31" in lib.svbrdf_last_error()
        args = [fake] * 8 + [9, h, w, 17.0, 0, 1, 0.01, 0.9, 0.999, 1e-8, fake, fake, 1 << 20, None]
        assert lib.svbrdf_fused_step(*args) == -2
        assert lib.svbrdf_fused_step_noalloc(*(args[:19] + [None])) == -2


def test_batched_render_loss_sums_and_conv_entries_reject_bad_arguments_on_host(lib):
    """The batched render, the loss sums, the fused Gram-gradient GEMM, the TF32 convolution
    with a workspace, the pool-backward and render epilogues of the BF16 convolution and
    conv1_1's tensor-core data gradient refuse bad arguments before touching the device
    (nothing is launched)."""
    fake = ctypes.c_void_p(16)
    # batched render: batch must be >= 1; the per-material shape checks still apply
    assert lib.svbrdf_render_fwd_batch(fake, fake, fake, fake, 9, 8, 8, 17.0, 0, fake, None, -1, None, None, 0,
                                       None) == -1
    assert lib.svbrdf_render_bwd_batch(fake, fake, fake, fake, 9, 8, 8, 17.0, -1, fake, fake, None, None, 0,
                                       None) == -1
    assert lib.svbrdf_render_fwd_batch(fake, fake, fake, fake, 9, 46341, 46341, 17.0, 2, fake, None, -1, None,
                                       None, 0, None) == -2
    # loss sums: 1 to 16 segments, groups 0 or 1
    off = (ctypes.c_longlong * 2)(0, 4)
    ln = (ctypes.c_longlong * 2)(4, 4)
    w = (ctypes.c_double * 2)(1.0, 1.0)
    g_ok = (ctypes.c_int * 2)(0, 1)
    g_bad = (ctypes.c_int * 2)(0, 2)
    a = [ctypes.addressof(x) for x in (off, ln, w)]
    assert lib.svbrdf_desc_loss_sums(fake, 0, *a, ctypes.addressof(g_ok), fake, None) == -2
    assert lib.svbrdf_desc_loss_sums(fake, 17, *a, ctypes.addressof(g_ok), fake, None) == -2
    assert lib.svbrdf_desc_loss_sums(fake, 2, *a, ctypes.addressof(g_bad), fake, None) == -1
    assert lib.svbrdf_desc_loss_sums(None, 2, *a, ctypes.addressof(g_ok), fake, None) == -1
    # fused Gram gradient: m a multiple of 128, k of 64, the feature pointers present
    err = fake
    assert lib.svbrdf_desc_gemm_nt_feat(fake, fake, fake, 1, fake, 0.1, 0, fake, fake, 1, 100, 64, 64, err,
                                        None) == -2
    assert lib.svbrdf_desc_gemm_nt_feat(fake, fake, None, 1, fake, 0.1, 0, fake, fake, 1, 128, 64, 64, err,
                                        None) == -1
    assert lib.svbrdf_desc_gemm_nt_feat(fake, fake, fake, 4, fake, 0.1, 0, fake, fake, 1, 128, 64, 64, err,
                                        None) == -1  # dtypes 0..3
    assert lib.svbrdf_desc_gemm_nt_feat_partials(0, 128, 64) == 0
    assert lib.svbrdf_desc_gemm_nt_feat_partials(2, 256, 64) == 2 * 2 * 1 * 4
    # TF32 convolution with a workspace: the same shape rules as without
    assert lib.svbrdf_gen_conv_tf32_ex(fake, fake, fake, None, 0, 1, 8, 8, 48, 64, 3, 1, err, None) == -2
    assert lib.svbrdf_gen_conv_tf32_ex(fake, fake, fake, None, 0, 1, 8, 8, 64, 64, 5, 1, err, None) == -1
    # BF16 convolution: epilogues 4 and 5 (pool backward) need the pool's input as mask; 6 and
    # up are not epilogues of this entry
    assert lib.svbrdf_conv3x3_bf16_ex(fake, fake, None, None, None, fake, 1, 16, 16, 64, 64, 4, err, None) == -1
    assert lib.svbrdf_conv3x3_bf16_ex(fake, fake, None, fake, None, fake, 1, 16, 16, 64, 64, 6, err, None) == -1
    # conv1_1's tensor-core data gradient: shape granularity and null pointers
    assert lib.svbrdf_desc_conv1_bwd_tc(fake, fake, fake, fake, 1, 12, 16, 1, err, None) == -2
    assert lib.svbrdf_desc_conv1_bwd_tc(fake, None, fake, fake, 1, 16, 16, 1, err, None) == -1
