"""The no-allocation fused step against the regular one, through the C ABI.

svbrdf_fused_step_noalloc is for callers that cannot call cudaMalloc when they step the
optimiser (they pass only tensors they already own); its scratch is a static device array
inside the library. Here both entry points start from the same maps and moments and run
two iterations in a row each; the updated maps, Adam moments and losses must agree within
1e-6 relative L2 (the same kernel runs in both, so they normally agree bit for bit).
This file is collected last so that a failure here leaves every other test already run.
"""
import ctypes

import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _scene(svb, dev):
    from oracle import microfacet_ref as R

    sc = svb.scenes.single_scene(res=64, seed=1006)
    svb.scenes.add_targets(sc, lambda *a: R.render(*a, dtype=torch.float32))
    state = (0.6 * sc.init + 0.4 * sc.gt).contiguous()
    return sc, state.to(dev), sc.targets.to(dev), sc.camera_pos.to(dev).contiguous(), \
        sc.light_pos.to(dev).contiguous(), sc.light_pow.to(dev).contiguous()


def _run(lib, noalloc, tex, m, v, tgt, cam, lit, lp, size, loss, ws, stream):
    for step in (1, 2):
        common = [ctypes.c_void_p(tex.data_ptr()), ctypes.c_void_p(m.data_ptr()), ctypes.c_void_p(v.data_ptr()),
                  ctypes.c_void_p(tgt.data_ptr()), ctypes.c_void_p(cam.data_ptr()), ctypes.c_void_p(lit.data_ptr()),
                  ctypes.c_void_p(lp.data_ptr()), None, 9, 64, 64, ctypes.c_float(size), 1, step,
                  ctypes.c_float(0.01), ctypes.c_float(0.9), ctypes.c_float(0.999), ctypes.c_float(1e-8),
                  ctypes.c_void_p(loss[step - 1].data_ptr())]
        if noalloc:
            rc = lib.svbrdf_fused_step_noalloc(*common, ctypes.c_void_p(stream))
        else:
            rc = lib.svbrdf_fused_step(*common, ctypes.c_void_p(ws.data_ptr()), ctypes.c_size_t(ws.numel()),
                                       ctypes.c_void_p(stream))
        assert rc == 0, lib.svbrdf_last_error()


def test_noalloc_matches_workspace_entry_point(svb, cuda):
    lib = svb._native.lib()
    sc, state, tgt, cam, lit, lp = _scene(svb, cuda)
    stream = torch.cuda.current_stream(cuda).cuda_stream
    ws = torch.zeros(int(lib.svbrdf_workspace_bytes()), dtype=torch.uint8, device=cuda)
    ref = [state.clone(), torch.zeros_like(state), torch.zeros_like(state), torch.zeros(2, device=cuda)]
    new = [state.clone(), torch.zeros_like(state), torch.zeros_like(state), torch.zeros(2, device=cuda)]
    _run(lib, False, ref[0], ref[1], ref[2], tgt, cam, lit, lp, sc.size, ref[3], ws, stream)
    _run(lib, True, new[0], new[1], new[2], tgt, cam, lit, lp, sc.size, new[3], None, stream)
    torch.cuda.synchronize()
    for a, b in zip(new[:3], ref[:3]):
        assert rel_l2(a, b) <= 1e-6
    for k in range(2):
        assert abs(float(new[3][k]) - float(ref[3][k])) <= 1e-6 * abs(float(ref[3][k]))
    assert float(new[3][1]) < float(new[3][0])  # the second step lowers the loss
