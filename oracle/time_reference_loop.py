"""Times the reference's own per-pixel loop beside this repository's CPU restatement of it.

TEST/MEASUREMENT INFRASTRUCTURE ONLY: the reference cannot travel to the GPU machine, so the
benchmark's CPU legs time ``oracle/microfacet_ref.py`` (the op-for-op restatement) there. This
script shows, on one host, how the two compare, on the single-material workload of the
reference's own scale: one 256^2 material, 9 co-located flash views on the 3x3 grid, 20 Adam
iterations (lr 0.01), MSE loss (src/optimization.py:28-29), all host threads.

* ``verbatim``: the reference's ``SvbrdfOptim.optim`` (src/svbrdf.py:44-83) with
  ``src/microfacet.py``'s renderer, imported from a reference checkout (``--ref``), its image
  and plot modules (cv2, PIL, matplotlib) stubbed, PNG save points included as no-ops;
* ``restated``: the same loop body on ``oracle/microfacet_ref.py`` (``optim_loop``).

Run from the repository root:  python oracle/time_reference_loop.py --ref /path/to/reference
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import pathlib
import sys
import tempfile
import time
import types

import torch

REPO = pathlib.Path(__file__).resolve().parent.parent
sys.path.insert(0, str(REPO))


def _stub_modules():
    class _Any(types.ModuleType):
        def __getattr__(self, name):
            if name.startswith("__"):
                raise AttributeError(name)
            return lambda *a, **k: None

    for name in ("cv2", "PIL", "PIL.Image", "matplotlib", "matplotlib.pyplot"):
        sys.modules.setdefault(name, _Any(name))
    sys.modules["PIL"].Image = sys.modules["PIL.Image"]
    sys.modules["matplotlib"].pyplot = sys.modules["matplotlib.pyplot"]


class _SvbrdfObj:
    """The part of SvbrdfIO that SvbrdfOptim.optim touches: cl, optimize_dir and the savers."""

    def __init__(self, cl, tmp):
        self.cl = cl
        self.optimize_dir = pathlib.Path(tmp)

    def save_textures_th(self, *a, **k):
        pass

    def save_images_th(self, *a, **k):
        pass


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="root of a checkout of the reference repository")
    ap.add_argument("--res", type=int, default=256)
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--repeats", type=int, default=3)
    a = ap.parse_args()
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    _stub_modules()
    sys.path.insert(0, a.ref)
    micro = importlib.import_module("src.microfacet")
    svbrdf = importlib.import_module("src.svbrdf")
    from oracle import microfacet_ref as R

    scenes = importlib.import_module("svbrdf-diff-renderer_gb300.scenes")
    sc = scenes.single_scene(res=a.res, seed=1000, render_fn=lambda *x: R.render(*x, dtype=torch.float32))
    tv = a.res * a.res * sc.n_views * a.epochs
    out = {"workload": f"1 material {a.res}^2, {sc.n_views} co-located views, {a.epochs} Adam iterations, MSE",
           "threads": threads, "texel_views": tv}
    best_v, best_r = float("inf"), float("inf")
    for _ in range(a.repeats):
        cl = [sc.camera_pos.clone(), sc.light_pos.clone(), sc.light_pow.clone()]
        renderer = micro.Microfacet(a.res, sc.n_views, sc.size, cl, "cpu")
        opt = svbrdf.SvbrdfOptim("cpu", renderer)
        opt.load_targets(sc.targets)
        opt.init_from_const(rgh=0.5)
        with tempfile.TemporaryDirectory() as tmp:
            t0 = time.perf_counter()
            opt.optim(a.epochs, 0.01, _SvbrdfObj(cl, tmp), False)
            best_v = min(best_v, time.perf_counter() - t0)
        t0 = time.perf_counter()
        R.optim_loop(sc.init, sc.targets, sc.camera_pos, sc.light_pos, sc.light_pow, sc.size, a.epochs, 0.01, "mse",
                     False, torch.float32)
        best_r = min(best_r, time.perf_counter() - t0)
    out["verbatim_s"] = best_v
    out["restated_s"] = best_r
    out["verbatim_texel_views_per_s"] = tv / best_v
    out["restated_texel_views_per_s"] = tv / best_r
    out["restated_over_verbatim"] = best_v / best_r
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
