#!/usr/bin/env python
"""Benchmark: texel*view render+adjoint+Adam updates/s, fused batched vs plain, on GB300.

Workload (the uneven batched per-pixel optimisation): 64 seeded synthetic materials,
resolution drawn from {256, 512, 1024}, 5-16 co-located flash views within +-8 cm at
25-35 cm, log(1+x) L2 loss, Adam lr 0.01. One *step* is one replay of a CUDA graph of
100 iterations over every material: with the autotuner's usual pick, the resident-state
kernel, that is 4 persistent launches of 25 iterations each (one launch per iteration for
the other kernels). Metric unit: texel*view updates per second = sum(H*W*V) * iterations / s.

Lines printed (rank 0, one JSON line):
* ``value``: device-resident inputs, CUDA events around K graph replays;
* ``e2e``: the same job through the public API from pinned host buffers: each step copies
  the initial maps and the targets host->device, restarts the optimiser, runs the 100
  iterations and copies the optimised maps and the loss history back;
* ``roofline``: the batched kernel's algorithmic bytes per launch (params+moments read and
  written, targets read: sum H*W*(216+12V) per iteration, times the iterations the launch
  runs) over its average launch time, against the measured HBM copy bandwidth; ``traffic``
  is the kernel's DRAM bytes per launch (ncu), far below the algorithmic bytes for the
  resident-state kernel, which moves its state through DRAM once per launch;
* ``per_iteration_kernel``: the one-launch-per-iteration texel-pair kernel on the same
  materials, whose DRAM traffic equals its algorithmic bytes;
* ``plain`` / ``fused_single``: the unfused single-material GPU form (forward kernel +
  torch loss + adjoint kernel via autograd + torch.optim.Adam) and the fused single-material
  kernel, both on the 1024^2, 9-view scene;
* ``cpu_baseline``: the reference's PyTorch CPU loop (the oracle restatement, same op
  sequence) on a bounded sample of the workload, all host threads;
* ``config0``: the reference's own scale (1 material 256^2, 9 views, 20 iterations, MSE) on
  the CPU (the same restatement, all host threads) and through the GPU drop-in optimiser;
* ``descriptor``, ``latent``, ``envmap``: the VGG-feature loss, the MaterialGAN latent loop
  with the per-pixel refinement, and a frame of the environment-map video.

``--impl reference`` times only that CPU implementation (rank 0), one step = one
iteration over the sample.

The inputs are larger than L2 (several GB of targets and state), so no L2 flush is done.
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import pathlib
import statistics
import subprocess
import sys
import tempfile
import time

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))

import torch  # noqa: E402

PKG = importlib.import_module("svbrdf-diff-renderer_gb300")
METRIC = "texel*view render+adjoint+Adam updates/s, fused batched vs plain, 1 GB300"
UNIT = "texel*view updates/s"
KERNEL_NAMES = {0: "batched_step_kernel", 1: "batched_tma_kernel", 2: "batched_pair_kernel", 3: "batched_fuse_kernel",
                4: "batched_fuse2_kernel"}
WORKLOAD = "batched 64 materials, res {256,512,1024}, V 5-16, 100 iterations per graph replay, log1p L2, Adam lr 0.01"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--materials", type=int, default=64)
    ap.add_argument("--iters", type=int, default=100, help="iterations per step (graph replay)")
    ap.add_argument("--no-extras", action="store_true", help="skip the plain/single/cpu comparison legs")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU baseline budget")
    ap.add_argument("--config", default=None, help="threads,tile_texels[,ctas[,variant]] instead of autotuning")
    ap.add_argument("--only", default=None, choices=["descriptor", "latent", "envmap", "single"],
                    help="run one comparison leg alone")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def material_cost(res, views):
    """Cost model of one material per iteration, as the planner's: texels x (views + 5)."""
    return res * res * (views + 5)


def shard(costs, world):
    """Greedy (largest first) assignment of materials to ranks; returns a list per rank."""
    order = sorted(range(len(costs)), key=lambda i: -costs[i])
    load = [0.0] * world
    out = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        out[r].append(i)
        load[r] += costs[i]
    return [sorted(x) for x in out]


def workload_specs(n, scene_seed=0):
    """Resolutions and view counts of the batch, without generating maps."""
    g = torch.Generator().manual_seed(scene_seed)
    specs = []
    for _ in range(n):
        res = (256, 512, 1024)[int(torch.randint(3, (1,), generator=g))]
        v = int(torch.randint(5, 17, (1,), generator=g))
        torch.rand(v, 2, generator=g)  # keep the draw order of scenes.batched_scenes
        torch.rand(v, 1, generator=g)
        specs.append((res, v))
    return specs


def gpu_render_fn(dev):
    def fn(tex, cam, lit, lp, size):
        r = PKG.Microfacet(tex.shape[-1], cam.shape[0], size, [cam.to(dev), lit.to(dev), lp.to(dev)], dev)
        with torch.no_grad():
            return r.eval(tex.to(dev))
    return fn


# ---------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, dev_index=0):
        self.proc = None
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        sel = []
        try:
            uuid = str(torch.cuda.get_device_properties(dev_index).uuid)
            sel = ["-i", uuid if uuid.startswith("GPU-") else "GPU-" + uuid]
        except Exception:
            sel = []
        self.cmd = ["nvidia-smi", *sel, f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200"]

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(self.cmd, stdout=self.file, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        self.file.flush()
        self.file.seek(0)
        rows = [l.strip().split(",") for l in self.file.read().splitlines() if l.strip()]
        try:
            os.unlink(self.file.name)
        except OSError:
            pass
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            if len(r) < 8:
                continue
            try:
                sm.append(float(r[0]))
                mx.append(float(r[1]))
            except ValueError:
                continue
            for nm, val in zip(names, r[4:8]):
                if val.strip().lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    p = HERE / "MEASURED_PEAKS.json"
    try:
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ---------------------------------------------------------------- CPU reference (oracle port)
def cpu_reference_sample(specs_idx, specs, budget_texel_views):
    """Materials of the workload (in order) up to a texel*view budget, generated on CPU."""
    from oracle import microfacet_ref as R

    chosen = []
    tot = 0
    for i in specs_idx:
        res, v = specs[i]
        # 1024^2 materials are left out of the CPU sample: the reference's autograd graph
        # holds ~60 [V,3,H,W] temporaries, several GB per material at that size
        if res > 512 or (chosen and tot + res * res * v > budget_texel_views):
            continue
        chosen.append(i)
        tot += res * res * v
        if tot >= budget_texel_views:
            break
    all_sc = PKG.scenes.batched_scenes(n=max(chosen) + 1, render_fn=None)
    mats = []
    for i in chosen:
        sc = all_sc[i]
        PKG.scenes.add_targets(sc, lambda *a: R.render(*a, dtype=torch.float32))
        mats.append(sc)
    return mats, tot


class CpuReferenceLoop:
    """The reference's loop (src/svbrdf.py:48-71) through the oracle's restatement of
    Microfacet.eval, one torch.optim.Adam per material, on the host cores."""

    def __init__(self, mats, lr=0.01):
        from oracle import microfacet_ref as R

        self.R = R
        self.mats = mats
        self.tex = [m.init.clone().requires_grad_(True) for m in mats]
        self.opts = [torch.optim.Adam([t], lr=lr, betas=(0.9, 0.999)) for t in self.tex]

    def step(self):
        for m, t, o in zip(self.mats, self.tex, self.opts):
            out = self.R.render(t.clamp(-1, 1), m.camera_pos, m.light_pos, m.light_pow, m.size, torch.float32)
            loss = self.R.image_loss(out, m.targets, "log1p")
            o.zero_grad()
            loss.backward()
            o.step()


def run_cpu_baseline(specs, seconds, threads):
    torch.set_num_threads(threads)
    mats, tv = cpu_reference_sample(range(len(specs)), specs, budget_texel_views=6e6)
    loop = CpuReferenceLoop(mats)
    loop.step()  # warm
    n, t0 = 0, time.perf_counter()
    while True:
        loop.step()
        n += 1
        el = time.perf_counter() - t0
        if el >= seconds or n >= 50:
            break
    return {"value": tv * n / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{len(mats)} materials (res <= 512) of the batch ({tv} texel*views), {n} Adam iterations, "
                      f"reference loop restated in torch (oracle), {threads} threads"}


def time_config0(dev, threads):
    """The reference's own scale (configs[0]): one 256^2 material, 9 co-located views on the 3x3
    grid, 20 Adam iterations (lr 0.01), MSE loss. CPU: the oracle's restatement of the
    reference's loop on all host threads; GPU: the drop-in SvbrdfOptim.optim (one-material
    batched plan, graph replay), warmed by one identical call."""
    from oracle import microfacet_ref as R

    sc = PKG.scenes.single_scene(res=256, seed=1000, render_fn=lambda *a: R.render(*a, dtype=torch.float32))
    tv = 256 * 256 * sc.n_views * 20
    torch.set_num_threads(threads)
    R.optim_loop(sc.init, sc.targets, sc.camera_pos, sc.light_pos, sc.light_pow, sc.size, 2, 0.01, "mse", False,
                 torch.float32)
    t0 = time.perf_counter()
    R.optim_loop(sc.init, sc.targets, sc.camera_pos, sc.light_pos, sc.light_pow, sc.size, 20, 0.01, "mse", False,
                 torch.float32)
    cpu_s = time.perf_counter() - t0
    r = PKG.Microfacet(256, sc.n_views, sc.size, [t.to(dev) for t in sc.cl], dev)
    o = PKG.SvbrdfOptim(dev, r, loss="mse", graph=True)
    o.load_targets(sc.targets.to(dev))
    o.init_from_tex(sc.init.to(dev))
    o.optim(20, 0.01, None, False)
    with torch.no_grad():
        o.textures.copy_(sc.init.to(dev))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    o.optim(20, 0.01, None, False)
    torch.cuda.synchronize()
    gpu_s = time.perf_counter() - t0
    sample = "1 material 256^2, 9 co-located views, 20 Adam iterations, MSE (the reference's scale)"
    return {"workload": sample,
            "cpu": {"value": tv / cpu_s, "unit": UNIT, "cores": threads, "kind": "port", "seconds": cpu_s,
                    "sample": sample + ", reference loop restated in torch (oracle)"},
            "gpu": {"value": tv / gpu_s, "unit": UNIT, "seconds": gpu_s,
                    "form": "drop-in SvbrdfOptim.optim, one-material batched plan in one CUDA graph, wall clock"},
            "gpu_over_cpu": cpu_s / gpu_s}


def impl_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    specs = workload_specs(args.materials)
    mats, tv = cpu_reference_sample(range(len(specs)), specs, budget_texel_views=1.2e7)
    loop = CpuReferenceLoop(mats)
    for _ in range(args.warmup):
        loop.step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        loop.step()
    el = time.perf_counter() - t0
    value = tv * args.steps / el
    sample = (f"{len(mats)} materials (res <= 512) of the batched workload ({tv} texel*views per step), one Adam iteration per "
              f"step, reference loop restated in torch (oracle), {threads} threads")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "sample": sample},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------- GPU legs
def time_single(dev, fused, iters, res=1024, kernel="batched"):
    """Single material 1024^2, 9 views, through the drop-in SvbrdfOptim: plain (unfused), or
    fused with the default one-material batched plan (kernel="batched") or the per-epoch
    single-material kernel (kernel="single"); texel*view/s."""
    sc = PKG.scenes.single_scene(res=res, device=dev, render_fn=gpu_render_fn(dev))
    r = PKG.Microfacet(res, 9, sc.size, sc.cl, dev)
    o = PKG.SvbrdfOptim(dev, r, loss="log1p", fused=fused, graph=fused, kernel=kernel)
    o.load_targets(sc.targets)
    o.init_from_tex(sc.init.clone())
    o.optim(iters, 0.01, None, False)  # warm: the same call (plan, tuning and graph are reused after it)
    with torch.no_grad():
        o.textures.copy_(sc.init)  # restart from the initial maps in the same buffer
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    o.optim(iters, 0.01, None, False)
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    form = (", forward kernel + torch loss + adjoint kernel (autograd) + torch.optim.Adam" if not fused else
            ", one-material plan of the batched kernels in one CUDA graph" if kernel == "batched" else
            ", single-material fused kernel, one launch per iteration, in one CUDA graph")
    out = {"value": res * res * 9 * iters / el, "unit": UNIT,
           "workload": f"1 material {res}^2, 9 views, {iters} Adam iterations, log1p L2" + form}
    b = getattr(o, "_batched", None) if fused and kernel == "batched" else None
    if b is not None:
        out["batch_config"] = b.config.__dict__
        out["autotune_ms"] = [list(r) for r in getattr(b, "tune_results", [])[:6]]
    return out


def time_envmap(dev, res=256, spp=256, frames=5):
    """One frame of the reference's novel-view video (src/scripts.py:44-59, Mitsuba at
    256 spp in the reference, src/mitsubarender.py:36): a 256^2 seeded material under the
    seeded synthetic environment, 256 samples per pixel, CUDA events over `frames` frames."""
    mat = PKG.scenes.make_material(256, 777)[0]
    r = PKG.EnvmapRenderer([res, res], None, mat, device=dev, spp=spp, seed=0)
    out = r.render_device(0.0, 0.5)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for k, a in enumerate(PKG.envmap.video_angles(frames)):
        r.render_device(float(a), 0.5, out=out)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / frames
    return {"workload": f"{res}^2 frame, {spp} spp, 256^2 material, synthetic {r.env.shape[0]}x{r.env.shape[1]} "
                        "environment (the reference's fig/ennis.exr is not in its repository)",
            "ms_per_frame": ms, "camera_samples_per_s": res * res * spp / (ms / 1e3)}


def time_descriptor(dev, iters=10, views=9, res=512):
    """Descriptor loss forward + backward over `views` renders of res^2 (2x2-downsampled to
    (res/2)^2), VGG19-shaped conv1_1..conv4_1. Reports the tcgen05 convolutions' FLOP rate."""
    d = PKG.descriptor.VGGDescriptor(dev, seed=0)
    sc = PKG.scenes.single_scene(res=res, device=dev, render_fn=gpu_render_fn(dev))
    cam, lit = sc.camera_pos[:views], sc.light_pos[:views]
    r0 = gpu_render_fn(dev)(sc.init, cam, lit, sc.light_pow, sc.size)
    d.load(sc.targets[:views])
    h = res // 2
    flops = 0.0
    for item in PKG.descriptor.VGG19_TO_CONV4_1:
        if item == "pool":
            h //= 2
            continue
        _, cin, cout = item
        if cin >= 64:  # the tensor-core convolutions: forward and data gradient
            flops += 2 * 2.0 * h * h * cin * cout * 9 * views
    for _ in range(2):
        d.loss_and_grad(r0)  # captures the forward + backward graph on first use
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.nvtx.range_push("descriptor")
    e0.record()
    for _ in range(iters):
        d.loss_and_grad(r0)
    e1.record()
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / iters
    tf = flops / (ms / 1e3) / 1e12
    peak = 1910.1
    try:
        peak = float(json.loads((HERE / "MEASURED_PEAKS.json").read_text())["bf16_tflops"])
    except Exception:
        pass
    return {"workload": f"{views} renders {res}^2 -> {res // 2}^2, conv1_1..conv4_1 forward + data gradient, "
                        "feature + Gram loss, one CUDA-graph replay per iteration", "ms_per_iteration": ms, "tc_conv_tflops": tf,
            "tc_conv_gflop_per_iteration": flops / 1e9, "bf16_peak_tflops": peak, "frac_of_bf16_peak": tf / peak,
            "device_error": d.device_error()}


def time_latent(dev, batch=16, iters=10, refine_iters=20):
    """Latent-space optimisation of a batch of materials (StyleGAN2-shaped generator, seeded
    weights, W+ [batch, 14, 512]) through the renderer adjoint at 256^2, then per-pixel
    refinement of the Lanczos-upsampled maps at 512^2 and 1024^2 with the batched fused kernel."""
    MG = PKG.materialgan
    rf = gpu_render_fn(dev)
    gen = MG.StyleGAN2Generator(256, seed=0)
    cam = PKG.scenes.grid_views().to(dev)
    lp = torch.full((3,), PKG.scenes.LIGHT_POW, device=dev)
    gts = [PKG.scenes.make_material(1024, 2000 + i, dev) for i in range(batch)]

    def targets_at(res):
        out = []
        for gt in gts:
            g = torch.nn.functional.interpolate(gt, size=(res, res), mode="area") if res != 1024 else gt
            out.append(rf(g, cam, cam, lp, PKG.scenes.GRID_SIZE_CM))
        return out

    t256 = torch.cat(targets_at(256))
    r = PKG.Microfacet(256, 9, PKG.scenes.GRID_SIZE_CM, [cam, cam, lp], dev)
    o = MG.MaterialGANOptim(dev, r, gen)
    o.load_targets(t256)
    o.init_from(batch=batch, seed=1)
    o.optim([2, 10, 10], 0.02)  # warm
    o.loss_image_list = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    tex = o.optim([iters, 10, 10], 0.02)
    torch.cuda.synchronize()
    lat_s = (time.perf_counter() - t0) / iters
    # one more latent epoch (a graph replay) in its own NVTX range, so a profiler can list
    # exactly one epoch's launches; it runs after the timing and the refinement starts from tex
    graph, _, _ = o._graph_for(True, 0.02)
    torch.cuda.nvtx.range_push("latent_epoch")
    graph.replay()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    out = {"workload": f"{batch} materials, W+ [{batch},14,512], generator 256^2 (seeded weights), 9 views, Adam lr 0.02",
           "latent_ms_per_iteration": lat_s * 1e3,
           "latent_texel_views_per_s": batch * 256 * 256 * 9 / lat_s,
           "latent_loss_first_last": [o.loss_image_list[0], o.loss_image_list[-1]]}
    for res in (512, 1024):
        tex = MG.upsample_textures(tex, res)
        tg = targets_at(res)
        mats = []
        for i in range(batch):
            sc = PKG.scenes.Scene(res=res, size=PKG.scenes.GRID_SIZE_CM, camera_pos=cam, light_pos=cam, light_pow=lp,
                                  gt=gts[i], targets=tg[i], init=tex[i:i + 1])
            mats.append(sc)
        b = PKG.BatchedOptim(mats, lr=0.01, loss="mse", device=dev, hist_len=refine_iters)
        b.capture(refine_iters)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b.run(refine_iters)
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        out[f"refine_{res}_ms"] = el * 1e3
        out[f"refine_{res}_texel_views_per_s"] = batch * res * res * 9 * refine_iters / el
        tex = torch.cat([t.clamp(-1, 1) for t in b.tex])
        del b, mats
    return out


def impl_ours(args):
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    specs = workload_specs(args.materials)
    costs = [material_cost(r, v) for r, v in specs]
    mine = shard(costs, world)[rank]
    all_sc = PKG.scenes.batched_scenes(n=args.materials, device=dev, render_fn=None)
    mats = []
    for i in mine:
        PKG.scenes.add_targets(all_sc[i], gpu_render_fn(dev))
        mats.append(all_sc[i])
    del all_sc
    cfg = None
    if args.config:
        parts = [int(x) for x in args.config.split(",")]
        cfg = PKG.BatchConfig(parts[0], parts[1], parts[2] if len(parts) > 2 else 0, parts[3] if len(parts) > 3 else 0)
    opt = PKG.BatchedOptim(mats, lr=0.01, loss="log1p", device=dev, hist_len=args.iters, config=cfg)
    tv = opt.texel_views()
    abytes = opt.algorithmic_bytes()
    opt.capture(args.iters)
    for _ in range(args.warmup):
        opt.run(args.iters)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()

    stream = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("timed")  # profilers filter the timed launches by this range
        e0.record(stream)
        for _ in range(args.steps):
            opt.run(args.iters)
        e1.record(stream)
        torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
        barrier()
    ms = e0.elapsed_time(e1)
    clocks = clk.summary()
    if world > 1:
        import torch.distributed as dist

        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t)
        tvt = torch.tensor([float(tv)], device=dev)
        dist.all_reduce(tvt)
        tv_all = float(tvt)
    else:
        tv_all = float(tv)
    value = tv_all * args.iters * args.steps / (ms / 1e3)
    launches_per_run = opt.launches(args.iters)
    iters_per_launch = args.iters / launches_per_run
    launch_ms = ms / (args.steps * launches_per_run)
    peak, peak_kind = peaks()
    # algorithmic bytes of one launch: the per-texel-iteration figure x the iterations it runs
    launch_abytes = abytes * iters_per_launch
    achieved = launch_abytes / (launch_ms / 1e3) / 1e9
    # DRAM bytes per launch: an ncu capture of a smaller case of the same kernel, scaled to
    # this launch by the algorithmic bytes (traffic is proportional to texels x views)
    traffic = None
    cfg_used = opt.config
    n_ctas = opt.n_ctas()
    tune = [list(r) for r in getattr(opt, "tune_results", [])[:8]]
    kernel = KERNEL_NAMES[cfg_used.variant]
    tfile = HERE / "profiles" / f"{kernel}_traffic.json"
    issue = None
    if tfile.exists():
        try:
            tj = json.loads(tfile.read_text())
            # a resident-state launch moves its state and targets once, whatever its iterations
            traffic = float(tj["dram_bytes_per_algorithmic_byte"]) * (abytes if tj.get("per_launch_pass") else launch_abytes)
            # the instruction-issue roofline: warp instructions per texel*view (from the same
            # capture) times the measured rate, against one issue per cycle per scheduler
            if tj.get("warp_instructions_per_texel_view"):
                wi = float(tj["warp_instructions_per_texel_view"])
                sms = torch.cuda.get_device_properties(dev).multi_processor_count
                mhz = None
                try:
                    mhz = float(json.loads((HERE / "MEASURED_PEAKS.json").read_text())["sm_max_mhz"])
                except Exception:
                    mhz = 2070.0
                issue_rate = value * wi
                issue_peak = sms * 4 * mhz * 1e6
                issue = {"warp_instructions_per_texel_view": wi, "achieved": issue_rate, "peak": issue_peak,
                         "unit": "warp instructions/s", "frac": issue_rate / issue_peak,
                         "source": f"profiles/{kernel}_traffic.json"}
        except Exception:
            traffic = None

    # ---- end to end through the public API, host buffers ----
    h_init = [m.init.detach().cpu().pin_memory() for m in mats]
    h_tgt = [m.targets.detach().cpu().pin_memory() for m in mats]
    h_out = [torch.empty(t.shape, dtype=t.dtype).pin_memory() for t in opt.tex]
    h_loss = torch.empty(opt.loss_hist.shape, dtype=torch.float32).pin_memory()
    h2d = sum(t.numel() * 4 for t in h_init) + sum(t.numel() * 4 for t in h_tgt)
    d2h = sum(t.numel() * 4 for t in h_out) + h_loss.numel() * 4

    def e2e_step():
        opt.reset(inits=h_init, targets=h_tgt)
        opt.run(args.iters)
        for i, t in enumerate(opt.tex):
            h_out[i].copy_(t, non_blocking=True)
        h_loss.copy_(opt.loss_hist, non_blocking=True)

    def max_over_ranks(x):
        if world > 1:
            import torch.distributed as dist

            t = torch.tensor([x], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            return float(t)
        return x

    # sequential: each step uploads, optimises and downloads before the next starts
    e2e_step()
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    torch.cuda.synchronize()
    barrier()
    seq_s = max_over_ranks(time.perf_counter() - t0)
    seq_value = tv_all * args.iters * args.steps / seq_s

    # pipelined (the public BatchedPipeline): the next batch uploads and the previous one
    # downloads on copy streams while the current one runs; every step still moves its
    # inputs in and its maps and losses out
    del opt
    torch.cuda.empty_cache()
    pipe = PKG.BatchedPipeline(mats, iters=args.iters, lr=0.01, loss="log1p", device=dev, config=cfg_used)
    pipe.result(pipe.submit(h_init, h_tgt))
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    torch.cuda.nvtx.range_push("e2e")
    tickets = [pipe.submit(h_init, h_tgt) for _ in range(args.steps)]
    pipe.result(tickets[-1])
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    barrier()
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    e2e_value = tv_all * args.iters * args.steps / e2e_s
    pipe_err = pipe.device_error()
    del pipe
    torch.cuda.empty_cache()

    # the one-launch-per-iteration kernel (variant 2) on the same materials: the HBM-bound
    # form, for which the per-iteration algorithmic bytes are the real DRAM traffic
    per_iter = None
    if cfg_used.variant >= 3:
        pairs = [r for r in tune if r[1] == 2]
        pc = PKG.BatchConfig(pairs[0][2], pairs[0][2] * pairs[0][3], 0, 2) if pairs else PKG.BatchConfig(480, 960, 0, 2)
        o2 = PKG.BatchedOptim(mats, lr=0.01, loss="log1p", device=dev, hist_len=args.iters, config=pc)
        o2.capture(args.iters)
        for _ in range(args.warmup):
            o2.run(args.iters)
        torch.cuda.synchronize()
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record(stream)
        for _ in range(args.steps):
            o2.run(args.iters)
        a1.record(stream)
        torch.cuda.synchronize()
        ms2 = a0.elapsed_time(a1)
        l2ms = ms2 / (args.steps * args.iters)
        ach2 = abytes / (l2ms / 1e3) / 1e9
        per_iter = {"kernel": KERNEL_NAMES[2], "batch_config": pc.__dict__,
                    "value": float(tv) * args.iters * args.steps / (ms2 / 1e3), "launch_ms": l2ms,
                    "achieved_gbs": ach2, "frac": ach2 / peak, "device_error": o2.device_error()}
        del o2
        torch.cuda.empty_cache()

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded materials and flash views)",
            "config": {"workload": WORKLOAD, "materials": args.materials, "materials_this_rank": len(mats),
                       "texel_views_per_iteration": tv_all, "iterations_per_step": args.iters,
                       "batch_config": cfg_used.__dict__, "ctas": n_ctas, "autotune_ms": tune,
                       "l2": "inputs larger than L2 (no flush)", "parallelism": f"materials sharded over {world} GPU(s)"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                         "kernel": kernel,
                         "algorithmic_bytes_per_launch": launch_abytes,
                         "iterations_per_launch": iters_per_launch,
                         "launch_ms": launch_ms, "issue": issue},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "mode": "BatchedPipeline: two buffers, uploads and downloads on copy streams overlap the compute",
                    "sequential_value": seq_value, "device_error": pipe_err},
            "per_iteration_kernel": per_iter,
            "gpu_launches": args.steps * launches_per_run,
            "clocks": clocks}
    if rank == 0 and not args.no_extras:
        line["plain"] = time_single(dev, fused=False, iters=20)
        line["fused_single"] = time_single(dev, fused=True, iters=200)
        line["fused_single_kernel"] = time_single(dev, fused=True, iters=200, kernel="single")
        line["fused_vs_plain"] = value / line["plain"]["value"]
        line["descriptor"] = time_descriptor(dev)
        line["latent"] = time_latent(dev, iters=5)
        line["envmap"] = time_envmap(dev)
        if world == 1:
            line["cpu_baseline"] = run_cpu_baseline(specs, args.cpu_seconds, os.cpu_count() or 1)
            line["config0"] = time_config0(dev, os.cpu_count() or 1)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.only == "descriptor":
        dev = torch.device("cuda", dist_env()[2])
        print(json.dumps({"descriptor": time_descriptor(dev, iters=max(args.steps, 1))}), flush=True)
        return 0
    if args.only == "latent":
        dev = torch.device("cuda", dist_env()[2])
        print(json.dumps({"latent": time_latent(dev, iters=max(args.steps, 1))}), flush=True)
        return 0
    if args.only == "envmap":
        dev = torch.device("cuda", dist_env()[2])
        print(json.dumps({"envmap": time_envmap(dev)}), flush=True)
        return 0
    if args.only == "single":
        # the drop-in single-material forms on the 1024^2, 9-view scene: plain (forward and
        # adjoint kernels behind autograd, torch loss and Adam) and fused
        dev = torch.device("cuda", dist_env()[2])
        torch.cuda.nvtx.range_push("single")
        out = {"plain": time_single(dev, fused=False, iters=max(args.steps, 1)),
               "fused_single": time_single(dev, fused=True, iters=max(args.steps, 1) * 10),
               "fused_single_kernel": time_single(dev, fused=True, iters=max(args.steps, 1) * 10, kernel="single")}
        torch.cuda.nvtx.range_pop()
        print(json.dumps(out), flush=True)
        return 0
    if args.impl == "reference":
        return impl_reference(args)
    return impl_ours(args)


if __name__ == "__main__":
    sys.exit(main())
