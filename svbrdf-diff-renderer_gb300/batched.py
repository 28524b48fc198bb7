"""Many materials of uneven resolution and view count, optimised together.

Each material is what one ``SvbrdfOptim`` owns in the reference (src/svbrdf.py:15-83):
textures, Adam moments, targets and its own views. ``BatchedOptim`` advances all of them
with persistent launches of fused render, loss, adjoint and Adam (``svbrdf_batched_steps``):
one launch per iteration, or, with the resident-state variant, one launch per up to 32
iterations. ``run(iters)`` captures the launches of ``iters`` iterations into one CUDA graph.

The launch shape (threads per CTA, texels per work tile, persistent CTA count) comes from
``autotune``: it times each candidate on the real workload for a few iterations, on copies
of the state, and caches the winner per workload signature.
"""
from __future__ import annotations

import ctypes
import hashlib
import json
import os
import pathlib
from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np
import torch

from . import _native as N

LOSS_KINDS = {"mse": 0, "log1p": 1, "log1p_pre": 2}
FUSE_MAX = 32  # iterations per launch of the resident-state variants (kFuseMax in fused.cu)
# (variant, threads, tile_texels / threads)
CANDIDATES = ([(3, t, 2) for t in (224, 256, 384, 480)] +
              [(4, t, 2) for t in (512, 256)] +
              [(2, t, 2) for t in (224, 256, 384, 480)] +
              [(1, t, 1) for t in (256, 384, 480, 608)] +
              [(0, t, k) for t in (128, 256, 512) for k in (1, 4, 16)])
CACHE_FILE = pathlib.Path(os.environ.get("SVBRDF_TUNE_CACHE", str(pathlib.Path.home() / ".cache" / "svbrdf_gb300_tune.json")))


@dataclass
class BatchConfig:
    threads: int = 256
    tile_texels: int = 1024
    ctas: int = 0     # 0 = SM count x resident CTAs per SM
    variant: int = 0  # 0 direct loads, 1 bulk-copy (TMA) pipeline, 2 the pipeline on texel pairs,
    #                   3 texel pairs with the state resident across the iterations of a launch,
    #                   4 the same without a producer warp (the last reader of a buffer refills it)

    def as_c(self):
        return N.svbrdf_batch_config(self.threads, self.tile_texels, self.ctas, self.variant)


class BatchedOptim:
    """Batched per-pixel optimisation. ``materials`` items need ``init`` ([1,9,H,W]),
    ``targets`` ([V,3,H,W]), ``camera_pos``/``light_pos`` ([V,3]), ``light_pow`` ([3]) and
    ``size`` (cm); e.g. ``scenes.Scene`` objects.

    With ``optim_light`` every material's light power is optimised with its maps, as
    ``SvbrdfOptim.optim(..., optim_light=True)`` does (src/svbrdf.py:48-50, 58-59); the
    current values are ``light_pow(i)``. That needs the texel-pair kernels (variants 2 and 3),
    and each iteration is then its own launch. With ``adopt_maps`` a material's ``init``
    tensor that is already a contiguous FP32 tensor on the device becomes the optimised
    maps in place instead of being copied."""

    def __init__(self, materials: Sequence, lr: float = 0.01, loss: str = "log1p", device="cuda",
                 config: Optional[BatchConfig] = None, betas=(0.9, 0.999), eps: float = 1e-8,
                 hist_len: int = 100, optim_light: bool = False, adopt_maps: bool = False,
                 candidates=None):
        self.L = N.lib()
        self.device = torch.device(device)
        self.lr, self.betas, self.eps = float(lr), betas, float(eps)
        self.n = len(materials)
        self.tex, self.m1, self.m2, self.tgt, self.lpow = [], [], [], [], []
        self.cam_host, self.lit_host, self.meta = [], [], []
        if loss not in ("mse", "log1p"):
            raise ValueError("loss must be 'mse' or 'log1p'")
        self.loss = loss
        self.kind = LOSS_KINDS["mse"] if loss == "mse" else LOSS_KINDS["log1p_pre"]
        self.optim_light = bool(optim_light)
        self.lstate, self.lpow0 = [], []
        for m in materials:
            t = m.init.detach()
            if not (adopt_maps and t.device == self.device and t.dtype == torch.float32 and t.is_contiguous()):
                t = t.to(self.device, torch.float32).contiguous().clone()
            self.tex.append(t)
            self.m1.append(torch.zeros_like(t))
            self.m2.append(torch.zeros_like(t))
            tg = m.targets.to(self.device, torch.float32).contiguous()
            self.tgt.append(torch.log1p(tg) if loss == "log1p" else tg)
            self.lpow.append(torch.as_tensor(m.light_pow, dtype=torch.float32).to(self.device).contiguous().clone())
            self.lpow0.append(self.lpow[-1].clone())
            self.lstate.append(torch.zeros(6, device=self.device, dtype=torch.float32) if self.optim_light else None)
            self.cam_host.append(np.ascontiguousarray(torch.as_tensor(m.camera_pos).cpu().numpy(), dtype=np.float32))
            self.lit_host.append(np.ascontiguousarray(torch.as_tensor(m.light_pos).cpu().numpy(), dtype=np.float32))
            _, _, H, W = t.shape
            self.meta.append((H, W, int(self.cam_host[-1].shape[0]), float(m.size)))
        self.hist_len = int(hist_len)
        self.loss_hist = torch.zeros(self.hist_len, self.n, device=self.device, dtype=torch.float32)
        self.step_dev = torch.zeros(1, device=self.device, dtype=torch.int32)
        self.step_count = 0
        self.graph = None
        if config is None and self.optim_light:
            candidates = candidates or [c for c in CANDIDATES if c[0] in (2, 3)]
        self.config = config or autotune(self, candidates)
        self._build_plan(self.config)

    # ---- work accounting ----
    def texel_views(self) -> int:
        return sum(H * W * V for H, W, V, _ in self.meta)

    def algorithmic_bytes(self) -> int:
        """HBM bytes one iteration must move: params+m+v read and written, targets read."""
        return sum(H * W * (216 + 12 * V) for H, W, V, _ in self.meta)

    def launches(self, iters: int) -> int:
        """Kernel launches ``iters`` iterations take with this plan's variant."""
        return -(-iters // FUSE_MAX) if self.config.variant >= 3 and not self.optim_light else iters

    def light_pow(self, i: int) -> torch.Tensor:
        """Material ``i``'s light power (optimised in place with ``optim_light``)."""
        return self.lpow[i]

    def signature(self) -> str:
        h = hashlib.sha1(json.dumps(sorted(self.meta)).encode()).hexdigest()[:16]
        return f"{torch.cuda.get_device_name(self.device)}|{self.loss}|{h}"

    def tune_key(self) -> str:
        """The autotuner's cache key: the workload signature plus the library's ABI version and
        build hash, so a pick made with another build of the kernels is never reused."""
        return f"{self.signature()}|{N.build_id()}" + ("|light" if self.optim_light else "")

    # ---- plan ----
    def _mat_array(self, tex=None, m1=None, m2=None, lpow=None, lstate=None):
        tex = tex or self.tex
        m1 = m1 or self.m1
        m2 = m2 or self.m2
        lpow = lpow or self.lpow
        lstate = lstate or self.lstate
        arr = (N.svbrdf_material * self.n)()
        for i in range(self.n):
            H, W, V, size = self.meta[i]
            arr[i] = N.svbrdf_material(tex[i].data_ptr(), m1[i].data_ptr(), m2[i].data_ptr(), self.tgt[i].data_ptr(),
                                       lpow[i].data_ptr(), self.cam_host[i].ctypes.data,
                                       self.lit_host[i].ctypes.data, V, H, W, size, N.ptr(lstate[i]))
        return arr

    def _make_plan(self, cfg: BatchConfig, tex=None, m1=None, m2=None, lpow=None, lstate=None):
        arr = self._mat_array(tex, m1, m2, lpow, lstate)
        c = cfg.as_c()
        nbytes = self.L.svbrdf_batched_plan_bytes(arr, self.n, ctypes.byref(c))
        if nbytes == 0:
            N.check(-1)
        host = np.zeros(nbytes, dtype=np.uint8)
        N.check(self.L.svbrdf_batched_plan(arr, self.n, ctypes.byref(c), host.ctypes.data, nbytes))
        dev = torch.from_numpy(host).to(self.device)
        ws_bytes = self.L.svbrdf_batched_workspace_bytes(host.ctypes.data)
        ws = torch.zeros(int(ws_bytes), dtype=torch.uint8, device=self.device)
        return host, dev, ws

    def _build_plan(self, cfg: BatchConfig):
        self.plan_host, self.plan_dev, self.ws = self._make_plan(cfg)
        self.graph = None

    def n_ctas(self) -> int:
        return int(np.frombuffer(self.plan_host[:16].tobytes(), dtype=np.int32)[3])

    # ---- stepping ----
    def _launch(self, plan_host, plan_dev, ws, step_dev, loss_hist, iters: int = 1):
        b1, b2 = self.betas
        N.check(self.L.svbrdf_batched_steps(plan_dev.data_ptr(), plan_host.ctypes.data, self.kind,
                                            step_dev.data_ptr(), self.lr, float(b1), float(b2), self.eps,
                                            loss_hist.data_ptr(), int(loss_hist.shape[0]), int(iters),
                                            ws.data_ptr(), ws.numel(), N.stream_handle(self.device)))

    def step(self):
        """One iteration for every material (one eager launch). The step count is kept on
        the device; the losses of this iteration land in ``loss_hist[(step-1) % len]``."""
        self._launch(self.plan_host, self.plan_dev, self.ws, self.step_dev, self.loss_hist)
        self.step_count += 1

    @property
    def loss_out(self) -> torch.Tensor:
        """Per-material loss of the most recent iteration."""
        return self.loss_hist[(self.step_count - 1) % self.loss_hist.shape[0]]

    def capture(self, iters: int):
        """Capture ``iters`` iterations into one CUDA graph. Each replay advances every
        material by ``iters`` Adam steps (the step counter is device-resident)."""
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self._launch(self.plan_host, self.plan_dev, self.ws, self.step_dev, self.loss_hist, iters)
        self.graph, self.graph_iters = g, iters
        return g

    def run(self, iters: int):
        """Advance ``iters`` iterations through one CUDA-graph replay (captured on first use)."""
        if self.graph is None or self.graph_iters != iters:
            self.capture(iters)
        self.graph.replay()
        self.step_count += iters

    def reset(self, inits=None, targets=None):
        """Restart the optimisation (step 0, zero moments), optionally from new initial maps
        and targets (host or device tensors; pinned host memory copies asynchronously)."""
        self.upload(inits, targets)
        self.prepare(targets is not None)

    def upload(self, inits=None, targets=None):
        """The copy half of ``reset``: new initial maps and raw targets into the device
        buffers (copies only, no kernels, so it can run on a copy stream beside the compute)."""
        for i in range(self.n):
            if inits is not None:
                self.tex[i].copy_(inits[i], non_blocking=True)
            if targets is not None:
                self.tgt[i].copy_(targets[i], non_blocking=True)

    def prepare(self, new_targets: bool = True):
        """The device half of ``reset``: transform freshly uploaded targets for the loss, zero
        the moments, the step counter and the loss history (and, with ``optim_light``, put
        each light power back to its initial value with a fresh Adam state)."""
        for i in range(self.n):
            if new_targets and self.loss == "log1p":
                self.tgt[i].log1p_()
            self.m1[i].zero_()
            self.m2[i].zero_()
            if self.optim_light:
                self.lpow[i].copy_(self.lpow0[i])
                self.lstate[i].zero_()
        self.step_dev.zero_()
        self.loss_hist.zero_()
        self.step_count = 0

    def textures(self, i: int) -> torch.Tensor:
        return self.tex[i]

    # ---- checkpoints ---------------------------------------------------------------------
    def state_dict(self) -> dict:
        """Everything a later run needs to continue bit-identically: maps, both Adam moments,
        the device step counter and the loss history (FP32, on the host)."""
        torch.cuda.synchronize(self.device)
        st = {"tex": [t.cpu() for t in self.tex], "exp_avg": [t.cpu() for t in self.m1],
              "exp_avg_sq": [t.cpu() for t in self.m2], "step": int(self.step_dev.item()),
              "loss_hist": self.loss_hist.cpu(), "step_count": self.step_count, "signature": self.signature()}
        if self.optim_light:
            st["light_pow"] = [t.cpu() for t in self.lpow]
            st["light_adam"] = [t.cpu() for t in self.lstate]
        return st

    def load_state_dict(self, st: dict):
        if st.get("signature") not in (None, self.signature()):
            raise ValueError("checkpoint was written for a different set of materials")
        for dst, src in ((self.tex, st["tex"]), (self.m1, st["exp_avg"]), (self.m2, st["exp_avg_sq"])):
            if len(dst) != len(src):
                raise ValueError("checkpoint has a different number of materials")
            for d, s_ in zip(dst, src):
                d.copy_(s_)
        if self.optim_light and "light_pow" in st:
            for d, s_ in zip(self.lpow, st["light_pow"]):
                d.copy_(s_)
            for d, s_ in zip(self.lstate, st["light_adam"]):
                d.copy_(s_)
        self.step_dev.fill_(int(st["step"]))
        lh = st["loss_hist"]
        if lh.shape == self.loss_hist.shape:
            self.loss_hist.copy_(lh)
        self.step_count = int(st.get("step_count", st["step"]))

    def save(self, path):
        torch.save(self.state_dict(), path)

    def load(self, path):
        self.load_state_dict(torch.load(path, map_location="cpu"))

    def device_error(self) -> int:
        """The workspace error word (0 = healthy); synchronises with the device."""
        off = N.WORKSPACE_ERROR_OFFSET
        return int(self.ws[off:off + 4].view(torch.int32).item())

    def check(self):
        """Raise if a pipelined launch gave up waiting (see svbrdf_gb300.h)."""
        e = self.device_error()
        if e:
            raise N.SvbrdfError(-3, f"batched kernel reported device error {e}")


class BatchedPipeline:
    """A stream of batches of one shape, double-buffered so the host transfers hide behind
    the compute.

    Every batch has the same materials layout as ``materials``: resolutions, view counts,
    cameras, lights and light power. Only the initial maps and targets change. While one
    buffer's batch is optimised, the next batch's maps and targets upload on a copy stream
    and the previous batch's results download on another; the short device-side preparation
    of a batch (target transform, zeroed moments) runs on the compute stream.

    * ``submit(inits, targets)`` enqueues ``iters`` iterations of one batch and returns a
      ticket. The inputs are host tensors, pinned for asynchronous copies, one per material.
      They must stay unchanged until the batch's upload has run.
    * ``result(ticket)`` waits for that batch. It returns (maps, loss history) as pinned host
      tensors, valid until the submit two tickets later reuses the buffer."""

    def __init__(self, materials: Sequence, iters: int, lr: float = 0.01, loss: str = "log1p", device="cuda",
                 config: Optional[BatchConfig] = None, betas=(0.9, 0.999), eps: float = 1e-8):
        self.device = torch.device(device)
        self.iters = int(iters)
        a = BatchedOptim(materials, lr=lr, loss=loss, device=device, config=config, betas=betas, eps=eps,
                         hist_len=self.iters)
        b = BatchedOptim(materials, lr=lr, loss=loss, device=device, config=a.config, betas=betas, eps=eps,
                         hist_len=self.iters)
        self.bufs = [a, b]
        for o in self.bufs:
            o.capture(self.iters)
        self.config = a.config
        self.up = torch.cuda.Stream(self.device)
        self.down = torch.cuda.Stream(self.device)
        self.host_maps = [[torch.empty(t.shape, dtype=torch.float32).pin_memory() for t in o.tex] for o in self.bufs]
        self.host_loss = [torch.empty(o.loss_hist.shape, dtype=torch.float32).pin_memory() for o in self.bufs]
        self.done: List[Optional[torch.cuda.Event]] = [None, None]
        self.next_ticket = 0

    def h2d_bytes(self, inits, targets) -> int:
        return sum(t.numel() * t.element_size() for t in inits) + sum(t.numel() * t.element_size() for t in targets)

    def d2h_bytes(self) -> int:
        return sum(t.numel() * 4 for t in self.host_maps[0]) + self.host_loss[0].numel() * 4

    def submit(self, inits, targets) -> int:
        j = self.next_ticket % 2
        o = self.bufs[j]
        comp = torch.cuda.current_stream(self.device)
        with torch.cuda.stream(self.up):
            if self.done[j] is not None:  # the buffer's previous batch has been read back
                self.up.wait_event(self.done[j])
            o.upload(inits=inits, targets=targets)  # copy engines only
            uploaded = torch.cuda.Event()
            uploaded.record(self.up)
        comp.wait_event(uploaded)
        # the kernels of the reset run on the compute stream: on the copy stream they would
        # wait for SMs that the persistent launches of the previous batch hold
        o.prepare()
        o.graph.replay()
        o.step_count += self.iters
        computed = torch.cuda.Event()
        computed.record(comp)
        with torch.cuda.stream(self.down):
            self.down.wait_event(computed)
            for h, t in zip(self.host_maps[j], o.tex):
                h.copy_(t, non_blocking=True)
            self.host_loss[j].copy_(o.loss_hist, non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(self.down)
        self.done[j] = ev
        self.next_ticket += 1
        return self.next_ticket - 1

    def result(self, ticket: int):
        if not (self.next_ticket - 2 <= ticket < self.next_ticket):
            raise ValueError(f"ticket {ticket} is no longer (or not yet) held; the pipeline keeps two")
        j = ticket % 2
        self.done[j].synchronize()
        return self.host_maps[j], self.host_loss[j]

    def device_error(self) -> int:
        return max(o.device_error() for o in self.bufs)


def _time_config(opt: BatchedOptim, cfg: BatchConfig, iters: int = 16, repeats: int = 2) -> float:
    """Milliseconds per iteration of ``cfg``: the best of ``repeats`` timings of ``iters``
    iterations in one call (so the resident-state variant runs them in one launch, as a graph
    of a longer run does)."""
    tex = [t.clone() for t in opt.tex]
    m1 = [torch.zeros_like(t) for t in tex]
    m2 = [torch.zeros_like(t) for t in tex]
    lpow = [t.clone() for t in opt.lpow]
    lstate = [None if t is None else torch.zeros_like(t) for t in opt.lstate]
    host, dev, ws = opt._make_plan(cfg, tex, m1, m2, lpow, lstate)
    loss = torch.zeros(1, opt.n, device=opt.device)
    step = torch.zeros(1, device=opt.device, dtype=torch.int32)
    opt._launch(host, dev, ws, step, loss, 2)  # warm
    best = float("inf")
    for _ in range(repeats):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        opt._launch(host, dev, ws, step, loss, iters)
        e.record()
        e.synchronize()
        best = min(best, s.elapsed_time(e) / iters)
    off = N.WORKSPACE_ERROR_OFFSET
    if int(ws[off:off + 4].view(torch.int32).item()):
        raise N.SvbrdfError(-3, "device error during tuning")
    return best


def _load_cache():
    try:
        return json.loads(CACHE_FILE.read_text())
    except Exception:
        return {}


def autotune(opt: BatchedOptim, candidates=None, use_cache: bool = True) -> BatchConfig:
    """Pick threads/tile_texels/ctas for ``opt``'s workload by timing every candidate."""
    key = opt.tune_key()
    cache = _load_cache() if use_cache else {}
    if key in cache:
        return BatchConfig(**cache[key])
    best, best_ms = None, float("inf")
    results = []
    for variant, threads, mult in (candidates or CANDIDATES):
        cfg = BatchConfig(threads=threads, tile_texels=threads * mult, ctas=0, variant=variant)
        try:
            ms = _time_config(opt, cfg)
        except N.SvbrdfError:
            continue
        results.append((ms, variant, threads, mult))
        if ms < best_ms:
            best, best_ms = cfg, ms
    opt.tune_results = sorted(results)
    if best is None:
        best = BatchConfig()
    if use_cache:
        cache[key] = best.__dict__
        try:
            CACHE_FILE.parent.mkdir(parents=True, exist_ok=True)
            CACHE_FILE.write_text(json.dumps(cache, indent=1))
        except OSError:
            pass
    return best
