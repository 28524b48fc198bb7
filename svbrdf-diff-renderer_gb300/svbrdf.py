"""Drop-in per-pixel optimiser ``SvbrdfOptim`` (src/svbrdf.py:15-83) on the fused kernel.

Same interface as the reference class: ``SvbrdfOptim(device, renderer_obj)``,
``init_from_tex``, ``init_from_const``, ``init_from_randn``, ``load_targets`` and
``optim(epochs, lr, svbrdf_obj, optim_light)``.

``optim`` runs the loop body of src/svbrdf.py:56-71 (render of clamp(textures, -1, 1),
image loss, hand-written adjoint and Adam(lr, betas=(0.9, 0.999))) as one fused pass per
texel. By default (``kernel="batched"``) the material is a one-material plan of the batched
persistent kernels: the resident-state kernel runs up to 32 epochs per launch on state held
in shared memory, or, with ``optim_light``, the texel-pair kernels run one launch per epoch
with the light-power gradient reduced on the device. ``kernel="single"`` runs the
single-material kernel ``svbrdf_fused_step`` once per epoch instead (it also serves shapes
the batched kernels do not take: H*W not a multiple of 4). The per-epoch losses stay on the
device and are read once at the end (the reference reads them every epoch,
src/svbrdf.py:64-66). With ``graph=True`` the whole epoch loop is captured once into a CUDA
graph and replayed.

Setting ``fused=False`` gives the plain, unfused GPU form instead: the reference's own loop
(``eval`` -> loss -> ``backward`` -> ``torch.optim.Adam.step``) with the forward and
adjoint kernels behind ``torch.autograd``.
"""
from __future__ import annotations

import pathlib
from datetime import datetime

import torch

from . import _native as N

LOSS_KINDS = {"mse": 0, "log1p": 1, "log1p_pre": 2}


class SvbrdfOptim:
    def __init__(self, device, renderer_obj, loss="mse", fused=True, graph=False, save_process=False,
                 descriptor=None, descriptor_weight=0.1, kernel="batched"):
        self.device = torch.device(device)
        # optional descriptor (VGG-feature) term, e.g. descriptor.VGGDescriptor; like the
        # reference's loss + 0.1 * VGG loss (src/materialgan.py:139-146) it needs the renders,
        # so it runs the unfused form
        self.descriptor = descriptor
        self.descriptor_weight = float(descriptor_weight)
        if descriptor is not None:
            fused = False
        self.eps = 1e-4
        self.renderer_obj = renderer_obj
        self.res = renderer_obj.res
        if loss not in ("mse", "log1p"):
            raise ValueError("loss must be 'mse' or 'log1p'")
        self.loss = loss
        self.fused = fused
        if kernel not in ("batched", "single"):
            raise ValueError("kernel must be 'batched' or 'single'")
        self.kernel = kernel
        self.graph = graph
        self.save_process = save_process
        self.loss_image_list = []

    # ---- init_from_* : src/svbrdf.py:20-39 ----
    def _leaf(self, t):
        return t.detach().to(self.device, torch.float32).contiguous().requires_grad_(True)

    def init_from_tex(self, textures):
        self.textures = self._leaf(textures)

    def init_from_const(self, dif=0.5, spe=0.04, rgh=0.2):
        r = self.res
        normal = torch.zeros(1, 2, r, r, device=self.device)
        diffuse = torch.ones(1, 3, r, r, device=self.device) * dif * 2 - 1
        specular = torch.ones(1, 3, r, r, device=self.device) * spe * 2 - 1
        roughness = torch.ones(1, 1, r, r, device=self.device) * rgh * 2 - 1
        self.textures = self._leaf(torch.cat((diffuse, normal, roughness, specular), 1))

    def init_from_randn(self, dif=0.5, spe=0.04, rgh=0.2):
        r = self.res
        normal = (torch.randn(1, 2, r, r, device=self.device) / 4).clamp(-1, 1)
        diffuse = (torch.randn(1, 3, r, r, device=self.device) / 8 + dif).clamp(0, 1) * 2 - 1
        specular = (torch.randn(1, 3, r, r, device=self.device) / 32 + spe).clamp(0, 1) * 2 - 1
        roughness = (torch.randn(1, 1, r, r, device=self.device) / 16 + rgh).clamp(0, 1) * 2 - 1
        self.textures = self._leaf(torch.cat((diffuse, normal, roughness, specular), 1))

    def load_targets(self, targets):
        self.targets = targets.to(self.device, torch.float32).contiguous()
        if self.descriptor is not None:
            self.descriptor.load(self.targets)

    # ---- checkpoints: FP32 maps, the last call's Adam moments and step, the light -------
    # The reference keeps 8-bit PNG maps as its only per-pixel checkpoint
    # (src/svbrdf.py:74-83) and resumes by reloading them; these keep full precision.
    def state_dict(self) -> dict:
        return _optimiser_state(self)

    def load_state_dict(self, st: dict):
        """Restore the maps (and, when present, the last call's moments and the optimised
        light). The next ``optim`` call starts a fresh Adam from these maps, as the
        reference's does from reloaded maps."""
        self.textures = self._leaf(st["textures"])
        self._step = int(st.get("step", 0))
        self.loss_image_list = list(st.get("loss_image_list", []))
        for k in ("exp_avg", "exp_avg_sq", "light_pow", "light_exp_avg", "light_exp_avg_sq"):
            if k in st:
                setattr(self, k, st[k].to(self.device))
        if "light_pow" in st:
            self.renderer_obj.update_light(st["light_pow"].to(self.device))

    def save(self, path):
        torch.save(self.state_dict(), path)

    def load(self, path):
        self.load_state_dict(torch.load(path, map_location=self.device))

    def gradient(self, parameters):
        """The reference's helper (src/optimization.py:17-23): leaves that require grad."""
        if isinstance(parameters, list):
            return [p.detach().requires_grad_(True) for p in parameters]
        return parameters.detach().requires_grad_(True)

    def compute_image_loss(self, predicts):
        """src/optimization.py:28-29 (MSE), or the log(1+x) L2 loss."""
        if self.loss == "mse":
            return torch.nn.functional.mse_loss(predicts, self.targets)
        return torch.nn.functional.mse_loss(torch.log1p(predicts), torch.log1p(self.targets))

    # ---- optim : src/svbrdf.py:44-83 ----
    def optim(self, epochs, lr, svbrdf_obj=None, optim_light=False):
        if self.fused:
            return self._optim_fused(epochs, lr, svbrdf_obj, optim_light)
        return self._optim_plain(epochs, lr, svbrdf_obj, optim_light)

    def _light_tensor(self, svbrdf_obj):
        if svbrdf_obj is not None and hasattr(svbrdf_obj, "cl"):
            lp = svbrdf_obj.cl[2]
        else:
            lp = self.renderer_obj.light_pow
        return lp

    def _save_dir(self, svbrdf_obj):
        if not self.save_process or svbrdf_obj is None or not hasattr(svbrdf_obj, "optimize_dir"):
            return None
        stamp = str(datetime.now()).replace(" ", "-").replace(":", "-").replace(".", "-")
        d = pathlib.Path(svbrdf_obj.optimize_dir) / "tmp" / stamp
        d.mkdir(parents=True, exist_ok=True)
        return d

    def _maybe_save(self, tmp_dir, epoch, epochs, svbrdf_obj):
        # save points of src/svbrdf.py:74-83 (textures and re-renders; no loss plot)
        if tmp_dir is None or not ((epoch + 1) % 100 == 0 or epoch == 0 or epoch == epochs - 1):
            return
        d = tmp_dir / f"{epoch + 1}"
        d.mkdir(parents=True, exist_ok=True)
        with torch.no_grad():
            tex = self.textures.detach().clamp(-1, 1)
            if hasattr(svbrdf_obj, "save_textures_th"):
                svbrdf_obj.save_textures_th(tex, d)
            if hasattr(svbrdf_obj, "save_images_th"):
                svbrdf_obj.save_images_th(self.renderer_obj.eval(tex), d)

    def _optim_plain(self, epochs, lr, svbrdf_obj, optim_light):
        params = [self.textures]
        if optim_light:
            lp = self._light_tensor(svbrdf_obj)
            lp = lp.detach().to(self.device, torch.float32).clone().requires_grad_(True)
            if svbrdf_obj is not None and hasattr(svbrdf_obj, "cl"):
                svbrdf_obj.cl[2] = lp
            params.append(lp)
        self.optimizer = torch.optim.Adam(params, lr=lr, betas=(0.9, 0.999))
        tmp_dir = self._save_dir(svbrdf_obj)
        losses = []
        for epoch in range(epochs):
            if optim_light:
                self.renderer_obj.update_light(params[1])
            rendereds = self.renderer_obj.eval(self.textures.clamp(-1, 1))
            loss = self.compute_image_loss(rendereds)
            losses.append(loss.detach())
            if self.descriptor is not None:
                from .descriptor import descriptor_term

                loss = loss + self.descriptor_weight * descriptor_term(rendereds, self.descriptor)
            self.optimizer.zero_grad()
            loss.backward()
            self.optimizer.step()
            self._maybe_save(tmp_dir, epoch, epochs, svbrdf_obj)
        self.loss_image_list = torch.stack(losses).tolist() if losses else []
        st = self.optimizer.state[self.textures]
        self.exp_avg, self.exp_avg_sq = st.get("exp_avg"), st.get("exp_avg_sq")

    def _optim_fused(self, epochs, lr, svbrdf_obj, optim_light):
        tex = self.textures.detach()
        if self.kernel == "batched" and tex.shape[2] * tex.shape[3] % 4 == 0 and tex.data_ptr() % 16 == 0:
            return self._optim_batched(epochs, lr, svbrdf_obj, optim_light)
        return self._optim_single(epochs, lr, svbrdf_obj, optim_light)

    def _optim_batched(self, epochs, lr, svbrdf_obj, optim_light):
        """The epoch loop as a one-material plan of the batched persistent kernels."""
        from .batched import BatchedOptim, CANDIDATES
        from .scenes import Scene

        r = self.renderer_obj
        tex = self.textures.detach()  # same storage: the kernels update the leaf in place
        _, _, H, W = tex.shape
        lp = self._light_tensor(svbrdf_obj)
        sc = Scene(res=H, size=float(r.size), camera_pos=r._cam, light_pos=r._lit,
                   light_pow=lp.detach().to(self.device, torch.float32), gt=None, targets=self.targets, init=tex)
        n = max(epochs, 1)
        # A repeated call on the same maps, targets and settings reuses the previous call's plan,
        # buffers and captured graph; every call still starts a fresh Adam (src/svbrdf.py:48-52).
        key = (tex.data_ptr(), tuple(tex.shape), self.targets.data_ptr(), tuple(self.targets.shape), float(lr),
               self.loss, bool(optim_light), n, r._cam.data_ptr(), r._lit.data_ptr(), float(r.size))
        b = self._batched if getattr(self, "_batched_key", None) == key else None
        if b is not None:  # the light may have changed since (update_light, or the last call's optim_light)
            b.lpow0[0].copy_(sc.light_pow)
            b.lpow[0].copy_(sc.light_pow)
            b.prepare(new_targets=False)
        else:
            # the texel-pair kernels (the resident-state one first) suit one material; the
            # tuner's pick is cached per shape and library build
            cands = [c for c in CANDIDATES if c[0] in (2, 3)]
            b = BatchedOptim([sc], lr=lr, loss=self.loss, device=self.device, hist_len=n, optim_light=optim_light,
                             adopt_maps=True, candidates=cands)
            self._batched, self._batched_key = b, key
        tmp_dir = self._save_dir(svbrdf_obj)
        if tmp_dir is None:
            if epochs > 0:
                if self.graph:
                    b.run(epochs)
                else:
                    b._launch(b.plan_host, b.plan_dev, b.ws, b.step_dev, b.loss_hist, epochs)
                    b.step_count += epochs
        else:
            # save points of src/svbrdf.py:74-83: run to each one, then save
            done = 0
            for e in range(epochs):
                if (e + 1) % 100 == 0 or e == 0 or e == epochs - 1:
                    b._launch(b.plan_host, b.plan_dev, b.ws, b.step_dev, b.loss_hist, e + 1 - done)
                    b.step_count += e + 1 - done
                    done = e + 1
                    self._maybe_save(tmp_dir, e, epochs, svbrdf_obj)
        self.exp_avg, self.exp_avg_sq = b.m1[0], b.m2[0]
        self._step = epochs
        self.loss_image_list = b.loss_hist[:epochs, 0].tolist()
        b.check()
        if optim_light:
            lp_dev = b.lpow[0]
            with torch.no_grad():
                if svbrdf_obj is not None and hasattr(svbrdf_obj, "cl"):
                    svbrdf_obj.cl[2] = lp_dev.clone().requires_grad_(True)
                r.update_light(lp_dev.clone())
            self.light_exp_avg, self.light_exp_avg_sq = b.lstate[0][:3].clone(), b.lstate[0][3:].clone()
            self.light_pow = lp_dev

    def _optim_single(self, epochs, lr, svbrdf_obj, optim_light):
        L = N.lib()
        r = self.renderer_obj
        tex = self.textures.detach()  # same storage: the kernel updates the leaf in place
        # every call starts a fresh Adam, as the reference creates one per call (src/svbrdf.py:48-52)
        self.exp_avg = torch.zeros_like(tex)
        self.exp_avg_sq = torch.zeros_like(tex)
        self._step = 0
        targets = self.targets
        kind = LOSS_KINDS[self.loss]
        if self.loss == "log1p":
            targets = torch.log1p(self.targets)  # constant over the run: transform once
            kind = LOSS_KINDS["log1p_pre"]
        lp = self._light_tensor(svbrdf_obj)
        lp_dev = lp.detach().to(self.device, torch.float32).contiguous().clone()
        lstate = torch.zeros(6, device=self.device, dtype=torch.float32) if optim_light else None
        ws = torch.zeros(int(L.svbrdf_workspace_bytes()), dtype=torch.uint8, device=self.device)
        losses = torch.zeros(max(epochs, 1), device=self.device, dtype=torch.float32)
        _, _, H, W = tex.shape
        V = r.n_of_imgs
        tmp_dir = self._save_dir(svbrdf_obj)

        def launch(step, loss_slot):
            N.check(L.svbrdf_fused_step(tex.data_ptr(), self.exp_avg.data_ptr(), self.exp_avg_sq.data_ptr(),
                                        targets.data_ptr(), r._cam.data_ptr(), r._lit.data_ptr(),
                                        lp_dev.data_ptr(), N.ptr(lstate), V, H, W, float(r.size), kind, step,
                                        float(lr), 0.9, 0.999, 1e-8, losses.data_ptr() + 4 * loss_slot,
                                        ws.data_ptr(), ws.numel(), N.stream_handle(self.device)))

        if self.graph and tmp_dir is None and epochs > 1:
            # Warm once outside capture (occupancy queries), then undo its effect by restarting
            # from a snapshot so the captured run is the whole trajectory.
            snap = [tex.clone(), self.exp_avg.clone(), self.exp_avg_sq.clone(), lp_dev.clone()]
            if lstate is not None:
                snap.append(lstate.clone())
            launch(1, 0)
            tex.copy_(snap[0]); self.exp_avg.copy_(snap[1]); self.exp_avg_sq.copy_(snap[2]); lp_dev.copy_(snap[3])
            if lstate is not None:
                lstate.copy_(snap[4])
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                for e in range(epochs):
                    launch(e + 1, e)
            g.replay()
            self._graph = g
        else:
            for e in range(epochs):
                launch(e + 1, e)
                if tmp_dir is not None:
                    self._maybe_save(tmp_dir, e, epochs, svbrdf_obj)
        self._step = epochs
        self.loss_image_list = losses[:epochs].tolist()
        if optim_light:
            with torch.no_grad():
                if svbrdf_obj is not None and hasattr(svbrdf_obj, "cl"):
                    svbrdf_obj.cl[2] = lp_dev.clone().requires_grad_(True)
                r.update_light(lp_dev.clone())
            self.light_exp_avg, self.light_exp_avg_sq = lstate[:3].clone(), lstate[3:].clone()
        self.light_pow = lp_dev


def load_texture_maps(textures_dir, res=None, device="cpu") -> torch.Tensor:
    """[1, 9, H, W] parameters in [-1, 1] from nom/dif/spe/rgh.png (src/svbrdf.py:150-166),
    resized to res x res (None: the files' own size)."""
    from .imageio import imread

    d = pathlib.Path(textures_dir)
    dim = (res, res) if res is not None else None
    normal = imread(d / "nom.png", "normal", dim)
    diffuse = imread(d / "dif.png", "srgb", dim)
    specular = imread(d / "spe.png", "srgb", dim)
    roughness = imread(d / "rgh.png", "rough", dim)
    t = lambda a: torch.from_numpy(a).to(device)
    return torch.cat((t(diffuse * 2 - 1).permute(2, 0, 1).unsqueeze(0),
                      t(normal).permute(2, 0, 1).unsqueeze(0)[:, :2],
                      t(roughness * 2 - 1).unsqueeze(0).unsqueeze(0),
                      t(specular * 2 - 1).permute(2, 0, 1).unsqueeze(0)), 1)


def _optimiser_state(o) -> dict:
    st = {"textures": o.textures.detach().clone(), "step": int(getattr(o, "_step", 0)),
          "loss_image_list": list(getattr(o, "loss_image_list", []))}
    for k in ("exp_avg", "exp_avg_sq", "light_pow", "light_exp_avg", "light_exp_avg_sq"):
        v = getattr(o, k, None)
        if isinstance(v, torch.Tensor):
            st[k] = v.detach().clone()
    return st


class SvbrdfIO:
    """Scene and map I/O of the reference (src/svbrdf.py:86-221), on the package's own PNG codec.

    JSON keys (all optional, paths relative to the JSON file): reference_dir, target_dir,
    optimize_dir, rerender_dir, im_size (cm), idx (view ids), camera_pos, light_pos,
    light_pow. ``cl = [camera_pos[idx], light_pos[idx], light_pow]`` as FP32 tensors on
    ``device`` (src/svbrdf.py:134-146). Errors raise instead of printing and exiting.
    """

    def __init__(self, json_dir, device):
        import json

        self.device = torch.device(device)
        json_dir = pathlib.Path(json_dir)
        if not json_dir.exists():
            raise FileNotFoundError(f"{json_dir} does not exist")
        data = json.loads(json_dir.read_text())
        for key in ("reference_dir", "target_dir", "optimize_dir", "rerender_dir"):
            if key in data:
                setattr(self, key, json_dir.parent / data[key])
        if "im_size" in data:
            self.im_size = data["im_size"]
        if "idx" in data:
            self.idx = list(data["idx"])
            self.n_of_imgs = len(self.idx)
        for key in ("camera_pos", "light_pos"):
            if key in data:
                setattr(self, key, data[key])
        if "light_pow" in data:
            self.light_pow = data["light_pow"]
            self.load_calibration_th()

    def np_to_th(self, arr):
        return torch.from_numpy(arr).to(self.device)

    def th_to_np(self, arr):
        return arr.detach().cpu().numpy()

    def reconstruct_normal(self, texture):
        """Unit normals from the stored xy (src/svbrdf.py:126-132)."""
        return self._normal3(texture)

    def load_calibration_th(self):
        import numpy as np

        cam = np.asarray(self.camera_pos, dtype=np.float32)[self.idx, :]
        lit = np.asarray(self.light_pos, dtype=np.float32)[self.idx, :]
        pw = np.asarray(self.light_pow, dtype=np.float32)
        self.cl = [torch.from_numpy(cam).to(self.device), torch.from_numpy(lit).to(self.device),
                   torch.from_numpy(pw).to(self.device)]

    def load_textures_th(self, textures_dir, res):
        """[1, 9, res, res] in [-1, 1] from nom/dif/spe/rgh.png (src/svbrdf.py:150-166)."""
        return load_texture_maps(textures_dir, res, self.device)

    @staticmethod
    def _normal3(t2):
        nx = t2[:, 0].clamp(-1, 1)
        ny = t2[:, 1].clamp(-1, 1)
        nz = (1 - (nx ** 2 + ny ** 2).clamp(0, 1)).sqrt()
        n = torch.stack((nx, ny, nz), 1)
        return n / n.norm(2.0, 1, keepdim=True)

    def save_textures_th(self, textures_th, textures_dir):
        """nom/dif/spe/rgh.png from [1, 9, H, W], and their tex.png mosaic (src/svbrdf.py:168-189)."""
        from .imageio import imwrite, tex4to1

        d = pathlib.Path(textures_dir)
        d.mkdir(parents=True, exist_ok=True)
        t = textures_th.detach()
        np_ = lambda x: x.squeeze(0).permute(1, 2, 0).cpu().numpy()
        imwrite(np_(self._normal3(t[:, 3:5])), d / "nom.png", "normal")
        imwrite(np_((t[:, 0:3] + 1) / 2), d / "dif.png", "srgb")
        imwrite(np_((t[:, 6:9] + 1) / 2), d / "spe.png", "srgb")
        imwrite(((t[0, 5] + 1) / 2).cpu().numpy(), d / "rgh.png", "rough")
        tex4to1(d)

    def load_images_th(self, images_dir, res=256):
        """[n, 3, res, res] from {idx:02d}.png (src/svbrdf.py:191-204)."""
        from .imageio import imread

        d = pathlib.Path(images_dir)
        out = torch.zeros(self.n_of_imgs, 3, res, res, device=self.device)
        for i, idx in enumerate(self.idx):
            out[i] = torch.from_numpy(imread(d / f"{idx:02d}.png", "srgb", (res, res))).permute(2, 0, 1)
        return out

    def save_images_th(self, images_th, images_dir):
        """{idx:02d}.png per view, and with nine views their all.png mosaic (src/svbrdf.py:206-221)."""
        from .imageio import img9to1, imwrite

        d = pathlib.Path(images_dir)
        d.mkdir(parents=True, exist_ok=True)
        if images_th.shape[0] != self.n_of_imgs:
            raise ValueError(f"expected {self.n_of_imgs} images, got {images_th.shape[0]}")
        for i, idx in enumerate(self.idx):
            imwrite(images_th[i].detach().permute(1, 2, 0).cpu().numpy(), d / f"{idx:02d}.png", "srgb")
        if self.n_of_imgs == 9:
            img9to1(d, [f"{idx:02d}.png" for idx in self.idx])
