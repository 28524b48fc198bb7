"""Novel-view rendering of a material under an environment map.

The reference renders the video of an optimised material with Mitsuba 3 on the CPU
(``MitsubaRender``, src/mitsubarender.py:7-105, driven by ``render_envmap``,
src/scripts.py:44-59): a textured rectangle under ``fig/ennis.exr`` with the ``direct``
integrator at 256 samples per pixel. ``EnvmapRenderer`` keeps that interface and renders the
same scene with one CUDA kernel (``svbrdf_envmap_render``): direct illumination with one
importance-sampled environment sample and one BSDF sample per camera sample, combined by the
power heuristic. The material is a normal map over a 0.5 / 0.5 blend of a GGX conductor and a
diffuse lobe, read from the stored texture parameters the way the reference's PNG maps
encode them (sRGB values for diffuse, specular and roughness, raw normals).

``fig/ennis.exr`` is not in the reference repository, so ``synthetic_envmap`` makes a seeded
stand-in (sky gradient, ground, a few bright lobes). Any [He, We, 3] linear-radiance array,
or a lat-long OpenEXR file (``imageio.exr_read``), can be passed instead.
"""
from __future__ import annotations

import pathlib
from typing import List, Optional, Sequence

import numpy as np
import torch

from . import _native as N


def synthetic_envmap(he: int = 64, we: int = 128, seed: int = 0) -> np.ndarray:
    """A seeded lat-long environment [he, we, 3] (linear radiance, FP32): a blue sky that
    brightens toward the horizon, a dim ground, and three bright lobes ("sun" and windows)."""
    g = np.random.default_rng(seed)
    v = (np.arange(he) + 0.5) / he  # 0 at the zenith
    u = (np.arange(we) + 0.5) / we
    theta = np.pi * v[:, None]
    phi = 2.0 * np.pi * u[None, :]
    d = np.stack([np.sin(theta) * np.sin(phi), np.cos(theta) * np.ones_like(phi), -np.sin(theta) * np.cos(phi)], -1)
    up = np.clip(d[..., 1], 0.0, 1.0)
    sky = np.array([0.35, 0.5, 0.9]) * (0.4 + 0.6 * (1.0 - up))[..., None]
    ground = np.array([0.25, 0.22, 0.2]) * np.ones_like(up)[..., None]
    env = np.where((d[..., 1] >= 0.0)[..., None], sky, ground)
    for k in range(3):
        c = g.normal(size=3)
        c[1] = abs(c[1]) + 0.3
        c /= np.linalg.norm(c)
        sharp = 40.0 + 160.0 * g.random()
        power = (8.0 if k == 0 else 2.0) * (1.0 + g.random())
        lobe = np.exp(sharp * (np.clip((d * c).sum(-1), -1.0, 1.0) - 1.0))
        env = env + power * lobe[..., None] * np.array([1.0, 0.95, 0.85])
    return env.astype(np.float32)


def env_distribution(env: np.ndarray):
    """Importance-sampling tables of a lat-long map: weight luminance x sin(theta) per texel,
    (row_cdf [He+1], row_pdf [He], col_cdf [He, We+1], col_pdf [He, We]) as FP32 arrays. The
    CPU oracle draws from the same arrays, so both make the same discrete choices."""
    e = np.asarray(env, dtype=np.float64)
    he, we = e.shape[:2]
    lum = 0.2126 * e[..., 0] + 0.7152 * e[..., 1] + 0.0722 * e[..., 2]
    w = np.maximum(lum, 0.0) * np.sin(np.pi * (np.arange(he) + 0.5) / he)[:, None]
    rows = w.sum(1)
    total = rows.sum()
    if total <= 0:
        raise ValueError("environment map has no energy")
    row_pdf = rows / total
    row_cdf = np.concatenate([[0.0], np.cumsum(row_pdf)])
    row_cdf[-1] = 1.0
    col_pdf = np.where(rows[:, None] > 0, w / np.where(rows[:, None] > 0, rows[:, None], 1.0), 1.0 / we)
    col_cdf = np.concatenate([np.zeros((he, 1)), np.cumsum(col_pdf, 1)], 1)
    col_cdf[:, -1] = 1.0
    f = lambda a: np.ascontiguousarray(a, dtype=np.float32)
    return f(row_cdf), f(row_pdf), f(col_cdf), f(col_pdf)


def video_angles(n: int = 59) -> np.ndarray:
    """The reference's sweep: -cos(linspace(0, pi, 59)) x 40 degrees (src/scripts.py:49)."""
    return -np.cos(np.linspace(0, np.pi, n)) * 40


class EnvmapRenderer:
    """``MitsubaRender``'s interface (src/mitsubarender.py:7-19) on the GPU.

    ``EnvmapRenderer(im_size, envmap, textures)``: ``im_size`` [res, res]; ``envmap`` a
    [He, We, 3] linear-radiance array or the path of a lat-long OpenEXR file (None:
    ``synthetic_envmap()``); ``textures`` the
    material's [9, H, W] (or [1, 9, H, W]) parameters in [-1, 1], the layout the optimisers
    produce. ``render(angle, light_intensity)`` returns the [res, res, 3] image clipped to
    [0, 1] and raised to 1/2.2, as the reference's does."""

    def __init__(self, im_size: Sequence[int], envmap: Optional[np.ndarray], textures: torch.Tensor,
                 device="cuda", spp: int = 256, seed: int = 0):
        if im_size[0] != im_size[1]:
            raise ValueError("square images only (the reference renders [res, res])")
        self.res = int(im_size[0])
        self.device = torch.device(device)
        self.spp, self.seed = int(spp), int(seed)
        self.load_envmap(synthetic_envmap() if envmap is None else envmap)
        self.load_texturemaps(textures)

    def load_envmap(self, env):
        """A [He, We, 3] linear-radiance array, or the path of a lat-long OpenEXR file."""
        if isinstance(env, (str, pathlib.Path)):
            from .imageio import exr_read

            env = exr_read(env)
        env = np.ascontiguousarray(env, dtype=np.float32)
        if env.ndim != 3 or env.shape[2] != 3:
            raise ValueError("envmap must be [He, We, 3]")
        self.env_np = env
        self.tables_np = env_distribution(env)
        self.env = torch.from_numpy(env).to(self.device)
        self.tables = [torch.from_numpy(t).to(self.device) for t in self.tables_np]

    def load_texturemaps(self, textures: torch.Tensor):
        t = textures.detach()
        if t.dim() == 4:
            t = t[0]
        if t.shape[0] != 9:
            raise ValueError("textures must be [9, H, W]")
        self.textures = t.to(self.device, torch.float32).contiguous()

    def render_device(self, angle: float, light_intensity: float = 1.0, out: Optional[torch.Tensor] = None):
        """The image as a [res, res, 3] FP32 device tensor (no host copy)."""
        if out is None:
            out = torch.empty(self.res, self.res, 3, device=self.device, dtype=torch.float32)
        L = N.lib()
        _, h, w = self.textures.shape
        he, we = self.env.shape[:2]
        rc, rp, cc, cp = self.tables
        N.check(L.svbrdf_envmap_render(self.textures.data_ptr(), h, w, self.env.data_ptr(), he, we, rc.data_ptr(),
                                       rp.data_ptr(), cc.data_ptr(), cp.data_ptr(), out.data_ptr(), self.res,
                                       float(angle), float(light_intensity), self.spp, self.seed & 0xFFFFFFFF,
                                       N.stream_handle(self.device)))
        return out

    def render(self, angle: float, light_intensity: float = 1.0) -> np.ndarray:
        return self.render_device(angle, light_intensity).cpu().numpy()

    def render_video(self, n: int = 59, light_intensity: float = 0.5) -> List[np.ndarray]:
        """The frames of ``render_envmap`` (src/scripts.py:44-59): n angles forward, then the
        same frames backward (without the two ends), at light intensity 0.5."""
        frames = [self.render_device(a, light_intensity) for a in video_angles(n)]
        frames = frames + frames[-2:0:-1]
        return [f.cpu().numpy() for f in frames]
