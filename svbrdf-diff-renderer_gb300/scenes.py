"""Seeded synthetic flash-lit scenes that stand in for captured 9-view datasets.

The reference ships no datasets for this path (its captured photos are not part of the
repository), so the workloads here are generated. They keep the shape of the reference's
captures: co-located camera and flash on a 3x3 grid above a flat sample
(data/random/render.json:5-25, src/capture.py:63-73), light power 1500 per channel
(src/capture.py:72) and maps stored in the reference's texture space, where a PNG value
x in [0, 1] becomes the parameter 2x - 1 (src/svbrdf.py:23-30, 160-166).

Material maps, in texture space [0, 1]:

* diffuse RGB in [0.05, 0.9], specular RGB in [0.02, 0.5], roughness in [0.1, 0.9]: each
  channel is seeded white noise, smoothed by a Gaussian of sigma 4 px and rescaled
  affinely to the range;
* normal: a smoothed height field h gives n ~ (-dh/dx, -dh/dy, 1), scaled so that the
  steepest texel is tilted 30 degrees from +z; channels 3:5 hold (nx, ny) of the unit normal.

Material i draws from ``torch.Generator().manual_seed(1000 + i)``. Scene-level draws
(resolutions, view counts and positions of the batched workload) use seed 0.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Callable, List, Optional

import torch

LIGHT_POW = 1500.0
GRID_SIZE_CM = 17.0


@dataclass
class Scene:
    """One material and its views. Tensors are FP32; ``textures`` is ``[1, 9, res, res]``."""

    res: int
    size: float
    camera_pos: torch.Tensor  # [V, 3] cm
    light_pos: torch.Tensor   # [V, 3] cm
    light_pow: torch.Tensor   # [3]
    gt: torch.Tensor          # ground-truth textures [1, 9, res, res] in [-1, 1]
    targets: Optional[torch.Tensor] = None  # [V, 3, res, res] in [0, 1]
    init: Optional[torch.Tensor] = None     # initial textures [1, 9, res, res]
    seed: int = 0
    meta: dict = field(default_factory=dict)

    @property
    def n_views(self) -> int:
        return int(self.camera_pos.shape[0])

    @property
    def cl(self) -> List[torch.Tensor]:
        """The reference's ``cl = [camera_pos, light_pos, light_pow]`` list (src/svbrdf.py:146)."""
        return [self.camera_pos, self.light_pos, self.light_pow]


def _gauss_kernel(sigma: float) -> torch.Tensor:
    r = int(math.ceil(3 * sigma))
    x = torch.arange(-r, r + 1, dtype=torch.float32)
    k = torch.exp(-0.5 * (x / sigma) ** 2)
    return k / k.sum()


def smooth_field(noise: torch.Tensor, sigma: float = 4.0) -> torch.Tensor:
    """Separable Gaussian blur of ``noise[C, H, W]`` with wrap-around borders."""
    k = _gauss_kernel(sigma).to(noise.device)
    r = (k.numel() - 1) // 2
    c, h, w = noise.shape
    x = noise.unsqueeze(1)  # [C,1,H,W]
    x = torch.nn.functional.pad(x, (r, r, 0, 0), mode="circular")
    x = torch.nn.functional.conv2d(x, k.view(1, 1, 1, -1))
    x = torch.nn.functional.pad(x, (0, 0, r, r), mode="circular")
    x = torch.nn.functional.conv2d(x, k.view(1, 1, -1, 1))
    return x.squeeze(1)


def _rescale(f: torch.Tensor, lo: float, hi: float) -> torch.Tensor:
    fmin = f.amin(dim=(-2, -1), keepdim=True)
    fmax = f.amax(dim=(-2, -1), keepdim=True)
    return lo + (f - fmin) / (fmax - fmin).clamp_min(1e-12) * (hi - lo)


def make_material(res: int, seed: int, device="cpu", max_tilt_deg: float = 30.0) -> torch.Tensor:
    """Ground-truth textures ``[1, 9, res, res]`` (parameter space [-1, 1]) for one material."""
    g = torch.Generator().manual_seed(seed)
    noise = torch.randn(8, res, res, generator=g).to(device)
    f = smooth_field(noise)
    dif = _rescale(f[0:3], 0.05, 0.9)
    spe = _rescale(f[3:6], 0.02, 0.5)
    rgh = _rescale(f[6:7], 0.1, 0.9)
    hgt = f[7]
    dx = 0.5 * (torch.roll(hgt, -1, 1) - torch.roll(hgt, 1, 1))
    dy = 0.5 * (torch.roll(hgt, -1, 0) - torch.roll(hgt, 1, 0))
    slope = torch.sqrt(dx * dx + dy * dy).max().clamp_min(1e-12)
    scale = math.tan(math.radians(max_tilt_deg)) / slope
    nx, ny = -dx * scale, -dy * scale
    inv = torch.rsqrt(nx * nx + ny * ny + 1.0)
    tex = torch.cat((dif * 2 - 1, (nx * inv).unsqueeze(0), (ny * inv).unsqueeze(0),
                     rgh * 2 - 1, spe * 2 - 1), 0)
    return tex.unsqueeze(0).contiguous()


def const_init(res: int, dif=0.5, spe=0.04, rgh=0.5, device="cpu") -> torch.Tensor:
    """Constant initial maps (the layout of src/svbrdf.py:23-30) with a flat normal."""
    t = torch.empty(1, 9, res, res, device=device)
    t[:, 0:3] = dif * 2 - 1
    t[:, 3:5] = 0.0
    t[:, 5] = rgh * 2 - 1
    t[:, 6:9] = spe * 2 - 1
    return t


def grid_views(offset_cm: float = 6.0, height_cm: float = 30.0) -> torch.Tensor:
    """3x3 co-located flash grid in the row order of data/random/render.json:5-14."""
    pts = [[x, y, height_cm] for y in (offset_cm, 0.0, -offset_cm) for x in (-offset_cm, 0.0, offset_cm)]
    return torch.tensor(pts, dtype=torch.float32)


def random_views(n: int, g: torch.Generator, offset_cm: float = 8.0, zlo: float = 25.0, zhi: float = 35.0):
    xy = (torch.rand(n, 2, generator=g) * 2 - 1) * offset_cm
    z = zlo + torch.rand(n, 1, generator=g) * (zhi - zlo)
    return torch.cat((xy, z), 1).to(torch.float32)


RenderFn = Callable[[torch.Tensor, torch.Tensor, torch.Tensor, torch.Tensor, float], torch.Tensor]


def add_targets(scene: Scene, render_fn: RenderFn, noise_std: float = 0.01) -> Scene:
    """targets = clamp(render(gt) + N(0, noise_std), 0, 1); the noise uses the material seed."""
    img = render_fn(scene.gt, scene.camera_pos, scene.light_pos, scene.light_pow, scene.size)
    g = torch.Generator().manual_seed(scene.seed + 7777)
    noise = torch.randn(img.shape, generator=g).to(img.device) * noise_std
    scene.targets = (img + noise).clamp(0, 1).contiguous()
    return scene


def single_scene(res: int = 256, seed: int = 1000, device="cpu", render_fn: Optional[RenderFn] = None,
                 offset_cm: float = 6.0, height_cm: float = 30.0) -> Scene:
    """One material under the 3x3 co-located grid: the 256^2 and 1024^2 per-pixel workloads."""
    cam = grid_views(offset_cm, height_cm).to(device)
    sc = Scene(res=res, size=GRID_SIZE_CM, camera_pos=cam, light_pos=cam.clone(),
               light_pow=torch.full((3,), LIGHT_POW, device=device),
               gt=make_material(res, seed, device), seed=seed)
    sc.init = const_init(res, device=device)
    if render_fn is not None:
        add_targets(sc, render_fn)
    return sc


def batched_scenes(n: int = 64, resolutions=(256, 512, 1024), vmin: int = 5, vmax: int = 16,
                   device="cpu", render_fn: Optional[RenderFn] = None, scene_seed: int = 0,
                   colocated: bool = True) -> List[Scene]:
    """The uneven batched workload: ``n`` materials, resolution drawn from ``resolutions``,
    view counts uniform in [vmin, vmax], flash positions uniform within +-8 cm at 25-35 cm."""
    g = torch.Generator().manual_seed(scene_seed)
    out = []
    for i in range(n):
        res = int(resolutions[int(torch.randint(len(resolutions), (1,), generator=g))])
        v = int(torch.randint(vmin, vmax + 1, (1,), generator=g))
        cam = random_views(v, g)
        lit = cam.clone() if colocated else random_views(v, g)
        sc = Scene(res=res, size=GRID_SIZE_CM, camera_pos=cam.to(device), light_pos=lit.to(device),
                   light_pow=torch.full((3,), LIGHT_POW, device=device),
                   gt=make_material(res, 1000 + i, device), seed=1000 + i)
        sc.init = const_init(res, device=device)
        if render_fn is not None:
            add_targets(sc, render_fn)
        out.append(sc)
    return out
