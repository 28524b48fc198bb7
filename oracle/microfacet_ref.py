"""CPU oracle for the flash-lit GGX/Cook-Torrance renderer and its per-pixel optimiser.

TEST INFRASTRUCTURE ONLY. Only the tests, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` import this module,
and only to check or time against it. The product path never calls it. There
is no CPU fallback in the product.

What it restates (files are cited by their path inside tflsguoyu/svbrdf-diff-renderer):

* ``render``: ``Microfacet.__init__`` / ``Microfacet.eval`` (src/microfacet.py:10-26, 84-120),
  with the helper terms ``GGX`` (:28-32), ``Fresnel`` (:43-45), ``Smith`` (:47-52),
  ``dot``/``normalize``/``get_dir`` (:54-62), ``reconstruct_normal`` (:64-70) and
  ``tex2map`` (:72-79). The op sequence is the reference's, which matters for FP32
  rounding, including the 3-channel expansion of the dot products and the eps placements.
* ``image_loss``: ``Optim.compute_image_loss`` (src/optimization.py:14, 28-29), which is
  ``nn.MSELoss`` (a mean over V*3*H*W). A second kind, ``"log1p"``, is the log(1+x) L2 loss
  of the per-pixel workloads: mean((log1p(render) - log1p(target))^2).
* ``optim_loop``: the loop body of ``SvbrdfOptim.optim`` (src/svbrdf.py:44-71). One
  ``torch.optim.Adam(lr, betas=(0.9, 0.999))`` is made once, then each epoch does
  eval(clamp(textures, -1, 1)), loss, zero_grad, backward, step. The optional learnable
  light power follows svbrdf.py:48-50, 58-59 and ``update_light`` (src/microfacet.py:81-82).
  The periodic PNG dumps (svbrdf.py:74-83) are host I/O and are left out.
* ``init_const``: ``SvbrdfOptim.init_from_const`` (src/svbrdf.py:23-30).

Every function takes a ``dtype``. FP32 reproduces the reference's own arithmetic; FP64
is the high-precision oracle that the FP32 results (the reference's and the CUDA
kernels') are both measured against.

Parity is pinned: ``tests/golden/make_golden.py`` imports the reference's own
``src/microfacet.py`` and ``src/svbrdf.py`` (I/O modules stubbed) and commits their
renders, autograd gradients and optimiser trajectories as fixtures; the CPU tests check
this module against them.
"""
from __future__ import annotations

import math

import torch

EPS = 1e-6  # Microfacet.eps (src/microfacet.py:14)


def pixel_positions(res: int, size: float, dtype=torch.float64) -> torch.Tensor:
    """Pixel-centre grid ``pos[3, res, res]`` of src/microfacet.py:16-19.

    ``x`` runs along the column index and ``y`` is flipped, so texel (i, j) sits at
    ``(((j+0.5)/res - 0.5)*size, -((i+0.5)/res - 0.5)*size, 0)``. The grid is built in
    FP32 like the reference and then cast, so both precisions share the same positions.
    """
    tmp = torch.arange(res, dtype=torch.float32)
    tmp = ((tmp + 0.5) / res - 0.5) * size
    x, y = torch.meshgrid(tmp, tmp, indexing="xy")
    pos = torch.stack((x, -y, torch.zeros_like(x)), 2).permute(2, 0, 1)
    return pos.to(dtype)


def _dot(a, b):
    # src/microfacet.py:54-55: channel sum, then expand to 3 channels
    return (a * b).sum(1, keepdim=True).expand(-1, 3, -1, -1)


def _normalize(vec):
    # src/microfacet.py:57-58
    return vec / vec.norm(2.0, 1, keepdim=True)


def _reconstruct_normal(t2):
    # src/microfacet.py:64-70
    nx = t2[:, 0, :, :].clamp(-1, 1)
    ny = t2[:, 1, :, :].clamp(-1, 1)
    nxy = (nx ** 2 + ny ** 2).clamp(0, 1 - EPS)
    nz = (1 - nxy).sqrt()
    return _normalize(torch.stack((nx, ny, nz), 1))


def _ggx(cos_h, alpha):
    # src/microfacet.py:28-32
    c2 = cos_h ** 2
    a2 = alpha ** 2
    den = c2 * a2 + (1 - c2)
    return a2 / (math.pi * den ** 2 + EPS)


def _fresnel(cos, specular):
    # src/microfacet.py:43-45 (spherical-Gaussian Schlick)
    sphg = torch.pow(2.0, ((-5.55473 * cos) - 6.98316) * cos)
    return specular + (1.0 - specular) * sphg


def _smith(n_dot_v, n_dot_l, alpha):
    # src/microfacet.py:47-52
    k = alpha * 0.5 + EPS

    def g1(c):
        return c / (c * (1.0 - k) + k)

    return g1(n_dot_v) * g1(n_dot_l)


def render(textures, camera_pos, light_pos, light_pow, size, dtype=torch.float32):
    """Render ``textures[1, 9, H, W]`` under V flash views -> ``[V, 3, H, W]``.

    Restates ``Microfacet(res, V, size, cl).eval(textures)`` (src/microfacet.py:10-26,
    84-120). ``camera_pos``/``light_pos`` are ``[V, 3]`` in cm, ``light_pow`` is ``[3]``.
    Channel layout of ``textures``: 0:3 diffuse, 3:5 normal xy, 5 roughness, 6:9 specular.
    Autograd flows to ``textures`` and, if it requires grad, ``light_pow``.
    """
    assert textures.dim() == 4 and textures.shape[0] == 1 and textures.shape[1] == 9
    assert textures.shape[2] == textures.shape[3]  # src/microfacet.py:85
    res = textures.shape[2]
    cam = camera_pos.to(dtype).unsqueeze(2).unsqueeze(3)
    lit = light_pos.to(dtype).unsqueeze(2).unsqueeze(3)
    lpow = light_pow.to(dtype).unsqueeze(0).unsqueeze(2).unsqueeze(3)
    return _render_at(textures, pixel_positions(res, size, dtype), cam, lit, lpow, dtype)


def texel_positions(idx, height, width, size):
    """FP32 pixel centres ``(px[n], py[n])`` of flat texel indices ``idx`` (row-major, H x W),
    computed as ``pixel_positions`` builds the grid (src/microfacet.py:16-19)."""
    idx = torch.as_tensor(idx, dtype=torch.int64)
    i = (idx // width).to(torch.float32)
    j = (idx % width).to(torch.float32)
    px = ((j + 0.5) / width - 0.5) * size
    py = -(((i + 0.5) / height - 0.5) * size)
    return px, py


def render_texels(t9, px, py, camera_pos, light_pos, light_pow, dtype=torch.float64):
    """Render ``n`` texels ``t9[9, n]`` at pixel centres ``(px[n], py[n])`` -> ``[V, 3, n]``.

    Rendered pixel (i, j) of src/microfacet.py:84-120 depends only on texel (i, j) and its
    position, so any set of texels can be rendered on its own: this is ``render`` on a
    1 x n strip with the strip's positions given instead of the regular grid (same op
    sequence). ``camera_pos``/``light_pos`` are ``[V, 3]`` (shared) or ``[V, 3, n]`` (per
    texel, for texels of different materials in one call), ``light_pow`` ``[3]`` or ``[3, n]``."""
    n = t9.shape[1]
    pos = torch.stack((px.to(torch.float32), py.to(torch.float32), torch.zeros(n)), 0).view(3, 1, n)
    cam = camera_pos.to(dtype)
    lit = light_pos.to(dtype)
    lpow = light_pow.to(dtype)
    cam = cam.view(*cam.shape[:2], 1, n) if cam.dim() == 3 else cam.unsqueeze(2).unsqueeze(3)
    lit = lit.view(*lit.shape[:2], 1, n) if lit.dim() == 3 else lit.unsqueeze(2).unsqueeze(3)
    lpow = lpow.view(1, 3, 1, n) if lpow.dim() == 2 else lpow.view(1, 3, 1, 1)
    out = _render_at(t9.reshape(1, 9, 1, n), pos.to(dtype), cam, lit, lpow, dtype)
    return out.reshape(-1, 3, n)


def _render_at(textures, pos3, cam4, lit4, lpow4, dtype):
    """src/microfacet.py:84-120 for textures ``[1, 9, H, W]`` at positions ``pos3[3, H, W]``;
    ``cam4``/``lit4`` broadcast to ``[V, 3, H, W]``, ``lpow4`` to ``[1, 3, H, W]``."""
    hh, ww = textures.shape[2], textures.shape[3]
    n = cam4.shape[0]
    t = textures.to(dtype)
    pos = pos3.to(dtype).unsqueeze(0).expand(n, -1, -1, -1)
    cam = cam4.expand(-1, -1, hh, ww)
    lit = lit4.expand(-1, -1, hh, ww)
    lpow = lpow4.expand(n, -1, hh, ww)

    # tex2map, src/microfacet.py:72-79
    diffuse = (((t[:, 0:3] + 1) / 2) ** 2.2).expand(n, -1, -1, -1)
    normal = _reconstruct_normal(t[:, 3:5]).expand(n, -1, -1, -1)
    rough = (((t[:, 5] + 1) / 2) ** 2.2).expand(n, 3, -1, -1)
    specular = (((t[:, 6:9] + 1) / 2) ** 2.2).expand(n, -1, -1, -1)

    # get_dir, src/microfacet.py:60-62, 91-93
    vv = cam - pos
    v = _normalize(vv)
    lv = lit - pos
    l = _normalize(lv)
    dist_l_sq = _dot(lv, lv)
    h = _normalize(l + v)

    n_dot_v = _dot(normal, v).clamp(min=0)
    n_dot_l = _dot(normal, l).clamp(min=0)
    n_dot_h = _dot(normal, h).clamp(min=0)
    v_dot_h = _dot(v, h).clamp(min=0)

    f1 = diffuse / math.pi
    f1 = f1 * (1 - specular)
    D = _ggx(n_dot_h, rough ** 2)
    F = _fresnel(v_dot_h, specular)
    G = _smith(n_dot_v, n_dot_l, rough ** 2)
    f2 = D * F * G / (4 * n_dot_v * n_dot_l + EPS)
    f = 1 * f1 + 1 * f2
    img = lpow * f * n_dot_l / dist_l_sq
    return img.clamp(EPS, 1) ** (1 / 2.2)


def image_loss(rendered, targets, kind="mse"):
    """``kind="mse"``: src/optimization.py:14,28-29. ``kind="log1p"``: log(1+x) L2."""
    if kind == "mse":
        return torch.nn.functional.mse_loss(rendered, targets.to(rendered.dtype))
    if kind == "log1p":
        return torch.nn.functional.mse_loss(torch.log1p(rendered), torch.log1p(targets.to(rendered.dtype)))
    raise ValueError(f"unknown loss kind {kind!r}")


def init_const(res, dif=0.5, spe=0.04, rgh=0.2, dtype=torch.float32):
    """``SvbrdfOptim.init_from_const`` (src/svbrdf.py:23-30): constant maps in [-1, 1]."""
    normal = torch.zeros(1, 2, res, res, dtype=dtype)
    diffuse = torch.ones(1, 3, res, res, dtype=dtype) * dif * 2 - 1
    specular = torch.ones(1, 3, res, res, dtype=dtype) * spe * 2 - 1
    roughness = torch.ones(1, 1, res, res, dtype=dtype) * rgh * 2 - 1
    return torch.cat((diffuse, normal, roughness, specular), 1)


def optim_loop(textures0, targets, camera_pos, light_pos, light_pow, size, epochs, lr,
               loss_kind="mse", optim_light=False, dtype=torch.float32):
    """The loop of ``SvbrdfOptim.optim`` (src/svbrdf.py:44-71), without the PNG dumps.

    Returns a dict with the final ``textures`` (unclamped leaf, like the reference's
    ``self.textures``), Adam's ``exp_avg``/``exp_avg_sq``, the per-epoch ``loss`` list and,
    with ``optim_light``, the final ``light_pow``.
    """
    tex = textures0.detach().to(dtype).clone().requires_grad_(True)
    params = [tex]
    lpow = light_pow.detach().to(dtype).clone()
    if optim_light:
        lpow.requires_grad_(True)
        params.append(lpow)
    opt = torch.optim.Adam(params, lr=lr, betas=(0.9, 0.999))
    losses = []
    tgt = targets.to(dtype)
    for _ in range(epochs):
        out = render(tex.clamp(-1, 1), camera_pos, light_pos, lpow, size, dtype)
        loss = image_loss(out, tgt, loss_kind)
        losses.append(float(loss.item()))
        opt.zero_grad()
        loss.backward()
        opt.step()
    st = opt.state[tex]
    res = {"textures": tex.detach(), "exp_avg": st["exp_avg"].detach(),
           "exp_avg_sq": st["exp_avg_sq"].detach(), "loss": losses}
    if optim_light:
        res["light_pow"] = lpow.detach()
    return res


def optim_texels(t9, px, py, targets, camera_pos, light_pos, light_pow, n_full, epochs, lr,
                 loss_kind="mse", dtype=torch.float64, view_mask=None):
    """``optim_loop`` (src/svbrdf.py:44-71) restricted to ``n`` texels.

    ``t9[9, n]`` are the texels' initial parameters at pixel centres ``(px, py)``,
    ``targets[V, 3, n]`` their targets, ``n_full`` the element count ``V*3*H*W`` of the whole
    material, which the reference's mean loss divides by. Each texel's render, gradient and
    Adam update (elementwise) depend on that texel alone, so its trajectory here is the one
    it follows in the full-material loop. Texels of several materials can share one call:
    per-texel views ``[V, 3, n]`` (see ``render_texels``), ``n_full`` per texel ``[n]``, and
    ``view_mask[V, n]`` (1 for a material's own views, 0 for padding up to the largest V).
    The summed loss is then the sum of the materials' losses, whose gradient at each texel
    is its own material's. Returns the final ``textures`` (unclamped), ``exp_avg``,
    ``exp_avg_sq`` (all ``[9, n]``) and ``sq_err[epochs, n]``: each texel's summed squared
    error per epoch (before that epoch's update), in the loss's units."""
    tex = t9.detach().to(dtype).clone().requires_grad_(True)
    opt = torch.optim.Adam([tex], lr=lr, betas=(0.9, 0.999))
    tgt = targets.to(dtype)
    if loss_kind == "log1p":
        tgt = torch.log1p(tgt)
    mask = None if view_mask is None else view_mask.to(dtype).unsqueeze(1)
    per_texel = torch.is_tensor(n_full) and n_full.dim() > 0
    inv_n = (1.0 / n_full.to(dtype)) if per_texel else None
    sq = []
    for _ in range(epochs):
        out = render_texels(tex.clamp(-1, 1), px, py, camera_pos, light_pos, light_pow, dtype)
        if loss_kind == "log1p":
            out = torch.log1p(out)
        e2 = (out - tgt) ** 2
        if mask is not None:
            e2 = e2 * mask
        sq.append(e2.detach().sum((0, 1)))
        loss = (e2 * inv_n).sum() if per_texel else e2.sum() / n_full
        opt.zero_grad()
        loss.backward()
        opt.step()
    st = opt.state[tex]
    return {"textures": tex.detach(), "exp_avg": st["exp_avg"].detach(), "exp_avg_sq": st["exp_avg_sq"].detach(),
            "sq_err": torch.stack(sq)}


def loss_texels(t9, px, py, targets, camera_pos, light_pos, light_pow, loss_kind="mse", dtype=torch.float64):
    """Summed squared error (the numerator of ``image_loss``) of ``n`` texels, FP64 sum."""
    out = render_texels(t9.clamp(-1, 1), px, py, camera_pos, light_pos, light_pow, dtype)
    tgt = targets.to(dtype)
    if loss_kind == "log1p":
        out, tgt = torch.log1p(out), torch.log1p(tgt)
    return float(((out - tgt) ** 2).sum(dtype=torch.float64))


def loss_and_grad(textures, targets, camera_pos, light_pos, light_pow, size, loss_kind="mse",
                  dtype=torch.float64, grad_light=False):
    """Loss and autograd gradient w.r.t. ``textures`` (and ``light_pow``) at ``dtype``."""
    tex = textures.detach().to(dtype).clone().requires_grad_(True)
    lp = light_pow.detach().to(dtype).clone().requires_grad_(grad_light)
    loss = image_loss(render(tex, camera_pos, light_pos, lp, size, dtype), targets, loss_kind)
    loss.backward()
    return float(loss.item()), tex.grad.detach(), (lp.grad.detach() if grad_light else None)


def fd_gradient(textures, targets, camera_pos, light_pos, light_pow, size, texels, loss_kind="mse", h=1e-6):
    """FP64 central finite differences of the loss w.r.t. all 9 channels of ``texels``.

    ``texels`` is a list of (i, j). Only the rendered pixel (i, j) depends on texel (i, j)
    (src/microfacet.py:84-120 is per-pixel), so each difference re-renders a 1x1 crop of
    the scene at that texel's position instead of the whole image; the loss normaliser
    is the full image's V*3*H*W. Returns ``[len(texels), 9]`` float64.
    """
    t64 = textures.detach().to(torch.float64)
    res = t64.shape[2]
    n = camera_pos.shape[0]
    norm = float(n * 3 * res * res)
    pos = pixel_positions(res, size, torch.float64)
    out = torch.zeros(len(texels), 9, dtype=torch.float64)
    for k, (i, j) in enumerate(texels):
        p = pos[:, i, j]
        for c in range(9):
            vals = []
            for sgn in (1.0, -1.0):
                t = t64[:, :, i, j].clone()
                t[0, c] += sgn * h
                img = _render_point(t[0], p, camera_pos.to(torch.float64), light_pos.to(torch.float64),
                                    light_pow.to(torch.float64))
                tg = targets[:, :, i, j].to(torch.float64)
                if loss_kind == "mse":
                    vals.append(((img - tg) ** 2).sum() / norm)
                else:
                    vals.append(((torch.log1p(img) - torch.log1p(tg)) ** 2).sum() / norm)
            out[k, c] = (vals[0] - vals[1]) / (2 * h)
    return out


def _render_point(t9, p, cam, lit, lpow):
    """Render one texel ``t9[9]`` at world position ``p[3]`` for all views -> ``[V, 3]``.

    The same formula as ``render`` (src/microfacet.py:84-120) evaluated for one pixel.
    """
    dif = ((t9[0:3] + 1) / 2) ** 2.2
    nx = t9[3].clamp(-1, 1)
    ny = t9[4].clamp(-1, 1)
    nz = (1 - (nx ** 2 + ny ** 2).clamp(0, 1 - EPS)).sqrt()
    nrm = torch.stack((nx, ny, nz))
    nrm = nrm / nrm.norm()
    rgh = ((t9[5] + 1) / 2) ** 2.2
    spe = ((t9[6:9] + 1) / 2) ** 2.2
    vv = cam - p
    v = vv / vv.norm(dim=1, keepdim=True)
    lv = lit - p
    l = lv / lv.norm(dim=1, keepdim=True)
    d2 = (lv * lv).sum(1, keepdim=True)
    h = l + v
    h = h / h.norm(dim=1, keepdim=True)
    nv = (v @ nrm).clamp(min=0).unsqueeze(1)
    nl = (l @ nrm).clamp(min=0).unsqueeze(1)
    nh = (h @ nrm).clamp(min=0).unsqueeze(1)
    vh = (v * h).sum(1, keepdim=True).clamp(min=0)
    alpha = rgh ** 2
    c2 = nh ** 2
    a2 = alpha ** 2
    D = a2 / (math.pi * (c2 * a2 + (1 - c2)) ** 2 + EPS)
    F = spe + (1.0 - spe) * torch.pow(2.0, ((-5.55473 * vh) - 6.98316) * vh)
    k = alpha * 0.5 + EPS
    G = (nv / (nv * (1 - k) + k)) * (nl / (nl * (1 - k) + k))
    f = dif / math.pi * (1 - spe) + D * F * G / (4 * nv * nl + EPS)
    img = lpow * f * nl / d2
    return img.clamp(EPS, 1) ** (1 / 2.2)
