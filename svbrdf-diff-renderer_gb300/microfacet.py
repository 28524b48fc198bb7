"""Drop-in ``Microfacet`` renderer backed by the sm_103a forward and adjoint kernels.

Same constructor, attributes and methods that the reference's callers use
(src/microfacet.py:9-26, 81-120; used by src/svbrdf.py:18,59-60,82 and
src/materialgan.py:134-136,168): ``Microfacet(res, n, size, cl, device)``, ``.res``,
``.n_of_imgs``, ``.update_light(light_pow)`` and ``.eval(textures) -> [n, 3, res, res]``.

``eval`` is differentiable. Its backward is the hand-written adjoint kernel
(``svbrdf_render_bwd``) behind a ``torch.autograd.Function``: the forward terms are
recomputed texel by texel, nothing but the textures is saved for backward. Gradients
flow to ``textures`` and, when it requires grad, to the light power.
"""
from __future__ import annotations

import torch

from . import _native as N


def _as_dev(x, device):
    return torch.as_tensor(x, dtype=torch.float32).to(device).contiguous()


class _RenderFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, textures, light_pow, r):
        L = N.lib()
        tex = textures.detach().to(torch.float32).contiguous()
        lp = light_pow.detach().to(torch.float32).contiguous()
        B, _, H, W = tex.shape
        out = torch.empty(B * r.n_of_imgs, 3, H, W, device=tex.device, dtype=torch.float32)
        s = N.stream_handle(tex.device)
        # the whole batch in one launch
        N.check(L.svbrdf_render_fwd_batch(tex.data_ptr(), r._cam.data_ptr(), r._lit.data_ptr(), lp.data_ptr(),
                                          r.n_of_imgs, H, W, float(r.size), B, out.data_ptr(), None, -1, None, None,
                                          0, s))
        ctx.save_for_backward(tex, lp)
        ctx.r = r
        return out

    @staticmethod
    def backward(ctx, gout):
        L = N.lib()
        tex, lp = ctx.saved_tensors
        r = ctx.r
        gout = gout.to(torch.float32).contiguous()
        B, _, H, W = tex.shape
        gtex = torch.empty_like(tex)
        want_pow = ctx.needs_input_grad[1]
        gpow = torch.zeros(3, device=tex.device, dtype=torch.float32) if want_pow else None
        s = N.stream_handle(tex.device)
        # the whole batch in one launch; the light-power gradient sums over all of it
        N.check(L.svbrdf_render_bwd_batch(tex.data_ptr(), r._cam.data_ptr(), r._lit.data_ptr(), lp.data_ptr(),
                                          r.n_of_imgs, H, W, float(r.size), B, gout.data_ptr(), gtex.data_ptr(),
                                          N.ptr(gpow), r._workspace.data_ptr(), r._workspace.numel(), s))
        return gtex, gpow, None


class Microfacet:
    """Flash-lit GGX/Cook-Torrance renderer (src/microfacet.py:9-120) on sm_103a.

    ``cl = [camera_pos [n,3], light_pos [n,3], light_pow [3]]`` in cm, as built by
    ``SvbrdfIO.load_calibration_th`` (src/svbrdf.py:134-146). ``textures`` is
    ``[1, 9, res, res]`` (a leading batch of B materials renders to ``[B*n, 3, res, res]``).
    """

    def __init__(self, res, n, size, cl, device):
        self.res = int(res)
        self.n_of_imgs = int(n)
        self.f0 = 0.04
        self.eps = 1e-6
        self.size = float(size)
        self.device = torch.device(device)
        if self.device.type != "cuda":
            raise RuntimeError("Microfacet (GB300) renders on a CUDA device only; there is no CPU fallback")
        N.lib()
        self._cam = _as_dev(cl[0], self.device).reshape(self.n_of_imgs, 3)
        self._lit = _as_dev(cl[1], self.device).reshape(self.n_of_imgs, 3)
        lp = cl[2]
        self.light_pow = lp if torch.is_tensor(lp) and lp.device == self.device else _as_dev(lp, self.device)
        if self.n_of_imgs > N.load().svbrdf_max_views():
            raise ValueError(f"n={self.n_of_imgs} views exceeds the kernel maximum {N.load().svbrdf_max_views()}")
        self._workspace = torch.zeros(int(N.load().svbrdf_workspace_bytes()), dtype=torch.uint8, device=self.device)

    @property
    def camera_pos(self):
        return self._cam

    @property
    def light_pos(self):
        return self._lit

    # ---- the reference's tensor helpers (src/microfacet.py:16-20, 54-79) in torch, on the
    # renderer's device. The kernels compute the same quantities in registers; these are for
    # callers of the reference's methods.
    @property
    def pos(self):
        """Pixel-centre grid [n, 3, res, res]: (x, -y, 0), x = ((k + 0.5) / res - 0.5) size."""
        if getattr(self, "_pos", None) is None:
            k = (torch.arange(self.res, dtype=torch.float32, device=self.device) + 0.5) / self.res - 0.5
            k = k * self.size
            x = k.view(1, -1).expand(self.res, -1)
            y = k.view(-1, 1).expand(-1, self.res)
            self._pos = torch.stack((x, -y, torch.zeros_like(x)), 0).unsqueeze(0).expand(self.n_of_imgs, -1, -1, -1)
        return self._pos

    def dot(self, a, b):
        """Channel dot product, expanded to 3 channels (src/microfacet.py:54-55)."""
        return (a * b).sum(1, keepdim=True).expand(-1, 3, -1, -1)

    def normalize(self, vec):
        """vec / |vec| over channels (src/microfacet.py:57-58)."""
        return vec / vec.norm(2.0, 1, keepdim=True)

    def get_dir(self, pos):
        """(unit direction, squared distance) from every pixel to ``pos`` ([n, 3] or
        [n, 3, res, res]) (src/microfacet.py:60-62)."""
        if pos.dim() == 2:
            pos = pos[:, :, None, None]
        vec = pos - self.pos
        return self.normalize(vec), self.dot(vec, vec)

    def reconstruct_normal(self, texture):
        """Unit normals [B, 3, H, W] from the stored xy [B, 2, H, W] (src/microfacet.py:64-70)."""
        nx = texture[:, 0].clamp(-1, 1)
        ny = texture[:, 1].clamp(-1, 1)
        nz = (1 - (nx ** 2 + ny ** 2).clamp(0, 1 - self.eps)).sqrt()
        return self.normalize(torch.stack((nx, ny, nz), 1))

    def tex2map(self, textures):
        """(normal, diffuse, specular, roughness), each [n, 3, res, res], from [1, 9, res, res]
        (src/microfacet.py:72-79): the sRGB-like maps decoded with ^2.2."""
        n = self.n_of_imgs
        diffuse = (((textures[:, 0:3] + 1) / 2) ** 2.2).expand(n, -1, -1, -1)
        normal = self.reconstruct_normal(textures[:, 3:5]).expand(n, -1, -1, -1)
        roughness = (((textures[:, 5] + 1) / 2) ** 2.2).expand(n, 3, -1, -1)
        specular = (((textures[:, 6:9] + 1) / 2) ** 2.2).expand(n, -1, -1, -1)
        return normal, diffuse, specular, roughness

    def update_light(self, light_pow):
        """src/microfacet.py:81-82: use ``light_pow [3]`` (possibly a learnable tensor)."""
        self.light_pow = light_pow

    def eval(self, textures):
        """Render ``textures [1,9,res,res]`` to ``[n, 3, res, res]`` (src/microfacet.py:84-120)."""
        assert textures.shape[2] == textures.shape[3]
        assert self.res == textures.shape[2]
        if textures.device != self.device:
            raise ValueError(f"textures on {textures.device}, renderer on {self.device}")
        lp = self.light_pow
        if not torch.is_tensor(lp):
            lp = _as_dev(lp, self.device)
        return _RenderFn.apply(textures, lp, self)

    def render_loss(self, textures, targets, loss="mse"):
        """Forward render and mean image loss in one kernel, without materialising renders.

        Returns a 0-d device tensor (no host sync). ``loss`` is ``"mse"`` (the reference's
        ``compute_image_loss``, src/optimization.py:28-29) or ``"log1p"``.
        """
        L = N.lib()
        kind = {"mse": 0, "log1p": 1}[loss]
        tex = textures.detach().to(torch.float32).contiguous()
        tg = targets.to(torch.float32).contiguous()
        out = torch.empty((), device=self.device, dtype=torch.float32)
        lp = self.light_pow if torch.is_tensor(self.light_pow) else _as_dev(self.light_pow, self.device)
        N.check(L.svbrdf_render_fwd(tex.data_ptr(), self._cam.data_ptr(), self._lit.data_ptr(),
                                    lp.detach().contiguous().data_ptr(), self.n_of_imgs, self.res, self.res,
                                    self.size, None, tg.data_ptr(), kind, out.data_ptr(),
                                    self._workspace.data_ptr(), self._workspace.numel(),
                                    N.stream_handle(self.device)))
        return out
