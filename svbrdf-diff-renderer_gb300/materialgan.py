"""Latent-space SVBRDF optimisation through the GPU renderer (the MaterialGAN path).

The reference optimises a StyleGAN2 W+ latent (and its noise maps) so that the generated
maps, rendered by ``Microfacet``, match the photos (src/materialgan.py:21-206, generator in
src/higan_models/). Its trained checkpoint is downloaded at run time and is not available
here, so ``StyleGAN2Generator`` is a StyleGAN2 ("config F", skip architecture) generator of
the same shape with seeded random weights:

* mapping: 8 equalised-learning-rate dense layers (lr multiplier 0.01), leaky ReLU, z -> w;
* synthesis at 256^2: learned 4x4 constant, one modulated 3x3 conv at 4^2, then per
  resolution 8 .. 256 an up-sampling modulated conv and a modulated conv (weight
  demodulation, per-layer noise with learned strength, bias, leaky ReLU x sqrt 2), and a
  modulated 1x1 toRGB whose output is up-sampled with a [1, 3, 3, 1] FIR filter and added
  (skip connections); channels 512 up to 32^2, then 512, 256, 128;
* W+ = 14 x 512 (2 log2(256) - 2); 13 noise maps (4^2, 8^2 x 2, ..., 256^2 x 2);
* output: 9 texture channels (the repository's layout: diffuse 3, normal xy 2, roughness 1,
  specular 3), clamped like ``latent_to_textures`` (src/materialgan.py:91-100).

``MaterialGANOptim`` keeps the reference's loop (src/materialgan.py:102-173): alternating
latent and noise phases of ``[total, l, n]`` epochs, Adam re-created every iteration (as the
reference does, so its moments never accumulate), loss = image MSE (+ 0.1 x descriptor loss
when a descriptor is given). Renders go through the drop-in ``Microfacet``, so the texture
gradient is the hand-written adjoint kernel. A batch of materials is one generator batch,
each material rendered under its own copy of the view set.
"""
from __future__ import annotations

import math
from typing import List, Optional

import torch
import torch.nn.functional as Fn

LRELU_GAIN = math.sqrt(2.0)


def _nf(res: int, fmap_base: int = 16384, fmap_max: int = 512) -> int:
    """Channels of the block producing res^2: fmap_base / 2^(log2(res) - 1), capped."""
    return min(int(fmap_base * 2 / res), fmap_max)


class _Dense(torch.nn.Module):
    """Equalised learning-rate dense layer: N(0, 1/lr_mul^2) weights scaled at run time."""

    def __init__(self, cin, cout, g, lr_mul=1.0, bias_init=0.0, act=False):
        super().__init__()
        self.weight = torch.nn.Parameter(torch.randn(cout, cin, generator=g) / lr_mul)
        self.bias = torch.nn.Parameter(torch.full((cout,), float(bias_init)))
        self.scale = lr_mul / math.sqrt(cin)
        self.lr_mul = lr_mul
        self.act = act

    def forward(self, x):
        if self.weight.requires_grad or self.bias.requires_grad:
            w, b = self.weight * self.scale, self.bias * self.lr_mul
        else:  # frozen: the scaled pair once, while the parameters are unchanged
            key = (self.weight.data_ptr(), self.weight._version, self.bias.data_ptr(), self.bias._version,
                   self.weight.dtype)
            if getattr(self, "_scaled_key", None) != key:
                with torch.no_grad():
                    self._w_scaled, self._b_scaled = self.weight * self.scale, self.bias * self.lr_mul
                self._scaled_key = key
            w, b = self._w_scaled, self._b_scaled
        y = Fn.linear(x, w, b)
        return Fn.leaky_relu(y, 0.2) * LRELU_GAIN if self.act else y


def _fir_kernel(device=None, dtype=torch.float32):
    k = torch.tensor([1.0, 3.0, 3.0, 1.0], device=device, dtype=dtype)
    k2 = torch.outer(k, k)
    return k2 / k2.sum()


_FIR_CACHE = {}


def _fir_depthwise(device, dtype, c):
    """The [c, 1, 4, 4] depthwise FIR weight, built once per (device, dtype, c): a capture
    of the generator in a CUDA graph cannot copy a new constant to the device."""
    key = (str(device), dtype, c)
    if key not in _FIR_CACHE:
        _FIR_CACHE[key] = _fir_kernel(device, dtype).view(1, 1, 4, 4).repeat(c, 1, 1, 1)
    return _FIR_CACHE[key]


def _blur(x, pad):
    """Depthwise [1,3,3,1] x [1,3,3,1] FIR with (pad0, pad1) padding on both axes."""
    c = x.shape[1]
    k = _fir_depthwise(x.device, x.dtype, c)
    x = Fn.pad(x, (pad[0], pad[1], pad[0], pad[1]))
    return Fn.conv2d(x, k, groups=c)


def _upsample2_fir(x):
    """2x up-sampling as written: zero insertion, then the FIR (gain 4 keeps the mean)."""
    b, c, h, w = x.shape
    up = torch.zeros(b, c, h * 2, w * 2, device=x.device, dtype=x.dtype)
    up[:, :, ::2, ::2] = x * 4.0
    return _blur(up, (2, 1))


def _up1d(x, dim):
    """One axis of _upsample2_fir in polyphase form: out[2m] = (x[m-1] + 3 x[m]) / 4 and
    out[2m+1] = (3 x[m] + x[m+1]) / 4, with x zero outside (the FIR's zero padding)."""
    n = x.shape[dim]
    xp = Fn.pad(x, (1, 1) if dim == -1 else (0, 0, 1, 1))
    lo, mid, hi = xp.narrow(dim, 0, n), xp.narrow(dim, 1, n), xp.narrow(dim, 2, n)
    even = 0.25 * lo + 0.75 * mid
    odd = 0.75 * mid + 0.25 * hi
    if dim == -1:
        return torch.stack((even, odd), dim=-1).flatten(-2, -1)
    return torch.stack((even, odd), dim=-2).flatten(-3, -2)


class _Upsample2Cuda(torch.autograd.Function):
    """The polyphase 2x up-sampling as one kernel each way (svbrdf_gen_upsample2[_bwd])."""

    @staticmethod
    def forward(ctx, x):
        from . import _native as N

        L = N.lib()
        x = x.contiguous()
        b, c, h, w = x.shape
        y = torch.empty(b, c, 2 * h, 2 * w, device=x.device, dtype=torch.float32)
        N.check(L.svbrdf_gen_upsample2(x.data_ptr(), y.data_ptr(), b * c, h, w, N.stream_handle(x.device)))
        ctx.hw = (b, c, h, w)
        return y

    @staticmethod
    def backward(ctx, g):
        from . import _native as N

        L = N.lib()
        b, c, h, w = ctx.hw
        g = g.contiguous()
        gx = torch.empty(b, c, h, w, device=g.device, dtype=torch.float32)
        N.check(L.svbrdf_gen_upsample2_bwd(g.data_ptr(), gx.data_ptr(), b * c, h, w, N.stream_handle(g.device)))
        return gx


def _upsample2(x):
    """2x up-sampling (zero insertion + [1,3,3,1] FIR, gain 4), computed separably in
    polyphase form: the same function as _upsample2_fir without multiplying the zeros. On the
    GPU (FP32) it is one kernel each way, in the map's layout; the torch form serves CPU
    tensors."""
    if x.is_cuda and x.dtype == torch.float32:
        return _UpsampleNHWC.apply(x, None, 0) if _is_nhwc(x) else _Upsample2Cuda.apply(x)
    return _up1d(_up1d(x, -1), -2)


def _upsample2_halo(x):
    """``_upsample2`` with one more up-sampled sample on each side ([B, C, 2H+2, 2W+2]: the
    samples at -1 and 2H, x[0] / 4 and x[H-1] / 4 per axis). A valid 3x3 convolution of it is
    the reference's up-sampling convolution, a stride-2 transposed convolution followed by
    the [1, 3, 3, 1] filter (src/higan_models/stylegan2_generator_network.py:715-729): both
    are the same shift-invariant map of the zero-extended input, cropped alike. Computed as
    the up-sampling of the input zero-padded by one, cropped by one."""
    if x.is_cuda and x.dtype == torch.float32 and _is_nhwc(x):
        return _UpsampleNHWC.apply(x, None, 1)
    return _upsample2(Fn.pad(x, (1, 1, 1, 1)))[:, :, 1:-1, 1:-1]


def _use_kernels(x):
    return x.is_cuda and x.dtype == torch.float32


CL = torch.channels_last


def _is_nhwc(x):
    """A channels-last map (and not also a plain contiguous one, as C = 1 maps are)."""
    return x.dim() == 4 and x.is_contiguous(memory_format=CL) and not x.is_contiguous()


def _cl(t):
    return t.contiguous(memory_format=CL)


class _UpsampleNHWC(torch.autograd.Function):
    """2x up-sampling of channels-last maps, optionally of x[b, c] * s[b, c] (the modulation
    of an up-sampling conv) in the same kernel (svbrdf_gen_upsample2_nhwc). The backward is
    the up-sampling adjoint, then with s svbrdf_gen_scale_nhwc_bwd for the input and style
    gradients."""

    @staticmethod
    def forward(ctx, x, s, halo=0):
        from . import _native as N

        x = _cl(x)
        s = s.contiguous() if s is not None else None
        b, c, h, w = x.shape
        y = torch.empty(b, c, 2 * h + 2 * halo, 2 * w + 2 * halo, device=x.device, dtype=torch.float32,
                        memory_format=CL)
        N.check(N.lib().svbrdf_gen_upsample2_nhwc(x.data_ptr(), s.data_ptr() if s is not None else None, y.data_ptr(),
                                                  b, h, w, c, halo, N.stream_handle(x.device)))
        ctx.save_for_backward(x, s)
        ctx.halo = halo
        return y

    @staticmethod
    def backward(ctx, g):
        from . import _native as N

        x, s = ctx.saved_tensors
        b, c, h, w = x.shape
        L, st = N.lib(), N.stream_handle(x.device)
        g = _cl(g)
        gu = torch.empty_like(x)
        N.check(L.svbrdf_gen_upsample2_nhwc_bwd(g.data_ptr(), gu.data_ptr(), b, h, w, c, ctx.halo, st))
        if s is None:
            return gu, None, None
        gx = torch.empty_like(x)
        gs = torch.empty(b, c, device=x.device, dtype=torch.float32)
        part = torch.empty(L.svbrdf_gen_nhwc_partial_floats(b, c), device=x.device, dtype=torch.float32)
        N.check(L.svbrdf_gen_scale_nhwc_bwd(gu.data_ptr(), x.data_ptr(), s.data_ptr(), gx.data_ptr(), gs.data_ptr(),
                                            part.data_ptr(), b, h * w, c, st))
        return gx, gs, None


_TF32_ERR = {}


def _tf32_err(device):
    """Per-device error word of the TF32 convolutions (non-zero if a launch gave up waiting)."""
    key = str(device)
    if key not in _TF32_ERR:
        _TF32_ERR[key] = torch.zeros(1, dtype=torch.int32, device=device)
    return _TF32_ERR[key]


def generator_device_error(device="cuda") -> int:
    """The TF32 convolutions' error word (0 = healthy); synchronises with the device."""
    return int(_tf32_err(torch.device(device)).item())


def _conv_tf32(x, w, y, b, h, wd, cin, cout, k, pad):
    """One svbrdf_gen_conv_tf32_ex call; maps with few tiles split K over a workspace."""
    from . import _native as N

    L = N.lib()
    nb = int(L.svbrdf_gen_conv_tf32_ws_bytes(b, h, wd, cin, cout, k, pad))
    ws = torch.empty(nb, device=x.device, dtype=torch.uint8) if nb > 0 else None
    N.check(L.svbrdf_gen_conv_tf32_ex(x.data_ptr(), w.data_ptr(), y.data_ptr(), N.ptr(ws), max(nb, 0), b, h, wd, cin,
                                      cout, k, pad, _tf32_err(x.device).data_ptr(), N.stream_handle(x.device)))


class _ConvTF32(torch.autograd.Function):
    """A k x k convolution (k = 3 or 1) of a channels-last FP32 map on the tensor cores in TF32
    (svbrdf_gen_conv_tf32_ex): ``pad`` 1 for a same-padded 3x3 convolution, 0 for a valid one (the
    up-sampling layers) or a 1x1. The weights come prepared: ``w_fwd`` [Cout_p][k*k][Cin] and
    ``w_dg`` [Cin][k*k][Cout_p] (transposed, taps flipped), Cout_p = Cout padded to the
    kernel's minimum of 32 with zero rows. The data gradient is the same kernel on w_dg with pad
    k - 1 - pad; the weights are frozen (no weight gradient)."""

    @staticmethod
    def forward(ctx, x, w_fwd, w_dg, cout, k, pad, keep_pad=False):
        from . import _native as N

        x = _cl(x)
        b, c, h, wd = x.shape
        coutp = w_fwd.shape[0]
        ho, wo = h + 2 * pad - (k - 1), wd + 2 * pad - (k - 1)
        y = torch.empty(b, coutp, ho, wo, device=x.device, dtype=torch.float32, memory_format=CL)
        _conv_tf32(x, w_fwd, y, b, h, wd, c, coutp, k, pad)
        ctx.save_for_backward(w_dg)
        ctx.geom = (b, c, h, wd, coutp, cout, k, pad, ho, wo)
        ctx.keep_pad = keep_pad
        return y if (coutp == cout or keep_pad) else y[:, :cout]

    @staticmethod
    def backward(ctx, gy):
        from . import _native as N

        (w_dg,) = ctx.saved_tensors
        b, c, h, wd, coutp, cout, k, pad, ho, wo = ctx.geom
        if coutp != cout and not ctx.keep_pad:
            gp = torch.empty(b, coutp, ho, wo, device=gy.device, dtype=torch.float32, memory_format=CL)
            gp[:, cout:].zero_()
            gp[:, :cout] = gy
            gy = gp
        gy = _cl(gy)
        gx = torch.empty(b, c, h, wd, device=gy.device, dtype=torch.float32, memory_format=CL)
        _conv_tf32(gy, w_dg, gx, b, ho, wo, coutp, c, k, k - 1 - pad)
        return gx, None, None, None, None, None, None


class _ActScaleNHWC(torch.autograd.Function):
    """_ActNHWC followed by the next layer's input scaling (x s2[b, c]) in one pass each way
    (svbrdf_gen_act_scale_nhwc[_bwd]), for an output whose only consumer is that layer: the
    unscaled activation is never stored, the backward recomputes it from y."""

    @staticmethod
    def forward(ctx, y, d, noise, ns, bias, gain, s2):
        from . import _native as N

        y, d, bias, s2 = _cl(y), d.contiguous(), bias.contiguous(), s2.contiguous()
        noise = noise.contiguous() if noise is not None else None
        b, c, h, w = y.shape
        out = torch.empty_like(y)
        N.check(N.lib().svbrdf_gen_act_scale_nhwc(y.data_ptr(), d.data_ptr(), N.ptr(noise),
                                                  ns.data_ptr() if noise is not None else None, bias.data_ptr(), gain,
                                                  s2.data_ptr(), out.data_ptr(), b, h * w, c,
                                                  N.stream_handle(y.device)))
        ctx.save_for_backward(y, d, noise, ns, bias, s2)
        ctx.gain = gain
        return out

    @staticmethod
    def backward(ctx, g):
        from . import _native as N

        y, d, noise, ns, bias, s2 = ctx.saved_tensors
        b, c, h, w = y.shape
        L = N.lib()
        g = _cl(g)
        gy = torch.empty_like(y)
        gd = torch.empty(b, c, device=y.device, dtype=torch.float32)
        gs2 = torch.empty(b, c, device=y.device, dtype=torch.float32)
        want_noise = noise is not None and ctx.needs_input_grad[2]
        gn = torch.empty_like(noise) if want_noise else None
        nparts = L.svbrdf_gen_nhwc_partial_floats(b, c)
        part = torch.empty(nparts, device=y.device, dtype=torch.float32)
        part2 = torch.empty(nparts, device=y.device, dtype=torch.float32)
        N.check(L.svbrdf_gen_act_scale_nhwc_bwd(g.data_ptr(), y.data_ptr(), d.data_ptr(), N.ptr(noise),
                                                ns.data_ptr() if noise is not None else None, bias.data_ptr(), ctx.gain,
                                                s2.data_ptr(), gy.data_ptr(), gd.data_ptr(), gs2.data_ptr(), N.ptr(gn),
                                                part.data_ptr(), part2.data_ptr(), b, h * w, c,
                                                N.stream_handle(y.device)))
        return gy, gd, gn, None, None, None, gs2


class _RgbNHWC(torch.autograd.Function):
    """The toRGB epilogue (svbrdf_gen_rgb_nhwc[_bwd]): the 1x1 convolution's padded
    channels-last output yp [B, cp, H, W] plus the bias plus the up-sampled previous image
    ``prev`` (NCHW, or None), written as one NCHW image [B, c, H, W]. The bias is frozen."""

    @staticmethod
    def forward(ctx, yp, bias, prev, c):
        from . import _native as N

        b, cp, h, w = yp.shape
        img = torch.empty(b, c, h, w, device=yp.device, dtype=torch.float32)
        N.check(N.lib().svbrdf_gen_rgb_nhwc(yp.data_ptr(), cp, bias.data_ptr(), N.ptr(prev), img.data_ptr(), b, c, h, w,
                                            N.stream_handle(yp.device)))
        ctx.geom = (b, cp, c, h, w, prev is not None)
        return img

    @staticmethod
    def backward(ctx, g):
        from . import _native as N

        b, cp, c, h, w, has_prev = ctx.geom
        L = N.lib()
        st = N.stream_handle(g.device)
        g = g.contiguous()
        gyp = torch.empty(b, cp, h, w, device=g.device, dtype=torch.float32, memory_format=CL)
        N.check(L.svbrdf_gen_rgb_nhwc_bwd(g.data_ptr(), gyp.data_ptr(), cp, b, c, h, w, st))
        gprev = None
        if has_prev and ctx.needs_input_grad[2]:
            gprev = torch.empty(b, c, h // 2, w // 2, device=g.device, dtype=torch.float32)
            N.check(L.svbrdf_gen_upsample2_bwd(g.data_ptr(), gprev.data_ptr(), b * c, h // 2, w // 2, st))
        return gyp, None, gprev, None


class _ScaleNHWC(torch.autograd.Function):
    """x[b, c] * s[b, c] on channels-last maps (svbrdf_gen_scale_nhwc[_bwd])."""

    @staticmethod
    def forward(ctx, x, s):
        from . import _native as N

        x, s = _cl(x), s.contiguous()
        b, c, h, w = x.shape
        y = torch.empty_like(x)
        N.check(N.lib().svbrdf_gen_scale_nhwc(x.data_ptr(), s.data_ptr(), y.data_ptr(), b, h * w, c,
                                              N.stream_handle(x.device)))
        ctx.save_for_backward(x, s)
        return y

    @staticmethod
    def backward(ctx, g):
        from . import _native as N

        x, s = ctx.saved_tensors
        b, c, h, w = x.shape
        L = N.lib()
        g = _cl(g)
        gx = torch.empty_like(x)
        gs = torch.empty(b, c, device=x.device, dtype=torch.float32)
        part = torch.empty(L.svbrdf_gen_nhwc_partial_floats(b, c), device=x.device, dtype=torch.float32)
        N.check(L.svbrdf_gen_scale_nhwc_bwd(g.data_ptr(), x.data_ptr(), s.data_ptr(), gx.data_ptr(), gs.data_ptr(),
                                            part.data_ptr(), b, h * w, c, N.stream_handle(x.device)))
        return gx, gs


class _ActNHWC(torch.autograd.Function):
    """The style layer's epilogue on channels-last maps (svbrdf_gen_act_nhwc[_bwd]); the
    arguments are those of _ActCuda."""

    @staticmethod
    def forward(ctx, y, d, noise, ns, bias, gain):
        from . import _native as N

        y, d, bias = _cl(y), d.contiguous(), bias.contiguous()
        noise = noise.contiguous() if noise is not None else None
        b, c, h, w = y.shape
        out = torch.empty_like(y)
        N.check(N.lib().svbrdf_gen_act_nhwc(y.data_ptr(), d.data_ptr(), noise.data_ptr() if noise is not None else None,
                                            ns.data_ptr() if noise is not None else None, bias.data_ptr(), gain,
                                            out.data_ptr(), b, h * w, c, N.stream_handle(y.device)))
        ctx.save_for_backward(y, d, noise, ns, bias)
        ctx.gain = gain
        return out

    @staticmethod
    def backward(ctx, g):
        from . import _native as N

        y, d, noise, ns, bias = ctx.saved_tensors
        b, c, h, w = y.shape
        L = N.lib()
        g = _cl(g)
        gy = torch.empty_like(y)
        gd = torch.empty(b, c, device=y.device, dtype=torch.float32)
        want_noise = noise is not None and ctx.needs_input_grad[2]
        gn = torch.empty_like(noise) if want_noise else None
        part = torch.empty(L.svbrdf_gen_nhwc_partial_floats(b, c), device=y.device, dtype=torch.float32)
        N.check(L.svbrdf_gen_act_nhwc_bwd(g.data_ptr(), y.data_ptr(), d.data_ptr(),
                                          noise.data_ptr() if noise is not None else None,
                                          ns.data_ptr() if noise is not None else None, bias.data_ptr(), ctx.gain,
                                          gy.data_ptr(), gd.data_ptr(), gn.data_ptr() if want_noise else None,
                                          part.data_ptr(), b, h * w, c, N.stream_handle(y.device)))
        return gy, gd, gn, None, None, None


class _ScaleCuda(torch.autograd.Function):
    """x[b, c] * s[b, c] (a modulated conv's input scaling) as one kernel each way; the
    backward also forms the style gradient sum_hw g x per plane (svbrdf_gen_scale[_bwd])."""

    @staticmethod
    def forward(ctx, x, s):
        from . import _native as N

        x, s = x.contiguous(), s.contiguous()
        b, c, h, w = x.shape
        y = torch.empty_like(x)
        N.check(N.lib().svbrdf_gen_scale(x.data_ptr(), s.data_ptr(), y.data_ptr(), b * c, h * w,
                                         N.stream_handle(x.device)))
        ctx.save_for_backward(x, s)
        return y

    @staticmethod
    def backward(ctx, g):
        from . import _native as N

        x, s = ctx.saved_tensors
        b, c, h, w = x.shape
        g = g.contiguous()
        gx = torch.empty_like(x)
        gs = torch.empty(b, c, device=x.device, dtype=torch.float32)
        N.check(N.lib().svbrdf_gen_scale_bwd(g.data_ptr(), x.data_ptr(), s.data_ptr(), gx.data_ptr(), gs.data_ptr(),
                                             b * c, h * w, N.stream_handle(x.device)))
        return gx, gs


class _ActCuda(torch.autograd.Function):
    """A style layer's epilogue lrelu(y d + ns noise + bias, 0.2) gain as one kernel each way
    (svbrdf_gen_act[_bwd]). d: [B, C] demodulation; noise: [B, 1, H, W] or None; ns: the
    0-d noise strength; bias: [C]. The generator is frozen, so bias and ns get no gradient."""

    @staticmethod
    def forward(ctx, y, d, noise, ns, bias, gain):
        from . import _native as N

        y, d, bias = y.contiguous(), d.contiguous(), bias.contiguous()
        noise = noise.contiguous() if noise is not None else None
        b, c, h, w = y.shape
        out = torch.empty_like(y)
        N.check(N.lib().svbrdf_gen_act(y.data_ptr(), d.data_ptr(), noise.data_ptr() if noise is not None else None,
                                       ns.data_ptr() if noise is not None else None, bias.data_ptr(), gain,
                                       out.data_ptr(), b, c, h * w, N.stream_handle(y.device)))
        ctx.save_for_backward(y, d, noise, ns, bias)
        ctx.gain = gain
        return out

    @staticmethod
    def backward(ctx, g):
        from . import _native as N

        y, d, noise, ns, bias = ctx.saved_tensors
        b, c, h, w = y.shape
        g = g.contiguous()
        gy = torch.empty_like(y)
        gd = torch.empty(b, c, device=y.device, dtype=torch.float32)
        want_noise = noise is not None and ctx.needs_input_grad[2]
        gn = torch.empty_like(noise) if want_noise else None
        N.check(N.lib().svbrdf_gen_act_bwd(g.data_ptr(), y.data_ptr(), d.data_ptr(),
                                           noise.data_ptr() if noise is not None else None,
                                           ns.data_ptr() if noise is not None else None, bias.data_ptr(), ctx.gain,
                                           gy.data_ptr(), gd.data_ptr(), gn.data_ptr() if want_noise else None,
                                           b, c, h * w, N.stream_handle(y.device)))
        return gy, gd, gn, None, None, None


class _ModConv(torch.nn.Module):
    """Modulated (and optionally demodulated) conv, optionally 2x up-sampling first."""

    def __init__(self, cin, cout, k, w_dim, g, demod=True, up=False):
        super().__init__()
        self.weight = torch.nn.Parameter(torch.randn(cout, cin, k, k, generator=g))
        self.affine = _Dense(w_dim, cin, g, bias_init=1.0)
        self.scale = 1.0 / math.sqrt(cin * k * k)
        self.demod, self.up, self.k = demod, up, k

    def forward(self, x, w):
        # The modulated weight scale w_oi s_bi d_bo factors out of the convolution: scale the
        # input channels by the style, convolve with the shared weight, scale the output
        # channels by the demodulation d_bo = rsqrt(sum_i,taps (scale w_oi s_bi)^2 + 1e-8).
        # This is the same function as convolving with per-sample weights (StyleGAN2's fused
        # form), but it runs as one batched convolution. With the generator frozen, its
        # backward is a data gradient plus small reductions, with no per-sample weight
        # gradients.
        y, d = self.parts(x, w)
        return y if d is None else y * d[:, :, None, None]

    def _tf32_ok(self, x) -> bool:
        """The TF32 tensor-core convolution serves a frozen layer whenever TF32 is allowed
        (cuDNN's default, and what the reference's PyTorch GPU path computes in); with TF32 off
        the layer runs in FP32 through cuDNN."""
        cin = self.weight.shape[1]
        return (torch.backends.cudnn.allow_tf32 and not self.weight.requires_grad and cin % 32 == 0 and
                x.shape[-1] + 2 * (0 if self.up else self.k // 2) - (self.k - 1) >= 4)

    def _tf32_weights(self, wsc):
        """(w_fwd [Cout_p][k*k][Cin], w_dg [Cin][k*k][Cout_p]) of the scaled weight, Cout_p =
        Cout rounded up to 32; cached while the weight is unchanged."""
        key = (self.weight.data_ptr(), self.weight._version, str(self.weight.device))
        if getattr(self, "_tf32_key", None) != key:
            with torch.no_grad():
                w = wsc.detach().float()
                cout, cin, k, _ = w.shape
                coutp = max(32, -(-cout // 32) * 32)
                if coutp != cout:
                    w = torch.cat((w, torch.zeros(coutp - cout, cin, k, k, device=w.device)), 0)
                self._w_fwd = w.permute(0, 2, 3, 1).reshape(coutp, k * k, cin).contiguous()
                self._w_dg = w.flip(2, 3).permute(1, 2, 3, 0).reshape(cin, k * k, coutp).contiguous()
            self._tf32_key = key
        return self._w_fwd, self._w_dg

    def parts(self, x, w, keep_pad=False, sd=None, prescaled=False):
        """The shared-weight convolution of the style-scaled input, and the demodulation
        d [B, cout] (None without demodulation) still to be applied to its output. With
        ``keep_pad`` the TF32 path returns its output with the channels padded to 32; ``sd``
        is this layer's (style, demodulation) pair when the generator computed them for all
        layers at once (StyleGAN2Generator._styles); ``prescaled`` says that the
        channels-last input already carries this layer's style scaling (_ActScaleNHWC)."""
        s = self.affine(w) if sd is None else sd[0]  # [B, cin]
        wsc, w2t = self._scaled_weight()
        # an up-sampling layer convolves the up-sampled map with its one-sample halo, unpadded
        # (_upsample2_halo): the reference's transposed convolution + filter on the border too
        pad = 0 if self.up else self.k // 2
        if _use_kernels(x) and _is_nhwc(x):
            # channels-last: the layout of the TF32 tensor-core convolutions (and of cuDNN's)
            if self.up:
                x = _UpsampleNHWC.apply(x, s, 1)
            elif not prescaled:
                x = _ScaleNHWC.apply(x, s)
            if self._tf32_ok(x):
                w_fwd, w_dg = self._tf32_weights(wsc)
                y = _ConvTF32.apply(x, w_fwd, w_dg, self.weight.shape[0], self.k, pad, keep_pad)
            else:
                y = Fn.conv2d(x, _cl(wsc), padding=pad)
        else:
            x = _ScaleCuda.apply(x, s) if _use_kernels(x) else x * s[:, :, None, None]
            if self.up:
                x = _upsample2_halo(x)  # per-channel linear: commutes with the channel scaling
            y = Fn.conv2d(x, wsc, padding=pad)
        d = None
        if self.demod:
            d = torch.rsqrt(s.pow(2) @ w2t + 1e-8) if sd is None else sd[1]  # [B, cout]
        return y, d

    def _scaled_weight(self):
        """(scale * weight, its squared sums over the taps transposed, [cin, cout]). A frozen
        weight's pair is computed once and cached while the weight is unchanged; a trainable
        one is recomputed on every call, inside autograd."""
        if self.weight.requires_grad:
            wsc = self.weight * self.scale
            return wsc, wsc.pow(2).sum(dim=(2, 3)).t()
        key = (self.weight.data_ptr(), self.weight._version, str(self.weight.device), self.weight.dtype)
        if getattr(self, "_wsc_key", None) != key:
            with torch.no_grad():
                wsc = self.weight * self.scale
                self._wsc = wsc
                self._w2t = wsc.pow(2).sum(dim=(2, 3)).t().contiguous()
            self._wsc_key = key
        return self._wsc, self._w2t


class _StyleLayer(torch.nn.Module):
    def __init__(self, cin, cout, w_dim, g, up=False):
        super().__init__()
        self.conv = _ModConv(cin, cout, 3, w_dim, g, up=up)
        self.noise_strength = torch.nn.Parameter(torch.zeros(()))
        self.bias = torch.nn.Parameter(torch.zeros(cout))

    def kernel_ok(self, x, noise) -> bool:
        """Whether forward takes the CUDA-kernel path for this input and noise map."""
        return _use_kernels(x) and not (self.bias.requires_grad or self.noise_strength.requires_grad) and (
            noise is None or (noise.shape[0] == x.shape[0] and noise.shape[1] == 1))

    def forward(self, x, w, noise, sd=None, s_next=None, prescaled=False):
        """``s_next``: the next layer's style, to scale this layer's output by in the same pass
        (channels-last kernel path only; the caller then passes ``prescaled`` to that layer)."""
        if self.kernel_ok(x, noise):
            y, d = self.conv.parts(x, w, sd=sd, prescaled=prescaled)
            if s_next is not None and _is_nhwc(y):
                return _ActScaleNHWC.apply(y, d, noise, self.noise_strength, self.bias, LRELU_GAIN, s_next)
            act = _ActNHWC if _is_nhwc(y) else _ActCuda
            return act.apply(y, d, noise, self.noise_strength, self.bias, LRELU_GAIN)
        y = self.conv(x, w)
        if noise is not None:
            y = y + self.noise_strength * noise
        return Fn.leaky_relu(y + self.bias.view(1, -1, 1, 1), 0.2) * LRELU_GAIN


class _ToRGB(torch.nn.Module):
    def __init__(self, cin, cout, w_dim, g):
        super().__init__()
        self.conv = _ModConv(cin, cout, 1, w_dim, g, demod=False)
        self.bias = torch.nn.Parameter(torch.zeros(cout))

    def forward(self, x, w, skip, sd=None):
        cout = self.bias.shape[0]
        if (_use_kernels(x) and _is_nhwc(x) and not self.bias.requires_grad and self.conv._tf32_ok(x) and
                x.shape[-1] % 2 == 0 and x.shape[-2] % 2 == 0 and
                (skip is None or (skip.is_contiguous() and skip.dtype == torch.float32 and
                                  tuple(skip.shape) == (x.shape[0], cout, x.shape[-2] // 2, x.shape[-1] // 2)))):
            # the TF32 convolution's padded channels-last output, bias and the up-sampled skip
            # image in one pass that writes the image in NCHW
            yp, _ = self.conv.parts(x, w, keep_pad=True, sd=sd)
            return _RgbNHWC.apply(_cl(yp), self.bias, skip, cout)
        y = self.conv(x, w) + self.bias.view(1, -1, 1, 1)
        return y if skip is None else y + _upsample2(skip)


class StyleGAN2Generator(torch.nn.Module):
    """StyleGAN2-shaped generator (seeded random weights) producing [B, 9, res, res] textures."""

    def __init__(self, resolution: int = 256, w_dim: int = 512, out_channels: int = 9, seed: int = 0,
                 fmap_base: int = 16384, fmap_max: int = 512, mapping_layers: int = 8, channels_last: bool = True):
        super().__init__()
        # on the GPU the feature maps run channels-last (NHWC), cuDNN's convolution layout
        self.channels_last = channels_last
        g = torch.Generator().manual_seed(seed)
        self.resolution, self.w_dim = resolution, w_dim
        log2 = int(round(math.log2(resolution)))
        assert 2 ** log2 == resolution and resolution >= 8
        self.num_ws = 2 * log2 - 2
        nf = lambda r: _nf(r, fmap_base, fmap_max)
        self.mapping = torch.nn.ModuleList([_Dense(w_dim, w_dim, g, lr_mul=0.01, act=True)
                                            for _ in range(mapping_layers)])
        self.register_buffer("w_avg", torch.zeros(w_dim))
        self.const = torch.nn.Parameter(torch.randn(1, nf(4), 4, 4, generator=g))
        self.conv4 = _StyleLayer(nf(4), nf(4), w_dim, g)
        self.rgb4 = _ToRGB(nf(4), out_channels, w_dim, g)
        self.ups, self.convs, self.rgbs = torch.nn.ModuleList(), torch.nn.ModuleList(), torch.nn.ModuleList()
        self.noise_res = [4]
        for l in range(3, log2 + 1):
            r = 2 ** l
            self.ups.append(_StyleLayer(nf(r // 2), nf(r), w_dim, g, up=True))
            self.convs.append(_StyleLayer(nf(r), nf(r), w_dim, g))
            self.rgbs.append(_ToRGB(nf(r), out_channels, w_dim, g))
            self.noise_res += [r, r]
        with torch.no_grad():  # average w of the random mapping (truncation centre)
            z = torch.randn(4096, w_dim, generator=g)
            self.w_avg.copy_(self.map(z).mean(0))

    def map(self, z: torch.Tensor) -> torch.Tensor:
        x = z * torch.rsqrt(z.pow(2).mean(dim=1, keepdim=True) + 1e-8)
        for layer in self.mapping:
            x = layer(x)
        return x

    def truncate(self, w: torch.Tensor, psi: float = 1.0) -> torch.Tensor:
        """w_avg + psi (w - w_avg); MaterialGAN builds its generator with psi 1
        (src/higan_models/stylegan2_generator.py:32), the default here."""
        return self.w_avg + (w - self.w_avg) * psi

    @torch.no_grad()
    def load_reference_state_dict(self, sd: dict):
        """Load the weights of the reference's ``StyleGAN2GeneratorNet`` (its ``state_dict``, e.g.
        MaterialGAN's ``ckp/materialgan.pth``; src/higan_models/stylegan2_generator_network.py:36,
        base_generator.py:129-135) into this generator. Key by key:

        * ``mapping.dense{i}.fc.weight`` / ``.bias`` -> ``mapping[i]`` (both scale by lr 0.01 and
          1/sqrt(512) at run time, stylegan2_generator_network.py:762-824);
        * ``synthesis.early_layer.const`` -> ``const``;
        * ``synthesis.layer0`` -> ``conv4``; ``layer{2b-1}`` (2x up-sampling) -> ``ups[b-1]``,
          ``layer{2b}`` -> ``convs[b-1]``; ``output0`` -> ``rgb4``, ``output{b}`` -> ``rgbs[b-1]``.
          Conv weights are stored [k, k, in, out] and become [out, in, k, k]; the style layer's
          constant bias 1 (``init_bias``) moves into the affine bias; ``noise_strength`` and
          ``bias`` copy over;
        * ``truncation.w_avg`` -> ``w_avg``.

        The reference's up-sampling layer (a stride-2 transposed convolution with the flipped
        kernel, then the [1, 3, 3, 1] filter) is the same linear map as this generator's
        (zero insertion and the filter, then the 3x3 convolution), so the weights carry over
        unchanged."""
        def src(k):
            if k not in sd:
                raise KeyError(f"reference state dict has no {k!r}")
            return torch.as_tensor(sd[k])

        for i, layer in enumerate(self.mapping):
            layer.weight.copy_(src(f"mapping.dense{i}.fc.weight"))
            layer.bias.copy_(src(f"mapping.dense{i}.bias"))
        self.const.copy_(src("synthesis.early_layer.const"))
        if "truncation.w_avg" in sd:
            self.w_avg.copy_(src("truncation.w_avg"))

        def modconv(dst, key):
            dst.weight.copy_(src(f"{key}.weight").permute(3, 2, 0, 1))
            dst.affine.weight.copy_(src(f"{key}.style.fc.weight"))
            # the style DenseBlock adds a constant init_bias of 1 (stylegan2_generator_network.py:661)
            dst.affine.bias.copy_(src(f"{key}.style.bias") + 1.0)

        def style(dst, key):
            modconv(dst.conv, key)
            dst.bias.copy_(src(f"{key}.bias"))
            dst.noise_strength.copy_(src(f"{key}.noise_strength").reshape(()))

        def rgb(dst, key):
            modconv(dst.conv, key)
            dst.bias.copy_(src(f"{key}.bias"))

        style(self.conv4, "synthesis.layer0")
        rgb(self.rgb4, "synthesis.output0")
        for b, (up, conv, out) in enumerate(zip(self.ups, self.convs, self.rgbs), start=1):
            style(up, f"synthesis.layer{2 * b - 1}")
            style(conv, f"synthesis.layer{2 * b}")
            rgb(out, f"synthesis.output{b}")
        return self

    def make_noises(self, mode: str = "zero", batch: int = 1, device=None, seed: int = 0) -> List[torch.Tensor]:
        """One noise map per style layer ([batch, 1, r, r]); 'zero' like the reference's "avg"."""
        g = torch.Generator().manual_seed(seed)
        out = []
        for r in self.noise_res:
            n = torch.zeros(batch, 1, r, r) if mode == "zero" else torch.randn(batch, 1, r, r, generator=g)
            out.append(n.to(device))
        return out

    def _layers(self):
        """Every modulated convolution in the order synthesis runs them, with its W+ row."""
        out = [(self.conv4.conv, 0), (self.rgb4.conv, 1)]
        for i, (up, conv, rgb) in enumerate(zip(self.ups, self.convs, self.rgbs)):
            out += [(up.conv, 1 + 2 * i), (conv.conv, 2 + 2 * i), (rgb.conv, 3 + 2 * i)]
        return out

    def _styles(self, wp: torch.Tensor):
        """The styles s = affine(w) and demodulations d = rsqrt(s^2 sum_taps (scale w)^2 + 1e-8)
        of every layer, for frozen weights: layers of one shape (input and output channels,
        demodulated or not) share one batched product each (torch.baddbmm / bmm), in place of
        two small GEMMs and a few elementwise ops per layer. Returns {layer: (s, d)}; {} when
        a weight is trainable (each layer then computes its own, inside autograd)."""
        layers = self._layers()
        if any(m.weight.requires_grad or m.affine.weight.requires_grad or m.affine.bias.requires_grad
               for m, _ in layers):
            return {}
        key = tuple((m.weight.data_ptr(), m.weight._version, m.affine.weight._version, m.affine.bias._version)
                    for m, _ in layers) + (wp.device, wp.dtype)
        if getattr(self, "_style_key", None) != key:
            groups = {}
            for m, widx in layers:
                groups.setdefault((m.weight.shape[1], m.weight.shape[0], m.demod), []).append((m, widx))
            packed = []
            with torch.no_grad():
                for (cin, cout, demod), ms in groups.items():
                    a = torch.stack([(m.affine.weight * m.affine.scale).t() for m, _ in ms]).to(wp.device, wp.dtype)
                    b = torch.stack([(m.affine.bias * m.affine.lr_mul) for m, _ in ms]).unsqueeze(1).to(wp.device, wp.dtype)
                    w2 = (torch.stack([m._scaled_weight()[1] for m, _ in ms]).to(wp.device, wp.dtype).contiguous()
                          if demod else None)
                    idx = torch.tensor([wi for _, wi in ms], device=wp.device)
                    packed.append(([m for m, _ in ms], idx, a.contiguous(), b.contiguous(), w2))
            self._style_packed, self._style_key = packed, key
        sd = {}
        for mods, idx, a, b, w2 in self._style_packed:
            st = torch.baddbmm(b, wp.index_select(1, idx).transpose(0, 1), a)  # [L, B, cin]
            dm = torch.rsqrt(torch.bmm(st * st, w2) + 1e-8) if w2 is not None else None  # [L, B, cout]
            ss = torch.unbind(st, 0)
            ds = torch.unbind(dm, 0) if dm is not None else [None] * len(mods)
            for m, si, di in zip(mods, ss, ds):
                sd[m] = (si, di)
        return sd

    def synthesis(self, wp: torch.Tensor, noises: Optional[List[torch.Tensor]] = None) -> torch.Tensor:
        """W+ [B, num_ws, w_dim] -> [B, out_channels, res, res]."""
        b = wp.shape[0]
        noises = noises if noises is not None else [None] * len(self.noise_res)
        x = self.const.expand(b, -1, -1, -1)
        if self.channels_last and _use_kernels(x):
            x = _cl(x)
        # all layers' styles and demodulations at once on the GPU path with frozen weights
        sd = self._styles(wp) if _use_kernels(x) else {}
        x = self.conv4(x, wp[:, 0], noises[0], sd.get(self.conv4.conv))
        img = self.rgb4(x, wp[:, 1], None, sd.get(self.rgb4.conv))
        for i, (up, conv, rgb) in enumerate(zip(self.ups, self.convs, self.rgbs)):
            n_up, n_conv = noises[1 + 2 * i], noises[2 + 2 * i]
            # an up-sampling layer's output feeds only the next convolution: on the
            # channels-last kernel path its epilogue also applies that layer's style scaling
            fuse = (bool(sd) and _is_nhwc(x) and up.kernel_ok(x, n_up) and conv.kernel_ok(x, n_conv)
                    and conv.conv in sd)
            if fuse:
                x = up(x, wp[:, 1 + 2 * i], n_up, sd.get(up.conv), s_next=sd[conv.conv][0])
                x = conv(x, wp[:, 2 + 2 * i], n_conv, sd.get(conv.conv), prescaled=True)
            else:
                x = up(x, wp[:, 1 + 2 * i], n_up, sd.get(up.conv))
                x = conv(x, wp[:, 2 + 2 * i], n_conv, sd.get(conv.conv))
            img = rgb(x, wp[:, 3 + 2 * i], img, sd.get(rgb.conv))
        return img


def latent_to_textures(gen: StyleGAN2Generator, latent: torch.Tensor, noises=None) -> torch.Tensor:
    """synthesis + the reference's per-group clamps (src/materialgan.py:91-100)."""
    t = gen.synthesis(latent, noises)
    return torch.cat((t[:, 0:5].clamp(-1, 1), t[:, 5:6].clamp(-0.5, 0.5), t[:, 6:9].clamp(-1, 1)), 1)


class MaterialGANOptim:
    """Latent (W+) and noise optimisation through the renderer (src/materialgan.py:21-206).

    ``descriptor``: None (image loss only), one feature loss, or a (latent-phase,
    noise-phase) pair such as ``descriptor.reference_descriptors()``, the reference's "L"
    and "N" VGG losses; the feature term is weighted by ``descriptor_weight`` (0.1)."""

    def __init__(self, device, renderer_obj, generator: StyleGAN2Generator, descriptor=None,
                 descriptor_weight: float = 0.1):
        self.device = torch.device(device)
        self.renderer_obj = renderer_obj
        self.net = generator.to(self.device).eval()
        for p in self.net.parameters():
            p.requires_grad_(False)
        self.descriptor = descriptor
        self.descriptor_weight = descriptor_weight
        self.loss_image_list, self.loss_feature_list = [], []
        self._graphs = {}

    def init_from(self, latent: Optional[torch.Tensor] = None, batch: int = 1, seed: int = 0, noise: str = "zero"):
        """W+ from a given latent, else the truncated mapping of seeded z (src/materialgan.py:58-75)."""
        if latent is None:
            g = torch.Generator().manual_seed(seed)
            z = torch.randn(batch, self.net.w_dim, generator=g).to(self.device)
            with torch.no_grad():
                w = self.net.truncate(self.net.map(z))
            latent = w[:, None, :].repeat(1, self.net.num_ws, 1)
        self.latent = latent.detach().to(self.device, torch.float32).clone().requires_grad_(True)
        self.noises = [n.requires_grad_(True) for n in
                       self.net.make_noises(noise, self.latent.shape[0], self.device, seed)]
        self._graphs = {}  # captured epochs hold the previous parameters' addresses

    def save_latent(self, latent_path, noise_path=None):
        """The latent and the noise maps with torch.save, as the reference's save points do
        (src/materialgan.py:161-162: optim_latent.pt, optim_noise.pt)."""
        torch.save(self.latent.detach().cpu(), latent_path)
        if noise_path is not None:
            torch.save([n.detach().cpu() for n in self.noises], noise_path)

    def load_latent(self, latent_path, noise_path=None):
        """Resume from save_latent's files."""
        self.latent = torch.load(latent_path, map_location="cpu").to(self.device, torch.float32).requires_grad_(True)
        if noise_path is not None:
            self.noises = [n.to(self.device, torch.float32).requires_grad_(True)
                           for n in torch.load(noise_path, map_location="cpu")]
        self._graphs = {}  # captured epochs hold the previous parameters' addresses

    # ---- the reference's helpers (src/optimization.py:17-29, src/materialgan.py:82-89) ----
    def gradient(self, parameters):
        """Leaves that require grad, as the reference's ``Optim.gradient``."""
        if isinstance(parameters, list):
            return [p.detach().requires_grad_(True) for p in parameters]
        return parameters.detach().requires_grad_(True)

    def compute_image_loss(self, predicts):
        """MSE against the loaded targets (src/optimization.py:28-29)."""
        return torch.nn.functional.mse_loss(predicts, self.targets)

    def compute_feature_loss(self, predicts, flag):
        """The feature loss of the latent ("L") or noise ("N") phase (src/materialgan.py:82-89),
        0 without a descriptor."""
        if flag not in ("L", "N"):
            raise ValueError(f"flag must be 'L' or 'N', not {flag!r}")
        desc = self._descriptor_for(flag == "L")
        if desc is None:
            return torch.zeros((), device=predicts.device)
        from .descriptor import descriptor_term

        return descriptor_term(predicts, desc)

    def _descriptors(self):
        d = self.descriptor
        if d is None:
            return []
        return list(d) if isinstance(d, (tuple, list)) else [d]

    def _descriptor_for(self, phase_latent: bool):
        """The feature loss of this phase: a (latent-phase, noise-phase) pair picks by phase,
        as the reference's "L" and "N" losses do (src/materialgan.py:28-34, 137-139)."""
        d = self.descriptor
        if isinstance(d, (tuple, list)):
            return d[0] if phase_latent else d[1]
        return d

    def load_targets(self, targets: torch.Tensor):
        """targets [B*V, 3, H, W] (materials major)."""
        self.targets = targets.to(self.device, torch.float32).contiguous()
        self._graphs = {}
        for d in self._descriptors():
            d.load(self.targets)

    def latent_to_textures(self, latent=None):
        return latent_to_textures(self.net, self.latent if latent is None else latent, self.noises)

    # ---- one epoch as a CUDA graph -------------------------------------------------------
    # An epoch is a few hundred small kernels (the generator's layers, forward and backward),
    # so launching them one by one costs more host time than they take on the GPU. With the
    # reference's fresh Adam every epoch (src/materialgan.py:119-129), an epoch is a fixed
    # function of the parameters and replays as one graph: forward, backward and a
    # capturable torch Adam whose state is zeroed inside the graph, which is what a new
    # Adam's first step computes.
    def _epoch(self, params):
        for p in (self.latent, *self.noises):
            p.grad = None
        rendered = self.renderer_obj.eval(self.latent_to_textures())
        loss = torch.nn.functional.mse_loss(rendered, self.targets)
        loss.backward()
        return loss

    def _graph_for(self, phase_latent: bool, lr: float):
        key = (phase_latent, float(lr))
        if key in self._graphs:
            return self._graphs[key]
        params = [self.latent] if phase_latent else self.noises
        opt = torch.optim.Adam(params, lr=lr, betas=(0.9, 0.999), capturable=True)
        for p in params:
            opt.state[p] = {"step": torch.zeros((), dtype=torch.float32, device=self.device),
                            "exp_avg": torch.zeros_like(p), "exp_avg_sq": torch.zeros_like(p)}
        side = torch.cuda.Stream(self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(side):  # warm autograd and the allocator; the parameters stay as they are
            for _ in range(2):
                self._epoch(params)
        torch.cuda.current_stream(self.device).wait_stream(side)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            loss = self._epoch(params)
            for st in opt.state.values():
                st["step"].zero_()
                st["exp_avg"].zero_()
                st["exp_avg_sq"].zero_()
            opt.step()
        self._graphs[key] = (graph, loss, opt)
        return self._graphs[key]

    def optim(self, epochs, lr, svbrdf_obj=None, optim_light=False, reset_adam_each_iter=True, graph=True):
        """``epochs = [total, l, n]``: alternate l latent epochs and n noise epochs. With
        ``graph`` (and the reference's fresh Adam each epoch, no descriptor term, no light
        optimisation) each epoch is one CUDA-graph replay.

        ``optim_light``: the light power ``svbrdf_obj.cl[2]`` joins each epoch's Adam and is
        handed to the renderer before each render, as src/materialgan.py:110-135 does; it is
        left as the optimised leaf in ``svbrdf_obj.cl[2]`` and in the renderer."""
        total, l_ep, n_ep = epochs
        cycle = l_ep + n_ep
        # this call's losses stay on the device and are read once at the end; the lists
        # accumulate over calls, as the reference's do
        img_losses, feat_losses = [], []
        if (graph and reset_adam_each_iter and self.descriptor is None and self.device.type == "cuda"
                and not optim_light):
            for epoch in range(total):
                g, loss, _ = self._graph_for((epoch % cycle) < l_ep, lr)
                g.replay()
                img_losses.append(loss.detach().clone())
            for p in (self.latent, *self.noises):
                p.grad = None
            self.textures = self.latent_to_textures().detach()
            if img_losses:
                self.loss_image_list += [float(x) for x in torch.stack(img_losses).tolist()]
            return self.textures
        light = None
        if optim_light:
            if svbrdf_obj is None or not hasattr(svbrdf_obj, "cl"):
                raise ValueError("optim_light needs svbrdf_obj with the scene's cl = [camera, light, light power]")
            light = torch.as_tensor(svbrdf_obj.cl[2]).detach().to(self.device, torch.float32).clone()
            light.requires_grad_(True)
            svbrdf_obj.cl[2] = light
        opt = None
        for epoch in range(total):
            phase_latent = (epoch % cycle) < l_ep
            params = ([self.latent] if phase_latent else list(self.noises)) + ([light] if light is not None else [])
            if opt is None or reset_adam_each_iter or getattr(self, "_phase", None) != phase_latent:
                opt = torch.optim.Adam(params, lr=lr, betas=(0.9, 0.999))
            self._phase = phase_latent
            if light is not None:
                self.renderer_obj.update_light(light)
            textures = self.latent_to_textures()
            rendered = self.renderer_obj.eval(textures)
            loss = torch.nn.functional.mse_loss(rendered, self.targets)
            img_losses.append(loss.detach())
            desc = self._descriptor_for(phase_latent)
            if desc is not None:
                from .descriptor import descriptor_term

                fl = descriptor_term(rendered, desc) * self.descriptor_weight
                feat_losses.append(fl.detach())
                loss = loss + fl
            opt.zero_grad()
            loss.backward()
            opt.step()
        self.textures = self.latent_to_textures().detach()
        if img_losses:
            self.loss_image_list += [float(x) for x in torch.stack(img_losses).tolist()]
        if feat_losses:
            self.loss_feature_list += [float(x) for x in torch.stack(feat_losses).tolist()]
        return self.textures


def upsample_textures(textures: torch.Tensor, res: int) -> torch.Tensor:
    """Lanczos up-sampling of [B, 9, r, r] maps to res (the reference resizes the saved PNG maps,
    src/svbrdf.py:155-158, src/imageio.py:75-76), normal xy renormalised with z >= 0."""
    from .imageio import imresize

    b, c, r, _ = textures.shape
    x = textures.permute(0, 2, 3, 1)  # [B, r, r, 9]
    out = torch.stack([imresize(x[i], (res, res)) for i in range(b)])
    out = out.permute(0, 3, 1, 2).contiguous().clamp(-1, 1)
    nxy = out[:, 3:5]
    norm = nxy.pow(2).sum(1, keepdim=True).clamp_min(1.0).sqrt()
    out[:, 3:5] = nxy / norm
    return out
