"""Pipeline drop-ins: ``gen_textures_from_materialgan``, ``render``, ``render_envmap``,
``optim_perpixel`` and ``optim_ganlatent`` (src/scripts.py:18-143).

Same arguments and file layout as the reference: a scene JSON read by ``SvbrdfIO``,
target photos ``{idx:02d}.png`` in ``target_dir``, maps ``nom/dif/spe/rgh.png`` in
``reference_dir`` / ``optimize_dir``, re-renders in ``rerender_dir``. The optimisation runs
on the fused sm_103a kernel (``SvbrdfOptim``); there is no CPU path.
"""
from __future__ import annotations

import pathlib

import torch

from .microfacet import Microfacet
from .svbrdf import SvbrdfIO, SvbrdfOptim, load_texture_maps


def gen_textures_from_materialgan(json_dir, device="cuda:0", generator=None, seed=0):
    """Maps of a random material from the generator into ``reference_dir``
    (src/scripts.py:18-28): the truncated mapping of a random z, no optimisation. The
    generator defaults to the seeded StyleGAN2-shaped one at 256 (the trained MaterialGAN
    weights are downloaded at run time by the reference and are not available offline)."""
    from .materialgan import MaterialGANOptim, StyleGAN2Generator

    io = SvbrdfIO(pathlib.Path(json_dir), device)
    gen = generator if generator is not None else StyleGAN2Generator(256, seed=seed)
    opt = MaterialGANOptim(device, None, gen)
    opt.init_from(batch=1, seed=seed, noise="random")
    with torch.no_grad():
        textures = opt.latent_to_textures().detach()
    io.save_textures_th(textures, io.reference_dir)
    return textures


def render(json_dir, res, device="cuda:0"):
    """Render the reference maps of the scene to ``target_dir`` (src/scripts.py:31-41)."""
    io = SvbrdfIO(pathlib.Path(json_dir), device)
    textures = io.load_textures_th(io.reference_dir, res)
    r = Microfacet(res, io.n_of_imgs, io.im_size, io.cl, device)
    with torch.no_grad():
        out = r.eval(textures)
    io.save_images_th(out, io.target_dir)
    return out


def render_envmap(data_dir, res, envmap=None, device="cuda:0", spp=256, seed=0):
    """The novel-view video of the maps in ``data_dir`` (src/scripts.py:44-59): the material
    (nom/dif/spe/rgh.png at their own size) under ``envmap`` (an OpenEXR path or a [He, We, 3]
    array; None: the seeded synthetic environment), written as ``data_dir/vid/000.png`` ...
    ``115.png`` (59 angles forward, then 57 back, light intensity 0.5) and packed into
    ``data_dir/vid.gif`` (40 ms a frame, looping). Returns the frames."""
    from .envmap import EnvmapRenderer
    from .imageio import img2gif, imwrite

    data_dir = pathlib.Path(data_dir)
    vid = data_dir / "vid"
    vid.mkdir(parents=True, exist_ok=True)
    textures = load_texture_maps(data_dir, None, device)
    frames = EnvmapRenderer([res, res], envmap, textures, device=device, spp=spp, seed=seed).render_video(59, 0.5)
    names = []
    for i, f in enumerate(frames):
        names.append(vid / f"{i:03d}.png")
        imwrite(f, names[-1], flag="srgb")
    img2gif(names, data_dir / "vid.gif")
    return frames


def optim_perpixel(json_dir, res, lr, epochs, tex_init, optim_light=False, device="cuda:0", loss="mse",
                   graph=True, seed=None):
    """Per-pixel SVBRDF fit (src/scripts.py:67-97): targets -> fused optimisation -> maps.

    ``tex_init`` is "random", "const" or "textures" (the maps in ``reference_dir``). Returns
    the ``SvbrdfOptim`` (its ``textures``, ``loss_image_list``, Adam moments).
    """
    io = SvbrdfIO(pathlib.Path(json_dir), device)
    targets = io.load_images_th(io.target_dir, res)
    renderer = Microfacet(res, io.n_of_imgs, io.im_size, io.cl, device)
    opt = SvbrdfOptim(device, renderer, loss=loss, graph=graph and not optim_light)
    opt.load_targets(targets)
    if tex_init == "random":
        if seed is not None:
            torch.manual_seed(seed)
        opt.init_from_randn()
    elif tex_init == "const":
        opt.init_from_const()
    elif tex_init == "textures":
        opt.init_from_tex(io.load_textures_th(io.reference_dir, res))
    else:
        raise ValueError(f"tex_init must be 'random', 'const' or 'textures', not {tex_init!r}")
    opt.optim(epochs, lr, io, optim_light)
    io.save_textures_th(opt.textures.detach().clamp(-1, 1), io.optimize_dir)
    if optim_light:
        renderer.update_light(io.cl[2].detach())
    with torch.no_grad():
        out = renderer.eval(opt.textures.detach().clamp(-1, 1))
    io.save_images_th(out, io.rerender_dir)
    return opt


def optim_ganlatent(json_dir, res, lr, epochs, tex_init, optim_light=False, device="cuda:0", generator=None,
                    seed=0, feature_loss=None):
    """MaterialGAN latent fit (src/scripts.py:100-143): targets -> latent (and noise) Adam
    through the generator and the renderer -> maps in ``optimize_dir``, re-renders in
    ``rerender_dir``.

    ``epochs`` is [total, latent epochs, noise epochs] per cycle. ``tex_init`` follows the
    reference's ``init_from`` (src/materialgan.py:58-75): [] starts from the truncated
    mapping of a random z with random noise, [latent.pt] from a saved latent with the
    average (zero) noise, [latent.pt, noise.pt] from both (``MaterialGANOptim.save_latent``'s
    files). The reference's "auto" choice between its two downloaded starting latents needs
    those checkpoints, which are not available offline. ``generator`` defaults to the
    seeded StyleGAN2-shaped generator at ``res`` (the trained MaterialGAN weights are not
    available either). ``feature_loss`` (default: on for CUDA devices) adds the reference's
    two phase-dependent VGG feature losses (``descriptor.reference_descriptors``, seeded
    weights) at 0.1; their tensor-core convolutions need ``res`` a multiple of 128 (relu4_2
    at 1/8 resolution fills the 8 x 16 tile). Returns the ``MaterialGANOptim``.
    """
    from .materialgan import MaterialGANOptim, StyleGAN2Generator

    if tex_init == "auto":
        raise ValueError("tex_init 'auto' needs the reference's latent_avg / latent_const checkpoints, which are "
                         "downloaded at run time and not available offline; pass [latent.pt] or [latent.pt, noise.pt]")
    paths = list(tex_init or [])
    if len(paths) > 2:
        raise ValueError("tex_init holds at most a latent file and a noise file")
    io = SvbrdfIO(pathlib.Path(json_dir), device)
    targets = io.load_images_th(io.target_dir, res)
    renderer = Microfacet(res, io.n_of_imgs, io.im_size, io.cl, device)
    gen = generator if generator is not None else StyleGAN2Generator(res, seed=seed)
    if feature_loss is None:
        feature_loss = torch.device(device).type == "cuda"
    desc = None
    if feature_loss:
        from .descriptor import reference_descriptors

        desc = reference_descriptors(device, seed=seed)
    opt = MaterialGANOptim(device, renderer, gen, descriptor=desc)
    opt.load_targets(targets)
    opt.init_from(batch=1, seed=seed, noise="random" if not paths else "zero")
    if paths:
        opt.load_latent(paths[0], paths[1] if len(paths) == 2 else None)
    textures = opt.optim(epochs, lr, io, optim_light)
    io.save_textures_th(textures, io.optimize_dir)
    if optim_light:
        renderer.update_light(io.cl[2].detach())
    with torch.no_grad():
        out = renderer.eval(textures)
    io.save_images_th(out, io.rerender_dir)
    return opt
