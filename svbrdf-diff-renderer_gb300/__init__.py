"""GB300-native (sm_103a) differentiable SVBRDF renderer and per-pixel optimiser.

Drop-ins for the hot path of tflsguoyu/svbrdf-diff-renderer:

* ``Microfacet`` - the flash-lit GGX/Cook-Torrance renderer (src/microfacet.py), with a
  hand-written adjoint behind torch.autograd;
* ``SvbrdfOptim`` - the per-pixel Adam loop (src/svbrdf.py:15-83) as one fused
  render+adjoint+Adam kernel per iteration;
* ``BatchedOptim`` - many materials of uneven size in one persistent launch per iteration;
* ``BatchedPipeline`` - a stream of such batches, double-buffered so the host transfers
  overlap the compute.

The package directory name contains hyphens; import it with
``importlib.import_module("svbrdf-diff-renderer_gb300")``.
"""
from . import _native
from ._native import SvbrdfError, build
from .batched import BatchConfig, BatchedOptim, BatchedPipeline, autotune
from .microfacet import Microfacet
from .svbrdf import SvbrdfIO, SvbrdfOptim
from .scripts import gen_textures_from_materialgan, optim_ganlatent, optim_perpixel, render, render_envmap
from . import descriptor, envmap, imageio, materialgan, scenes
from .envmap import EnvmapRenderer

__all__ = ["Microfacet", "SvbrdfOptim", "SvbrdfIO", "optim_perpixel", "render", "BatchedOptim", "BatchedPipeline",
           "EnvmapRenderer", "render_envmap", "optim_ganlatent", "gen_textures_from_materialgan",
           "BatchConfig",
           "autotune", "SvbrdfError", "build", "scenes", "imageio", "descriptor", "materialgan", "_native"]
