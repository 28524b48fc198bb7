"""Build and load the sm_103a C-ABI library (``_lib/libsvbrdf_gb300.so``) through ctypes.

The library is compiled in-tree with ``nvcc -gencode arch=compute_103a,code=sm_103a``.
There is no CPU fallback: every entry point needs this library and a CUDA device, and
``lib()`` raises if either is missing.
"""
from __future__ import annotations

import ctypes
import os
import pathlib
import subprocess
import sys
import threading
from concurrent.futures import ThreadPoolExecutor

PKG = pathlib.Path(__file__).resolve().parent
REPO = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = REPO / "include"
LIBDIR = PKG / "_lib"
LIBNAME = "libsvbrdf_gb300.so"
SOURCES = ["render.cu", "fused.cu", "conv_tc.cu", "gram_tc.cu", "conv_tf32.cu", "desc_ops.cu", "gen_ops.cu",
           "gen_nhwc.cu", "envmap.cu"]
HEADERS = ["svbrdf_math.cuh", "svbrdf_common.cuh", "svbrdf_plan.cuh", "tc_ptx.cuh"]
WORKSPACE_ERROR_OFFSET = 4
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]

_lock = threading.Lock()
_lib = None


class SvbrdfError(RuntimeError):
    """A C-ABI call returned a negative status."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"svbrdf error {code}: {msg}")
        self.code = code


def nvcc() -> str:
    cand = os.environ.get("NVCC") or "/usr/local/cuda/bin/nvcc"
    return cand if os.path.exists(cand) else "nvcc"


def lib_path() -> pathlib.Path:
    return LIBDIR / LIBNAME


def _stale(target: pathlib.Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> pathlib.Path:
    """Compile every .cu of csrc/ (in parallel) and link the shared library."""
    LIBDIR.mkdir(exist_ok=True)
    out = lib_path()
    deps = [CSRC / s for s in SOURCES] + [CSRC / h for h in HEADERS] + [INCLUDE / "svbrdf_gb300.h"]
    if not force and not _stale(out, deps):
        return out
    objdir = LIBDIR / "obj"
    objdir.mkdir(exist_ok=True)

    def compile_one(src):
        obj = objdir / (pathlib.Path(src).stem + ".o")
        cmd = [nvcc(), *ARCH, *NVCC_FLAGS, f"-I{INCLUDE}", f"-I{CSRC}", "-c", str(CSRC / src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            sys.stderr.write(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = out.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, out)
    return out


class svbrdf_material(ctypes.Structure):
    _fields_ = [
        ("textures", ctypes.c_void_p),
        ("exp_avg", ctypes.c_void_p),
        ("exp_avg_sq", ctypes.c_void_p),
        ("targets", ctypes.c_void_p),
        ("light_pow", ctypes.c_void_p),
        ("camera_pos", ctypes.c_void_p),
        ("light_pos", ctypes.c_void_p),
        ("n_views", ctypes.c_int),
        ("height", ctypes.c_int),
        ("width", ctypes.c_int),
        ("size", ctypes.c_float),
        ("light_adam_state", ctypes.c_void_p),
    ]


class svbrdf_batch_config(ctypes.Structure):
    _fields_ = [("threads", ctypes.c_int), ("tile_texels", ctypes.c_int), ("ctas", ctypes.c_int),
                ("variant", ctypes.c_int)]


def _declare(L):
    P, I, F, S = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_size_t
    L.svbrdf_last_error.restype = ctypes.c_char_p
    L.svbrdf_last_error.argtypes = []
    L.svbrdf_abi_version.restype = I
    L.svbrdf_max_views.restype = I
    L.svbrdf_workspace_bytes.restype = S
    L.svbrdf_render_fwd.restype = I
    L.svbrdf_render_fwd.argtypes = [P, P, P, P, I, I, I, F, P, P, I, P, P, S, P]
    L.svbrdf_render_bwd.restype = I
    L.svbrdf_render_bwd.argtypes = [P, P, P, P, I, I, I, F, P, P, P, P, S, P]
    L.svbrdf_render_fwd_batch.restype = I
    L.svbrdf_render_fwd_batch.argtypes = [P, P, P, P, I, I, I, F, I, P, P, I, P, P, S, P]
    L.svbrdf_render_bwd_batch.restype = I
    L.svbrdf_render_bwd_batch.argtypes = [P, P, P, P, I, I, I, F, I, P, P, P, P, S, P]
    L.svbrdf_fused_step.restype = I
    L.svbrdf_fused_step.argtypes = [P, P, P, P, P, P, P, P, I, I, I, F, I, I, F, F, F, F, P, P, S, P]
    L.svbrdf_fused_step_noalloc.restype = I
    L.svbrdf_fused_step_noalloc.argtypes = [P, P, P, P, P, P, P, P, I, I, I, F, I, I, F, F, F, F, P, P]
    L.svbrdf_conv3x3_bf16.restype = I
    L.svbrdf_conv3x3_bf16.argtypes = [P, P, P, P, P, I, I, I, I, I, I, P, P]
    L.svbrdf_conv3x3_bf16_ex.restype = I
    L.svbrdf_conv3x3_bf16_ex.argtypes = [P, P, P, P, P, P, I, I, I, I, I, I, P, P]
    L.svbrdf_desc_partials.restype = I
    L.svbrdf_desc_conv1_fwd.restype = I
    L.svbrdf_desc_conv1_fwd.argtypes = [P, P, P, P, P, I, I, I, I, P]
    L.svbrdf_desc_conv1_bwd.restype = I
    L.svbrdf_desc_conv1_bwd.argtypes = [P, P, P, I, I, I, I, P]
    L.svbrdf_desc_conv1_bwd_tc.restype = I
    L.svbrdf_desc_conv1_bwd_tc.argtypes = [P, P, P, P, I, I, I, I, P, P]
    L.svbrdf_desc_pool_fwd.restype = I
    L.svbrdf_desc_pool_fwd.argtypes = [P, P, I, I, I, I, P]
    L.svbrdf_desc_pool_bwd.restype = I
    L.svbrdf_desc_pool_bwd.argtypes = [P, P, P, P, I, I, I, I, P]
    L.svbrdf_desc_avgpool_fwd.restype = I
    L.svbrdf_desc_avgpool_fwd.argtypes = [P, P, I, I, I, I, P]
    L.svbrdf_desc_avgpool_bwd.restype = I
    L.svbrdf_desc_avgpool_bwd.argtypes = [P, P, P, P, I, I, I, I, P]
    L.svbrdf_desc_feat_loss.restype = I
    L.svbrdf_desc_feat_loss.argtypes = [P, I, P, P, F, I, P, P, ctypes.c_longlong, P]
    L.svbrdf_desc_loss_sums.restype = I
    L.svbrdf_desc_loss_sums.argtypes = [P, I, P, P, P, P, P, P]
    L.svbrdf_desc_gram_splits.restype = I
    L.svbrdf_desc_gram_splits.argtypes = [I, I, I]
    L.svbrdf_desc_gram.restype = I
    L.svbrdf_desc_gram.argtypes = [P, P, I, I, I, I, P, P]
    L.svbrdf_desc_gram_finish.restype = I
    L.svbrdf_desc_gram_finish.argtypes = [P, I, I, I, I, P, F, P, P, P, P]
    L.svbrdf_desc_gemm_nt.restype = I
    L.svbrdf_desc_gemm_nt.argtypes = [P, P, P, I, I, I, I, P, P]
    L.svbrdf_desc_gemm_nt_feat_partials.restype = ctypes.c_longlong
    L.svbrdf_desc_gemm_nt_feat_partials.argtypes = [I, I, I]
    L.svbrdf_desc_gemm_nt_feat.restype = I
    L.svbrdf_desc_gemm_nt_feat.argtypes = [P, P, P, I, P, F, I, P, P, I, I, I, I, P, P]
    L.svbrdf_gen_conv_tf32.restype = I
    L.svbrdf_gen_conv_tf32.argtypes = [P, P, P, I, I, I, I, I, I, I, P, P]
    L.svbrdf_gen_conv_tf32_ws_bytes.restype = ctypes.c_longlong
    L.svbrdf_gen_conv_tf32_ws_bytes.argtypes = [I, I, I, I, I, I, I]
    L.svbrdf_gen_conv_tf32_ex.restype = I
    L.svbrdf_gen_conv_tf32_ex.argtypes = [P, P, P, P, ctypes.c_longlong, I, I, I, I, I, I, I, P, P]
    L.svbrdf_gen_upsample2.restype = I
    L.svbrdf_gen_upsample2.argtypes = [P, P, ctypes.c_longlong, I, I, P]
    L.svbrdf_gen_upsample2_scaled.restype = I
    L.svbrdf_gen_upsample2_scaled.argtypes = [P, P, P, ctypes.c_longlong, I, I, P]
    L.svbrdf_gen_upsample2_bwd.restype = I
    L.svbrdf_gen_upsample2_bwd.argtypes = [P, P, ctypes.c_longlong, I, I, P]
    L.svbrdf_gen_scale.restype = I
    L.svbrdf_gen_scale.argtypes = [P, P, P, ctypes.c_longlong, I, P]
    L.svbrdf_gen_scale_bwd.restype = I
    L.svbrdf_gen_scale_bwd.argtypes = [P, P, P, P, P, ctypes.c_longlong, I, P]
    L.svbrdf_gen_act.restype = I
    L.svbrdf_gen_act.argtypes = [P, P, P, P, P, F, P, I, I, I, P]
    L.svbrdf_gen_act_bwd.restype = I
    L.svbrdf_gen_act_bwd.argtypes = [P, P, P, P, P, P, F, P, P, P, I, I, I, P]
    L.svbrdf_gen_nhwc_partial_floats.restype = I
    L.svbrdf_gen_nhwc_partial_floats.argtypes = [I, I]
    L.svbrdf_gen_upsample2_nhwc.restype = I
    L.svbrdf_gen_upsample2_nhwc.argtypes = [P, P, P, I, I, I, I, I, P]
    L.svbrdf_gen_upsample2_nhwc_bwd.restype = I
    L.svbrdf_gen_upsample2_nhwc_bwd.argtypes = [P, P, I, I, I, I, I, P]
    L.svbrdf_gen_rgb_nhwc.restype = I
    L.svbrdf_gen_rgb_nhwc.argtypes = [P, I, P, P, P, I, I, I, I, P]
    L.svbrdf_gen_rgb_nhwc_bwd.restype = I
    L.svbrdf_gen_rgb_nhwc_bwd.argtypes = [P, P, I, I, I, I, I, P]
    L.svbrdf_gen_scale_nhwc.restype = I
    L.svbrdf_gen_scale_nhwc.argtypes = [P, P, P, I, I, I, P]
    L.svbrdf_gen_scale_nhwc_bwd.restype = I
    L.svbrdf_gen_scale_nhwc_bwd.argtypes = [P, P, P, P, P, P, I, I, I, P]
    L.svbrdf_gen_act_nhwc.restype = I
    L.svbrdf_gen_act_nhwc.argtypes = [P, P, P, P, P, F, P, I, I, I, P]
    L.svbrdf_gen_act_nhwc_bwd.restype = I
    L.svbrdf_gen_act_nhwc_bwd.argtypes = [P, P, P, P, P, P, F, P, P, P, P, I, I, I, P]
    L.svbrdf_gen_act_scale_nhwc.restype = I
    L.svbrdf_gen_act_scale_nhwc.argtypes = [P, P, P, P, P, F, P, P, I, I, I, P]
    L.svbrdf_gen_act_scale_nhwc_bwd.restype = I
    L.svbrdf_gen_act_scale_nhwc_bwd.argtypes = [P, P, P, P, P, P, F, P, P, P, P, P, P, P, I, I, I, P]
    L.svbrdf_selftest_wait_timeout.restype = I
    L.svbrdf_selftest_wait_timeout.argtypes = [P, S, I, P]
    L.svbrdf_envmap_render.restype = I
    L.svbrdf_envmap_render.argtypes = [P, I, I, P, I, I, P, P, P, P, P, I, F, F, I, ctypes.c_uint, P]
    L.svbrdf_batched_plan_bytes.restype = S
    L.svbrdf_batched_plan_bytes.argtypes = [ctypes.POINTER(svbrdf_material), I, ctypes.POINTER(svbrdf_batch_config)]
    L.svbrdf_batched_plan.restype = I
    L.svbrdf_batched_plan.argtypes = [ctypes.POINTER(svbrdf_material), I, ctypes.POINTER(svbrdf_batch_config), P, S]
    L.svbrdf_batched_workspace_bytes.restype = S
    L.svbrdf_batched_workspace_bytes.argtypes = [P]
    L.svbrdf_batched_step.restype = I
    L.svbrdf_batched_step.argtypes = [P, P, I, P, F, F, F, F, P, I, P, S, P]
    L.svbrdf_batched_steps.restype = I
    L.svbrdf_batched_steps.argtypes = [P, P, I, P, F, F, F, F, P, I, I, P, S, P]
    return L


# Every symbol include/svbrdf_gb300.h declares.
EXPORTS = [
    "svbrdf_last_error", "svbrdf_abi_version", "svbrdf_max_views", "svbrdf_workspace_bytes",
    "svbrdf_render_fwd", "svbrdf_render_bwd", "svbrdf_render_fwd_batch", "svbrdf_render_bwd_batch",
    "svbrdf_fused_step", "svbrdf_fused_step_noalloc",
    "svbrdf_batched_plan_bytes",
    "svbrdf_batched_plan", "svbrdf_batched_workspace_bytes", "svbrdf_batched_step", "svbrdf_batched_steps", "svbrdf_conv3x3_bf16",
    "svbrdf_conv3x3_bf16_ex", "svbrdf_desc_partials", "svbrdf_desc_conv1_fwd", "svbrdf_desc_conv1_bwd", "svbrdf_desc_conv1_bwd_tc",
    "svbrdf_desc_pool_fwd", "svbrdf_desc_pool_bwd", "svbrdf_desc_avgpool_fwd", "svbrdf_desc_avgpool_bwd",
    "svbrdf_desc_feat_loss", "svbrdf_desc_loss_sums", "svbrdf_desc_gram_splits", "svbrdf_desc_gram", "svbrdf_desc_gram_finish",
    "svbrdf_desc_gemm_nt", "svbrdf_desc_gemm_nt_feat_partials", "svbrdf_desc_gemm_nt_feat",
    "svbrdf_gen_upsample2",
    "svbrdf_gen_upsample2_bwd", "svbrdf_gen_upsample2_scaled", "svbrdf_gen_scale", "svbrdf_gen_scale_bwd", "svbrdf_gen_act", "svbrdf_gen_act_bwd",
    "svbrdf_gen_nhwc_partial_floats", "svbrdf_gen_upsample2_nhwc", "svbrdf_gen_upsample2_nhwc_bwd",
    "svbrdf_gen_rgb_nhwc", "svbrdf_gen_rgb_nhwc_bwd",
    "svbrdf_gen_scale_nhwc", "svbrdf_gen_scale_nhwc_bwd", "svbrdf_gen_act_nhwc", "svbrdf_gen_act_nhwc_bwd",
    "svbrdf_gen_act_scale_nhwc", "svbrdf_gen_act_scale_nhwc_bwd",
    "svbrdf_gen_conv_tf32", "svbrdf_gen_conv_tf32_ws_bytes", "svbrdf_gen_conv_tf32_ex",
    "svbrdf_envmap_render", "svbrdf_selftest_wait_timeout",
]


def load(path=None):
    """Load (building first if needed) the library without requiring a GPU."""
    global _lib
    with _lock:
        if _lib is None:
            p = pathlib.Path(path) if path else build()
            _lib = _declare(ctypes.CDLL(str(p)))
        return _lib


_build_id = None


def build_id() -> str:
    """ABI version and a hash of the loaded library file: tuning results and other cached
    choices are keyed on it, so a rebuilt library never reuses a stale pick."""
    global _build_id
    if _build_id is None:
        import hashlib

        L = load()
        h = hashlib.sha1(lib_path().read_bytes()).hexdigest()[:12]
        _build_id = f"abi{L.svbrdf_abi_version()}-{h}"
    return _build_id


def lib():
    """The loaded library, for compute calls: raises when no CUDA device is present."""
    import torch

    if not torch.cuda.is_available():
        raise RuntimeError("svbrdf-diff-renderer_gb300 needs a CUDA device (sm_103a); there is no CPU fallback")
    return load()


def check(rc: int):
    if rc != 0:
        msg = load().svbrdf_last_error().decode(errors="replace")
        raise SvbrdfError(rc, msg)


def ptr(t) -> int:
    return 0 if t is None else t.data_ptr()


def stream_handle(device=None) -> int:
    import torch

    return torch.cuda.current_stream(device).cuda_stream
