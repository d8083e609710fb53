"""ctypes binding of the C ABI in include/renderx.h (librenderx_gb300.so).

There is no fallback: if the library cannot be built or loaded, every entry point
raises. Device buffers are passed as raw CUDA pointers (e.g. ``tensor.data_ptr()``).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

RX_OK = 0
STATUS = {0: "RX_OK", 1: "RX_ERR_INVALID", 2: "RX_ERR_CUDA", 3: "RX_ERR_OOM", 4: "RX_ERR_STATE",
          5: "RX_ERR_TIMEOUT", 6: "RX_ERR_UNSUPPORTED"}


class RxError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class rx_object(ctypes.Structure):
    _fields_ = [("tri_begin", ctypes.c_uint32), ("tri_count", ctypes.c_uint32), ("material", ctypes.c_uint32),
                ("has_vertex_normals", ctypes.c_uint32), ("color", ctypes.c_float * 3), ("coeff", ctypes.c_float),
                ("diffuse_color", ctypes.c_float * 3), ("ior", ctypes.c_float), ("sigma_s", ctypes.c_float * 3),
                ("sigma_a", ctypes.c_float * 3), ("g", ctypes.c_float), ("decay", ctypes.c_float * 3),
                ("step_size", ctypes.c_float)]


class rx_camera(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("sight_dist", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32), ("position", ctypes.c_float * 3), ("focus", ctypes.c_float * 3),
                ("up", ctypes.c_float * 3)]


class rx_pt_options(ctypes.Structure):
    _fields_ = [("spp", ctypes.c_uint32), ("max_depth", ctypes.c_uint32), ("rr_mode", ctypes.c_uint32),
                ("nee", ctypes.c_uint32), ("seed", ctypes.c_uint64), ("paths_per_pass", ctypes.c_uint32),
                ("flags", ctypes.c_uint32), ("time_budget_s", ctypes.c_float), ("reserved", ctypes.c_uint32)]


class rx_config_info(ctypes.Structure):
    _fields_ = [("renderer", ctypes.c_char * 32), ("estimator", ctypes.c_int32), ("max_depth", ctypes.c_uint32),
                ("spp", ctypes.c_uint32), ("radius", ctypes.c_float), ("runtime_s", ctypes.c_double),
                ("num_objects", ctypes.c_uint32), ("num_triangles", ctypes.c_uint32), ("camera", rx_camera),
                ("save_path", ctypes.c_char * 256)]


class rx_batch_item(ctypes.Structure):
    _fields_ = [("scene", ctypes.c_void_p), ("camera", rx_camera), ("options", rx_pt_options),
                ("film_rgb", ctypes.c_void_p)]


class rx_batch_options(ctypes.Structure):
    _fields_ = [("paths_per_pass", ctypes.c_uint32), ("use_graph", ctypes.c_uint32), ("autotune", ctypes.c_uint32),
                ("chosen_paths_per_pass", ctypes.c_uint32), ("chosen_blocks_per_sm", ctypes.c_int32),
                ("chosen_stack", ctypes.c_int32)]


class rx_vcm_options(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_uint32), ("max_depth", ctypes.c_uint32), ("light_paths", ctypes.c_uint32),
                ("flags", ctypes.c_uint32), ("radius", ctypes.c_float), ("alpha", ctypes.c_float),
                ("seed", ctypes.c_uint64), ("time_budget_s", ctypes.c_float), ("reserved", ctypes.c_uint32)]


class rx_bpt_options(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_uint32), ("max_depth", ctypes.c_uint32), ("flags", ctypes.c_uint32),
                ("time_budget_s", ctypes.c_float), ("seed", ctypes.c_uint64)]


class rx_pm_options(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_uint32), ("max_depth", ctypes.c_uint32), ("light_paths", ctypes.c_uint32),
                ("flags", ctypes.c_uint32), ("radius", ctypes.c_float), ("alpha", ctypes.c_float),
                ("seed", ctypes.c_uint64), ("time_budget_s", ctypes.c_float), ("reserved", ctypes.c_uint32)]


class rx_render_stats(ctypes.Structure):
    _fields_ = [("extension_rays", ctypes.c_uint64), ("shadow_rays", ctypes.c_uint64), ("paths", ctypes.c_uint64),
                ("ms", ctypes.c_float), ("merge_ms", ctypes.c_float), ("merges", ctypes.c_uint64),
                ("merge_queries", ctypes.c_uint64), ("photons", ctypes.c_uint64)]


class rx_guide_options(ctypes.Structure):
    _fields_ = [("learning_rate", ctypes.c_float), ("bsdf_fraction", ctypes.c_float), ("batch", ctypes.c_uint32),
                ("train_passes", ctypes.c_uint32), ("steps_per_pass", ctypes.c_uint32),
                ("warmup_passes", ctypes.c_uint32), ("seed", ctypes.c_uint64)]


class rx_build_options(ctypes.Structure):
    _fields_ = [("split_policy", ctypes.c_int32), ("leaf_size", ctypes.c_int32), ("host_threads", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


_LIB = None

# (name, restype, argtypes) of every exported entry point of include/renderx.h
P, U32, I32, S = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int32, ctypes.c_int
# rx_snapshot_fn(user, elapsed_s, samples, film_rgb, width, height)
SNAPSHOT_FN = ctypes.CFUNCTYPE(None, P, ctypes.c_double, ctypes.c_double, ctypes.POINTER(ctypes.c_double), U32, U32)
SIGNATURES = [
    ("rx_create", S, [ctypes.POINTER(P), S]),
    ("rx_destroy", None, [P]),
    ("rx_last_error", ctypes.c_char_p, [P]),
    ("rx_version", ctypes.c_char_p, []),
    ("rx_scene_set_geometry", S, [P, P, U32, P, U32, P, P, P]),
    ("rx_scene_set_objects", S, [P, P, U32]),
    ("rx_build_accel", S, [P, P]),
    ("rx_accel_stats", S, [P, P]),
    ("rx_reftree_serialize", S, [P, U32, P, U32, I32, P, P, P, P]),
    ("rx_config_read", S, [ctypes.c_char_p, ctypes.POINTER(P), P, P, ctypes.c_size_t]),
    ("rx_host_scene_free", None, [P]),
    ("rx_host_scene_arrays", S, [P, P, P, P, P, P, P, P, P, P]),
    ("rx_scene_load_config", S, [P, ctypes.c_char_p, P]),
    ("rx_write_pfm", S, [ctypes.c_char_p, U32, U32, P]),
    ("rx_set_snapshots", S, [P, ctypes.c_double, SNAPSHOT_FN, P]),
    ("rx_trace_closest", S, [P, P, U32, P, P]),
    ("rx_trace_closest_device", S, [P, P, U32, P, P, P]),
    ("rx_trace_closest_noalloc", S, [P, P, U32, P, P, P]),
    ("rx_trace_closest_reforder_device", S, [P, P, U32, P, P, P]),
    ("rx_trace_counters", S, [P, P, S]),
    ("rx_trace_set_config", S, [P, I32, I32]),
    ("rx_trace_set_timing", S, [P, I32]),
    ("rx_trace_set_options", S, [P, I32, U32, I32]),
    ("rx_trace_set_staging", S, [P, U32]),
    ("rx_trace_set_binning", S, [P, I32, I32, I32]),
    ("rx_diag_umma_gemm", S, [P, U32, U32, U32, I32, I32, P, P, P]),
    ("rx_diag_umma_rate", S, [P, U32, U32, P, P]),
    ("rx_guide_init", S, [P, P, P]),
    ("rx_guide_get_params", S, [P, P]),
    ("rx_guide_set_params", S, [P, P]),
    ("rx_guide_eval", S, [P, P, U32, P, P]),
    ("rx_guide_eval_device", S, [P, P, U32, P, P, P]),
    ("rx_guide_gradient", S, [P, P, U32, P, P]),
    ("rx_guide_train_step", S, [P, P, U32, P, P]),
    ("rx_trace_read_timing", S, [P, P, P]),
    ("rx_render_pt", S, [P, P, P, P, P, P]),
    ("rx_render_vcm", S, [P, P, P, P, P]),
    ("rx_render_bpt", S, [P, P, P, P, P]),
    ("rx_render_pm", S, [P, P, P, P, P]),
    ("rx_render_pt_batch", S, [P, P, U32, P, P]),
]


def library_path() -> str:
    return _build.LIB


def lib():
    """Builds (when sources changed) and loads the library; raises on failure."""
    global _LIB
    if _LIB is None:
        path = _build.build()
        L = ctypes.CDLL(path, mode=ctypes.RTLD_GLOBAL)
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def ptr(a) -> ctypes.c_void_p:
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data_as(ctypes.c_void_p)
    if isinstance(a, int):
        return ctypes.c_void_p(a)
    if hasattr(a, "data_ptr"):
        return ctypes.c_void_p(a.data_ptr())
    raise TypeError(type(a))


CUDA_STREAM_LEGACY = 0x1  # cudaStreamLegacy


def stream_arg(stream):
    """None -> NULL (the context's own stream); a handle -> that stream, where handle 0
    (the legacy default stream, torch's default) is passed as cudaStreamLegacy."""
    if stream is None:
        return None
    return ctypes.c_void_p(int(stream) or CUDA_STREAM_LEGACY)


def check(ctx, status: int):
    if status != RX_OK:
        msg = lib().rx_last_error(ctx).decode() if ctx else ""
        raise RxError(status, msg)
