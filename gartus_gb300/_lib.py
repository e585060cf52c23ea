"""Loads libgartus_gpu.so (built in-tree by gartus_gb300.build) and declares its C ABI.

There is no fallback: if the library is missing or fails to load, every entry point
raises.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

from . import abi

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libgartus_gpu.so"
_lock = threading.Lock()
_lib = None


class GartusError(RuntimeError):
    """A gt_status other than GT_OK, with the library's message."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{abi.STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def _declare(L: C.CDLL) -> None:
    P = C.POINTER
    st = C.c_int
    sig = {
        "gt_abi_version": (C.c_uint32, []),
        "gt_last_error": (C.c_char_p, []),
        "gt_camera_default": (st, [C.c_uint32, C.c_double, P(abi.gt_camera_desc)]),
        "gt_camera_image_size": (st, [P(abi.gt_camera_desc), P(C.c_uint32), P(C.c_uint32), P(C.c_uint32)]),
        "gt_context_create": (st, [C.c_int, P(C.c_void_p)]),
        "gt_context_destroy": (None, [C.c_void_p]),
        "gt_scene_create": (st, [C.c_void_p, P(abi.gt_scene_desc), P(C.c_void_p)]),
        "gt_scene_destroy": (None, [C.c_void_p]),
        "gt_scene_bvh_node_count": (st, [C.c_void_p, P(C.c_uint32)]),
        "gt_scene_update_primitives": (st, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p]),
        "gt_scene_emissive_targets": (st, [C.c_void_p, C.c_void_p, C.c_uint32, P(C.c_uint32)]),
        "gt_lights_create": (st, [C.c_void_p, C.c_void_p, C.c_uint32, P(C.c_void_p)]),
        "gt_lights_destroy": (None, [C.c_void_p]),
        "gt_environment_create": (st, [C.c_void_p, P(abi.gt_environment_desc), P(C.c_void_p)]),
        "gt_environment_destroy": (None, [C.c_void_p]),
        "gt_render": (st, [C.c_void_p, C.c_void_p, C.c_void_p, P(abi.gt_camera_desc), P(abi.gt_render_opts),
                           P(abi.gt_frame)]),
        "gt_trace_rays": (st, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_double, C.c_double, C.c_void_p,
                               C.c_void_p, P(abi.gt_bvh_stats)]),
        "gt_trace_primary": (st, [C.c_void_p, P(abi.gt_camera_desc), C.c_uint32, C.c_void_p, C.c_void_p,
                                  P(abi.gt_bvh_stats)]),
        "gt_trace_rays_f32": (st, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_double, C.c_double, C.c_void_p,
                                   C.c_void_p, C.c_void_p, P(abi.gt_trace_report)]),
        "gt_trace_primary_f32": (st, [C.c_void_p, P(abi.gt_camera_desc), C.c_uint32, C.c_void_p, C.c_void_p,
                                      C.c_void_p, P(abi.gt_trace_report)]),
        "gt_render_noalloc": (st, [C.c_void_p, C.c_void_p, C.c_void_p, P(abi.gt_camera_desc), C.c_void_p,
                                   C.c_void_p]),
        "gt_render_batch": (st, [C.c_void_p, C.c_void_p, C.c_void_p, P(abi.gt_frame_job), C.c_uint32,
                                 P(abi.gt_render_opts)]),
        "gt_accumulator_create": (st, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, P(C.c_void_p)]),
        "gt_accumulator_destroy": (None, [C.c_void_p]),
        "gt_accumulator_samples": (st, [C.c_void_p, P(C.c_uint32)]),
        "gt_accumulator_save": (st, [C.c_void_p, C.c_void_p, C.c_uint64, P(C.c_uint64)]),
        "gt_accumulator_load": (st, [C.c_void_p, C.c_void_p, C.c_uint64]),
        "gt_render_accumulate": (st, [C.c_void_p, C.c_void_p, C.c_void_p, P(abi.gt_camera_desc), C.c_uint32,
                                      C.c_void_p, P(abi.gt_render_opts), P(abi.gt_frame)]),
        "gt_autotune": (st, [C.c_void_p, C.c_void_p, C.c_void_p, P(abi.gt_frame_job), C.c_uint32,
                             P(abi.gt_render_opts), P(abi.gt_autotune_report)]),
        "gt_denoiser_create": (st, [C.c_void_p, C.c_uint64, P(C.c_void_p)]),
        "gt_denoiser_destroy": (None, [C.c_void_p]),
        "gt_denoiser_param_count": (st, [C.c_void_p, P(C.c_uint64)]),
        "gt_denoiser_get_params": (st, [C.c_void_p, C.c_void_p, C.c_uint64]),
        "gt_denoiser_set_params": (st, [C.c_void_p, C.c_void_p, C.c_uint64]),
        "gt_denoiser_train_step": (st, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32,
                                        C.c_uint32, C.c_uint32, C.c_float, P(C.c_float), C.c_void_p]),
        "gt_denoise": (st, [C.c_void_p, P(abi.gt_denoise_input), C.c_uint32, C.c_float, C.c_void_p, C.c_void_p,
                            P(C.c_uint32)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args


def lib() -> C.CDLL:
    """The loaded library; raises if it has not been built."""
    global _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise RuntimeError(
                    f"{LIB_PATH} is missing: build it with `python -m gartus_gb300.build` "
                    "(or __graft_entry__.build()) before rendering")
            L = C.CDLL(str(LIB_PATH))
            _declare(L)
            if L.gt_abi_version() != abi.GT_ABI_VERSION:
                raise RuntimeError("libgartus_gpu.so ABI version does not match gartus_gb300.abi")
            _lib = L
        return _lib


def check(status: int) -> None:
    if status != abi.GT_OK:
        msg = lib().gt_last_error()
        raise GartusError(status, msg.decode() if msg else "")


EXPORTED_SYMBOLS = [
    "gt_abi_version", "gt_last_error", "gt_camera_default", "gt_camera_image_size", "gt_context_create",
    "gt_context_destroy", "gt_scene_create", "gt_scene_destroy", "gt_scene_bvh_node_count", "gt_scene_update_primitives",
    "gt_scene_emissive_targets", "gt_lights_create", "gt_lights_destroy", "gt_environment_create",
    "gt_environment_destroy", "gt_render", "gt_trace_rays", "gt_trace_primary", "gt_trace_rays_f32",
    "gt_trace_primary_f32", "gt_render_noalloc",
    "gt_render_batch", "gt_accumulator_create", "gt_accumulator_destroy", "gt_accumulator_samples",
    "gt_accumulator_save", "gt_accumulator_load", "gt_render_accumulate", "gt_autotune", "gt_denoiser_create",
    "gt_denoiser_destroy", "gt_denoiser_param_count", "gt_denoiser_get_params", "gt_denoiser_set_params",
    "gt_denoiser_train_step", "gt_denoise",
]
