"""Loads libphoton_cuda.so and declares the C-ABI of include/photon_cuda.h and
include/photon_pbrt.h.

The product path has no fallback: when the library is missing or fails to
load, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os

from . import _abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libphoton_cuda.so")

# name -> (restype, argtypes); every symbol the headers in include/ declare.
vp = C.c_void_p
SIGNATURES = {
    "phc_material_default": (None, [vp]),
    "phc_sampler_default": (None, [vp]),
    "phc_light_default": (None, [vp]),
    "phc_volume_default": (None, [vp]),
    "phc_camera_default": (None, [vp]),
    "phc_settings_default": (None, [vp]),
    "phc_scene_desc_default": (None, [vp]),
    "phc_abi_version": (C.c_int, []),
    "phc_global_error": (C.c_char_p, []),
    "phc_create": (C.c_int, [C.POINTER(vp)]),
    "phc_destroy": (None, [vp]),
    "phc_backend_name": (C.c_char_p, [vp]),
    "phc_set_scene": (C.c_int, [vp, vp]),
    "phc_render": (C.c_int, [vp, vp, vp, C.c_int]),
    "phc_accumulated_samples": (C.c_uint32, [vp]),
    "phc_read_color": (C.c_int, [vp, vp]),
    "phc_read_depth": (C.c_int, [vp, vp]),
    "phc_read_normal": (C.c_int, [vp, vp]),
    "phc_read_albedo": (C.c_int, [vp, vp]),
    "phc_render_stats_get": (C.c_int, [vp, vp]),
    "phc_scene_table": (C.c_int, [vp, C.c_int32, vp, C.c_uint64, C.POINTER(C.c_uint64)]),
    "phc_render_batch": (C.c_int, [vp, C.c_uint32, vp]),
    "phc_last_error": (C.c_char_p, [vp]),
    "phc_adjoint": (C.c_int, [vp, vp, vp, C.c_uint32, vp, vp]),
    "phc_adjoint_sizes": (C.c_int, [vp, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "phc_accel_create": (C.c_int, [C.POINTER(vp), vp, C.c_uint64, vp, C.c_uint64, vp, vp]),
    "phc_accel_create_instanced": (C.c_int, [C.POINTER(vp), vp, C.c_uint64, vp, C.c_uint64, vp, vp, vp, C.c_uint32,
                                             vp, C.c_uint32]),
    "phc_accel_destroy": (None, [vp]),
    "phc_trace_closest": (C.c_int, [vp, vp, vp, vp, vp, C.c_uint32, vp, vp]),
    "phc_trace_closest_compact": (C.c_int, [vp, vp, vp, vp, vp, C.c_uint32, vp, vp]),
    "phc_trace_occluded": (C.c_int, [vp, vp, vp, vp, vp, C.c_uint32, vp, vp]),
    "phc_accel_counters": (C.c_int, [vp, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "phc_accel_info": (C.c_int, [vp, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "phc_accel_error": (C.c_char_p, []),
    "phc_trace_closest_compact_static": (C.c_int, [vp, vp, vp, vp, vp, C.c_uint32, vp, vp]),
    "phc_tuning_set": (C.c_int, [C.c_char_p, C.c_int64]),
    "phc_tuning_get": (C.c_int64, [C.c_char_p]),
    # include/photon_pbrt.h
    "phc_pbrt_load": (C.c_int, [C.c_char_p, vp, C.POINTER(vp)]),
    "phc_pbrt_free": (None, [vp]),
    "phc_pbrt_scene_desc": (C.c_int, [vp, C.POINTER(vp)]),
    "phc_pbrt_camera": (C.c_int, [vp, vp]),
    "phc_pbrt_settings": (C.c_int, [vp, vp]),
    "phc_pbrt_info_get": (C.c_int, [vp, vp]),
}

_lib = None


def load(path: str = LIB_PATH):
    """The loaded library (raises when it is missing: there is no CPU path)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"libphoton_cuda.so is not built ({path}); run photon_gb300.build.build()")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


class PhotonError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{_abi.ERROR_NAMES.get(code, code)}: {msg}")
        self.code = code
