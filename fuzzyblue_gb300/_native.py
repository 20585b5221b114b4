"""ctypes bindings of lib/libfuzzyblue_cuda.so (the C ABI of include/fuzzyblue.h).

The library is the only compute path: if it is missing, importing the API
raises instead of falling back to anything else. Build it with
`python -m fuzzyblue_gb300.build` (or `__graft_entry__.build()`).
"""
from __future__ import annotations

import ctypes
import os

from .params import c_params

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libfuzzyblue_cuda.so")

FB_OK = 0
FB_NOT_READY = 1
FB_ERR_INVALID_ARGUMENT = -1
FB_ERR_INVALID_PARAMS = -2
FB_ERR_OUT_OF_MEMORY = -3
FB_ERR_CUDA = -4
FB_ERR_BUDGET = -5
FB_ERR_CANCELLED = -6
FB_ERR_NOT_FOUND = -7
FB_ERR_SHUTDOWN = -8
FB_ERR_NO_KERNEL = -9


class c_draw_parameters(ctypes.Structure):
    """fb_draw_parameters: inverse_viewproj[column][row], camera (km), sun direction."""
    _fields_ = [("inverse_viewproj", (ctypes.c_float * 4) * 4), ("camera_position", ctypes.c_float * 3),
                ("_pad0", ctypes.c_float), ("sun_direction", ctypes.c_float * 3), ("_pad1", ctypes.c_float)]


class c_extent(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("depth", ctypes.c_uint32)]


class c_tables(ctypes.Structure):
    _fields_ = [
        ("transmittance", ctypes.c_void_p),
        ("irradiance", ctypes.c_void_p),
        ("scattering", ctypes.c_void_p),
        ("transmittance_extent", c_extent),
        ("irradiance_extent", c_extent),
        ("scattering_extent", c_extent),
    ]


class c_intermediates(ctypes.Structure):
    _fields_ = [
        ("delta_irradiance", ctypes.c_void_p * 2),
        ("delta_rayleigh", ctypes.c_void_p),
        ("delta_mie", ctypes.c_void_p),
        ("delta_multiple_scattering", ctypes.c_void_p),
        ("scattering_density", ctypes.c_void_p),
        ("scattering_density_stride", ctypes.c_uint32),
    ]


class c_server_config(ctypes.Structure):
    _fields_ = [
        ("hbm_budget_bytes", ctypes.c_uint64),
        ("max_batch", ctypes.c_uint32),
        ("max_inflight", ctypes.c_uint32),
        ("cache_entries", ctypes.c_uint32),
        ("max_queue", ctypes.c_uint32),
        ("reserved", ctypes.c_uint32 * 6),
    ]


class c_server_stats(ctypes.Structure):
    _fields_ = [
        ("submitted", ctypes.c_uint64),
        ("completed", ctypes.c_uint64),
        ("rejected", ctypes.c_uint64),
        ("cancelled", ctypes.c_uint64),
        ("cache_hits", ctypes.c_uint64),
        ("evictions", ctypes.c_uint64),
        ("batches", ctypes.c_uint64),
        ("resident_bytes", ctypes.c_uint64),
        ("inflight_bytes", ctypes.c_uint64),
        ("queued", ctypes.c_uint64),
        ("p50_ms", ctypes.c_double),
        ("p99_ms", ctypes.c_double),
        ("mean_ms", ctypes.c_double),
        ("mean_batch", ctypes.c_double),
    ]


class c_tile_shape(ctypes.Structure):
    _fields_ = [
        ("density_columns", ctypes.c_uint32),
        ("density_rows", ctypes.c_uint32),
        ("density_variant", ctypes.c_uint32),
        ("multiple_variant", ctypes.c_uint32),
        ("density_ms", ctypes.c_float),
        ("multiple_ms", ctypes.c_float),
    ]


class c_launch_profile(ctypes.Structure):
    _fields_ = [
        ("kernel", ctypes.c_uint32),
        ("order", ctypes.c_uint32),
        ("precision", ctypes.c_uint32),
        ("grid", ctypes.c_uint32),
        ("items", ctypes.c_uint64),
        ("texels", ctypes.c_uint64),
        ("ms", ctypes.c_float),
        ("_pad", ctypes.c_float),
    ]


KERNEL_NAMES = {0: "transmittance", 1: "single+direct", 2: "density+indirect", 3: "multiple"}

ALLOC_FN = ctypes.CFUNCTYPE(ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p)
FREE_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p)

_V = ctypes.c_void_p
_P = ctypes.POINTER(c_params)
_I = ctypes.c_int
_U32 = ctypes.c_uint32
_U64 = ctypes.c_uint64

# name -> (restype, argtypes); every symbol include/fuzzyblue.h declares.
SIGNATURES = {
    "fb_params_default": (None, [_P]),
    "fb_params_validate": (_I, [_P]),
    "fb_params_extents": (_I, [_P, ctypes.POINTER(c_extent), ctypes.POINTER(c_extent), ctypes.POINTER(c_extent)]),
    "fb_params_device_bytes": (_I, [_P, ctypes.POINTER(_U64), ctypes.POINTER(_U64)]),
    "fb_builder_create": (_I, [_I, ctypes.POINTER(_V)]),
    "fb_builder_destroy": (None, [_V]),
    "fb_builder_device": (_I, [_V, ctypes.POINTER(_I)]),
    "fb_builder_sm_count": (_I, [_V, ctypes.POINTER(_I)]),
    "fb_builder_set_allocator": (_I, [_V, ALLOC_FN, FREE_FN, _V]),
    "fb_atmosphere_build": (_I, [_V, _V, _P, ctypes.POINTER(_V)]),
    "fb_pending_query": (_I, [_V]),
    "fb_pending_wait": (_I, [_V]),
    "fb_pending_acquire": (_I, [_V, _V]),
    "fb_pending_count": (_I, [_V, ctypes.POINTER(_U32)]),
    "fb_pending_atmosphere": (_I, [_V, _U32, ctypes.POINTER(_V)]),
    "fb_pending_take": (_I, [_V, _U32, ctypes.POINTER(_V)]),
    "fb_pending_intermediates": (_I, [_V, _U32, ctypes.POINTER(c_intermediates)]),
    "fb_pending_release": (None, [_V]),
    "fb_atmosphere_tables": (_I, [_V, ctypes.POINTER(c_tables)]),
    "fb_atmosphere_copy_to_host": (_I, [_V, _V, _V, _V, _V]),
    "fb_atmosphere_copy_to_host_async": (_I, [_V, _V, _V, _V, _V]),
    "fb_atmosphere_export_scattering_f16": (_I, [_V, _V, _V]),
    "fb_atmosphere_params": (_I, [_V, _P]),
    "fb_atmosphere_destroy": (None, [_V]),
    "fb_batch_build": (_I, [_V, _V, _P, _U32, ctypes.POINTER(_V)]),
    "fb_atmosphere_build_noalloc": (_I, [_V, _P, _V, _V, _V]),
    "fb_atmosphere_render_sky": (_I, [_V, _V, ctypes.POINTER(c_draw_parameters), _V, _U32, _U32, _V, _V]),
    "fb_atmosphere_sun_and_sky_irradiance": (_I, [_V, _V, _V, _V, ctypes.POINTER(ctypes.c_float), _U32, _V, _V]),
    "fb_builder_set_profiling": (_I, [_V, _I]),
    "fb_builder_autotune": (_I, [_V, _P, _U32, _U32]),
    "fb_builder_tuned_shape": (_I, [_V, _P, ctypes.POINTER(c_tile_shape)]),
    "fb_builder_save_tuning": (_I, [_V, ctypes.c_char_p]),
    "fb_builder_load_tuning": (_I, [_V, ctypes.c_char_p]),
    "fb_server_config_default": (None, [ctypes.POINTER(c_server_config)]),
    "fb_server_create": (_I, [_V, ctypes.POINTER(c_server_config), ctypes.POINTER(_V)]),
    "fb_server_submit": (_I, [_V, _P, ctypes.POINTER(_U64)]),
    "fb_server_poll": (_I, [_V, _U64, ctypes.POINTER(_V)]),
    "fb_server_wait": (_I, [_V, _U64, _U32, ctypes.POINTER(_V)]),
    "fb_server_release": (_I, [_V, _U64]),
    "fb_server_completed": (_I, [_V, ctypes.POINTER(_U64), _U32, _U32, ctypes.POINTER(_U32)]),
    "fb_server_cancel": (_I, [_V, _U64]),
    "fb_server_get_stats": (_I, [_V, ctypes.POINTER(c_server_stats)]),
    "fb_server_destroy": (None, [_V]),
    "fb_pending_profile": (_I, [_V, ctypes.POINTER(c_launch_profile), _U32, ctypes.POINTER(_U32)]),
    "fb_status_string": (ctypes.c_char_p, [_I]),
    "fb_last_error": (ctypes.c_char_p, []),
    "fb_abi_version": (_I, []),
}

_lib = None


def lib():
    """Loads the library (once). Raises OSError when it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError("libfuzzyblue_cuda.so is not built (%s); run python -m fuzzyblue_gb300.build" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class FuzzyblueError(RuntimeError):
    def __init__(self, status, what):
        L = lib()
        msg = L.fb_last_error().decode(errors="replace")
        super().__init__("%s: %s (%d)%s" % (what, L.fb_status_string(status).decode(), status,
                                           (": " + msg) if msg else ""))
        self.status = status


def check(status, what):
    if status < 0:
        raise FuzzyblueError(status, what)
    return status
