"""ctypes binding of the C ABI in include/walkray.h (libwalkray_gpu.so).

The shared library is the product; this module only declares its entry
points and structs for Python callers (tests, bench, serving driver).  There
is no Python or CPU fallback: if the library is missing, importing the
high-level API raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libwalkray_gpu.so")

WR_OK = 0
ERRORS = {
    1: "WR_ERR_INVALID_ARGUMENT",
    2: "WR_ERR_OUT_OF_MEMORY",
    3: "WR_ERR_CUDA",
    4: "WR_ERR_NOT_FOUND",
    5: "WR_ERR_TIMEOUT",
    6: "WR_ERR_BUSY",
    7: "WR_ERR_CANCELLED",
    8: "WR_ERR_UNSUPPORTED",
    9: "WR_ERR_INTERNAL",
}
WR_NO_HIT = 0xFFFFFFFF


class wr_object_desc(C.Structure):
    _fields_ = [
        ("type", C.c_uint32), ("vert_begin", C.c_uint32), ("vert_count", C.c_uint32),
        ("tri_begin", C.c_uint32), ("tri_count", C.c_uint32), ("grid_index", C.c_uint32),
        ("albedo", C.c_float * 3), ("emission", C.c_float * 3), ("power", C.c_float), ("ior", C.c_float),
        ("decay", C.c_float * 3), ("rs", C.c_float * 3), ("rd", C.c_float * 3), ("nu", C.c_float),
        ("nv", C.c_float), ("sigma_s", C.c_float * 3), ("sigma_a", C.c_float * 3), ("g", C.c_float),
        ("density_scale", C.c_float), ("step_size", C.c_float),
    ]


class wr_camera_desc(C.Structure):
    _fields_ = [
        ("position", C.c_float * 3), ("focus", C.c_float * 3), ("up", C.c_float * 3),
        ("width", C.c_uint32), ("height", C.c_uint32), ("image_plane_dist", C.c_float),
        ("lens_radius", C.c_float), ("focal_dist", C.c_float),
    ]


class wr_grid_desc(C.Structure):
    _fields_ = [
        ("nx", C.c_uint32), ("ny", C.c_uint32), ("nz", C.c_uint32), ("pad", C.c_uint32),
        ("density", C.POINTER(C.c_float)), ("p0", C.c_float * 3), ("p1", C.c_float * 3),
    ]


class wr_scene_desc(C.Structure):
    _fields_ = [
        ("num_objects", C.c_uint32), ("num_vertices", C.c_uint32), ("num_triangles", C.c_uint32),
        ("num_grids", C.c_uint32), ("objects", C.c_void_p), ("vertices", C.c_void_p),
        ("triangles", C.c_void_p), ("grids", C.c_void_p), ("camera", wr_camera_desc),
    ]


class wr_scene_file_settings(C.Structure):
    _fields_ = [("renderer", C.c_char * 32), ("spp", C.c_uint32), ("max_path_len", C.c_uint32),
                ("radius", C.c_float), ("mode", C.c_uint32)]


class wr_hit(C.Structure):
    _fields_ = [("tri", C.c_uint32), ("t", C.c_float), ("b1", C.c_float), ("b2", C.c_float)]


class wr_scene_info(C.Structure):
    _fields_ = [
        ("num_triangles", C.c_uint32), ("num_nodes", C.c_uint32), ("num_leaves", C.c_uint32),
        ("max_depth", C.c_uint32), ("device_bytes", C.c_uint64), ("build_seconds", C.c_double),
    ]


class wr_ctx_desc(C.Structure):
    _fields_ = [("device", C.c_int), ("device_memory_budget", C.c_uint64), ("flags", C.c_uint32),
                ("pad", C.c_uint32)]


class wr_trace_filter(C.Structure):
    _fields_ = [("inside_obj", C.c_void_p), ("contact_obj", C.c_void_p)]


class wr_render_desc(C.Structure):
    _fields_ = [("spp", C.c_uint32), ("max_path_len", C.c_uint32), ("seed", C.c_uint64), ("mode", C.c_uint32),
                ("flags", C.c_uint32), ("spp_offset", C.c_uint32), ("radius", C.c_float)]


class wr_wavefront_config(C.Structure):
    _fields_ = [("capacity", C.c_uint32), ("extend_block", C.c_int32), ("shade_block", C.c_int32),
                ("ctas_per_sm", C.c_int32), ("iters_per_graph", C.c_int32), ("refill_min", C.c_int32),
                ("leaf_min", C.c_int32), ("drain_paths", C.c_int32), ("pixel_tile", C.c_int32),
                ("steps_per_turn", C.c_int32), ("mpaths_per_s", C.c_double)]


class wr_serve_desc(C.Structure):
    _fields_ = [("film_bytes", C.c_uint64), ("max_active", C.c_uint32), ("flags", C.c_uint32),
                ("paths_in_flight", C.c_uint32), ("reserved", C.c_uint32)]


class wr_request_desc(C.Structure):
    _fields_ = [("scene", C.c_uint32), ("width", C.c_uint32), ("height", C.c_uint32), ("spp", C.c_uint32),
                ("max_path_len", C.c_uint32), ("flags", C.c_uint32), ("seed", C.c_uint64)]


class wr_req_status(C.Structure):
    _fields_ = [("state", C.c_uint32), ("pad", C.c_uint32), ("paths_total", C.c_uint64),
                ("paths_done", C.c_uint64), ("submit_s", C.c_double), ("admit_s", C.c_double),
                ("finish_s", C.c_double)]


class wr_render_profile(C.Structure):
    _fields_ = [("ms_extend", C.c_double), ("ms_shade", C.c_double), ("ms_shadow", C.c_double),
                ("ms_generate", C.c_double), ("ms_total", C.c_double), ("iterations", C.c_uint64),
                ("rays", C.c_uint64), ("box_tests", C.c_uint64), ("tri_tests", C.c_uint64), ("paths", C.c_uint64),
                ("ms_drain", C.c_double), ("drained_paths", C.c_uint64), ("iter_rays", C.c_uint32 * 32),
                ("iter_extend_ms", C.c_float * 32), ("iter_shade_ms", C.c_float * 32)]


WR_RENDER_NEE = 1
WR_RENDER_EXACT_TRAVERSAL = 2
WR_RENDER_NEE_MIS = 4
WR_RENDER_PHONG_MIRROR = 8
WR_CTX_EXACT_TRAVERSAL = 1
WR_SERVE_FIFO = 1

HIT_DTYPE = np.dtype([("tri", "<u4"), ("t", "<f4"), ("b1", "<f4"), ("b2", "<f4")])

assert C.sizeof(wr_object_desc) == 136
assert C.sizeof(wr_hit) == 16

# name -> (restype, argtypes)
_SIGS = {
    "wr_get_abi_version": (C.c_int, [C.POINTER(C.c_uint32)]),
    "wr_ctx_create": (C.c_int, [C.POINTER(wr_ctx_desc), C.POINTER(C.c_void_p)]),
    "wr_ctx_destroy": (C.c_int, [C.c_void_p]),
    "wr_last_error": (C.c_char_p, [C.c_void_p]),
    "wr_scene_upload": (C.c_int, [C.c_void_p, C.POINTER(wr_scene_desc), C.POINTER(C.c_uint32)]),
    "wr_scene_release": (C.c_int, [C.c_void_p, C.c_uint32]),
    "wr_scene_get_info": (C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(wr_scene_info)]),
    "wr_trace_closest": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint64, C.POINTER(wr_trace_filter),
                                   C.c_void_p]),
    "wr_trace_closest_device": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p,
                                          C.c_void_p, C.c_void_p]),
    "wr_render": (C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(wr_render_desc), C.c_void_p]),
    "wr_render_device": (C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(wr_render_desc), C.c_void_p, C.c_void_p,
                                   C.c_void_p]),
    "wr_set_wavefront_config": (C.c_int, [C.c_void_p, C.POINTER(wr_wavefront_config)]),
    "wr_autotune": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(wr_wavefront_config)]),
    "wr_profile_render": (C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(wr_render_desc), C.c_void_p,
                                    C.POINTER(wr_render_profile)]),
    "wr_serve_start": (C.c_int, [C.c_void_p, C.POINTER(wr_serve_desc)]),
    "wr_serve_stop": (C.c_int, [C.c_void_p]),
    "wr_submit": (C.c_int, [C.c_void_p, C.POINTER(wr_request_desc), C.POINTER(C.c_uint64)]),
    "wr_poll": (C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(wr_req_status)]),
    "wr_fetch": (C.c_int, [C.c_void_p, C.c_uint64, C.c_void_p]),
    "wr_cancel": (C.c_int, [C.c_void_p, C.c_uint64]),
    "wr_scene_file_load": (C.c_int, [C.c_char_p, C.POINTER(C.c_void_p), C.c_char_p, C.c_size_t]),
    "wr_scene_file_get": (C.c_int, [C.c_void_p, C.POINTER(wr_scene_desc), C.POINTER(wr_scene_file_settings)]),
    "wr_scene_file_free": (C.c_int, [C.c_void_p]),
    "wr_kdtree_build_host": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_int,
                                       C.POINTER(C.c_void_p)]),
    "wr_kdtree_host_sizes": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                       C.POINTER(C.c_uint32)]),
    "wr_kdtree_host_export": (C.c_int, [C.c_void_p] + [C.c_void_p] * 6),
    "wr_kdtree_host_free": (C.c_int, [C.c_void_p]),
    "wr_rng_draws": (C.c_int, [C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p,
                               C.c_void_p]),
    "wr_render_noalloc_status": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_uint)]),
    "wr_render_progressive": (C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(wr_render_desc), C.c_uint32, C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.POINTER(C.c_uint32)]),
}

# int (*)(void* user, const float* rgb, uint32_t spp_done)
PROGRESS_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(C.c_float), C.c_uint32)

_lib = None


def load() -> C.CDLL:
    """Load the in-tree library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run `python -m walkray_gb300.build` (no CPU fallback exists)")
        lib = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            if hasattr(lib, name):
                f = getattr(lib, name)
                f.restype = res
                f.argtypes = args
        _lib = lib
    return _lib


def declared_symbols() -> list[str]:
    """Every function declared in include/*.h (parsed from the headers)."""
    import re

    names = []
    inc = os.path.join(os.path.dirname(HERE), "include")
    for fn in sorted(os.listdir(inc)):
        if fn.endswith(".h"):
            src = open(os.path.join(inc, fn)).read()
            names += re.findall(r"^(?:int|const char\*|void)\s+\**(wr_\w+)\s*\(", src, flags=re.M)
    return names


class WRError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


def check(rc: int, ctx=None) -> None:
    if rc != WR_OK:
        msg = load().wr_last_error(ctx).decode() if ctx else ""
        raise WRError(rc, msg)


def ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)
