"""ctypes wrapper of the C restatement (oracle/build/libwr_oracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline legs as the checker / timed CPU reference.  The
library never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "build", "libwr_oracle.so")
_lib = None

NEE = 1
DELTA = 4  # heterogeneous media by delta / ratio tracking (the GPU's scheme)


def ppm_ellipse(in_d, n, sp, hn, nu: float, nv: float):
    """The photon query's ellipse set-up (wro_ppm_ellipse): (kind, ratio,
    ex, ey); kind 0 elliptic, 1 and 2 the two fallbacks to the round kernel."""
    lib = load()
    fp = C.POINTER(C.c_float)
    vs = [np.ascontiguousarray(v, np.float32) for v in (in_d, n, sp, hn)]
    ratio = C.c_float()
    ex, ey = np.zeros(3, np.float32), np.zeros(3, np.float32)
    k = lib.wro_ppm_ellipse(*[v.ctypes.data_as(fp) for v in vs], nu, nv, C.byref(ratio), ex.ctypes.data_as(fp),
                            ey.ctypes.data_as(fp))
    return k, np.float32(ratio.value), ex, ey


def build() -> None:
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        lib = C.CDLL(LIB)
        lib.wro_build.restype = C.c_void_p
        lib.wro_build.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32]
        lib.wro_tree_free.argtypes = [C.c_void_p]
        lib.wro_tree_num_nodes.restype = C.c_uint32
        lib.wro_tree_num_nodes.argtypes = [C.c_void_p]
        lib.wro_tree_dump.restype = C.c_uint64
        lib.wro_tree_dump.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64]
        lib.wro_trace.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.c_void_p, C.c_void_p, C.c_int, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
        lib.wro_philox4x32_10.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        lib.wro_draw.restype = C.c_float
        lib.wro_draw.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32]
        lib.wro_scene_create.restype = C.c_void_p
        lib.wro_scene_create.argtypes = [C.c_void_p]
        lib.wro_scene_free.argtypes = [C.c_void_p]
        lib.wro_render.argtypes = [C.c_void_p, C.c_uint32, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32,
                                   C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_int, C.POINTER(C.c_uint64)]
        lib.wro_render_bpt.restype = C.c_int
        lib.wro_render_bpt.argtypes = [C.c_void_p, C.c_uint32, C.c_uint64, C.c_uint32, C.c_uint32, C.c_void_p,
                                       C.c_void_p, C.c_int, C.POINTER(C.c_uint64)]
        lib.wro_render_vcm.restype = C.c_int
        lib.wro_render_vcm.argtypes = [C.c_void_p, C.c_uint32, C.c_uint64, C.c_float, C.c_uint32, C.c_uint32,
                                       C.c_void_p, C.c_void_p, C.c_int, C.POINTER(C.c_uint64)]
        lib.wro_render_ppm.restype = C.c_int
        lib.wro_render_ppm.argtypes = lib.wro_render_vcm.argtypes
        lib.wro_vcm_radius.restype = C.c_float
        lib.wro_vcm_radius.argtypes = [C.c_float, C.c_uint32]
        fp = C.POINTER(C.c_float)
        lib.wro_ppm_ellipse.restype = C.c_int
        lib.wro_ppm_ellipse.argtypes = [fp, fp, fp, fp, C.c_float, C.c_float, fp, fp, fp]
        _lib = lib
    return _lib


def _p(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


class Tree:
    def __init__(self, verts: np.ndarray, gtris: np.ndarray, tri_obj: np.ndarray | None = None):
        self.lib = load()
        self.verts = np.ascontiguousarray(verts, np.float32).reshape(-1, 3)
        self.tris = np.ascontiguousarray(gtris, np.uint32).reshape(-1, 3)
        self.tri_obj = None if tri_obj is None else np.ascontiguousarray(tri_obj, np.int32)
        self.h = self.lib.wro_build(_p(self.verts), len(self.verts), _p(self.tris), len(self.tris))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.wro_tree_free(self.h)
            self.h = None

    def dump(self) -> bytes:
        n = self.lib.wro_tree_dump(self.h, None, 0)
        buf = (C.c_char * max(1, n))()
        self.lib.wro_tree_dump(self.h, buf, n)
        return bytes(buf[:n])

    def trace(self, rays: np.ndarray, inside=None, contact=None, threads: int = 0):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
        n = len(rays)
        tri = np.empty(n, np.uint32)
        t = np.empty(n, np.float32)
        nb, nt = C.c_uint64(), C.c_uint64()
        ins = None if inside is None else np.ascontiguousarray(inside, np.int32)
        con = None if contact is None else np.ascontiguousarray(contact, np.int32)
        self.lib.wro_trace(self.h, _p(rays), n, _p(ins), _p(con), _p(self.tri_obj), _p(tri), _p(t), threads,
                           C.byref(nb), C.byref(nt))
        return tri, t, nb.value, nt.value


def philox(ctr, key):
    lib = load()
    c = np.asarray(ctr, np.uint32)
    k = np.asarray(key, np.uint32)
    out = np.empty(4, np.uint32)
    lib.wro_philox4x32_10(_p(c), _p(k), _p(out))
    return out


def draw(seed: int, pixel: int, sample: int, dim: int) -> float:
    return load().wro_draw(seed, pixel, sample, dim)


class SceneOracle:
    """The restated path tracer on a scenes.Scene."""

    def __init__(self, scene):
        import sys

        sys.path.insert(0, os.path.dirname(HERE))
        from walkray_gb300.api import scene_desc

        self.lib = load()
        self.scene = scene
        d, self._keep = scene_desc(scene)
        self._desc = d
        self.h = self.lib.wro_scene_create(C.byref(d))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.wro_scene_free(self.h)
            self.h = None

    def render(self, spp: int, max_path_len: int, seed: int, flags: int = 0, s0: int = 0, p0: int = 0,
               p1: int | None = None, threads: int = 0, want_sumsq: bool = False):
        c = self.scene.camera
        npx = c.width * c.height
        p1 = npx if p1 is None else p1
        s = np.zeros((p1 - p0, 3), np.float64)
        s2 = np.zeros((p1 - p0, 3), np.float64) if want_sumsq else None
        rays = C.c_uint64()
        self.lib.wro_render(self.h, max_path_len, seed, flags, p0, p1, s0, s0 + spp, _p(s), _p(s2), threads,
                            C.byref(rays))
        return s, s2, rays.value

    def render_bpt(self, spp: int, max_path_len: int, seed: int, s0: int = 0, threads: int = 0,
                   want_sumsq: bool = False):
        """The restated BidirectionalPathTracer: per-pixel sums over samples
        [s0, s0 + spp) of each sample's image (after isLegalColor and
        fixVignetting), like render()."""
        c = self.scene.camera
        npx = c.width * c.height
        s = np.zeros((npx, 3), np.float64)
        s2 = np.zeros((npx, 3), np.float64) if want_sumsq else None
        rays = C.c_uint64()
        rc = self.lib.wro_render_bpt(self.h, max_path_len, seed, s0, s0 + spp, _p(s), _p(s2), threads,
                                     C.byref(rays))
        if rc:
            raise RuntimeError("wro_render_bpt failed")
        return s, s2, rays.value

    def render_vcm(self, spp: int, max_path_len: int, seed: int, radius: float = 0.01, s0: int = 0,
                   threads: int = 0, want_sumsq: bool = False):
        """The restated VCMTracer with base merge radius `radius`: per-pixel
        sums over samples [s0, s0 + spp), like render()."""
        c = self.scene.camera
        npx = c.width * c.height
        s = np.zeros((npx, 3), np.float64)
        s2 = np.zeros((npx, 3), np.float64) if want_sumsq else None
        rays = C.c_uint64()
        rc = self.lib.wro_render_vcm(self.h, max_path_len, seed, radius, s0, s0 + spp, _p(s), _p(s2), threads,
                                     C.byref(rays))
        if rc:
            raise RuntimeError("wro_render_vcm failed")
        return s, s2, rays.value

    def render_ppm(self, spp: int, max_path_len: int, seed: int, radius: float = 0.01, s0: int = 0,
                   threads: int = 0, want_sumsq: bool = False):
        """The restated PhotonMap (progressive photon mapping) with base radius
        `radius`: per-pixel sums over samples [s0, s0 + spp), like render()."""
        c = self.scene.camera
        npx = c.width * c.height
        s = np.zeros((npx, 3), np.float64)
        s2 = np.zeros((npx, 3), np.float64) if want_sumsq else None
        rays = C.c_uint64()
        rc = self.lib.wro_render_ppm(self.h, max_path_len, seed, radius, s0, s0 + spp, _p(s), _p(s2), threads,
                                     C.byref(rays))
        if rc:
            raise RuntimeError("wro_render_ppm failed")
        return s, s2, rays.value
