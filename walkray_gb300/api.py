"""Python front end of the C ABI: a thin object layer over libwalkray_gpu.so.

    ctx = Context()                      # wr_ctx_create
    sid = ctx.upload(scene)              # wr_scene_upload (tree build + residency)
    hits = ctx.trace_closest(sid, rays)  # wr_trace_closest (host buffers)
    img = ctx.render(sid, spp=64, max_path_len=8)   # wr_render
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib as L
from .scenes import Scene


def scene_desc(scene: Scene):
    """wr_scene_desc for a scenes.Scene plus the arrays that back it (keep both alive)."""
    objs, verts, tris, grids = scene.flatten()
    keep = [objs, verts, tris]
    gd = (L.wr_grid_desc * max(1, len(grids)))()
    for i, g in enumerate(grids):
        dens = np.ascontiguousarray(g.density, np.float32)
        keep.append(dens)
        nz, ny, nx = dens.shape
        gd[i].nx, gd[i].ny, gd[i].nz = nx, ny, nz
        gd[i].density = dens.ctypes.data_as(C.POINTER(C.c_float))
        gd[i].p0[:] = list(g.p0)
        gd[i].p1[:] = list(g.p1)
    keep.append(gd)
    d = L.wr_scene_desc()
    d.num_objects, d.num_vertices, d.num_triangles, d.num_grids = len(objs), len(verts), len(tris), len(grids)
    d.objects = objs.ctypes.data
    d.vertices = verts.ctypes.data
    d.triangles = tris.ctypes.data
    d.grids = C.addressof(gd)
    c = scene.camera
    if c is not None:
        d.camera.position[:] = list(c.position)
        d.camera.focus[:] = list(c.focus)
        d.camera.up[:] = list(c.up)
        d.camera.width, d.camera.height = c.width, c.height
        d.camera.image_plane_dist = c.image_plane_dist
        d.camera.lens_radius = c.lens_radius
        d.camera.focal_dist = c.focal_dist
    return d, keep


class Context:
    def __init__(self, device: int = 0, memory_budget: int = 0, exact_traversal: bool = False):
        """`exact_traversal`: trace_closest visits every box the reference
        visits (WR_CTX_EXACT_TRAVERSAL) instead of pruning by distance."""
        self.lib = L.load()
        desc = L.wr_ctx_desc(device, memory_budget, L.WR_CTX_EXACT_TRAVERSAL if exact_traversal else 0, 0)
        h = C.c_void_p()
        rc = self.lib.wr_ctx_create(C.byref(desc), C.byref(h))
        if rc != L.WR_OK:
            raise L.WRError(rc, "wr_ctx_create failed (no usable CUDA device?)")
        self.h = h
        self._cams: dict[int, tuple[int, int]] = {}

    def _check(self, rc):
        L.check(rc, self.h)

    def close(self):
        if self.h:
            self.lib.wr_ctx_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- scenes -------------------------------------------------------
    def upload(self, scene: Scene) -> int:
        d, keep = scene_desc(scene)
        sid = C.c_uint32()
        self._check(self.lib.wr_scene_upload(self.h, C.byref(d), C.byref(sid)))
        del keep
        if scene.camera is not None:
            self._cams[sid.value] = (scene.camera.width, scene.camera.height)
        return sid.value

    def release(self, sid: int) -> None:
        self._check(self.lib.wr_scene_release(self.h, sid))

    def info(self, sid: int) -> dict:
        inf = L.wr_scene_info()
        self._check(self.lib.wr_scene_get_info(self.h, sid, C.byref(inf)))
        return {k: getattr(inf, k) for k, _ in L.wr_scene_info._fields_}

    # ---- traversal ----------------------------------------------------
    def trace_closest(self, sid: int, rays: np.ndarray, inside=None, contact=None, out=None) -> np.ndarray:
        """Closest hits of host rays (n x 6 float32).  `out` may be a
        preallocated (e.g. pinned) buffer of n x 16 bytes."""
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
        n = len(rays)
        if out is not None:
            assert out.flags.c_contiguous and out.nbytes == 16 * n
            hits = out
        else:
            hits = np.empty(n, L.HIT_DTYPE)
        filt = None
        if inside is not None:
            ins = np.ascontiguousarray(inside, np.int32)
            con = np.ascontiguousarray(contact, np.int32)
            filt = L.wr_trace_filter(ins.ctypes.data, con.ctypes.data)
        self._check(self.lib.wr_trace_closest(self.h, sid, L.ptr(rays), n, C.byref(filt) if filt else None,
                                              L.ptr(hits)))
        return hits

    def trace_closest_device(self, sid: int, d_rays: int, n: int, d_hits: int, stream: int = 0,
                             d_inside: int = 0, d_contact: int = 0) -> None:
        self._check(self.lib.wr_trace_closest_device(self.h, sid, C.c_void_p(d_rays), n,
                                                     C.c_void_p(d_inside or None), C.c_void_p(d_contact or None),
                                                     C.c_void_p(d_hits), C.c_void_p(stream or None)))


    # ---- rendering ------------------------------------------------------
    def render(self, sid: int, spp: int, max_path_len: int, seed: int = 1, mode: str = "megakernel",
               nee: bool = False, spp_offset: int = 0, exact: bool = False, radius: float = 0.0,
               flags: int = 0) -> np.ndarray:
        """Mean image (H, W, 3) float32, row 0 at the top (wr_render); `radius`
        is the base radius of modes "vcm" and "photon_map" (0 = 0.01);
        `flags`: further WR_RENDER_* bits (e.g. LOW_VARIANCE)."""
        w, h = self._camera_size(sid)
        out = np.empty((h, w, 3), np.float32)
        d = L.wr_render_desc(spp, max_path_len, seed, MODES[mode], _flags(nee, exact) | flags, spp_offset, radius)
        self._check(self.lib.wr_render(self.h, sid, C.byref(d), L.ptr(out)))
        return out

    def render_progressive(self, sid: int, spp: int, max_path_len: int, seed: int = 1, mode: str = "wavefront",
                           chunk_spp: int = 0, progress=None, nee: bool = False, flags: int = 0):
        """wr_render_progressive: the running mean after every chunk of
        samples; `progress(image, spp_done)` may return True to stop.
        Returns (image, spp_done)."""
        w, h = self._camera_size(sid)
        out = np.empty((h, w, 3), np.float32)

        def cb(user, rgb, done):
            return 1 if (progress is not None and progress(out, int(done))) else 0

        fn = L.PROGRESS_FN(cb)
        d = L.wr_render_desc(spp, max_path_len, seed, MODES[mode], _flags(nee, False) | flags, 0, 0)
        done = C.c_uint32()
        self._check(self.lib.wr_render_progressive(self.h, sid, C.byref(d), chunk_spp, L.ptr(out), fn, None,
                                                   C.byref(done)))
        return out, done.value

    def render_device(self, sid: int, spp: int, max_path_len: int, d_sum: int, d_sumsq: int = 0, seed: int = 1,
                      mode: str = "megakernel", nee: bool = False, spp_offset: int = 0, stream: int = 0,
                      exact: bool = False, radius: float = 0.0, flags: int = 0) -> None:
        """Adds spp samples to a device film (wr_render_device), asynchronous on `stream`."""
        d = L.wr_render_desc(spp, max_path_len, seed, MODES[mode], _flags(nee, exact) | flags, spp_offset, radius)
        self._check(self.lib.wr_render_device(self.h, sid, C.byref(d), C.c_void_p(d_sum), C.c_void_p(d_sumsq or None),
                                              C.c_void_p(stream or None)))

    def render_stats(self, sid: int, spp: int, max_path_len: int, seed: int = 1, mode: str = "megakernel",
                     nee: bool = False, exact: bool = False, radius: float = 0.0, flags: int = 0):
        """Per-pixel sum and sum of squares (H, W, 3) over spp samples, via torch device buffers."""
        import torch

        w, h = self._camera_size(sid)
        s = torch.zeros((h, w, 3), dtype=torch.float32, device="cuda")
        s2 = torch.zeros((h, w, 3), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        self.render_device(sid, spp, max_path_len, s.data_ptr(), s2.data_ptr(), seed, mode, nee,
                           stream=torch.cuda.current_stream().cuda_stream, exact=exact, radius=radius, flags=flags)
        torch.cuda.synchronize()
        return s.cpu().numpy().astype(np.float64), s2.cpu().numpy().astype(np.float64)

    def profile_render(self, sid: int, spp: int, max_path_len: int, d_sum: int, seed: int = 1,
                       nee: bool = False, exact: bool = False, flags: int = 0) -> dict:
        """Wavefront render with per-stage CUDA-event timings and traversal work counts."""
        d = L.wr_render_desc(spp, max_path_len, seed, 1, _flags(nee, exact) | flags, 0, 0)
        p = L.wr_render_profile()
        self._check(self.lib.wr_profile_render(self.h, sid, C.byref(d), C.c_void_p(d_sum), C.byref(p)))
        return {k: (list(getattr(p, k)) if k.startswith("iter_") else getattr(p, k))
                for k, _ in L.wr_render_profile._fields_}

    def set_wavefront_config(self, capacity: int, extend_block: int = 128, shade_block: int = 128,
                             ctas_per_sm: int = 0, iters_per_graph: int = 4, refill_min: int = 0,
                             leaf_min: int = 0, drain_paths: int = 0, pixel_tile: int = 0,
                             steps_per_turn: int = 0) -> None:
        """Queue sizes and block shapes of the wavefront renderer; refill_min,
        leaf_min and steps_per_turn (0 = defaults) tune the warp traversal
        loop of both the extend stage and trace_closest; pixel_tile orders
        camera paths by square pixel tiles (0 = rows)."""
        c = L.wr_wavefront_config(capacity, extend_block, shade_block, ctas_per_sm, iters_per_graph, refill_min,
                                  leaf_min, drain_paths, pixel_tile, steps_per_turn, 0.0)
        self._check(self.lib.wr_set_wavefront_config(self.h, C.byref(c)))

    def autotune(self, sid: int, spp_per_trial: int, max_path_len: int) -> dict:
        c = L.wr_wavefront_config()
        self._check(self.lib.wr_autotune(self.h, sid, spp_per_trial, max_path_len, C.byref(c)))
        return {k: getattr(c, k) for k, _ in L.wr_wavefront_config._fields_}

    def rng_draws(self, seed: int, pixel, sample, dim):
        """The device random stream (wr_rng_draws): (words (n, 4) uint32,
        draws (n,) float32) of draw dim[i] of (pixel[i], sample[i])."""
        px = np.ascontiguousarray(pixel, np.uint32)
        sm = np.ascontiguousarray(sample, np.uint32)
        dm = np.ascontiguousarray(dim, np.uint32)
        n = len(px)
        assert len(sm) == n and len(dm) == n
        words = np.empty((n, 4), np.uint32)
        draws = np.empty(n, np.float32)
        self._check(self.lib.wr_rng_draws(self.h, seed, L.ptr(px), L.ptr(sm), L.ptr(dm), n, L.ptr(words),
                                          L.ptr(draws)))
        return words, draws

    def _camera_size(self, sid):
        cam = self._cams.get(sid)
        if cam is None:
            raise KeyError(f"scene {sid} was not uploaded through this Context")
        return cam


MODES = {"megakernel": 0, "wavefront": 1, "bidirectional": 2, "vcm": 3, "photon_map": 4}
# the low-variance estimators of the path tracer: unbiased NEE with MIS and
# mirror-lobe Phong sampling (same expectation as the reference's estimator)
LOW_VARIANCE = L.WR_RENDER_NEE_MIS | L.WR_RENDER_PHONG_MIRROR


def _flags(nee: bool, exact: bool) -> int:
    """WR_RENDER_* bits: the NEE branch; exact = no distance pruning in traversal."""
    return (L.WR_RENDER_NEE if nee else 0) | (L.WR_RENDER_EXACT_TRAVERSAL if exact else 0)

REQ_STATES = {0: "queued", 1: "running", 2: "done", 3: "cancelled", 4: "failed"}


class Server:
    """The serving loop of a Context (wr_serve_start ... wr_serve_stop):
    requests admitted by film memory, their paths sharing the wavefront queues."""

    def __init__(self, ctx: Context, film_bytes: int = 0, max_active: int = 0, fifo: bool = False,
                 paths_in_flight: int = 0):
        """`fifo`: queue slots go to the requests in admission order instead
        of in equal shares (WR_SERVE_FIFO); `paths_in_flight`: the queue
        length while no request waits for admission (0 = 2^22,
        WR_SERVE_DEFAULT_PATHS; the full capacity while requests wait)."""
        self.ctx = ctx
        d = L.wr_serve_desc(film_bytes, max_active, L.WR_SERVE_FIFO if fifo else 0, paths_in_flight, 0)
        ctx._check(ctx.lib.wr_serve_start(ctx.h, C.byref(d)))
        self.sizes: dict[int, tuple[int, int]] = {}

    def submit(self, sid: int, width: int, height: int, spp: int, max_path_len: int, seed: int = 1,
               nee: bool = False, exact: bool = False, flags: int = 0) -> int:
        r = L.wr_request_desc(sid, width, height, spp, max_path_len, _flags(nee, exact) | flags, seed)
        rid = C.c_uint64()
        self.ctx._check(self.ctx.lib.wr_submit(self.ctx.h, C.byref(r), C.byref(rid)))
        self.sizes[rid.value] = (width, height)
        return rid.value

    def poll(self, rid: int) -> dict:
        st = L.wr_req_status()
        self.ctx._check(self.ctx.lib.wr_poll(self.ctx.h, rid, C.byref(st)))
        return {"state": REQ_STATES[st.state], "paths_total": st.paths_total, "paths_done": st.paths_done,
                "submit_s": st.submit_s, "admit_s": st.admit_s, "finish_s": st.finish_s}

    def fetch(self, rid: int) -> np.ndarray:
        w, h = self.sizes.pop(rid)
        out = np.empty((h, w, 3), np.float32)
        self.ctx._check(self.ctx.lib.wr_fetch(self.ctx.h, rid, L.ptr(out)))
        return out

    def cancel(self, rid: int) -> None:
        self.ctx._check(self.ctx.lib.wr_cancel(self.ctx.h, rid))

    def stop(self) -> None:
        self.ctx._check(self.ctx.lib.wr_serve_stop(self.ctx.h))

    def wait(self, rids, timeout: float = 600.0, poll_s: float = 0.002) -> dict:
        import time

        t0 = time.time()
        left = set(rids)
        status = {}
        while left:
            for r in list(left):
                st = self.poll(r)
                if st["state"] in ("done", "cancelled", "failed"):
                    status[r] = st
                    left.discard(r)
            if left:
                if time.time() - t0 > timeout:
                    raise TimeoutError(f"{len(left)} requests unfinished")
                time.sleep(poll_s)
        return status


def load_scene_file(path: str):
    """WalkRay's XML scene configuration (and the .obj / .shp meshes and
    density files it names) read by the library (wr_scene_file_load), as a
    scenes.Scene with world-space vertices, plus the render settings
    {renderer, spp, max_path_len}.  No GPU is needed."""
    from .scenes import OBJECT_DTYPE, Camera, Grid

    lib = L.load()
    h = C.c_void_p()
    err = C.create_string_buffer(512)
    rc = lib.wr_scene_file_load(path.encode(), C.byref(h), err, len(err))
    if rc != L.WR_OK:
        raise L.WRError(rc, err.value.decode(errors="replace") or "wr_scene_file_load failed")
    try:
        d, st = L.wr_scene_desc(), L.wr_scene_file_settings()
        lib.wr_scene_file_get(h, C.byref(d), C.byref(st))
        objs = np.frombuffer((C.c_char * (d.num_objects * OBJECT_DTYPE.itemsize)).from_address(d.objects),
                             OBJECT_DTYPE).copy() if d.num_objects else np.zeros(0, OBJECT_DTYPE)
        verts = np.ctypeslib.as_array((C.c_float * (3 * d.num_vertices)).from_address(d.vertices)).reshape(-1, 3).copy() \
            if d.num_vertices else np.zeros((0, 3), np.float32)
        tris = np.ctypeslib.as_array((C.c_uint32 * (3 * d.num_triangles)).from_address(d.triangles)).reshape(-1, 3).copy() \
            if d.num_triangles else np.zeros((0, 3), np.uint32)
        grids = []
        gds = (L.wr_grid_desc * d.num_grids).from_address(d.grids) if d.num_grids else []
        for g in gds:
            dens = np.ctypeslib.as_array(g.density, shape=(g.nz * g.ny * g.nx,)).reshape(g.nz, g.ny, g.nx).copy()
            grids.append(Grid(dens, tuple(g.p0), tuple(g.p1)))
        s = Scene(os.path.basename(path))
        s.grids = grids
        skip = {"type", "vert_begin", "vert_count", "tri_begin", "tri_count"}
        for o in objs:
            vb, vc, tb, tc = int(o["vert_begin"]), int(o["vert_count"]), int(o["tri_begin"]), int(o["tri_count"])
            params = {k: (tuple(float(x) for x in o[k]) if o[k].shape else o[k].item())
                      for k in OBJECT_DTYPE.names if k not in skip}
            s.add(int(o["type"]), verts[vb:vb + vc], tris[tb:tb + tc], **params)
        c = d.camera
        s.camera = Camera(tuple(c.position), tuple(c.focus), tuple(c.up), int(c.width), int(c.height),
                          float(c.image_plane_dist), float(c.lens_radius), float(c.focal_dist))
        mode = {v: k for k, v in MODES.items()}.get(int(st.mode))
        settings = {"renderer": st.renderer.decode(), "spp": int(st.spp), "max_path_len": int(st.max_path_len),
                    "radius": float(st.radius), "mode": mode}
        return s, settings
    finally:
        lib.wr_scene_file_free(h)


def build_tree_host(verts: np.ndarray, tris: np.ndarray, threads: int = 0) -> dict:
    """The reference tree built by the library on the host only (no GPU)."""
    lib = L.load()
    verts = np.ascontiguousarray(verts, np.float32).reshape(-1, 3)
    tris = np.ascontiguousarray(tris, np.uint32).reshape(-1, 3)
    h = C.c_void_p()
    rc = lib.wr_kdtree_build_host(L.ptr(verts), len(verts), L.ptr(tris), len(tris), threads, C.byref(h))
    if rc != L.WR_OK:
        raise L.WRError(rc, "wr_kdtree_build_host failed")
    try:
        nn, nlt, md = C.c_uint32(), C.c_uint32(), C.c_uint32()
        lib.wr_kdtree_host_sizes(h, C.byref(nn), C.byref(nlt), C.byref(md))
        N = nn.value
        out = {
            "left": np.empty(N, np.int32), "right": np.empty(N, np.int32), "box": np.empty((N, 6), np.float32),
            "leaf_first": np.empty(N, np.uint32), "leaf_count": np.empty(N, np.uint32),
            "leaf_tris": np.empty(nlt.value, np.uint32), "max_depth": md.value,
        }
        lib.wr_kdtree_host_export(h, *(L.ptr(out[k]) for k in ("left", "right", "box", "leaf_first", "leaf_count",
                                                               "leaf_tris")))
        return out
    finally:
        lib.wr_kdtree_host_free(h)


def tree_dump_bytes(t: dict) -> bytes:
    """The tree in the pre-order dump format of the oracle programs."""
    parts = []
    stack = [0]
    while stack:
        n = stack.pop()
        leaf = t["left"][n] < 0
        cnt = int(t["leaf_count"][n]) if leaf else 0
        parts.append(np.array([1 if leaf else 0], np.uint32).tobytes())
        parts.append(t["box"][n].astype(np.float32).tobytes())
        parts.append(np.array([cnt], np.uint32).tobytes())
        if leaf:
            f = int(t["leaf_first"][n])
            parts.append(t["leaf_tris"][f:f + cnt].astype(np.uint32).tobytes())
        else:
            stack.append(int(t["right"][n]))
            stack.append(int(t["left"][n]))
    return b"".join(parts)
