"""wr_render_noalloc: rendering for callers that may not allocate device
memory while they render (real-time loops that avoid cudaMalloc / cudaFree
because they can stall the device, applications whose device memory belongs
to their own pool).  Through the C ABI it must give the image wr_render gives,
on two calls in a row (the shared film array keeps the previous call's
contents and must be cleared by each call) without the device's free memory
moving between them, report a clean traversal status through
wr_render_noalloc_status, reject images larger than its fixed film,
refuse scenes whose rendering tables were never built and scenes wr_render
itself refuses.  Collected last on purpose (file name)."""
import ctypes as C

import numpy as np
import pytest

from walkray_gb300 import _lib as L
from walkray_gb300 import scenes as S
from walkray_gb300.api import Context

pytestmark = pytest.mark.gpu


def _noalloc(lib):
    f = lib.wr_render_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(L.wr_render_desc), C.c_void_p, C.c_void_p]
    return f


def _status(lib):
    f = lib.wr_render_noalloc_status
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_uint)]
    return f


def test_noalloc_matches_wr_render_twice(built):
    torch = pytest.importorskip("torch")
    ctx = Context()
    try:
        s = S.cornell(128, 96)
        sid = ctx.upload(s)
        fn = _noalloc(ctx.lib)
        d = L.wr_render_desc(16, 8, 5, 0, 0, 0, 0)  # 16 spp, depth 8, seed 5, megakernel
        out = torch.empty((96, 128, 3), dtype=torch.float32, device="cuda")
        # before any wr_render the scene's rendering tables are not resident: refused, nothing allocated
        assert fn(ctx.h, sid, C.byref(d), C.c_void_p(out.data_ptr()), None) == 8
        ref = ctx.render(sid, 16, 8, seed=5, mode="megakernel")
        stream = torch.cuda.current_stream()
        free = []
        for _ in range(2):
            out.fill_(-1.0)
            rc = fn(ctx.h, sid, C.byref(d), C.c_void_p(out.data_ptr()), C.c_void_p(stream.cuda_stream))
            assert rc == 0, ctx.lib.wr_last_error(ctx.h)
            torch.cuda.synchronize()
            got = out.cpu().numpy()
            assert np.allclose(got, ref, rtol=1e-4, atol=1e-5), np.abs(got - ref).max()
            word = C.c_uint(12345)
            assert _status(ctx.lib)(ctx.h, C.c_void_p(stream.cuda_stream), C.byref(word)) == 0
            assert word.value == 0
            torch.cuda.synchronize()
            free.append(torch.cuda.mem_get_info()[0])
        # the first call may load its kernels' code; the second allocates nothing
        assert free[0] == free[1], free
        # a different image through the same film after a larger one
        d2 = L.wr_render_desc(4, 8, 6, 0, 0, 0, 0)
        ref2 = ctx.render(sid, 4, 8, seed=6, mode="megakernel")
        rc = fn(ctx.h, sid, C.byref(d2), C.c_void_p(out.data_ptr()), C.c_void_p(stream.cuda_stream))
        assert rc == 0
        torch.cuda.synchronize()
        assert np.allclose(out.cpu().numpy(), ref2, rtol=1e-4, atol=1e-5)
    finally:
        ctx.close()


def test_noalloc_rejects_oversized_and_wavefront(built):
    torch = pytest.importorskip("torch")
    ctx = Context()
    try:
        fn = _noalloc(ctx.lib)
        big = S.cornell(2048, 1024)  # 2,097,152 pixels > WR_NOALLOC_MAX_PIXELS
        sid = ctx.upload(big)
        out = torch.empty(8, dtype=torch.float32, device="cuda")
        d = L.wr_render_desc(1, 8, 1, 0, 0, 0, 0)
        assert fn(ctx.h, sid, C.byref(d), C.c_void_p(out.data_ptr()), None) == 1
        assert b"WR_NOALLOC_MAX_PIXELS" in ctx.lib.wr_last_error(ctx.h)
        small = ctx.upload(S.cornell(16, 16))
        ctx.render(small, 1, 8)
        dw = L.wr_render_desc(1, 8, 1, 1, 0, 0, 0)  # wavefront mode
        assert fn(ctx.h, small, C.byref(dw), C.c_void_p(out.data_ptr()), None) == 8
    finally:
        ctx.close()


def test_noalloc_refuses_what_wr_render_refuses(built):
    """A heterogeneous medium whose sigma_t is not grey: wr_render answers
    WR_ERR_UNSUPPORTED (delta tracking needs equal channels), and so must the
    no-allocation entry point, instead of rendering a wrong image."""
    torch = pytest.importorskip("torch")
    ctx = Context()
    try:
        s = S.cornell_media(16, 16, grid_n=8)
        het = next(o for o in s.objects if o.type == S.MAT_HETEROGENEOUS)
        het.params["sigma_s"] = (0.8, 0.5, 0.8)
        sid = ctx.upload(s)
        with pytest.raises(RuntimeError):
            ctx.render(sid, 1, 8, mode="megakernel")  # builds the tables, then refuses
        fn = _noalloc(ctx.lib)
        out = torch.empty((16, 16, 3), dtype=torch.float32, device="cuda")
        d = L.wr_render_desc(1, 8, 1, 0, 0, 0, 0)
        assert fn(ctx.h, sid, C.byref(d), C.c_void_p(out.data_ptr()), None) == 8
        assert b"grey" in ctx.lib.wr_last_error(ctx.h)
    finally:
        ctx.close()
