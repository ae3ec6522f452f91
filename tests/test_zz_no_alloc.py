"""wr_render_noalloc: rendering for callers that may not allocate device
memory while they render (CUDA-graph capture in global mode, real-time loops,
applications with their own memory pools).  Through the C ABI it must give
the image wr_render gives, on two calls in a row (the shared film array keeps
the previous call's contents and must be cleared by each call), reject
images larger than its fixed film, and refuse scenes whose rendering tables
were never built.  Collected last on purpose (file name)."""
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
        for _ in range(2):
            out.fill_(-1.0)
            rc = fn(ctx.h, sid, C.byref(d), C.c_void_p(out.data_ptr()), C.c_void_p(stream.cuda_stream))
            assert rc == 0, ctx.lib.wr_last_error(ctx.h)
            torch.cuda.synchronize()
            got = out.cpu().numpy()
            assert np.allclose(got, ref, rtol=1e-4, atol=1e-5), np.abs(got - ref).max()
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
