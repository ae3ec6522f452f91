"""The serving loop (continuous batching over the wavefront queues):
every request's image is the same alone and in a mix of concurrent requests
of other scenes, resolutions and sample counts; requests wait for film memory
and still all finish; cancellation stops a running request."""
import numpy as np
import pytest

import make_golden
from walkray_gb300 import scenes as S
from walkray_gb300.api import Context, Server

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sctx(built):
    ctx = Context()
    sc = make_golden.golden_scenes()
    ids = {
        "cornell": ctx.upload(sc["cornell"]),
        "mixed": ctx.upload(sc["mixed_l2"]),
        "media": ctx.upload(sc["media_small"]),
    }
    yield ctx, ids
    ctx.close()


MIX = [  # scene, width, height, spp, max depth, seed
    ("cornell", 64, 64, 16, 8, 11),
    ("mixed", 96, 64, 8, 16, 12),
    ("media", 48, 48, 8, 24, 13),
    ("cornell", 128, 128, 4, 8, 14),
    ("mixed", 32, 32, 32, 16, 15),
    ("cornell", 16, 16, 64, 8, 16),
    ("media", 64, 32, 4, 24, 17),
]


def test_results_equal_alone_and_in_mix(sctx):
    ctx, ids = sctx
    srv = Server(ctx)
    try:
        alone = []
        for name, w, h, spp, d, seed in MIX:
            r = srv.submit(ids[name], w, h, spp, d, seed)
            srv.wait([r])
            alone.append(srv.fetch(r))
        rids = [srv.submit(ids[name], w, h, spp, d, seed) for name, w, h, spp, d, seed in MIX]
        st = srv.wait(rids)
        for k, r in enumerate(rids):
            assert st[r]["state"] == "done"
            assert st[r]["paths_done"] == MIX[k][1] * MIX[k][2] * MIX[k][3]
            img = srv.fetch(r)
            # same paths, same draws; only the order of the FP32 film additions differs
            assert np.allclose(img, alone[k], rtol=1e-4, atol=1e-5), (k, np.abs(img - alone[k]).max())
    finally:
        srv.stop()


def test_serving_image_matches_wr_render(sctx):
    """A served request renders the same image as wr_render at that resolution."""
    ctx, ids = sctx
    srv = Server(ctx)
    try:
        r = srv.submit(ids["cornell"], 32, 32, 16, 8, seed=21)
        srv.wait([r])
        img = srv.fetch(r)
    finally:
        srv.stop()
    ref = ctx.render(ids["cornell"], 16, 8, seed=21, mode="megakernel")
    assert np.allclose(img, ref, rtol=1e-4, atol=1e-5)


@pytest.mark.parametrize("paths", [4096, 1 << 16])
def test_queue_length_does_not_change_images(sctx, paths):
    """wr_serve_desc.paths_in_flight sets the serving queue's length while no
    request waits for admission (a request's paths then pass through it in
    many more rounds); the images stay the same, and lengths outside
    1024 .. 2^25 are refused."""
    ctx, ids = sctx
    srv = Server(ctx, paths_in_flight=paths)
    try:
        rids = [srv.submit(ids[name], w, h, spp, d, seed) for name, w, h, spp, d, seed in MIX[:3]]
        srv.wait(rids)
        imgs = [srv.fetch(r) for r in rids]
    finally:
        srv.stop()
    for (name, w, h, spp, d, seed), img in zip(MIX[:3], imgs):
        srv1 = Server(ctx)
        try:
            r = srv1.submit(ids[name], w, h, spp, d, seed)
            srv1.wait([r])
            ref = srv1.fetch(r)
        finally:
            srv1.stop()
        assert np.allclose(img, ref, rtol=1e-4, atol=1e-5), (name, np.abs(img - ref).max())
    with pytest.raises(RuntimeError):
        Server(ctx, paths_in_flight=512)


def test_admission_waits_for_film_memory(sctx):
    """A film arena with room for about two 128x128 films: requests queue,
    are admitted as memory frees, and all finish in submission order of
    admission."""
    ctx, ids = sctx
    film = 2 * 128 * 128 * 12 + 4096
    srv = Server(ctx, film_bytes=film)
    try:
        rids = [srv.submit(ids["cornell"], 128, 128, 4, 8, seed=30 + k) for k in range(6)]
        st = srv.wait(rids)
        admits = [st[r]["admit_s"] for r in rids]
        assert all(st[r]["state"] == "done" for r in rids)
        assert admits == sorted(admits)
        # at most two films resident at once: the third request was admitted after the first finished
        assert st[rids[2]]["admit_s"] >= min(st[rids[0]]["finish_s"], st[rids[1]]["finish_s"]) - 1e-6
        for r in rids:
            srv.fetch(r)
        with pytest.raises(Exception):
            srv.submit(ids["cornell"], 1024, 1024, 1, 8)  # film larger than the arena
    finally:
        srv.stop()


def test_cancel(sctx):
    ctx, ids = sctx
    srv = Server(ctx)
    try:
        big = srv.submit(ids["mixed"], 256, 256, 4096, 16, seed=40)
        queued = [srv.submit(ids["cornell"], 16, 16, 1, 8, seed=41)]
        srv.cancel(big)
        st = srv.wait([big] + queued, timeout=300)
        assert st[big]["state"] == "cancelled"
        assert st[queued[0]]["state"] == "done"
    finally:
        srv.stop()
