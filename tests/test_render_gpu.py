"""Path-tracing parity on the GPU through the C ABI (wr_render / wr_render_device).

Statistical against the reference's own renders (golden fixtures from
PathTracer::renderPixels) and against the oracle; paired against the oracle
on the same counter-based random stream (same draws per path); and exact
agreement between the megakernel and the wavefront renderer, which compute
the same paths.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN
import make_golden
import wr_oracle

pytestmark = pytest.mark.gpu


def block_z(a, b, k):
    """z-scores of block means of two stacks of independent images (n, H, W, 3)."""
    def blk(x):
        n, h, w, c = x.shape
        return x.reshape(n, h // k, k, w // k, k, c).mean((2, 4))
    ba, bb = blk(a), blk(b)
    va = ba.var(0, ddof=1) / len(a)
    vb = bb.var(0, ddof=1) / len(b)
    return (ba.mean(0) - bb.mean(0)) / np.sqrt(va + vb + 1e-12)


def mean_z(a, b):
    """z-score of the difference of the image means of two stacks of independent images."""
    ma, mb = a.mean((1, 2, 3)), b.mean((1, 2, 3))
    se = np.sqrt(ma.var(ddof=1) / len(ma) + mb.var(ddof=1) / len(mb))
    return (ma.mean() - mb.mean()) / se


def gpu_images(ctx, sid, seeds, spp, maxlen, mode="megakernel"):
    return np.stack([ctx.render(sid, spp, maxlen, seed=s, mode=mode).astype(np.float64) for s in seeds])


def test_megakernel_matches_reference_renders(ctx):
    """Cornell 32x32, 8 x 256 spp against 8 reference renders of 256 spp."""
    g = np.load(os.path.join(GOLDEN, "render_cornell.npz"))
    ref = g["images"].astype(np.float64)
    s = make_golden.golden_scenes()["cornell"]
    sid = ctx.upload(s)
    gpu = gpu_images(ctx, sid, range(100, 108), 256, 8)
    z = block_z(gpu, ref, 4)
    assert np.abs(z).max() < 4.5, np.abs(z).max()
    assert abs(gpu.mean() / ref.mean() - 1) < 0.015
    ctx.release(sid)


def test_megakernel_paired_with_oracle(ctx):
    """Same seed => same Philox draws per path: the GPU and oracle estimates
    are nearly identical pixel by pixel (paths only part where FP32 libm
    results differ in the last bits and a decision flips)."""
    s = make_golden.golden_scenes()["cornell"]
    sid = ctx.upload(s)
    spp = 256
    gsum, gsq = ctx.render_stats(sid, spp, 8, seed=7)
    osum, osq, _ = wr_oracle.SceneOracle(s).render(spp, 8, seed=7, want_sumsq=True)
    osum, osq = osum.reshape(gsum.shape), osq.reshape(gsq.shape)
    gm, om = gsum / spp, osum / spp
    sem = np.sqrt(np.maximum(osq / spp - om * om, 0) / spp) + 1e-6
    d = np.abs(gm - om) / sem
    assert abs(gm.mean() / om.mean() - 1) < 0.003, (gm.mean(), om.mean())
    assert np.median(d) < 0.05, np.median(d)
    assert np.mean(d > 3) < 0.01
    ctx.release(sid)


def test_wavefront_equals_megakernel(ctx):
    """Both renderers trace the same paths with the same draws; only the order
    of the FP32 film additions differs."""
    s = make_golden.golden_scenes()["mixed_l2"]
    sid = ctx.upload(s)
    a = ctx.render(sid, 32, 16, seed=3, mode="megakernel")
    ctx.set_wavefront_config(capacity=1 << 14, iters_per_graph=2)  # small queue: many refills
    try:
        b = ctx.render(sid, 32, 16, seed=3, mode="wavefront")
    finally:
        ctx.set_wavefront_config(capacity=1 << 24)
    assert np.allclose(a, b, rtol=1e-4, atol=1e-5), np.abs(a - b).max()
    ctx.release(sid)


def test_wavefront_after_scene_release_and_reupload(ctx):
    """A released scene leaves the wavefront's scene table; a scene uploaded
    afterwards (possibly at the same host address) renders correctly."""
    sc = make_golden.golden_scenes()
    for name in ("cornell", "mixed_l2", "cornell", "media_small"):
        sid = ctx.upload(sc[name])
        a = ctx.render(sid, 4, 8, seed=5, mode="wavefront")
        b = ctx.render(sid, 4, 8, seed=5, mode="megakernel")
        assert np.allclose(a, b, rtol=1e-4, atol=1e-5)
        ctx.release(sid)


def test_nee_wavefront_equals_megakernel(ctx):
    s = make_golden.golden_scenes()["mixed_l2"]
    sid = ctx.upload(s)
    a = ctx.render(sid, 16, 16, seed=8, mode="megakernel", nee=True)
    b = ctx.render(sid, 16, 16, seed=8, mode="wavefront", nee=True)
    assert np.allclose(a, b, rtol=1e-4, atol=1e-5), np.abs(a - b).max()
    ctx.release(sid)


def test_nee_matches_oracle_paired(ctx):
    """The reference's NEE branch (biased by design: it adds a light
    connection to paths that escaped) on the same seeds as the oracle."""
    s = make_golden.golden_scenes()["cornell"]
    sid = ctx.upload(s)
    orc = wr_oracle.SceneOracle(s)
    h, w = s.camera.height, s.camera.width
    d, m = [], []
    for seed in range(60, 66):
        g = ctx.render(sid, 64, 8, seed=seed, nee=True).astype(np.float64)
        o = orc.render(64, 8, seed=seed, flags=wr_oracle.NEE)[0].reshape(h, w, 3) / 64
        d.append(g.mean() - o.mean())
        m.append(o.mean())
    d, m = np.array(d), np.array(m)
    assert abs(d.mean()) < 0.25 * m.std(ddof=1) + 1e-4 * m.mean(), (d, m)
    ctx.release(sid)


def test_nee_matches_reference_renders_statistically(ctx):
    """NEE renders of the Cornell box against the oracle's NEE (pinned to the
    reference's NEE mode in tests/test_oracle.py)."""
    s = make_golden.golden_scenes()["cornell"]
    sid = ctx.upload(s)
    gpu = gpu_images(ctx, sid, range(70, 78), 64, 8)
    gn = np.stack([ctx.render(sid, 64, 8, seed=k, nee=True).astype(np.float64) for k in range(70, 78)])
    # the reference's NEE adds light to escaped paths: brighter than plain path tracing
    assert gn.mean() > gpu.mean()
    ctx.release(sid)


def test_mixed_materials_match_oracle(ctx):
    """Diffuse, isotropic Phong and dielectric spheres, two lights, depth 16."""
    s = make_golden.golden_scenes()["mixed_l2"]
    sid = ctx.upload(s)
    seeds = range(20, 28)
    gpu = gpu_images(ctx, sid, seeds, 32, 16, mode="wavefront")
    orc = wr_oracle.SceneOracle(s)
    h, w = s.camera.height, s.camera.width
    ora = np.stack([orc.render(32, 16, seed=1000 + k)[0].reshape(h, w, 3) / 32 for k in range(8)])
    z = block_z(gpu, ora, 8)
    assert np.abs(z).max() < 4.5, np.abs(z).max()
    # Phong lobes sampled about the normal (powerCosHemiSphereSampler.h) make
    # the estimator heavy-tailed: compare the image means by their standard error
    assert abs(mean_z(gpu, ora)) < 4.0, mean_z(gpu, ora)
    ctx.release(sid)


def test_mixed_materials_paired_with_oracle(ctx):
    """Same seeds on both sides: per-image means of the GPU and oracle renders
    differ far less than their sampling noise."""
    s = make_golden.golden_scenes()["mixed_l2"]
    sid = ctx.upload(s)
    orc = wr_oracle.SceneOracle(s)
    h, w = s.camera.height, s.camera.width
    d, m = [], []
    for seed in range(20, 28):
        g = ctx.render(sid, 32, 16, seed=seed).astype(np.float64)
        o = orc.render(32, 16, seed=seed)[0].reshape(h, w, 3) / 32
        d.append(g.mean() - o.mean())
        m.append(o.mean())
    d, m = np.array(d), np.array(m)
    assert abs(d.mean()) < 0.25 * m.std(ddof=1), (d, m)
    ctx.release(sid)


def test_media_paired_with_oracle_delta_tracking(ctx):
    """Heterogeneous fBm medium + homogeneous sphere, the oracle in its delta
    tracking mode (the GPU's scheme): same seeds, same draws, per-image means
    equal far below their noise."""
    s = make_golden.golden_scenes()["media_small"]
    sid = ctx.upload(s)
    orc = wr_oracle.SceneOracle(s)
    h, w = s.camera.height, s.camera.width
    d, m = [], []
    for seed in range(40, 46):
        g = ctx.render(sid, 16, 24, seed=seed).astype(np.float64)
        o = orc.render(16, 24, seed=seed, flags=wr_oracle.DELTA)[0].reshape(h, w, 3) / 16
        d.append(g.mean() - o.mean())
        m.append(o.mean())
    d, m = np.array(d), np.array(m)
    assert abs(d.mean()) < 0.25 * m.std(ddof=1), (d, m)
    ctx.release(sid)


def test_media_match_reference_algorithm(ctx):
    """GPU delta tracking against the reference's own free-flight algorithm
    (Simpson integration + Newton inversion, restated in the oracle): image
    means agree within their standard error (the reference's quadrature bias
    is below it at this sample count)."""
    s = make_golden.golden_scenes()["media_small"]
    sid = ctx.upload(s)
    gpu = gpu_images(ctx, sid, range(40, 48), 64, 24)
    orc = wr_oracle.SceneOracle(s)
    h, w = s.camera.height, s.camera.width
    ora = np.stack([orc.render(16, 24, seed=2000 + k)[0].reshape(h, w, 3) / 16 for k in range(8)])
    assert abs(mean_z(gpu, ora)) < 4.0, (gpu.mean(), ora.mean(), mean_z(gpu, ora))
    z = block_z(gpu, ora, 8)
    assert np.abs(z).max() < 5.0, np.abs(z).max()
    ctx.release(sid)


def test_render_rejects_bad_requests(ctx):
    from walkray_gb300 import _lib as L

    s = make_golden.golden_scenes()["cornell"]
    sid = ctx.upload(s)
    with pytest.raises(KeyError):
        ctx.render(sid + 99, 1, 8)
    d = L.wr_render_desc(1, 8, 1, 7, 0, 0, 0)  # unknown mode
    out = np.empty((32, 32, 3), np.float32)
    import ctypes as C

    assert ctx.lib.wr_render(ctx.h, sid, C.byref(d), L.ptr(out)) == 1
    img = ctx.render(sid, 0, 8)
    assert not img.any()
    ctx.release(sid)


def test_pruned_traversal_equals_exact_traversal(ctx):
    """Front-to-back pruning (the renderers' default) against the reference's
    visit-every-passing-box traversal (WR_RENDER_EXACT_TRAVERSAL) on the same
    random stream: the same closest hits give the same paths, so the images
    agree pixel for pixel but for rays grazing a triangle in its plane."""
    s = make_golden.golden_scenes()["mixed_l2"]
    sid = ctx.upload(s)
    for mode in ("megakernel", "wavefront"):
        a = ctx.render(sid, 16, 16, seed=41, mode=mode).astype(np.float64)
        b = ctx.render(sid, 16, 16, seed=41, mode=mode, exact=True).astype(np.float64)
        close = np.isclose(a, b, rtol=1e-4, atol=1e-5).all(-1)
        assert close.mean() > 0.999, (mode, close.mean())
        assert abs(a.mean() / b.mean() - 1) < 1e-3
    ctx.release(sid)


def test_pruning_reduces_traversal_work(ctx):
    import torch

    s = make_golden.golden_scenes()["mixed_l2"]
    sid = ctx.upload(s)
    w, h = s.camera.width, s.camera.height
    film = torch.zeros(w * h * 3, dtype=torch.float32, device="cuda")
    ctx.set_wavefront_config(capacity=1 << 24, drain_paths=0)  # every ray through the extend stages
    try:
        pr = ctx.profile_render(sid, 1, 16, film.data_ptr(), seed=3)
        ex = ctx.profile_render(sid, 1, 16, film.data_ptr(), seed=3, exact=True)
    finally:
        ctx.set_wavefront_config(capacity=1 << 24)
    assert pr["drained_paths"] == 0 and pr["rays"] > 0
    assert abs(pr["rays"] - ex["rays"]) <= 1e-3 * ex["rays"]
    assert pr["box_tests"] < ex["box_tests"]
    ctx.release(sid)


def test_drain_equals_bounce_loop(ctx):
    """Finishing the last paths one per thread (k_wf_drain) computes the same
    paths as running the bounce loop to the end."""
    s = make_golden.golden_scenes()["mixed_l2"]
    sid = ctx.upload(s)
    try:
        ctx.set_wavefront_config(capacity=1 << 16, drain_paths=0)  # loop to the end
        a = ctx.render(sid, 32, 16, seed=9, mode="wavefront", nee=True)
        ctx.set_wavefront_config(capacity=1 << 16, drain_paths=1 << 15)  # drain early
        b = ctx.render(sid, 32, 16, seed=9, mode="wavefront", nee=True)
    finally:
        ctx.set_wavefront_config(capacity=1 << 24)
    assert np.allclose(a, b, rtol=1e-4, atol=1e-5), np.abs(a - b).max()
    assert a.mean() > 0
    ctx.release(sid)


def test_mirror_matches_reference_and_oracle(ctx):
    """ReflectiveObject on the GPU: against the reference's renders of the
    mirror Cornell box (statistically), against the oracle on the same random
    streams (paired), and wavefront against megakernel (same paths)."""
    s = make_golden.golden_scenes()["mirror"]
    sid = ctx.upload(s)
    ref = np.load(os.path.join(GOLDEN, "render_mirror.npz"))["images"].astype(np.float64)
    gpu = gpu_images(ctx, sid, range(30, 38), 256, 8)
    z = block_z(gpu, ref, 4)
    assert np.abs(z).max() < 4.5, np.abs(z).max()
    assert abs(gpu.mean() / ref.mean() - 1) < 0.02
    orc = wr_oracle.SceneOracle(s)
    for seed in (30, 31):
        o = orc.render(256, 8, seed=seed)[0].reshape(32, 32, 3) / 256
        g = ctx.render(sid, 256, 8, seed=seed).astype(np.float64)
        assert abs(g.mean() / o.mean() - 1) < 2e-3, (g.mean(), o.mean())
    w = ctx.render(sid, 64, 8, seed=40, mode="wavefront")
    m = ctx.render(sid, 64, 8, seed=40, mode="megakernel")
    assert np.allclose(w, m, rtol=1e-4, atol=1e-5), np.abs(w - m).max()
    ctx.release(sid)


def test_thin_lens_matches_oracle_paired(ctx):
    """Depth of field (camera.cpp:30-47): the GPU's camera rays draw the
    lens sample as the oracle does, so the same seeds give the same images."""
    s = make_golden.golden_scenes()["dof"]
    sid = ctx.upload(s)
    orc = wr_oracle.SceneOracle(s)
    for seed in (50, 51):
        o = orc.render(256, 8, seed=seed)[0].reshape(32, 32, 3) / 256
        g = ctx.render(sid, 256, 8, seed=seed).astype(np.float64)
        assert abs(g.mean() / o.mean() - 1) < 2e-3, (g.mean(), o.mean())
        assert np.median(np.abs(g - o)) < 1e-3
    ref = np.load(os.path.join(GOLDEN, "render_dof.npz"))["images"].astype(np.float64)
    gpu = gpu_images(ctx, sid, range(60, 68), 2048, 8)
    assert np.abs(block_z(gpu, ref, 4)).max() < 4.5
    ctx.release(sid)


def test_scene_file_renders_through_both_renderers(ctx):
    """A scene read from WalkRay's XML / .obj / .shp files (wr_scene_file_load)
    uploads and renders: wavefront equal to megakernel, and the same paths as
    the oracle on the same random streams (delta tracking for its grid)."""
    from walkray_gb300 import api

    s, st = api.load_scene_file(os.path.join(GOLDEN, "xml", "config.xml"))
    sid = ctx.upload(s)
    n = st["max_path_len"]
    w = ctx.render(sid, 64, n, seed=70, mode="wavefront")
    m = ctx.render(sid, 64, n, seed=70, mode="megakernel")
    assert np.allclose(w, m, rtol=1e-4, atol=1e-5), np.abs(w - m).max()
    h_, w_ = s.camera.height, s.camera.width
    o = wr_oracle.SceneOracle(s).render(64, n, seed=70, flags=wr_oracle.DELTA)[0].reshape(h_, w_, 3) / 64
    assert m.mean() > 0 and abs(m.mean() / o.mean() - 1) < 5e-3, (m.mean(), o.mean())
    ctx.release(sid)


def test_autotuner_pick_renders_the_same_image(ctx):
    """wr_autotune's coordinate descent starts from the shipped defaults
    (2^24 paths in flight, 6 traversal CTAs per SM, refill / leaf 8, six
    steps per turn, rows) and keeps a value only if it is faster; its pick --
    whatever it is -- renders the image the defaults render (only the order
    of the FP32 film additions differs), and the camera-path pixel tile, an
    order of work only, leaves the image alone."""
    s = make_golden.golden_scenes()["mixed_l2"]
    sid = ctx.upload(s)
    want = ctx.render(sid, 8, 16, seed=12, mode="wavefront")
    try:
        best = ctx.autotune(sid, 4, 16)
        assert best["capacity"] in (1 << 22, 1 << 23, 1 << 24)
        assert best["ctas_per_sm"] in (6, 7, 8) and best["pixel_tile"] in (0, 8, 16, 32)
        assert best["steps_per_turn"] in (1, 2, 4, 6, 8)
        assert best["mpaths_per_s"] > 0
        got = ctx.render(sid, 8, 16, seed=12, mode="wavefront")
        assert np.allclose(got, want, rtol=1e-4, atol=1e-5), np.abs(got - want).max()
        for tile in (8, 13, 32):
            ctx.set_wavefront_config(capacity=1 << 16, pixel_tile=tile)
            got = ctx.render(sid, 8, 16, seed=12, mode="wavefront")
            assert np.allclose(got, want, rtol=1e-4, atol=1e-5), (tile, np.abs(got - want).max())
    finally:
        ctx.set_wavefront_config(capacity=1 << 24)
    ctx.release(sid)


def test_progressive_render_refines_like_the_reference(ctx):
    """wr_render_progressive: the running mean after every chunk (the
    reference's per-iteration film update, pathTracer.cpp:15-73), a stop from
    the progress callback, and in the end the image of one wr_render of the
    same samples."""
    s = make_golden.golden_scenes()["cornell"]
    sid = ctx.upload(s)
    seen = []

    def progress(img, done):
        seen.append((done, img.copy()))
        return False

    img, done = ctx.render_progressive(sid, 40, 8, seed=21, chunk_spp=16, progress=progress)
    assert done == 40 and [d for d, _ in seen] == [16, 32, 40]
    want = ctx.render(sid, 40, 8, seed=21, mode="wavefront")
    assert np.allclose(img, want, rtol=1e-4, atol=1e-5), np.abs(img - want).max()
    first = ctx.render(sid, 16, 8, seed=21, mode="wavefront")
    assert np.allclose(seen[0][1], first, rtol=1e-4, atol=1e-5)
    # a stop after the second chunk: the mean of 32 samples
    img2, done2 = ctx.render_progressive(sid, 1 << 30, 8, seed=21, chunk_spp=16, progress=lambda im, d: d >= 32)
    assert done2 == 32
    assert np.allclose(img2, ctx.render(sid, 32, 8, seed=21, mode="wavefront"), rtol=1e-4, atol=1e-5)
    ctx.release(sid)
