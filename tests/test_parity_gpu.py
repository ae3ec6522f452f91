"""Image parity of the path tracer at the configurations themselves and on
every material, through the C ABI:

* configuration 0 as specified (Cornell box 256x256, 64 spp, depth 8)
  against 256 of the reference's own PathTracer renders (c0_ref.npz): the
  per-pixel 3-sigma rule, 8x8 block means, the image mean, and relMSE
  against the reference's 16,384-spp FP64-accumulated image;
* the reference's PathTracer renders of the mixed-material scene (Phong and
  refractive spheres), the anisotropic Phong floor, the homogeneous sphere
  and the heterogeneous grid (render_pt_*.npz);
* per-pixel pairing with the oracle on the same random streams (same draws
  per path) on the mixed-material, media and anisotropic scenes, the rule
  the Cornell box is held to in test_render_gpu.py;
* the same pairing at configurations 2 and 3 as configured (the 1024^2
  mixed-material scene of 512,006 triangles, depth 16; the 512^2 Cornell
  box with both media, depth 24) on a band of rows the oracle renders in
  seconds, through the wavefront renderer the benchmark times.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, means_agree
import make_golden
import wr_oracle
from walkray_gb300 import scenes as S

pytestmark = pytest.mark.gpu


def block_z(a, b, k):
    """z-scores of k x k block means of two stacks of independent images."""
    def blk(x):
        n, h, w, c = x.shape
        return x.reshape(n, h // k, k, w // k, k, c).mean((2, 4))
    ba, bb = blk(a), blk(b)
    va = ba.var(0, ddof=1) / len(a)
    vb = bb.var(0, ddof=1) / len(b)
    return (ba.mean(0) - bb.mean(0)) / np.sqrt(va + vb + 1e-12)


@pytest.fixture(scope="module")
def c0():
    g = np.load(os.path.join(GOLDEN, "c0_ref.npz"))
    return {k: g[k] for k in g.files}


@pytest.mark.parametrize("mode", ["wavefront", "megakernel"])
def test_configuration_0_against_reference_renders(ctx, c0, mode):
    """Cornell 256x256, 64 spp, depth 8, two seeds.  R = the mean of 256
    reference renders of 64 spp (FP64 sums), var64 = the variance of one
    64-spp reference render.  Pixel-channel z = (I - R) / sqrt(var64 (1 +
    1/256) + (1e-5 R)^2) (the last term: FP32 rounding of pixels the light
    covers, which have no variance).
    * per-pixel 3 sigma: the share of |z| > 3 is no larger than the
      reference's own share for its renders against the others (null_frac3,
      largest over 256 renders, plus 0.2 %);
    * 8x8 block means within 6 sigma, the image mean within 4 sigma;
    * relMSE against R equals its expectation from var64 within 10 %: any
      bias would add to it."""
    R = c0["mean"].astype(np.float64)
    v64 = c0["var64"].astype(np.float64)
    n = int(c0["renders"])
    sid = ctx.upload(S.cornell(256, 256))
    expect = float(np.mean(v64 * (1 + 1 / n) / (R ** 2 + 1e-2)))
    for seed in (1001, 1002):
        img = ctx.render(sid, 64, 8, seed=seed, mode=mode).astype(np.float64)
        sig = np.sqrt(v64 * (1 + 1 / n) + (1e-5 * R) ** 2 + 1e-30)
        z = (img - R) / sig
        frac3 = float(np.mean(np.abs(z) > 3))
        assert frac3 <= float(np.max(c0["null_frac3"])) + 0.002, (frac3, np.max(c0["null_frac3"]))
        k = 8
        bI = img.reshape(32, k, 32, k, 3).mean((1, 3))
        bR = R.reshape(32, k, 32, k, 3).mean((1, 3))
        bv = (sig ** 2).reshape(32, k, 32, k, 3).sum((1, 3)) / k ** 4
        zb = (bI - bR) / np.sqrt(bv)
        assert np.abs(zb).max() < 6.0, np.abs(zb).max()
        zm = (img.mean() - R.mean()) / (np.sqrt((sig ** 2).sum()) / img.size)
        assert abs(zm) < 4.0, zm
        rel = float(np.mean((img - R) ** 2 / (R ** 2 + 1e-2)))
        assert abs(rel / expect - 1) < 0.1, (rel, expect)
    ctx.release(sid)


@pytest.mark.parametrize("name,depth_note", [("mixed_l2", "Phong + refractive"), ("aniso", "anisotropic Phong"),
                                             ("fog", "homogeneous medium"), ("hetero", "heterogeneous medium")])
def test_materials_match_reference_pt_renders(ctx, name, depth_note):
    """8 GPU renders against the reference's 8 PathTracer renders of the same
    scene and spp (depth 8): block means within 4.5 sigma and image means
    within 1 % or 4 standard errors.  For the heterogeneous grid the
    reference integrates free flights by Simpson steps of 2 x 0.01 (its
    quadrature bias is part of the comparison) and the GPU by delta
    tracking."""
    g = np.load(os.path.join(GOLDEN, f"render_pt_{name}.npz"))
    ref = g["images"].astype(np.float64)
    spp = int(g["spp"])
    sid = ctx.upload(make_golden.golden_scenes()[name])
    gpu = np.stack([ctx.render(sid, spp, 8, seed=s, mode="wavefront").astype(np.float64) for s in range(500, 508)])
    k = 8 if ref.shape[1] >= 64 else 4
    z = block_z(gpu, ref, k)
    assert np.abs(z).max() < 4.5, (depth_note, np.abs(z).max())
    assert means_agree(gpu, ref, 0.01), (depth_note, gpu.mean(), ref.mean())
    ctx.release(sid)


def paired(ctx, name, spp, depth, seed, flags=0, mode="megakernel"):
    """GPU and oracle on the same streams: per-pixel |mean difference| in
    units of the oracle's standard error, and the two image means."""
    s = make_golden.golden_scenes()[name]
    sid = ctx.upload(s)
    gsum, gsq = ctx.render_stats(sid, spp, depth, seed=seed, mode=mode)
    osum, osq, _ = wr_oracle.SceneOracle(s).render(spp, depth, seed=seed, flags=flags, want_sumsq=True)
    osum, osq = osum.reshape(gsum.shape), osq.reshape(gsq.shape)
    gm, om = gsum / spp, osum / spp
    sem = np.sqrt(np.maximum(osq / spp - om * om, 0) / spp) + 1e-6
    ctx.release(sid)
    return np.abs(gm - om) / sem, gm.mean(), om.mean()


@pytest.mark.parametrize("name,depth,flags,mean_tol", [
    ("mixed_l2", 16, 0, 0.01),
    ("aniso", 8, 0, 0.003),
    ("media_small", 24, wr_oracle.DELTA, 0.01),
])
def test_per_pixel_paired_with_oracle(ctx, name, depth, flags, mean_tol):
    """Per pixel, the GPU's estimate and the oracle's on the same streams
    differ far less than their noise: the median difference is below 0.05
    standard errors and under 1 % of pixel-channels differ by more than 3
    (paths part only where FP32 library functions round differently in the
    last bit and a decision flips; refraction and media make that more
    frequent than on the Cornell box)."""
    d, gmean, omean = paired(ctx, name, 128, depth, seed=77, flags=flags)
    assert np.median(d) < 0.05, np.median(d)
    assert np.mean(d > 3) < 0.01, np.mean(d > 3)
    assert abs(gmean / omean - 1) < mean_tol, (gmean, omean)


@pytest.mark.parametrize("name,depth,flags,spp,rows", [
    ("mixed_1024", 16, 0, 16, (448, 576)),
    ("media_512", 24, wr_oracle.DELTA, 32, (224, 288)),
])
def test_configuration_scenes_paired_with_oracle(ctx, name, depth, flags, spp, rows):
    """Configurations 2 and 3 at their own resolution, scene and depth: the
    wavefront renderer's per-pixel estimates on a band of rows against the
    oracle's on the same streams, by the rule of the paired test above."""
    s = S.mixed_spheres(1024, 1024, seed=7) if name == "mixed_1024" else S.cornell_media(512, 512)
    sid = ctx.upload(s)
    gsum, gsq = ctx.render_stats(sid, spp, depth, seed=91, mode="wavefront")
    ctx.release(sid)
    w = s.camera.width
    p0, p1 = rows[0] * w, rows[1] * w
    osum, osq, _ = wr_oracle.SceneOracle(s).render(spp, depth, seed=91, flags=flags, p0=p0, p1=p1, want_sumsq=True)
    gm = gsum[rows[0]:rows[1]].reshape(-1, 3) / spp
    om = osum / spp
    sem = np.sqrt(np.maximum(osq / spp - om * om, 0) / spp) + 1e-6
    d = np.abs(gm - om) / sem
    assert np.median(d) < 0.05, np.median(d)
    assert np.mean(d > 3) < 0.01, np.mean(d > 3)
    assert abs(gm.mean() / om.mean() - 1) < 0.01, (gm.mean(), om.mean())
