"""The path tracer's low-variance estimators (WR_RENDER_NEE_MIS,
WR_RENDER_PHONG_MIRROR) keep the reference's expectation: renders with them
agree statistically with the reference's own PathTracer renders (golden
fixtures) on the Cornell box, the mixed-material scene (isotropic Phong and
refractive spheres) and the anisotropic floor; the wavefront computes the
same per-sample values as the megakernel (sums and sums of squares); and the
variance actually drops."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, means_agree
import make_golden
from walkray_gb300 import _lib as L
from walkray_gb300.api import LOW_VARIANCE

pytestmark = pytest.mark.gpu

MIS = L.WR_RENDER_NEE_MIS
MIRROR = L.WR_RENDER_PHONG_MIRROR


def block_z(a, b, k):
    """z-scores of k x k block means of two stacks of independent images."""
    def blk(x):
        n, h, w, c = x.shape
        return x.reshape(n, h // k, k, w // k, k, c).mean((2, 4))
    ba, bb = blk(a), blk(b)
    va = ba.var(0, ddof=1) / len(a)
    vb = bb.var(0, ddof=1) / len(b)
    return (ba.mean(0) - bb.mean(0)) / np.sqrt(va + vb + 1e-12)


def renders(ctx, sid, flags, seeds, spp, mode="megakernel"):
    return np.stack([ctx.render(sid, spp, 8, seed=s, mode=mode, flags=flags).astype(np.float64) for s in seeds])


@pytest.mark.parametrize("flags", [MIS, LOW_VARIANCE])
def test_cornell_matches_reference_renders(ctx, flags):
    """Cornell 32x32 (diffuse walls and boxes, the small ceiling light): 8 x
    256 spp against the reference's 8 x 256 spp, 4x4 block means within 4.5
    standard errors, image means within 1 %."""
    ref = np.load(os.path.join(GOLDEN, "render_cornell.npz"))["images"].astype(np.float64)
    sid = ctx.upload(make_golden.golden_scenes()["cornell"])
    gpu = renders(ctx, sid, flags, range(300, 308), 256)
    z = block_z(gpu, ref, 4)
    assert np.abs(z).max() < 4.5, np.abs(z).max()
    assert abs(gpu.mean() / ref.mean() - 1) < 0.01, (gpu.mean(), ref.mean())
    ctx.release(sid)


@pytest.mark.parametrize("name,flags", [("mixed_l2", MIRROR), ("mixed_l2", LOW_VARIANCE), ("aniso", MIS),
                                        ("fog", MIS)])
def test_scene_matches_reference_pt_renders(ctx, name, flags):
    """Isotropic Phong (mirror-lobe sampling), refractive spheres, the
    anisotropic floor and the homogeneous sphere against the reference's
    PathTracer renders (render_pt_*.npz): block means and image means."""
    ref = np.load(os.path.join(GOLDEN, f"render_pt_{name}.npz"))["images"].astype(np.float64)
    sid = ctx.upload(make_golden.golden_scenes()[name])
    gpu = renders(ctx, sid, flags, range(400, 408), int(np.load(os.path.join(GOLDEN, f"render_pt_{name}.npz"))["spp"]))
    k = 8 if ref.shape[1] >= 64 else 4
    z = block_z(gpu, ref, k)
    assert np.abs(z).max() < 4.5, np.abs(z).max()
    assert means_agree(gpu, ref, 0.01)
    ctx.release(sid)


@pytest.mark.parametrize("name", ["mixed_l2", "cornell", "fog"])
def test_wavefront_equals_megakernel_with_estimators(ctx, name):
    """Both renderers call the same bounce code with the same draws; the
    wavefront's light connections go through its shadow stage and a path's
    accumulator, so per-pixel sums AND sums of squares (per-sample values)
    must match the megakernel's."""
    sid = ctx.upload(make_golden.golden_scenes()[name])
    a1, a2 = ctx.render_stats(sid, 16, 16, seed=9, mode="megakernel", flags=LOW_VARIANCE)
    ctx.set_wavefront_config(capacity=1 << 14, iters_per_graph=2)  # small queue: many refills
    try:
        b1, b2 = ctx.render_stats(sid, 16, 16, seed=9, mode="wavefront", flags=LOW_VARIANCE)
    finally:
        ctx.set_wavefront_config(capacity=1 << 24)
    assert np.allclose(a1, b1, rtol=1e-4, atol=1e-4), np.abs(a1 - b1).max()
    assert np.allclose(a2, b2, rtol=1e-3, atol=1e-3), np.abs(a2 - b2).max()
    ctx.release(sid)


def test_low_variance_estimators_cut_the_variance(ctx):
    """On the mixed-material scene the per-sample relative variance
    (mean of Var / (R^2 + 1e-2)) drops by more than 5x."""
    sid = ctx.upload(make_golden.golden_scenes()["mixed_l2"])
    ref = ctx.render(sid, 1024, 8, seed=5, flags=LOW_VARIANCE).astype(np.float64)
    rel = {}
    for f in (0, LOW_VARIANCE):
        s1, s2 = ctx.render_stats(sid, 256, 8, seed=6, flags=f)
        var = np.maximum(s2 / 256 - (s1 / 256) ** 2, 0)
        rel[f] = float(np.mean(var / (ref ** 2 + 1e-2)))
    assert rel[LOW_VARIANCE] * 5 < rel[0], rel
    ctx.release(sid)


def test_flag_combinations_are_checked(ctx):
    sid = ctx.upload(make_golden.golden_scenes()["cornell"])
    with pytest.raises(L.WRError):
        ctx.render(sid, 1, 8, nee=True, flags=MIS)
    with pytest.raises(L.WRError):
        ctx.render(sid, 1, 8, mode="bidirectional", flags=MIRROR)
    with pytest.raises(L.WRError):
        ctx.render(sid, 1, 8, flags=1 << 20)
    ctx.release(sid)
