"""Vertex connection and merging (WR_MODE_VCM) on the GPU through the C ABI:
paired with the oracle's restatement of VCMTracer on the same random streams
(same sub-paths, same merge radius per iteration computed on the host, the
reference's hash grid on both sides), and statistical against the
reference's own VCMTracer renders (golden fixtures through the reference
harness).

The reference's hash grid drops a query outside the bounding box of the
light points (hashgrid.hxx:103-109).  In an axis-aligned scene the extreme
walls hold both light points and queries, so whether a query on such a wall
is kept depends on the last bit of two hit points; the GPU's and the
oracle's FP32 shading differ in last bits, so the paired comparison runs on
the same scenes rotated off the axes, where the box's extremes are corners."""
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN, means_agree
import make_golden
import wr_oracle
from walkray_gb300 import _lib as L

pytestmark = pytest.mark.gpu

R = make_golden.VCM_RADIUS


def block_z(a, b, k):
    def blk(x):
        n, h, w, c = x.shape
        return x.reshape(n, h // k, k, w // k, k, c).mean((2, 4))
    ba, bb = blk(a), blk(b)
    return (ba.mean(0) - bb.mean(0)) / np.sqrt(ba.var(0, ddof=1) / len(a) + bb.var(0, ddof=1) / len(b) + 1e-12)


def rotated(s):
    """The scene and its camera rotated 20 degrees about y and 10 about x."""
    a, b = math.radians(20), math.radians(10)
    ry = np.array([[math.cos(a), 0, math.sin(a)], [0, 1, 0], [-math.sin(a), 0, math.cos(a)]])
    rx = np.array([[1, 0, 0], [0, math.cos(b), -math.sin(b)], [0, math.sin(b), math.cos(b)]])
    m = rx @ ry
    for o in s.objects:
        o.verts = np.ascontiguousarray((o.verts.astype(np.float64) @ m.T).astype(np.float32))
    c = s.camera
    rot = lambda v: tuple(float(x) for x in m @ np.asarray(v, np.float64))
    c.position, c.focus, c.up = rot(c.position), rot(c.focus), rot(c.up)
    return s


@pytest.mark.parametrize("name", ["cornell", "mirror", "dof", "mixed_l2", "fog", "hetero"])
def test_vcm_paired_with_oracle(ctx, name):
    """The heterogeneous medium as in test_bpt_gpu.PAIRED_BAR, at radius 0.02
    only (at 0.05 one ulp in the oracle alone already moves 3 % of the values)."""
    s = rotated(make_golden.golden_scenes()[name])
    h, w = s.camera.height, s.camera.width
    hetero = name == "hetero"
    frac, mean_tol = (0.85, 1e-2) if hetero else (0.99, 2e-3)
    sid = ctx.upload(s)
    orc = wr_oracle.SceneOracle(s)
    for seed, radius in ((43, R), (44, R if hetero else 0.05)):
        o = orc.render_vcm(8, 8, seed=seed, radius=radius)[0].reshape(h, w, 3) / 8
        g = ctx.render(sid, 8, 8, seed=seed, mode="vcm", radius=radius).astype(np.float64)
        assert abs(g.mean() / o.mean() - 1) < mean_tol, (g.mean(), o.mean())
        close = np.isclose(g, o, rtol=1e-3, atol=1e-5)
        assert close.mean() > frac, close.mean()
    ctx.release(sid)


@pytest.mark.parametrize("name", make_golden.VCM_SCENES)
def test_vcm_matches_reference_renders(ctx, name):
    ref = np.load(os.path.join(GOLDEN, f"render_vcm_{name}.npz"))["images"].astype(np.float64)
    s = make_golden.golden_scenes()[name]
    sid = ctx.upload(s)
    gpu = np.stack([ctx.render(sid, 64, 8, seed=950 + k, mode="vcm", radius=R).astype(np.float64)
                    for k in range(8)])
    assert np.abs(block_z(gpu, ref, 4)).max() < 5.0
    assert means_agree(gpu, ref, 0.015), (gpu.mean(), ref.mean())
    ctx.release(sid)


def test_vcm_paired_on_the_axis_aligned_box(ctx):
    """Unrotated: a small radius (merges all but absent) pairs exactly; with
    merges the images differ only through queries on the extreme walls."""
    s = make_golden.golden_scenes()["cornell"]
    sid = ctx.upload(s)
    orc = wr_oracle.SceneOracle(s)
    o = orc.render_vcm(8, 8, seed=43, radius=1e-6)[0].reshape(32, 32, 3) / 8
    g = ctx.render(sid, 8, 8, seed=43, mode="vcm", radius=1e-6).astype(np.float64)
    assert np.isclose(g, o, rtol=1e-3, atol=1e-5).mean() > 0.99
    ctx.release(sid)


def test_vcm_merging_changes_the_image_and_radius_zero_is_default(ctx):
    """Merging contributes (VCM differs from the bidirectional image on the
    same streams), and radius 0 means the reference's default 0.01."""
    s = make_golden.golden_scenes()["cornell"]
    sid = ctx.upload(s)
    v = ctx.render(sid, 16, 8, seed=9, mode="vcm", radius=0.05).astype(np.float64)
    b = ctx.render(sid, 16, 8, seed=9, mode="bidirectional").astype(np.float64)
    assert np.abs(v - b).max() > 1e-3
    d0 = ctx.render(sid, 4, 8, seed=9, mode="vcm", radius=0.0)
    d1 = ctx.render(sid, 4, 8, seed=9, mode="vcm", radius=0.01)
    assert np.allclose(d0, d1, rtol=1e-5, atol=1e-7)  # equal up to the order of the film's atomic adds
    with pytest.raises(L.WRError):
        ctx.render(sid, 1, 8, mode="vcm", radius=float("nan"))
    ctx.release(sid)


@pytest.mark.parametrize("name,depth", [("cornell", 2), ("mixed_l2", 12)])
def test_vcm_paired_at_other_depths(ctx, name, depth):
    s = rotated(make_golden.golden_scenes()[name])
    h, w = s.camera.height, s.camera.width
    sid = ctx.upload(s)
    o = wr_oracle.SceneOracle(s).render_vcm(8, depth, seed=62, radius=0.03)[0].reshape(h, w, 3) / 8
    g = ctx.render(sid, 8, depth, seed=62, mode="vcm", radius=0.03).astype(np.float64)
    assert abs(g.mean() / o.mean() - 1) < 2e-3, (g.mean(), o.mean())
    assert np.isclose(g, o, rtol=1e-3, atol=1e-5).mean() > 0.99
    ctx.release(sid)
