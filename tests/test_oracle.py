"""The oracle (C restatement) against the reference's own answers: golden
fixtures made by tests/golden/make_golden.py from WalkRay's code, and the
published Philox4x32-10 known-answer vectors."""
import hashlib
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, means_agree
import make_golden
import wr_oracle
from walkray_gb300 import scenes as S


def test_philox_known_answers(built):
    # Random123 known-answer vectors for Philox4x32-10: (counter, key) -> output
    kat = [
        ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
        ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
        ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
         [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
    ]
    for ctr, key, out in kat:
        assert list(wr_oracle.philox(ctr, key)) == out


def test_draw_stream_layout(built):
    # draw d of (pixel, sample) is word d%4 of philox({d/4, sample, pixel, 0}, seed) >> 8 * 2^-24
    seed = 0x123456789ABCDEF
    for pixel, sample, dim in [(0, 0, 0), (5, 3, 7), (65535, 255, 41), (2**31, 17, 3)]:
        w = wr_oracle.philox([dim >> 2, sample, pixel, 0], [seed & 0xFFFFFFFF, seed >> 32])[dim & 3]
        assert wr_oracle.draw(seed, pixel, sample, dim) == np.float32((int(w) >> 8) / 16777216.0)


@pytest.mark.parametrize("name", ["cornell", "ico4", "mixed_l2", "media_small"])
def test_oracle_tree_equals_reference(built, name):
    s = make_golden.golden_scenes()[name]
    _, v, _, _ = s.flatten()
    tree = wr_oracle.Tree(v, s.global_triangles())
    want = json.load(open(os.path.join(GOLDEN, "trees.json")))[name]
    assert hashlib.sha256(tree.dump()).hexdigest() == want


def test_oracle_hits_equal_reference(built):
    s = make_golden.golden_scenes()["ico4"]
    _, v, _, _ = s.flatten()
    g = np.load(os.path.join(GOLDEN, "trace_ico4.npz"))
    rays = S.kd_rays(s, 32768, seed=2)
    tri, t, nb, nt = wr_oracle.Tree(v, s.global_triangles()).trace(rays)
    assert np.array_equal(tri, g["tri"])
    hit = tri != 0xFFFFFFFF
    assert np.array_equal(t[hit].view(np.uint32), g["t"][hit].view(np.uint32))
    assert 0.05 < hit.mean() < 0.5


def test_oracle_filtered_hits_equal_reference(built):
    s = make_golden.golden_scenes()["mixed_l2"]
    _, v, _, _ = s.flatten()
    g = np.load(os.path.join(GOLDEN, "trace_filtered.npz"))
    rays, ids = make_golden.filtered_rays(s, 32768, seed=5)
    tree = wr_oracle.Tree(v, s.global_triangles(), s.tri_object_ids())
    tri, t, _, _ = tree.trace(rays, ids[:, 0], ids[:, 1])
    assert np.array_equal(tri, g["tri"])


def test_oracle_nee_matches_reference_statistically(built):
    """The NEE branch (pathTracer.cpp:39-66) against 8 reference NEE renders."""
    g = np.load(os.path.join(GOLDEN, "render_cornell_nee.npz"))
    ref = g["images"].astype(np.float64)
    plain = np.load(os.path.join(GOLDEN, "render_cornell.npz"))["images"].astype(np.float64)
    s = make_golden.golden_scenes()["cornell"]
    orc = wr_oracle.SceneOracle(s)
    port = np.stack([(orc.render(256, 8, seed=3000 + k, flags=wr_oracle.NEE)[0] / 256).reshape(32, 32, 3)
                     for k in range(8)])
    blk = lambda a: a.reshape(a.shape[0], 8, 4, 8, 4, 3).mean((2, 4))
    br, bp = blk(ref), blk(port)
    z = (br.mean(0) - bp.mean(0)) / np.sqrt(br.var(0, ddof=1) / 8 + bp.var(0, ddof=1) / 8 + 1e-12)
    assert np.abs(z).max() < 4.5, np.abs(z).max()
    assert abs(port.mean() / ref.mean() - 1) < 0.015
    assert ref.mean() > 1.03 * plain.mean()  # the reference NEE mode is biased upwards


def test_oracle_delta_tracking_agrees_with_regular_tracking(built):
    """The heterogeneous medium by delta tracking (the GPU's scheme) against
    the reference's Simpson/Newton regular tracking, both in the oracle, on
    the media scene: image means within 4 standard errors."""
    s = make_golden.golden_scenes()["media_small"]
    orc = wr_oracle.SceneOracle(s)
    reg = np.array([orc.render(8, 24, seed=700 + k)[0].mean() / 8 for k in range(8)])
    dlt = np.array([orc.render(64, 24, seed=800 + k, flags=wr_oracle.DELTA)[0].mean() / 64 for k in range(8)])
    se = np.sqrt(reg.var(ddof=1) / 8 + dlt.var(ddof=1) / 8)
    assert abs(reg.mean() - dlt.mean()) < 4 * se, (reg.mean(), dlt.mean(), se)


def test_oracle_render_matches_reference_statistically(built):
    """Cornell 32x32: the restated PathTracer vs 8 reference renders of 256 spp.
    Per-pixel z on 4x4 blocks; |z| > 4 on no block, mean within 1.5 %."""
    g = np.load(os.path.join(GOLDEN, "render_cornell.npz"))
    ref = g["images"].astype(np.float64)  # (8, 32, 32, 3)
    s = make_golden.golden_scenes()["cornell"]
    orc = wr_oracle.SceneOracle(s)
    imgs = []
    for seed in range(8):
        sm, _, _ = orc.render(256, 8, seed=1000 + seed)
        imgs.append((sm / 256).reshape(32, 32, 3))
    port = np.stack(imgs)
    blk = lambda a: a.reshape(a.shape[0], 8, 4, 8, 4, 3).mean((2, 4))
    br, bp = blk(ref), blk(port)
    z = (br.mean(0) - bp.mean(0)) / np.sqrt(br.var(0, ddof=1) / 8 + bp.var(0, ddof=1) / 8 + 1e-12)
    assert np.abs(z).max() < 4.5, np.abs(z).max()
    assert abs(port.mean() / ref.mean() - 1) < 0.015


def test_oracle_mirror_matches_reference_statistically(built):
    """ReflectiveObject (reflectiveObj.h:17-43), including the reference's
    unparenthesised MAX_VEC_COMP: the restated renderer vs 8 reference
    renders of the mirror Cornell box."""
    g = np.load(os.path.join(GOLDEN, "render_mirror.npz"))
    ref = g["images"].astype(np.float64)
    s = make_golden.golden_scenes()["mirror"]
    orc = wr_oracle.SceneOracle(s)
    port = np.stack([(orc.render(256, 8, seed=1100 + k)[0] / 256).reshape(32, 32, 3) for k in range(8)])
    blk = lambda a: a.reshape(a.shape[0], 8, 4, 8, 4, 3).mean((2, 4))
    br, bp = blk(ref), blk(port)
    z = (br.mean(0) - bp.mean(0)) / np.sqrt(br.var(0, ddof=1) / 8 + bp.var(0, ddof=1) / 8 + 1e-12)
    assert np.abs(z).max() < 4.5, np.abs(z).max()
    assert abs(port.mean() / ref.mean() - 1) < 0.02
    # the mirror shows the scene: different from the all-diffuse box
    plain = np.load(os.path.join(GOLDEN, "render_cornell.npz"))["images"].astype(np.float64)
    assert abs(plain.mean() / ref.mean() - 1) > 0.01 or np.abs(blk(plain).mean(0) - br.mean(0)).max() > 0.05


def test_oracle_thin_lens_matches_reference_statistically(built):
    """Camera::generateRay with depth of field (camera.cpp:30-47,
    concentricSampleDisk :207-249) vs 8 reference renders."""
    g = np.load(os.path.join(GOLDEN, "render_dof.npz"))
    ref = g["images"].astype(np.float64)
    s = make_golden.golden_scenes()["dof"]
    orc = wr_oracle.SceneOracle(s)
    port = np.stack([(orc.render(2048, 8, seed=1200 + k)[0] / 2048).reshape(32, 32, 3) for k in range(8)])
    blk = lambda a: a.reshape(a.shape[0], 8, 4, 8, 4, 3).mean((2, 4))
    br, bp = blk(ref), blk(port)
    z = (br.mean(0) - bp.mean(0)) / np.sqrt(br.var(0, ddof=1) / 8 + bp.var(0, ddof=1) / 8 + 1e-12)
    assert np.abs(z).max() < 4.5, np.abs(z).max()
    assert abs(port.mean() / ref.mean() - 1) < 0.015
    # and the lens matters at this noise level: the pinhole oracle is told apart
    pin = wr_oracle.SceneOracle(make_golden.golden_scenes()["cornell"])
    pim = np.stack([(pin.render(2048, 8, seed=1300 + k)[0] / 2048).reshape(32, 32, 3) for k in range(8)])
    bq = blk(pim)
    zp = (br.mean(0) - bq.mean(0)) / np.sqrt(br.var(0, ddof=1) / 8 + bq.var(0, ddof=1) / 8 + 1e-12)
    assert np.abs(zp).max() > 4.5, np.abs(zp).max()


@pytest.mark.parametrize("name", make_golden.BPT_SCENES)
def test_oracle_bidirectional_matches_reference_statistically(built, name):
    """BidirectionalPathTracer (bidirPathTracer.cpp:10-313): the restated
    connections, MIS weights and light-tracing splats vs 8 reference renders
    of 64 spp.  Per-pixel z on 4x4 blocks, mean within 1.5 % (or 4 standard
    errors: the heterogeneous medium's estimate is noisier than that)."""
    g = np.load(os.path.join(GOLDEN, f"render_bpt_{name}.npz"))
    ref = g["images"].astype(np.float64)
    s = make_golden.golden_scenes()[name]
    h, w = s.camera.height, s.camera.width
    orc = wr_oracle.SceneOracle(s)
    port = np.stack([(orc.render_bpt(64, 8, seed=500 + k)[0] / 64).reshape(h, w, 3) for k in range(8)])
    blk = lambda a: a.reshape(a.shape[0], h // 4, 4, w // 4, 4, 3).mean((2, 4))
    br, bp = blk(ref), blk(port)
    z = (br.mean(0) - bp.mean(0)) / np.sqrt(br.var(0, ddof=1) / 8 + bp.var(0, ddof=1) / 8 + 1e-12)
    assert np.abs(z).max() < 4.8, np.abs(z).max()
    assert means_agree(port, ref, 0.015), (port.mean(), ref.mean())


@pytest.mark.parametrize("name", make_golden.VCM_SCENES)
def test_oracle_vcm_matches_reference_statistically(built, name):
    """VCMTracer (vcmTracer.cpp:6-446), base radius 0.02: the restated
    connections with VCM weights and merges through the reference's hash grid
    vs 8 reference renders of 64 spp."""
    g = np.load(os.path.join(GOLDEN, f"render_vcm_{name}.npz"))
    ref = g["images"].astype(np.float64)
    s = make_golden.golden_scenes()[name]
    h, w = s.camera.height, s.camera.width
    orc = wr_oracle.SceneOracle(s)
    port = np.stack([(orc.render_vcm(64, 8, seed=600 + k, radius=make_golden.VCM_RADIUS)[0] / 64).reshape(h, w, 3)
                     for k in range(8)])
    blk = lambda a: a.reshape(a.shape[0], h // 4, 4, w // 4, 4, 3).mean((2, 4))
    br, bp = blk(ref), blk(port)
    z = (br.mean(0) - bp.mean(0)) / np.sqrt(br.var(0, ddof=1) / 8 + bp.var(0, ddof=1) / 8 + 1e-12)
    assert np.abs(z).max() < 5.0, np.abs(z).max()
    assert means_agree(port, ref, 0.015), (port.mean(), ref.mean())


def test_oracle_vcm_radius_schedule(built):
    """r_s = max(r0 sqrt((s+1)^(alpha-1)), 1e-5) with alpha = 2/3 (vcmTracer.cpp:27)."""
    lib = wr_oracle.load()
    for s in (0, 1, 7, 1000):
        want = np.float32(0.02) * np.sqrt(np.float32(s + 1) ** (np.float32(2.0 / 3) - np.float32(1)))
        assert abs(lib.wro_vcm_radius(0.02, s) / want - 1) < 1e-6
    assert lib.wro_vcm_radius(1e-9, 5) == np.float32(1e-5)


@pytest.mark.parametrize("name", make_golden.PPM_SCENES)
def test_oracle_photon_map_matches_reference_statistically(built, name):
    """PhotonMap (photonMap.cpp:20-625, progressive, base radius 0.02): the
    restated photon density estimation vs 8 reference renders of 64 spp
    ("aniso": the elliptic estimate behind an anisotropic floor; "fog" and
    "hetero": volume photons and the ray-marched eye segments)."""
    g = np.load(os.path.join(GOLDEN, f"render_ppm_{name}.npz"))
    ref = g["images"].astype(np.float64)
    s = make_golden.golden_scenes()[name]
    h, w = s.camera.height, s.camera.width
    orc = wr_oracle.SceneOracle(s)
    port = np.stack([(orc.render_ppm(64, 8, seed=700 + k, radius=make_golden.PPM_RADIUS)[0] / 64).reshape(h, w, 3)
                     for k in range(8)])
    blk = lambda a: a.reshape(a.shape[0], h // 4, 4, w // 4, 4, 3).mean((2, 4))
    br, bp = blk(ref), blk(port)
    z = (br.mean(0) - bp.mean(0)) / np.sqrt(br.var(0, ddof=1) / 8 + bp.var(0, ddof=1) / 8 + 1e-12)
    assert np.abs(z).max() < 5.0, np.abs(z).max()
    assert means_agree(port, ref, 0.02), (port.mean(), ref.mean())


def test_oracle_ellipse_matches_reference_records(built):
    """The anisotropic photon query's ellipse set-up (photonMap.cpp:384-613)
    against the reference's own, recorded in its PhotonMap renders of the
    anisotropic-floor scene for five (Nu, Nv) lobes: the same branch (ellipse,
    sharp-ellipse or projection fallback) everywhere, and bit-identical axis
    ratio and frame (both built with the same C library's acosf, sin, cos,
    exp and sqrt)."""
    g = np.load(os.path.join(GOLDEN, "ppm_ellipse_ref.npz"))
    kind, x = g["kind"], g["inputs"]
    assert set(np.unique(kind)) == {0, 1, 2}
    for i in range(len(kind)):
        k, ratio, ex, ey = wr_oracle.ppm_ellipse(x[i, 0:3], x[i, 3:6], x[i, 6:9], x[i, 9:12], x[i, 12], x[i, 13])
        assert k == kind[i], i
        if k == 0:
            assert ratio == g["ratio"][i] and np.array_equal(ex, g["ex"][i]) and np.array_equal(ey, g["ey"][i]), i


