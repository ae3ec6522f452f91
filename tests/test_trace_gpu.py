"""Closest-hit parity on the GPU, through the C ABI (wr_trace_closest):
bit-exact triangle ids and distances against the reference's own answers
(golden fixtures) and against the oracle at full size (2^24 rays on the
1.31M-triangle icosphere), plus edge cases."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
import make_golden
import wr_oracle
from walkray_gb300 import scenes as S

pytestmark = pytest.mark.gpu

NO_HIT = 0xFFFFFFFF


def bary_fp64(scene, rays, tri, t):
    """Barycentrics of v1, v2 at the reference hit point, in FP64 (mesh.h:67-73)."""
    _, V, _, _ = scene.flatten()
    G = scene.global_triangles()
    V = V.astype(np.float64)
    v0, v1, v2 = V[G[tri, 0]], V[G[tri, 1]], V[G[tri, 2]]
    p = rays[:, 0:3].astype(np.float64) + rays[:, 3:6].astype(np.float64) * t.astype(np.float64)[:, None]
    b1, b2, v = v1 - v0, v2 - v0, p - v0
    d12 = np.einsum("ij,ij->i", b1, b2)
    l1 = np.einsum("ij,ij->i", b1, b1)
    l2 = np.einsum("ij,ij->i", b2, b2)
    vb1, vb2 = np.einsum("ij,ij->i", v, b1), np.einsum("ij,ij->i", v, b2)
    u2 = (vb1 * d12 - vb2 * l1) / (d12 * d12 - l1 * l2)
    u1 = (vb1 - u2 * d12) / l1
    return u1, u2


def test_trace_matches_reference_golden(ctx):
    s = make_golden.golden_scenes()["ico4"]
    g = np.load(os.path.join(GOLDEN, "trace_ico4.npz"))
    rays = S.kd_rays(s, 32768, seed=2)
    sid = ctx.upload(s)
    h = ctx.trace_closest(sid, rays)
    assert np.array_equal(h["tri"], g["tri"])
    hit = h["tri"] != NO_HIT
    assert np.array_equal(h["t"][hit].view(np.uint32), g["t"][hit].view(np.uint32))
    # barycentrics: FP32 on the GPU vs FP64 from the reference hit point, 1e-5 relative to the
    # barycentric scale (1) -- the coordinates themselves lie in [0, 1]
    u1, u2 = bary_fp64(s, rays[hit], h["tri"][hit], g["t"][hit])
    assert np.max(np.abs(h["b1"][hit] - u1)) < 1e-5
    assert np.max(np.abs(h["b2"][hit] - u2)) < 1e-5
    ctx.release(sid)


def test_filtered_trace_matches_reference_golden(ctx):
    s = make_golden.golden_scenes()["mixed_l2"]
    g = np.load(os.path.join(GOLDEN, "trace_filtered.npz"))
    rays, ids = make_golden.filtered_rays(s, 32768, seed=5)
    sid = ctx.upload(s)
    h = ctx.trace_closest(sid, rays, ids[:, 0], ids[:, 1])
    assert np.array_equal(h["tri"], g["tri"])
    hit = h["tri"] != NO_HIT
    assert np.array_equal(h["t"][hit].view(np.uint32), g["t"][hit].view(np.uint32))
    ctx.release(sid)


@pytest.mark.parametrize("refill_min,leaf_min,steps", [(1, 1, 1), (32, 32, 1), (4, 3, 1), (8, 8, 2), (4, 8, 8)])
def test_traversal_loop_settings_do_not_change_hits(ctx, refill_min, leaf_min, steps):
    """The warp loop's refill threshold, leaf postponement and steps per turn
    change only the order of work: filtered hits stay equal to the
    reference's."""
    s = make_golden.golden_scenes()["mixed_l2"]
    g = np.load(os.path.join(GOLDEN, "trace_filtered.npz"))
    rays, ids = make_golden.filtered_rays(s, 32768, seed=5)
    sid = ctx.upload(s)
    ctx.set_wavefront_config(capacity=1 << 24, refill_min=refill_min, leaf_min=leaf_min, steps_per_turn=steps)
    try:
        h = ctx.trace_closest(sid, rays, ids[:, 0], ids[:, 1])
    finally:
        ctx.set_wavefront_config(capacity=1 << 24)
    assert np.array_equal(h["tri"], g["tri"])
    hit = h["tri"] != NO_HIT
    assert np.array_equal(h["t"][hit].view(np.uint32), g["t"][hit].view(np.uint32))
    ctx.release(sid)


def test_full_size_icosphere_matches_oracle(ctx):
    """1,310,720 triangles, 2^24 rays: every id and distance bit-identical to
    the oracle (which is pinned to the reference in test_oracle)."""
    s = S.icosphere_kd(8, seed=1)
    rays = S.kd_rays(s, 1 << 24, seed=1)
    sid = ctx.upload(s)
    info = ctx.info(sid)
    assert info["num_nodes"] == 930661
    h = ctx.trace_closest(sid, rays)
    _, v, _, _ = s.flatten()
    tri, t, nb, nt = wr_oracle.Tree(v, s.global_triangles()).trace(rays)
    assert np.array_equal(h["tri"], tri)
    hit = tri != NO_HIT
    assert np.array_equal(h["t"][hit].view(np.uint32), t[hit].view(np.uint32))
    # per-ray traversal work of the reference on this workload (used by the roofline)
    assert abs(nb / len(rays) - 22.5567) < 1e-3 and abs(nt / len(rays) - 2.9383) < 1e-3
    ctx.release(sid)


def test_edge_cases_match_oracle(ctx):
    """Axis-aligned walls (flat boxes), rays along the axes (zero direction
    components), origins on vertices / edges / inside boxes, a zero direction,
    degenerate triangles, and a one-triangle scene (root is a leaf)."""
    rng = np.random.default_rng(3)
    s = S.cornell(16, 16)
    # add a degenerate (zero-area) triangle object and a sliver
    s.add(S.MAT_DIFFUSE, [[0.2, 0.2, 0.2], [0.4, 0.4, 0.4], [0.6, 0.6, 0.6]], [[0, 1, 2]], albedo=(0.5, 0.5, 0.5))
    s.add(S.MAT_DIFFUSE, [[0.1, 0.5, 0.5], [0.9, 0.5, 0.5], [0.5, 0.5000001, 0.5]], [[0, 1, 2]],
          albedo=(0.5, 0.5, 0.5))
    _, V, _, _ = s.flatten()
    G = s.global_triangles()
    n = 40000
    o = np.empty((n, 3), np.float32)
    d = np.empty((n, 3), np.float32)
    k = n // 5
    o[:k] = rng.random((k, 3)) * 1.4 - 0.2
    axes = np.eye(3, dtype=np.float32)[rng.integers(0, 3, k)] * rng.choice([-1, 1], (k, 1))
    d[:k] = axes
    o[k:2 * k] = V[rng.integers(0, len(V), k)]
    d[k:2 * k] = rng.standard_normal((k, 3))
    a, b = V[G[rng.integers(0, len(G), k), 0]], V[G[rng.integers(0, len(G), k), 1]]
    w = rng.random((k, 1)).astype(np.float32)
    o[2 * k:3 * k] = a * w + b * (1 - w)
    d[2 * k:3 * k] = rng.standard_normal((k, 3))
    o[3 * k:4 * k] = rng.random((k, 3))
    d[3 * k:4 * k] = rng.standard_normal((k, 3))
    d[3 * k:3 * k + 100] = 0.0
    o[4 * k:] = np.round(rng.random((n - 4 * k, 3)) * 4) / 4
    d[4 * k:] = np.round(rng.standard_normal((n - 4 * k, 3)) * 2) / 2
    rays = np.concatenate([o, d], 1).astype(np.float32)
    inside = rng.integers(-1, len(s.objects), n).astype(np.int32)
    contact = inside.copy()
    m = rng.random(n) < 0.5
    contact[m] = rng.integers(-1, len(s.objects), m.sum())
    sid = ctx.upload(s)
    tree = wr_oracle.Tree(V, G, s.tri_object_ids())
    for filt in (False, True):
        h = ctx.trace_closest(sid, rays, inside, contact) if filt else ctx.trace_closest(sid, rays)
        tri, t, _, _ = tree.trace(rays, inside, contact) if filt else tree.trace(rays)
        assert np.array_equal(h["tri"], tri)
        hit = tri != NO_HIT
        assert np.array_equal(h["t"][hit].view(np.uint32), t[hit].view(np.uint32))
    ctx.release(sid)
    # one triangle: the root is a leaf
    one = S.Scene("one")
    one.add(S.MAT_DIFFUSE, [[0, 0, 1], [1, 0, 1], [0, 1, 1]], [[0, 1, 2]], albedo=(1, 1, 1))
    sid = ctx.upload(one)
    r = np.array([[0.2, 0.2, 0, 0, 0, 1], [0.9, 0.9, 0, 0, 0, 1], [0.2, 0.2, 2, 0, 0, 1]], np.float32)
    h = ctx.trace_closest(sid, r)
    assert list(h["tri"]) == [0, NO_HIT, NO_HIT] and h["t"][0] == np.float32(1.0)
    ctx.release(sid)


def test_empty_batch_and_bad_arguments(ctx):
    from walkray_gb300 import _lib as L

    s = make_golden.golden_scenes()["cornell"]
    sid = ctx.upload(s)
    assert len(ctx.trace_closest(sid, np.zeros((0, 6), np.float32))) == 0
    with pytest.raises(L.WRError):
        ctx.trace_closest(sid + 1000, np.zeros((1, 6), np.float32))
    ctx.release(sid)
    with pytest.raises(L.WRError):
        ctx.release(sid)


def test_device_entry_point_matches_host_entry_point(ctx):
    torch = pytest.importorskip("torch")
    s = make_golden.golden_scenes()["ico4"]
    rays = S.kd_rays(s, 100000, seed=9)
    sid = ctx.upload(s)
    d_rays = torch.from_numpy(rays).cuda()
    d_hits = torch.empty((len(rays), 4), dtype=torch.int32, device="cuda")
    ctx.trace_closest_device(sid, d_rays.data_ptr(), len(rays), d_hits.data_ptr(),
                             stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    got = d_hits.cpu().numpy().view(np.uint32)
    want = ctx.trace_closest(sid, rays)
    assert np.array_equal(got[:, 0], want["tri"])
    assert np.array_equal(got[:, 1], want["t"].view(np.uint32))
    ctx.release(sid)


@pytest.mark.parametrize("n", [1_000_000, 1_500_000, 4_194_305])
def test_host_batch_chunks_match_device_entry_point(ctx, n):
    """Host batches below, in and above the two-chunk range of the copy
    pipeline (2^20 .. 2^22 rays; 4 chunks from 2^22, here with a ragged last
    chunk): the same hits as the device-buffer entry point."""
    torch = pytest.importorskip("torch")
    s = make_golden.golden_scenes()["ico4"]
    rays = S.kd_rays(s, n, seed=31)
    sid = ctx.upload(s)
    want = ctx.trace_closest(sid, rays)
    d_rays = torch.from_numpy(rays).cuda()
    d_hits = torch.empty((n, 4), dtype=torch.int32, device="cuda")
    ctx.trace_closest_device(sid, d_rays.data_ptr(), n, d_hits.data_ptr(),
                             stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    got = d_hits.cpu().numpy().view(np.uint32)
    assert np.array_equal(got[:, 0], want["tri"])
    assert np.array_equal(got[:, 1], want["t"].view(np.uint32))
    ctx.release(sid)


def test_large_filtered_host_batch_matches_device_entry_point(ctx):
    """4.5 M filtered rays through the host-buffer entry point (four chunks
    through its copy pipeline): the same hits as the device-buffer entry
    point."""
    torch = pytest.importorskip("torch")
    s = make_golden.golden_scenes()["mixed_l2"]
    n = 4_500_000
    rays = S.kd_rays(s, n, seed=21)
    rng = np.random.default_rng(21)
    ids = rng.integers(-1, len(s.objects), size=(n, 2)).astype(np.int32)
    sid = ctx.upload(s)
    want = ctx.trace_closest(sid, rays, ids[:, 0], ids[:, 1])
    d_rays = torch.from_numpy(rays).cuda()
    d_in = torch.from_numpy(np.ascontiguousarray(ids[:, 0])).cuda()
    d_ct = torch.from_numpy(np.ascontiguousarray(ids[:, 1])).cuda()
    d_hits = torch.empty((n, 4), dtype=torch.int32, device="cuda")
    ctx.trace_closest_device(sid, d_rays.data_ptr(), n, d_hits.data_ptr(),
                             stream=torch.cuda.current_stream().cuda_stream, d_inside=d_in.data_ptr(),
                             d_contact=d_ct.data_ptr())
    torch.cuda.synchronize()
    got = d_hits.cpu().numpy().view(np.uint32)
    assert np.array_equal(got[:, 0], want["tri"])
    assert np.array_equal(got[:, 1], want["t"].view(np.uint32))
    assert (want["tri"] != NO_HIT).mean() > 0.05
    ctx.release(sid)



def test_exact_context_visits_every_box_with_the_same_hits():
    """WR_CTX_EXACT_TRAVERSAL (no distance pruning, every box the reference
    visits): the reference's golden hits, filtered and unfiltered, and the
    same answers as the default pruned traversal on 1M random rays."""
    from walkray_gb300.api import Context

    with Context(exact_traversal=True) as ex, Context() as pr:
        s = make_golden.golden_scenes()["ico4"]
        g = np.load(os.path.join(GOLDEN, "trace_ico4.npz"))
        rays = S.kd_rays(s, 32768, seed=2)
        sid = ex.upload(s)
        h = ex.trace_closest(sid, rays)
        assert np.array_equal(h["tri"], g["tri"])
        s2 = make_golden.golden_scenes()["mixed_l2"]
        g2 = np.load(os.path.join(GOLDEN, "trace_filtered.npz"))
        rays2, ids = make_golden.filtered_rays(s2, 32768, seed=5)
        sid2 = ex.upload(s2)
        h2 = ex.trace_closest(sid2, rays2, ids[:, 0], ids[:, 1])
        assert np.array_equal(h2["tri"], g2["tri"])
        big = S.kd_rays(s, 1 << 20, seed=31)
        psid = pr.upload(s)
        a, b = ex.trace_closest(sid, big), pr.trace_closest(psid, big)
        assert np.array_equal(a["tri"], b["tri"])
        assert np.array_equal(a["t"].view(np.uint32), b["t"].view(np.uint32))


def test_device_random_stream_matches_oracle_word_for_word(ctx):
    """The renderers' PathRng on the device, drawn sequentially (block caching
    included), against the oracle's Philox4x32-10 restatement: every raw
    word and every draw bit-identical, for seeds that use both key halves,
    pixels and samples up to 2^32 - 1 and draw indices across block
    boundaries."""
    rng = np.random.default_rng(12)
    n = 4096
    pixel = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    sample = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    dim = rng.integers(0, 130, n).astype(np.uint32)
    pixel[:4] = [0, 0xFFFFFFFF, 1, 7]
    sample[:4] = [0, 0xFFFFFFFF, 2, 0]
    dim[:8] = [0, 1, 2, 3, 4, 5, 127, 128]
    for seed in (1, 0xDEADBEEF, (0x12345678 << 32) | 0x9ABCDEF0):
        words, draws = ctx.rng_draws(seed, pixel, sample, dim)
        key = [seed & 0xFFFFFFFF, seed >> 32]
        for i in range(n):
            w = wr_oracle.philox([int(dim[i]) >> 2, int(sample[i]), int(pixel[i]), 0], key)
            assert np.array_equal(words[i], w), (seed, i)
            d = np.float32(wr_oracle.draw(seed, int(pixel[i]), int(sample[i]), int(dim[i])))
            assert draws[i].view(np.uint32) == d.view(np.uint32), (seed, i)
