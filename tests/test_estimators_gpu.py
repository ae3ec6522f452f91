"""The path tracer's low-variance estimators (WR_RENDER_NEE_MIS,
WR_RENDER_PHONG_MIRROR) keep the reference's expectation:

* NEE with MIS agrees statistically with the reference's own PathTracer
  renders (golden fixtures) on the Cornell box and the homogeneous and
  heterogeneous media scenes (light connections from diffuse surfaces);
* the Phong samplers -- the reference's, about the normal, and the
  mirror-lobe one -- and NEE with MIS on the anisotropic lobe converge to
  the directional albedo of the reference's BRDFs, computed by quadrature
  (a Phong plane in an emissive dome).  The reference's Phong estimator has
  infinite variance for exponents of 3 and more (its weight grows like
  (R.w / N.w)^n near the horizon), and its anisotropic sampler reaches the
  BRDF's diffuse term only through the specular lobe's tails, so renders
  made with them (the mixed-material spheres, exponents 20-200; the
  anisotropic floor) cannot resolve the expectation statistically at any
  practical spp; the quadrature pins it instead;
* the wavefront computes the same per-sample values as the megakernel (sums
  and sums of squares), and the variance actually drops."""
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


@pytest.mark.parametrize("name,flags", [("fog", MIS), ("hetero", MIS)])
def test_scene_matches_reference_pt_renders(ctx, name, flags):
    """The homogeneous sphere and the heterogeneous grid (light connections
    from the diffuse surfaces outside the media) against the reference's
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


def phong_albedo(power, rho, cos_in):
    """Directional albedo of the reference's isotropic Phong BRDF
    (isotropicPhong.h:41-49: rho (n+2)/(2 pi) max(R.w, 0)^n on the upper
    hemisphere) for incoming directions at cosines `cos_in` (array) to the
    normal, by numerical integration in coordinates about the mirror
    direction R: Gauss-Legendre in u = R.w (u^n is a polynomial) times a
    uniform rule in the azimuth.  It depends on the incidence angle only."""
    c = np.atleast_1d(np.asarray(cos_in, np.float64))
    x, wx = np.polynomial.legendre.leggauss(256)
    u, wu = 0.5 * (x + 1.0), 0.5 * wx
    nphi = 4096
    phi = (np.arange(nphi) + 0.5) * (2 * np.pi / nphi)
    s = np.sqrt(np.maximum(0.0, 1.0 - u * u))
    out = np.empty(len(c))
    for i, ci in enumerate(c):
        # R = (sin, cos, 0) about the normal y; w = u R + s (cos(phi) t1 + sin(phi) t2),
        # t1 = (cos, -sin, 0), t2 = (0, 0, 1): the normal component is u cos - s cos(phi) sin
        si = np.sqrt(max(0.0, 1.0 - ci * ci))
        ny = u[:, None] * ci + s[:, None] * (np.cos(phi)[None] * -si)
        out[i] = (wu[:, None] * (u ** power)[:, None] * np.maximum(ny, 0.0)).sum() * (2 * np.pi / nphi)
    return rho * (power + 2) / (2 * np.pi) * out


def camera_rays(scene, sub):
    """The pixels' ray directions (camera.cpp:6-60) on a sub x sub grid of
    each pixel (H, W, sub, sub, 3), the pixel centres' (H, W, 3) and the
    camera's front vector."""
    c = scene.camera
    pos, foc, up = (np.asarray(v, np.float64) for v in (c.position, c.focus, c.up))
    front = (foc - pos) / np.linalg.norm(foc - pos)
    right = np.cross(front, up)
    right /= np.linalg.norm(right)
    top = np.cross(right, front)
    ys, xs = np.mgrid[0:c.height, 0:c.width]
    off = (np.arange(sub) + 0.5) / sub
    u = xs[..., None, None] + off[None, None, :, None]
    v = ys[..., None, None] + off[None, None, None, :]
    d = (front * c.image_plane_dist + right * (u - c.width / 2)[..., None] + top * (c.height / 2 - v)[..., None])
    d /= np.linalg.norm(d, axis=-1, keepdims=True)
    dc = (front * c.image_plane_dist + right * (xs + 0.5 - c.width / 2)[..., None]
          + top * (c.height / 2 - 0.5 - ys)[..., None])
    dc /= np.linalg.norm(dc, axis=-1, keepdims=True)
    return d, dc, front


def dome_expected(scene, power, rho, sub=8):
    """Expected pixel values of the dome scene: per pixel the mean over a
    sub x sub grid of the pixel's rays of cos(front, d) x albedo(d), divided
    by the pixel centre's cosine (fixVignetting)."""
    d, dc, front = camera_rays(scene, sub)
    cos_in = -d[..., 1]
    grid = np.linspace(cos_in.min() - 1e-4, cos_in.max() + 1e-4, 129)
    alb = np.interp(cos_in, grid, phong_albedo(power, rho, grid))
    return ((d @ front) * alb).mean((-1, -2)) / np.abs(dc @ front)


def dome_render(ctx, sc, flags, spp=65536, chunk=4096, seed=700):
    sid = ctx.upload(sc)
    s1 = s2 = 0.0
    for k in range(spp // chunk):
        a, b = ctx.render_stats(sid, chunk, 4, seed=seed + k, flags=flags)
        s1, s2 = s1 + a, s2 + b
    ctx.release(sid)
    m = s1 / spp
    return m, np.sqrt(np.maximum(s2 / spp - m * m, 0) / spp) + 1e-9


@pytest.mark.parametrize("power,flags", [(2.0, 0), (2.0, MIRROR), (100.0, MIRROR), (100.0, LOW_VARIANCE)])
def test_phong_samplers_integrate_the_reference_brdf(ctx, power, flags):
    """The Phong plane in the emissive dome, 60 degrees from the normal: a
    pixel's expectation is the BRDF's directional albedo, computed here by
    quadrature.  The reference's sampler (about the normal; finite variance
    only for exponents below 3) and the mirror-lobe sampler (any exponent,
    alone and with NEE by MIS) converge to it: every pixel within 5
    standard errors and the image mean within 0.3 %."""
    from walkray_gb300 import scenes as S

    rho = 0.8
    sc = S.phong_dome(16, 16, power=power, albedo=rho, elevation_deg=30.0)
    want = dome_expected(sc, power, rho)
    m, se = dome_render(ctx, sc, flags)
    z = (m - want[..., None]) / se
    assert np.abs(z).max() < 5.0, (np.abs(z).max(), m.mean(), want.mean())
    assert abs(m.mean() / want.mean() - 1) < 0.003, (m.mean(), want.mean())


def aniso_brdf(rs, rd, nu, nv, wi, wo):
    """AnisotropicPhong::evalBSDF (anisotropicPhong.h:62-101) on the plane
    y = 0 (normal N = y, Frame::setFromN gives X = x, Z = z), vectorised over
    outgoing directions wo (..., 3); the reference's quirks kept: the
    unparenthesised MAX in the specular denominator, t1 = 1 + (wi.N)/2."""
    N = np.array([0.0, 1.0, 0.0])
    a = abs(wi @ N)
    b = np.abs(wo @ N)
    h = wo - wi
    h /= np.linalg.norm(h, axis=-1, keepdims=True)
    ndh = h @ N
    kdh = np.abs(h @ wi)
    F = rs + (1 - rs) * (1 - kdh) ** 5
    hu, hv = h[..., 2], h[..., 0]
    expo = np.where(np.abs(ndh) < 1e-5, 1.0, (nu * hu * hu + nv * hv * hv) / np.maximum(1 - ndh * ndh, 1e-30))
    den = np.where(kdh * a > b, a, b)
    spec = F * np.sqrt((nu + 1) * (nv + 1)) / (8 * np.pi) * np.maximum(ndh, 0) ** expo / den
    t1, t2 = 1 - (-(wi @ N)) / 2, 1 - (wo @ N) / 2
    diff = rd * (28 / (23 * np.pi)) * (1 - rs) * (1 - t1 ** 5) * (1 - t2 ** 5)
    return spec + diff


def aniso_albedo(rs, rd, nu, nv, wi, n_mu=512, n_phi=2048):
    """Directional albedo of the anisotropic BRDF for incoming direction wi:
    Gauss-Legendre in cos(theta) on (0, 1] times a uniform azimuth rule."""
    x, wx = np.polynomial.legendre.leggauss(n_mu)
    mu, wmu = 0.5 * (x + 1.0), 0.5 * wx
    phi = (np.arange(n_phi) + 0.5) * (2 * np.pi / n_phi)
    st = np.sqrt(1 - mu * mu)
    wo = np.stack([st[:, None] * np.cos(phi)[None], np.broadcast_to(mu[:, None], (n_mu, n_phi)),
                   st[:, None] * np.sin(phi)[None]], -1)
    f = aniso_brdf(rs, rd, nu, nv, wi, wo)
    return float((wmu[:, None] * f * mu[:, None]).sum() * (2 * np.pi / n_phi))


def test_anisotropic_lobe_with_mis_integrates_the_reference_brdf(ctx):
    """The anisotropic Phong plane (Rs 0.6, Rd 0.3, Nu 10, Nv 100, as the
    anisotropic test scene) in the emissive dome, 60 degrees from the normal,
    with next-event estimation by MIS: light samples on the dome weighed
    against the half-vector sampler.  The pixel's expectation is the BRDF's
    directional albedo at the pixel centre's direction (quadrature; the
    albedo changes by under 1e-5 across a pixel); each pixel within 5
    standard errors, the image mean within 0.3 %."""
    from walkray_gb300 import scenes as S

    rs, rd, nu, nv = 0.6, 0.3, 10.0, 100.0
    sc = S.phong_dome(2, 2, aniso=(rs, rd, nu, nv), elevation_deg=30.0, fov=1.0)
    _, dc, _ = camera_rays(sc, 1)
    want = np.array([[aniso_albedo(rs, rd, nu, nv, dc[y, x]) for x in range(2)] for y in range(2)])
    m, se = dome_render(ctx, sc, MIS, spp=1 << 18, chunk=1 << 15, seed=900)
    z = (m - want[..., None]) / se
    assert np.abs(z).max() < 5.0, (np.abs(z).max(), m.mean(), want.mean())
    assert abs(m.mean() / want.mean() - 1) < 0.003, (m.mean(), want.mean())
