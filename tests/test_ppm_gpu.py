"""Progressive photon mapping (WR_MODE_PHOTON_MAP) on the GPU through the C
ABI: paired with the oracle's restatement of PhotonMap on the same random
streams, on rotated scenes (the reference's hash grid drops queries outside
the photons' bounding box, which makes the extreme walls of an axis-aligned
scene depend on last bits; see tests/test_vcm_gpu.py), and statistical
against the reference's own PhotonMap renders."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, means_agree
import make_golden
import wr_oracle
from test_vcm_gpu import block_z, rotated
from walkray_gb300 import _lib as L
from walkray_gb300 import scenes as S

pytestmark = pytest.mark.gpu

R = make_golden.PPM_RADIUS


@pytest.mark.parametrize("name", ["cornell", "mirror", "dof", "mixed_l2", "aniso", "fog", "hetero"])
def test_photon_map_paired_with_oracle(ctx, name):
    """The anisotropic-floor scene (already turned off the axes) takes the
    elliptic estimate in about a quarter of its diffuse queries; the fog and
    heterogeneous scenes take volume photons and marched eye segments (the
    heterogeneous medium held to the bar of test_bpt_gpu.PAIRED_BAR)."""
    s = make_golden.golden_scenes()[name]
    s = s if name == "aniso" else rotated(s)
    h, w = s.camera.height, s.camera.width
    frac, mean_tol = (0.85, 1e-2) if name == "hetero" else (0.99, 2e-3)
    sid = ctx.upload(s)
    orc = wr_oracle.SceneOracle(s)
    for seed, radius in ((53, R), (54, 0.05)):
        o = orc.render_ppm(8, 8, seed=seed, radius=radius)[0].reshape(h, w, 3) / 8
        g = ctx.render(sid, 8, 8, seed=seed, mode="photon_map", radius=radius).astype(np.float64)
        assert abs(g.mean() / o.mean() - 1) < mean_tol, (g.mean(), o.mean())
        close = np.isclose(g, o, rtol=1e-3, atol=1e-5)
        assert close.mean() > frac, close.mean()
    ctx.release(sid)


@pytest.mark.parametrize("name", make_golden.PPM_SCENES)
def test_photon_map_matches_reference_renders(ctx, name):
    ref = np.load(os.path.join(GOLDEN, f"render_ppm_{name}.npz"))["images"].astype(np.float64)
    s = make_golden.golden_scenes()[name]
    sid = ctx.upload(s)
    gpu = np.stack([ctx.render(sid, 64, 8, seed=970 + k, mode="photon_map", radius=R).astype(np.float64)
                    for k in range(8)])
    assert np.abs(block_z(gpu, ref, 4)).max() < 5.0
    assert means_agree(gpu, ref, 0.02), (gpu.mean(), ref.mean())
    ctx.release(sid)


def test_photon_map_needs_a_march_step(ctx):
    """A medium's segments are marched in steps of its step_size: zero is rejected."""
    s = make_golden.golden_scenes()["fog"]
    for o in s.objects:
        if o.type == S.MAT_HOMOGENEOUS:
            o.params["step_size"] = 0.0
    sid = ctx.upload(s)
    with pytest.raises(L.WRError) as e:
        ctx.render(sid, 1, 8, mode="photon_map")
    assert "step_size" in str(e.value)
    ctx.render(sid, 1, 8, mode="vcm")  # the other modes do not march
    ctx.release(sid)
