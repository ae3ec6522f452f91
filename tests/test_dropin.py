"""The C++ drop-in renderer (walkray_gb300/host/gpuPathTracer.*) compiled
against WalkRay's own headers, and its reading of WalkRay's material objects
(wrDefaultDescribe) checked against the scene descriptions.  Needs a
WalkRay source tree (the environment variable WR_REFERENCE_DIR, else the
oracle Makefile's default); skipped without one."""
import os
import subprocess

import numpy as np
import pytest

import make_golden
from walkray_gb300 import scenes as S
from walkray_gb300.build import reference_dir

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = reference_dir()


@pytest.fixture(scope="module")
def dropin(built):
    if not REF or not os.path.isfile(os.path.join(REF, "kdtree.cpp")):
        pytest.skip("no WalkRay source tree (WR_REFERENCE_DIR)")
    subprocess.run(["make", "-s", "-j8", "-C", os.path.join(ROOT, "oracle"), "dropin", f"REF={REF}"], check=True)
    return os.path.join(ROOT, "oracle", "_ref", "wr_ref_dropin")


@pytest.mark.parametrize("name", ["cornell", "mixed_l2", "mirror"])
def test_dropin_reads_materials(dropin, tmp_path, name):
    s = make_golden.golden_scenes()[name]
    p = str(tmp_path / "s.wrs")
    s.save(p)
    out = str(tmp_path / "d.bin")
    subprocess.run([dropin, "describe", p, out], check=True)
    got = np.fromfile(out, S.OBJECT_DTYPE)
    want, _, _, _ = s.flatten()
    assert len(got) == len(want)
    for g, w in zip(got, want):
        assert g["type"] == w["type"]
        t = int(w["type"])
        if t in (S.MAT_DIFFUSE, S.MAT_GLOSSY):
            assert np.allclose(g["albedo"], w["albedo"], rtol=1e-4)
        if t == S.MAT_GLOSSY:
            assert abs(g["power"] / w["power"] - 1) < 1e-4
        if t == S.MAT_EMISSIVE:
            assert np.array_equal(g["emission"], w["emission"])
        if t == S.MAT_REFRACTIVE:
            assert g["ior"] == w["ior"] and np.array_equal(g["decay"], w["decay"])
        if t == S.MAT_REFLECTIVE:
            assert np.allclose(g["albedo"], w["albedo"], rtol=1e-5)


def test_dropin_rejects_media(dropin, tmp_path):
    s = make_golden.golden_scenes()["media_small"]
    p = str(tmp_path / "s.wrs")
    s.save(p)
    out = str(tmp_path / "d.bin")
    subprocess.run([dropin, "describe", p, out], check=True)
    got = np.fromfile(out, S.OBJECT_DTYPE)
    want, _, _, _ = s.flatten()
    media = np.isin(want["type"], [S.MAT_HOMOGENEOUS, S.MAT_HETEROGENEOUS])
    assert (got["type"][media] == 0xFFFFFFFF).all()
    assert (got["type"][~media] == want["type"][~media]).all()
