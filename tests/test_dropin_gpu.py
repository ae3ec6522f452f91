"""The drop-in renderer itself on the GPU: GpuPathTracer::renderPixels()
(walkray_gb300/host/gpuPathTracer.cpp) built against stand-ins of the
WalkRay interfaces it uses (tests/dropin_stub/: the renderer base class,
engine, scene, camera, film and object, with WalkRay's names; WalkRay's own
headers are not where the GPU is) and run on configuration 0 as specified.
Its image is held to the rule configuration 0 is held to in
test_parity_gpu.py, against 256 of the reference's own PathTracer renders;
the film and PFM updates after every chunk, and a progress hook that stops
an unbounded render, behave as the reference's progressive loop."""
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN
from walkray_gb300 import scenes as S

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def driver(built, tmp_path_factory):
    d = tmp_path_factory.mktemp("dropin")
    exe = str(d / "run_dropin")
    lib = os.path.join(ROOT, "walkray_gb300")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "tests", "dropin_stub"),
                    "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "walkray_gb300", "host"),
                    "-I", os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests", "dropin_stub", "run_dropin.cpp"),
                    os.path.join(ROOT, "walkray_gb300", "host", "gpuPathTracer.cpp"), "-L", lib, "-lwalkray_gpu",
                    f"-Wl,-rpath,{lib}", "-o", exe], check=True)
    scene = str(d / "cornell.wrs")
    S.cornell(256, 256).save(scene)
    return exe, scene, d


def run(driver, spp, seed, stop=0):
    exe, scene, d = driver
    out = str(d / f"img_{spp}_{seed}.bin")
    r = subprocess.run([exe, scene, str(spp), "8", str(seed), out] + ([str(stop)] if stop else []),
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    stats = {k: int(v) for k, v in re.findall(r"(\w+)=(\d+)", r.stdout)}
    return np.fromfile(out, np.float32).reshape(256, 256, 3).astype(np.float64), stats


def test_renderpixels_matches_reference_renders(driver):
    g = np.load(os.path.join(GOLDEN, "c0_ref.npz"))
    R = g["mean"].astype(np.float64)
    v64 = g["var64"].astype(np.float64)
    n = int(g["renders"])
    img, st = run(driver, 64, 4001)
    assert st["chunks"] >= 1 and st["spp_done"] == 64
    assert st["film_sets"] == st["chunks"] and st["pfm_saves"] == st["chunks"]
    sig = np.sqrt(v64 * (1 + 1 / n) + (1e-5 * R) ** 2 + 1e-30)
    z = (img - R) / sig
    assert np.mean(np.abs(z) > 3) <= float(np.max(g["null_frac3"])) + 0.002
    zm = (img.mean() - R.mean()) / (np.sqrt((sig ** 2).sum()) / img.size)
    assert abs(zm) < 4.0, zm
    expect = float(np.mean(v64 * (1 + 1 / n) / (R ** 2 + 1e-2)))
    rel = float(np.mean((img - R) ** 2 / (R ** 2 + 1e-2)))
    assert abs(rel / expect - 1) < 0.1, (rel, expect)


def test_unbounded_render_stops_when_the_hook_says(driver):
    """spp = INT_MAX, as Config::load gives when a configuration has no
    <iter>: the render runs chunk after chunk until the hook returns true
    after the second, and returns that running mean."""
    img, st = run(driver, 2 ** 31 - 1, 4002, stop=2)
    assert st["chunks"] == 2 and st["spp_done"] > 0
    assert st["film_sets"] == 2 and st["pfm_saves"] == 2
    R = np.load(os.path.join(GOLDEN, "c0_ref.npz"))["mean"].astype(np.float64)
    assert abs(img.mean() / R.mean() - 1) < 0.01, (img.mean(), R.mean())
