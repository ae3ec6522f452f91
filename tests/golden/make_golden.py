"""Regenerates the golden fixtures in tests/golden/ from WalkRay's own code.

Runs the reference harness (oracle/_ref/wr_ref, built by `make -C oracle ref`
from the reference sources) on small seeded scenes and stores its answers:

  trace_ico4.npz      level-4 displaced icosphere, 32768 rays: reference
                      triangle id and distance per ray (KDTree::intersect)
  trace_filtered.npz  small mixed-material scene, 32768 rays with random
                      inside / contact object ids: reference hits under
                      NoSelfCondition
  trees.json          sha256 of the reference tree dumps (pre-order) of
                      several scenes
  render_cornell.npz  Cornell box 32x32, 8 independent reference renders of
                      256 spp each (PathTracer::renderPixels), as images
  render_cornell_nee.npz  the same with the NEE branch on
  render_mirror.npz   the Cornell box with a mirror tall box (ReflectiveObject),
                      8 reference renders of 256 spp
  render_dof.npz      the Cornell box through a thin lens (depth of field),
                      8 reference renders of 2048 spp
  render_pt_*.npz     PathTracer::renderPixels on the mixed-material (64x64,
                      Phong and refractive spheres), anisotropic-floor,
                      homogeneous-fog and heterogeneous-medium scenes, 8
                      reference renders of 256 spp each
  c0_ref.npz          configuration 0 (Cornell 256x256, 64 spp, depth 8):
                      mean of 256 reference renders (16,384 spp, FP64 sums)
                      and the per-pixel variance of one 64-spp render
  xml/                a scene in WalkRay's file layout (config, scene and
                      material XML, .obj / .shp meshes, a density grid)
  mesh_ref.npz        the reference's Mesh::loadShape of those meshes
                      (single objects and a group), world positions
  render_bpt_*.npz    BidirectionalPathTracer::renderPixels on the Cornell,
                      mirror, thin-lens, mixed-material, homogeneous-fog and
                      heterogeneous-medium (16x16, march step 0.01) scenes,
                      8 reference renders of 64 spp each
  render_vcm_*.npz    VCMTracer::renderPixels (base radius 0.02) on the
                      Cornell, mirror, thin-lens, homogeneous-fog and
                      heterogeneous-medium scenes, 8 reference renders of
                      64 spp each

  render_ppm_*.npz    PhotonMap::renderPixels (base radius 0.02) on the
                      Cornell, mirror, thin-lens, mixed-material,
                      anisotropic-floor, homogeneous-fog and
                      heterogeneous-medium scenes, 8 reference renders of
                      64 spp each
  ppm_ellipse_ref.npz the reference's ellipse set-ups of the anisotropic
                      photon query (inputs and results), recorded in its own
                      PhotonMap renders of the anisotropic-floor scene

Usage: python tests/golden/make_golden.py [pt|c0|bpt|vcm|ppm|ellipse [scene ...]]   (needs
the reference tree on this machine; `pt` / `c0` / `bpt` / `vcm` / `ppm` remake only those
renders, of the scenes named after it if any; the fixtures it writes are what
the tests read elsewhere)
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from walkray_gb300 import scenes as S  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref", "wr_ref")


def golden_scenes():
    """The scenes the fixtures are made on (also rebuilt by the tests)."""
    return {
        "cornell": S.cornell(32, 32),
        "ico4": S.icosphere_kd(4, seed=1),
        "mixed_l2": S.mixed_spheres(64, 64, seed=7, level=2),
        "media_small": S.cornell_media(32, 32, grid_n=16, seed=3),
        "mirror": S.cornell_mirror(32, 32),
        "dof": S.cornell_dof(32, 32, lens_radius=0.2),
        "fog": S.cornell_fog(32, 32, ior=1.2),
        "aniso": S.cornell_aniso(32, 32),
        "hetero": S.cornell_media(16, 16, grid_n=16, seed=3, step_size=0.01),
    }


def filtered_rays(scene: S.Scene, n: int, seed: int):
    rays = S.kd_rays(scene, n, seed=seed)
    rng = np.random.default_rng(seed + 100)
    nobj = len(scene.objects)
    ids = rng.integers(-1, nobj, size=(n, 2)).astype(np.int32)
    same = rng.random(n) < 0.3
    ids[same, 1] = ids[same, 0]
    return rays, ids


def run(args, env=None):
    subprocess.run([REF, *args], check=True, env=env, stdout=subprocess.DEVNULL)


def render_set(scene, p, td, name, extra=(), spp=256):
    """8 single-threaded reference renders (seeds 1..8, depth 8) into `name`."""
    scene.save(p)
    env = dict(os.environ, OMP_NUM_THREADS="1", WR_REF_WORKDIR=td)
    procs, outs = [], []
    for seed in range(1, 9):
        out = os.path.join(td, f"{name}.{seed}.bin")
        procs.append(subprocess.Popen([REF, "render", p, str(spp), "8", str(seed), out, *extra], env=env,
                                      stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL))
        outs.append(out)
    for pr in procs:
        assert pr.wait() == 0
    h, w = scene.camera.height, scene.camera.width
    imgs = np.stack([np.fromfile(o, np.float32).reshape(h, w, 3) for o in outs])
    np.savez_compressed(os.path.join(HERE, name), images=imgs, spp=spp, max_path_len=8)


# --------------------------------------------------------------------------
# a WalkRay-format scene on disk: config, scene and material XML files, meshes
# (.obj with groups and every face form, .shp) and a density grid
# --------------------------------------------------------------------------
XML_DIR = os.path.join(HERE, "xml")
T_QUAD = [0.8, -0.6, 0.0, 0.3, 0.6, 0.8, 0.0, -0.25, 0.0, 0.0, 1.0, 1.2, 0.0, 0.0, 0.0, 1.0]
T_GROUP = [0.35, 0.0, 0.0, 0.5, 0.0, 0.35, 0.0, 0.3, 0.0, 0.0, 0.35, 0.6, 0.0, 0.0, 0.0, 1.0]
T_SHP = [0.2, 0.0, 0.0, 0.3, 0.0, 0.2, 0.0, 0.2, 0.0, 0.0, 0.2, 0.4, 0.0, 0.0, 0.0, 1.0]
T_GRID = [0.15, 0.0, 0.0, 0.7, 0.0, 0.15, 0.0, 0.2, 0.0, 0.0, 0.15, 0.3, 0.0, 0.0, 0.0, 1.0]
MESH_CASES = [  # file, loadShape flow, transform (row-major)
    ("quad_forms.obj", "single", T_QUAD),
    ("two_groups.obj", "group", T_GROUP),
    ("tri.shp", "single", T_SHP),
]


def _mat(T):
    return "".join("[" + ", ".join(repr(float(x)) for x in T[4 * r:4 * r + 4]) + "]" for r in range(4))


def write_xml_fixtures(d=XML_DIR):
    """The scene files (all seeded / fixed, small)."""
    os.makedirs(d, exist_ok=True)
    with open(os.path.join(d, "quad_forms.obj"), "w") as f:
        f.write("# faces in every form Mesh::loadShape reads\n"
                "v -1.0 0.0 -1.0\nv 1.0 0.0 -1.0\nv 1.0 0.0 1.0\nv -1.0 0.0 1.0\nv 0.0 0.5 0.0\n"
                "vt 0 0\nvt 1 0\nvt 1 1\nvn 0 1 0\n"
                "f 1 2 3\nf 1/1 3/2 4/3\nf 1/1/1 2/2/1 5/3/1\nf 2//1 3//1 5//1\nf 3 4 5 1\n")
    with open(os.path.join(d, "two_groups.obj"), "w") as f:
        f.write("v 9 9 9\n"  # before the first group: counted by unitize, in no shape
                "g tetra\nv 0 0 0\nv 1 0 0\nv 0 1 0\nv 0 0 1\nf 2 3 4\nf 2 4 3\nf 2 3 5\nf 3 4 5\n"
                "g slab\nv 2 0 0\nv 3 0 0\nv 3 0.25 2\nv 2 0.25 2\nf 6 7 8\nf 6 8 9\n")
    # .shp: a count n then n floats, a count m then m unsigned (mesh.cpp:20-25)
    vdata = np.array([0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1, 1, 1, 1], np.float32)
    fdata = np.array([0, 1, 2, 0, 1, 3, 1, 2, 4], np.uint32)
    with open(os.path.join(d, "tri.shp"), "wb") as f:
        f.write(np.int32(len(vdata)).tobytes() + vdata.tobytes() + np.int32(len(fdata)).tobytes() + fdata.tobytes())
    rng = np.random.default_rng(11)
    dens = rng.random((4, 3, 2)).astype(np.float32) * 3
    with open(os.path.join(d, "density.txt"), "w") as f:
        f.write("2 3 4\n" + " ".join(repr(float(x)) for x in dens.ravel()) + "\n")
    with open(os.path.join(d, "materials.xml"), "w") as f:
        f.write("""<Material Name="white"><type>Diffuse</type><color>(0.73, 0.73, 0.73)</color></Material>
<Material Name="red"><type>Diffuse</type><color>(0.63, 0.065, 0.05)</color></Material>
<Material Name="phong"><type>Glossy</type><color>(0.5, 0.4, 0.3)</color><power>40</power></Material>
<Material Name="glass"><type>Refractive</type><IOR>1.33</IOR><decayColor>(0.9, 0.95, 1.0)</decayColor></Material>
<Material Name="mirror"><type>Reflective</type><color>(0.9, 0.6, 0.95)</color></Material>
<Material Name="light"><type>Emissive</type><color>(17, 12, 4)</color></Material>
<Material Name="aniso"><type>AnisotropicGlossy</type><Rs>(0.3, 0.3, 0.3)</Rs><Rd>(0.2, 0.1, 0.05)</Rd><Nu>10</Nu><Nv>100</Nv></Material>
<Material Name="fog"><type>GridVolume</type><g>0.3</g><IOR>1.0</IOR><sigma_s>(0.8, 0.8, 0.8)</sigma_s><sigma_a>(0.2, 0.2, 0.2)</sigma_a><density_scale>1</density_scale><density_file>density.txt</density_file></Material>
""")
    with open(os.path.join(d, "scene.xml"), "w") as f:
        f.write(f"""<?xml version="1.0"?>
<!-- a WalkRay scene in the reference's layout -->
<Scene Name="test">
  <GroupObject>
    <filePath>two_groups.obj</filePath>
    <transform>{_mat(T_GROUP)}</transform>
    <Object Name="tetra"><Material><path>materials.xml</path><name>phong</name></Material></Object>
    <Object Name="slab"><Material><path>materials.xml</path><name>mirror</name></Material></Object>
  </GroupObject>
  <Object>
    <filePath>quad_forms.obj</filePath>
    <Material><path>materials.xml</path><name>aniso</name></Material>
    <transform>{_mat(T_QUAD)}</transform>
  </Object>
  <Object>
    <filePath>tri.shp</filePath>
    <Material><path>materials.xml</path><name>glass</name></Material>
    <transform>{_mat(T_SHP)}</transform>
  </Object>
  <Object>
    <filePath>quad_forms.obj</filePath>
    <Material><path>materials.xml</path><name>fog</name></Material>
    <transform>{_mat(T_GRID)}</transform>
  </Object>
  <Object>
    <filePath>quad_forms.obj</filePath>
    <Material><path>materials.xml</path><name>light</name></Material>
    <transform>[0.2, 0.0, 0.0, 0.5][0.0, -0.2, 0.0, 1.0][0.0, 0.0, 0.2, 0.5][0.0, 0.0, 0.0, 1.0]</transform>
  </Object>
  <Camera Name="main">
    <position>(0.5, 0.5, -1.4)</position><focus>(0.5, 0.5, 0.0)</focus><up>(0.0, 1.0, 0.0)</up>
    <width>48</width><height>32</height><sightDist>43.95</sightDist>
    <lensRadius>0.01</lensRadius><focalDist>1.9</focalDist>
  </Camera>
</Scene>
""")
    with open(os.path.join(d, "config.xml"), "w") as f:
        f.write("""<Config>
  <Scene><path>scene.xml</path><name>test</name><camera>main</camera></Scene>
  <renderer>PathTracer</renderer>
  <iter>64</iter>
</Config>
""")


def mesh_fixtures(td):
    """The reference's own Mesh::loadShape of MESH_CASES (harness `mesh`)."""
    out = {}
    for k, (fname, mode, T) in enumerate(MESH_CASES):
        o = os.path.join(td, f"m{k}.bin")
        run(["mesh", os.path.join(XML_DIR, fname), mode, o, *[repr(float(x)) for x in T]])
        b = open(o, "rb").read()
        off, n = 4, int(np.frombuffer(b[:4], np.uint32)[0])
        for j in range(n):
            ln = int(np.frombuffer(b[off:off + 4], np.uint32)[0])
            name = b[off + 4:off + 4 + ln].decode()
            off += 4 + ln
            nv = int(np.frombuffer(b[off:off + 4], np.uint32)[0])
            v = np.frombuffer(b[off + 4:off + 4 + 12 * nv], np.float32).reshape(nv, 3)
            off += 4 + 12 * nv
            nf = int(np.frombuffer(b[off:off + 4], np.uint32)[0])
            f = np.frombuffer(b[off + 4:off + 4 + 12 * nf], np.uint32).reshape(nf, 3)
            off += 4 + 12 * nf
            out[f"{k}_{j}_v"], out[f"{k}_{j}_f"] = v, f
            out[f"{k}_{j}_name"] = np.array(name)
    np.savez_compressed(os.path.join(HERE, "mesh_ref.npz"), **out)


BPT_SCENES = ("cornell", "mirror", "dof", "mixed_l2", "fog", "hetero")


def bpt_fixtures(td, names=BPT_SCENES):
    """BidirectionalPathTracer::renderPixels (bidirPathTracer.cpp:10-56), 8
    reference renders of 64 spp per scene, depth 8."""
    sc = golden_scenes()
    p = os.path.join(td, "s.wrs")
    for name in names:
        render_set(sc[name], p, td, f"render_bpt_{name}.npz", extra=("bpt",), spp=64)


VCM_SCENES = ("cornell", "mirror", "dof", "fog", "hetero")
VCM_RADIUS = 0.02


def vcm_fixtures(td, names=VCM_SCENES):
    """VCMTracer::renderPixels (vcmTracer.cpp:6-92), base radius 0.02, 8
    reference renders of 64 spp per scene, depth 8."""
    sc = golden_scenes()
    p = os.path.join(td, "s.wrs")
    for name in names:
        render_set(sc[name], p, td, f"render_vcm_{name}.npz", extra=("vcm", str(VCM_RADIUS)), spp=64)


PPM_SCENES = ("cornell", "mirror", "dof", "mixed_l2", "aniso", "fog", "hetero")
PPM_RADIUS = 0.02


def ppm_fixtures(td, names=PPM_SCENES):
    """PhotonMap::renderPixels (photonMap.cpp:20-148), base radius 0.02, 8
    reference renders of 64 spp per scene, depth 8."""
    sc = golden_scenes()
    p = os.path.join(td, "s.wrs")
    for name in names:
        render_set(sc[name], p, td, f"render_ppm_{name}.npz", extra=("ppm", str(PPM_RADIUS)), spp=64)


PT_SCENES = ("mixed_l2", "aniso", "fog", "hetero")


def pt_fixtures(td, names=PT_SCENES):
    """PathTracer::renderPixels (pathTracer.cpp:7-76) on the scenes whose
    materials the Cornell fixtures do not cover: isotropic Phong and
    refractive spheres (mixed_l2), the anisotropic Phong floor (aniso), the
    homogeneous sphere (fog) and the heterogeneous grid (hetero, the
    reference's own regular tracking: Simpson steps of 2 x 0.01 and
    Newton-bisection, HeterogeneousVolume.cpp:354-404).  8 reference renders
    of 256 spp per scene, depth 8."""
    sc = golden_scenes()
    p = os.path.join(td, "s.wrs")
    for name in names:
        render_set(sc[name], p, td, f"render_pt_{name}.npz", spp=256)


C0_RENDERS, C0_SPP, C0_DEPTH = 256, 64, 8


def c0_fixture(td, names=None):
    """Configuration 0 as specified (Cornell box, 256x256, 64 spp, depth 8)
    rendered by the reference's PathTracer 256 times (seeds 1..256, one
    thread each, eight at a time).  c0_ref.npz holds the 16,384-spp mean of
    those renders accumulated in FP64 (`mean`, stored as f32), the per-pixel
    variance of one 64-spp render across them (`var64`, 255 degrees of
    freedom, f32), and the reference's own rate of pixel-channels beyond
    3 sigma: for each render, the share of its pixel-channels whose
    difference to the mean of the other 255 exceeds 3 sqrt(var64 (1 +
    1/255)) (`null_frac3`: f64, one per render).  At 64 spp a pixel's
    estimate is far from Gaussian (few paths reach the small light), so this
    share is well above the 0.27 % of a normal distribution; it is the
    yardstick of the per-pixel 3-sigma test."""
    s = S.cornell(256, 256)
    p = os.path.join(td, "c0.wrs")
    s.save(p)
    env = dict(os.environ, OMP_NUM_THREADS="1", WR_REF_WORKDIR=td)
    n = C0_RENDERS
    imgs = np.empty((n, 256, 256, 3), np.float32)
    seeds = list(range(1, n + 1))
    while seeds:
        batch, seeds = seeds[:8], seeds[8:]
        procs = []
        for seed in batch:
            out = os.path.join(td, f"c0.{seed}.bin")
            procs.append((seed, out, subprocess.Popen([REF, "render", p, str(C0_SPP), str(C0_DEPTH), str(seed), out],
                                                      env=env, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)))
        for seed, out, pr in procs:
            assert pr.wait() == 0
            imgs[seed - 1] = np.fromfile(out, np.float32).reshape(256, 256, 3)
            os.remove(out)
    acc = np.zeros((256, 256, 3), np.float64)
    acc2 = np.zeros((256, 256, 3), np.float64)
    for img in imgs:
        x = img.astype(np.float64)
        acc += x
        acc2 += x * x
    mean = acc / n
    var64 = np.maximum(acc2 / n - mean * mean, 0.0) * n / (n - 1)
    null = np.empty(n)
    for k in range(n):
        x = imgs[k].astype(np.float64)
        rest = (acc - x) / (n - 1)
        null[k] = np.mean(np.abs(x - rest) > 3.0 * np.sqrt(var64 * (1.0 + 1.0 / (n - 1)) + 1e-30))
    np.savez_compressed(os.path.join(HERE, "c0_ref.npz"), mean=mean.astype(np.float32),
                        var64=var64.astype(np.float32), null_frac3=null, renders=n, spp=C0_SPP,
                        max_path_len=C0_DEPTH)


ELLIPSE_LOBES = ((10.0, 100.0), (100.0, 10.0), (50.0, 50.0), (5.0, 500.0), (2.0, 20.0))


def ellipse_fixture(td, names=None):
    """The reference's own ellipse set-ups of the anisotropic photon query
    (photonMap.cpp:384-652), recorded by the harness (WR_REF_ELLIPSE_LOG) in
    one 16-spp PhotonMap render of the anisotropic-floor scene per (Nu, Nv) of
    ELLIPSE_LOBES: every elliptic and degenerate-projection record, at most
    400 sharp-ellipse fallbacks per lobe.  ppm_ellipse_ref.npz: kind (i32;
    0 ellipse, 1 sharp, 2 projection), inputs (n, 14) f32 {in_dir, aniso
    normal, reflected dir, hit normal, Nu, Nv}, ratio (n) f32, ex, ey (n, 3)
    f32 (the ellipse frame's mX, mY)."""
    p = os.path.join(td, "s.wrs")
    recs = []
    for nu, nv in ELLIPSE_LOBES:
        S.cornell_aniso(32, 32, nu=nu, nv=nv).save(p)
        log = os.path.join(td, "ellipse.bin")
        env = dict(os.environ, OMP_NUM_THREADS="1", WR_REF_WORKDIR=td, WR_REF_ELLIPSE_LOG=log)
        subprocess.run([REF, "render", p, "16", "8", "1", os.path.join(td, "o.bin"), "ppm", str(PPM_RADIUS)],
                       env=env, check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        r = np.fromfile(log, np.float32).reshape(-1, 22)
        sharp = np.flatnonzero(r[:, 0] == 1)[:400]
        keep = np.sort(np.concatenate([np.flatnonzero(r[:, 0] != 1), sharp]))
        recs.append(r[keep])
    r = np.concatenate(recs)
    np.savez_compressed(os.path.join(HERE, "ppm_ellipse_ref.npz"), kind=r[:, 0].astype(np.int32),
                        inputs=r[:, 1:15], ratio=r[:, 15], ex=r[:, 16:19], ey=r[:, 19:22])


def main():
    if not os.path.exists(REF):
        sys.exit("build the reference harness first: make -C oracle ref")
    only = {"bpt": bpt_fixtures, "vcm": vcm_fixtures, "ppm": ppm_fixtures, "ellipse": ellipse_fixture,
            "pt": pt_fixtures, "c0": c0_fixture}
    if len(sys.argv) >= 2 and sys.argv[1] in only:  # only those renders (of the scenes named after it)
        with tempfile.TemporaryDirectory() as td:
            if len(sys.argv) > 2:
                only[sys.argv[1]](td, sys.argv[2:])
            else:
                only[sys.argv[1]](td)
        return
    sc = golden_scenes()
    with tempfile.TemporaryDirectory() as td:
        # plain traversal
        s = sc["ico4"]
        p = os.path.join(td, "s.wrs")
        s.save(p)
        rays = S.kd_rays(s, 32768, seed=2)
        S.save_rays(os.path.join(td, "r.wrr"), rays)
        run(["trace", p, os.path.join(td, "r.wrr"), os.path.join(td, "h.bin")])
        h = np.fromfile(os.path.join(td, "h.bin"), np.uint32).reshape(-1, 2)
        np.savez_compressed(os.path.join(HERE, "trace_ico4.npz"), tri=h[:, 0], t=h[:, 1].view(np.float32))
        # filtered traversal
        s = sc["mixed_l2"]
        s.save(p)
        rays, ids = filtered_rays(s, 32768, seed=5)
        S.save_rays(os.path.join(td, "r.wrr"), rays)
        ids.tofile(os.path.join(td, "f.bin"))
        run(["trace", p, os.path.join(td, "r.wrr"), os.path.join(td, "h.bin"), os.path.join(td, "f.bin")])
        h = np.fromfile(os.path.join(td, "h.bin"), np.uint32).reshape(-1, 2)
        np.savez_compressed(os.path.join(HERE, "trace_filtered.npz"), tri=h[:, 0], t=h[:, 1].view(np.float32))
        # trees
        trees = {}
        for name in ("cornell", "ico4", "mixed_l2", "media_small"):
            sc[name].save(p)
            run(["dumptree", p, os.path.join(td, "t.bin")])
            trees[name] = hashlib.sha256(open(os.path.join(td, "t.bin"), "rb").read()).hexdigest()
        json.dump(trees, open(os.path.join(HERE, "trees.json"), "w"), indent=1, sort_keys=True)
        # renders (single-threaded: the reference's shared RNG is raced under OpenMP)
        s = sc["cornell"]
        s.save(p)
        env = dict(os.environ, OMP_NUM_THREADS="1", WR_REF_WORKDIR=td)
        procs, outs = [], []
        for seed in range(1, 9):
            out = os.path.join(td, f"img{seed}.bin")
            procs.append(subprocess.Popen([REF, "render", p, "256", "8", str(seed), out], env=env,
                                          stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL))
            outs.append(out)
        for pr in procs:
            assert pr.wait() == 0
        imgs = np.stack([np.fromfile(o, np.float32).reshape(32, 32, 3) for o in outs])
        np.savez_compressed(os.path.join(HERE, "render_cornell.npz"), images=imgs, spp=256, max_path_len=8)
        # the same with the NEE branch switched on (pathTracer.cpp:39-66)
        procs, outs = [], []
        for seed in range(1, 9):
            out = os.path.join(td, f"nee{seed}.bin")
            procs.append(subprocess.Popen([REF, "render", p, "256", "8", str(seed), out, "nee"], env=env,
                                          stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL))
            outs.append(out)
        for pr in procs:
            assert pr.wait() == 0
        imgs = np.stack([np.fromfile(o, np.float32).reshape(32, 32, 3) for o in outs])
        np.savez_compressed(os.path.join(HERE, "render_cornell_nee.npz"), images=imgs, spp=256, max_path_len=8)
        render_set(sc["mirror"], p, td, "render_mirror.npz")
        render_set(sc["dof"], p, td, "render_dof.npz", spp=2048)
        write_xml_fixtures()
        mesh_fixtures(td)
        pt_fixtures(td)
        c0_fixture(td)
        bpt_fixtures(td)
        vcm_fixtures(td)
        ppm_fixtures(td)
        ellipse_fixture(td)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
