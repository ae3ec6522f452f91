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

Usage: python tests/golden/make_golden.py   (needs the reference tree on this
machine; the fixtures it writes are what the tests read elsewhere)
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


def main():
    if not os.path.exists(REF):
        sys.exit("build the reference harness first: make -C oracle ref")
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
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
