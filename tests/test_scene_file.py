"""WalkRay's scene files through the library's loader (wr_scene_file_load):
mesh positions bit-identical to the reference's own Mesh::loadShape of the
same files (golden fixture made by tests/golden/make_golden.py with the
reference harness), materials, camera and settings as written, and clear
errors for what the loader does not support.  No GPU needed."""
import os
import shutil

import numpy as np
import pytest

from conftest import GOLDEN
from walkray_gb300 import _lib as L
from walkray_gb300 import api
from walkray_gb300 import scenes as S

XML = os.path.join(GOLDEN, "xml")


@pytest.fixture(scope="module")
def loaded(built):
    return api.load_scene_file(os.path.join(XML, "config.xml"))


def test_meshes_match_reference_loadshape(loaded):
    """Objects in Config::load's order: the group's shapes first, then the
    single objects; every world position and index equal to the reference's."""
    scene, _ = loaded
    ref = np.load(os.path.join(GOLDEN, "mesh_ref.npz"))
    pairs = [(0, "1_0"), (1, "1_1"), (2, "0_0"), (3, "2_0")]  # tetra, slab (group), quad (single), .shp
    assert str(ref["1_0_name"]) == "tetra" and str(ref["1_1_name"]) == "slab"
    for i, key in pairs:
        o = scene.objects[i]
        assert np.array_equal(o.verts.view(np.uint32), ref[key + "_v"].view(np.uint32)), key
        assert np.array_equal(o.faces, ref[key + "_f"]), key


def test_reference_quirks_are_kept(loaded):
    scene, _ = loaded
    ref = np.load(os.path.join(GOLDEN, "mesh_ref.npz"))
    # the group's shapes are scaled by 2 / 9 (the stray vertex at (9, 9, 9)
    # sets the extent) and not centred: the tetra's origin vertex lands on
    # the group transform's translation
    assert np.allclose(scene.objects[0].verts[0], [0.5, 0.3, 0.6])
    # .shp: n floats into n vertices, m indices into m faces, the rest zero
    assert len(scene.objects[3].verts) == 15 and len(scene.objects[3].faces) == 9
    assert not scene.objects[3].faces[3:].any()
    # a single .obj object is centred and scaled into [-1, 1] before its transform
    assert len(ref["0_0_v"]) == 5


def test_materials_camera_and_settings(loaded):
    scene, settings = loaded
    assert settings == {"renderer": "PathTracer", "spp": 64, "max_path_len": 20, "radius": 0.0, "mode": "wavefront"}
    objs, _, _, grids = scene.flatten()
    t = [int(x) for x in objs["type"]]
    assert t == [S.MAT_GLOSSY, S.MAT_REFLECTIVE, S.MAT_ANISO, S.MAT_REFRACTIVE, S.MAT_HETEROGENEOUS,
                 S.MAT_EMISSIVE]
    f32 = lambda *v: np.array(v, np.float32)
    assert np.array_equal(objs[0]["albedo"], f32(0.5, 0.4, 0.3)) and objs[0]["power"] == 40
    assert np.array_equal(objs[1]["albedo"], f32(0.9, 0.6, 0.95))
    assert np.array_equal(objs[2]["rs"], f32(0.3, 0.3, 0.3)) and np.array_equal(objs[2]["rd"], f32(0.2, 0.1, 0.05))
    assert objs[2]["nu"] == 10 and objs[2]["nv"] == 100
    assert objs[3]["ior"] == np.float32(1.33) and np.array_equal(objs[3]["decay"], f32(0.9, 0.95, 1.0))
    fog = objs[4]
    assert fog["g"] == np.float32(0.3) and fog["density_scale"] == 1 and fog["ior"] == 1
    assert np.array_equal(fog["sigma_s"], f32(0.8, 0.8, 0.8)) and np.array_equal(fog["sigma_a"], f32(0.2, 0.2, 0.2))
    assert np.array_equal(objs[5]["emission"], f32(17, 12, 4))
    # the grid: "nx ny nz" then z-major values, spanning the object's box
    (g,) = grids
    assert g.density.shape == (4, 3, 2)
    lines = open(os.path.join(XML, "density.txt")).read().split()
    assert np.array_equal(g.density.ravel(), np.array([float(x) for x in lines[3:]], np.float32))
    v = scene.objects[4].verts
    assert np.allclose(g.p0, v.min(0)) and np.allclose(g.p1, v.max(0))
    c = scene.camera
    assert (c.width, c.height) == (48, 32) and c.image_plane_dist == np.float32(43.95)
    assert c.lens_radius == np.float32(0.01) and c.focal_dist == np.float32(1.9)
    assert tuple(c.position) == tuple(np.float32([0.5, 0.5, -1.4]))


def _variant(tmp_path, old, new, file="materials.xml"):
    d = tmp_path / "xml"
    shutil.copytree(XML, d)
    p = d / file
    s = p.read_text()
    assert old in s
    p.write_text(s.replace(old, new))
    return str(d / "config.xml")


@pytest.mark.parametrize("old,new,file,msg", [
    ("<type>Diffuse</type><color>(0.73", "<type>BumpMapping</type><color>(0.73", "materials.xml", None),
    ("<name>phong</name>", "<name>phong</name></Material><motion/><Material>", "scene.xml", None),
    ("quad_forms.obj</filePath>\n    <Material><path>materials.xml</path><name>aniso",
     "missing.obj</filePath>\n    <Material><path>materials.xml</path><name>aniso", "scene.xml", "missing.obj"),
    ("<power>40</power>", "", "materials.xml", "power"),
    ("<sightDist>43.95</sightDist>", "", "scene.xml", "sightDist"),
    ("</Scene>", "", "scene.xml", "Scene"),
])
def test_unsupported_or_broken_files_fail_clearly(built, tmp_path, old, new, file, msg):
    cfg = _variant(tmp_path, old, new, file)
    if "BumpMapping" in new:  # make the bump-mapped material the one an object uses
        s = open(cfg.replace("config.xml", "scene.xml")).read().replace("<name>phong</name>", "<name>white</name>")
        open(cfg.replace("config.xml", "scene.xml"), "w").write(s)
    with pytest.raises(L.WRError) as e:
        api.load_scene_file(cfg)
    if msg:
        assert msg in str(e.value)


@pytest.mark.parametrize("name,mode", [("BPT", "bidirectional"), ("BidirPathTracer", "bidirectional"),
                                       ("VCMTracer", "vcm"), ("PM", "photon_map"), ("Whitted", None)])
def test_renderer_names_select_modes(built, tmp_path, name, mode):
    """Config::load's renderer names (config.cpp:530-572) and <radius>."""
    cfg = _variant(tmp_path, "<renderer>PathTracer</renderer>", f"<renderer>{name}</renderer><radius>0.03</radius>",
                   "config.xml")
    _, st = api.load_scene_file(cfg)
    assert st["mode"] == mode and st["renderer"] == name and st["radius"] == pytest.approx(0.03)


def test_missing_config_file(built):
    with pytest.raises(L.WRError):
        api.load_scene_file("/nonexistent/config.xml")
