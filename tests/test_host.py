"""Host-side logic of the library without a GPU: the C ABI loads and exports
every declared entry point, the Python binding's structures have the
header's sizes and field offsets, the host tree equals the reference tree,
and the boundary rejects malformed input."""
import ctypes as C
import hashlib
import json
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN
import make_golden
import wr_oracle
from walkray_gb300 import _lib as L
from walkray_gb300 import api, scenes as S


def test_library_exports_declared_symbols(built):
    lib = L.load()
    names = L.declared_symbols()
    assert len(names) >= 13
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    v = C.c_uint32()
    assert lib.wr_get_abi_version(C.byref(v)) == 0 and v.value == 2


ABI_STRUCTS = ["wr_object_desc", "wr_camera_desc", "wr_grid_desc", "wr_scene_desc", "wr_scene_file_settings",
               "wr_hit", "wr_scene_info", "wr_ctx_desc", "wr_trace_filter", "wr_render_desc",
               "wr_wavefront_config", "wr_serve_desc", "wr_request_desc", "wr_req_status", "wr_render_profile"]


def test_binding_structs_match_header(tmp_path):
    """Every structure the ctypes binding passes across the C ABI has the
    size and field offsets that include/walkray.h gives it (a C program
    compiled against the header prints them)."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "walkray.h"', "int main(void) {"]
    for name in ABI_STRUCTS:
        lines.append(f'printf("{name} %zu\\n", sizeof({name}));')
        for f, _ in getattr(L, name)._fields_:
            lines.append(f'printf("{name}.{f} %zu\\n", offsetof({name}, {f}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(root, "include"), str(src), "-o", str(exe)], check=True)
    got = dict(line.split() for line in subprocess.run([str(exe)], check=True, capture_output=True,
                                                       text=True).stdout.splitlines())
    for name in ABI_STRUCTS:
        T = getattr(L, name)
        assert int(got[name]) == C.sizeof(T), (name, got[name], C.sizeof(T))
        for f, _ in T._fields_:
            assert int(got[f"{name}.{f}"]) == getattr(T, f).offset, (name, f)


@pytest.mark.parametrize("name", ["cornell", "ico4", "mixed_l2", "media_small"])
def test_host_tree_equals_reference(built, name):
    s = make_golden.golden_scenes()[name]
    _, v, _, _ = s.flatten()
    t = api.build_tree_host(v, s.global_triangles())
    want = json.load(open(os.path.join(GOLDEN, "trees.json")))[name]
    assert hashlib.sha256(api.tree_dump_bytes(t)).hexdigest() == want


@pytest.mark.parametrize("threads", [1, 4])
def test_host_tree_equals_oracle_on_soups(built, threads):
    """Random triangle soups with shared and coincident vertices (leaves with
    several triangles, ratio-0/1 stops): library build == oracle build, for any
    thread count."""
    rng = np.random.default_rng(11)
    for trial in range(6):
        nv = int(rng.integers(3, 400))
        v = rng.random((nv, 3)).astype(np.float32)
        if trial % 2:
            v = np.round(v * 4) / 4  # many coincident coordinates
        nt = int(rng.integers(1, 700))
        tris = rng.integers(0, nv, size=(nt, 3)).astype(np.uint32)
        t = api.build_tree_host(v.astype(np.float32), tris, threads)
        assert api.tree_dump_bytes(t) == wr_oracle.Tree(v, tris).dump()


def test_host_tree_empty_and_single(built):
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    t = api.build_tree_host(v, np.array([[0, 1, 2]], np.uint32))
    assert len(t["left"]) == 1 and t["left"][0] == -1 and list(t["leaf_tris"]) == [0]
    t = api.build_tree_host(v, np.zeros((0, 3), np.uint32))
    assert len(t["left"]) == 1 and t["leaf_count"][0] == 0


def test_host_tree_rejects_bad_indices(built):
    lib = L.load()
    v = np.zeros((3, 3), np.float32)
    tris = np.array([[0, 1, 5]], np.uint32)
    h = C.c_void_p()
    assert lib.wr_kdtree_build_host(L.ptr(v), 3, L.ptr(tris), 1, 1, C.byref(h)) == 1


def test_no_cpu_fallback_without_library(tmp_path, monkeypatch):
    monkeypatch.setattr(L, "LIB_PATH", str(tmp_path / "missing.so"))
    monkeypatch.setattr(L, "_lib", None)
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        L.load()
