"""Seeded synthetic scenes for the path-tracing workloads, and the `.wrs` file format.

The reference loads its scenes from XML + OBJ files (config.cpp:432-575,
mesh.cpp:5-130); none ship with it, so every workload here is generated in
code from a seed:

* ``cornell()``           -- Cornell box, 36 triangles, diffuse walls and boxes,
                             one emissive quad (256x256, 64 spp, depth 8).
* ``icosphere_kd()``      -- level-8 icosphere (1,310,720 triangles), radially
                             displaced by 4-octave value noise, plus 2^24 rays
                             (``kd_rays``) for the closest-hit microbenchmark.
* ``mixed_spheres()``     -- 25 displaced level-5 icospheres (20,480 tris each)
                             on a diffuse ground, 40 % diffuse / 40 % Phong /
                             20 % refractive, two area lights (1024^2, 256 spp,
                             depth 16).
* ``cornell_media()``     -- the Cornell box plus a 128^3 fBm heterogeneous
                             medium filling the box and a homogeneous sphere.

Objects carry world-space vertices (the reference's Mesh with an identity
transform, mesh.h:106) and triangle indices local to the object
(faceVertexIndexList, mesh.h:22).  ``Scene.flatten`` produces the arrays of
``wr_scene_desc`` (include/walkray.h); ``save``/``load`` write them to a
``.wrs`` file that the oracle programs read.
"""
from __future__ import annotations

import math
import struct
from dataclasses import dataclass, field

import numpy as np

MAT_DIFFUSE = 0
MAT_GLOSSY = 1
MAT_ANISO = 2
MAT_REFRACTIVE = 3
MAT_EMISSIVE = 4
MAT_HOMOGENEOUS = 5
MAT_HETEROGENEOUS = 6
MAT_REFLECTIVE = 7

MAT_NAMES = {
    MAT_DIFFUSE: "diffuse",
    MAT_GLOSSY: "glossy",
    MAT_ANISO: "aniso",
    MAT_REFRACTIVE: "refractive",
    MAT_EMISSIVE: "emissive",
    MAT_HOMOGENEOUS: "homogeneous",
    MAT_HETEROGENEOUS: "heterogeneous",
    MAT_REFLECTIVE: "reflective",
}

# numpy mirror of wr_object_desc (136 bytes, every field 4 bytes wide)
OBJECT_DTYPE = np.dtype(
    [
        ("type", "<u4"),
        ("vert_begin", "<u4"),
        ("vert_count", "<u4"),
        ("tri_begin", "<u4"),
        ("tri_count", "<u4"),
        ("grid_index", "<u4"),
        ("albedo", "<f4", 3),
        ("emission", "<f4", 3),
        ("power", "<f4"),
        ("ior", "<f4"),
        ("decay", "<f4", 3),
        ("rs", "<f4", 3),
        ("rd", "<f4", 3),
        ("nu", "<f4"),
        ("nv", "<f4"),
        ("sigma_s", "<f4", 3),
        ("sigma_a", "<f4", 3),
        ("g", "<f4"),
        ("density_scale", "<f4"),
        ("step_size", "<f4"),
    ]
)
assert OBJECT_DTYPE.itemsize == 136

FLT_MAX = float(np.finfo(np.float32).max)


@dataclass
class Camera:
    """Camera::setup (camera.h:28-48).  image_plane_dist is in pixels."""

    position: tuple
    focus: tuple
    up: tuple
    width: int
    height: int
    image_plane_dist: float
    lens_radius: float = 0.0
    focal_dist: float = FLT_MAX

    @staticmethod
    def from_fov(position, focus, up, width, height, fov_y_deg):
        dist = (height / 2.0) / math.tan(math.radians(fov_y_deg) / 2.0)
        return Camera(tuple(position), tuple(focus), tuple(up), int(width), int(height), float(np.float32(dist)))


@dataclass
class SceneObject:
    type: int
    verts: np.ndarray  # (n, 3) float32, world space
    faces: np.ndarray  # (m, 3) uint32, local indices
    params: dict = field(default_factory=dict)


@dataclass
class Grid:
    density: np.ndarray  # (nz, ny, nx) float32  -> z-major flat order
    p0: tuple
    p1: tuple


class Scene:
    def __init__(self, name: str = "scene"):
        self.name = name
        self.objects: list[SceneObject] = []
        self.grids: list[Grid] = []
        self.camera: Camera | None = None

    def add(self, type_: int, verts, faces, **params) -> int:
        v = np.ascontiguousarray(np.asarray(verts, dtype=np.float32).reshape(-1, 3))
        f = np.ascontiguousarray(np.asarray(faces, dtype=np.uint32).reshape(-1, 3))
        assert f.size == 0 or int(f.max()) < len(v)
        self.objects.append(SceneObject(type_, v, f, dict(params)))
        return len(self.objects) - 1

    # ------------------------------------------------------------------
    @property
    def num_triangles(self) -> int:
        return int(sum(len(o.faces) for o in self.objects))

    @property
    def num_vertices(self) -> int:
        return int(sum(len(o.verts) for o in self.objects))

    def flatten(self):
        """Arrays of wr_scene_desc: objects (structured), vertices (nv,3) f32,
        triangles (nt,3) u32 with object-local indices, grids."""
        objs = np.zeros(len(self.objects), dtype=OBJECT_DTYPE)
        vb = tb = 0
        for i, o in enumerate(self.objects):
            r = objs[i]
            r["type"] = o.type
            r["vert_begin"], r["vert_count"] = vb, len(o.verts)
            r["tri_begin"], r["tri_count"] = tb, len(o.faces)
            r["grid_index"] = 0xFFFFFFFF
            # reference defaults: RefractiveObject IOR 1.5 / decay 1 (refractiveObj.h:10-11),
            # HeterogeneousVolume IOR 1.5, step 0.002, densityScale 100 (HeterogeneousVolume.h:82-86)
            r["ior"] = 1.5
            r["decay"] = (1.0, 1.0, 1.0)
            r["density_scale"] = 100.0
            r["step_size"] = 0.002
            if o.type == MAT_REFLECTIVE:
                r["albedo"] = (1.0, 1.0, 1.0)  # ReflectiveObject's default color (reflectiveObj.h:10)
            for k, val in o.params.items():
                r[k] = val
            vb += len(o.verts)
            tb += len(o.faces)
        verts = (np.concatenate([o.verts for o in self.objects]) if self.objects else np.zeros((0, 3), np.float32))
        tris = (np.concatenate([o.faces for o in self.objects]) if self.objects else np.zeros((0, 3), np.uint32))
        return objs, np.ascontiguousarray(verts, np.float32), np.ascontiguousarray(tris, np.uint32), self.grids

    def global_triangles(self) -> np.ndarray:
        """(nt,3) triangle indices into the concatenated vertex array
        (the vi_offset renumbering of Scene::buildKDTree, scene.cpp:20-44)."""
        out = []
        off = 0
        for o in self.objects:
            out.append(o.faces.astype(np.int64) + off)
            off += len(o.verts)
        return np.concatenate(out).astype(np.uint32) if out else np.zeros((0, 3), np.uint32)

    def tri_object_ids(self) -> np.ndarray:
        return np.concatenate([np.full(len(o.faces), i, np.int32) for i, o in enumerate(self.objects)])

    # ------------------------------------------------------------------
    def save(self, path: str) -> None:
        objs, verts, tris, grids = self.flatten()
        c = self.camera or Camera((0, 0, 0), (0, 0, 1), (0, 1, 0), 1, 1, 1.0)
        with open(path, "wb") as fh:
            fh.write(b"WRS1")
            fh.write(struct.pack("<5I", 1, len(objs), len(verts), len(tris), len(grids)))
            fh.write(struct.pack("<9f", *c.position, *c.focus, *c.up))
            fh.write(struct.pack("<2I3f", c.width, c.height, c.image_plane_dist, c.lens_radius, c.focal_dist))
            fh.write(objs.tobytes())
            fh.write(verts.tobytes())
            fh.write(tris.tobytes())
            for g in grids:
                nz, ny, nx = g.density.shape
                fh.write(struct.pack("<3I6f", nx, ny, nz, *g.p0, *g.p1))
                fh.write(np.ascontiguousarray(g.density, np.float32).tobytes())

    @staticmethod
    def load(path: str) -> "Scene":
        with open(path, "rb") as fh:
            data = fh.read()
        assert data[:4] == b"WRS1", "not a .wrs scene file"
        off = 4
        ver, no, nv, nt, ng = struct.unpack_from("<5I", data, off)
        off += 20
        cam9 = struct.unpack_from("<9f", data, off)
        off += 36
        w, h, ipd, lr, fd = struct.unpack_from("<2I3f", data, off)
        off += 20
        objs = np.frombuffer(data, OBJECT_DTYPE, no, off).copy()
        off += no * OBJECT_DTYPE.itemsize
        verts = np.frombuffer(data, np.float32, nv * 3, off).reshape(nv, 3).copy()
        off += nv * 12
        tris = np.frombuffer(data, np.uint32, nt * 3, off).reshape(nt, 3).copy()
        off += nt * 12
        s = Scene()
        s.camera = Camera(cam9[0:3], cam9[3:6], cam9[6:9], w, h, ipd, lr, fd)
        for g in range(ng):
            nx, ny, nz = struct.unpack_from("<3I", data, off)
            p = struct.unpack_from("<6f", data, off + 12)
            off += 36
            dens = np.frombuffer(data, np.float32, nx * ny * nz, off).reshape(nz, ny, nx).copy()
            off += nx * ny * nz * 4
            s.grids.append(Grid(dens, p[0:3], p[3:6]))
        skip = {"type", "vert_begin", "vert_count", "tri_begin", "tri_count"}
        for r in objs:
            vb, vc, tb, tc = int(r["vert_begin"]), int(r["vert_count"]), int(r["tri_begin"]), int(r["tri_count"])
            params = {k: (r[k].tolist() if np.ndim(r[k]) else r[k].item()) for k in OBJECT_DTYPE.names if k not in skip}
            s.objects.append(SceneObject(int(r["type"]), verts[vb:vb + vc], tris[tb:tb + tc], params))
        return s


# ----------------------------------------------------------------------------
# geometry helpers
# ----------------------------------------------------------------------------
def _face_normal(p0, p1, p2):
    return np.cross(np.asarray(p1, float) - p0, np.asarray(p2, float) - p0)


def quad(p0, p1, p2, p3, normal):
    """Planar quad p0..p3 (in order around the rim) as two triangles whose
    reference face normal normalize((v1-v0)x(v2-v0)) (mesh.h:52-56) points
    along `normal`."""
    pts = np.asarray([p0, p1, p2, p3], dtype=np.float64)
    faces = np.array([[0, 1, 2], [0, 2, 3]], dtype=np.uint32)
    if np.dot(_face_normal(pts[0], pts[1], pts[2]), normal) < 0:
        faces = faces[:, ::-1].copy()
    return pts.astype(np.float32), faces


def box_mesh(center, size, rot_y_deg=0.0):
    """Closed box (12 triangles, outward normals) rotated about the y axis."""
    c = np.asarray(center, np.float64)
    hx, hy, hz = (np.asarray(size, np.float64) / 2.0)
    corners = np.array([[sx * hx, sy * hy, sz * hz] for sx in (-1, 1) for sy in (-1, 1) for sz in (-1, 1)])
    a = math.radians(rot_y_deg)
    R = np.array([[math.cos(a), 0, math.sin(a)], [0, 1, 0], [-math.sin(a), 0, math.cos(a)]])
    world = corners @ R.T + c

    def idx(sx, sy, sz):
        return ((sx > 0) << 2) | ((sy > 0) << 1) | (sz > 0)

    faces = []
    # each face: 4 corners around the rim, and the outward axis
    rims = {
        (1, 0, 0): [(1, -1, -1), (1, 1, -1), (1, 1, 1), (1, -1, 1)],
        (-1, 0, 0): [(-1, -1, -1), (-1, -1, 1), (-1, 1, 1), (-1, 1, -1)],
        (0, 1, 0): [(-1, 1, -1), (-1, 1, 1), (1, 1, 1), (1, 1, -1)],
        (0, -1, 0): [(-1, -1, -1), (1, -1, -1), (1, -1, 1), (-1, -1, 1)],
        (0, 0, 1): [(-1, -1, 1), (1, -1, 1), (1, 1, 1), (-1, 1, 1)],
        (0, 0, -1): [(-1, -1, -1), (-1, 1, -1), (1, 1, -1), (1, -1, -1)],
    }
    for axis, rim in rims.items():
        ids = [idx(*r) for r in rim]
        n_world = R @ np.asarray(axis, np.float64)
        for tri in ((0, 1, 2), (0, 2, 3)):
            t = [ids[k] for k in tri]
            if np.dot(_face_normal(world[t[0]], world[t[1]], world[t[2]]), n_world) < 0:
                t = t[::-1]
            faces.append(t)
    return world.astype(np.float32), np.asarray(faces, np.uint32)


def icosphere(level: int):
    """Unit icosphere: 20*4^level triangles, outward winding (float64 verts)."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    V = np.array(
        [[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t],
         [0, -1, -t], [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]],
        dtype=np.float64,
    )
    V /= np.linalg.norm(V, axis=1, keepdims=True)
    F = np.array(
        [[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4],
         [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8],
         [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]],
        dtype=np.int64,
    )
    for _ in range(level):
        nv, m = len(V), len(F)
        e = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]])
        es = np.sort(e, axis=1)
        key = es[:, 0] * nv + es[:, 1]
        uniq, inv = np.unique(key, return_inverse=True)
        a, b = uniq // nv, uniq % nv
        mid = V[a] + V[b]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        nid = nv + inv
        m01, m12, m20 = nid[0:m], nid[m:2 * m], nid[2 * m:3 * m]
        F = np.concatenate(
            [np.stack([F[:, 0], m01, m20], 1), np.stack([F[:, 1], m12, m01], 1),
             np.stack([F[:, 2], m20, m12], 1), np.stack([m01, m12, m20], 1)]
        )
        V = np.concatenate([V, mid])
    # outward winding for the reference face normal
    n = np.cross(V[F[:, 1]] - V[F[:, 0]], V[F[:, 2]] - V[F[:, 0]])
    c = (V[F[:, 0]] + V[F[:, 1]] + V[F[:, 2]])
    flip = np.einsum("ij,ij->i", n, c) < 0
    F[flip] = F[flip][:, ::-1]
    return V, F.astype(np.uint32)


# ----------------------------------------------------------------------------
# seeded value noise
# ----------------------------------------------------------------------------
def _hash3(ix, iy, iz, seed):
    with np.errstate(over="ignore"):
        h = (ix.astype(np.uint32) * np.uint32(0x8DA6B343)) ^ (iy.astype(np.uint32) * np.uint32(0xD8163841))
        h ^= iz.astype(np.uint32) * np.uint32(0xCB1AB31F)
        h ^= np.uint32((seed * 0x165667B1) & 0xFFFFFFFF)
        h ^= h >> np.uint32(15)
        h *= np.uint32(0x2C1B3C6D)
        h ^= h >> np.uint32(12)
        h *= np.uint32(0x297A2D39)
        h ^= h >> np.uint32(15)
    return h


def value_noise(p: np.ndarray, seed: int) -> np.ndarray:
    """Trilinear value noise in [-1, 1] on the integer lattice (smoothstep fade)."""
    p = np.asarray(p, np.float64)
    i = np.floor(p)
    f = p - i
    u = f * f * (3.0 - 2.0 * f)
    i = i.astype(np.int64)
    out = np.zeros(len(p))
    for dx in (0, 1):
        wx = u[:, 0] if dx else 1.0 - u[:, 0]
        for dy in (0, 1):
            wy = u[:, 1] if dy else 1.0 - u[:, 1]
            for dz in (0, 1):
                wz = u[:, 2] if dz else 1.0 - u[:, 2]
                h = _hash3(i[:, 0] + dx, i[:, 1] + dy, i[:, 2] + dz, seed)
                val = h.astype(np.float64) * (2.0 / 4294967296.0) - 1.0
                out += wx * wy * wz * val
    return out


def fbm(p: np.ndarray, octaves: int, seed: int, base_freq: float = 2.0) -> np.ndarray:
    """Fractal sum of value noise, normalised to [-1, 1]."""
    total = np.zeros(len(p))
    amp, freq, norm = 1.0, base_freq, 0.0
    for o in range(octaves):
        total += amp * value_noise(np.asarray(p) * freq, seed + 7919 * o)
        norm += amp
        amp *= 0.5
        freq *= 2.0
    return total / norm


def displaced_icosphere(level, center, radius, amplitude, seed, octaves=4):
    V, F = icosphere(level)
    r = 1.0 + amplitude * fbm(V, octaves, seed)
    P = V * (radius * r)[:, None] + np.asarray(center, np.float64)
    return P.astype(np.float32), F


# ----------------------------------------------------------------------------
# workloads
# ----------------------------------------------------------------------------
CORNELL_CAMERA = dict(position=(0.5, 0.5, -1.4), focus=(0.5, 0.5, 0.0), up=(0.0, 1.0, 0.0), fov=40.0)


def _cornell_objects(s: Scene):
    grey = (0.73, 0.73, 0.73)
    s.add(MAT_DIFFUSE, *quad((0, 0, 0), (0, 0, 1), (1, 0, 1), (1, 0, 0), (0, 1, 0)), albedo=grey)   # floor
    s.add(MAT_DIFFUSE, *quad((0, 1, 0), (1, 1, 0), (1, 1, 1), (0, 1, 1), (0, -1, 0)), albedo=grey)  # ceiling
    s.add(MAT_DIFFUSE, *quad((0, 0, 1), (0, 1, 1), (1, 1, 1), (1, 0, 1), (0, 0, -1)), albedo=grey)  # back
    s.add(MAT_DIFFUSE, *quad((0, 0, 0), (0, 1, 0), (0, 1, 1), (0, 0, 1), (1, 0, 0)),
          albedo=(0.63, 0.065, 0.05))                                                             # left (x=0)
    s.add(MAT_DIFFUSE, *quad((1, 0, 0), (1, 0, 1), (1, 1, 1), (1, 1, 0), (-1, 0, 0)),
          albedo=(0.14, 0.45, 0.09))                                                              # right (x=1)
    s.add(MAT_DIFFUSE, *box_mesh((0.68, 0.15, 0.38), (0.3, 0.3, 0.3), -17.0), albedo=grey)  # short box
    s.add(MAT_DIFFUSE, *box_mesh((0.32, 0.30, 0.65), (0.3, 0.6, 0.3), 17.0), albedo=grey)   # tall box
    ly = 0.999
    s.add(MAT_EMISSIVE, *quad((0.375, ly, 0.375), (0.625, ly, 0.375), (0.625, ly, 0.625), (0.375, ly, 0.625),
                              (0, -1, 0)), emission=(17.0, 12.0, 4.0))


def cornell(width=256, height=256) -> Scene:
    """Cornell box: 36 triangles (5 walls, two boxes rotated -17/+17 deg, one
    0.25 x 0.25 light of radiance (17, 12, 4) facing -y), camera at
    (0.5, 0.5, -1.4) looking +z with a 40 deg vertical field of view."""
    s = Scene("cornell")
    _cornell_objects(s)
    c = CORNELL_CAMERA
    s.camera = Camera.from_fov(c["position"], c["focus"], c["up"], width, height, c["fov"])
    assert s.num_triangles == 36
    return s


def cornell_mirror(width=256, height=256, color=(0.9, 0.6, 0.95)) -> Scene:
    """The Cornell box with the tall box a mirror (ReflectiveObject,
    reflectiveObj.h).  The default colour has x > y but z largest, where the
    reference's MAX_VEC_COMP (macros.h:13-16) gives x rather than max(x, y, z)."""
    s = cornell(width, height)
    s.name = "cornell_mirror"
    tall = s.objects[6]
    tall.type = MAT_REFLECTIVE
    tall.params = {"albedo": tuple(color)}
    return s


def cornell_dof(width=256, height=256, lens_radius=0.05, focal_dist=1.8) -> Scene:
    """The Cornell box seen through a thin lens (Camera::setDOFParameters,
    camera.cpp:30-47): lens radius and distance to the plane of focus (the
    tall box is about 1.9 from the camera, the back wall 2.4)."""
    s = cornell(width, height)
    s.name = "cornell_dof"
    s.camera.lens_radius = float(lens_radius)
    s.camera.focal_dist = float(focal_dist)
    return s


def rotate_scene(s: Scene, y_deg: float, x_deg: float) -> Scene:
    """Rotate every vertex and the camera by y_deg about y, then x_deg about x
    (in place; rotation in float64, vertices rounded back to float32)."""
    a, b = math.radians(y_deg), math.radians(x_deg)
    ry = np.array([[math.cos(a), 0, math.sin(a)], [0, 1, 0], [-math.sin(a), 0, math.cos(a)]])
    rx = np.array([[1, 0, 0], [0, math.cos(b), -math.sin(b)], [0, math.sin(b), math.cos(b)]])
    m = rx @ ry
    for o in s.objects:
        o.verts = np.ascontiguousarray((o.verts.astype(np.float64) @ m.T).astype(np.float32))
    c = s.camera
    rot = lambda v: tuple(float(x) for x in m @ np.asarray(v, np.float64))
    c.position, c.focus, c.up = rot(c.position), rot(c.focus), rot(c.up)
    return s


def cornell_aniso(width=256, height=256, nu=10.0, nv=100.0) -> Scene:
    """The Cornell box with an anisotropic glossy floor (AnisotropicGlossyObject,
    anisotropicGlossyObj.h; Ashikhmin-Shirley lobe with exponents Nu, Nv), the
    whole scene turned 20 deg about y and 10 deg about x.  The camera sees the
    walls and boxes reflected in the floor, where photon mapping takes its
    elliptic estimate (photonMap.cpp:383-652); the turn sets the floor's
    tangent frame (Frame::setFromN, frame.h:30-49) about 20 deg off the view,
    since the estimate falls back to the round kernel when the ellipse is
    within about 8 deg of that frame's axes (|cs| or |sn| > 0.99)."""
    s = cornell(width, height)
    s.name = "cornell_aniso"
    floor = s.objects[0]
    floor.type = MAT_ANISO
    floor.params = {"rs": (0.6, 0.6, 0.6), "rd": (0.3, 0.3, 0.3), "nu": float(nu), "nv": float(nv)}
    return rotate_scene(s, 20.0, 10.0)


def icosphere_kd(level=8, seed=1, amplitude=0.05) -> Scene:
    """Closest-hit microbenchmark mesh: unit icosphere of 20*4^level
    triangles displaced radially by 4-octave value noise of the given
    amplitude (level 8: 1,310,720 triangles)."""
    s = Scene(f"icosphere_l{level}")
    P, F = displaced_icosphere(level, (0.0, 0.0, 0.0), 1.0, amplitude, seed)
    s.add(MAT_DIFFUSE, P, F, albedo=(0.5, 0.5, 0.5))
    s.camera = Camera.from_fov((0, 0, -4), (0, 0, 0), (0, 1, 0), 64, 64, 40.0)
    return s


def kd_rays(scene: Scene, n: int, seed=1) -> np.ndarray:
    """n rays (n x 6 float32: origin, direction): origins uniform in a box
    twice the mesh bounds about its centre, directions uniform on the sphere."""
    _, verts, _, _ = scene.flatten()
    lo, hi = verts.min(0).astype(np.float64), verts.max(0).astype(np.float64)
    c, h = (lo + hi) / 2, (hi - lo) / 2
    rng = np.random.default_rng(seed)
    out = np.empty((n, 6), np.float32)
    chunk = 1 << 22
    for s in range(0, n, chunk):
        m = min(chunk, n - s)
        o = c + (rng.random((m, 3)) * 2 - 1) * (2 * h)
        d = rng.standard_normal((m, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        out[s:s + m, 0:3] = o
        out[s:s + m, 3:6] = d
    return out


def mixed_spheres(width=1024, height=1024, seed=7, level=5) -> Scene:
    """25 seeded displaced icospheres (20*4^level triangles each) on a diffuse
    ground; materials by seeded permutation: 10 diffuse (albedo U[0.1,0.9]),
    10 isotropic Phong (exponent U[20,200]), 5 refractive (IOR 1.5); two
    downward-facing area lights."""
    rng = np.random.default_rng(seed)
    s = Scene("mixed_spheres")
    g = 6.0
    s.add(MAT_DIFFUSE, *quad((-g, 0, -g), (-g, 0, g), (g, 0, g), (g, 0, -g), (0, 1, 0)), albedo=(0.5, 0.5, 0.5))
    kinds = np.array([MAT_DIFFUSE] * 10 + [MAT_GLOSSY] * 10 + [MAT_REFRACTIVE] * 5)
    kinds = kinds[rng.permutation(25)]
    for k in range(25):
        cx, cz = (k % 5) - 2.0, (k // 5) - 2.0
        P, F = displaced_icosphere(level, (cx, 0.45, cz), 0.4, 0.05, seed * 1000 + k)
        kind = int(kinds[k])
        albedo = tuple(float(x) for x in rng.uniform(0.1, 0.9, 3))
        power = float(rng.uniform(20.0, 200.0))
        if kind == MAT_DIFFUSE:
            s.add(kind, P, F, albedo=albedo)
        elif kind == MAT_GLOSSY:
            s.add(kind, P, F, albedo=albedo, power=power)
        else:
            s.add(kind, P, F, ior=1.5)
    ly = 4.0
    for (x0, z0, e) in ((-2.25, -1.75, (9.0, 9.0, 8.0)), (0.75, 0.25, (5.0, 6.0, 8.0))):
        x1, z1 = x0 + 1.5, z0 + 1.5
        s.add(MAT_EMISSIVE, *quad((x0, ly, z0), (x1, ly, z0), (x1, ly, z1), (x0, ly, z1), (0, -1, 0)), emission=e)
    s.camera = Camera.from_fov((0.0, 3.2, -6.5), (0.0, 0.3, 0.0), (0, 1, 0), width, height, 40.0)
    return s


def fbm_grid(n=128, octaves=5, seed=3, lo=0.0, hi=4.0) -> np.ndarray:
    """n^3 fBm density (z-major, shape (n, n, n) = [z][y][x]) remapped to [lo, hi]."""
    ax = (np.arange(n) + 0.5) / n
    z, y, x = np.meshgrid(ax, ax, ax, indexing="ij")
    p = np.stack([x.ravel(), y.ravel(), z.ravel()], 1)
    v = fbm(p, octaves, seed, base_freq=3.0)
    v = (v - v.min()) / (v.max() - v.min())
    return (lo + (hi - lo) * v).reshape(n, n, n).astype(np.float32)


def cornell_media(width=512, height=512, grid_n=128, seed=3, step_size=0.002) -> Scene:
    """Cornell box plus a heterogeneous medium (grid_n^3 fBm density in
    [0, 4], HG g = 0.3, albedo 0.8, sigma_t = 1, densityScale 1, IOR 1,
    ray-marching step `step_size`, HeterogeneousVolume's default 0.002) in a
    box just inside the walls, and a homogeneous sphere (sigma_t = 1.5,
    albedo 0.8, g = -0.2, IOR 1) inside that medium."""
    s = Scene("cornell_media")
    _cornell_objects(s)
    lo, hi = (0.001, 0.001, 0.001), (0.999, 0.998, 0.999)
    V, F = box_mesh(((lo[0] + hi[0]) / 2, (lo[1] + hi[1]) / 2, (lo[2] + hi[2]) / 2),
                    (hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]))
    s.grids.append(Grid(fbm_grid(grid_n, 5, seed), tuple(float(x) for x in V.min(0)), tuple(float(x) for x in V.max(0))))
    s.add(MAT_HETEROGENEOUS, V, F, sigma_s=(0.8, 0.8, 0.8), sigma_a=(0.2, 0.2, 0.2), g=0.3, ior=1.0,
          density_scale=1.0, step_size=float(step_size), grid_index=0)
    P, F2 = icosphere(3)
    P = (P * 0.15 + np.array([0.6, 0.55, 0.25])).astype(np.float32)
    s.add(MAT_HOMOGENEOUS, P, F2, sigma_s=(1.2, 1.2, 1.2), sigma_a=(0.3, 0.3, 0.3), g=-0.2, ior=1.0)
    c = CORNELL_CAMERA
    s.camera = Camera.from_fov(c["position"], c["focus"], c["up"], width, height, c["fov"])
    return s


def cornell_fog(width=256, height=256, ior=1.0) -> Scene:
    """Cornell box plus one homogeneous sphere (radius 0.2, sigma_t = 1.5,
    albedo 0.8, HG g = -0.2): participating media without a density grid."""
    s = Scene("cornell_fog")
    _cornell_objects(s)
    P, F = icosphere(3)
    P = (P * 0.2 + np.array([0.55, 0.5, 0.35])).astype(np.float32)
    s.add(MAT_HOMOGENEOUS, P, F, sigma_s=(1.2, 1.2, 1.2), sigma_a=(0.3, 0.3, 0.3), g=-0.2, ior=ior)
    c = CORNELL_CAMERA
    s.camera = Camera.from_fov(c["position"], c["focus"], c["up"], width, height, c["fov"])
    return s


def phong_dome(width=16, height=16, power=100.0, albedo=0.8, elevation_deg=30.0, fov=4.0, aniso=None) -> Scene:
    """One isotropic Phong plane (y = 0, 60 x 60, exponent `power`, grey
    albedo) inside an emissive sphere of radius 50 and radiance 1 facing
    inwards, seen by a narrow camera `elevation_deg` above the plane: every
    pixel shows the plane, and a path of length 2 (plane, then sphere) gives
    the Phong BRDF's directional albedo at the pixel's incidence angle --
    a value fixed by the BRDF alone, against which any sampler of it can be
    checked by numerical integration.  `aniso` = (rs, rd, nu, nv) makes the
    plane anisotropic Phong instead (AnisotropicGlossyObject)."""
    s = Scene("phong_dome")
    g = 30.0
    plane = quad((-g, 0, -g), (-g, 0, g), (g, 0, g), (g, 0, -g), (0, 1, 0))
    if aniso is None:
        s.add(MAT_GLOSSY, *plane, albedo=(albedo, albedo, albedo), power=float(power))
    else:
        rs, rd, nu, nv = aniso
        s.add(MAT_ANISO, *plane, rs=(rs, rs, rs), rd=(rd, rd, rd), nu=float(nu), nv=float(nv))
    V, F = icosphere(4)
    s.add(MAT_EMISSIVE, (V * 50.0).astype(np.float32), F[:, ::-1].copy(), emission=(1.0, 1.0, 1.0))
    e = math.radians(elevation_deg)
    pos = (0.0, 3.0 * math.sin(e), -3.0 * math.cos(e))
    s.camera = Camera.from_fov(pos, (0.0, 0.0, 0.0), (0, 1, 0), width, height, fov)
    return s


def save_rays(path: str, rays: np.ndarray) -> None:
    rays = np.ascontiguousarray(rays, np.float32)
    with open(path, "wb") as fh:
        fh.write(b"WRR1")
        fh.write(struct.pack("<Q", len(rays)))
        fh.write(rays.tobytes())


def load_rays(path: str) -> np.ndarray:
    with open(path, "rb") as fh:
        assert fh.read(4) == b"WRR1"
        (n,) = struct.unpack("<Q", fh.read(8))
        return np.frombuffer(fh.read(n * 24), np.float32).reshape(n, 6).copy()
