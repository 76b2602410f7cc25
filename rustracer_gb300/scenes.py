"""Seeded synthetic scenes in the reference's device layout.

A scene is what the reference's GeoBuilder/Doc produce for its Vulkan path
(crates/libs/asset_loader/src/geometry.rs:100-267, scene_graph.rs:55-81): one
vertex/index pool, one PrimInfo and BLAS per geometry, one TLAS instance per
(node, primitive) whose custom index is the geometry id, MaterialRaw and
LightRaw arrays.  Generators:

* cornell()     -- the 34-triangle Cornell box (explicit, seed-free geometry)
* icosphere_scene() -- Cornell box + seeded noise-displaced icosphere with 24
                   random metallic-roughness materials and 4 point lights
* random_soup() -- random triangles, for traversal tests
"""
from dataclasses import dataclass, field
import math

import numpy as np

from . import types as T
from .camera import make_ubo


@dataclass
class SceneData:
    vertices: np.ndarray
    indices: np.ndarray
    prims: np.ndarray
    materials: np.ndarray
    geo_ranges: np.ndarray
    instances: np.ndarray
    dlights: np.ndarray
    plights: np.ndarray
    textures: list = field(default_factory=list)   # (w, h, format, wrap_s, wrap_t, np.ndarray)
    skybox: tuple = None                           # (face_size, uint8 array 6*size*size*4)
    camera: dict = field(default_factory=dict)     # eye, direction, fov_deg
    skins: np.ndarray = None
    name: str = ""

    @property
    def num_triangles(self):
        return int(sum(int(r["i_len"]) // 3 for r in self.geo_ranges))

    def ubo(self, width, height, **kw):
        cam = dict(self.camera)
        cam.update({k: kw.pop(k) for k in list(kw) if k in ("eye", "direction", "fov_deg")})
        return make_ubo(width, height, cam["eye"], cam["direction"], cam.get("fov_deg", 60.0), **kw)

    @property
    def fully_opaque(self):
        """GeoBuilder::fully_opaque (geometry.rs:60-62)."""
        return bool(np.all(self.geo_ranges["opaque"] != 0))


class GeoBuilder:
    """Accumulates geometries the way the reference's GeoBuilder does:
    vertices and indices appended to shared pools, [v_offset, i_offset,
    material] per geometry (geometry.rs:256-262)."""

    def __init__(self):
        self.vchunks, self.ichunks = [], []
        self.nv = 0
        self.ni = 0
        self.prims, self.ranges = [], []
        self.materials = []

    def add_material(self, m):
        self.materials.append(m)
        return len(self.materials) - 1

    def add_vertices(self, pos, normal=None, uv=None, color=None, tangent=None, skin_index=-1,
                     joints=None, weights=None):
        n = len(pos)
        v = np.zeros(n, T.VERTEX)
        v["pos"][:, :3] = pos
        if normal is not None:
            v["normal"][:, :3] = normal
        v["tangent"] = (1, 0, 0, 0) if tangent is None else tangent
        v["color"] = (1, 1, 1, 1) if color is None else color
        if uv is not None:
            v["uv0"] = uv
        v["skin_index"] = skin_index
        if joints is not None:
            v["joints"] = joints
        if weights is not None:
            v["weights"] = weights
        base = self.nv
        self.vchunks.append(v)
        self.nv += n
        return base

    def add_geometry(self, v_offset, nvert, tri_indices, material_id):
        """tri_indices are relative to v_offset; returns the geometry id."""
        idx = np.asarray(tri_indices, np.uint32).reshape(-1)
        geo = len(self.prims)
        p = np.zeros((), T.PRIMINFO)
        p["v_offset"], p["i_offset"], p["material_id"] = v_offset, self.ni, material_id
        self.prims.append(p)
        r = np.zeros((), T.GEO_RANGE)
        r["geo_id"], r["v_len"], r["i_len"] = geo, nvert, len(idx)
        r["opaque"] = int(self.materials[material_id]["alpha_mode"] == T.ALPHA_OPAQUE)
        self.ranges.append(r)
        self.ichunks.append(idx)
        self.ni += len(idx)
        return geo

    def add_mesh(self, pos, idx, material_id, normal=None, **kw):
        base = self.add_vertices(pos, normal, **kw)
        return self.add_geometry(base, len(pos), idx, material_id)

    def finish(self, instances=None, dlights=None, plights=None, **kw):
        ngeo = len(self.prims)
        if instances is None:
            instances = identity_instances(range(ngeo))
        if dlights is None or len(dlights) == 0:
            dlights = np.array([T.default_dir_light()], T.LIGHT)
        if plights is None:
            plights = np.zeros(0, T.LIGHT)
        return SceneData(
            vertices=np.concatenate(self.vchunks) if self.vchunks else np.zeros(0, T.VERTEX),
            indices=np.concatenate(self.ichunks).astype(np.uint32) if self.ichunks else np.zeros(0, np.uint32),
            prims=np.array(self.prims, T.PRIMINFO), materials=np.array(self.materials, T.MATERIAL),
            geo_ranges=np.array(self.ranges, T.GEO_RANGE), instances=instances,
            dlights=np.asarray(dlights, T.LIGHT), plights=np.asarray(plights, T.LIGHT), **kw)


def identity_instances(geo_ids, transforms=None):
    geo_ids = list(geo_ids)
    inst = np.zeros(len(geo_ids), T.INSTANCE)
    for i, g in enumerate(geo_ids):
        inst[i]["transform"] = T.IDENTITY34 if transforms is None else transforms[i]
        inst[i]["custom_index_and_mask"] = (g & 0xFFFFFF) | (0xFF << 24)
        inst[i]["sbt_offset_and_flags"] = 0x01 << 24  # TRIANGLE_FACING_CULL_DISABLE
        inst[i]["blas_handle"] = g
    return inst


def lambert(rgb, emissive=(0, 0, 0)):
    """'Lambertian' in the reference BRDF: metallic 0, roughness 1."""
    m = T.default_material()
    m["base_color"] = (*rgb, 1.0)
    m["metallic_factor"] = 0.0
    m["roughness_factor"] = 1.0
    m["emissive_factor"] = (*emissive, 0.0)
    return m


def _quad(p0, p1, p2, p3):
    """Two triangles (p0,p1,p2), (p0,p2,p3) with the face normal of p0,p1,p2."""
    pos = np.array([p0, p1, p2, p3], np.float64)
    n = np.cross(pos[1] - pos[0], pos[2] - pos[0])
    n /= np.linalg.norm(n)
    return pos, np.tile(n, (4, 1)), np.array([[0, 1, 2], [0, 2, 3]])


def _box(center, size, angle_deg, drop_bottom=False):
    """Axis box rotated about +y; outward normals; 6 faces (or 5)."""
    sx, sy, sz = (s / 2 for s in size)
    c = np.array(center, np.float64)
    a = math.radians(angle_deg)
    R = np.array([[math.cos(a), 0, math.sin(a)], [0, 1, 0], [-math.sin(a), 0, math.cos(a)]])
    corners = lambda pts: [tuple(R @ np.array(p) + c) for p in pts]
    faces = [
        corners([(-sx, sy, sz), (sx, sy, sz), (sx, sy, -sz), (-sx, sy, -sz)]),    # top (+y)
        corners([(-sx, -sy, sz), (sx, -sy, sz), (sx, sy, sz), (-sx, sy, sz)]),    # front (+z)
        corners([(sx, -sy, -sz), (-sx, -sy, -sz), (-sx, sy, -sz), (sx, sy, -sz)]),  # back (-z)
        corners([(sx, -sy, sz), (sx, -sy, -sz), (sx, sy, -sz), (sx, sy, sz)]),    # right (+x)
        corners([(-sx, -sy, -sz), (-sx, -sy, sz), (-sx, sy, sz), (-sx, sy, -sz)]),  # left (-x)
    ]
    if not drop_bottom:
        faces.append(corners([(-sx, -sy, -sz), (sx, -sy, -sz), (sx, -sy, sz), (-sx, -sy, sz)]))  # bottom
    return faces


class _Soup:
    def __init__(self):
        self.pos, self.nrm, self.idx = [], [], []
        self.n = 0

    def quad(self, *pts):
        p, n, i = _quad(*pts)
        self.pos.append(p)
        self.nrm.append(n)
        self.idx.append(i + self.n)
        self.n += 4

    def arrays(self):
        return np.concatenate(self.pos), np.concatenate(self.nrm), np.concatenate(self.idx)


CORNELL_EYE = (0.0, 0.0, 3.8)
CORNELL_DIR = (0.0, 0.0, -1.0)


def _cornell_into(b):
    grey = b.add_material(lambert((0.73, 0.73, 0.73)))
    red = b.add_material(lambert((0.63, 0.065, 0.05)))
    green = b.add_material(lambert((0.14, 0.45, 0.091)))
    light = b.add_material(lambert((0.78, 0.78, 0.78), emissive=(15.0, 15.0, 15.0)))
    g = _Soup()
    g.quad((-1, -1, 1), (1, -1, 1), (1, -1, -1), (-1, -1, -1))       # floor, normal +y
    g.quad((-1, 1, -1), (1, 1, -1), (1, 1, 1), (-1, 1, 1))           # ceiling, normal -y
    g.quad((-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1))       # back wall, normal +z
    for f in _box((0.35, -0.7, 0.3), (0.6, 0.6, 0.6), -18.0, drop_bottom=True):
        g.quad(*f)
    for f in _box((-0.35, -0.4, -0.3), (0.6, 1.2, 0.6), 18.0):
        g.quad(*f)
    r = _Soup()
    r.quad((-1, -1, 1), (-1, -1, -1), (-1, 1, -1), (-1, 1, 1))       # left wall (red), normal +x
    gr = _Soup()
    gr.quad((1, -1, -1), (1, -1, 1), (1, 1, 1), (1, 1, -1))          # right wall (green), normal -x
    li = _Soup()
    y = 0.999
    li.quad((-0.25, y, -0.25), (0.25, y, -0.25), (0.25, y, 0.25), (-0.25, y, 0.25))  # normal -y
    for soup, mat in ((g, grey), (r, red), (gr, green), (li, light)):
        p, n, i = soup.arrays()
        b.add_mesh(p, i, mat, n)


def cornell():
    """The 34-triangle Cornell box: a 2x2x2 room (5 walls), a 0.5x0.5
    ceiling light with emission 15, a short box 0.6^3 at -18 degrees without
    its bottom face and a tall box 0.6x1.2x0.6 at +18 degrees.  No point
    lights; the default zero-intensity directional light."""
    b = GeoBuilder()
    _cornell_into(b)
    sc = b.finish(camera=dict(eye=CORNELL_EYE, direction=CORNELL_DIR, fov_deg=40.0), name="cornell")
    assert sc.num_triangles == 34
    return sc


def _icosphere(subdiv):
    t = (1.0 + 5 ** 0.5) / 2.0
    verts = np.array([(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t),
                      (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)], np.float64)
    faces = np.array([(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
                      (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
                      (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)], np.int64)
    verts /= np.linalg.norm(verts, axis=1, keepdims=True)
    for _ in range(subdiv):
        e = np.concatenate([faces[:, [0, 1]], faces[:, [1, 2]], faces[:, [2, 0]]])
        e.sort(axis=1)
        uniq, inv = np.unique(e, axis=0, return_inverse=True)
        inv = inv.reshape(-1)
        mid = verts[uniq[:, 0]] + verts[uniq[:, 1]]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        base = len(verts)
        verts = np.concatenate([verts, mid])
        nf = len(faces)
        m01, m12, m20 = (inv[:nf] + base, inv[nf:2 * nf] + base, inv[2 * nf:] + base)
        a, b_, c = faces[:, 0], faces[:, 1], faces[:, 2]
        faces = np.concatenate([np.stack([a, m01, m20], 1), np.stack([b_, m12, m01], 1),
                                np.stack([c, m20, m12], 1), np.stack([m01, m12, m20], 1)])
    return verts, faces


def _value_noise(p, seed, freq=4.0):
    """Seeded trilinear value noise in [0,1)."""
    rng = np.random.default_rng(seed)
    lat = rng.random((17, 17, 17))
    q = (p + 2.0) * freq
    i0 = np.floor(q).astype(np.int64)
    f = q - i0
    f = f * f * (3 - 2 * f)
    i0 %= 16
    out = 0.0
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                w = (f[:, 0] if dx else 1 - f[:, 0]) * (f[:, 1] if dy else 1 - f[:, 1]) * \
                    (f[:, 2] if dz else 1 - f[:, 2])
                out = out + w * lat[i0[:, 0] + dx, i0[:, 1] + dy, i0[:, 2] + dz]
    return out


def _vertex_normals(pos, faces):
    fn = np.cross(pos[faces[:, 1]] - pos[faces[:, 0]], pos[faces[:, 2]] - pos[faces[:, 0]])
    n = np.zeros_like(pos)
    for k in range(3):
        np.add.at(n, faces[:, k], fn)
    return n / np.linalg.norm(n, axis=1, keepdims=True)


def random_pbr_material(rng, rough_lo=0.05, rough_hi=1.0, p_metal=0.3):
    m = T.default_material()
    m["base_color"] = (*rng.uniform(0.1, 0.9, 3), 1.0)
    m["metallic_factor"] = float(rng.random() < p_metal)
    m["roughness_factor"] = rng.uniform(rough_lo, rough_hi)
    return m


def point_light(pos, color, intensity):
    l = np.zeros((), T.LIGHT)
    l["color"] = (*color, 0.0)
    l["transform"] = (*pos, 1.0)
    l["kind"] = 1
    l["range"] = np.finfo(np.float32).max
    l["intensity"] = intensity
    return l


def icosphere_scene(subdiv=7, nmat=24, seed=2, center=(0.3, 0.05, 0.35), radius=0.3):
    """Cornell box + an icosphere of 20*4^subdiv triangles (subdivision 7:
    327,680), displaced along the normal by seeded value noise (amplitude
    0.05*r), per-vertex normals recomputed; nmat random metallic-roughness
    materials (roughness U[0.05,1], metallic Bernoulli(0.3), base colour
    U[0.1,0.9]^3) assigned per face, one geometry per material; 4 point
    lights."""
    rng = np.random.default_rng(seed)
    b = GeoBuilder()
    _cornell_into(b)
    v, f = _icosphere(subdiv)
    disp = 1.0 + 0.05 * (2.0 * _value_noise(v, seed) - 1.0)
    pos = v * (radius * disp)[:, None] + np.asarray(center)
    nrm = _vertex_normals(pos, f)
    mats = [b.add_material(random_pbr_material(rng)) for _ in range(nmat)]
    vbase = b.add_vertices(pos.astype(np.float32), nrm.astype(np.float32))
    assign = rng.integers(0, nmat, len(f))
    for k in range(nmat):
        fk = f[assign == k]
        if len(fk):
            b.add_geometry(vbase, len(pos), fk, mats[k])
    plights = [point_light((-0.5, 0.8, -0.5), (1.0, 0.9, 0.8), 2.0),
               point_light((0.5, 0.8, -0.5), (0.8, 0.9, 1.0), 2.0),
               point_light((-0.5, 0.6, 0.6), (1.0, 1.0, 1.0), 1.5),
               point_light((0.6, 0.5, 0.6), (1.0, 0.8, 0.6), 1.5)]
    return b.finish(plights=np.array(plights, T.LIGHT),
                    camera=dict(eye=CORNELL_EYE, direction=CORNELL_DIR, fov_deg=40.0),
                    name=f"icosphere{subdiv}")


def random_soup(ntri, seed=0, extent=1.0, size=0.05, nmat=4, alpha_mask_fraction=0.0):
    """ntri random small triangles in a cube; optional MASK materials."""
    rng = np.random.default_rng(seed)
    b = GeoBuilder()
    mats = []
    for k in range(nmat):
        m = random_pbr_material(rng)
        if rng.random() < alpha_mask_fraction:
            m["alpha_mode"] = T.ALPHA_MASK
            m["base_color"][3] = rng.uniform(0.2, 0.9)
        mats.append(b.add_material(m))
    c = rng.uniform(-extent, extent, (ntri, 1, 3))
    p = (c + rng.normal(0, size, (ntri, 3, 3))).reshape(-1, 3)
    idx = np.arange(3 * ntri).reshape(-1, 3)
    col = np.ones((3 * ntri, 4))
    col[:, 3] = rng.uniform(0, 1, 3 * ntri)
    nrm = np.repeat(np.cross(p[1::3] - p[0::3], p[2::3] - p[0::3]), 3, axis=0)
    nrm /= np.maximum(np.linalg.norm(nrm, axis=1, keepdims=True), 1e-20)
    per = np.array_split(np.arange(ntri), nmat)
    vbase = b.add_vertices(p.astype(np.float32), nrm.astype(np.float32), color=col.astype(np.float32))
    for k in range(nmat):
        b.add_geometry(vbase, 3 * ntri, idx[per[k]], mats[k])
    return b.finish(camera=dict(eye=(0, 0, 3.0), direction=(0, 0, -1), fov_deg=60.0), name=f"soup{ntri}")


def random_rays(n, seed=0, origin_box=1.5, tmin=0.0, tmax=1e4):
    rng = np.random.default_rng(seed)
    r = np.zeros(n, T.RAY)
    r["org"] = rng.uniform(-origin_box, origin_box, (n, 3))
    d = rng.normal(0, 1, (n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r["dir"] = d
    r["tmin"] = tmin
    r["tmax"] = tmax
    return r
