"""Seeded synthetic workloads of the batched and serving configurations.

* batched_scene(seed): one of the 32 scenes of the batched configuration --
  a TLAS of instanced procedural meshes (tori) whose triangle counts are
  log-uniform in [1k, 2M]; half of the materials alpha-tested (MASK, cutoff
  0.5) with a 256x256 random FP16 mask in the texture's alpha channel, a
  fifth transmissive (transmission 1, volume on, IOR U[1.3, 1.7]); one
  resolution from {256^2, 512^2, 1280x720, 1920x1080} and spp from
  {1, 4, 16, 64}.  The reference's shaders read alpha from RGBA8 textures;
  FP16 masks are a deviation the oracle shares (same texels, same bilinear
  math).
* serving_pool(): the eight scenes of the serving configuration, 10k to 5M
  triangles, one of them a 64-bone skinned tube animated per job.
* serving_trace(seed, n, rate): n jobs with Poisson arrivals (rate per
  second) over the pool, resolution and spp log-uniform.
* city_scene(): the radiance-cache configuration -- 4,000 instances of a box
  and an icosphere (about 2M instanced triangles), glossy materials, 16
  point lights and a procedural sky.
"""
import math

import numpy as np

from . import types as T
from .scenes import (GeoBuilder, _cornell_into, icosphere_scene, identity_instances, lambert, point_light,
                     random_pbr_material, CORNELL_EYE, CORNELL_DIR)
from . import zoo

RESOLUTIONS = [(256, 256), (512, 512), (1280, 720), (1920, 1080)]
SPPS = [1, 4, 16, 64]


def torus(ntri, R=1.0, r=0.3):
    """A torus of about ntri triangles (nu x nv quads, nu = 2 nv)."""
    nv = max(3, int(round(math.sqrt(ntri / 4.0))))
    nu = max(3, 2 * nv)
    u = np.arange(nu) * (2 * np.pi / nu)
    v = np.arange(nv) * (2 * np.pi / nv)
    uu, vv = np.meshgrid(u, v, indexing="ij")
    x = (R + r * np.cos(vv)) * np.cos(uu)
    z = (R + r * np.cos(vv)) * np.sin(uu)
    y = r * np.sin(vv)
    pos = np.stack([x, y, z], -1).reshape(-1, 3)
    nrm = np.stack([np.cos(vv) * np.cos(uu), np.sin(vv), np.cos(vv) * np.sin(uu)], -1).reshape(-1, 3)
    uv = np.stack([uu / (2 * np.pi) * 4, vv / (2 * np.pi)], -1).reshape(-1, 2)
    i, j = np.meshgrid(np.arange(nu), np.arange(nv), indexing="ij")
    a = i * nv + j
    b = ((i + 1) % nu) * nv + j
    c = ((i + 1) % nu) * nv + (j + 1) % nv
    d = i * nv + (j + 1) % nv
    idx = np.concatenate([np.stack([a, b, c], -1).reshape(-1, 3), np.stack([a, c, d], -1).reshape(-1, 3)])
    return pos.astype(np.float32), nrm.astype(np.float32), uv.astype(np.float32), idx


def _rot(axis, ang):
    axis = np.asarray(axis, np.float64)
    axis /= np.linalg.norm(axis)
    x, y, z = axis
    c, s = math.cos(ang), math.sin(ang)
    return np.array([[c + x * x * (1 - c), x * y * (1 - c) - z * s, x * z * (1 - c) + y * s],
                     [y * x * (1 - c) + z * s, c + y * y * (1 - c), y * z * (1 - c) - x * s],
                     [z * x * (1 - c) - y * s, z * y * (1 - c) + x * s, c + z * z * (1 - c)]])


def mask_texture(rng, n=256):
    """n x n RGBA16F texture: white, alpha uniform random (MASK cutoff 0.5)."""
    img = np.ones((n, n, 4), np.float16)
    img[..., 3] = rng.random((n, n)).astype(np.float16)
    return (n, n, T.TEX_RGBA16F, T.WRAP_REPEAT, T.WRAP_REPEAT, img.view(np.uint16))


def batched_scene(seed, max_tri=2_000_000, min_tri=1_000, nmesh=3, inst_per_mesh=(2, 6)):
    """One scene of the batched configuration (see module docstring).
    Returns (SceneData, width, height, spp)."""
    rng = np.random.default_rng(1000 + seed)
    b = GeoBuilder()
    floor = b.add_material(lambert((0.6, 0.6, 0.6)))
    fpos = np.array([(-8, -1.2, -8), (8, -1.2, -8), (8, -1.2, 8), (-8, -1.2, 8)], np.float32)
    g_floor = b.add_mesh(fpos, np.array([[0, 2, 1], [0, 3, 2]]), floor, np.tile([0, 1.0, 0], (4, 1)).astype(np.float32))
    tex = []
    geos, xforms = [g_floor], [T.IDENTITY34]
    for m in range(nmesh):
        ntri = int(math.exp(rng.uniform(math.log(min_tri), math.log(max_tri))))
        mat = random_pbr_material(rng, rough_lo=0.05, rough_hi=0.8)
        u = rng.random()
        if u < 0.5:
            tex.append(mask_texture(rng))
            mat["alpha_mode"] = T.ALPHA_MASK
            mat["alpha_cutoff"] = 0.5
            mat["base_color_texture"] = (len(tex) - 1, 0)
        elif u < 0.7:
            mat["transmission_exist"] = 1
            mat["transmission_factor"] = 1.0
            mat["volume_exists"] = 1
            mat["ior"] = rng.uniform(1.3, 1.7)
            mat["metallic_factor"] = 0.0
        mid = b.add_material(mat)
        pos, nrm, uv, idx = torus(ntri)
        g = b.add_mesh(pos, idx, mid, nrm, uv=uv)
        for _ in range(int(rng.integers(inst_per_mesh[0], inst_per_mesh[1] + 1))):
            R = _rot(rng.normal(size=3), rng.uniform(0, 2 * np.pi)) * rng.uniform(0.4, 1.0)
            t = rng.uniform((-3, -0.6, -3), (3, 1.5, 3))
            geos.append(g)
            xforms.append(np.concatenate([R, t[:, None]], 1).astype(np.float32).reshape(12))
    inst = identity_instances(geos, transforms=xforms)
    plights = [point_light(rng.uniform((-4, 2, -4), (4, 4, 4)), (1.0, 0.95, 0.9), rng.uniform(4, 8))
               for _ in range(3)]
    W, H = RESOLUTIONS[int(rng.integers(len(RESOLUTIONS)))]
    spp = int(SPPS[int(rng.integers(len(SPPS)))])
    sd = b.finish(instances=inst, plights=np.array(plights, T.LIGHT), textures=tex,
                  camera=dict(eye=(0.0, 2.0, 9.0), direction=(0.0, -0.25, -1.0), fov_deg=50.0),
                  name=f"batched{seed}")
    return sd, W, H, spp


def skinned_scene(bones=64, rings=160, segments=64):
    """Cornell box + a tube of rings x segments quads on a 64-bone chain."""
    return zoo.skinned_tube(rings=rings, segments=segments, bones=bones)


def serving_pool(max_subdiv=9):
    """Eight scenes, 10k..5M triangles; index 7 is the skinned one."""
    pool = [zoo.material_zoo(subdiv=3),             # ~11k
            icosphere_scene(subdiv=5, seed=3),      # ~20k
            icosphere_scene(subdiv=6, seed=4),      # ~82k
            icosphere_scene(subdiv=7, seed=2),      # ~328k
            icosphere_scene(subdiv=8, seed=5),      # ~1.3M
            icosphere_scene(subdiv=max_subdiv, seed=6),  # ~5.2M
            batched_scene(7, max_tri=400_000, min_tri=100_000)[0],
            skinned_scene()]
    return pool


def serving_trace(seed=0, n=200, rate=200.0, nscenes=8, skinned=7, res_lo=256 * 256, res_hi=1920 * 1080,
                  spp_lo=1, spp_hi=256, cache_frac=0.25):
    """n jobs: Poisson arrivals at `rate` per second; scene uniform over the
    pool; pixel count log-uniform in [res_lo, res_hi] at 16:9 (256^2 .. 1080p);
    spp log-uniform in [spp_lo, spp_hi]; jobs on the skinned scene carry an
    animation time; a fraction cache_frac of the jobs (own stream, seed + 1)
    render through their scene's radiance cache."""
    rng = np.random.default_rng(seed)
    use_cache = np.random.default_rng(seed + 1).random(n) < cache_frac
    t = np.cumsum(rng.exponential(1.0 / rate, n))
    jobs = []
    for i in range(n):
        npix = math.exp(rng.uniform(math.log(res_lo), math.log(res_hi)))
        h = max(16, int(round(math.sqrt(npix * 9 / 16))))
        w = max(16, int(round(h * 16 / 9)))
        spp = int(round(math.exp(rng.uniform(math.log(spp_lo), math.log(spp_hi)))))
        k = int(rng.integers(nscenes))
        jobs.append(dict(arrival=float(t[i]), scene=k, width=w, height=h, spp=max(1, spp),
                         anim_time=float(rng.uniform(0, 6.28)) if k == skinned else None,
                         cache=bool(use_cache[i])))
    return jobs


def _box_mesh():
    """Unit cube [-0.5, 0.5]^3 with face normals (24 vertices, 12 triangles)."""
    pos, nrm, idx = [], [], []
    for axis in range(3):
        for sgn in (-1.0, 1.0):
            n = np.zeros(3)
            n[axis] = sgn
            u = np.zeros(3)
            u[(axis + 1) % 3] = 1.0
            v = np.cross(n, u)
            base = len(pos)
            for a, b in ((-1, -1), (1, -1), (1, 1), (-1, 1)):
                pos.append(0.5 * n + 0.5 * a * u + 0.5 * b * v)
                nrm.append(n)
            idx += [(base, base + 1, base + 2), (base, base + 2, base + 3)]
    return np.array(pos, np.float32), np.array(nrm, np.float32), np.array(idx)


def sky_faces(size=32, zenith=(70, 120, 220), horizon=(200, 215, 235), ground=(60, 55, 50)):
    """Procedural cubemap (+X, -X, +Y, -Y, +Z, -Z), RGBA8: a vertical
    gradient from ground through horizon to zenith."""
    faces = np.zeros((6, size, size, 4), np.uint8)
    lerp = lambda a, b, t: (np.asarray(a)[None, None] * (1 - t[..., None]) + np.asarray(b)[None, None] * t[..., None])
    v = (np.arange(size) + 0.5) / size
    t = np.repeat(1.0 - v[:, None], size, 1)  # 1 at the top row, 0 at the bottom
    side = np.where(t[..., None] > 0.5, lerp(horizon, zenith, (t - 0.5) * 2), lerp(ground, horizon, t * 2))
    for f in (0, 1, 4, 5):
        faces[f, ..., :3] = side
    faces[2, ..., :3] = np.asarray(zenith)
    faces[3, ..., :3] = np.asarray(ground)
    faces[..., 3] = 255
    return size, faces.reshape(-1)


def city_scene(seed=0, n_boxes=2500, n_spheres=1500, sphere_subdiv=3, nmat=16):
    """The radiance-cache configuration: a city block of instanced boxes
    (buildings) and spheres, ~2M instanced triangles, glossy materials
    (roughness U[0.02, 0.5]), 16 point lights and a procedural sky."""
    from .scenes import _icosphere
    rng = np.random.default_rng(500 + seed)
    b = GeoBuilder()
    ground_m = b.add_material(lambert((0.35, 0.35, 0.38)))
    gp = np.array([(-60, 0, -40), (60, 0, -40), (60, 0, 40), (-60, 0, 40)], np.float32)
    g_ground = b.add_mesh(gp, np.array([[0, 2, 1], [0, 3, 2]]), ground_m, np.tile([0, 1.0, 0], (4, 1)).astype(np.float32))
    mats = []
    for _ in range(nmat):
        m = random_pbr_material(rng, rough_lo=0.02, rough_hi=0.5)
        mats.append(b.add_material(m))
    bp, bn, bi = _box_mesh()
    vb = b.add_vertices(bp, bn)
    box_geos = [b.add_geometry(vb, len(bp), bi, mats[k]) for k in range(nmat)]
    sv, sf = _icosphere(sphere_subdiv)
    vs = b.add_vertices(sv.astype(np.float32), sv.astype(np.float32))
    sph_geos = [b.add_geometry(vs, len(sv), sf, mats[k]) for k in range(nmat)]
    geos, xf = [g_ground], [T.IDENTITY34]
    for _ in range(n_boxes):  # buildings on a jittered grid
        w, d, h = rng.uniform(1.0, 3.0), rng.uniform(1.0, 3.0), rng.uniform(2.0, 14.0)
        x, z = rng.uniform(-55, 55), rng.uniform(-35, 35)
        ang = rng.uniform(0, np.pi / 2)
        R = _rot((0, 1, 0), ang) @ np.diag([w, h, d])
        geos.append(box_geos[int(rng.integers(nmat))])
        xf.append(np.concatenate([R, np.array([[x], [h / 2], [z]])], 1).astype(np.float32).reshape(12))
    for _ in range(n_spheres):
        r = rng.uniform(0.3, 1.5)
        x, y, z = rng.uniform(-55, 55), rng.uniform(r, 16.0), rng.uniform(-35, 35)
        geos.append(sph_geos[int(rng.integers(nmat))])
        xf.append(np.concatenate([np.eye(3) * r, np.array([[x], [y], [z]])], 1).astype(np.float32).reshape(12))
    inst = identity_instances(geos, transforms=xf)
    plights = [point_light((rng.uniform(-50, 50), rng.uniform(3, 12), rng.uniform(-30, 30)),
                           tuple(rng.uniform(0.7, 1.0, 3)), rng.uniform(20, 60)) for _ in range(16)]
    sd = b.finish(instances=inst, plights=np.array(plights, T.LIGHT), skybox=sky_faces(),
                  camera=dict(eye=(0.0, 28.0, 60.0), direction=(0.0, -0.45, -1.0), fov_deg=55.0), name="city")
    sd.instanced_triangles = int(n_boxes * 12 + n_spheres * len(sf) + 2)
    return sd


def world_box(sd, pad=0.5):
    """Axis-aligned box around a scene's world-space geometry: the vertex
    box's corners carried through every instance transform, padded."""
    p = sd.vertices["pos"][:, :3].astype(np.float64)
    lo, hi = p.min(0), p.max(0)
    corners = np.array([[x, y, z, 1.0] for x in (lo[0], hi[0]) for y in (lo[1], hi[1]) for z in (lo[2], hi[2])])
    if len(sd.instances):
        m = sd.instances["transform"].reshape(-1, 3, 4).astype(np.float64)
        w = np.einsum("nij,cj->nci", m, corners).reshape(-1, 3)
    else:
        w = corners[:, :3]
    return tuple(map(float, w.min(0) - pad)), tuple(map(float, w.max(0) + pad))

