"""GPU ray queries vs the CPU oracle, through the C ABI (gbrt_trace_rays).

Contract: the closest hit of every ray -- (t, u, v, instance, primitive,
custom index) -- is bit-identical to the oracle's, whatever BVH each side
built, with ties in t going to the smaller (instance, primitive).  Any-hit
queries (terminate on first hit) agree on hit / no hit.
"""
import numpy as np
import pytest

from rustracer_gb300 import scenes, types as T

pytestmark = pytest.mark.gpu


def oracle_scene(sd):
    import pyoracle as O
    return O.OracleScene(sd)


def assert_hits_equal(gpu, ref):
    assert gpu.dtype == T.HIT and ref.dtype == T.HIT
    for f in ("instance_id", "primitive_id", "custom_index"):
        bad = np.nonzero(gpu[f] != ref[f])[0]
        assert len(bad) == 0, f"{f} differs on {len(bad)} rays, first {bad[:5]}: {gpu[bad[:3]]} vs {ref[bad[:3]]}"
    for f in ("t", "u", "v"):
        assert np.array_equal(gpu[f].view(np.uint32), ref[f].view(np.uint32)), f"{f} not bit-identical"


def test_golden_soup_hits(gpu_ctx):
    from rustracer_gb300 import gbrt
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden_trace_soup.npz"))
    sd = scenes.random_soup(500, seed=7)
    sc = gbrt.Scene(gpu_ctx, sd)
    hits, st = sc.trace(g["rays"])
    assert_hits_equal(hits, g["hits"])
    assert st["device_status"] == 0


@pytest.mark.parametrize("ntri,nray,seed", [(1, 256, 0), (7, 1000, 1), (2000, 20000, 2), (50000, 50000, 3)])
def test_random_soup_closest(gpu_ctx, ntri, nray, seed):
    from rustracer_gb300 import gbrt
    sd = scenes.random_soup(ntri, seed=seed, size=0.05 if ntri > 10 else 0.8)
    rays = scenes.random_rays(nray, seed=seed + 100)
    if ntri < 10:  # aim at the triangles so that some rays hit
        p = sd.vertices["pos"][:, :3].astype(np.float64)
        tgt = p[np.random.default_rng(seed).integers(0, len(p), nray)] * 0.9 + p.mean(0) * 0.1
        d = tgt - rays["org"]
        rays["dir"] = d / np.linalg.norm(d, axis=1, keepdims=True)
    ref, _ = oracle_scene(sd).trace(rays)
    hits, _ = gbrt.Scene(gpu_ctx, sd).trace(rays)
    assert (ref["instance_id"] != 0xFFFFFFFF).sum() > 0
    assert_hits_equal(hits, ref)


def test_random_soup_anyhit(gpu_ctx):
    from rustracer_gb300 import gbrt
    sd = scenes.random_soup(5000, seed=11)
    rays = scenes.random_rays(20000, seed=12)
    rays["tmax"] = np.random.default_rng(3).uniform(0.1, 3.0, len(rays)).astype(np.float32)
    ref, _ = oracle_scene(sd).trace(rays, flags=T.RAY_TERMINATE_ON_FIRST)
    hits, _ = gbrt.Scene(gpu_ctx, sd).trace(rays, flags=T.RAY_TERMINATE_ON_FIRST)
    assert np.array_equal(hits["instance_id"] != 0xFFFFFFFF, ref["instance_id"] != 0xFFFFFFFF)


def test_alpha_mask_closest(gpu_ctx):
    """MASK materials run the any-hit alpha test during traversal
    (RayTracing.rahit:96-98); the accepted closest hit must match."""
    from rustracer_gb300 import gbrt
    sd = scenes.random_soup(3000, seed=21, alpha_mask_fraction=1.0)
    assert not sd.fully_opaque
    rays = scenes.random_rays(20000, seed=22)
    ref, _ = oracle_scene(sd).trace(rays)
    ref_op, _ = oracle_scene(sd).trace(rays, flags=T.RAY_OPAQUE)
    assert (ref["instance_id"] != ref_op["instance_id"]).sum() + (ref["t"] != ref_op["t"]).sum() > 0
    hits, _ = gbrt.Scene(gpu_ctx, sd).trace(rays)
    assert_hits_equal(hits, ref)
    hits_op, _ = gbrt.Scene(gpu_ctx, sd).trace(rays, flags=T.RAY_OPAQUE)
    assert_hits_equal(hits_op, ref_op)


def test_cornell_camera_rays(gpu_ctx):
    from rustracer_gb300 import gbrt
    sd = scenes.cornell()
    rng = np.random.default_rng(5)
    n = 65536
    rays = np.zeros(n, T.RAY)
    rays["org"] = (0.0, 0.0, 3.8)
    d = np.stack([rng.uniform(-0.4, 0.4, n), rng.uniform(-0.4, 0.4, n), -np.ones(n)], 1)
    rays["dir"] = d / np.linalg.norm(d, axis=1, keepdims=True)
    rays["tmin"], rays["tmax"] = 0.001, 10000.0
    ref, _ = oracle_scene(sd).trace(rays)
    hits, _ = gbrt.Scene(gpu_ctx, sd).trace(rays)
    assert_hits_equal(hits, ref)


def _instanced_scene(seed=31, ninst=40):
    """Two-level scene: a few meshes instanced with random rotations,
    scales and translations, plus one identity instance."""
    rng = np.random.default_rng(seed)
    base = scenes.random_soup(300, seed=seed, extent=0.3, size=0.08, nmat=3)
    inst = []
    for i in range(ninst):
        g = int(rng.integers(0, len(base.prims)))
        if i == 0:
            M = T.IDENTITY34.copy()
        else:
            a = rng.normal(size=3)
            a /= np.linalg.norm(a)
            th = rng.uniform(0, 2 * np.pi)
            K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
            R = np.eye(3) + np.sin(th) * K + (1 - np.cos(th)) * K @ K
            R = R * rng.uniform(0.5, 1.5)
            t = rng.uniform(-1.5, 1.5, 3)
            M = np.concatenate([R, t[:, None]], 1).astype(np.float32).reshape(12)
        inst.append((g, M))
    instances = scenes.identity_instances([g for g, _ in inst], [M for _, M in inst])
    base.instances = instances
    return base


@pytest.mark.parametrize("flags", [0, 1], ids=["flattened", "tlas"])
def test_instanced_two_level(gpu_ctx, flags):
    """Transformed instances, flattened into the world BVH (default) or kept
    in BLASes under a TLAS (GBRT_BUILD_NO_FLATTEN); the oracle follows the
    same rule, so hits are bit-identical either way."""
    import pyoracle as O
    from rustracer_gb300 import gbrt
    sd = _instanced_scene()
    rays = scenes.random_rays(30000, seed=32, origin_box=2.0)
    ref, _ = O.OracleScene(sd, build_flags=flags).trace(rays)
    assert len(np.unique(ref["instance_id"])) > 10
    hits, _ = gbrt.Scene(gpu_ctx, sd, build_flags=flags).trace(rays)
    assert_hits_equal(hits, ref)


def test_icosphere_rays_match(gpu_ctx):
    from rustracer_gb300 import gbrt
    sd = scenes.icosphere_scene(subdiv=5)
    rays = scenes.random_rays(50000, seed=41, origin_box=0.9)
    ref, _ = oracle_scene(sd).trace(rays)
    hits, st = gbrt.Scene(gpu_ctx, sd).trace(rays)
    assert_hits_equal(hits, ref)
    assert st["device_status"] == 0


@pytest.mark.parametrize("layout", ["coincident", "grid"])
def test_degenerate_layouts_build_and_match(gpu_ctx, layout):
    """Boxes that tie under the clustering's merge cost: 30,000 copies of one
    triangle (every ray hitting one of them ties in t, so the smallest
    primitive must win) and a regular 200 x 150 grid of equal triangles.  The
    build converges (the clustering pairs tied neighbours) and every hit is
    the oracle's."""
    from rustracer_gb300 import gbrt
    from rustracer_gb300.scenes import GeoBuilder, random_pbr_material
    rng = np.random.default_rng(5)
    b = GeoBuilder()
    mat = b.add_material(random_pbr_material(rng))
    if layout == "coincident":
        n = 30000
        tri = np.array([[-0.5, -0.5, 0.0], [0.5, -0.5, 0.0], [0.0, 0.6, 0.0]])
        p = np.tile(tri, (n, 1))
    else:
        xs, ys = np.meshgrid(np.arange(200), np.arange(150))
        o = np.stack([xs.ravel(), ys.ravel(), np.zeros(xs.size)], 1) * 0.01 - np.array([1.0, 0.75, 0.0])
        p = (o[:, None, :] + np.array([[0.0, 0.0, 0.0], [0.01, 0.0, 0.0], [0.0, 0.01, 0.0]])[None]).reshape(-1, 3)
        n = len(o)
    nrm = np.tile([[0.0, 0.0, 1.0]], (3 * n, 1))
    vb = b.add_vertices(p.astype(np.float32), nrm.astype(np.float32))
    b.add_geometry(vb, 3 * n, np.arange(3 * n).reshape(-1, 3), mat)
    sd = b.finish(camera=dict(eye=(0, 0, 3.0), direction=(0, 0, -1), fov_deg=60.0), name=f"degenerate_{layout}")
    sc = gbrt.Scene(gpu_ctx, sd)
    rays = np.zeros(4096, T.RAY)
    rays["org"] = np.column_stack([rng.uniform(-1, 1, 4096), rng.uniform(-0.8, 0.8, 4096), np.full(4096, 2.0)])
    rays["dir"] = np.tile([0.0, 0.0, -1.0], (4096, 1))
    rays["tmin"] = 0.0
    rays["tmax"] = 1e4
    hits, st = sc.trace(rays)
    ref, _ = oracle_scene(sd).trace(rays)
    assert_hits_equal(hits, ref)
    assert st["device_status"] == 0
    assert (hits["instance_id"] != 0xFFFFFFFF).sum() > 100
