"""Animated instances through gbrt_tlas_update (the reference rebuilds its
TLAS every animated frame: gltf_viewer main.rs:395-402 ->
acceleration_structures.rs:136-172 create_top_as).

For a glTF scene whose nodes are moved by keyframe animation
(GltfScene.animate), and for a scene of randomly spinning instances, each
frame's instances go to the GPU through the incremental update and to the
oracle through a full TLAS build; ray hits (t, u, v and ids) are bit-identical
every frame, flattened into the world BVH (default) or kept under a TLAS
(GBRT_BUILD_NO_FLATTEN), and the updates are incremental (no full build).
A rendered frame after the updates meets the per-sample contract.
"""
import numpy as np
import pytest

from rustracer_gb300 import gltf, png, scenes, types as T

from test_gpu_trace import assert_hits_equal
import parity

pytestmark = pytest.mark.gpu


def _rays_at(sd, n, seed):
    """Rays from a box around the scene aimed at random points of its geometry."""
    rng = np.random.default_rng(seed)
    xf = sd.instances["transform"].reshape(-1, 3, 4)
    pts = []
    for x, g in zip(xf, sd.instances["blas_handle"]):
        off, m = int(sd.prims[g]["v_offset"]), int(sd.geo_ranges[g]["v_len"])
        p = sd.vertices["pos"][off:off + m, :3].astype(np.float64)
        pts.append(p @ x[:, :3].T + x[:, 3])
    pts = np.concatenate(pts)
    lo, hi = pts.min(0), pts.max(0)
    c, r = (lo + hi) / 2, np.linalg.norm(hi - lo) / 2 + 1e-3
    tgt = pts[rng.integers(0, len(pts), n)] + rng.normal(0, 0.02 * r, (n, 3))
    org = c + rng.normal(size=(n, 3)) * r * 1.5
    d = tgt - org
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros(n, T.RAY)
    rays["org"], rays["dir"], rays["tmin"], rays["tmax"] = org, d, 0.0, 1e4
    return rays


def _spinning(seed=11, ninst=40):
    rng = np.random.default_rng(seed)
    base = scenes.random_soup(500, seed=seed, extent=0.3, size=0.06, nmat=3)
    axes = rng.normal(size=(ninst, 3))
    axes /= np.linalg.norm(axes, axis=1, keepdims=True)
    pos = rng.uniform(-1.5, 1.5, (ninst, 3))
    geos = rng.integers(0, len(base.prims), ninst)
    identity = np.zeros(ninst, bool)
    identity[::7] = True  # some instances stay at the identity

    def instances(t):
        xfs = []
        for i in range(ninst):
            if identity[i]:
                xfs.append(T.IDENTITY34.copy())
                continue
            a, th = axes[i], 0.7 * t * (1 + i % 3)
            K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
            R = np.eye(3) + np.sin(th) * K + (1 - np.cos(th)) * K @ K
            xfs.append(np.concatenate([R, (pos[i] + 0.1 * t)[:, None]], 1).astype(np.float32).reshape(12))
        return scenes.identity_instances(geos.tolist(), xfs)
    base.instances = instances(0.0)
    return base, instances


@pytest.mark.parametrize("flags", [0, 1], ids=["flattened", "tlas"])
def test_spinning_instances_update(gpu_ctx, flags):
    import pyoracle as O
    from rustracer_gb300 import gbrt
    sd, instances = _spinning()
    sc = gbrt.Scene(gpu_ctx, sd, build_flags=flags)
    orc = O.OracleScene(sd, build_flags=flags, diag=True)
    for frame, t in enumerate((0.4, 0.9, 1.7)):
        inst = instances(t)
        sc.update_tlas(inst)
        orc.tlas(inst)
        sd.instances = inst
        rays = _rays_at(sd, 20000, seed=frame)
        ref, _ = orc.trace(rays)
        hits, st = sc.trace(rays)
        assert st["device_status"] == 0
        assert (ref["instance_id"] != 0xFFFFFFFF).mean() > 0.3
        assert len(np.unique(ref["instance_id"])) > 20
        assert_hits_equal(hits, ref)
        info = sc.info()
        assert info["instance_updates"] >= 1, info  # served without a full build
    # a frame rendered after the updates, against the oracle
    ubo = sd.ubo(64, 48, samples=2, bounces=6, exposure=1.0)
    ref = orc.render(ubo, 64, 48, want_samples=True, want_hits=True, want_margins=True)
    r = sc.render(ubo, gbrt.Accum(gpu_ctx, 64, 48), want_samples=True, want_hits=True, mode=gbrt.MODE_WAVEFRONT)
    assert np.array_equal(r["hits"]["primitive_id"], ref["hits"]["primitive_id"])
    parity.assert_samples(r["samples"], ref, orc, ubo, 64, 48)


def test_topology_change_takes_full_build(gpu_ctx):
    """A changed mask or geometry is not a transform update: the call falls
    back to a full build and still matches the oracle."""
    import pyoracle as O
    from rustracer_gb300 import gbrt
    sd, instances = _spinning(seed=12, ninst=20)
    sc = gbrt.Scene(gpu_ctx, sd)
    inst = instances(0.5)
    inst[3]["custom_index_and_mask"] = inst[3]["custom_index_and_mask"] & 0xFFFFFF  # mask 0: hidden
    sc.update_tlas(inst)
    assert sc.info()["instance_updates"] == 0
    orc = O.OracleScene(sd)
    orc.tlas(inst)
    sd.instances = inst
    rays = _rays_at(sd, 10000, seed=4)
    ref, _ = orc.trace(rays)
    hits, _ = sc.trace(rays)
    assert_hits_equal(hits, ref)
    with pytest.raises(gbrt.GbrtError) as e:
        sc.update_tlas(inst[:-1])
    assert e.value.code == gbrt.E_INVALID


def test_gltf_keyframe_animation(gpu_ctx, tmp_path):
    """GltfScene.animate(t) -> instances() -> gbrt_tlas_update, two frames
    and a wrap of the animation clock, against the oracle."""
    import pyoracle as O
    import test_gltf as TG
    from rustracer_gb300 import gbrt
    tex = np.full((4, 4, 4), 200, np.uint8)
    png.write_png(str(tmp_path / "t.png"), tex)
    TG._write_gltf(str(tmp_path / "s.gltf"), (tmp_path / "t.png").read_bytes())
    sd = gltf.load(str(tmp_path / "s.gltf"))
    g = sd.gltf
    sc = gbrt.Scene(gpu_ctx, sd)
    orc = O.OracleScene(sd)
    moved = []
    for t in (0.5, 1.5, 2.7):
        g.animate(t)
        inst = g.instances()
        moved.append(inst["transform"].copy())
        sc.update_tlas(inst)
        orc.tlas(inst)
        sd.instances = inst
        rays = _rays_at(sd, 8000, seed=int(10 * t))
        ref, _ = orc.trace(rays)
        hits, _ = sc.trace(rays)
        assert (ref["instance_id"] != 0xFFFFFFFF).mean() > 0.2
        assert_hits_equal(hits, ref)
    assert not np.array_equal(moved[0], moved[1])  # the animation moved something
    assert sc.info()["instance_updates"] >= 1
