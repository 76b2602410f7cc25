"""GPU vs oracle on every material path of the hit group and on skinning.

* material zoo: textured base colour (sRGB), metallic-roughness texture,
  normal map + tangents, emissive texture, MASK alpha from an RGBA16F
  texture, BLEND from vertex alpha, specular-glossiness, transmission with a
  volume, KHR_materials_specular, unlit, point + directional lights and a
  skybox -- primary hits bit-exact, per-sample radiance within the render
  contract of tests/parity.py, in both the megakernel and the wavefront.
* skinning (AnimationCompute.comp): after gbrt_skin_and_refit the GPU's
  hits on the skinned tube are bit-identical to the oracle's hits on its own
  skinned vertices, for two consecutive animation frames.
"""
import numpy as np
import pytest

import parity
from rustracer_gb300 import scenes, zoo

pytestmark = pytest.mark.gpu

@pytest.fixture(scope="module")
def zoo_ref():
    import pyoracle as O
    sd = zoo.material_zoo()
    ubo = sd.ubo(96, 96, samples=8, bounces=8, exposure=1.0, has_sky=True)
    orc = O.OracleScene(sd, diag=True)
    ref = orc.render(ubo, 96, 96, want_samples=True, want_hits=True, want_margins=True)
    return sd, ubo, ref, orc


@pytest.mark.parametrize("mode", [1, 2], ids=["megakernel", "wavefront"])
def test_material_zoo(gpu_ctx, zoo_ref, mode):
    from rustracer_gb300 import gbrt
    sd, ubo, ref, orc = zoo_ref
    sc = gbrt.Scene(gpu_ctx, sd)
    acc = gbrt.Accum(gpu_ctx, 96, 96)
    r = sc.render(ubo, acc, want_samples=True, want_hits=True, mode=mode)
    gh, rh = r["hits"].reshape(-1), ref["hits"].reshape(-1)
    for f in ("instance_id", "primitive_id"):
        assert np.array_equal(gh[f], rh[f]), f
    assert np.array_equal(gh["t"].view(np.uint32), rh["t"].view(np.uint32))
    # every material sphere is on screen
    prims = set(np.unique(gh["primitive_id"][gh["primitive_id"] >= 0]).tolist())
    assert len(prims) > 500
    parity.assert_samples(r["samples"], ref, orc, ubo, 96, 96)
    diff = np.abs(r["image"].astype(int) - ref["image"].astype(int))
    assert (diff <= 1).mean() > 0.98


def _tube_rays(sd, n=20000, seed=3):
    rng = np.random.default_rng(seed)
    rays = scenes.random_rays(n, seed=seed, origin_box=0.95)
    # half of them aimed at the tube's axis so most hit the skinned surface
    k = n // 2
    tgt = np.stack([rng.uniform(-0.3, 0.3, k), rng.uniform(-0.8, 0.6, k), rng.uniform(-0.3, 0.3, k)], 1)
    o = np.stack([rng.uniform(-0.95, 0.95, k), rng.uniform(-0.9, 0.9, k), np.full(k, 0.95)], 1)
    d = tgt - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays["org"][:k] = o
    rays["dir"][:k] = d
    return rays


def test_skinned_tube_hits_bit_exact(gpu_ctx):
    import pyoracle as O
    from rustracer_gb300 import gbrt
    sd = zoo.skinned_tube()
    rays = _tube_rays(sd)
    sc = gbrt.Scene(gpu_ctx, sd)
    orc = O.OracleScene(sd)
    tube = sd.num_triangles - 34
    for time in (0.7, 1.9):
        skins = zoo.bone_matrices(sd.bones, time)
        sc.skin_and_refit(skins)
        orc.skin(skins)
        g, _ = sc.trace(rays)
        o, _ = orc.trace(rays)
        for f in ("instance_id", "primitive_id"):
            assert np.array_equal(g[f], o[f]), (time, f)
        assert np.array_equal(g["t"].view(np.uint32), o["t"].view(np.uint32)), time
        on_tube = g["instance_id"] == len(sd.prims) - 1
        assert on_tube.mean() > 0.25, "too few rays hit the tube"
    assert tube == 32 * 24 * 2


def test_skinned_tube_render(gpu_ctx):
    import pyoracle as O
    from rustracer_gb300 import gbrt
    sd = zoo.skinned_tube()
    skins = zoo.bone_matrices(sd.bones, 1.3)
    ubo = sd.ubo(64, 64, samples=4, bounces=6, exposure=1.0)
    orc = O.OracleScene(sd, diag=True)
    orc.skin(skins)
    ref = orc.render(ubo, 64, 64, want_samples=True, want_hits=True, want_margins=True)
    sc = gbrt.Scene(gpu_ctx, sd)
    sc.skin_and_refit(skins)
    r = sc.render(ubo, gbrt.Accum(gpu_ctx, 64, 64), want_samples=True, want_hits=True, mode=2)
    assert np.array_equal(r["hits"]["primitive_id"], ref["hits"]["primitive_id"])
    parity.assert_samples(r["samples"], ref, orc, ubo, 64, 64)


def test_refit_drift_triggers_rebuild(gpu_ctx):
    """A mild bend refits the wide BVH in place (SAH cost proxy within 1.3x of
    the built tree's); scattering the bones across the box makes the proxy
    grow past that, so the refit becomes a full rebuild.  Hits match the
    oracle's after both."""
    import pyoracle as O
    from rustracer_gb300 import gbrt
    sd = zoo.skinned_tube()
    rays = _tube_rays(sd)
    sc = gbrt.Scene(gpu_ctx, sd)
    orc = O.OracleScene(sd)
    info0 = sc.info()
    assert info0["sah_built"] > 1.0 and info0["refits"] == 0 and info0["wide_nodes"] > 0
    mild = zoo.bone_matrices(sd.bones, 0.7)
    sc.skin_and_refit(mild)
    info1 = sc.info()
    assert info1["refits"] == 1 and info1["drift_rebuilds"] == 0
    assert info1["sah_now"] < 1.3 * info1["sah_built"]
    scatter = zoo.bone_matrices(sd.bones, 0.7)
    for k in range(sd.bones):
        M = scatter[0]["joints"][k].reshape(4, 4).T.copy()  # column-major storage
        M[0, 3] += 0.85 * (1 if k % 2 == 0 else -1)
        M[2, 3] += 0.85 * (1 if (k // 2) % 2 == 0 else -1)
        scatter[0]["joints"][k] = M.T.reshape(16)
    sc.skin_and_refit(scatter)
    info2 = sc.info()
    assert info2["drift_rebuilds"] == 1 and info2["refits"] == 0
    orc.skin(scatter)
    g, _ = sc.trace(rays)
    o, _ = orc.trace(rays)
    for f in ("instance_id", "primitive_id"):
        assert np.array_equal(g[f], o[f]), f
    assert np.array_equal(g["t"].view(np.uint32), o["t"].view(np.uint32))
