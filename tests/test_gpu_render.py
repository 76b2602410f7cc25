"""GPU path tracing vs the CPU oracle through gbrt_render_ex.

Contract (per sample; D1 seeding makes every sample depend only on its pixel
and global sample index), asserted by tests/parity.py:
* primary-ray hits are bit-identical;
* per-sample radiance agrees within 1e-4 relative (|a-b| <= 1e-4 *
  max(|a|, |b|) + 1e-6), except samples the oracle shows to be
  ill-conditioned at the ulp level (a branch decision within 2^-14 of its
  threshold, a secondary hit within 2^-14 of a triangle edge, or a sample
  that leaves the band itself when the oracle's transcendentals and dot
  products move by 1-3 ulps); no other mismatch is allowed, and at most
  0.2% of the samples may mismatch at all.
"""
import os

import numpy as np
import pytest

import parity
from rustracer_gb300 import scenes, types as T

pytestmark = pytest.mark.gpu

FLIP_MAX = parity.FLIP_MAX

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def oracle_ref(sd, ubo, w, h, rows=None):
    """The oracle (diagnostics build) with samples, hits and margins."""
    import pyoracle as O
    orc = O.OracleScene(sd, diag=True)
    return orc, orc.render(ubo, w, h, rows=rows, want_samples=True, want_hits=True, want_margins=True)


def render_gpu(ctx, sd, ubo, w, h, mode=0, **kw):
    from rustracer_gb300 import gbrt
    sc = gbrt.Scene(ctx, sd)
    acc = gbrt.Accum(ctx, w, h)
    return sc.render(ubo, acc, want_samples=True, want_hits=True, mode=mode, **kw)


def test_golden_cornell_32(gpu_ctx):
    g = np.load(os.path.join(GOLDEN, "golden_cornell_32.npz"))
    ubo = np.frombuffer(g["ubo"].tobytes(), T.UBO)[0]
    sd = scenes.cornell()
    orc, ref = oracle_ref(sd, ubo, 32, 32)
    assert np.array_equal(ref["samples"].view(np.uint32), g["samples"].view(np.uint32))  # the fixture is the oracle's
    r = render_gpu(gpu_ctx, sd, ubo, 32, 32)
    h, gh = r["hits"].reshape(-1), g["hits"].reshape(-1)
    assert np.array_equal(h["primitive_id"], gh["primitive_id"])
    assert np.array_equal(h["t"].view(np.uint32), gh["t"].view(np.uint32))
    parity.assert_samples(r["samples"], ref, orc, ubo, 32, 32)


def test_golden_ico2(gpu_ctx):
    g = np.load(os.path.join(GOLDEN, "golden_ico2.npz"))
    ubo = np.frombuffer(g["ubo"].tobytes(), T.UBO)[0]
    sd = scenes.icosphere_scene(subdiv=2)
    orc, ref = oracle_ref(sd, ubo, 24, 16)
    assert np.array_equal(ref["samples"].view(np.uint32), g["samples"].view(np.uint32))
    r = render_gpu(gpu_ctx, sd, ubo, 24, 16)
    assert np.array_equal(r["hits"]["primitive_id"], g["hits"]["primitive_id"])
    parity.assert_samples(r["samples"], ref, orc, ubo, 24, 16)


@pytest.mark.parametrize("mode", [1, 2], ids=["megakernel", "wavefront"])
def test_cornell_256_16spp(gpu_ctx, mode):
    """Config 1: 256x256, 16 spp, depth 8, pinhole fov 40, AA on."""
    sd = scenes.cornell()
    ubo = sd.ubo(256, 256, samples=16, bounces=8, exposure=1.0)
    orc, ref = oracle_ref(sd, ubo, 256, 256)
    r = render_gpu(gpu_ctx, sd, ubo, 256, 256, mode=mode)
    gh, rh = r["hits"].reshape(-1), ref["hits"].reshape(-1)
    for f in ("instance_id", "primitive_id"):
        assert np.array_equal(gh[f], rh[f]), f
    assert np.array_equal(gh["t"].view(np.uint32), rh["t"].view(np.uint32))
    parity.assert_samples(r["samples"], ref, orc, ubo, 256, 256)
    # ray counts agree up to flipped paths
    st, rs = r["stats"], ref["stats"]
    assert st["rays_camera"] == rs["rays_camera"] == 256 * 256 * 16
    assert abs(int(st["rays_extension"]) - int(rs["rays_extension"])) <= 0.002 * rs["rays_extension"]
    # tone-mapped image within one code value on almost every pixel
    diff = np.abs(r["image"].astype(int) - ref["image"].astype(int))
    assert (diff <= 1).mean() > 0.99


@pytest.mark.parametrize("mode", [1, 2], ids=["megakernel", "wavefront"])
def test_icosphere_nee(gpu_ctx, mode):
    """Point lights exercise NEE (sampleLightRIS + shadow rays) and the
    metallic-roughness BRDF."""
    sd = scenes.icosphere_scene(subdiv=4)
    ubo = sd.ubo(96, 64, samples=4, bounces=8, exposure=1.0)
    orc, ref = oracle_ref(sd, ubo, 96, 64)
    r = render_gpu(gpu_ctx, sd, ubo, 96, 64, mode=mode)
    assert np.array_equal(r["hits"]["primitive_id"], ref["hits"]["primitive_id"])
    assert ref["stats"]["rays_shadow"] > 0
    assert abs(int(r["stats"]["rays_shadow"]) - int(ref["stats"]["rays_shadow"])) <= 0.002 * ref["stats"]["rays_shadow"]
    parity.assert_samples(r["samples"], ref, orc, ubo, 96, 64)


@pytest.mark.parametrize("band", [(508, 572), (120, 152)], ids=["middle", "upper"])
def test_headline_frame_band(gpu_ctx, band):
    """The bench's own workload: the icosphere of subdivision 7 (327,714
    triangles, 24 random metallic-roughness materials, 4 point lights) at
    1920x1080, depth 8, with the bench's tuning (8-wide BVH, ray-sort key).
    The GPU renders the full frame at 2 spp; a band of full-width rows is
    compared with the oracle: primary hits bit-exact, per-sample radiance
    within the contract."""
    from rustracer_gb300 import gbrt
    sd = scenes.icosphere_scene(subdiv=7)
    W, H = 1920, 1080
    ubo = sd.ubo(W, H, samples=2, bounces=8, exposure=1.0)
    orc, ref = oracle_ref(sd, ubo, W, H, rows=band)
    sc = gbrt.Scene(gpu_ctx, sd)
    sc.set_tuning(width=8, sort_rays=True)
    r = sc.render(ubo, gbrt.Accum(gpu_ctx, W, H), want_samples=True, want_hits=True, mode=gbrt.MODE_WAVEFRONT)
    r0, r1 = band
    gh = r["hits"].reshape(H, W, 2)[r0:r1]
    rh = ref["hits"].reshape(H, W, 2)[r0:r1]
    for f in ("instance_id", "primitive_id"):
        assert np.array_equal(gh[f], rh[f]), f
    assert np.array_equal(gh["t"].view(np.uint32), rh["t"].view(np.uint32))
    assert (rh["primitive_id"] != 0xFFFFFFFF).mean() > 0.4
    c = parity.assert_samples(r["samples"].reshape(H, W, 2, 3)[r0:r1], ref, orc, ubo, W, H, rows=band)
    assert c["n"] == (r1 - r0) * W * 2


def test_unused_material_features_keep_the_bits(gpu_ctx):
    """A material that no geometry uses but that has a texture, the
    specular-glossiness workflow and a volume moves the frame from the
    specialised shade kernel to the one with every feature compiled in; the
    samples, hits and image stay bit-identical."""
    import copy
    from rustracer_gb300 import gbrt
    sd = scenes.icosphere_scene(subdiv=3)
    ubo = sd.ubo(64, 48, samples=4, bounces=8, exposure=1.0)
    plain = render_gpu(gpu_ctx, sd, ubo, 64, 48, mode=gbrt.MODE_WAVEFRONT)
    full = copy.deepcopy(sd)
    extra = full.materials[:1].copy()
    extra["workflow"] = 1
    extra["volume_exists"] = 1
    extra["base_color_texture"]["index"] = 0
    full.materials = np.concatenate([full.materials, extra])
    r = render_gpu(gpu_ctx, full, ubo, 64, 48, mode=gbrt.MODE_WAVEFRONT)
    assert np.array_equal(r["samples"].view(np.uint32), plain["samples"].view(np.uint32))
    assert np.array_equal(r["hits"], plain["hits"]) and np.array_equal(r["image"], plain["image"])


def test_accumulation_across_frames(gpu_ctx):
    """Two frames of 2 spp accumulate like one frame of 4 spp (rgen:132-135)."""
    from rustracer_gb300 import gbrt
    sd = scenes.cornell()
    sc = gbrt.Scene(gpu_ctx, sd)
    a1, a2 = gbrt.Accum(gpu_ctx, 64, 64), gbrt.Accum(gpu_ctx, 64, 64)
    sc.render(sd.ubo(64, 64, samples=2, total=2, bounces=8, exposure=1.0), a1)
    sc.render(sd.ubo(64, 64, samples=2, total=4, bounces=8, exposure=1.0), a1)
    sc.render(sd.ubo(64, 64, samples=4, total=4, bounces=8, exposure=1.0), a2)
    x, y = a1.download(), a2.download()
    assert np.allclose(x, y, rtol=1e-5, atol=1e-6)


def test_sky_and_dir_light(gpu_ctx):
    """Miss shader: directional light term on secondary misses and the
    skybox (RayTracing.rmiss:18-37)."""
    sd = scenes.cornell()
    rng = np.random.default_rng(3)
    sd.skybox = (8, rng.integers(0, 256, 6 * 8 * 8 * 4).astype(np.uint8))
    d = T.default_dir_light()
    d["transform"] = (0.3, -1.0, -0.5, 0.0)
    d["intensity"] = 2.0
    sd.dlights = np.array([d], T.LIGHT)
    ubo = sd.ubo(64, 64, samples=4, bounces=6, exposure=1.0, has_sky=True, eye=(0.3, 0.2, 3.8),
                 direction=(0.3, 0.1, -1.0))
    orc, ref = oracle_ref(sd, ubo, 64, 64)
    r = render_gpu(gpu_ctx, sd, ubo, 64, 64)
    parity.assert_samples(r["samples"], ref, orc, ubo, 64, 64)


def test_wavefront_matches_megakernel(gpu_ctx):
    """Both kernel forms run the same per-path code; per-sample radiance
    agrees within the per-sample tolerance and primary hits are identical."""
    sd = scenes.icosphere_scene(subdiv=5)
    ubo = sd.ubo(160, 90, samples=8, bounces=8, exposure=1.0)
    a = render_gpu(gpu_ctx, sd, ubo, 160, 90, mode=1)
    b = render_gpu(gpu_ctx, sd, ubo, 160, 90, mode=2)
    assert np.array_equal(a["hits"], b["hits"])
    assert parity.mismatched(b["samples"], a["samples"]).mean() <= FLIP_MAX
    for f in ("rays_camera", "rays_extension", "rays_shadow"):
        assert abs(int(a["stats"][f]) - int(b["stats"][f])) <= 0.002 * int(a["stats"][f]) + 2, f


def test_wavefront_pixel_chunks(gpu_ctx):
    """A frame with more pixels than one wave holds (2^21 paths) is split
    into pixel ranges; it must match the megakernel."""
    from rustracer_gb300 import gbrt
    sd = scenes.cornell()
    W, H = 2048, 1056  # 2,162,688 pixels > 2^21
    ubo = sd.ubo(W, H, samples=1, bounces=4, exposure=1.0)
    sc = gbrt.Scene(gpu_ctx, sd)
    a1, a2 = gbrt.Accum(gpu_ctx, W, H), gbrt.Accum(gpu_ctx, W, H)
    ra = sc.render(ubo, a1, mode=1)
    rb = sc.render(ubo, a2, mode=2)
    x, y = a1.download(), a2.download()
    ok = np.all(np.abs(x - y) <= 1e-4 * np.maximum(np.abs(x), np.abs(y)) + 1e-6, axis=-1)
    assert ok.mean() > 1 - FLIP_MAX
    assert int(ra["stats"]["rays_camera"]) == int(rb["stats"]["rays_camera"]) == W * H


def test_async_frames_equal_sync(gpu_ctx):
    """Four frames queued with GBRT_RENDER_ASYNC, then gbrt_sync: the same
    accumulation and last image as four synchronous frames."""
    from rustracer_gb300 import gbrt
    sd = scenes.icosphere_scene(subdiv=3)
    sc = gbrt.Scene(gpu_ctx, sd)
    W, H = 200, 120
    ubos = [sd.ubo(W, H, samples=2, total=2 * (f + 1), bounces=6, exposure=1.0) for f in range(4)]
    a_sync, a_async = gbrt.Accum(gpu_ctx, W, H), gbrt.Accum(gpu_ctx, W, H)
    for u in ubos:
        img_sync = sc.render(u, a_sync)["image"]
    out = np.zeros((H, W, 4), np.uint8)
    for u in ubos:
        r = sc.render(u, a_async, asynchronous=True, out=out)
        assert r["stats"]["kernel_launches"] > 0
    gpu_ctx.sync()
    assert np.array_equal(out, img_sync)
    assert np.array_equal(a_async.download(), a_sync.download())
    with pytest.raises(gbrt.GbrtError):  # no debug outputs on the asynchronous form
        sc.render(ubos[0], a_async, asynchronous=True, want_samples=True)


def test_hdr_float_skybox(gpu_ctx):
    """An RGBA32F (linear, HDR: texels up to 20) skybox through
    gbrt_skybox_set_ex: per-sample radiance matches the oracle's."""
    sd = scenes.icosphere_scene(subdiv=2)
    rng = np.random.default_rng(4)
    sd.skybox = (8, (rng.random(6 * 8 * 8 * 4) * 20.0).astype(np.float32))
    ubo = sd.ubo(64, 48, samples=4, bounces=6, exposure=1.0, has_sky=True, eye=(0.3, 0.2, 3.8),
                 direction=(0.3, 0.1, -1.0))
    orc, ref = oracle_ref(sd, ubo, 64, 48)
    r = render_gpu(gpu_ctx, sd, ubo, 64, 48)
    parity.assert_samples(r["samples"], ref, orc, ubo, 64, 48)


def test_converged_vs_fp64_reference(gpu_ctx):
    """Converged images: the GPU's FP32 render (16384 spp, samples 0..16383)
    and the oracle's FP64-intersection render of other samples
    (16384..32767) of the Cornell box agree to relMSE = mean((x - ref)^2 /
    (ref^2 + 1e-2)) below 1e-2, the contract's convergence measure (two
    independent estimates: about 3e-3 expected from their noise)."""
    import pyoracle as O
    from rustracer_gb300 import gbrt
    sd = scenes.cornell()
    W = H = 16
    sc = gbrt.Scene(gpu_ctx, sd)
    acc = gbrt.Accum(gpu_ctx, W, H)
    N = 16384
    sc.render(sd.ubo(W, H, samples=N, total=N, bounces=8, exposure=1.0), acc, image=False)
    x = acc.download()[..., :3] / float(N)
    ref_acc = np.zeros((H * W, 4), np.float32)
    O.OracleScene(sd).render(sd.ubo(W, H, samples=N, total=2 * N, bounces=8, exposure=1.0), W, H,
                             accum=ref_acc, fp64=True, out=False)
    ref = ref_acc.reshape(H, W, 4)[..., :3] / float(N)
    relmse = float(np.mean((x - ref) ** 2 / (ref ** 2 + 1e-2)))
    assert np.isfinite(relmse) and relmse < 1e-2, relmse
    assert ref.mean() > 0.05  # the box is lit


def _furnace(albedo):
    """A closed 2x2x2 box, every wall emitting (1, 1, 1) with the reference's
    'Lambertian' material of the given albedo, camera at the centre."""
    from rustracer_gb300.scenes import GeoBuilder, lambert, _Soup
    b = GeoBuilder()
    m = b.add_material(lambert((albedo, albedo, albedo), emissive=(1.0, 1.0, 1.0)))
    g = _Soup()
    g.quad((-1, -1, 1), (1, -1, 1), (1, -1, -1), (-1, -1, -1))   # floor, normal +y
    g.quad((-1, 1, -1), (1, 1, -1), (1, 1, 1), (-1, 1, 1))       # ceiling, -y
    g.quad((-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1))   # back, +z
    g.quad((1, -1, 1), (-1, -1, 1), (-1, 1, 1), (1, 1, 1))       # front, -z
    g.quad((-1, -1, 1), (-1, -1, -1), (-1, 1, -1), (-1, 1, 1))   # left, +x
    g.quad((1, -1, -1), (1, -1, 1), (1, 1, 1), (1, 1, -1))       # right, -x
    p, n, i = g.arrays()
    b.add_mesh(p, i, m, n)
    return b.finish(camera=dict(eye=(0.0, 0.0, 0.0), direction=(0.2, 0.1, -1.0), fov_deg=90.0),
                    name=f"furnace{albedo}")


def test_white_furnace(gpu_ctx):
    """Analytic furnace (a closed box of unit emitters): every sample carries
    the emission of its first hit at least once, so no radiance is below 1;
    with albedo 0 only the dielectric specular lobe (Fresnel at normal
    incidence 0.04) reflects, so the radiance stays below 1.1; with albedo
    0.5 it grows (1 < mean < 1 / (1 - 0.75), the largest per-bounce weight of
    the reference's lobes at roughness 1); the GPU meets the per-sample parity
    contract against the oracle in both."""
    for albedo, lo, hi in ((0.0, 1.0, 1.1), (0.5, 1.05, 4.0)):
        sd = _furnace(albedo)
        ubo = sd.ubo(32, 32, samples=4, bounces=8, exposure=1.0)
        orc, ref = oracle_ref(sd, ubo, 32, 32)
        r = render_gpu(gpu_ctx, sd, ubo, 32, 32)
        s = r["samples"]
        assert s.min() >= 1.0 and ref["samples"].min() >= 1.0
        assert lo <= float(s.mean()) < hi, (albedo, float(s.mean()))
        parity.assert_samples(s, ref, orc, ubo, 32, 32)


def test_checkpoint_resume(gpu_ctx, tmp_path):
    """Progressive rendering resumes from a saved running sum: frames 1-2,
    save (to a file), a fresh accumulation buffer restored from it, frame 3,
    equal three frames rendered without a break, bit for bit."""
    from rustracer_gb300 import gbrt
    sd = scenes.icosphere_scene(subdiv=2)
    sc = gbrt.Scene(gpu_ctx, sd)
    W, H = 96, 64
    ubos = [sd.ubo(W, H, samples=2, total=2 * (f + 1), bounces=6, exposure=1.0) for f in range(3)]
    a = gbrt.Accum(gpu_ctx, W, H)
    for u in ubos:
        img_ref = sc.render(u, a)["image"]
    b = gbrt.Accum(gpu_ctx, W, H)
    for u in ubos[:2]:
        sc.render(u, b)
    np.save(tmp_path / "ckpt.npy", b.download())  # with the sample count (4) kept by the caller
    c = gbrt.Accum(gpu_ctx, W, H)
    c.upload(np.load(tmp_path / "ckpt.npy"))
    img = sc.render(ubos[2], c)["image"]
    assert np.array_equal(c.download(), a.download())
    assert np.array_equal(img, img_ref)
