"""Job API (gbrt_job_submit / poll / wait): continuous batching of frames of
several scenes in shared waves.

The contract: a job's accumulation buffer and image are bit-identical to
the same frame rendered alone through gbrt_render_ex (wavefront mode),
whatever other jobs share its waves and however its pixels and samples are
split across waves.
"""
import numpy as np
import pytest

from rustracer_gb300 import scenes, zoo

pytestmark = pytest.mark.gpu


def _solo(ctx, sc, ubo, w, h):
    from rustracer_gb300 import gbrt
    acc = gbrt.Accum(ctx, w, h)
    r = sc.render(ubo, acc, mode=gbrt.MODE_WAVEFRONT)
    return r["image"], acc.download()


def test_single_job_matches_render(gpu_ctx):
    from rustracer_gb300 import gbrt
    sd = scenes.cornell()
    sc = gbrt.Scene(gpu_ctx, sd)
    ubo = sd.ubo(128, 96, samples=6, bounces=8, exposure=1.0)
    img, acc_ref = _solo(gpu_ctx, sc, ubo, 128, 96)
    acc = gbrt.Accum(gpu_ctx, 128, 96)
    job = gpu_ctx.submit(sc, ubo, acc)
    info = job.wait()
    assert info["state"] == gbrt.JOB_DONE and info["status"] == 0
    assert np.array_equal(job.image.reshape(img.shape), img)
    assert np.array_equal(acc.download(), acc_ref)
    st = info["stats"]
    assert st["rays_camera"] == 128 * 96 * 6 and st["rays_total"] > st["rays_camera"]
    assert info["latency_ms"] >= info["queue_ms"] >= 0.0
    # the handle is released once its result has been reported
    assert gpu_ctx.L.gbrt_job_poll(gpu_ctx.h, job.id, None) == gbrt.E_INVALID


def test_mixed_jobs_equal_solo_renders(gpu_ctx):
    """Twelve jobs on three scenes, sizes from 48x32 to 1280x720 and 1-16
    spp, submitted at once (many share waves; the large ones span several)."""
    from rustracer_gb300 import gbrt
    sds = [scenes.cornell(), scenes.icosphere_scene(subdiv=3), zoo.material_zoo(subdiv=2)]
    scs = [gbrt.Scene(gpu_ctx, sd) for sd in sds]
    rng = np.random.default_rng(11)
    sizes = [(48, 32), (64, 64), (200, 120), (1280, 720), (96, 64), (320, 240)]
    specs = []
    for i in range(12):
        k = i % 3
        w, h = sizes[rng.integers(len(sizes))]
        spp = int(rng.choice([1, 2, 4, 16]))
        ubo = sds[k].ubo(w, h, samples=spp, bounces=int(rng.integers(3, 9)), exposure=1.0, has_sky=(k == 2))
        specs.append((k, w, h, ubo))
    solo = [_solo(gpu_ctx, scs[k], ubo, w, h) for k, w, h, ubo in specs]
    accs = [gbrt.Accum(gpu_ctx, w, h) for _, w, h, _ in specs]
    jobs = [gpu_ctx.submit(scs[k], ubo, accs[i]) for i, (k, w, h, ubo) in enumerate(specs)]
    for i, j in enumerate(jobs):
        info = j.wait()
        assert info["status"] == 0, i
        img, acc = solo[i]
        assert np.array_equal(j.image.reshape(img.shape), img), i
        assert np.array_equal(accs[i].download(), acc), i


def test_policies_agree(gpu_ctx):
    """Submission-order and shortest-first filling give the same images."""
    from rustracer_gb300 import gbrt
    sd = scenes.icosphere_scene(subdiv=2)
    sc = gbrt.Scene(gpu_ctx, sd)
    ubos = [sd.ubo(160, 90, samples=s, bounces=6, exposure=1.0) for s in (8, 1, 3)]
    out = []
    for pol in (gbrt.POLICY_FIFO, gbrt.POLICY_SRPT):
        gpu_ctx.jobs_configure(policy=pol)
        accs = [gbrt.Accum(gpu_ctx, 160, 90) for _ in ubos]
        js = [gpu_ctx.submit(sc, u, a) for u, a in zip(ubos, accs)]
        out.append([(j.wait(), j.image.copy())[1] for j in js])
    for a, b in zip(*out):
        assert np.array_equal(a, b)


def test_skinned_job_equals_skin_then_render(gpu_ctx):
    from rustracer_gb300 import gbrt
    sd = zoo.skinned_tube()
    ubo = sd.ubo(96, 96, samples=2, bounces=6, exposure=1.0)
    sc = gbrt.Scene(gpu_ctx, sd)
    ref = []
    for t in (0.4, 1.6):
        sc.skin_and_refit(zoo.bone_matrices(sd.bones, t))
        ref.append(_solo(gpu_ctx, sc, ubo, 96, 96))
    accs = [gbrt.Accum(gpu_ctx, 96, 96) for _ in range(2)]
    jobs = [gpu_ctx.submit(sc, ubo, accs[i], skins=zoo.bone_matrices(sd.bones, t)) for i, t in enumerate((0.4, 1.6))]
    for i, j in enumerate(jobs):
        assert j.wait()["status"] == 0
        assert np.array_equal(j.image.reshape(ref[i][0].shape), ref[i][0]), i
        assert np.array_equal(accs[i].download(), ref[i][1]), i


def test_busy_while_jobs_outstanding(gpu_ctx):
    from rustracer_gb300 import gbrt
    sd = scenes.icosphere_scene(subdiv=4)
    sc = gbrt.Scene(gpu_ctx, sd)
    big = sd.ubo(1280, 720, samples=32, bounces=8, exposure=1.0)
    acc = gbrt.Accum(gpu_ctx, 1280, 720)
    job = gpu_ctx.submit(sc, big, acc, image=False)
    with pytest.raises(gbrt.GbrtError) as e:
        sc.render(sd.ubo(16, 16, samples=1), gbrt.Accum(gpu_ctx, 16, 16))
    assert e.value.code == gbrt.E_BUSY
    with pytest.raises(gbrt.GbrtError) as e:
        acc.reset()
    assert e.value.code == gbrt.E_BUSY
    assert job.poll() is None or job.info["state"] == gbrt.JOB_DONE
    assert job.wait()["status"] == 0
    sc.render(sd.ubo(16, 16, samples=1), gbrt.Accum(gpu_ctx, 16, 16))  # usable again


def test_cache_jobs_equal_render_nrc(gpu_ctx):
    """Jobs carrying a radiance cache, submitted among plain jobs: a cache
    job's accumulation and image are bit-identical to gbrt_render_nrc's on a
    cache in the same state (a second cache given the same parameters), its
    training steps run (the parameters move), and the plain jobs still equal
    their solo renders."""
    from rustracer_gb300 import gbrt
    sd = scenes.icosphere_scene(subdiv=4)
    sc = gbrt.Scene(gpu_ctx, sd)
    p = sd.vertices["pos"][:, :3]
    lo, hi = tuple(map(float, p.min(0) - 0.05)), tuple(map(float, p.max(0) + 0.05))
    ca = gbrt.Nrc(gpu_ctx, lo, hi, log2_table=16, learning_rate=1e-3)
    cb = gbrt.Nrc(gpu_ctx, lo, hi, log2_table=16, learning_rate=1e-3, seed=99)
    W, H = 160, 120
    warm = sd.ubo(W, H, samples=1, total=1, bounces=8, exposure=1.0)
    ca.render(sc, warm, gbrt.Accum(gpu_ctx, W, H), image=False, train_samples=4096, train_steps=4)
    mlp, grid = ca.params()
    cb.set_params(mlp, grid)
    u = sd.ubo(W, H, samples=2, total=3, bounces=8, exposure=1.0)
    acc_a = gbrt.Accum(gpu_ctx, W, H)
    ref = ca.render(sc, u, acc_a, image=True, min_roughness=0.0, train_samples=4096, train_steps=2)
    plain = [(sd.ubo(w, h, samples=s, bounces=6, exposure=1.0), w, h) for w, h, s in ((64, 48, 4), (320, 200, 2))]
    solo = [_solo(gpu_ctx, sc, ub, w, h) for ub, w, h in plain]
    acc_b = gbrt.Accum(gpu_ctx, W, H)
    accs = [gbrt.Accum(gpu_ctx, w, h) for _, w, h in plain]
    jobs = [gpu_ctx.submit(sc, plain[0][0], accs[0]),
            gpu_ctx.submit(sc, u, acc_b, cache=cb, min_roughness=0.0, train_samples=4096, train_steps=2),
            gpu_ctx.submit(sc, plain[1][0], accs[1])]
    infos = [j.wait() for j in jobs]
    assert all(i["status"] == 0 for i in infos)
    assert np.array_equal(acc_b.download(), acc_a.download())
    assert np.array_equal(jobs[1].image.reshape(ref["image"].shape), ref["image"])
    assert infos[1]["stats"]["rays_camera"] == W * H * 2
    for k, (img, acc_ref) in enumerate(solo):
        assert np.array_equal(jobs[2 * k].image.reshape(img.shape), img)
        assert np.array_equal(accs[k].download(), acc_ref)
    m2, _ = cb.params()
    assert not np.array_equal(m2, mlp)


def test_cache_calls_busy_while_jobs_outstanding(gpu_ctx):
    from rustracer_gb300 import gbrt
    sd = scenes.icosphere_scene(subdiv=4)
    sc = gbrt.Scene(gpu_ctx, sd)
    c = gbrt.Nrc(gpu_ctx, (-2.0, -2.0, -2.0), (2.0, 2.0, 2.0), log2_table=12)
    acc = gbrt.Accum(gpu_ctx, 1280, 720)
    job = gpu_ctx.submit(sc, sd.ubo(1280, 720, samples=32, bounces=8, exposure=1.0), acc, image=False)
    with pytest.raises(gbrt.GbrtError) as e:
        c.query(np.zeros((4, 3), np.float32))
    assert e.value.code == gbrt.E_BUSY
    assert job.wait()["status"] == 0
    assert c.query(np.zeros((4, 3), np.float32)).shape == (4, 3)


def test_large_waves_equal_solo_render():
    """GBRT_JOB_LARGE_WAVES (waves up to 2^26 paths on a deep queue): a
    frame of 83M paths as a job equals the solo render, beside a small job."""
    from rustracer_gb300 import build, gbrt
    build.build()
    ctx = gbrt.Context(0)
    try:
        ctx.jobs_configure(policy=gbrt.POLICY_SRPT | gbrt.JOB_LARGE_WAVES)
        sd = scenes.icosphere_scene(subdiv=3)
        sc = gbrt.Scene(ctx, sd)
        big = sd.ubo(1920, 1080, samples=40, bounces=4, exposure=1.0)
        small = sd.ubo(64, 64, samples=2, bounces=4, exposure=1.0)
        ref = [_solo(ctx, sc, u, w, h) for u, w, h in ((big, 1920, 1080), (small, 64, 64))]
        accs = [gbrt.Accum(ctx, 1920, 1080), gbrt.Accum(ctx, 64, 64)]
        js = [ctx.submit(sc, big, accs[0]), ctx.submit(sc, small, accs[1])]
        for j, a, (img, acc_ref) in zip(js, accs, ref):
            assert j.wait()["status"] == 0
            assert np.array_equal(j.image.reshape(img.shape), img)
            assert np.array_equal(a.download(), acc_ref)
    finally:
        ctx.close()


def test_job_cancel_queued_and_running():
    """gbrt_job_cancel on a queued job (an HBM budget of one byte admits one
    job at a time) ends it at once; on a running job whose segments are not
    yet on the stream it ends after the waves in flight.  Both report
    GBRT_E_CANCELLED, and the job left alone still equals its solo render."""
    from rustracer_gb300 import build, gbrt
    build.build()
    ctx = gbrt.Context(0)
    try:
        sd = scenes.icosphere_scene(subdiv=3)
        sc = gbrt.Scene(ctx, sd)
        big = sd.ubo(1280, 720, samples=16, bounces=6, exposure=1.0)
        img_ref, acc_ref = _solo(ctx, sc, big, 1280, 720)
        # queued: one job admitted at a time
        ctx.jobs_configure(hbm_budget=1, policy=gbrt.POLICY_FIFO)
        acc_a, acc_b = gbrt.Accum(ctx, 1280, 720), gbrt.Accum(ctx, 64, 64)
        ja = ctx.submit(sc, big, acc_a)
        jb = ctx.submit(sc, sd.ubo(64, 64, samples=1, bounces=6, exposure=1.0), acc_b)
        jb.cancel()
        with pytest.raises(gbrt.GbrtError) as e:
            jb.wait()
        assert e.value.code == gbrt.E_CANCELLED
        assert ja.wait()["status"] == 0
        assert np.array_equal(ja.image.reshape(img_ref.shape), img_ref)
        assert np.array_equal(acc_a.download(), acc_ref)
        # running: first in submission order is the large job, so the second one's segments wait
        ctx.jobs_configure(hbm_budget=1 << 34, policy=gbrt.POLICY_FIFO)
        acc_c, acc_d = gbrt.Accum(ctx, 1280, 720), gbrt.Accum(ctx, 1280, 720)
        jc = ctx.submit(sc, big, acc_c)
        jd = ctx.submit(sc, big, acc_d)
        jd.cancel()
        with pytest.raises(gbrt.GbrtError) as e:
            jd.wait()
        assert e.value.code == gbrt.E_CANCELLED
        assert jc.wait()["status"] == 0
        assert np.array_equal(acc_c.download(), acc_ref)
        with pytest.raises(gbrt.GbrtError):  # finished: nothing left to cancel
            jc.cancel()
    finally:
        ctx.close()


def test_injected_admission_failure():
    """Host-side fault injection: the first admission fails as if out of
    memory (GBRT_E_OOM); the other jobs of the batch still finish and equal
    their solo renders."""
    from rustracer_gb300 import build, gbrt
    build.build()
    ctx = gbrt.Context(0)
    try:
        sd = scenes.icosphere_scene(subdiv=2)
        sc = gbrt.Scene(ctx, sd)
        ubos = [sd.ubo(96, 64, samples=s, bounces=6, exposure=1.0) for s in (2, 3, 1)]
        solo = [_solo(ctx, sc, u, 96, 64) for u in ubos]
        ctx.jobs_inject(gbrt.INJECT_ADMIT_OOM, 1)
        accs = [gbrt.Accum(ctx, 96, 64) for _ in ubos]
        js = [ctx.submit(sc, u, a) for u, a in zip(ubos, accs)]
        with pytest.raises(gbrt.GbrtError) as e:
            js[0].wait()
        assert e.value.code == gbrt.E_OOM
        for j, a, (img, acc_ref) in list(zip(js, accs, solo))[1:]:
            assert j.wait()["status"] == 0
            assert np.array_equal(j.image.reshape(img.shape), img)
            assert np.array_equal(a.download(), acc_ref)
    finally:
        ctx.close()


@pytest.mark.parametrize("seed", [1, 4, 12])
def test_batched_scene_jobs_vs_oracle(gpu_ctx, seed):
    """Scenes of the batched configuration (seeded instanced tori: FP16 MASK
    alpha textures, transmissive materials with a volume and random IOR,
    three point lights), capped at 60k triangles so the oracle builds them
    quickly: submitted as jobs beside another job, each job's accumulation
    and image equal the solo render's bit for bit, and the solo render meets
    the per-sample parity contract against the oracle (primary hits
    bit-exact)."""
    import parity
    import pyoracle as O
    from rustracer_gb300 import gbrt, types as T, workloads
    sd, _, _, _ = workloads.batched_scene(seed, max_tri=60_000, min_tri=1_000)
    assert (sd.materials["alpha_mode"] == T.ALPHA_MASK).any() and (sd.materials["transmission_exist"] == 1).any()
    W, H = 96, 64
    ubo = sd.ubo(W, H, samples=4, bounces=8, exposure=1.0)
    sc = gbrt.Scene(gpu_ctx, sd)
    acc_solo = gbrt.Accum(gpu_ctx, W, H)
    solo = sc.render(ubo, acc_solo, want_samples=True, want_hits=True, mode=gbrt.MODE_WAVEFRONT)
    orc = O.OracleScene(sd, diag=True)
    ref = orc.render(ubo, W, H, want_samples=True, want_hits=True, want_margins=True)
    for f in ("instance_id", "primitive_id"):
        assert np.array_equal(solo["hits"][f], ref["hits"][f]), f
    assert np.array_equal(solo["hits"]["t"].view(np.uint32), ref["hits"]["t"].view(np.uint32))
    parity.assert_samples(solo["samples"], ref, orc, ubo, W, H)
    other = scenes.icosphere_scene(subdiv=3)
    sc2 = gbrt.Scene(gpu_ctx, other)
    acc, acc2 = gbrt.Accum(gpu_ctx, W, H), gbrt.Accum(gpu_ctx, 200, 120)
    j2 = gpu_ctx.submit(sc2, other.ubo(200, 120, samples=3, bounces=6, exposure=1.0), acc2)
    j = gpu_ctx.submit(sc, ubo, acc)
    assert j.wait()["status"] == 0 and j2.wait()["status"] == 0
    assert np.array_equal(acc.download(), acc_solo.download())
    assert np.array_equal(j.image.reshape(H, W, 4), solo["image"])


def test_serving_skinned_job_vs_oracle(gpu_ctx):
    """The serving pool's skinned scene (a tube on a 64-bone chain in the
    Cornell box): a job carrying its joint matrices skins, refits and renders;
    its result equals skin-then-render, whose samples meet the contract
    against the oracle skinned with the same matrices."""
    import parity
    import pyoracle as O
    from rustracer_gb300 import gbrt, workloads
    sd = workloads.skinned_scene(rings=40, segments=24)
    skins = zoo.bone_matrices(sd.bones, 1.1)
    W, H = 80, 64
    ubo = sd.ubo(W, H, samples=4, bounces=6, exposure=1.0)
    sc = gbrt.Scene(gpu_ctx, sd)
    acc = gbrt.Accum(gpu_ctx, W, H)
    j = gpu_ctx.submit(sc, ubo, acc, skins=skins)
    assert j.wait()["status"] == 0
    sc.skin_and_refit(skins)
    acc_solo = gbrt.Accum(gpu_ctx, W, H)
    solo = sc.render(ubo, acc_solo, want_samples=True, want_hits=True, mode=gbrt.MODE_WAVEFRONT)
    assert np.array_equal(acc.download(), acc_solo.download())
    orc = O.OracleScene(sd, diag=True)
    orc.skin(skins)
    ref = orc.render(ubo, W, H, want_samples=True, want_hits=True, want_margins=True)
    assert np.array_equal(solo["hits"]["primitive_id"], ref["hits"]["primitive_id"])
    parity.assert_samples(solo["samples"], ref, orc, ubo, W, H)
