"""Benchmark: Mrays/s of the GB300 path tracer on the icosphere workload.

Workload (one step = one frame): Cornell box + seeded noise-displaced
icosphere, subdivision 7 (327,680 + 34 triangles), 24 random metallic-
roughness materials, 4 point lights, 1920x1080, 64 samples per pixel, 8
bounces, Russian roulette after bounce 3.  Each step renders the next 64
samples into the resident accumulation buffer (progressive accumulation like
the reference's frame loop), so no step repeats another's work.

Rays counted: camera, extension and shadow segments (every traced segment
once).  `value` is device throughput with the scene resident in HBM, timed
with CUDA events on the library's stream; L2 (the scene is ~60 MB, below the
129 MB L2) is flushed between steps by writing a 256 MiB buffer.  `e2e` is
the same metric through the public C-ABI call gbrt_render with a host UBO in
and the tone-mapped RGBA8 image copied back to host memory every step.

--impl reference times the CPU oracle (the C++ restatement of the reference
shaders, all host threads) on a bounded sample of the same workload.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

W, H, SPP, DEPTH, SUBDIV = 1920, 1080, 64, 8, 7
WORKLOAD = f"icosphere{SUBDIV}_cornell_{W}x{H}_{SPP}spp_depth{DEPTH}"
MODES = {"auto": 0, "megakernel": 1, "wavefront": 2}
B_SHADE = 608  # algorithmic bytes per shaded hit (index, PrimInfo, 3 vertex subsets, material, new ray, path state)


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def measured_bf16_tflops():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        return float(json.load(open(p))["bf16_tflops"]), "measured"
    return 1900.0, "fallback"


NRC_MLP_FLOPS = 2 * (32 * 64 + 4 * 64 * 64 + 64 * 3)  # per query: 32 -> 64 x5 -> 3, no bias


def nrc_mlp_rate(ctx, lo, hi, n=1 << 24, reps=10):
    """Device time of cache queries (hash-grid encoding + MLP) over n seeded
    positions in the box, for the tcgen05 and the mma.sync kernel, as MLP
    TFLOP/s against the bf16 peak.  n float4 in and out = 512 MiB, above L2."""
    import torch
    from rustracer_gb300 import gbrt
    g = torch.Generator(device="cuda").manual_seed(7)
    pos = torch.zeros(n, 4, device="cuda")
    lo_t, hi_t = torch.tensor(lo, device="cuda"), torch.tensor(hi, device="cuda")
    pos[:, :3] = lo_t + torch.rand(n, 3, device="cuda", generator=g) * (hi_t - lo_t)
    out = torch.empty_like(pos)
    torch.cuda.synchronize()
    peak, how = measured_bf16_tflops()
    res = {"queries": n, "flop_per_query": NRC_MLP_FLOPS, "peak_tflops": peak, "peak_kind": how,
           "note": "a query is 128 gathers from the FP16 hash table (16 levels x 8 corners) before 18,624 MACs; "
                   "the table gathers bound it, not the tensor pipe"}
    for name, flags in (("tcgen05", 0), ("mma_sync", gbrt.NRC_QUERY_MMA_SYNC)):
        c = gbrt.Nrc(ctx, lo, hi, log2_table=19, flags=flags)
        for _ in range(3):
            c.query_device(pos.data_ptr(), n, out.data_ptr())
        ms = sorted(c.query_device(pos.data_ptr(), n, out.data_ptr()) for _ in range(reps))[reps // 2]
        tf = n * NRC_MLP_FLOPS / (ms * 1e-3) / 1e12
        res[name] = {"device_ms": round(ms, 3), "mlp_tflops": round(tf, 2), "frac": round(tf / peak, 4),
                     "mqueries_per_s": round(n / ms / 1e3, 1)}
        c.close()
    return res


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while
    the timed region runs."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        self.f.flush()
        rows = []
        for line in open(self.f.name):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9 and parts[1].replace(".", "").isdigit():
                rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in rows]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": float(rows[0][2]), "reasons": reasons,
                "samples": len(rows), "power_w_max": max(float(r[3]) for r in rows if r[3][0].isdigit())}


def make_scene():
    from rustracer_gb300 import scenes
    return scenes.icosphere_scene(subdiv=SUBDIV)


def cpu_sample(sd, threads=0, target_s=12.0, rows=None):
    """Times the CPU oracle on a bounded sample of the workload: the full
    1920x1080 frame at 1 spp first (also the ray set for the N_node/N_tri
    statistics), repeated with more samples if that was much shorter than
    target_s.  Returns (result dict, stats)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O
    o = O.OracleScene(sd)
    r0, r1 = rows if rows else (0, H)
    spp = 1
    while True:
        ubo = sd.ubo(W, H, samples=spp, bounces=DEPTH, exposure=1.0)
        st = o.render(ubo, W, H, rows=(r0, r1), threads=threads, out=False)["stats"]
        if st["seconds"] >= target_s / 3 or spp >= SPP:
            break
        spp = min(SPP, max(spp * 2, int(spp * target_s / max(st["seconds"], 1e-3))))
    rays = int(st["rays_camera"] + st["rays_extension"] + st["rays_shadow"])
    return {"rays": rays, "seconds": float(st["seconds"]), "threads": int(st["threads"]), "spp": spp,
            "rows": (r0, r1), "node_visits": int(st["node_visits"]), "tri_tests": int(st["tri_tests"]),
            "hits_shaded": int(st["hits_shaded"]), "oracle": o}


def parity_band(sd, scene, o, rows=(508, 540), spp=2):
    """The benchmarked frame checked against the oracle (after the timed
    region): the GPU renders the 1080p frame at `spp` through the same
    entry point and tuning, the oracle the rows `rows`; primary hits must be
    bit-identical and per-sample radiance within 1e-4 relative (the tests'
    contract also explains the few ulp-sensitive samples)."""
    from rustracer_gb300 import gbrt
    ubo = sd.ubo(W, H, samples=spp, bounces=DEPTH, exposure=1.0)
    r = scene.render(ubo, gbrt.Accum(scene.ctx, W, H), image=False, want_samples=True, want_hits=True,
                     mode=MODES["wavefront"])
    ref = o.render(ubo, W, H, rows=rows, want_samples=True, want_hits=True, out=False)
    r0, r1 = rows
    gh, rh = r["hits"].reshape(H, W, spp)[r0:r1], ref["hits"].reshape(H, W, spp)[r0:r1]
    a = r["samples"].reshape(H, W, spp, 3)[r0:r1].reshape(-1, 3).astype(np.float64)
    b = ref["samples"].reshape(H, W, spp, 3)[r0:r1].reshape(-1, 3).astype(np.float64)
    bad = ~np.all(np.abs(a - b) <= 1e-4 * np.maximum(np.abs(a), np.abs(b)) + 1e-6, axis=1)
    exact = bool(np.array_equal(gh["primitive_id"], rh["primitive_id"]) and
                 np.array_equal(gh["instance_id"], rh["instance_id"]) and
                 np.array_equal(gh["t"].view(np.uint32), rh["t"].view(np.uint32)))
    return {"rows": list(rows), "spp": spp, "samples": int(len(a)), "primary_hits_bit_exact": exact,
            "samples_outside_1e-4": int(bad.sum()), "share_outside_1e-4": float(bad.mean())}


def b_ray(cs):
    """Algorithmic bytes per ray: 32 (ray) + 16 (hit) + N_node*64 + N_tri*36,
    N_node / N_tri the mean BVH2 inner-node visits and triangle tests per ray
    of the oracle's binned-SAH BVH2 on the same ray set."""
    n_node = cs["node_visits"] / cs["rays"]
    n_tri = cs["tri_tests"] / cs["rays"]
    return 48.0 + 64.0 * n_node + 36.0 * n_tri, n_node, n_tri


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def common_line(args, n, value, ms_per_step, extra_cfg=None):
    cfg = {"workload": WORKLOAD, "width": W, "height": H, "spp_per_step": SPP, "depth": DEPTH,
           "triangles": 20 * 4 ** SUBDIV + 34, "materials": 24 + 4, "point_lights": 4,
           "l2": "flushed between steps (256 MiB write)", "parallelism": f"replicas{n}" if n > 1 else "single"}
    if extra_cfg:
        cfg.update(extra_cfg)
    return {"metric": "Mrays/s", "value": value, "unit": "Mrays/s", "n_gpus": n, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded icosphere + Cornell box)",
            "config": cfg}


def traffic_from_profile(kernel, units_per_launch):
    """DRAM bytes (read + write) of one launch of `kernel`: the per-unit
    traffic of an ncu capture of that kernel on a small case of this workload
    (profiles/dram_traffic_icosphere7.json; units: rays for the traversal
    kernels, shaded hits for shade) times the units of a full launch, or None
    when that kernel has no capture."""
    p = os.path.join(ROOT, "profiles", "dram_traffic_icosphere7.json")
    if not os.path.exists(p):
        return None
    d = json.load(open(p)).get(kernel)
    if not d or not units_per_launch:
        return None
    return d["dram_bytes_per_unit"] * units_per_launch


def run_gpu(args):
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from rustracer_gb300 import build, gbrt
    build.build()
    sd = make_scene()
    ctx = gbrt.Context(local)
    scene = gbrt.Scene(ctx, sd)
    acc = gbrt.Accum(ctx, W, H)
    # traversal layout and ray-sort key: the autotuner's choice (untimed setup) or fixed
    if args.tune == "auto":
        tuning = scene.autotune(sd.ubo(W, H, samples=SPP, bounces=DEPTH, exposure=1.0), W, H)  # one step's frame
    else:
        tuning = {"chosen_width": int(args.tune[1]), "sort_rays": int(args.tune.endswith("s"))}
        scene.set_tuning(tuning["chosen_width"], bool(tuning["sort_rays"]))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    pinned = torch.empty((H, W, 4), dtype=torch.uint8, pin_memory=True)
    state = {"step": 0}

    def frame(out_ptr=None, timed=False):
        # this rank's samples of the next step (disjoint across ranks)
        from rustracer_gb300 import replicas
        _, last = replicas.sample_range(rank, world, state["step"], SPP)
        state["step"] += 1
        ubo = np.asarray(sd.ubo(W, H, samples=SPP, total=last, bounces=DEPTH, exposure=1.0)).reshape(())
        st = np.zeros((), gbrt.T.STATS)
        opts = gbrt.RenderOpts(MODES[args.mode], 1 if timed else 0, None, None)  # 1 = per-stage CUDA events
        ctx.check(ctx.L.gbrt_render_ex(scene.h, gbrt._p(ubo), acc.h, out_ptr, gbrt._p(st), C.byref(opts)))
        return st

    def flush_l2():
        flush.zero_()
        torch.cuda.synchronize()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        flush_l2()
        frame()
    barrier()
    rays = shaded = shaded_t = 0
    dev_ms = 0.0
    stage_ms, stage_rays, visits = [0.0] * 4, [0, 0, 0], [0, 0]
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            flush_l2()
            st = frame()
            rays += int(st["rays_total"])
            launches = int(st["kernel_launches"])
            dev_ms += float(st["device_ms"])
            shaded_t += int(st["hits_shaded"])
            visits[0] += int(st["node_visits"])
            visits[1] += int(st["tri_tests"])
        barrier()
        wall = time.perf_counter() - t0
    clocks = clk.summary()
    # per-stage CUDA events on separate frames: the stages then run one after
    # another (in the timed frames the shadow stage overlaps the next extension)
    stage_frames = max(1, min(args.steps, 2))
    for _ in range(stage_frames):
        flush_l2()
        st = frame(timed=True)
        shaded += int(st["hits_shaded"])
        for k in range(4):
            stage_ms[k] += float(st["stage_ms"][k])
        stage_rays[0] += int(st["rays_camera"] + st["rays_extension"])
        stage_rays[2] += int(st["rays_shadow"])
    # end to end through the C ABI: UBO in, RGBA8 image out to pinned host memory
    e2e_rays, e2e_s = 0, 0.0
    for _ in range(args.steps):
        flush_l2()
        t = time.perf_counter()
        st = frame(pinned.data_ptr())
        e2e_s += time.perf_counter() - t
        e2e_rays += int(st["rays_total"])

    from rustracer_gb300 import replicas
    (dev_ms, wall, e2e_s), (tot_rays, tot_e2e) = replicas.combine([dev_ms, wall, e2e_s], [rays, e2e_rays],
                                                                  device=f"cuda:{local}")
    if rank != 0:
        return
    cs = cpu_sample(sd, target_s=args.cpu_seconds) if world == 1 else cpu_sample(sd, target_s=0.0)
    parity = parity_band(sd, scene, cs["oracle"]) if (world == 1 and (W, H) == (1920, 1080)) else None
    bray, n_node, n_tri = b_ray(cs)
    value = tot_rays / (dev_ms / 1e3) / 1e6
    peak, peak_kind = measured_peaks()
    if sum(stage_ms) > 0:  # wavefront: the dominant stage kernel, bytes from its own units
        names = ["wf_extend", "wf_shade", "wf_shadow"]
        stage_bytes = [stage_rays[0] * bray, shaded * B_SHADE, stage_rays[2] * bray]
        stages = {names[k]: {"ms_per_step": stage_ms[k] / stage_frames,
                             "achieved_gbs": stage_bytes[k] / (stage_ms[k] / 1e3) / 1e9 if stage_ms[k] else None,
                             "share": stage_ms[k] / sum(stage_ms)} for k in range(3)}
        stages["other"] = {"ms_per_step": stage_ms[3] / stage_frames, "share": stage_ms[3] / sum(stage_ms)}
        stages["note"] = (f"stage times from {stage_frames} extra frame(s) with per-launch CUDA events, stages "
                          "serialised; the timed frames overlap the shadow stage with the next extension")
        dom = max(range(3), key=lambda k: stage_ms[k])
        kernel_name = names[dom]
        achieved = stage_bytes[dom] / (stage_ms[dom] / 1e3) / 1e9
    else:
        stages = None
        kernel_name = "pt_megakernel"
        achieved = (rays * bray + shaded_t * B_SHADE) / (dev_ms / 1e3) / 1e9
    max_wave = 1 << 26  # paths per single-frame wave (the library's kMaxWavePaths)
    waves = -(-(W * H * SPP) // min(W * H * SPP, max_wave))
    stage_launches = waves * DEPTH * stage_frames
    # units of one launch of the dominant kernel: rays (extend, shadow) or shaded hits (shade)
    units = {"wf_extend": stage_rays[0], "wf_shade": shaded, "wf_shadow": stage_rays[2]}.get(kernel_name, 0)
    traffic = traffic_from_profile(kernel_name, units / max(stage_launches, 1))
    line = common_line(args, world, value, dev_ms / args.steps,
                       {"kernel": args.mode, "wall_ms_per_step": wall / args.steps * 1e3,
                        "launches_per_step": launches,
                        "tuning": {k: (round(v, 3) if isinstance(v, float) else v) for k, v in tuning.items()}})
    line["roofline"] = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                        "traffic": traffic, "peak_source": peak_kind,
                        "bytes_per_ray": bray, "n_node": n_node, "n_tri": n_tri,
                        "bytes_per_shaded_hit": B_SHADE, "kernel": kernel_name,
                        "hbm_roofline_mrays": peak * 1e3 / bray,
                        "gpu_node_visits_per_ray": visits[0] / max(rays, 1),
                        "gpu_tri_tests_per_ray": visits[1] / max(rays, 1)}
    if stages:
        line["roofline"]["stages"] = stages
    line["e2e"] = {"value": tot_e2e / e2e_s / 1e6, "unit": "Mrays/s", "h2d_bytes_per_step": int(gbrt.T.UBO.itemsize),
                   "d2h_bytes_per_step": W * H * 4}
    if world == 1:
        line["cpu_baseline"] = {"value": cs["rays"] / cs["seconds"] / 1e6, "unit": "Mrays/s", "cores": cs["threads"],
                                "kind": "port",
                                "sample": f"{W}x{H} frame at {cs['spp']} spp ({cs['rays']} rays, "
                                          f"{cs['seconds']:.1f} s), same scene and depth"}
    if parity:
        line["parity"] = parity
    line["clocks"] = clocks
    line["gpu_launches"] = args.steps * launches
    print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def oracle_bytes_per_ray(sd, depth, w=96, h=54):
    """B_ray of one scene: 48 + 64 N_node + 36 N_tri from the oracle's BVH2
    on a small camera-driven sample (w x h at 1 spp, same depth)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O
    st = O.OracleScene(sd).render(sd.ubo(w, h, samples=1, bounces=depth, exposure=1.0), w, h, out=False)["stats"]
    rays = int(st["rays_camera"] + st["rays_extension"] + st["rays_shadow"])
    return 48.0 + (64.0 * int(st["node_visits"]) + 36.0 * int(st["tri_tests"])) / max(rays, 1)


def job_rays(info):
    st = info["stats"]
    return int(st["rays_total"]), int(st["hits_shaded"])


def run_batched(args):
    """32 seeded instanced scenes (alpha-tested, transmissive materials),
    each with its own resolution and spp, rendered as one batch of jobs that
    share waves (continuous batching); a step = the 32 frames.  Also times
    the same frames rendered one after another through gbrt_render_ex."""
    from rustracer_gb300 import build, gbrt, workloads as WL
    build.build()
    depth = DEPTH
    specs = [WL.batched_scene(i) for i in range(32)]
    if args.mix == "small":  # the same scenes as small frames: 256^2 / 512^2 at 1-4 spp (seeded)
        rng = np.random.default_rng(77)
        specs = [(sd, int(r), int(r), int(rng.choice([1, 2, 4])))
                 for (sd, _, _, _), r in zip(specs, rng.choice([256, 512], 32))]
    ctx = gbrt.Context(0)
    scs = [gbrt.Scene(ctx, sd) for sd, _, _, _ in specs]
    accs = [gbrt.Accum(ctx, w, h) for _, w, h, _ in specs]
    ubos = [sd.ubo(w, h, samples=spp, bounces=depth, exposure=1.0) for sd, w, h, spp in specs]
    pinned = [np.zeros((h, w, 4), np.uint8) for _, w, h, _ in specs]
    # autotuner (setup, untimed): per scene, a 640x360 2-spp probe of each BVH layout and the ray-sort key
    t_tune = time.perf_counter()
    tuned = [sc.autotune(sd.ubo(640, 360, samples=2, bounces=depth, exposure=1.0), 640, 360)
             for sc, (sd, _, _, _) in zip(scs, specs)]
    t_tune = time.perf_counter() - t_tune
    # throughput: waves up to 2^26 paths (large frames); small frames keep the default 2^24 cap
    ctx.jobs_configure(policy=gbrt.POLICY_SRPT | (gbrt.JOB_LARGE_WAVES if args.mix == "full" else 0))

    def batch():
        jobs = [ctx.submit(sc, u, a) for sc, u, a in zip(scs, ubos, accs)]
        infos = [j.wait() for j in jobs]
        for j in jobs:
            assert j.info["status"] == 0
        return infos

    def sequential():
        rays = 0
        for sc, u, a, img in zip(scs, ubos, accs, pinned):
            st = np.zeros((), gbrt.T.STATS)
            ctx.check(ctx.L.gbrt_render_ex(sc.h, gbrt._p(np.asarray(u).reshape(())), a.h, gbrt._p(img),
                                           gbrt._p(st), C.byref(gbrt.RenderOpts(MODES["wavefront"], 0, None, None))))
            rays += int(st["rays_total"])
        return rays

    for _ in range(args.warmup):
        batch()
    rays = shaded = 0
    per_scene = [0] * 32
    with ClockSampler(0) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            infos = batch()
            for i, inf in enumerate(infos):
                r, sh = job_rays(inf)
                rays += r
                shaded += sh
                per_scene[i] += r
        wall = time.perf_counter() - t0
    clocks = clk.summary()
    t1 = time.perf_counter()
    seq_rays = sum(sequential() for _ in range(args.steps))
    seq_wall = time.perf_counter() - t1
    brays = [oracle_bytes_per_ray(sd, depth) for sd, _, _, _ in specs]
    alg_bytes = sum(per_scene[i] * brays[i] for i in range(32)) + shaded * B_SHADE
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes / wall / 1e9
    value = rays / wall / 1e6
    px = sum(w * h * spp for _, w, h, spp in specs)
    line = {"metric": "Mrays/s", "value": value, "unit": "Mrays/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": wall / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (32 seeded scenes of instanced tori, 1k-2M triangles per mesh)",
            "config": {"workload": "batched32_instanced_alpha_transmissive" + ("_small_frames" if args.mix == "small"
                                                                                else ""), "scenes": 32,
                       "triangles_unique": int(sum(sd.num_triangles for sd, _, _, _ in specs)),
                       "instances": int(sum(len(sd.instances) for sd, _, _, _ in specs)),
                       "paths_per_step": int(px), "depth": depth,
                       "resolutions": "{256^2, 512^2}" if args.mix == "small" else "{256^2, 512^2, 1280x720, 1920x1080}",
                       "spp": "{1, 2, 4}" if args.mix == "small" else "{1, 4, 16, 64}",
                       "l2": "inputs (1.2 GB of vertices) larger than L2", "timing": "host wall clock, submit to last image on host",
                       "waves": "up to 2^26 paths (GBRT_JOB_LARGE_WAVES)" if args.mix == "full" else "up to 2^24 paths"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": None, "peak_source": peak_kind, "kernel": "whole batch (algorithmic bytes)",
                         "bytes_per_ray_by_scene": [round(b, 1) for b in brays]},
            "sequential": {"value": seq_rays / seq_wall / 1e6, "unit": "Mrays/s",
                           "ms_per_step": seq_wall / args.steps * 1e3,
                           "how": "the same 32 frames one after another through gbrt_render_ex"},
            "batched_over_sequential": (rays / wall) / (seq_rays / seq_wall),
            "autotune": {"seconds": round(t_tune, 3),
                         "chosen_width": {str(w): sum(t["chosen_width"] == w for t in tuned) for w in (2, 4, 8)},
                         "sort_rays": sum(t["sort_rays"] for t in tuned),
                         "probe": "640x360, 2 spp, binary / 4-wide / 8-wide, each with the ray-sort key off and on; best of 2 after a warm-up"},
            "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 32 * 324,
                    "d2h_bytes_per_step": int(sum(w * h * 4 for _, w, h, _ in specs))},
            "clocks": clocks}
    print(json.dumps(line), flush=True)


def run_serving(args):
    """Serving loop: seeded Poisson arrivals (rate --rate jobs/s, --jobs of
    them) over a pool of 8 scenes (10k-5M triangles, one a 64-bone skinned
    tube re-skinned and rebuilt for every job on it); resolution log-uniform
    256^2..1920x1080, spp log-uniform 1..256.  Latency = submit -> image on
    the host.  Reports p50/p99 latency, Mrays/s over the run, HBM fraction."""
    import threading as th
    from rustracer_gb300 import build, gbrt, workloads as WL, zoo
    build.build()
    depth = DEPTH
    pool = WL.serving_pool()
    trace = WL.serving_trace(seed=0, n=args.jobs, rate=args.rate)
    ctx = gbrt.Context(0)
    scs = [gbrt.Scene(ctx, sd) for sd in pool]
    bones = pool[7].bones
    accs = [gbrt.Accum(ctx, j["width"], j["height"]) for j in trace]
    ubos = [pool[j["scene"]].ubo(j["width"], j["height"], samples=j["spp"], bounces=depth, exposure=1.0)
            for j in trace]
    skins = [zoo.bone_matrices(bones, j["anim_time"]) if j["anim_time"] is not None else None for j in trace]
    # one radiance cache per scene, for the jobs that ask for it
    caches = {k: gbrt.Nrc(ctx, *WL.world_box(pool[k]), log2_table=19, learning_rate=1e-3)
              for k in sorted({j["scene"] for j in trace if j["cache"]})}
    copts = dict(min_roughness=0.25, train_samples=1 << 16, train_steps=1)
    # warm-up: one small job per scene
    warm = [gbrt.Accum(ctx, 64, 64) for _ in scs]
    for _ in range(max(1, args.warmup)):
        ws = [ctx.submit(sc, pool[k].ubo(64, 64, samples=1, bounces=depth, exposure=1.0), warm[k],
                         skins=zoo.bone_matrices(bones, 0.0) if k == 7 else None) for k, sc in enumerate(scs)]
        ws += [ctx.submit(scs[k], pool[k].ubo(64, 64, samples=1, bounces=depth, exposure=1.0), warm[k],
                          skins=zoo.bone_matrices(bones, 0.0) if k == 7 else None, cache=c, **copts)
               for k, c in caches.items()]
        for w in ws:
            w.wait()
    jobs = [None] * len(trace)
    with ClockSampler(0) as clk:
        t0 = time.perf_counter()

        def submitter():
            for i, j in enumerate(trace):
                dt = t0 + j["arrival"] - time.perf_counter()
                if dt > 0:
                    time.sleep(dt)
                c = caches[j["scene"]] if j["cache"] else None
                jobs[i] = ctx.submit(scs[j["scene"]], ubos[i], accs[i], skins=skins[i], cache=c,
                                     **(copts if c is not None else {}))

        thr = th.Thread(target=submitter)
        thr.start()
        thr.join()
        infos = [j.wait() for j in jobs]
        t_end = time.perf_counter()
    clocks = clk.summary()
    lat = np.array([inf["latency_ms"] for inf in infos])
    service = np.array([inf["latency_ms"] - inf["queue_ms"] for inf in infos])  # admitted (first wave) -> done
    cj = np.array([j["cache"] for j in trace], bool)
    rays = np.array([job_rays(inf)[0] for inf in infos], np.float64)
    shaded = np.array([job_rays(inf)[1] for inf in infos], np.float64)
    assert all(inf["status"] == 0 for inf in infos)
    makespan = t_end - t0
    brays = [oracle_bytes_per_ray(sd, depth) for sd in pool]
    alg = float(sum(rays[i] * brays[trace[i]["scene"]] for i in range(len(trace))) + shaded.sum() * B_SHADE)
    peak, peak_kind = measured_peaks()
    paths = np.array([j["width"] * j["height"] * j["spp"] for j in trace], np.float64)
    value = rays.sum() / makespan / 1e6
    line = {"metric": "p99 job latency", "value": float(np.percentile(lat, 99)), "unit": "ms", "n_gpus": 1,
            "steps": 1, "warmup": args.warmup, "ms_per_step": makespan * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded job trace over 8 seeded scenes)",
            "config": {"workload": f"serving_poisson{args.rate:g}_jobs{args.jobs}", "jobs": args.jobs,
                       "rate_per_s": args.rate, "scenes": [sd.name for sd in pool],
                       "triangles": [int(sd.num_triangles) for sd in pool], "depth": depth,
                       "paths_total": int(paths.sum()), "arrival_span_s": trace[-1]["arrival"],
                       "policy": "shortest remaining paths first", "skinned_scene": "64-bone tube, skinned + rebuilt per job",
                       "cache_fraction": 0.25},
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "cache_jobs": {"count": int(sum(j["cache"] for j in trace)),
                           "p50_ms": float(np.percentile(lat[cj], 50)) if cj.any() else None,
                           "p99_ms": float(np.percentile(lat[cj], 99)) if cj.any() else None,
                           "options": copts, "table": "16 x 2^19 x 2, one cache per scene"},
            "mean_queue_ms": float(np.mean([inf["queue_ms"] for inf in infos])),
            "service_ms": {"p50": float(np.percentile(service, 50)), "p99": float(np.percentile(service, 99)),
                           "how": "admission (the job's first wave) to image on the host"},
            "queue_ms": {"p50": float(np.percentile(lat - service, 50)), "p99": float(np.percentile(lat - service, 99))},
            "throughput": {"value": value, "unit": "Mrays/s", "makespan_s": makespan,
                           "offered_load": float(makespan / max(trace[-1]["arrival"], 1e-9))},
            "roofline": {"bound": "hbm", "achieved": alg / makespan / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": alg / makespan / 1e9 / peak, "traffic": None, "peak_source": peak_kind,
                         "kernel": "whole run (algorithmic bytes)",
                         "bytes_per_ray_by_scene": [round(b, 1) for b in brays]},
            "e2e": {"value": float(np.percentile(lat, 99)), "unit": "ms", "h2d_bytes_per_step": int(324 * len(trace)),
                    "d2h_bytes_per_step": int(sum(j["width"] * j["height"] * 4 for j in trace))},
            "clocks": clocks}
    print(json.dumps(line), flush=True)


def run_nrc(args):
    """Radiance cache vs plain path tracing on the city block (about 2M
    instanced triangles, glossy materials, 16 point lights, sky), 1920x1080,
    depth 12: device time until the running mean reaches relMSE <= 1e-2
    against a path-traced reference (--ref-spp samples), relMSE =
    mean((x - ref)^2 / (ref^2 + 1e-2)).  Plain path tracing adds 4 spp per
    frame; the cache run adds --nrc-spp per frame and trains from scratch (its
    training time is counted)."""
    from rustracer_gb300 import build, gbrt, workloads as WL
    build.build()
    Wn, Hn = (int(x) for x in (args.res or "1920x1080").lower().split("x"))
    depth, target = 12, 1e-2
    sd = WL.city_scene()
    ctx = gbrt.Context(0)
    sc = gbrt.Scene(ctx, sd)
    # traversal layout and ray-sort key for this scene (untimed setup, on a plain 4-spp frame), or fixed
    if args.tune == "auto":
        tuning = sc.autotune(sd.ubo(Wn, Hn, samples=4, bounces=depth, exposure=1.0, has_sky=True), Wn, Hn)
    else:
        tuning = {"chosen_width": int(args.tune[1]), "sort_rays": int(args.tune.endswith("s"))}
        sc.set_tuning(tuning["chosen_width"], bool(tuning["sort_rays"]))
    if args.reference_image == "cpu64":
        # the oracle with FP64 intersection and accumulation on every host core, over
        # samples disjoint from the GPU runs' (global indices from 2^24 up)
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import pyoracle as O
        acc64 = np.zeros((Hn * Wn, 4), np.float32)
        t0 = time.time()
        off = 1 << 24
        ref_st = O.OracleScene(sd).render(sd.ubo(Wn, Hn, samples=args.ref_spp, total=off + args.ref_spp,
                                                 bounces=depth, exposure=1.0, has_sky=True), Wn, Hn,
                                          accum=acc64, fp64=True, out=False)["stats"]
        ref = acc64.reshape(Hn, Wn, 4)[..., :3] / float(args.ref_spp)
        ref_image = {"kind": "FP64-intersection CPU oracle", "spp": args.ref_spp, "seconds": round(time.time() - t0, 1),
                 "threads": int(ref_st["threads"]), "samples": f"global indices {off}..{off + args.ref_spp - 1}"}
    else:
        ref_acc = gbrt.Accum(ctx, Wn, Hn)
        chunk = 32
        for k in range(0, args.ref_spp, chunk):
            sc.render(sd.ubo(Wn, Hn, samples=chunk, total=k + chunk, bounces=depth, exposure=1.0, has_sky=True),
                      ref_acc, image=False, mode=MODES["wavefront"])
        ref = ref_acc.download()[..., :3] / float(args.ref_spp)
        ref_image = {"kind": "FP32 GPU path tracing (wavefront)", "spp": args.ref_spp}
    den = ref * ref + 1e-2

    def relmse(acc, spp):
        x = acc.download()[..., :3] / float(spp)
        return float(np.mean((x - ref) ** 2 / den))

    def curve(step, max_frames):
        acc = gbrt.Accum(ctx, Wn, Hn)
        t, spp, pts, reached, rays = 0.0, 0, [], None, 0
        for f in range(max_frames):
            ms, r, n = step(acc, spp)
            t += ms
            spp += n
            rays += r
            e = relmse(acc, spp)
            pts.append((round(t, 2), spp, round(e, 5)))
            if e <= target:
                reached = t
                break
        return reached, pts, rays, t

    def pt_step(acc, spp):
        st = sc.render(sd.ubo(Wn, Hn, samples=4, total=spp + 4, bounces=depth, exposure=1.0, has_sky=True), acc,
                       image=False, mode=MODES["wavefront"])["stats"]
        return float(st["device_ms"]), int(st["rays_total"]), 4

    p = sd.vertices["pos"][:, :3]
    inst = sd.instances["transform"].reshape(-1, 3, 4)
    corners = np.concatenate([inst[:, :, 3] - 2.0, inst[:, :, 3] + 2.0, p])
    lo, hi = corners.min(0) - 0.5, corners.max(0) + 0.5
    cache = gbrt.Nrc(ctx, tuple(map(float, lo)), tuple(map(float, hi)), log2_table=19, learning_rate=1e-3)
    losses = []

    cache_mode = gbrt.NRC_MODE_PRIMARY_INDIRECT if args.nrc_mode == "primary" else gbrt.NRC_MODE_SUFFIX
    frames = [0]

    def nrc_step(acc, spp):
        # the first --nrc-warmup frames are plain path tracing that trains the cache (disabled = 1)
        k = args.nrc_spp
        warm = frames[0] < args.nrc_warmup
        frames[0] += 1
        r = cache.render(sc, sd.ubo(Wn, Hn, samples=k, total=spp + k, bounces=depth, exposure=1.0, has_sky=True),
                         acc, image=False, min_roughness=args.nrc_min_roughness, train_samples=args.nrc_samples,
                         train_steps=args.nrc_steps, disabled=warm, mode=cache_mode)
        losses.append(r["loss"])
        return float(r["stats"]["device_ms"]), int(r["stats"]["rays_total"]), k

    with ClockSampler(0) as clk:
        t_pt, pts_pt, rays_pt, tot_pt = curve(pt_step, args.max_frames)
        t_nrc, pts_nrc, rays_nrc, tot_nrc = curve(nrc_step, 4 * args.max_frames)
        mlp = nrc_mlp_rate(ctx, tuple(map(float, lo)), tuple(map(float, hi)))
    clocks = clk.summary()
    line = {"metric": "time to relMSE <= 1e-2", "value": None if t_nrc is None else t_nrc / 1e3, "unit": "s",
            "n_gpus": 1, "steps": 1, "warmup": 0, "ms_per_step": tot_nrc, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (cache MLP: bf16 x bf16 -> f32)",
            "data": "synthetic (seeded city block of instanced boxes and spheres)",
            "config": {"workload": f"city_nrc_{Wn}x{Hn}_depth{depth}", "instances": int(len(sd.instances)),
                       "instanced_triangles": int(sd.instanced_triangles), "point_lights": 16, "sky": True,
                       "reference": ref_image,
                       "cache": {"levels": 16, "table": 1 << 19, "features": 2, "mlp": "32-64x5-3 ReLU",
                                 "spp_per_frame": args.nrc_spp, "train_samples_per_frame": args.nrc_samples,
                                 "adam_steps_per_frame": args.nrc_steps, "lr": 1e-3,
                                 "min_roughness": args.nrc_min_roughness, "mode": args.nrc_mode,
                                 "warmup_frames": args.nrc_warmup},
                       "tuning": {"chosen_width": tuning["chosen_width"], "sort_rays": tuning["sort_rays"]}},
            "plain_pt": {"time_s": None if t_pt is None else t_pt / 1e3, "curve": pts_pt[:: max(1, len(pts_pt) // 24)],
                         "mrays_per_s": rays_pt / tot_pt / 1e3},
            "cache": {"time_s": None if t_nrc is None else t_nrc / 1e3,
                      "curve": pts_nrc[:: max(1, len(pts_nrc) // 24)], "mrays_per_s": rays_nrc / tot_nrc / 1e3,
                      "final_loss": losses[-1] if losses else None},
            "speedup": (t_pt / t_nrc) if (t_pt and t_nrc) else None,
            "mlp": mlp,
            "clocks": clocks}
    print(json.dumps(line), flush=True)


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    sd = make_scene()
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O
    o = O.OracleScene(sd)
    # A step is a bounded sample of the 64-spp frame with the frame's own per-pixel work: every 64th
    # row (offset by the step), each at all SPP samples, so rows from the whole image are covered.
    stride = 64

    def step_rows(k):
        return list(range(k % stride, H, stride))

    ubo = sd.ubo(W, H, samples=SPP, bounces=DEPTH, exposure=1.0)
    for k in range(args.warmup):
        o.render(ubo, W, H, rows=(step_rows(k)[0], step_rows(k)[0] + 1), out=False)
    rays, secs, threads, nrows = 0, 0.0, 1, 0
    for k in range(args.steps):
        for r in step_rows(k):
            st = o.render(ubo, W, H, rows=(r, r + 1), out=False)["stats"]
            rays += int(st["rays_camera"] + st["rays_extension"] + st["rays_shadow"])
            secs += float(st["seconds"])
            threads = int(st["threads"])
            nrows += 1
    value = rays / secs / 1e6
    sample = f"{args.steps} steps x every {stride}th row of the {W}x{H} frame ({nrows} rows) at {SPP} spp"
    line = common_line(args, world, value, secs / args.steps * 1e3,
                       {"kernel": "CPU oracle (C++ restatement of the reference shaders, OpenMP)",
                        "step_sample": sample})
    line["impl"] = "reference"
    line["cpu_baseline"] = {"value": value, "unit": "Mrays/s", "cores": threads, "kind": "port",
                            "sample": sample}
    line["e2e"] = {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gbrt", choices=["gbrt", "reference"])
    ap.add_argument("--mode", default="auto", choices=list(MODES), help="kernel form (auto = wavefront)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="target length of the CPU-baseline sample")
    ap.add_argument("--res", default=None, help="WxH override for small profiling cases (default 1920x1080)")
    ap.add_argument("--tune", default="auto", choices=["auto", "w2", "w4", "w8", "w2s", "w4s", "w8s"],
                    help="icosphere, nrc: autotuner (untimed setup) or a fixed BVH width w2/w4/w8, s = ray-sort key on")
    ap.add_argument("--spp", type=int, default=None, help="samples per step override (default 64)")
    ap.add_argument("--workload", default="icosphere", choices=["icosphere", "batched", "serving", "nrc"],
                    help="icosphere: the headline frame; batched: 32 scenes as one batch of jobs; "
                         "serving: Poisson job arrivals with p50/p99 latency")
    ap.add_argument("--jobs", type=int, default=200, help="serving: jobs in the trace")
    ap.add_argument("--mix", default="full", choices=["full", "small"],
                    help="batched: the configuration's resolutions and spp (full), or small frames (256^2/512^2 "
                         "at 1-4 spp) of the same scenes")
    ap.add_argument("--rate", type=float, default=200.0, help="serving: arrivals per second")
    ap.add_argument("--ref-spp", type=int, default=1024, help="nrc: samples of the reference image")
    ap.add_argument("--reference-image", default="gpu32", choices=["gpu32", "cpu64"],
                    help="nrc: reference image from FP32 GPU path tracing, or from the FP64-intersection CPU "
                         "oracle (use with a small --res, e.g. 240x136)")
    ap.add_argument("--max-frames", type=int, default=200, help="nrc: frame limit of the plain run (x4 for the cache)")
    ap.add_argument("--nrc-min-roughness", type=float, default=0.25, help="nrc: roughness a cache vertex needs")
    ap.add_argument("--nrc-spp", type=int, default=4, help="nrc: samples per cache frame")
    ap.add_argument("--nrc-samples", type=int, default=1 << 16, help="nrc: training samples per frame")
    ap.add_argument("--nrc-steps", type=int, default=1, help="nrc: Adam steps per frame")
    ap.add_argument("--nrc-mode", default="suffix", choices=["suffix", "primary"],
                    help="nrc: cache vertex = first rough hit after the camera hit (suffix), or the camera hit "
                         "itself for its indirect light (primary)")
    ap.add_argument("--nrc-warmup", type=int, default=0,
                    help="nrc: frames of plain path tracing that train the cache before it is used")
    args = ap.parse_args()
    global W, H, SPP, WORKLOAD
    if args.res:
        W, H = (int(x) for x in args.res.lower().split("x"))
    if args.spp:
        SPP = args.spp
    WORKLOAD = f"icosphere{SUBDIV}_cornell_{W}x{H}_{SPP}spp_depth{DEPTH}"
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batched":
        run_batched(args)
    elif args.workload == "serving":
        run_serving(args)
    elif args.workload == "nrc":
        run_nrc(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
