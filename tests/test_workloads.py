"""Host-side workload generators of the bench (CPU): the serving trace is
seeded and reproducible with the stated shape, and world_box encloses every
instanced triangle in world space."""
import numpy as np

from rustracer_gb300 import scenes, workloads as WL


def test_serving_trace_reproducible_and_shaped():
    a, b = WL.serving_trace(seed=3, n=400), WL.serving_trace(seed=3, n=400)
    assert a == b
    arr = np.array([j["arrival"] for j in a])
    assert np.all(np.diff(arr) > 0)
    assert 1.2 < arr[-1] < 2.8  # Poisson at 200 jobs/s: 400 jobs in about 2 s
    npix = np.array([j["width"] * j["height"] for j in a])
    assert npix.min() >= 200 * 100 and npix.max() <= 1920 * 1080 * 1.01
    spp = np.array([j["spp"] for j in a])
    assert spp.min() >= 1 and spp.max() <= 256
    assert all((j["anim_time"] is not None) == (j["scene"] == 7) for j in a)
    frac = np.mean([j["cache"] for j in a])
    assert 0.18 < frac < 0.32  # a quarter of the jobs use the radiance cache
    # the cache draw has its own stream: the rest of the trace is the same with or without it
    c = WL.serving_trace(seed=3, n=400, cache_frac=0.0)
    assert not any(j["cache"] for j in c)
    assert [dict(j, cache=False) for j in a] == c


def test_world_box_encloses_instances():
    sd, _, _, _ = WL.batched_scene(4, max_tri=20_000)
    lo, hi = (np.array(v) for v in WL.world_box(sd, pad=0.0))
    p = np.concatenate([sd.vertices["pos"][:, :3], np.ones((len(sd.vertices), 1), np.float32)], 1).astype(np.float64)
    m = sd.instances["transform"].reshape(-1, 3, 4).astype(np.float64)
    assert len(m) > 1
    for inst in m:  # every instance's image of every vertex (a superset of its own geometry)
        w = p @ inst.T
        assert np.all(w.min(0) >= lo - 1e-4) and np.all(w.max(0) <= hi + 1e-4)
    ico = scenes.icosphere_scene(subdiv=2)
    lo2, hi2 = WL.world_box(ico, pad=0.0)
    q = ico.vertices["pos"][:, :3]
    assert np.all(q.min(0) >= np.array(lo2) - 1e-6) and np.all(q.max(0) <= np.array(hi2) + 1e-6)
