"""The allocation-free world-BVH rebuild (gbrt_scene_rebuild_noalloc).

It is meant for callers that may not allocate device memory while they run,
such as a frame loop that rebuilds a deforming mesh's BVH every frame, or a
host whose device memory belongs to another allocator.  This test checks,
through the C ABI and on two calls in a row, that a scene rebuilt this way
returns exactly the hits (bit for bit, the tolerance of every trace test
here) of a scene built from the same vertices by the ordinary entry points
(gbrt_blas_build + gbrt_tlas_build); that the call allocates nothing (the
device's free memory and the stream-ordered pool's usage do not move around
it); that a scene of exactly the maximum size rebuilds correctly; and that the
size limit, the identity-instance rule and the busy rule are enforced with an
error.  (The test itself may allocate: it stages the replacement vertices in
device memory.)
"""
import ctypes as C

import numpy as np
import pytest

from rustracer_gb300 import scenes, types as T

pytestmark = pytest.mark.gpu


def _deformed(sd, k):
    """Same topology, vertices moved: the sphere part is scaled and sheared."""
    v = sd.vertices.copy()
    sph = np.arange(len(v)) >= 68  # the Cornell box owns the first 68 vertices
    p = v["pos"][sph, :3].astype(np.float64)
    c = p.mean(0)
    p = (p - c) * (1.0 + 0.15 * k) + c
    p[:, 0] += 0.05 * k * p[:, 1]
    v["pos"][sph, :3] = p.astype(np.float32)
    out = scenes.SceneData(**{**sd.__dict__, "vertices": v})
    return out


def _to_device(ctx, arr):
    ptr = C.c_void_p()
    ctx.check(ctx.L.gbrt_device_alloc(ctx.h, arr.nbytes, C.byref(ptr)))
    ctx.check(ctx.L.gbrt_memcpy_h2d(ctx.h, ptr, arr.ctypes.data_as(C.c_void_p), arr.nbytes))
    return ptr


class _PoolUsage:
    """Used bytes of the device's default stream-ordered memory pool (the pool
    cudaMallocAsync draws from), read through the driver API."""
    USED_MEM_CURRENT, USED_MEM_HIGH = 7, 8  # CUmemPool_attribute

    def __init__(self, device=0):
        self.cu = C.CDLL("libcuda.so.1")
        dev = C.c_int()
        assert self.cu.cuDeviceGet(C.byref(dev), device) == 0
        self.pool = C.c_void_p()
        assert self.cu.cuDeviceGetDefaultMemPool(C.byref(self.pool), dev) == 0

    def get(self, attr):
        v = C.c_uint64()
        assert self.cu.cuMemPoolGetAttribute(self.pool, attr, C.byref(v)) == 0
        return v.value

    def reset_high(self):
        zero = C.c_uint64(0)
        assert self.cu.cuMemPoolSetAttribute(self.pool, self.USED_MEM_HIGH, C.byref(zero)) == 0


def _assert_same_hits(hits, ref_hits, where):
    for f in ("instance_id", "primitive_id", "custom_index"):
        assert np.array_equal(hits[f], ref_hits[f]), (where, f)
    for f in ("t", "u", "v"):
        assert np.array_equal(hits[f].view(np.uint32), ref_hits[f].view(np.uint32)), (where, f)


def test_rebuild_noalloc_matches_regular_build(gpu_ctx):
    from rustracer_gb300 import gbrt
    base = scenes.icosphere_scene(subdiv=4)  # 5,154 triangles
    rays = scenes.random_rays(40000, seed=77, origin_box=0.95)
    target = gbrt.Scene(gpu_ctx, _deformed(base, 0))  # built once, then rebuilt in place
    pool = _PoolUsage()
    for call, k in enumerate((1, 2)):
        sd_k = _deformed(base, k)
        ref_hits, _ = gbrt.Scene(gpu_ctx, sd_k).trace(rays)  # the ordinary build path
        dv = _to_device(gpu_ctx, np.ascontiguousarray(sd_k.vertices))
        try:
            gpu_ctx.sync()
            pool.reset_high()
            used0, free0 = pool.get(pool.USED_MEM_CURRENT), gpu_ctx.mem_info()[0]
            target.rebuild_noalloc(dv.value)
            used1, free1 = pool.get(pool.USED_MEM_CURRENT), gpu_ctx.mem_info()[0]
            if call == 1:  # the first call may load the library's device module; the second must not allocate
                assert free1 == free0, ("device free memory moved", free0, free1)
                assert used1 == used0 and pool.get(pool.USED_MEM_HIGH) <= used0, \
                    ("stream-ordered pool used", used0, used1, pool.get(pool.USED_MEM_HIGH))
        finally:
            gpu_ctx.check(gpu_ctx.L.gbrt_device_free(gpu_ctx.h, dv))
        hits, st = target.trace(rays)
        assert st["device_status"] == 0
        assert (ref_hits["instance_id"] != 0xFFFFFFFF).mean() > 0.2
        _assert_same_hits(hits, ref_hits, call)
    # NULL vertices: rebuild from the current vertices gives the same hits again
    target.rebuild_noalloc(None)
    again, _ = target.trace(rays)
    assert np.array_equal(again, hits)
    # traversal above used the wide BVH refit in place; the rebuilt binary BVH gives the same hits
    target.set_tuning(width=2)
    binary, _ = target.trace(rays)
    _assert_same_hits(binary, hits, "binary")


def test_rebuild_noalloc_at_the_limit(gpu_ctx):
    """A world BVH of exactly GBRT_NOALLOC_MAX_TRIANGLES triangles fits the
    static scratch and rebuilds to the ordinary build's hits."""
    from rustracer_gb300 import gbrt
    n = gbrt.NOALLOC_MAX_TRIANGLES
    sd = scenes.random_soup(n, seed=5, nmat=2)
    assert len(sd.indices) // 3 == n
    rays = scenes.random_rays(30000, seed=78, origin_box=1.2)
    ref_hits, _ = gbrt.Scene(gpu_ctx, sd).trace(rays)
    sc = gbrt.Scene(gpu_ctx, sd)
    for call in range(2):
        sc.rebuild_noalloc(None)
        hits, st = sc.trace(rays)
        assert st["device_status"] == 0
        assert (ref_hits["instance_id"] != 0xFFFFFFFF).mean() > 0.1
        _assert_same_hits(hits, ref_hits, call)


def test_rebuild_noalloc_limits(gpu_ctx):
    from rustracer_gb300 import gbrt
    big = scenes.random_soup(gbrt.NOALLOC_MAX_TRIANGLES + 1, seed=3, nmat=1)
    sc = gbrt.Scene(gpu_ctx, big)
    with pytest.raises(gbrt.GbrtError) as e:
        sc.rebuild_noalloc(None)
    assert e.value.code == gbrt.E_INVALID and "at most" in str(e.value)
    moved = scenes.random_soup(100, seed=4, nmat=1)
    xf = T.IDENTITY34.copy()
    xf[3] = 0.5
    moved.instances = scenes.identity_instances([0], [xf])
    sc2 = gbrt.Scene(gpu_ctx, moved)
    with pytest.raises(gbrt.GbrtError) as e:
        sc2.rebuild_noalloc(None)
    assert e.value.code == gbrt.E_INVALID and "identity" in str(e.value)


def test_rebuild_noalloc_busy_while_jobs_run(gpu_ctx):
    """Queued jobs read the scene's BVH from the job thread, so the rebuild is
    refused while any job of the context is unfinished."""
    from rustracer_gb300 import gbrt
    sd = scenes.icosphere_scene(subdiv=4)
    sc = gbrt.Scene(gpu_ctx, sd)
    acc = gbrt.Accum(gpu_ctx, 1280, 720)
    job = gpu_ctx.submit(sc, sd.ubo(1280, 720, samples=32, bounces=8, exposure=1.0), acc, image=False)
    with pytest.raises(gbrt.GbrtError) as e:
        sc.rebuild_noalloc(None)
    assert e.value.code == gbrt.E_BUSY
    assert job.wait()["status"] == 0
    sc.rebuild_noalloc(None)  # allowed again once the jobs are done
