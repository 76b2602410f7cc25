"""The allocation-free world-BVH rebuild (gbrt_scene_rebuild_noalloc).

It is meant for callers that may not allocate device memory while they run,
such as a frame loop that rebuilds a deforming mesh's BVH every frame, or a
host whose device memory belongs to another allocator.  This test checks,
through the C ABI and on two calls in a row, that a scene rebuilt this way
returns exactly the hits (bit for bit, the tolerance of every trace test
here) of a scene built from the same vertices by the ordinary entry points
(gbrt_blas_build + gbrt_tlas_build), and that the size limit and the
identity-instance rule are enforced with an error.  (The test itself may
allocate: it stages the replacement vertices in device memory.)
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


def test_rebuild_noalloc_matches_regular_build(gpu_ctx):
    from rustracer_gb300 import gbrt
    base = scenes.icosphere_scene(subdiv=4)  # 5,154 triangles
    rays = scenes.random_rays(40000, seed=77, origin_box=0.95)
    target = gbrt.Scene(gpu_ctx, _deformed(base, 0))  # built once, then rebuilt in place
    for call, k in enumerate((1, 2)):
        sd_k = _deformed(base, k)
        ref_hits, _ = gbrt.Scene(gpu_ctx, sd_k).trace(rays)  # the ordinary build path
        dv = _to_device(gpu_ctx, np.ascontiguousarray(sd_k.vertices))
        try:
            target.rebuild_noalloc(dv.value)
        finally:
            gpu_ctx.check(gpu_ctx.L.gbrt_device_free(gpu_ctx.h, dv))
        hits, st = target.trace(rays)
        assert st["device_status"] == 0
        assert (ref_hits["instance_id"] != 0xFFFFFFFF).mean() > 0.2
        for f in ("instance_id", "primitive_id", "custom_index"):
            assert np.array_equal(hits[f], ref_hits[f]), (call, f)
        for f in ("t", "u", "v"):
            assert np.array_equal(hits[f].view(np.uint32), ref_hits[f].view(np.uint32)), (call, f)
    # NULL vertices: rebuild from the current vertices gives the same hits again
    target.rebuild_noalloc(None)
    again, _ = target.trace(rays)
    assert np.array_equal(again, hits)


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
