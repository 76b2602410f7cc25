"""Autotuner: the binary, 4-wide and 8-wide BVH layouts, and extension rays
grouped by octant or not, give the same image bit for bit, so what
gbrt_scene_autotune keeps changes speed only."""
import numpy as np
import pytest

from rustracer_gb300 import scenes

pytestmark = pytest.mark.gpu


def test_autotune_keeps_results(gpu_ctx):
    from rustracer_gb300 import gbrt
    sd = scenes.icosphere_scene(subdiv=4)
    sc = gbrt.Scene(gpu_ctx, sd)
    ubo = sd.ubo(160, 120, samples=4, bounces=6, exposure=1.0)
    a0 = gbrt.Accum(gpu_ctx, 160, 120)
    before = sc.render(ubo, a0, mode=gbrt.MODE_WAVEFRONT)["image"]
    rep = sc.autotune(sd.ubo(256, 256, samples=2, bounces=6, exposure=1.0), 256, 256)
    assert rep["chosen_width"] in (2, 4, 8)
    assert rep["ms_binary"] > 0 and rep["ms_wide"] > 0 and rep["ms_wide4"] > 0 and rep["ms_sorted"] > 0
    assert rep["sort_rays"] in (0, 1)
    a1 = gbrt.Accum(gpu_ctx, 160, 120)
    after = sc.render(ubo, a1, mode=gbrt.MODE_WAVEFRONT)["image"]
    assert np.array_equal(before, after)
    assert np.array_equal(a0.download(), a1.download())


@pytest.mark.parametrize("flatten", [True, False], ids=["flattened", "tlas"])
def test_width4_equals_width8(gpu_ctx, flatten):
    """The 4-wide build (world BVH, or BLASes under a TLAS) renders the 8-wide build's image bit for bit."""
    from rustracer_gb300 import gbrt, zoo
    sd = zoo.material_zoo(subdiv=3)
    base = 0 if flatten else gbrt.BUILD_NO_FLATTEN
    out = []
    for flags in (base, base | gbrt.BUILD_WIDTH4):
        sc = gbrt.Scene(gpu_ctx, sd, build_flags=flags)
        acc = gbrt.Accum(gpu_ctx, 160, 120)
        img = sc.render(sd.ubo(160, 120, samples=3, bounces=6, exposure=1.0, has_sky=True), acc,
                        mode=gbrt.MODE_WAVEFRONT)["image"]
        out.append((img, acc.download()))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("width", [2, 8])
def test_sorted_rays_equal_unsorted(gpu_ctx, width):
    """Extension rays grouped by octant (single-frame waves and batched job
    waves) render the ungrouped image bit for bit."""
    from rustracer_gb300 import gbrt, zoo
    sd = zoo.material_zoo(subdiv=3)
    sc = gbrt.Scene(gpu_ctx, sd)
    ubo = sd.ubo(200, 150, samples=3, bounces=8, exposure=1.0, has_sky=True)
    out = []
    for sort in (False, True):
        sc.set_tuning(width, sort)
        acc = gbrt.Accum(gpu_ctx, 200, 150)
        out.append((sc.render(ubo, acc, mode=gbrt.MODE_WAVEFRONT)["image"], acc.download()))
    acc = gbrt.Accum(gpu_ctx, 200, 150)
    job = gpu_ctx.submit(sc, ubo, acc)  # sorting still on
    assert job.wait()["status"] == 0
    out.append((job.image.reshape(out[0][0].shape), acc.download()))
    for img, a in out[1:]:
        assert np.array_equal(out[0][0], img)
        assert np.array_equal(out[0][1], a)
