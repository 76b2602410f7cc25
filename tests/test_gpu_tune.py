"""Autotuner: both BVH layouts give the same image bit for bit, so the
layout gbrt_scene_autotune keeps changes speed only."""
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
    assert rep["chosen_width"] in (2, 8)
    assert rep["ms_binary"] > 0 and rep["ms_wide"] > 0
    a1 = gbrt.Accum(gpu_ctx, 160, 120)
    after = sc.render(ubo, a1, mode=gbrt.MODE_WAVEFRONT)["image"]
    assert np.array_equal(before, after)
    assert np.array_equal(a0.download(), a1.download())
