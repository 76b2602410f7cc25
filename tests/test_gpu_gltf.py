"""A glTF scene (written by the test) loaded and rendered through the C ABI:
primary hits bit-identical to the oracle's, per-sample radiance within the
render contract, and the frame saved as PNG (the headless output)."""
import numpy as np
import pytest

from rustracer_gb300 import gltf, png

pytestmark = pytest.mark.gpu


def test_gltf_scene_render(gpu_ctx, tmp_path):
    import pyoracle as O
    import test_gltf as TG
    from rustracer_gb300 import gbrt
    tex = np.zeros((4, 4, 4), np.uint8)
    tex[...] = (200, 120, 60, 255)
    tex[::2, ::2, 3] = 20
    png.write_png(str(tmp_path / "t.png"), tex)
    TG._write_gltf(str(tmp_path / "s.gltf"), (tmp_path / "t.png").read_bytes())
    sd = gltf.load(str(tmp_path / "s.gltf"))
    ubo = sd.ubo(96, 96, samples=4, bounces=6, exposure=1.0)
    ref = O.OracleScene(sd).render(ubo, 96, 96, want_samples=True, want_hits=True)
    r = gbrt.Scene(gpu_ctx, sd).render(ubo, gbrt.Accum(gpu_ctx, 96, 96), want_samples=True, want_hits=True,
                                       mode=gbrt.MODE_WAVEFRONT)
    assert np.array_equal(r["hits"]["primitive_id"], ref["hits"]["primitive_id"])
    assert np.array_equal(r["hits"]["t"].view(np.uint32), ref["hits"]["t"].view(np.uint32))
    assert (r["hits"]["primitive_id"] != 0xFFFFFFFF).mean() > 0.05
    a, b = r["samples"].reshape(-1, 3).astype(np.float64), ref["samples"].reshape(-1, 3).astype(np.float64)
    ok = np.all(np.abs(a - b) <= 1e-4 * np.maximum(np.abs(a), np.abs(b)) + 1e-6, axis=1)
    assert 1.0 - ok.mean() <= 2e-3
    png.write_png(str(tmp_path / "frame.png"), r["image"])
    assert np.array_equal(png.read_png((tmp_path / "frame.png").read_bytes()), r["image"])
