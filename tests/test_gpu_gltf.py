"""A glTF scene (written by the test) loaded and rendered through the C ABI:
primary hits bit-identical to the oracle's, per-sample radiance within the
parity contract of tests/parity.py, and the frame saved as PNG (the
headless output)."""
import numpy as np
import pytest

import parity
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
    orc = O.OracleScene(sd, diag=True)
    ref = orc.render(ubo, 96, 96, want_samples=True, want_hits=True, want_margins=True)
    r = gbrt.Scene(gpu_ctx, sd).render(ubo, gbrt.Accum(gpu_ctx, 96, 96), want_samples=True, want_hits=True,
                                       mode=gbrt.MODE_WAVEFRONT)
    assert np.array_equal(r["hits"]["primitive_id"], ref["hits"]["primitive_id"])
    assert np.array_equal(r["hits"]["t"].view(np.uint32), ref["hits"]["t"].view(np.uint32))
    assert (r["hits"]["primitive_id"] != 0xFFFFFFFF).mean() > 0.05
    parity.assert_samples(r["samples"], ref, orc, ubo, 96, 96)
    png.write_png(str(tmp_path / "frame.png"), r["image"])
    assert np.array_equal(png.read_png((tmp_path / "frame.png").read_bytes()), r["image"])


@pytest.mark.parametrize("mode", [1, 2], ids=["megakernel", "wavefront"])
def test_reference_cornell_asset_render(gpu_ctx, mode):
    """The reference's own Cornell box asset (16,720 triangles, a BLEND
    sphere, an emissive panel; tests/golden/cornell_asset.npz, converted by
    tests/golden/make_cornell_asset.py) rendered through the C ABI: primary
    hits bit-identical to the oracle's and per-sample radiance within the
    parity contract."""
    import pyoracle as O
    import test_gltf as TG
    from rustracer_gb300 import gbrt
    sd = TG._asset_fixture().load()
    W, H = 96, 96
    ubo = sd.ubo(W, H, samples=4, bounces=8, exposure=5.0)
    orc = O.OracleScene(sd, diag=True)
    ref = orc.render(ubo, W, H, want_samples=True, want_hits=True, want_margins=True)
    r = gbrt.Scene(gpu_ctx, sd).render(ubo, gbrt.Accum(gpu_ctx, W, H), want_samples=True, want_hits=True, mode=mode)
    for f in ("instance_id", "primitive_id"):
        assert np.array_equal(r["hits"][f], ref["hits"][f]), f
    assert np.array_equal(r["hits"]["t"].view(np.uint32), ref["hits"]["t"].view(np.uint32))
    assert (r["hits"]["primitive_id"] != 0xFFFFFFFF).mean() > 0.5
    assert ref["samples"].max() > 0
    parity.assert_samples(r["samples"], ref, orc, ubo, W, H)
