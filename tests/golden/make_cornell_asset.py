"""Converts the reference's Cornell box asset into a test fixture.

Reads assets/models/CornellBox/cornellBox.gltf (+ .bin) of the reference
repository through rustracer_gb300.gltf.load -- the harness's glTF loader,
which restates the reference's scene flattening and 10-unit normalisation
(asset_loader/src/scene_graph.rs:277-289) -- and stores the resulting device
arrays (vertices, indices, PrimInfo, materials, geometry ranges, instances,
lights, textures, camera) in tests/golden/cornell_asset.npz, so GPU tests on
machines without the reference checkout render real glTF data.

Run:  python tests/golden/make_cornell_asset.py [path/to/reference]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
OUT = os.path.join(HERE, "cornell_asset.npz")


def main(ref_root):
    from rustracer_gb300 import gltf
    sd = gltf.load(os.path.join(ref_root, "assets", "models", "CornellBox", "cornellBox.gltf"))
    arrays = {k: getattr(sd, k) for k in ("vertices", "indices", "prims", "materials", "geo_ranges", "instances",
                                          "dlights", "plights")}
    for i, (w, h, fmt, ws, wt, data) in enumerate(sd.textures):
        arrays[f"tex{i}"] = np.ascontiguousarray(data)
        arrays[f"tex{i}_desc"] = np.array([w, h, fmt, ws, wt], np.uint32)
    arrays["camera"] = np.array([*sd.camera["eye"], *sd.camera["direction"], sd.camera.get("fov_deg", 60.0)],
                                np.float64)
    np.savez_compressed(OUT, **arrays)
    print(f"wrote {OUT}: {sd.num_triangles} triangles, {len(sd.materials)} materials, {len(sd.textures)} textures")


def load():
    """The fixture as SceneData."""
    from rustracer_gb300.scenes import SceneData
    z = np.load(OUT)
    ntex = sum(1 for k in z.files if k.endswith("_desc"))
    textures = []
    for i in range(ntex):
        w, h, fmt, ws, wt = (int(x) for x in z[f"tex{i}_desc"])
        textures.append((w, h, fmt, ws, wt, z[f"tex{i}"]))
    c = z["camera"]
    return SceneData(vertices=z["vertices"], indices=z["indices"], prims=z["prims"], materials=z["materials"],
                     geo_ranges=z["geo_ranges"], instances=z["instances"], dlights=z["dlights"],
                     plights=z["plights"], textures=textures,
                     camera=dict(eye=tuple(c[:3]), direction=tuple(c[3:6]), fov_deg=float(c[6])),
                     name="cornell_asset")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
