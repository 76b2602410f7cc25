"""glTF loader and PNG codec (CPU).

A glTF written by the test itself (embedded buffer and PNG texture) is
loaded and checked field by field against what the reference's loader
produces for it: geometry per primitive, generated indices and normals,
materials with their extensions, sRGB / linear classification, node
hierarchy, scene normalisation, instance transforms, lights and skin
indices.  The reference's own Cornell box asset is loaded too when it is
present on this machine.
"""
import base64
import json
import os

import numpy as np
import pytest

from rustracer_gb300 import gltf, png, types as T


def test_png_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    img = rng.integers(0, 256, (17, 23, 4)).astype(np.uint8)
    p = tmp_path / "a.png"
    png.write_png(str(p), img)
    assert np.array_equal(png.read_png(p.read_bytes()), img)
    rgb = img[..., :3].copy()
    png.write_png(str(p), rgb)
    back = png.read_png(p.read_bytes())
    assert np.array_equal(back[..., :3], rgb) and np.all(back[..., 3] == 255)


def _write_gltf(path, tex_png):
    # mesh 0: a quad (4 verts, indices, uv); mesh 1: one triangle, no normals, no indices
    quad = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], np.float32)
    quv = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
    qidx = np.array([0, 1, 2, 0, 2, 3], np.uint16)
    tri = np.array([[0, 0, 0], [2, 0, 0], [0, 0, 2]], np.float32)
    joints = np.array([[1, 2, 0, 0]] * 3, np.uint16)
    weights = np.array([[0.5, 0.5, 0, 0]] * 3, np.float32)
    times = np.array([0, 1, 2], np.float32)
    trans = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0]], np.float32)
    rots = np.array([[0, 0, 0, 1], [0, 0, 0.7071067811865476, 0.7071067811865476], [0, 0, 1, 0]], np.float32)
    ibm = np.stack([np.eye(4), np.diag([2.0, 2.0, 2.0, 1.0])]).astype(np.float32)  # column-major = row-major here
    blobs = [quad.tobytes(), quv.tobytes(), qidx.tobytes() + b"\0\0", tri.tobytes(), joints.tobytes(),
             weights.tobytes(), times.tobytes(), trans.tobytes(), rots.tobytes(), ibm.tobytes(), tex_png]
    views, off = [], 0
    for bl in blobs:
        views.append({"buffer": 0, "byteOffset": off, "byteLength": len(bl)})
        off += len(bl)
    buf = b"".join(blobs)
    acc = [
        {"bufferView": 0, "componentType": 5126, "count": 4, "type": "VEC3", "min": [0, 0, 0], "max": [1, 1, 0]},
        {"bufferView": 1, "componentType": 5126, "count": 4, "type": "VEC2"},
        {"bufferView": 2, "componentType": 5123, "count": 6, "type": "SCALAR"},
        {"bufferView": 3, "componentType": 5126, "count": 3, "type": "VEC3", "min": [0, 0, 0], "max": [2, 0, 2]},
        {"bufferView": 4, "componentType": 5123, "count": 3, "type": "VEC4"},
        {"bufferView": 5, "componentType": 5126, "count": 3, "type": "VEC4"},
        {"bufferView": 6, "componentType": 5126, "count": 3, "type": "SCALAR"},
        {"bufferView": 7, "componentType": 5126, "count": 3, "type": "VEC3"},
        {"bufferView": 8, "componentType": 5126, "count": 3, "type": "VEC4"},
        {"bufferView": 9, "componentType": 5126, "count": 2, "type": "MAT4"},
    ]
    doc = {
        "asset": {"version": "2.0"},
        "buffers": [{"byteLength": len(buf), "uri": "data:application/octet-stream;base64," +
                     base64.b64encode(buf).decode()}],
        "bufferViews": views, "accessors": acc,
        "images": [{"bufferView": 10, "mimeType": "image/png"}],
        "samplers": [{"wrapS": 33071, "wrapT": 33648}],
        "textures": [{"source": 0, "sampler": 0}],
        "materials": [
            {"pbrMetallicRoughness": {"baseColorFactor": [0.5, 0.6, 0.7, 1], "baseColorTexture": {"index": 0},
                                      "metallicFactor": 0.2, "roughnessFactor": 0.3},
             "emissiveFactor": [1, 2, 3], "doubleSided": True},
            {"pbrMetallicRoughness": {"metallicRoughnessTexture": {"index": 0}}, "alphaMode": "MASK",
             "extensions": {"KHR_materials_transmission": {"transmissionFactor": 0.8},
                            "KHR_materials_volume": {"attenuationColor": [0.9, 0.8, 0.7], "thicknessFactor": 0.1},
                            "KHR_materials_ior": {"ior": 1.33},
                            "KHR_materials_specular": {"specularFactor": 0.4, "specularColorFactor": [1, 0.5, 0.25]},
                            "KHR_materials_unlit": {}}},
        ],
        "meshes": [{"primitives": [{"attributes": {"POSITION": 0, "TEXCOORD_0": 1}, "indices": 2, "material": 0}]},
                   {"primitives": [{"attributes": {"POSITION": 3, "JOINTS_0": 4, "WEIGHTS_0": 5}, "material": 1}]}],
        "nodes": [
            {"children": [1, 2], "translation": [1, 0, 0]},
            {"mesh": 0, "scale": [2, 2, 2]},
            {"mesh": 1, "rotation": [0, 0.7071067811865476, 0, 0.7071067811865476], "translation": [0, 0, -3]},
            {"mesh": 1, "skin": 0},
            {"extensions": {"KHR_lights_punctual": {"light": 0}}, "translation": [0, 5, 0]},
        ],
        "extensions": {"KHR_lights_punctual": {"lights": [{"type": "point", "color": [1, 0.5, 0.5], "intensity": 7}]}},
        "scenes": [{"nodes": [0, 3, 4]}], "scene": 0,
        "skins": [{"joints": [1, 2], "inverseBindMatrices": 9}],
        "animations": [{"samplers": [{"input": 6, "output": 7, "interpolation": "LINEAR"},
                                     {"input": 6, "output": 8, "interpolation": "STEP"}],
                        "channels": [{"sampler": 0, "target": {"node": 1, "path": "translation"}},
                                     {"sampler": 1, "target": {"node": 2, "path": "rotation"}}]}],
    }
    with open(path, "w") as f:
        json.dump(doc, f)


def test_generated_gltf(tmp_path):
    tex = np.zeros((2, 2, 4), np.uint8)
    tex[0, 0] = (255, 0, 0, 255)
    tex[1, 1] = (0, 255, 0, 128)
    png.write_png(str(tmp_path / "t.png"), tex)
    path = tmp_path / "scene.gltf"
    _write_gltf(str(path), (tmp_path / "t.png").read_bytes())
    sd = gltf.load(str(path))
    # geometries: quad (4 v / 6 i), triangle (3 v / 3 generated indices)
    assert len(sd.prims) == 2 and list(sd.geo_ranges["v_len"]) == [4, 3] and list(sd.geo_ranges["i_len"]) == [6, 3]
    tri = sd.vertices[4:7]
    assert np.allclose(tri["normal"][:, :3], [0, -1, 0])  # generated: cross(e0, e1) of (x, z) edges
    assert np.all(sd.vertices["pos"][:, 3] == 0) and np.all(sd.vertices["tangent"] == (1, 0, 0, 0))
    # the triangle's mesh is used by the skinned node: skin index 0 on its vertices only
    assert list(sd.vertices["skin_index"]) == [-1] * 4 + [0] * 3
    assert np.array_equal(tri["joints"][0], [1, 2, 0, 0])
    # materials
    m0, m1 = sd.materials[0], sd.materials[1]
    assert np.allclose(m0["base_color"], [0.5, 0.6, 0.7, 1]) and tuple(m0["base_color_texture"]) == (1, 0)
    assert np.allclose(m0["emissive_factor"], [1, 2, 3, 0]) and m0["double_sided"] == 1
    assert m0["metallic_factor"] == np.float32(0.2) and m0["ior"] == np.float32(1.5)
    assert m1["alpha_mode"] == T.ALPHA_MASK and m1["alpha_cutoff"] == np.float32(0.5)
    assert m1["transmission_exist"] == 1 and m1["transmission_factor"] == np.float32(0.8)
    assert m1["volume_exists"] == 1 and m1["attenuation_distance"] == np.finfo(np.float32).max
    assert m1["ior"] == np.float32(1.33) and m1["unlit"] == 1
    assert m1["specular_exist"] == 1 and np.allclose(m1["specular_color_factor"], [1, 0.5, 0.25, 0])
    assert sd.geo_ranges["opaque"][1] == 0  # MASK material
    # textures: white slot 0, then the PNG -- used as base colour (sRGB) and as
    # metallic-roughness (linear): the linear use wins, as in the reference
    assert len(sd.textures) == 2
    w, h, fmt, ws, wt, img = sd.textures[1]
    assert (w, h, ws, wt) == (2, 2, T.WRAP_CLAMP_TO_EDGE, T.WRAP_MIRRORED_REPEAT) and fmt == T.TEX_RGBA8_UNORM
    assert np.array_equal(img, tex)
    # instances: quad under node 0 (translate 1) with scale 2; triangle rotated
    # 90 degrees about y and moved; skinned triangle with identity; all
    # normalised to 10 units along the longest side of the scene box
    xf = sd.instances["transform"].reshape(-1, 3, 4)
    assert len(xf) == 3
    assert np.allclose(xf[2], np.eye(4)[:3])
    s = xf[0][0, 0] / 2.0
    assert np.allclose(xf[0][:, :3], np.eye(3) * 2 * s, atol=1e-6)
    assert np.allclose(xf[1][:, :3], np.array([[0, 0, 1], [0, 1, 0], [-1, 0, 0]]) * s, atol=1e-6)
    assert np.allclose(xf[1][:, 3] - xf[0][:, 3], np.array([0, 0, -3]) * s, atol=1e-5)
    assert list(sd.instances["custom_index_and_mask"] & 0xFFFFFF) == [0, 1, 1]
    assert np.all((sd.instances["custom_index_and_mask"] >> 24) == 0xFF)
    # lights: the point light moved by its node and the normalisation; a
    # zero-intensity directional light added
    assert len(sd.plights) == 1 and sd.plights[0]["kind"] == 1 and sd.plights[0]["intensity"] == 7
    assert np.allclose(sd.plights[0]["color"], [1, 0.5, 0.5, 0])
    assert len(sd.dlights) == 1 and sd.dlights[0]["intensity"] == 0


def test_reference_cornell_asset():
    path = "/root/reference/assets/models/CornellBox/cornellBox.gltf"
    if not os.path.exists(path):
        pytest.skip("reference assets not on this machine")
    sd = gltf.load(path)
    assert len(sd.prims) == 9 and len(sd.instances) == 10 and sd.num_triangles == 16720
    p = sd.vertices["pos"][:, :3]
    xf = sd.instances["transform"].reshape(-1, 3, 4)
    parts = []
    for x, g in zip(xf, sd.instances["blas_handle"]):
        off, n = int(sd.prims[g]["v_offset"]), int(sd.geo_ranges[g]["v_len"])
        parts.append((x[:, :3] @ p[off:off + n].T).T + x[:, 3])
    world = np.concatenate(parts)
    size = world.max(0) - world.min(0)
    assert abs(size.max() - 10.0) < 0.2  # scene scaled to 10 units along its longest side
    assert len(sd.plights) == 5 and np.all(sd.plights["intensity"] == 0)  # no lights in the file


def test_gltf_animation_and_skins(tmp_path):
    tex = np.full((1, 1, 4), 255, np.uint8)
    png.write_png(str(tmp_path / "t.png"), tex)
    _write_gltf(str(tmp_path / "s.gltf"), (tmp_path / "t.png").read_bytes())
    sd = gltf.load(str(tmp_path / "s.gltf"))
    g = sd.gltf
    norm = g.norm
    # node 1 (the quad) is translated by the channel: (0.5, 0, 0) at t = 0.5,
    # (1, 0.5, 0) at t = 1.5, and t = 2.5 wraps to 0.5
    for t, tr in ((0.5, [0.5, 0, 0]), (1.5, [1, 0.5, 0]), (2.5, [0.5, 0, 0])):
        g.animate(t)
        xf = g.instances()["transform"].reshape(-1, 3, 4)[0]
        expect = norm @ np.array([[1, 0, 0, 1], [0, 1, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1.0]]) @ \
            np.block([[np.eye(3) * 2, np.array(tr, float)[:, None]], [np.zeros((1, 3)), np.ones((1, 1))]])
        assert np.allclose(xf, expect[:3], atol=1e-5), t
    # node 2 rotation by STEP: key 1 (90 degrees about z) holds on [1, 2)
    g.animate(1.5)
    w = g.world()
    R = w[2][:3, :3] / norm[0, 0]
    assert np.allclose(R, [[0, -1, 0], [1, 0, 0], [0, 0, 1]], atol=1e-6)
    # joint matrices: world(joint) x inverse bind matrix, column-major; unused slots zero
    sk = g.skins()
    assert sk.shape == (1,)
    m0 = sk[0]["joints"][0].reshape(4, 4).T
    m1 = sk[0]["joints"][1].reshape(4, 4).T
    assert np.allclose(m0, w[1], atol=1e-5)
    assert np.allclose(m1, w[2] @ np.diag([2.0, 2.0, 2.0, 1.0]), atol=1e-5)
    assert np.all(sk[0]["joints"][2:] == 0)


def test_cubemap_faces(tmp_path):
    names = ["right", "left", "top", "bottom", "front", "back"]
    for k, n in enumerate(names):
        png.write_png(str(tmp_path / f"{n}.png"), np.full((4, 4, 4), 10 * k, np.uint8))
    size, data = gltf.load_cubemap(str(tmp_path))
    assert size == 4 and data.size == 6 * 4 * 4 * 4
    assert [int(data[k * 64]) for k in range(6)] == [0, 10, 20, 30, 40, 50]


def test_mikktspace_tangents():
    """MikkTSpace tangents (mikktspace.py) for normal-mapped primitives
    without a TANGENT attribute: along +u of the mapping, orthogonal to the
    normal, unit length; w as the reference's set_tangent writes it (-1
    where the mapping preserves orientation, geometry.rs:333-349)."""
    from rustracer_gb300 import mikktspace
    pos = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], np.float32)
    nrm = np.tile([[0, 0, 1]], (4, 1)).astype(np.float32)
    tri = np.array([[0, 1, 2], [0, 2, 3]])
    uv = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
    assert np.allclose(mikktspace.tangents(pos, nrm, uv, tri), [[1, 0, 0, -1]] * 4, atol=1e-6)
    t = mikktspace.tangents(pos, nrm, uv[:, ::-1], tri)  # u along +y, v along +x: mirrored mapping
    assert np.allclose(t, [[0, 1, 0, 1]] * 4, atol=1e-6)
    # no texture coordinates (zeros): every triangle may join any group, none starts one
    assert np.array_equal(mikktspace.tangents(pos, nrm, np.zeros((4, 2)), tri), [[1, 0, 0, 1]] * 4)
    # a vertex no triangle names keeps the loader's default
    t = mikktspace.tangents(np.r_[pos, [[5, 5, 5]]], np.r_[nrm, [[0, 0, 1]]], np.r_[uv, [[0, 0]]], tri)
    assert np.array_equal(t[4], [1, 0, 0, 0])
    # duplicated vertices with equal attributes are welded: same result as the shared quad
    dpos, dnrm, duv = pos[[0, 1, 2, 0, 2, 3]], nrm[[0, 1, 2, 0, 2, 3]], uv[[0, 1, 2, 0, 2, 3]]
    assert np.allclose(mikktspace.tangents(dpos, dnrm, duv, [[0, 1, 2], [3, 4, 5]]), [[1, 0, 0, -1]] * 6, atol=1e-6)
    # the corner angle weights the sum: a vertex shared by a triangle mapped along +x and one
    # mapped diagonally takes the angle-weighted mean of the two directions
    # (corner angles 135 and 90 degrees; tangents (1, 0, 0) and (1, 1, 0) / sqrt 2)
    p2 = np.array([[0, 0, 0], [1, -1, 0], [0, 1, 0], [-1, 0, 0]], np.float32)
    u2 = np.array([[0, 0], [1, -1], [0, 1], [-1, 1]], np.float32)
    n2 = np.tile([[0, 0, 1]], (4, 1)).astype(np.float32)
    t = mikktspace.tangents(p2, n2, u2, [[0, 1, 2], [0, 2, 3]])
    want = 0.75 * np.pi * np.array([1, 0, 0]) + 0.5 * np.pi * np.array([1, 1, 0]) / np.sqrt(2)
    assert np.allclose(t[0], np.r_[want / np.linalg.norm(want), -1], atol=1e-6)
    # mirrored halves sharing seam vertices: the two orientations form separate groups and the
    # face that names a vertex last decides it
    p3 = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [2, 0, 0], [2, 1, 0]], np.float32)
    u3 = np.array([[0, 0], [1, 0], [1, 1], [0, 1], [0, 0], [0, 1]], np.float32)  # right half mirrored in u
    n3 = np.tile([[0, 0, 1]], (6, 1)).astype(np.float32)
    t = mikktspace.tangents(p3, n3, u3, [[0, 1, 2], [0, 2, 3], [1, 4, 5], [1, 5, 2]])
    assert np.allclose(t[[0, 3]], [[1, 0, 0, -1]] * 2, atol=1e-6)
    assert np.allclose(t[[1, 2, 4, 5]], [[-1, 0, 0, 1]] * 4, atol=1e-6)
    t = mikktspace.tangents(p3, n3, u3, [[1, 4, 5], [1, 5, 2], [0, 1, 2], [0, 2, 3]])
    assert np.allclose(t[[0, 1, 2, 3]], [[1, 0, 0, -1]] * 4, atol=1e-6)
    # a degenerate triangle (two equal positions) copies the first healthy corner of its vertex;
    # its other corners keep the default tangent space ((1, 0, 0), orientation not preserved)
    p4 = np.r_[pos, [[3, 3, 3], [3, 3, 3]]]
    t = mikktspace.tangents(p4, np.r_[nrm, nrm[:2]], np.r_[uv, [[0, 0], [0, 0]]], [[0, 1, 2], [0, 2, 3], [2, 4, 5]])
    assert np.allclose(t[2], [1, 0, 0, -1], atol=1e-6) and np.array_equal(t[4:], [[1, 0, 0, 1]] * 2)
    # a sphere with longitude / latitude mapping: unit tangents orthogonal to the normals, along
    # the direction in which u grows
    from rustracer_gb300.scenes import _icosphere
    v, f = _icosphere(2)
    v = v.astype(np.float32)
    uvs = np.stack([np.arctan2(v[:, 2], v[:, 0]) / (2 * np.pi) + 0.5, np.arccos(np.clip(v[:, 1], -1, 1)) / np.pi], 1)
    t = mikktspace.tangents(v, v, uvs, f)
    assert np.allclose(np.linalg.norm(t[:, :3], axis=1), 1.0, atol=1e-5)
    assert np.abs(np.einsum("ij,ij->i", t[:, :3], v)).max() < 1e-4
    du = np.stack([-v[:, 2], np.zeros(len(v)), v[:, 0]], 1)  # d(position)/d(longitude)
    ok = np.linalg.norm(du, axis=1) > 0.3  # away from the poles
    cosang = np.einsum("ij,ij->i", t[ok, :3], du[ok]) / np.linalg.norm(du[ok], axis=1)
    assert np.median(cosang) > 0.99


def test_loader_generates_tangents_for_normal_maps(tmp_path):
    """A normal-mapped primitive with UVs and no TANGENT gets generated
    tangents (geometry.rs:197-212); without the normal map it keeps the
    default (1, 0, 0, 0)."""
    tex = np.zeros((2, 2, 4), np.uint8)
    png.write_png(str(tmp_path / "t.png"), tex)
    path = tmp_path / "scene.gltf"
    _write_gltf(str(path), (tmp_path / "t.png").read_bytes())
    plain = gltf.load(str(path))
    assert np.allclose(plain.vertices["tangent"][:4], [[1, 0, 0, 0]] * 4)
    doc = json.load(open(path))
    doc["materials"][0]["normalTexture"] = {"index": 0}
    json.dump(doc, open(path, "w"))
    mapped = gltf.load(str(path))
    assert np.allclose(mapped.vertices["tangent"][:4], [[1, 0, 0, -1]] * 4, atol=1e-6)


def _asset_fixture():
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "make_cornell_asset", os.path.join(os.path.dirname(__file__), "golden", "make_cornell_asset.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def test_cornell_asset_fixture():
    """The committed fixture of the reference's Cornell box asset: the loader's
    arrays, with a BLEND material (alpha_mode 3) and an emissive one; equal to
    a fresh load when the reference checkout is on this machine."""
    m = _asset_fixture()
    sd = m.load()
    assert sd.num_triangles == 16720 and len(sd.materials) == 9 and len(sd.instances) == 10
    assert (sd.materials["alpha_mode"] == 3).sum() == 1 and not sd.fully_opaque
    assert (sd.materials["emissive_factor"][:, :3].sum(1) > 0).sum() == 1
    path = "/root/reference/assets/models/CornellBox/cornellBox.gltf"
    if os.path.exists(path):
        fresh = gltf.load(path)
        for k in ("vertices", "indices", "prims", "materials", "geo_ranges", "instances", "plights"):
            assert np.array_equal(getattr(fresh, k).view(np.uint8), getattr(sd, k).view(np.uint8)), k
    import pyoracle as O
    r = O.OracleScene(sd).render(sd.ubo(32, 32, samples=2, bounces=6, exposure=5.0), 32, 32, want_samples=True)
    assert np.all(np.isfinite(r["samples"])) and r["samples"].max() > 0
