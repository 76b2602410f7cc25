"""glTF 2.0 -> the device-layout scene the C ABI takes (SceneData).

Follows the reference's asset loader, step by step:
* one geometry per triangle primitive with a POSITION attribute
  (geometry.rs:100-267, is_primitive_supported :291-293), vertices laid out
  like Vertex (pos.w = 0, uv0/uv1 default 0, colour default 1, tangent
  default (1, 0, 0, 0), joints/weights default 0, skin_index -1), indices
  generated when absent, normals generated per triangle when absent
  (create_geo_normal, :270-289: the last triangle that touches a vertex
  wins);
* the geometry's material is the primitive's, material 0 when it has none
  (DEFAULT_MATERIAL_INDEX);
* materials packed like MaterialRaw::from (material.rs:130-381): texture
  index + 1 (slot 0 is a 1x1 white texture), alpha cutoff 0.5 by default,
  emissive (r, g, b, 0), ior 1.5 unless KHR_materials_ior, transmission /
  volume / specular / specular-glossiness / unlit from their extensions;
* textures: sRGB for colour textures, linear for normal, metallic-
  roughness, transmission and specular textures (find_linear_textures,
  material.rs:103-128), wrap modes from the sampler;
* the default scene's node tree walked depth first from its root nodes
  (scene_graph.rs:83-103); the whole scene scaled to 10 units along its
  longest side and centred (load_scene, aabb.rs:65-69), node boxes
  transformed by their min and max corners like Aabb * Mat4;
* one instance per (node with a mesh, primitive) in that order, with the
  node's world transform as a row-major 3x4, identity for skinned nodes,
  custom index = geometry id, mask 0xFF, facing-cull disabled
  (create_top_as, acceleration_structures.rs:136-172);
* vertices of meshes used by skinned nodes get that skin's index
  (duplicate_mesh_for_non_affine_transform, scene_graph.rs:191-235);
* KHR_lights_punctual lights transformed by their node (light.rs:9-47,
  spot lights as point lights); five zero-intensity point lights when the
  scene has none and one zero-intensity directional light when it has none
  (scene_graph.rs:55-81; the reference places the five at random, here
  they are seeded).

Animation (GltfScene.animate / instances / skins) follows animation.rs and
skinning.rs: every channel's time wraps into [first key, last key), the key
segment is found by a linear scan, translation and scale interpolate
linearly, by step or by cubic Hermite spline (glTF in / value / out
tangents), rotations by slerp (also for cubic splines) or step; the node's
TRS takes the channel's output and the world transforms are recomputed; a
skin's joint matrices are world(joint) x inverse bind matrix, column-major,
256 slots with zero matrices past the last joint.

Primitives whose material has a normal texture and that carry no TANGENT
attribute get MikkTSpace tangents (mikktspace.py, as the reference's
generate_tangents call, geometry.rs:192-212, with its w convention);
textures may be PNG or baseline JPEG (jpeg.py).  Morph targets are ignored,
as in the reference (animation.rs:141-142), and so are glTF cameras (the
reference's camera comes from its viewer).
"""
import base64
import json
import os
import struct

import numpy as np

from . import mikktspace
from . import types as T
from .scenes import GeoBuilder, SceneData, identity_instances

_COMP = {5120: np.int8, 5121: np.uint8, 5122: np.int16, 5123: np.uint16, 5125: np.uint32, 5126: np.float32}
_NCOMP = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4, "MAT2": 4, "MAT3": 9, "MAT4": 16}
_WRAP = {33071: T.WRAP_CLAMP_TO_EDGE, 33648: T.WRAP_MIRRORED_REPEAT, 10497: T.WRAP_REPEAT}


def _load(path):
    """(json dict, list of buffer bytes) of a .gltf or .glb file."""
    raw = open(path, "rb").read()
    base = os.path.dirname(os.path.abspath(path))
    glb_bin = None
    if raw[:4] == b"glTF":
        _, _, length = struct.unpack("<III", raw[:12])
        pos, doc = 12, None
        while pos < length:
            n, kind = struct.unpack("<II", raw[pos:pos + 8])
            body = raw[pos + 8:pos + 8 + n]
            if kind == 0x4E4F534A:
                doc = json.loads(body.decode("utf-8"))
            elif kind == 0x004E4942:
                glb_bin = body
            pos += 8 + n
    else:
        doc = json.loads(raw.decode("utf-8"))
    bufs = []
    for b in doc.get("buffers", []):
        uri = b.get("uri")
        if uri is None:
            bufs.append(glb_bin)
        elif uri.startswith("data:"):
            bufs.append(base64.b64decode(uri.split(",", 1)[1]))
        else:
            bufs.append(open(os.path.join(base, uri), "rb").read())
    return doc, bufs, base


def _accessor(doc, bufs, i):
    a = doc["accessors"][i]
    dt = np.dtype(_COMP[a["componentType"]])
    nc = _NCOMP[a["type"]]
    count = a["count"]
    out = np.zeros((count, nc), dt)
    if "bufferView" in a:
        bv = doc["bufferViews"][a["bufferView"]]
        data = bufs[bv["buffer"]]
        off = bv.get("byteOffset", 0) + a.get("byteOffset", 0)
        stride = bv.get("byteStride", 0) or dt.itemsize * nc
        arr = np.ndarray((count, nc), dt, buffer=data, offset=off, strides=(stride, dt.itemsize))
        out[:] = arr
    if a.get("normalized") and dt != np.float32:
        scale = float(np.iinfo(dt).max)
        out = np.maximum(out.astype(np.float32) / scale, -1.0)
    return out


def _trs_matrix(t, q, s):
    x, y, z, w = q
    R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                  [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                  [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])
    M = np.eye(4)
    M[:3, :3] = R * np.asarray(s, np.float64)[None, :]
    M[:3, 3] = t
    return M


def _mat_of_node(node):
    if "matrix" in node:
        return np.array(node["matrix"], np.float64).reshape(4, 4).T  # column-major
    return _trs_matrix(np.array(node.get("translation", [0, 0, 0]), np.float64), node.get("rotation", [0, 0, 0, 1]),
                       node.get("scale", [1, 1, 1]))


def _decompose(M):
    """TRS of an affine matrix (for matrix nodes that get animated)."""
    t = M[:3, 3].copy()
    s = np.linalg.norm(M[:3, :3], axis=0)
    R = M[:3, :3] / np.where(s == 0, 1, s)[None, :]
    w = np.sqrt(max(0.0, 1 + R[0, 0] + R[1, 1] + R[2, 2])) / 2
    x = np.sqrt(max(0.0, 1 + R[0, 0] - R[1, 1] - R[2, 2])) / 2
    y = np.sqrt(max(0.0, 1 - R[0, 0] + R[1, 1] - R[2, 2])) / 2
    z = np.sqrt(max(0.0, 1 - R[0, 0] - R[1, 1] + R[2, 2])) / 2
    x = np.copysign(x, R[2, 1] - R[1, 2])
    y = np.copysign(y, R[0, 2] - R[2, 0])
    z = np.copysign(z, R[1, 0] - R[0, 1])
    return t, np.array([x, y, z, w]), s


def _slerp(a, b, f):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    d = float(np.dot(a, b))
    if d < 0:
        b, d = -b, -d
    if d > 0.9995:
        q = a + (b - a) * f
        return q / np.linalg.norm(q)
    th = np.arccos(d)
    return (np.sin((1 - f) * th) * a + np.sin(f * th) * b) / np.sin(th)


def _hermite(p0, m0, p1, m1, t):
    t2, t3 = t * t, t * t * t
    return (2 * t3 - 3 * t2 + 1) * p0 + (t3 - 2 * t2 + t) * m0 + (-2 * t3 + 3 * t2) * p1 + (t3 - t2) * m1


class _Channel:
    def __init__(self, node, path, times, values, interp):
        self.node, self.path, self.times, self.values, self.interp = node, path, times, values, interp

    def sample(self, t):
        inp = self.times
        lo, hi = inp[0], inp[-1]
        if t > lo and hi > lo:
            t = (t - lo) % (hi - lo) + lo
        s = e = 0
        for i in range(len(inp) - 1):
            if inp[i] <= t <= inp[i + 1]:
                s, e = i, i + 1
        pt, nt = inp[s], inp[e]
        f = (t - pt) / (nt - pt) if nt > pt else 0.0
        v = self.values
        if self.interp == "CUBICSPLINE":
            key = lambda k: v[3 * k:3 * k + 3]  # in tangent, value, out tangent
            if self.path == "rotation":
                return _slerp(key(s)[1], key(e)[1], f)
            dt = nt - pt
            return _hermite(key(s)[1], dt * key(s)[2], key(e)[1], dt * key(e)[0], f)
        if self.interp == "STEP":
            return v[s]
        if self.path == "rotation":
            return _slerp(v[s], v[e], f)
        return v[s] + (v[e] - v[s]) * f


def _texinfo(info):
    if info is None:
        return (-1, -1)
    return (1 + int(info["index"]), int(info.get("texCoord", 0)))


def _material(m):
    raw = T.default_material()
    pbr = m.get("pbrMetallicRoughness", {})
    ext = m.get("extensions", {})
    raw["alpha_mode"] = {"OPAQUE": T.ALPHA_OPAQUE, "MASK": T.ALPHA_MASK, "BLEND": T.ALPHA_BLEND}[m.get("alphaMode", "OPAQUE")]
    raw["alpha_cutoff"] = m.get("alphaCutoff", 0.5)
    raw["double_sided"] = int(bool(m.get("doubleSided", False)))
    raw["base_color"] = pbr.get("baseColorFactor", [1, 1, 1, 1])
    raw["base_color_texture"] = _texinfo(pbr.get("baseColorTexture"))
    raw["metallic_factor"] = pbr.get("metallicFactor", 1.0)
    raw["roughness_factor"] = pbr.get("roughnessFactor", 1.0)
    raw["metallic_roughness_texture"] = _texinfo(pbr.get("metallicRoughnessTexture"))
    raw["normal_texture"] = _texinfo(m.get("normalTexture"))
    raw["emissive_texture"] = _texinfo(m.get("emissiveTexture"))
    raw["emissive_factor"] = list(m.get("emissiveFactor", [0, 0, 0])) + [0.0]
    raw["occlusion_texture"] = _texinfo(m.get("occlusionTexture"))
    raw["ior"] = ext.get("KHR_materials_ior", {}).get("ior", 1.5)
    raw["unlit"] = int("KHR_materials_unlit" in ext)
    if "KHR_materials_transmission" in ext:
        tr = ext["KHR_materials_transmission"]
        raw["transmission_texture"] = _texinfo(tr.get("transmissionTexture"))
        raw["transmission_factor"] = tr.get("transmissionFactor", 0.0)
        raw["transmission_exist"] = 1
    if "KHR_materials_volume" in ext:
        vo = ext["KHR_materials_volume"]
        raw["attenuation_color"] = vo.get("attenuationColor", [1, 1, 1])
        raw["thickness_factor"] = vo.get("thicknessFactor", 0.0)
        raw["thickness_texture"] = _texinfo(vo.get("thicknessTexture"))
        raw["attenuation_distance"] = vo.get("attenuationDistance", np.finfo(np.float32).max)
        raw["volume_exists"] = 1
    if "KHR_materials_specular" in ext:
        sp = ext["KHR_materials_specular"]
        raw["specular_texture"] = _texinfo(sp.get("specularTexture"))
        raw["specular_color_texture"] = _texinfo(sp.get("specularColorTexture"))
        raw["specular_color_factor"] = list(sp.get("specularColorFactor", [1, 1, 1])) + [0.0]
        raw["specular_factor"] = sp.get("specularFactor", 1.0)
        raw["specular_exist"] = 1
    if "KHR_materials_pbrSpecularGlossiness" in ext:
        sg = ext["KHR_materials_pbrSpecularGlossiness"]
        raw["workflow"] = 1
        raw["sg_diffuse_factor"] = sg.get("diffuseFactor", [1, 1, 1, 1])
        raw["sg_specular_glossiness_factor"] = list(sg.get("specularFactor", [1, 1, 1])) + [
            sg.get("glossinessFactor", 1.0)]
        raw["sg_diffuse_texture"] = _texinfo(sg.get("diffuseTexture"))
        raw["sg_specular_glossiness_texture"] = _texinfo(sg.get("specularGlossinessTexture"))
    return raw


def _linear_images(doc):
    lin = set()
    tex = doc.get("textures", [])

    def add(info):
        if info is not None and "source" in tex[info["index"]]:
            lin.add(tex[info["index"]]["source"])
    for m in doc.get("materials", []):
        add(m.get("normalTexture"))
        add(m.get("pbrMetallicRoughness", {}).get("metallicRoughnessTexture"))
        ext = m.get("extensions", {})
        add(ext.get("KHR_materials_transmission", {}).get("transmissionTexture"))
        add(ext.get("KHR_materials_specular", {}).get("specularTexture"))
    return lin


def _textures(doc, bufs, base):
    from .jpeg import read_jpeg
    from .png import read_png
    white = (1, 1, T.TEX_RGBA8_SRGB, T.WRAP_REPEAT, T.WRAP_REPEAT, np.full((1, 1, 4), 255, np.uint8))
    out = [white]
    lin = _linear_images(doc)
    images = doc.get("images", [])
    samplers = doc.get("samplers", [])
    for t in doc.get("textures", []):
        smp = samplers[t["sampler"]] if "sampler" in t else {}
        ws, wt = _WRAP[smp.get("wrapS", 10497)], _WRAP[smp.get("wrapT", 10497)]
        src = t.get("source")
        img = None
        if src is not None:
            im = images[src]
            if "bufferView" in im:
                bv = doc["bufferViews"][im["bufferView"]]
                data = bufs[bv["buffer"]][bv.get("byteOffset", 0):bv.get("byteOffset", 0) + bv["byteLength"]]
            elif im.get("uri", "").startswith("data:"):
                data = base64.b64decode(im["uri"].split(",", 1)[1])
            else:
                data = open(os.path.join(base, im["uri"]), "rb").read()
            if data[:8] == b"\x89PNG\r\n\x1a\n":
                img = read_png(data)
            elif data[:2] == b"\xff\xd8":
                img = read_jpeg(data)
        if img is None:
            out.append(white)
            continue
        fmt = T.TEX_RGBA8_UNORM if src in lin else T.TEX_RGBA8_SRGB
        out.append((img.shape[1], img.shape[0], fmt, ws, wt, img))
    return out


def load(path, light_seed=0):
    """Loads a .gltf / .glb file into SceneData (the arrays the C ABI takes)."""
    doc, bufs, base = _load(path)
    nodes = doc.get("nodes", [])
    meshes = doc.get("meshes", [])
    mats = doc.get("materials", [])
    b = GeoBuilder()
    for m in mats:
        b.add_material(_material(m))
    if not mats:
        b.add_material(T.default_material())
    # meshes -> geometries (one per supported primitive), object-space boxes
    mesh_geos, mesh_box = [], []
    for mesh in meshes:
        geos, lo, hi = [], np.full(3, np.inf), np.full(3, -np.inf)
        for p in mesh["primitives"]:
            attrs = p["attributes"]
            if "POSITION" not in attrs or p.get("mode", 4) != 4:
                continue
            pos = _accessor(doc, bufs, attrs["POSITION"]).astype(np.float32)
            n = len(pos)
            idx = (_accessor(doc, bufs, p["indices"]).reshape(-1).astype(np.uint32) if "indices" in p
                   else np.arange(n, dtype=np.uint32))
            if "NORMAL" in attrs:
                nrm = _accessor(doc, bufs, attrs["NORMAL"]).astype(np.float32)
            else:
                nrm = np.zeros((n, 3), np.float32)
                for t in idx.reshape(-1, 3):
                    p0, p1, p2 = pos[t[0]], pos[t[1]], pos[t[2]]
                    e0 = (p1 - p0) / np.linalg.norm(p1 - p0)
                    e1 = (p2 - p0) / np.linalg.norm(p2 - p0)
                    c = np.cross(e0, e1)
                    nrm[t] = c / np.linalg.norm(c)
            get = lambda k, dim: _accessor(doc, bufs, attrs[k]).astype(np.float32)[:, :dim] if k in attrs else None
            color = None
            if "COLOR_0" in attrs:
                c = _accessor(doc, bufs, attrs["COLOR_0"]).astype(np.float32)
                color = np.concatenate([c, np.ones((n, 1), np.float32)], 1) if c.shape[1] == 3 else c
            tangent = get("TANGENT", 4)
            mat_raw = mats[p.get("material", 0)] if mats else {}
            if tangent is None and "normalTexture" in mat_raw:  # uv0 defaults to zeros, as in geometry.rs:182-185
                uv0 = get("TEXCOORD_0", 2)
                tangent = mikktspace.tangents(pos, nrm, uv0 if uv0 is not None else np.zeros((n, 2), np.float32),
                                              idx.reshape(-1, 3))
            base_v = b.add_vertices(pos, nrm, uv=get("TEXCOORD_0", 2), color=color, tangent=tangent,
                                    joints=_accessor(doc, bufs, attrs["JOINTS_0"]).astype(np.uint32)
                                    if "JOINTS_0" in attrs else None,
                                    weights=get("WEIGHTS_0", 4))
            uv1 = get("TEXCOORD_1", 2)
            if uv1 is not None:
                b.vchunks[-1]["uv1"] = uv1
            mat = p.get("material", 0)
            geos.append(b.add_geometry(base_v, n, idx.reshape(-1, 3), mat))
            lo, hi = np.minimum(lo, pos.min(0)), np.maximum(hi, pos.max(0))
        mesh_geos.append(geos)
        mesh_box.append((lo, hi) if geos else None)
    # scene tree, normalisation
    scene = doc.get("scenes", [{"nodes": list(range(len(nodes)))}])[doc.get("scene", 0)]
    roots = scene.get("nodes", [])
    local = [_mat_of_node(nd) for nd in nodes]

    def node_box(i):
        boxes = [node_box(c) for c in nodes[i].get("children", [])]
        if "mesh" in nodes[i] and mesh_box[nodes[i]["mesh"]] is not None:
            boxes.append(mesh_box[nodes[i]["mesh"]])
        boxes = [bx for bx in boxes if bx is not None]
        if not boxes:
            return None
        lo = np.min([bx[0] for bx in boxes], 0)
        hi = np.max([bx[1] for bx in boxes], 0)
        a = local[i] @ np.append(lo, 1.0)
        c = local[i] @ np.append(hi, 1.0)
        return np.minimum(a[:3], c[:3]), np.maximum(a[:3], c[:3])
    boxes = [bx for bx in (node_box(r) for r in roots) if bx is not None]
    norm = np.eye(4)
    if boxes:
        lo, hi = np.min([bx[0] for bx in boxes], 0), np.max([bx[1] for bx in boxes], 0)
        size = hi - lo
        side = size[0] if (size[0] > size[1] and size[0] > size[2]) else (size[1] if size[1] > size[2] else size[2])
        scale = 10.0 / side if side > 0 else 1.0
        norm = np.diag([scale, scale, scale, 1.0]) @ np.block([[np.eye(3), -(lo + size / 2)[:, None]],
                                                               [np.zeros((1, 3)), np.ones((1, 1))]])
    lights = doc.get("extensions", {}).get("KHR_lights_punctual", {}).get("lights", [])
    state = GltfScene(doc, bufs, local, roots, norm, mesh_geos)
    world = state.world()
    dl, pl = [], []
    skinned_meshes = {}
    for i in state.order:
        nd = nodes[i]
        if "mesh" in nd and "skin" in nd:
            skinned_meshes.setdefault(nd["mesh"], nd["skin"])
        li = nd.get("extensions", {}).get("KHR_lights_punctual", {}).get("light")
        if li is not None:
            L = lights[li]
            raw = np.zeros((), T.LIGHT)
            raw["color"] = list(L.get("color", [1, 1, 1])) + [0.0]
            kind = L.get("type", "point")
            v = world[i] @ (np.array([0, 0, -1.0, 0]) if kind == "directional" else np.array([0, 0, 0, 1.0]))
            raw["transform"] = v.astype(np.float32)
            raw["kind"] = 0 if kind == "directional" else 1
            raw["range"] = L.get("range", np.finfo(np.float32).max)
            raw["intensity"] = L.get("intensity", 1.0)
            (dl if kind == "directional" else pl).append(raw)
    # skin indices of meshes used by skinned nodes
    for m, skin in skinned_meshes.items():
        for g in mesh_geos[m]:
            p = b.prims[g]
            off, n = int(p["v_offset"]), int(b.ranges[g]["v_len"])
            verts = np.concatenate(b.vchunks)
            verts["skin_index"][off:off + n] = skin
            b.vchunks = [verts]
    if not pl:
        rng = np.random.default_rng(light_seed)
        for _ in range(5):
            raw = np.zeros((), T.LIGHT)
            raw["color"] = (1, 1, 1, 1)
            raw["transform"] = ((rng.random(4) - 0.5) * 2.0 * 10.0).astype(np.float32)
            raw["kind"] = 1
            raw["range"] = np.inf
            raw["intensity"] = 0.0
            pl.append(raw)
    if not dl:
        dl.append(T.default_dir_light())
    inst = state.instances()
    sd = b.finish(instances=inst, dlights=np.array(dl, T.LIGHT), plights=np.array(pl, T.LIGHT),
                  textures=_textures(doc, bufs, base),
                  camera=dict(eye=(0.0, 0.0, 12.0), direction=(0.0, 0.0, -1.0), fov_deg=60.0),
                  name=os.path.basename(path))
    sd.gltf = state  # animation state: sd.gltf.animate(t), .instances(), .skins()
    return sd


class GltfScene:
    """Node tree, animations and skins of a loaded glTF (scene_graph.rs,
    animation.rs, skinning.rs): animate(t) moves the animated nodes,
    instances() gives the TLAS instances for gbrt_tlas_update and skins() the
    joint matrices for gbrt_skin_and_refit."""

    def __init__(self, doc, bufs, local, roots, norm, mesh_geos):
        self.nodes = doc.get("nodes", [])
        self.local = [m.copy() for m in local]
        self.roots, self.norm, self.mesh_geos = roots, norm, mesh_geos
        self.order = []  # depth-first pre-order from the roots
        stack = list(reversed(roots))
        while stack:
            i = stack.pop()
            self.order.append(i)
            stack.extend(reversed(self.nodes[i].get("children", [])))
        self.trs = {}
        self.channels = []
        for an in doc.get("animations", []):
            for ch in an.get("channels", []):
                tgt = ch.get("target", {})
                path = tgt.get("path")
                if "node" not in tgt or path not in ("translation", "rotation", "scale"):
                    continue  # morph weights are ignored, as in the reference
                smp = an["samplers"][ch["sampler"]]
                times = _accessor(doc, bufs, smp["input"]).reshape(-1).astype(np.float64)
                vals = _accessor(doc, bufs, smp["output"]).astype(np.float64)
                self.channels.append(_Channel(tgt["node"], path, times, vals, smp.get("interpolation", "LINEAR")))
        self.skin_joints = []
        for sk in doc.get("skins", []):
            joints = sk["joints"]
            ibm = (_accessor(doc, bufs, sk["inverseBindMatrices"]).reshape(-1, 4, 4).transpose(0, 2, 1)
                   if "inverseBindMatrices" in sk else np.tile(np.eye(4), (len(joints), 1, 1)))
            self.skin_joints.append((joints, ibm.astype(np.float64)))

    def world(self):
        w = {}

        def rec(i, parent):
            w[i] = parent @ self.local[i]
            for c in self.nodes[i].get("children", []):
                rec(c, w[i])
        for r in self.roots:
            rec(r, self.norm)
        return w

    def animate(self, t):
        """Applies every channel at time t (seconds)."""
        for ch in self.channels:
            i = ch.node
            if i not in self.trs:
                self.trs[i] = list(_decompose(self.local[i]))
            k = {"translation": 0, "rotation": 1, "scale": 2}[ch.path]
            self.trs[i][k] = np.asarray(ch.sample(t), np.float64)
        for i, (tt, q, sc) in self.trs.items():
            self.local[i] = _trs_matrix(tt, q, sc)

    def instances(self):
        w = self.world()
        geos, xfs = [], []
        for i in self.order:
            nd = self.nodes[i]
            if "mesh" not in nd:
                continue
            xf = np.eye(4) if "skin" in nd else w[i]
            for g in self.mesh_geos[nd["mesh"]]:
                geos.append(g)
                xfs.append(xf[:3, :4].astype(np.float32).reshape(12))
        return identity_instances(geos, transforms=xfs)

    def skins(self):
        w = self.world()
        out = np.zeros(max(1, len(self.skin_joints)), T.SKIN)
        for k, (joints, ibm) in enumerate(self.skin_joints):
            for j, node in enumerate(joints[:256]):
                out[k]["joints"][j] = (w[node] @ ibm[j]).T.reshape(16).astype(np.float32)
        return out


_FACE_ALIASES = {"posx": 0, "negx": 1, "posy": 2, "negy": 3, "posz": 4, "negz": 5,
                 "right": 0, "left": 1, "top": 2, "bottom": 3, "front": 4, "back": 5}


def load_cubemap(directory):
    """Six square PNG or JPEG faces named like the reference's skybox
    directories (posx/negx/... or right/left/top/bottom/front/back, cubumap.rs
    Face; the reference ships assets/skyboxs/Yokohama/*.jpg) -> (face size,
    RGBA8 bytes in +X, -X, +Y, -Y, +Z, -Z order) for gbrt_skybox_set."""
    from .jpeg import read_jpeg
    from .png import read_png
    faces = [None] * 6
    for name in os.listdir(directory):
        stem, ext = os.path.splitext(name)
        if stem not in _FACE_ALIASES:
            continue
        if ext.lower() == ".png":
            faces[_FACE_ALIASES[stem]] = read_png(open(os.path.join(directory, name), "rb").read())
        elif ext.lower() in (".jpg", ".jpeg"):
            faces[_FACE_ALIASES[stem]] = read_jpeg(open(os.path.join(directory, name), "rb").read())
    if any(f is None for f in faces):
        raise ValueError("a cubemap needs six PNG or JPEG faces")
    size = faces[0].shape[0]
    if any(f.shape[:2] != (size, size) for f in faces):
        raise ValueError("cubemap faces must be square and of one size")
    return size, np.concatenate([f.reshape(-1) for f in faces])
