"""Scenes that exercise every shading path of the reference hit group, and
a skinned mesh.

* material_zoo(): the Cornell box with nine spheres, one per material kind
  the shaders distinguish (RayTracing.rchit:166-336, RayTracing.rahit:44-104):
  sRGB base-colour texture, metallic-roughness texture, normal map with
  tangents, emissive texture, MASK alpha from an RGBA16F texture, BLEND alpha
  from vertex colour, specular-glossiness workflow with textures,
  transmission with a volume (IOR, attenuation) and KHR_materials_specular;
  plus an unlit quad, point lights, a directional light and a skybox.
* skinned_tube(): a tube of `rings x segments` quads skinned to a chain of
  bones (AnimationCompute.comp), with bone matrices for an animation time.
"""
import math

import numpy as np

from . import types as T
from .scenes import GeoBuilder, _cornell_into, _icosphere, lambert, point_light, CORNELL_EYE, CORNELL_DIR


def _sphere(subdiv, center, radius):
    v, f = _icosphere(subdiv)
    pos = v * radius + np.asarray(center)
    nrm = v.copy()
    u = np.arctan2(v[:, 2], v[:, 0]) / (2 * np.pi) + 0.5
    w = np.arccos(np.clip(v[:, 1], -1, 1)) / np.pi
    phi = np.arctan2(v[:, 2], v[:, 0])
    tangent = np.stack([-np.sin(phi), np.zeros_like(phi), np.cos(phi), np.ones_like(phi)], 1)
    return pos, nrm, np.stack([u * 3.0, w * 2.0], 1), tangent, f


def _tex_rgba8(rng, n, fmt=T.TEX_RGBA8_SRGB, wrap=T.WRAP_REPEAT, alpha=None):
    img = rng.integers(0, 256, (n, n, 4)).astype(np.uint8)
    if alpha is not None:
        img[..., 3] = alpha
    return (n, n, fmt, wrap, wrap, img)


def material_zoo(seed=5, subdiv=3):
    rng = np.random.default_rng(seed)
    b = GeoBuilder()
    _cornell_into(b)
    tex = []

    def add_tex(t):
        tex.append(t)
        return len(tex) - 1

    t_base = add_tex(_tex_rgba8(rng, 16))
    t_mr = add_tex(_tex_rgba8(rng, 8, T.TEX_RGBA8_UNORM, T.WRAP_MIRRORED_REPEAT))
    nm = np.zeros((8, 8, 4), np.uint8)  # normal map around +z
    nm[..., 0] = rng.integers(100, 156, (8, 8))
    nm[..., 1] = rng.integers(100, 156, (8, 8))
    nm[..., 2] = 240
    nm[..., 3] = 255
    t_nrm = add_tex((8, 8, T.TEX_RGBA8_UNORM, T.WRAP_REPEAT, T.WRAP_CLAMP_TO_EDGE, nm))
    t_emis = add_tex(_tex_rgba8(rng, 4))
    mask = np.ones((32, 32, 4), np.float16)
    mask[..., 3] = rng.random((32, 32)).astype(np.float16)
    t_mask = add_tex((32, 32, T.TEX_RGBA16F, T.WRAP_REPEAT, T.WRAP_REPEAT, mask.view(np.uint16)))
    t_sgd = add_tex(_tex_rgba8(rng, 8))
    t_sgs = add_tex(_tex_rgba8(rng, 8, T.TEX_RGBA8_SRGB))
    t_spec = add_tex(_tex_rgba8(rng, 8, T.TEX_RGBA8_UNORM))

    mats = []
    m = lambert((0.8, 0.8, 0.8))
    m["base_color_texture"] = (t_base, 0)
    m["roughness_factor"] = 0.6
    mats.append(m)
    m = T.default_material()
    m["metallic_roughness_texture"] = (t_mr, 0)
    m["base_color"] = (0.9, 0.7, 0.3, 1.0)
    mats.append(m)
    m = lambert((0.6, 0.6, 0.9))
    m["normal_texture"] = (t_nrm, 0)
    m["roughness_factor"] = 0.4
    mats.append(m)
    m = lambert((0.3, 0.3, 0.3), emissive=(2.0, 1.5, 1.0))
    m["emissive_texture"] = (t_emis, 0)
    mats.append(m)
    m = lambert((0.2, 0.8, 0.3))
    m["alpha_mode"] = T.ALPHA_MASK
    m["alpha_cutoff"] = 0.45
    m["base_color_texture"] = (t_mask, 0)
    mats.append(m)
    m = lambert((0.8, 0.2, 0.6))
    m["alpha_mode"] = T.ALPHA_BLEND
    m["base_color"][3] = 0.6
    mats.append(m)
    m = T.default_material()
    m["workflow"] = 1
    m["sg_diffuse_factor"] = (0.7, 0.5, 0.4, 1.0)
    m["sg_specular_glossiness_factor"] = (0.3, 0.3, 0.35, 0.6)
    m["sg_diffuse_texture"] = (t_sgd, 0)
    m["sg_specular_glossiness_texture"] = (t_sgs, 0)
    mats.append(m)
    m = lambert((0.9, 0.95, 1.0))
    m["roughness_factor"] = 0.05
    m["transmission_exist"] = 1
    m["transmission_factor"] = 0.9
    m["volume_exists"] = 1
    m["ior"] = 1.45
    m["attenuation_color"] = (0.8, 0.9, 0.7)
    m["attenuation_distance"] = 0.5
    mats.append(m)
    m = lambert((0.5, 0.4, 0.9))
    m["metallic_factor"] = 0.2
    m["roughness_factor"] = 0.3
    m["specular_exist"] = 1
    m["specular_factor"] = 0.7
    m["specular_color_factor"] = (1.0, 0.6, 0.6, 0.0)
    m["specular_texture"] = (t_spec, 0)
    m["specular_color_texture"] = (t_spec, 0)
    mats.append(m)
    ids = [b.add_material(x) for x in mats]
    centers = [(-0.6, -0.7, 0.2), (0.0, -0.7, 0.5), (0.6, -0.7, 0.2), (-0.6, 0.0, 0.0), (0.0, 0.05, 0.3),
               (0.6, 0.0, 0.0), (-0.5, 0.6, -0.2), (0.1, 0.55, 0.1), (0.6, 0.6, -0.3)]
    for c, mid in zip(centers, ids):
        pos, nrm, uv, tan, f = _sphere(subdiv, c, 0.22)
        col = np.ones((len(pos), 4))
        col[:, 3] = 0.5 + 0.5 * np.abs(nrm[:, 1])
        b.add_mesh(pos.astype(np.float32), f, mid, nrm.astype(np.float32), uv=uv.astype(np.float32),
                   tangent=tan.astype(np.float32), color=col.astype(np.float32))
    um = lambert((0.9, 0.1, 0.1))
    um["unlit"] = 1
    uid = b.add_material(um)
    quad = np.array([(-0.95, 0.2, -0.99), (-0.65, 0.2, -0.99), (-0.65, 0.5, -0.99), (-0.95, 0.5, -0.99)], np.float32)
    b.add_mesh(quad, np.array([[0, 1, 2], [0, 2, 3]]), uid, np.tile([0, 0, 1.0], (4, 1)).astype(np.float32))
    plights = [point_light((-0.4, 0.85, 0.4), (1.0, 0.9, 0.8), 2.5), point_light((0.5, 0.2, 0.7), (0.7, 0.8, 1.0), 1.5),
               point_light((0.0, -0.5, 0.8), (1.0, 1.0, 1.0), 1.0)]
    d = T.default_dir_light()
    d["transform"] = (0.2, -0.9, -0.4, 0.0)
    d["intensity"] = 1.5
    sky = (8, rng.integers(0, 256, 6 * 8 * 8 * 4).astype(np.uint8))
    return b.finish(plights=np.array(plights, T.LIGHT), dlights=np.array([d], T.LIGHT), textures=tex, skybox=sky,
                    camera=dict(eye=CORNELL_EYE, direction=CORNELL_DIR, fov_deg=40.0), name="material_zoo")


def skinned_tube(rings=32, segments=24, bones=8, seed=7):
    """A vertical tube (rings x segments quads) weighted to a chain of
    `bones` bones, inside the Cornell box."""
    b = GeoBuilder()
    _cornell_into(b)
    m = b.add_material(lambert((0.7, 0.5, 0.3)))
    pos, nrm, joints, weights = [], [], [], []
    for r in range(rings + 1):
        y = -0.8 + 1.4 * r / rings
        bf = (y + 0.8) / 1.4 * (bones - 1)
        j0 = min(int(bf), bones - 2)
        t = bf - j0
        for s in range(segments):
            a = 2 * np.pi * s / segments
            pos.append((0.2 * np.cos(a), y, 0.2 * np.sin(a)))
            nrm.append((np.cos(a), 0.0, np.sin(a)))
            joints.append((j0, j0 + 1, 0, 0))
            weights.append((1.0 - t, t, 0.0, 0.0))
    idx = []
    for r in range(rings):
        for s in range(segments):
            a, c = r * segments + s, r * segments + (s + 1) % segments
            idx += [(a, c, a + segments), (c, c + segments, a + segments)]
    base = b.add_vertices(np.array(pos, np.float32), np.array(nrm, np.float32), skin_index=0,
                          joints=np.array(joints, np.uint32), weights=np.array(weights, np.float32))
    b.add_geometry(base, len(pos), np.array(idx), m)
    sd = b.finish(camera=dict(eye=CORNELL_EYE, direction=CORNELL_DIR, fov_deg=40.0), name="skinned_tube")
    sd.bones = bones
    return sd


def bone_matrices(bones, time, nskins=1):
    """Skin matrices (world x inverse bind, skinning.rs:79-81) of a chain of
    bones bending about z: bone k rotates by 0.25*sin(time + k) about its own
    rest height.  Column-major mat4s, 256 per skin."""
    skins = np.zeros(nskins, T.SKIN)
    for si in range(nskins):
        for k in range(256):
            M = np.eye(4)
            if k < bones:
                y0 = -0.8 + 1.4 * k / max(bones - 1, 1)
                a = 0.25 * math.sin(time + k + si)
                R = np.array([[math.cos(a), -math.sin(a), 0, 0], [math.sin(a), math.cos(a), 0, 0], [0, 0, 1, 0],
                              [0, 0, 0, 1]])
                Tm = np.eye(4)
                Tm[1, 3] = y0
                Ti = np.eye(4)
                Ti[1, 3] = -y0
                M = Tm @ R @ Ti
            skins[si]["joints"][k] = M.T.reshape(16).astype(np.float32)  # column-major
    return skins
