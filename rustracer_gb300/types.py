"""numpy mirrors of the C-ABI structs in include/gbrt.h.

Each dtype has the byte layout of the reference's #[repr(C)] type it mirrors
(sizes asserted below), so arrays of them can be handed to the library as raw
pointers:

* VERTEX      crates/libs/asset_loader/src/geometry.rs:10-22      (128 B)
* PRIMINFO    crates/libs/asset_loader/src/geometry.rs:65-73      (16 B)
* MATERIAL    crates/libs/asset_loader/src/material.rs:130-160    (256 B)
* LIGHT       crates/libs/asset_loader/src/light.rs:62-71         (48 B)
* UBO         crates/examples/gltf_viewer/src/ubo.rs:3-31         (324 B)
* INSTANCE    VkAccelerationStructureInstanceKHR as filled by
              crates/libs/asset_loader/src/acceleration_structures.rs:157-167 (64 B)
"""
import numpy as np

VERTEX = np.dtype([
    ("pos", "<f4", 4), ("normal", "<f4", 4), ("tangent", "<f4", 4), ("color", "<f4", 4),
    ("weights", "<f4", 4), ("joints", "<u4", 4), ("uv0", "<f4", 2), ("uv1", "<f4", 2),
    ("skin_index", "<i4"), ("_pad", "<u4", 3),
])

PRIMINFO = np.dtype([("v_offset", "<u4"), ("i_offset", "<u4"), ("material_id", "<u4"), ("skin_id", "<u4")])

TEXINFO = np.dtype([("index", "<i4"), ("coord", "<i4")])

MATERIAL = np.dtype([
    ("alpha_mode", "<u4"), ("alpha_cutoff", "<f4"), ("double_sided", "<u4"), ("workflow", "<u4"),
    ("_pad0", "<f4", 2), ("base_color_texture", TEXINFO), ("base_color", "<f4", 4),
    ("metallic_factor", "<f4"), ("roughness_factor", "<f4"), ("metallic_roughness_texture", TEXINFO),
    ("normal_texture", TEXINFO), ("emissive_texture", TEXINFO), ("emissive_factor", "<f4", 4),
    ("occlusion_texture", TEXINFO), ("ior", "<f4"), ("unlit", "<u4"),
    ("transmission_texture", TEXINFO), ("transmission_factor", "<f4"), ("transmission_exist", "<u4"),
    ("attenuation_color", "<f4", 3), ("thickness_factor", "<f4"), ("thickness_texture", TEXINFO),
    ("attenuation_distance", "<f4"), ("volume_exists", "<u4"),
    ("specular_texture", TEXINFO), ("specular_color_texture", TEXINFO), ("specular_color_factor", "<f4", 4),
    ("specular_factor", "<f4"), ("specular_exist", "<u4"), ("_pad1", "<u4", 2),
    ("sg_diffuse_factor", "<f4", 4), ("sg_specular_glossiness_factor", "<f4", 4),
    ("sg_diffuse_texture", TEXINFO), ("sg_specular_glossiness_texture", TEXINFO),
])

LIGHT = np.dtype([("color", "<f4", 4), ("transform", "<f4", 4), ("kind", "<u4"), ("range", "<f4"),
                  ("intensity", "<f4"), ("_pad", "<u4")])

UBO = np.dtype([
    ("model_view", "<f4", 16), ("projection", "<f4", 16), ("model_view_inverse", "<f4", 16),
    ("projection_inverse", "<f4", 16), ("aperture", "<f4"), ("focus_distance", "<f4"), ("fov_angle", "<f4"),
    ("orthographic_fov_dis", "<f4"), ("heatmap_scale", "<f4"), ("total_number_of_samples", "<u4"),
    ("number_of_samples", "<u4"), ("number_of_bounces", "<u4"), ("random_seed", "<u4"), ("has_sky", "<u4"),
    ("antialiasing", "<u4"), ("mapping", "<u4"), ("frame_count", "<u4"), ("debug", "<u4"),
    ("fully_opaque", "<u4"), ("exposure", "<f4"), ("tone_mapping_mode", "<u4"),
])

INSTANCE = np.dtype([("transform", "<f4", 12), ("custom_index_and_mask", "<u4"),
                     ("sbt_offset_and_flags", "<u4"), ("blas_handle", "<u8")])

GEO_RANGE = np.dtype([("geo_id", "<u4"), ("v_len", "<u4"), ("i_len", "<u4"), ("opaque", "<u4")])

RAY = np.dtype([("org", "<f4", 3), ("tmin", "<f4"), ("dir", "<f4", 3), ("tmax", "<f4")])

HIT = np.dtype([("t", "<f4"), ("u", "<f4"), ("v", "<f4"), ("instance_id", "<u4"), ("primitive_id", "<u4"),
                ("custom_index", "<u4")])

STATS = np.dtype([("rays_total", "<u8"), ("rays_camera", "<u8"), ("rays_extension", "<u8"),
                  ("rays_shadow", "<u8"), ("hits_shaded", "<u8"), ("device_ms", "<f8"),
                  ("kernel_launches", "<u4"), ("device_status", "<u4"), ("node_visits", "<u8"),
                  ("tri_tests", "<u8"), ("stage_ms", "<f8", 4)])

SKIN = np.dtype([("joints", "<f4", (256, 16))])

JOB_INFO = np.dtype([("state", "<u4"), ("status", "<i4"), ("queue_ms", "<f8"), ("latency_ms", "<f8"),
                     ("stats", STATS)])

for _dt, _size in ((VERTEX, 128), (PRIMINFO, 16), (MATERIAL, 256), (LIGHT, 48), (UBO, 324),
                   (INSTANCE, 64), (GEO_RANGE, 16), (RAY, 32), (HIT, 24), (STATS, 104), (SKIN, 16384),
                   (JOB_INFO, 128)):
    assert _dt.itemsize == _size, (_dt, _dt.itemsize, _size)
assert MATERIAL.fields["base_color"][1] == 32
assert MATERIAL.fields["attenuation_color"][1] == 128
assert MATERIAL.fields["specular_texture"][1] == 160
assert MATERIAL.fields["sg_diffuse_factor"][1] == 208

# Texture formats / wrap modes (include/gbrt.h)
TEX_RGBA8_UNORM, TEX_RGBA8_SRGB, TEX_RGBA16F, TEX_RGBA32F = 0, 1, 2, 3
WRAP_REPEAT, WRAP_CLAMP_TO_EDGE, WRAP_MIRRORED_REPEAT = 0, 1, 2

# Ray flags
RAY_OPAQUE = 0x01
RAY_TERMINATE_ON_FIRST = 0x04

# Alpha modes as the shaders compare them (RayTracing.rahit:39-41)
ALPHA_OPAQUE, ALPHA_MASK, ALPHA_BLEND = 1, 2, 3

# Mappings (shaders/lib/RayTracingCommons.glsl:139-150)
MAP_RENDER, MAP_HEAT, MAP_INSTANCE, MAP_TRIANGLE, MAP_DISTANCE, MAP_ALBEDO = 0, 1, 2, 3, 4, 5


def default_material():
    """MaterialRaw with the defaults the reference writes for a glTF material
    that sets nothing (material.rs:162-190, 203-213, 314-325): alpha_cutoff
    0.5, ior 1.5, volume attenuation colour 1 / distance f32::MAX, specular
    factor 1 and colour 1, texture indices -1 (tex_coord -1)."""
    m = np.zeros((), MATERIAL)
    m["alpha_mode"] = ALPHA_OPAQUE
    m["alpha_cutoff"] = 0.5
    for f in ("base_color_texture", "metallic_roughness_texture", "normal_texture", "emissive_texture",
              "occlusion_texture", "transmission_texture", "thickness_texture", "specular_texture",
              "specular_color_texture", "sg_diffuse_texture", "sg_specular_glossiness_texture"):
        m[f]["index"] = -1
        m[f]["coord"] = -1
    m["base_color"] = (1, 1, 1, 1)
    m["metallic_factor"] = 1.0      # glTF default
    m["roughness_factor"] = 1.0
    m["ior"] = 1.5
    m["attenuation_color"] = (1, 1, 1)
    m["attenuation_distance"] = np.finfo(np.float32).max
    m["specular_color_factor"] = (1, 1, 1, 1)
    m["specular_factor"] = 1.0
    return m


def default_dir_light():
    """LightRaw::default() (light.rs:115-125): white, transform 1, kind
    directional, intensity 0 -- what the reference adds when a scene has no
    directional light (scene_graph.rs:75-79)."""
    l = np.zeros((), LIGHT)
    l["color"] = (1, 1, 1, 1)
    l["transform"] = (1, 1, 1, 1)
    l["kind"] = 0
    l["range"] = np.inf
    l["intensity"] = 0.0
    return l


IDENTITY34 = np.array([1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0], np.float32)
