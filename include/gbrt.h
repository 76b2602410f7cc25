/*
 * gbrt.h — C ABI of the GB300-native ray-tracing core.
 *
 * This header is the drop-in boundary for rustracer's Vulkan ray-tracing
 * pipeline (KaminariOS/rustracer).  Every struct is plain C with fixed sizes so
 * that a Rust host can mirror it with #[repr(C)]; every function returns an
 * int status (0 = GBRT_OK, negative = GBRT_E_*), never throws and never
 * aborts.  gbrt_last_error() gives the message of the last failure on a
 * context.  Host arrays passed in stay owned by the caller; the library copies
 * what it needs into device memory.
 *
 * Threading: a gbrt_ctx (and everything created from it) is used from one host
 * thread at a time, except the job API (gbrt_job_*), which is internally
 * locked.  All device work of a context runs on the context's CUDA stream.
 *
 * Citations below are paths inside the reference repository.
 */
#ifndef GBRT_H
#define GBRT_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------ */
/* Status codes                                                             */
/* ------------------------------------------------------------------------ */
#define GBRT_OK               0
#define GBRT_E_INVALID       -1  /* bad argument, size or state */
#define GBRT_E_CUDA          -2  /* a CUDA runtime call failed */
#define GBRT_E_OOM           -3  /* device allocation failed */
#define GBRT_E_DEVICE_LIMIT  -4  /* a kernel hit an iteration/stack/queue cap */
#define GBRT_E_NOT_BUILT     -5  /* render/trace before blas/tlas build */
#define GBRT_E_NO_DEVICE     -6  /* no CUDA device, or the library was built without it */
#define GBRT_E_BUSY          -7  /* job queue full / admission refused */
#define GBRT_E_CANCELLED     -8  /* the job was cancelled (gbrt_job_cancel) */

/* ------------------------------------------------------------------------ */
/* Data contract: byte-for-byte mirrors of the reference's #[repr(C)] types  */
/* ------------------------------------------------------------------------ */

/* Vertex, 128 B.  crates/libs/asset_loader/src/geometry.rs:10-22 and
 * shaders/lib/RayTracingCommons.glsl:54-63.  pos.w is 0 on upload
 * (geometry.rs:166); only pos.xyz is used by the BLAS build
 * (acceleration_structures.rs:35-40, stride 128). */
typedef struct gbrt_vertex {
    float    pos[4];
    float    normal[4];
    float    tangent[4];
    float    color[4];
    float    weights[4];
    uint32_t joints[4];
    float    uv0[2];
    float    uv1[2];
    int32_t  skin_index;
    uint32_t _pad[3];
} gbrt_vertex;

/* PrimInfo, 16 B: one per geometry (glTF primitive).  geometry.rs:65-73,
 * RayTracingCommons.glsl:47-52. */
typedef struct gbrt_priminfo {
    uint32_t v_offset;
    uint32_t i_offset;
    uint32_t material_id;
    uint32_t skin_id;
} gbrt_priminfo;

/* TextureInfo, 8 B.  material.rs:11-17; index -1 = no texture.  The
 * reference offsets texture indices by +1 for its dummy texture 0
 * (material.rs:36); the index here is the slot in the texture array given
 * to gbrt_scene_create, which the host fills the same way. */
typedef struct gbrt_texture_info {
    int32_t index;
    int32_t coord;
} gbrt_texture_info;

/* MaterialRaw, 256 B.  material.rs:130-160, shaders/lib/Material.glsl:51-73.
 * alpha_mode: 1 = OPAQUE, 2 = MASK, 3 = BLEND as the shaders compare it
 * (RayTracing.rahit:39-41).  workflow: 0 metallic-roughness, 1 specular-
 * glossiness (material.rs:327-330). */
typedef struct gbrt_material_raw {
    uint32_t alpha_mode;                  /*   0 */
    float    alpha_cutoff;                /*   4 */
    uint32_t double_sided;                /*   8 */
    uint32_t workflow;                    /*  12 */
    float    _pad0[2];                    /*  16 */
    gbrt_texture_info base_color_texture; /*  24 */
    float    base_color[4];               /*  32 */
    float    metallic_factor;             /*  48 */
    float    roughness_factor;            /*  52 */
    gbrt_texture_info metallic_roughness_texture; /* 56 */
    gbrt_texture_info normal_texture;     /*  64 */
    gbrt_texture_info emissive_texture;   /*  72 */
    float    emissive_factor[4];          /*  80 */
    gbrt_texture_info occlusion_texture;  /*  96 */
    float    ior;                         /* 104 */
    uint32_t unlit;                       /* 108 */
    /* TransmissionInfo (material.rs:250-256) */
    gbrt_texture_info transmission_texture; /* 112 */
    float    transmission_factor;         /* 120 */
    uint32_t transmission_exist;          /* 124 */
    /* VolumeInfo (material.rs:193-201) */
    float    attenuation_color[3];        /* 128 */
    float    thickness_factor;            /* 140 */
    gbrt_texture_info thickness_texture;  /* 144 */
    float    attenuation_distance;        /* 152 */
    uint32_t volume_exists;               /* 156 */
    /* SpecularInfo (material.rs:290-299) */
    gbrt_texture_info specular_texture;   /* 160 */
    gbrt_texture_info specular_color_texture; /* 168 */
    float    specular_color_factor[4];    /* 176 */
    float    specular_factor;             /* 192 */
    uint32_t specular_exist;              /* 196 */
    uint32_t _pad1[2];                    /* 200 */
    /* SpecularGlossiness (material.rs:268-276) */
    float    sg_diffuse_factor[4];        /* 208 */
    float    sg_specular_glossiness_factor[4]; /* 224: rgb specular, a glossiness */
    gbrt_texture_info sg_diffuse_texture; /* 240 */
    gbrt_texture_info sg_specular_glossiness_texture; /* 248 */
} gbrt_material_raw;

/* LightRaw, 48 B.  crates/libs/asset_loader/src/light.rs:62-71,
 * shaders/lib/PunctualLight.glsl:8-15.  kind 0 directional (transform =
 * direction), 1 point (transform = position); spot lights are uploaded as
 * point lights (light.rs:51-57). */
typedef struct gbrt_light_raw {
    float    color[4];
    float    transform[4];
    uint32_t kind;
    float    range;
    float    intensity;
    uint32_t _pad;
} gbrt_light_raw;

/* UniformBufferObject, 324 B.  crates/examples/gltf_viewer/src/ubo.rs:3-31,
 * shaders/lib/UniformBufferObject.glsl:3-30.  Matrices are column-major. */
typedef struct gbrt_ubo {
    float    model_view[16];
    float    projection[16];
    float    model_view_inverse[16];
    float    projection_inverse[16];
    float    aperture;
    float    focus_distance;
    float    fov_angle;
    float    orthographic_fov_dis;
    float    heatmap_scale;
    uint32_t total_number_of_samples;
    uint32_t number_of_samples;
    uint32_t number_of_bounces;
    uint32_t random_seed;
    uint32_t has_sky;
    uint32_t antialiasing;
    uint32_t mapping;
    uint32_t frame_count;
    uint32_t debug;
    uint32_t fully_opaque;
    float    exposure;
    uint32_t tone_mapping_mode;
} gbrt_ubo;

/* Skin: 256 column-major joint matrices, 16 KiB.
 * crates/libs/asset_loader/src/skinning.rs:9-10,53-57,
 * shaders/AnimationCompute.comp:4-7. */
#define GBRT_MAX_JOINTS 256
typedef struct gbrt_skin_raw {
    float joints[GBRT_MAX_JOINTS][16];
} gbrt_skin_raw;

/* TLAS instance, 64 B, laid out like VkAccelerationStructureInstanceKHR as
 * the reference fills it (acceleration_structures.rs:153-167): row-major 3x4
 * object-to-world transform, custom index (= geometry id) in the low 24 bits
 * and the 8-bit mask in the high bits; sbt offset 24 bits + flags 8 bits;
 * blas_handle = the geometry id whose BLAS this instance references. */
typedef struct gbrt_instance {
    float    transform[12];
    uint32_t custom_index_and_mask;
    uint32_t sbt_offset_and_flags;
    uint64_t blas_handle;
} gbrt_instance;

/* One BLAS input per geometry: the range of vertices/indices it owns
 * (GeoBuilder::len / offsets, geometry.rs:36-40) and whether its material is
 * OPAQUE (geometry.rs:56-58 -> GeometryFlagsKHR::OPAQUE,
 * acceleration_structures.rs:53-57). */
typedef struct gbrt_geo_range {
    uint32_t geo_id;
    uint32_t v_len;
    uint32_t i_len;
    uint32_t opaque;
} gbrt_geo_range;

/* Texture image.  The reference decodes every texture to RGBA8 and samples
 * it bilinearly without mips (crates/libs/vulkan/src/image.rs:48,102);
 * colour textures are sRGB, the rest linear (material.rs:102-128). */
#define GBRT_TEX_RGBA8_UNORM 0
#define GBRT_TEX_RGBA8_SRGB  1
#define GBRT_TEX_RGBA16F     2
#define GBRT_TEX_RGBA32F     3  /* linear float texels (HDR skyboxes; no reference counterpart) */
#define GBRT_WRAP_REPEAT          0
#define GBRT_WRAP_CLAMP_TO_EDGE   1
#define GBRT_WRAP_MIRRORED_REPEAT 2
typedef struct gbrt_texture_desc {
    uint32_t    width;
    uint32_t    height;
    uint32_t    format;   /* GBRT_TEX_* */
    uint32_t    wrap_s;   /* GBRT_WRAP_* */
    uint32_t    wrap_t;
    uint32_t    _pad;
    const void* data;     /* width*height texels, row-major, host memory */
} gbrt_texture_desc;

/* Ray query input / output for gbrt_trace_rays*.  A ray is 32 B. */
typedef struct gbrt_ray {
    float org[3];
    float tmin;
    float dir[3];
    float tmax;
} gbrt_ray;

/* instance_id = ~0u on a miss. */
typedef struct gbrt_hit {
    float    t;
    float    u;           /* barycentric weight of vertex 1 (gl HitAttributes.x) */
    float    v;           /* barycentric weight of vertex 2 */
    uint32_t instance_id; /* gl_InstanceID */
    uint32_t primitive_id;/* gl_PrimitiveID */
    uint32_t custom_index;/* gl_InstanceCustomIndexEXT = geometry id */
} gbrt_hit;

/* Ray flags for gbrt_trace_rays* (subset of gl_RayFlags*). */
#define GBRT_RAY_OPAQUE              0x01u  /* skip any-hit alpha tests */
#define GBRT_RAY_TERMINATE_ON_FIRST  0x04u  /* shadow/occlusion query */

/* Per-call statistics. */
typedef struct gbrt_stats {
    uint64_t rays_total;      /* camera + extension + shadow segments */
    uint64_t rays_camera;
    uint64_t rays_extension;
    uint64_t rays_shadow;
    uint64_t hits_shaded;
    double   device_ms;       /* CUDA-event time of the device work */
    uint32_t kernel_launches;
    uint32_t device_status;   /* 0, or GBRT_STATUS_* bits reported by kernels */
    uint64_t node_visits;     /* BVH inner nodes visited by all traversals */
    uint64_t tri_tests;       /* ray-triangle tests */
    double   stage_ms[4];     /* with GBRT_RENDER_STAGE_TIMING (wavefront form):
                                 extend, shade, shadow, other kernels */
} gbrt_stats;

#define GBRT_STATUS_STACK_OVERFLOW 0x1u
#define GBRT_STATUS_ITER_LIMIT     0x2u
#define GBRT_STATUS_QUEUE_OVERFLOW 0x4u

/* Render options for gbrt_render_ex. */
#define GBRT_MODE_AUTO       0
#define GBRT_MODE_MEGAKERNEL 1
#define GBRT_MODE_WAVEFRONT  2
#define GBRT_RENDER_STAGE_TIMING 0x1u  /* gbrt_render_opts.flags: CUDA-event time per stage */
/* gbrt_render_opts.flags: queue the frame on the context stream and return
 * at once (the non-blocking form of gbrt_render).  out_rgba8, if given, is
 * written when the stream reaches the frame: keep it valid and read it after
 * gbrt_sync (page-locked memory lets the copy run asynchronously; a pageable
 * buffer makes this call wait for it).  stats gets only kernel_launches; the
 * debug outputs and stage timing are not available.  gbrt_sync reports a
 * traversal limit hit by any asynchronous frame since the last gbrt_sync. */
#define GBRT_RENDER_ASYNC 0x2u
typedef struct gbrt_render_opts {
    uint32_t mode;            /* GBRT_MODE_* */
    uint32_t flags;           /* GBRT_RENDER_STAGE_TIMING, GBRT_RENDER_ASYNC or 0 */
    /* Optional debug outputs (host memory, may be NULL):
     * sample_radiance: width*height*number_of_samples*3 floats, per-sample
     *                  path radiance, laid out [pixel][sample][rgb];
     * primary_hits:    width*height*number_of_samples primary-ray hits. */
    float*    sample_radiance;
    gbrt_hit* primary_hits;
} gbrt_render_opts;

/* ------------------------------------------------------------------------ */
/* Opaque handles                                                           */
/* ------------------------------------------------------------------------ */
typedef struct gbrt_ctx   gbrt_ctx;
typedef struct gbrt_scene gbrt_scene;
typedef struct gbrt_accum gbrt_accum;

/* ------------------------------------------------------------------------ */
/* Context                                                                  */
/* ------------------------------------------------------------------------ */

/* Creates a context on CUDA device `device` with its own stream.  Replaces
 * the Vulkan Context creation in crates/libs/app/src/lib.rs:272-292. */
int gbrt_ctx_create(int device, gbrt_ctx** out);
int gbrt_ctx_destroy(gbrt_ctx* ctx);
/* Message of the last failed call on ctx ("" if none).  ctx may be NULL for
 * errors of gbrt_ctx_create. */
const char* gbrt_last_error(const gbrt_ctx* ctx);
/* Free / total device memory as seen by this context. */
int gbrt_ctx_mem_info(gbrt_ctx* ctx, uint64_t* free_bytes, uint64_t* total_bytes);
/* Waits for all work queued on the context's stream; returns
 * GBRT_E_DEVICE_LIMIT if a frame queued with GBRT_RENDER_ASYNC since the
 * last gbrt_sync hit a traversal limit. */
int gbrt_sync(gbrt_ctx* ctx);
/* Library version string, e.g. "gbrt 0.1 sm_103a". */
const char* gbrt_version(void);

/* ------------------------------------------------------------------------ */
/* Scene                                                                    */
/* ------------------------------------------------------------------------ */

/* Uploads the scene's device buffer set.  Replaces Buffers::new
 * (crates/libs/asset_loader/src/globals.rs:44-152) and the texture upload of
 * create_global (globals.rs:309-350).  ni must be a multiple of 3 for every
 * geometry's index range.  Textures may be NULL when ntex = 0. */
int gbrt_scene_create(gbrt_ctx* ctx,
                      const gbrt_vertex* vertices, uint32_t nv,
                      const uint32_t* indices, uint32_t ni,
                      const gbrt_priminfo* prims, uint32_t ngeo,
                      const gbrt_material_raw* materials, uint32_t nmat,
                      const gbrt_texture_desc* textures, uint32_t ntex,
                      gbrt_scene** out);
int gbrt_scene_destroy(gbrt_scene* scene);

/* Builds one BLAS per geometry range on the GPU (Morton LBVH).  Replaces the
 * per-primitive vkCmdBuildAccelerationStructuresKHR of create_as
 * (acceleration_structures.rs:17-76,79-111).
 *
 * flags: 0, or GBRT_BUILD_NO_FLATTEN and/or GBRT_BUILD_WIDTH4.  By default the next gbrt_tlas_build
 * flattens transformed instances into the world BVH when the flattened scene
 * has at most GBRT_FLATTEN_MAX_TRIANGLES triangles: their triangles are
 * transformed to world space once (row-major 3x4, each product and sum
 * rounded on its own) and intersected there, so every ray walks one 8-wide
 * BVH.  GBRT_BUILD_NO_FLATTEN keeps them in BLASes under a TLAS, where rays
 * are transformed to object space instead.  The two give hits that can
 * differ in the last bits of t, u, v (the oracle follows the same rule). */
#define GBRT_BUILD_NO_FLATTEN 0x1u
/* GBRT_BUILD_WIDTH4: the wide BVHs collapse to at most 4 children per node
 * (same compressed node format) instead of 8. */
#define GBRT_BUILD_WIDTH4 0x2u
#define GBRT_FLATTEN_MAX_TRIANGLES (1u << 26)
int gbrt_blas_build(gbrt_scene* scene, const gbrt_geo_range* ranges, uint32_t n,
                    uint32_t flags);

/* Builds the TLAS over instances.  Replaces create_top_as
 * (acceleration_structures.rs:136-249).  Instances whose transform is the
 * identity are merged into one world-space BVH; the others are traversed
 * two-level through their geometry's BLAS. */
int gbrt_tlas_build(gbrt_scene* scene, const gbrt_instance* instances, uint32_t n);

/* New instance transforms for an animated frame.  Replaces the reference's
 * per-frame create_top_as of animated scenes (crates/examples/gltf_viewer/
 * src/main.rs:395-402, acceleration_structures.rs:136-172).  n must equal
 * the built instance count.  When only the transforms changed (same
 * geometries, masks, custom indices and flags, and, for instances kept under
 * the TLAS, the same identity / non-identity class), the update is
 * incremental: transformed instances merged into the world BVH re-transform
 * their triangles, the binary world BVH is rebuilt with the fast Morton tree
 * and the wide one refit in place (a full build once the refit's SAH cost
 * proxy has drifted 1.3x); a TLAS is rebuilt over the instances' new world
 * boxes with the BLASes untouched.  Any other change takes a full build, as
 * gbrt_tlas_build.  Hits are the same as after gbrt_tlas_build with these
 * instances.  GBRT_E_BUSY while the context has unfinished jobs.
 * Synchronous. */
int gbrt_tlas_update(gbrt_scene* scene, const gbrt_instance* instances, uint32_t n);

/* Linear-blend skinning of every vertex with skin_index >= 0 (exactly
 * shaders/AnimationCompute.comp:14-39, dispatched by
 * crates/examples/gltf_viewer/src/compute_unit.rs:30-68), followed by a
 * bottom-up refit of the BVHs that hold skinned geometry.  The reference
 * does a full BLAS+TLAS rebuild instead (main.rs:383-404). */
int gbrt_skin_and_refit(gbrt_scene* scene, const gbrt_skin_raw* skins, uint32_t nskin);

/* Directional and point lights.  Replaces the dlights/plights buffers
 * (globals.rs:111-125) and their per-frame update (main.rs:353-374). */
int gbrt_lights_set(gbrt_scene* scene,
                    const gbrt_light_raw* dir_lights, uint32_t nd,
                    const gbrt_light_raw* point_lights, uint32_t np);

/* Skybox cubemap: 6 square RGBA8 (sRGB-encoded) faces of face_size^2 texels
 * in the order +X,-X,+Y,-Y,+Z,-Z (globals.rs:175-199).  NULL clears it. */
int gbrt_skybox_set(gbrt_scene* scene, uint32_t face_size, const uint8_t* rgba8_faces);
/* The same with the texel format given: GBRT_TEX_RGBA8_SRGB (as
 * gbrt_skybox_set) or GBRT_TEX_RGBA32F (linear floats, 16 B per texel, for
 * HDR environment maps). */
int gbrt_skybox_set_ex(gbrt_scene* scene, uint32_t face_size, const void* faces, uint32_t format);

/* ------------------------------------------------------------------------ */
/* Accumulation image                                                       */
/* ------------------------------------------------------------------------ */

/* Device-resident RGBA32F running sum, like the reference's acc_image
 * (crates/libs/app/src/lib.rs:316-326) plus its sample count. */
int gbrt_accum_create(gbrt_ctx* ctx, uint32_t width, uint32_t height, gbrt_accum** out);
int gbrt_accum_reset(gbrt_accum* acc);
/* Copies width*height*4 floats (the running sum) to host memory. */
int gbrt_accum_download(gbrt_accum* acc, float* rgba32f);
/* Restores a running sum saved with gbrt_accum_download (width*height*4
 * floats): with the saved sample count passed on as the next frame's
 * ubo.total_number_of_samples - number_of_samples, progressive rendering
 * resumes exactly where it stopped (checkpoint / resume of long renders; the
 * reference resets its accumulation image instead, main.rs:336-353). */
int gbrt_accum_upload(gbrt_accum* acc, const float* rgba32f);
int gbrt_accum_destroy(gbrt_accum* acc);

/* ------------------------------------------------------------------------ */
/* Rendering and ray queries                                                */
/* ------------------------------------------------------------------------ */

/* Renders ubo->number_of_samples samples per pixel into acc and (if out is
 * not NULL) writes the tone-mapped RGBA8 image (width*height*4 bytes) to
 * host memory.  Replaces the UBO upload + vkCmdTraceRaysKHR of
 * crates/examples/gltf_viewer/src/main.rs:215-270 and the shaders
 * RayTracing.{rgen,rchit,rahit,rmiss}, shadow.{rahit,rmiss}.  Synchronous.
 * stats may be NULL. */
int gbrt_render(gbrt_scene* scene, const gbrt_ubo* ubo, gbrt_accum* acc,
                uint8_t* out_rgba8, gbrt_stats* stats);
/* Same with explicit options (kernel form, debug outputs). */
int gbrt_render_ex(gbrt_scene* scene, const gbrt_ubo* ubo, gbrt_accum* acc,
                   uint8_t* out_rgba8, gbrt_stats* stats, const gbrt_render_opts* opts);

/* Closest-hit (or, with GBRT_RAY_TERMINATE_ON_FIRST, any-hit) queries for
 * n rays in host memory; hits written to host memory.  This is traceRayEXT
 * on its own (RayTracing.rgen:89-92, RayTracing.rchit:51-55). */
int gbrt_trace_rays(gbrt_scene* scene, const gbrt_ray* rays, uint32_t n,
                    uint32_t ray_flags, gbrt_hit* hits, gbrt_stats* stats);
/* Same with rays and hits already in device memory, enqueued on the
 * context's stream (asynchronous; call gbrt_sync before reading hits). */
int gbrt_trace_rays_device(gbrt_scene* scene, const gbrt_ray* d_rays, uint32_t n,
                           uint32_t ray_flags, gbrt_hit* d_hits);

/* ------------------------------------------------------------------------ */
/* Allocation-free world-BVH rebuild                                        */
/* ------------------------------------------------------------------------ */

/* No counterpart in the reference (it has no API of this kind).
 *
 * Rebuilds the merged world BVH of an already built scene, in place, without
 * allocating or freeing any device memory.  It exists for callers that must
 * not allocate while they run: a frame loop that rebuilds the BVH of a
 * deforming mesh every frame (cudaMalloc/cudaFree can synchronise the device
 * and stall the frame), a host whose device memory is owned by another
 * allocator or budget, or code that must not fail with out-of-memory half way
 * through a frame.
 *
 * d_vertices: NULL to rebuild from the scene's current vertices, or device
 * memory holding the scene's full vertex array (nv gbrt_vertex, same layout
 * and count as at gbrt_scene_create), which replaces the scene's vertices
 * first.  Indices, geometries and instances stay as built.
 *
 * Limits and rules:
 *  - at most GBRT_NOALLOC_MAX_TRIANGLES triangles in the world BVH; larger
 *    scenes get GBRT_E_INVALID with a message;
 *  - every instance must have an identity transform (scenes with transformed
 *    instances get GBRT_E_INVALID);
 *  - the build scratch is one static device array of 12 MiB, held by every
 *    GPU that loads the library until the process exits;
 *  - the first call on a device looks up that array's device address; make
 *    that first call before any CUDA stream capture;
 *  - all calls on a device share the array: calls from one context are
 *    ordered by its stream, but calls that overlap on the GPU (two contexts
 *    or threads on the same device at once) race and corrupt each other;
 *  - GBRT_E_BUSY while the context has unfinished jobs (they read the BVH);
 *  - the binary world BVH is rebuilt; the wide (4- or 8-wide) copy keeps its
 *    topology and is refit in place, so both traversal forms stay usable
 *    (the refit tree loses quality as the mesh deforms; gbrt_tlas_build
 *    builds a fresh one);
 *  - a failure after the rebuild has started leaves the scene unbuilt:
 *    later calls get GBRT_E_NOT_BUILT until gbrt_tlas_build.
 * Synchronous: returns after the rebuild has finished. */
#define GBRT_NOALLOC_MAX_TRIANGLES 65536u
int gbrt_scene_rebuild_noalloc(gbrt_scene* scene, const gbrt_vertex* d_vertices);

/* Autotuner (no reference counterpart; the reference leaves traversal to the
 * driver).  Renders a probe frame (probe_ubo's camera, samples and bounces at
 * width x height, into scratch memory) with the binary BVH, the 8-wide BVH
 * and the 4-wide BVH (rebuilt for the probe), each with the ray-sort key off
 * and on (on: shading writes each block's extension rays grouped by
 * direction octant, so traversal warps see more coherent rays), three rounds
 * each (the first warms up), and keeps the fastest pair (rebuilding the wide
 * BVH at the chosen width, which then stands in the scene's build flags) for
 * this scene's later renders and jobs.  No choice changes any result bit.
 * The probe should resemble the frames to come: differences between layouts
 * are a few percent.  Synchronous. */
typedef struct gbrt_tune_report {
    double ms_binary;       /* best probe time, binary layout */
    double ms_wide;         /* best probe time, 8-wide layout (0 if the scene has none) */
    double ms_wide4;        /* best probe time, 4-wide layout (0 if the scene has none) */
    double ms_sorted;       /* best probe time, chosen layout with the ray-sort key (the other times: key off) */
    uint32_t chosen_width;  /* 2, 4 or 8 */
    uint32_t sort_rays;     /* 1: ray-sort key kept */
} gbrt_tune_report;
int gbrt_scene_autotune(gbrt_scene* scene, const gbrt_ubo* probe_ubo, uint32_t width, uint32_t height,
                        gbrt_tune_report* report);
/* BVH figures of a scene.  gbrt_skin_and_refit refits the wide world BVH in
 * place (topology kept); once its SAH cost proxy has grown 1.3x over the
 * built tree's, the refit turns into a full rebuild. */
typedef struct gbrt_scene_info {
    uint32_t world_triangles;  /* triangles in the world BVH (flattened instances included) */
    uint32_t wide_nodes;       /* nodes of the wide world BVH */
    uint32_t wide_width;       /* 4 or 8 */
    uint32_t refits;           /* refits since the last full build */
    uint32_t drift_rebuilds;   /* full rebuilds forced by refit drift */
    uint32_t instance_updates; /* gbrt_tlas_update calls served incrementally (no full build) */
    double sah_built;          /* SAH cost proxy of the wide world BVH as built: summed child-box area
                                  over the root box's (0 when there is no wide world BVH) */
    double sah_now;            /* the same after the last refit */
} gbrt_scene_info;
int gbrt_scene_info_get(gbrt_scene* scene, gbrt_scene_info* info);

/* Sets the autotuner's two choices directly: BVH width 2 (binary), 4 or 8
 * (rebuilding the wide BVHs when the width changes) and the ray-sort key
 * (sort_rays != 0).  Synchronous. */
int gbrt_scene_set_tuning(gbrt_scene* scene, uint32_t width, uint32_t sort_rays);

/* ------------------------------------------------------------------------ */
/* Jobs: asynchronous frames with continuous batching                       */
/* ------------------------------------------------------------------------ */
/* No reference counterpart: the reference renders one frame at a time from
 * its render thread (record_raytracing_commands, crates/examples/
 * gltf_viewer/src/main.rs:244-270).  A job is one gbrt_render_ex call made
 * asynchronous.  Jobs on a context are traced by one scheduler thread on the
 * context's stream in waves of at most 2^22 paths; each wave packs segments
 * (a pixel range x a sample range) of up to 32 admitted jobs, possibly of
 * different scenes, so jobs join and leave the running batch at wave
 * boundaries.  A job's image and accumulation are bit-identical to the same
 * frame rendered alone by gbrt_render_ex in wavefront mode.
 *
 * Admission: a queued job is admitted when fewer than 32 jobs are active and
 * its device memory (20 B per pixel: frame sum + image) fits the HBM budget
 * still free; admission is in submission order.  Among admitted jobs, waves
 * are filled shortest-remaining-work first (GBRT_JOB_POLICY_SRPT, default)
 * or in submission order (GBRT_JOB_POLICY_FIFO).
 *
 * While a context has unfinished jobs, its synchronous calls that use the
 * stream (render, trace, builds, skinning, lights, skybox) return
 * GBRT_E_BUSY, and a scene or accumulation buffer used by an unfinished job
 * cannot be destroyed or reset.  A skinned scene is animated by jobs that
 * carry skins: the scheduler admits such a job once no active job uses that
 * scene, then skins it and rebuilds its BVH before the job's first wave.
 *
 * A job may carry a radiance cache (cache != NULL): it is then rendered in
 * waves of its own, exactly as gbrt_render_nrc renders the frame, followed
 * by its training steps, and its image is bit-identical to that call's on a
 * cache in the same state.  Jobs that share a cache train it in turn, in
 * the order the scheduler runs them.  The cache calls (query, train,
 * params, destroy) return GBRT_E_BUSY while the context has unfinished jobs. */
#define GBRT_JOB_QUEUED   0u
#define GBRT_JOB_RUNNING  1u
#define GBRT_JOB_DONE     2u
#define GBRT_JOB_POLICY_SRPT 0u
#define GBRT_JOB_POLICY_FIFO 1u
/* OR into the policy for throughput over latency: on a deep queue waves grow
 * to 2^26 paths instead of 2^24, and a job of at least 2^24 paths runs alone
 * through the single-frame kernels when its turn comes (it fills the GPU by
 * itself).  Set it before the context's first submit: the wave buffers
 * (216 B per path) are sized then. */
#define GBRT_JOB_LARGE_WAVES 0x100u

typedef struct gbrt_job_desc {
    gbrt_scene* scene;
    const gbrt_ubo* ubo;          /* copied at submit */
    gbrt_accum* accum;            /* image size = the accumulation buffer's */
    uint8_t* out_rgba8;           /* host image written when the job finishes, may be NULL */
    const gbrt_skin_raw* skins;   /* non-NULL: skin the scene (copied at submit) before the job */
    uint32_t nskin;
    uint32_t flags;               /* reserved, 0 */
    struct gbrt_nrc* cache;       /* non-NULL: render with this radiance cache (gbrt_render_nrc) */
    const struct gbrt_nrc_render_opts* cache_opts;  /* with cache: copied at submit */
} gbrt_job_desc;

typedef struct gbrt_job_info {
    uint32_t state;      /* GBRT_JOB_* */
    int32_t status;      /* GBRT_OK or the error of a finished job */
    double queue_ms;     /* submit -> admitted */
    double latency_ms;   /* submit -> finished (image on the host) */
    gbrt_stats stats;    /* the job's rays, shaded hits, node visits; device_ms = admitted -> finished */
} gbrt_job_info;

/* Queues a job; *job_id gets its handle.  Never blocks on the GPU. */
int gbrt_job_submit(gbrt_ctx* ctx, const gbrt_job_desc* desc, uint64_t* job_id);
/* GBRT_OK and the job's info once it has finished (the handle is then
 * released: a later poll of the same id is GBRT_E_INVALID); GBRT_E_BUSY
 * with the current state while it is queued or running. */
int gbrt_job_poll(gbrt_ctx* ctx, uint64_t job_id, gbrt_job_info* info);
/* Like poll, but waits up to timeout_ms (0xFFFFFFFF = no limit). */
int gbrt_job_wait(gbrt_ctx* ctx, uint64_t job_id, uint32_t timeout_ms, gbrt_job_info* info);
/* HBM budget for admitted jobs (0 = the device memory free when the first job
 * is submitted, minus 1 GiB) and the wave-filling policy. */
int gbrt_jobs_configure(gbrt_ctx* ctx, uint64_t hbm_budget_bytes, uint32_t policy);
/* Cancels a job: a queued job ends at once, a running one once the waves
 * already on the stream have drained (its image and accumulation are then
 * partial); its status becomes GBRT_E_CANCELLED.  GBRT_E_INVALID for an
 * unknown id, or when every path of the job is already on the stream (it then
 * finishes normally). */
int gbrt_job_cancel(gbrt_ctx* ctx, uint64_t job_id);
/* Host-side fault injection for tests of the serving loop (no device fault
 * is ever caused): GBRT_INJECT_ADMIT_OOM makes the next `count` job
 * admissions fail as if the device allocation had run out of memory; the job
 * ends with GBRT_E_OOM and the others carry on. */
#define GBRT_INJECT_ADMIT_OOM 1u
int gbrt_jobs_inject(gbrt_ctx* ctx, uint32_t kind, uint32_t count);

/* ------------------------------------------------------------------------ */
/* Neural radiance cache                                                     */
/* ------------------------------------------------------------------------ */
/* No reference counterpart (the reference path traces every bounce).  A
 * radiance cache maps a world position to outgoing radiance through a
 * multiresolution hash-grid encoding (16 levels x 2^log2_table entries x 2
 * features) and an MLP 32 -> 5 x 64 (ReLU) -> 3, trained online on path
 * suffixes.  Queries run the MLP on tensor cores in BF16 with FP32
 * accumulation: tcgen05.mma with the accumulator in tensor memory by
 * default, mma.sync with GBRT_NRC_QUERY_MMA_SYNC.  Training runs the
 * forward and backward passes and the weight gradient on the tensor cores
 * (mma.sync, BF16 operands, FP32 accumulation; GBRT_NRC_TRAIN_FP32: FP32 on
 * the CUDA cores), then Adam (b1 0.9, b2 0.99, eps 1e-15) on FP32 masters
 * on the loss mean((y - t)^2 / (y^2 + 0.01)) (y not differentiated in the
 * denominator).  Positions are normalised to [box_lo, box_hi]. */
typedef struct gbrt_nrc gbrt_nrc;

typedef struct gbrt_nrc_config {
    uint32_t log2_table;       /* entries per level = 2^log2_table (19 = the 32 MiB FP16 table) */
    uint32_t base_resolution;  /* coarsest level scale + 1 (16) */
    float growth;              /* per-level scale factor (about 1.45 for 16 -> 4096) */
    float learning_rate;       /* Adam step size (1e-2) */
    float box_lo[3], box_hi[3];
    uint64_t seed;             /* parameter initialisation */
    uint32_t flags;            /* GBRT_NRC_* bits; 0: queries on tcgen05, training on mma.sync */
    uint32_t _pad;
} gbrt_nrc_config;
#define GBRT_NRC_QUERY_MMA_SYNC 0x1u  /* queries on mma.sync instead of tcgen05 */
#define GBRT_NRC_TRAIN_FP32     0x2u  /* training in FP32 on the CUDA cores instead of the tensor cores */

int gbrt_nrc_create(gbrt_ctx* ctx, const gbrt_nrc_config* cfg, gbrt_nrc** out);
int gbrt_nrc_destroy(gbrt_nrc* nrc);
/* FP32 master parameters: mlp = 18,624 weights (W0 [64][32], W1..W4
 * [64][64], W5 [3][64], each [out][in]); grid = 16 * 2^log2_table * 2
 * features.  upload != 0 copies host -> device, else device -> host; either
 * pointer may be NULL. */
int gbrt_nrc_params(gbrt_nrc* nrc, float* mlp, float* grid, int upload);
/* n queries: pos4 = (x, y, z, payload) per query, out4 = (r, g, b, payload). */
int gbrt_nrc_query(gbrt_nrc* nrc, const float* pos4, uint32_t n, float* out4);
/* The same with device buffers (n float4 each, 16-byte aligned, on the
 * context's device, e.g. framework tensors): runs on the context stream,
 * waits for it, and returns the query kernel's device time in *device_ms
 * (may be NULL). */
int gbrt_nrc_query_device(gbrt_nrc* nrc, const float* pos4_dev, uint32_t n, float* out4_dev, float* device_ms);
/* Loss and gradients of one batch (pos4, target4 = (r, g, b, -)); step != 0
 * then applies one Adam step.  loss / grad_mlp / grad_grid may be NULL. */
int gbrt_nrc_train(gbrt_nrc* nrc, const float* pos4, const float* target4, uint32_t n, int step, float* loss,
                   float* grad_mlp, float* grad_grid);

/* A frame rendered with the cache (wavefront form).  About train_samples
 * paths per frame (chosen by a hash of pixel and sample) trace on as plain
 * path tracing and give one training sample each; after the frame,
 * train_steps Adam steps on those samples; *loss (may be NULL) gets the loss
 * of the last step.  disabled = 1: no path stops (the image is plain path
 * tracing; the cache still trains).  Modes:
 *  - GBRT_NRC_MODE_SUFFIX (0): a path's cache vertex is its first hit after
 *    the camera hit whose material roughness factor (1 - glossiness for
 *    specular-glossiness) is >= min_roughness.  Render paths stop there and
 *    add throughput x cache(position); a training sample is the radiance
 *    gathered from the cache vertex on, divided by the throughput reaching it.
 *  - GBRT_NRC_MODE_PRIMARY_INDIRECT (1): the cache vertex is the camera hit
 *    (roughness >= min_roughness).  Render paths shade it as usual (emission,
 *    next-event estimation) and then stop, adding cache(position) for all the
 *    radiance that would have come after it; a training sample is the
 *    radiance a full path gathers after the camera hit's own emission and
 *    next-event estimation (zero when the path ends there).  The camera sees
 *    each point from one direction, so the position-only cache represents the
 *    view-dependent indirect light of glossy surfaces for a fixed camera. */
typedef struct gbrt_nrc_render_opts {
    float min_roughness;
    uint32_t train_samples;
    uint32_t train_steps;
    uint32_t disabled;
    uint32_t mode;  /* GBRT_NRC_MODE_* */
} gbrt_nrc_render_opts;
#define GBRT_NRC_MODE_SUFFIX 0u
#define GBRT_NRC_MODE_PRIMARY_INDIRECT 1u
int gbrt_render_nrc(gbrt_scene* scene, gbrt_nrc* nrc, const gbrt_ubo* ubo, gbrt_accum* accum, uint8_t* out_rgba8,
                    gbrt_stats* stats, const gbrt_nrc_render_opts* opts, float* loss);

/* ------------------------------------------------------------------------ */
/* Device memory helpers (for callers without a CUDA runtime of their own)  */
/* ------------------------------------------------------------------------ */
int gbrt_device_alloc(gbrt_ctx* ctx, uint64_t bytes, void** d_ptr);
int gbrt_device_free(gbrt_ctx* ctx, void* d_ptr);
int gbrt_memcpy_h2d(gbrt_ctx* ctx, void* d_dst, const void* h_src, uint64_t bytes);
int gbrt_memcpy_d2h(gbrt_ctx* ctx, void* h_dst, const void* d_src, uint64_t bytes);

/* CUDA-event timer on the context's stream (ms between begin and end). */
int gbrt_timer_begin(gbrt_ctx* ctx);
int gbrt_timer_end(gbrt_ctx* ctx, double* ms);

#ifdef __cplusplus
}
#endif

#endif /* GBRT_H */
