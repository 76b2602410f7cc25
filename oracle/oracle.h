// oracle/oracle.h — C API of the CPU oracle.
//
// TEST INFRASTRUCTURE ONLY: the scalar C++ restatement of rustracer's ray-
// tracing shaders that the CUDA library is checked against and that bench.py
// times as the CPU baseline.  The shipped library never links it.
//
// Parity status: UNPINNED.  The reference's hot path is GLSL executed by a
// Vulkan ray-tracing driver (no Rust toolchain and no graphics stack exist on
// these machines), and the reference holds no golden vectors or tests for it.
// This oracle is therefore checked by known-answer and analytic tests only
// (white furnace, single-triangle hits, RNG sequences, BRDF identities).
#pragma once
#include <stdint.h>
#include "../include/gbrt.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_scene orc_scene;

typedef struct orc_stats {
    uint64_t rays_camera;
    uint64_t rays_extension;
    uint64_t rays_shadow;
    uint64_t hits_shaded;
    uint64_t node_visits;   /* BVH2 inner-node visits (TLAS + BLAS) */
    uint64_t tri_tests;     /* ray-triangle tests */
    double   seconds;       /* wall time of the call (steady clock) */
    uint32_t threads;       /* OpenMP threads used */
    uint32_t _pad;
} orc_stats;

orc_scene* orc_scene_create(const gbrt_vertex* v, uint32_t nv, const uint32_t* idx, uint32_t ni,
                            const gbrt_priminfo* prims, uint32_t ngeo,
                            const gbrt_material_raw* mats, uint32_t nmat,
                            const gbrt_texture_desc* tex, uint32_t ntex);
void orc_scene_destroy(orc_scene* s);
int  orc_blas_build(orc_scene* s, const gbrt_geo_range* ranges, uint32_t n);
int  orc_tlas_build(orc_scene* s, const gbrt_instance* inst, uint32_t n);
/* GBRT_BUILD_NO_FLATTEN keeps transformed instances in BLASes (set before orc_tlas_build). */
int  orc_build_flags(orc_scene* s, uint32_t flags);
int  orc_lights_set(orc_scene* s, const gbrt_light_raw* d, uint32_t nd,
                    const gbrt_light_raw* p, uint32_t np);
int  orc_skybox_set(orc_scene* s, uint32_t face_size, const uint8_t* rgba8_faces);
int  orc_skybox_set_ex(orc_scene* s, uint32_t face_size, const void* faces, uint32_t format);
/* Skins vertices like AnimationCompute.comp and rebuilds the BVHs. */
int  orc_skin(orc_scene* s, const gbrt_skin_raw* skins, uint32_t nskin);
/* Copies the (possibly skinned) vertex buffer out. */
int  orc_get_vertices(orc_scene* s, gbrt_vertex* out, uint32_t nv);

/* Ray queries.  fp64 != 0 runs traversal and triangle tests in double. */
int  orc_trace(orc_scene* s, const gbrt_ray* rays, uint32_t n, uint32_t flags,
               gbrt_hit* hits, int fp64, int nthreads, orc_stats* st);

/* Renders rows [row0, row1) of a width x height image with ubo semantics.
 * accum (width*height*4 floats, may be NULL) is read and written like the
 * accumulation image; out_rgba8 (may be NULL) receives the tone-mapped
 * image; sample_radiance (may be NULL) gets [pixel][sample][3] floats;
 * primary_hits (may be NULL) gets [pixel][sample] hits.  Pointers index the
 * full image.  fp64 != 0: double-precision intersection and accumulation. */
int  orc_render(orc_scene* s, const gbrt_ubo* ubo, uint32_t width, uint32_t height,
                uint32_t row0, uint32_t row1, float* accum, uint8_t* out_rgba8,
                float* sample_radiance, gbrt_hit* primary_hits, int fp64, int nthreads,
                orc_stats* st);

/* orc_render plus parity diagnostics.  sample_margins (may be NULL) gets
 * [pixel][sample][2] floats: [0] the smallest |operand - threshold| of the
 * branch decisions the sample's path took, [1] the smallest barycentric of
 * its secondary hits (both +inf when none).  nudge_ulps > 0 moves every
 * transcendental result (sin, cos, pow, exp, log), shading division and
 * square root, dot product, length and normalised vector component by
 * (nudge_ulps & 0xFFFF) ulps, up or down by a hash of the sample and of the
 * whole nudge_ulps value (the bits above 16 select another draw of signs), to
 * expose samples that ulp-level arithmetic differences change. */
int  orc_render_diag(orc_scene* s, const gbrt_ubo* ubo, uint32_t width, uint32_t height,
                     uint32_t row0, uint32_t row1, float* accum, uint8_t* out_rgba8,
                     float* sample_radiance, gbrt_hit* primary_hits, float* sample_margins,
                     uint32_t nudge_ulps, int fp64, int nthreads, orc_stats* st);

/* Shader-library entry points for known-answer tests. */
void     orc_pcg4d(const uint32_t in[4], uint32_t out[4]);
uint32_t orc_tea(uint32_t v0, uint32_t v1);
float    orc_rand(uint32_t state[4]);
float    orc_random_float(uint32_t* seed);
void     orc_eval_combined_brdf(const float N[3], const float L[3], const float V[3],
                                const float base_color[3], float metallic, float roughness,
                                float ior, float out[3]);
void     orc_tonemap(uint32_t mode, const float in[3], float out[3]);
void     orc_offset_ray(const float p[3], const float n[3], float out[3]);
void     orc_sample_texture(orc_scene* s, int32_t index, float u, float v, float out[4]);
void     orc_sample_skybox(orc_scene* s, const float dir[3], float out[3]);
uint32_t orc_blend_hash(uint32_t instance, uint32_t prim, uint32_t tag);

#ifdef __cplusplus
}
#endif
