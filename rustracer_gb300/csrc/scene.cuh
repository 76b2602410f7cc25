// scene.cuh — device-side scene layout shared by the build, trace and shade
// kernels.
//
// HBM layout of one scene:
//  * the reference's buffer set, unchanged: Vertex[] (128 B), u32 indices,
//    PrimInfo[] (16 B), MaterialRaw[] (256 B), LightRaw[] (48 B);
//  * one BVH2 node pool (BNode2, 64 B) holding every BVH of the scene: the
//    merged world BVH over identity instances, one BLAS per geometry used by
//    a transformed instance, and the TLAS over the transformed instances;
//  * one leaf-triangle pool (TriRec, 48 B: three float4 whose w lanes carry
//    the instance id, primitive id and BLAS geometry id + opaque bit), in
//    BVH leaf order, so a leaf test reads 48 contiguous bytes per triangle;
//  * DevInstance[] (object-to-world, world-to-object, ids).
#pragma once
#include "vec.cuh"
#include "../../include/gbrt.h"

namespace gbrt {

// Child encoding in BNode2: >= 0 inner node index in the pool; < 0 leaf,
// ~code where code = (first_tri << 3) | (count - 1), count in [1, 8].
struct alignas(16) BNode2 {
    float4 lxy;   // child 0: lo.x hi.x lo.y hi.y
    float4 rxy;   // child 1: lo.x hi.x lo.y hi.y
    float4 lrz;   // child 0: lo.z hi.z, child 1: lo.z hi.z
    int4 c;       // c.x child 0, c.y child 1, c.z/c.w unused
};
static_assert(sizeof(BNode2) == 64, "BNode2 is 64 B");

GB_HD int leaf_code(uint32_t first, uint32_t count) { return ~(int)((first << 3) | (count - 1)); }
GB_HD uint32_t leaf_first(int c) { return ((uint32_t)~c) >> 3; }
GB_HD uint32_t leaf_count(int c) { return (((uint32_t)~c) & 7u) + 1u; }
constexpr uint32_t kMaxLeaf = 8;

// TriRec w lanes: a.w = instance id, b.w = primitive id, c.w = BLAS geometry
// id | (opaque << 31).
struct alignas(16) TriRec {
    float4 a, b, c;
};

// Compressed 8-wide BVH node (after Ylitie, Karras, Laine 2017, "Efficient
// Incoherent Ray Traversal on GPUs Through Compressed Wide BVHs"), 80 B,
// fetched as five 16-byte loads.  Child boxes are 8-bit offsets on a
// per-node grid: lo = p + qlo * 2^(e-127) per axis, rounded outward and
// padded by one grid step at build time.  meta[s]: 0 = empty slot; inner
// child = 0x20 | (24 + s); leaf = (unary triangle count << 5) | offset of its
// first triangle from tri_base (count <= 3, offsets < 24).  Inner children
// are stored contiguously from child_base in slot order; a ray of octant o
// visits the inner children in increasing order of (slot ^ o).
struct alignas(16) CwNode {
    float p[3];
    uint8_t e[3];
    uint8_t imask;
    uint32_t child_base;
    uint32_t tri_base;
    uint8_t meta[8];
    uint8_t qlo[3][8];
    uint8_t qhi[3][8];
};
static_assert(sizeof(CwNode) == 80, "CwNode is 80 B");

struct DevInstance {
    float xf[12];      // object-to-world, row-major 3x4
    float inv[12];     // world-to-object
    uint32_t custom;   // gl_InstanceCustomIndexEXT (geometry id for shading)
    uint32_t mask;
    uint32_t blas_geo; // geometry whose BLAS this instance uses
    int32_t blas_root; // root of that BLAS in the pool (node index or leaf code)
    uint32_t has_blas; // 0 when the geometry has no triangles
    uint32_t identity; // 1 = merged into the world BVH
    uint32_t cw_node0; // its 8-wide BLAS: first node and first triangle slot in the BLAS pools
    uint32_t cw_tri0;
};

struct DevTexture {
    const void* data;
    uint32_t w, h, format, wrap_s, wrap_t, _pad;
};

struct DevScene {
    const BNode2* nodes;
    const TriRec* tris;
    const DevInstance* inst;
    uint32_t ninst;
    int32_t world_root;   // node index or leaf code, valid when has_world
    int32_t tlas_root;    // valid when has_tlas
    const CwNode* cw_nodes;  // 8-wide world BVH (root = node 0), null if not built
    const TriRec* cw_tris;   //   its triangles, in node-leaf order
    const CwNode* blas_cw_nodes;  // 8-wide BLASes of transformed instances (null: binary BLASes)
    const TriRec* blas_cw_tris;
    uint32_t has_world;   // some identity instance exists
    uint32_t has_tlas;    // some transformed instance exists
    float4 world_lo, world_hi;  // bounds of the world BVH root
    float4 tlas_lo, tlas_hi;
    const gbrt_vertex* vertices;
    const uint32_t* indices;
    const gbrt_priminfo* prims;
    const gbrt_material_raw* mats;
    const DevTexture* tex;
    uint32_t ntex;
    const gbrt_light_raw* dlights;
    uint32_t nd;
    const gbrt_light_raw* plights;
    uint32_t np;
    const void* sky;     // 6 faces, size^2 texels each
    uint32_t sky_size;
    uint32_t sky_format; // GBRT_TEX_RGBA8_SRGB or GBRT_TEX_RGBA32F
    uint32_t all_opaque; // every geometry is OPAQUE: the any-hit test never runs
    uint32_t prefer_binary;  // autotuner's choice: traverse the binary layout even where 8-wide nodes exist
    uint32_t sort_rays;      // autotuner's choice: shade writes each block's extension rays grouped by octant
    uint32_t shade_feat;     // kFeat* bits the scene's materials use (shade kernels specialise on them)
};

// Material features of the hit group (closest_hit) a shade kernel may be
// compiled without.  A scene whose materials never use a feature never takes
// its code, so a kernel compiled without it returns the same bits.
constexpr uint32_t kFeatTextures = 1u;   // some material samples a texture
constexpr uint32_t kFeatSpecGloss = 2u;  // some material uses the specular-glossiness workflow
constexpr uint32_t kFeatDebug = 4u;      // unlit materials, a debug mapping or the legacy debug branch
constexpr uint32_t kFeatVolume = 8u;     // some material has KHR_materials_volume (refraction, attenuation)
constexpr uint32_t kFeatAll = 15u;

}  // namespace gbrt
