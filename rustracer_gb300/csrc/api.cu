// api.cu — host implementation of the C ABI in include/gbrt.h.
//
// Every entry point validates its arguments, records a message on failure,
// returns a GBRT_* code and never throws across the ABI.  Device memory is
// owned by the handle that created it and released by its *_destroy.
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <algorithm>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "api_internal.h"

using namespace gbrt;
using namespace gbrt_host;

static_assert(sizeof(gbrt_vertex) == 128, "Vertex is 128 B (geometry.rs:10-22)");
static_assert(sizeof(gbrt_priminfo) == 16, "PrimInfo is 16 B");
static_assert(sizeof(gbrt_material_raw) == 256, "MaterialRaw is 256 B");
static_assert(offsetof(gbrt_material_raw, attenuation_color) == 128, "VolumeInfo at 128");
static_assert(offsetof(gbrt_material_raw, specular_texture) == 160, "SpecularInfo at 160");
static_assert(offsetof(gbrt_material_raw, sg_diffuse_factor) == 208, "SpecularGlossiness at 208");
static_assert(sizeof(gbrt_light_raw) == 48, "LightRaw is 48 B");
static_assert(sizeof(gbrt_ubo) == 324, "UniformBufferObject is 324 B");
static_assert(sizeof(gbrt_instance) == 64, "VkAccelerationStructureInstanceKHR is 64 B");
static_assert(sizeof(gbrt_skin_raw) == 16384, "Skin is 256 mat4");
static_assert(sizeof(gbrt_ray) == 32 && sizeof(gbrt_hit) == 24, "ray/hit records");
static_assert(sizeof(gbrt_stats) == 104, "stats record");
static_assert(sizeof(gbrt_job_info) == 128 && sizeof(gbrt_job_desc) == 64, "job records");
static_assert(sizeof(gbrt_nrc_config) == 56 && sizeof(gbrt_nrc_render_opts) == 20, "cache records");
static_assert(sizeof(gbrt_tune_report) == 40, "tune report");
static_assert(sizeof(gbrt_scene_info) == 40, "scene info");

namespace {
thread_local std::string g_create_error;
}  // namespace

namespace gbrt_host {

int fail(gbrt_ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    else g_create_error = msg;
    return code;
}
int cuda_fail(gbrt_ctx* c, cudaError_t e, const char* what) {
    cudaGetLastError();  // clear sticky-free errors
    return fail(c, e == cudaErrorMemoryAllocation ? GBRT_E_OOM : GBRT_E_CUDA,
                std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")");
}
// World-to-object transform: adjugate inverse of the 3x3 part in double and
// translation -R^-1 t, each rounded once to float (the oracle computes the
// same expression).
void affine_inverse(const float* m, float* inv) {
    double a00 = m[0], a01 = m[1], a02 = m[2], a10 = m[4], a11 = m[5], a12 = m[6];
    double a20 = m[8], a21 = m[9], a22 = m[10];
    double t0 = m[3], t1 = m[7], t2 = m[11];
    double det = a00 * (a11 * a22 - a12 * a21) - a01 * (a10 * a22 - a12 * a20) + a02 * (a10 * a21 - a11 * a20);
    double r[9] = {(a11 * a22 - a12 * a21) / det, (a02 * a21 - a01 * a22) / det, (a01 * a12 - a02 * a11) / det,
                   (a12 * a20 - a10 * a22) / det, (a00 * a22 - a02 * a20) / det, (a02 * a10 - a00 * a12) / det,
                   (a10 * a21 - a11 * a20) / det, (a01 * a20 - a00 * a21) / det, (a00 * a11 - a01 * a10) / det};
    for (int i = 0; i < 3; ++i) {
        inv[i * 4 + 0] = (float)r[i * 3 + 0];
        inv[i * 4 + 1] = (float)r[i * 3 + 1];
        inv[i * 4 + 2] = (float)r[i * 3 + 2];
        inv[i * 4 + 3] = (float)(-(r[i * 3 + 0] * t0 + r[i * 3 + 1] * t1 + r[i * 3 + 2] * t2));
    }
}

bool is_identity(const float* m) {
    static const float id[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
    return std::memcmp(m, id, sizeof(id)) == 0;
}

template <class T>
cudaError_t upload(DevBuf& b, const T* src, size_t n, cudaStream_t st) {
    cudaError_t e = b.alloc(n * sizeof(T));
    if (e != cudaSuccess || n == 0) return e;
    return cudaMemcpyAsync(b.p, src, n * sizeof(T), cudaMemcpyHostToDevice, st);
}

// Sizes the wavefront buffers for `cap` paths and `npix` pixels (grow only).
cudaError_t wavefront_reserve(gbrt_ctx* c, uint32_t cap, size_t npix) {
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    const size_t f4 = al((size_t)cap * sizeof(float4)), u1 = al((size_t)cap * 4);
    const size_t counts = al((size_t)kMaxWaveJobs * kWfCounters * sizeof(uint32_t));
    const size_t bytes = 16 * f4 + 2 * u1 + counts;
    if (c->wf.cap < cap || c->wf_mem.bytes < bytes) {
        cudaError_t e = c->wf_mem.alloc(bytes);
        if (e != cudaSuccess) {
            c->wf.cap = 0;
            return e;
        }
        char* p = c->wf_mem.as<char>();
        auto take = [&](size_t b) { void* r = p; p += b; return r; };
        WfState& w = c->wf;
        w.ray_o[0] = (float4*)take(f4);
        w.ray_o[1] = (float4*)take(f4);
        w.ray_d[0] = (float4*)take(f4);
        w.ray_d[1] = (float4*)take(f4);
        w.hit = (float4*)take(f4);
        w.q_tp[0] = (float4*)take(f4);
        w.q_tp[1] = (float4*)take(f4);
        w.q_rng[0] = (uint4*)take(f4);
        w.q_rng[1] = (uint4*)take(f4);
        w.q_rad[0] = (float4*)take(f4);
        w.q_rad[1] = (float4*)take(f4);
        // frames with a radiance cache keep throughput and RNG counters by path id and never touch
        // the queue-ordered copies; other frames never touch the by-path-id ones (a camera of a
        // frame without bounces writes tp, which no shade reads): they share memory
        w.tp = w.q_tp[0];
        w.rng = w.q_rng[0];
        w.rad = (float4*)take(f4);
        w.sh_o = (float4*)take(f4);
        w.sh_d = (float4*)take(f4);
        w.sh_e = (float4*)take(f4);
        w.sh_c = (float4*)take(f4);
        w.hit_prim = (uint32_t*)take(u1);
        w.sh_tp = (float*)take(u1);
        w.counts = (uint32_t*)take(counts);
        w.cap = cap;
    }
    cudaError_t e = c->wf_frame.reserve(npix * sizeof(float4));
    c->wf.frame_sum = c->wf_frame.as<float4>();
    return e;
}

int cw_width(const gbrt_scene* s) { return (s->build_flags & GBRT_BUILD_WIDTH4) ? 4 : 8; }

__global__ void or_status_kernel(const DeviceCounters* dc, uint32_t* acc) { *acc |= dc->status; }

size_t texel_bytes(uint32_t format) {
    return format == GBRT_TEX_RGBA32F ? 16u : format == GBRT_TEX_RGBA16F ? 8u : 4u;
}

// kFeat* bits the materials use: the shade kernels compiled without a feature
// serve scenes that never take its code.
uint32_t material_features(const gbrt_material_raw* mats, uint32_t nmat) {
    uint32_t f = 0;
    for (uint32_t i = 0; i < nmat; ++i) {
        const gbrt_material_raw& m = mats[i];
        const gbrt_texture_info* tex[] = {&m.base_color_texture,     &m.metallic_roughness_texture,
                                          &m.normal_texture,         &m.emissive_texture,
                                          &m.transmission_texture,   &m.specular_texture,
                                          &m.specular_color_texture, &m.sg_diffuse_texture,
                                          &m.sg_specular_glossiness_texture};
        for (const gbrt_texture_info* t : tex)
            if (t->index >= 0) f |= gbrt::kFeatTextures;
        if (m.workflow == 1u) f |= gbrt::kFeatSpecGloss;
        if (m.unlit) f |= gbrt::kFeatDebug;
        if (m.volume_exists) f |= gbrt::kFeatVolume;
    }
    return f;
}

void refresh_view(gbrt_scene* s) {
    DevScene& v = s->view;
    v.shade_feat = s->shade_feat;
    v.nodes = s->nodes.as<BNode2>();
    v.tris = s->tris.as<TriRec>();
    v.inst = s->inst.as<DevInstance>();
    v.ninst = (uint32_t)s->instances.size();
    v.vertices = s->vertices.as<gbrt_vertex>();
    v.indices = s->indices.as<uint32_t>();
    v.prims = s->prims.as<gbrt_priminfo>();
    v.mats = s->mats.as<gbrt_material_raw>();
    v.tex = s->tex_descs.as<DevTexture>();
    v.ntex = s->ntex;
    v.dlights = s->dlights.as<gbrt_light_raw>();
    v.nd = s->nd;
    v.plights = s->plights.as<gbrt_light_raw>();
    v.np = s->np;
    v.sky = s->sky.p;
    v.sky_size = s->sky_size;
    v.sky_format = s->sky_format;
    v.cw_nodes = s->cw_count ? s->cw_nodes.as<CwNode>() : nullptr;
    v.cw_tris = s->cw_count ? s->cw_tris.as<TriRec>() : nullptr;
    v.blas_cw_nodes = s->blas_cw_nodes.p ? s->blas_cw_nodes.as<CwNode>() : nullptr;
    v.blas_cw_tris = s->blas_cw_nodes.p ? s->blas_cw_tris.as<TriRec>() : nullptr;
}

// Builds the merged world BVH, the BLASes of transformed instances and the
// TLAS into fresh pools.
int build_all(gbrt_scene* s) {
    gbrt_ctx* c = s->ctx;
    cudaStream_t st = c->stream;
    const size_t ninst = s->instances.size();
    std::vector<DevInstance> hinst(ninst);
    std::vector<uint4> world_items;
    std::vector<uint32_t> tlas_ids;
    std::vector<uint8_t> blas_needed(s->ngeo, 0);
    bool all_opaque = true;
    // flatten transformed instances into the world BVH when the flattened
    // scene stays within GBRT_FLATTEN_MAX_TRIANGLES (and the build allows it)
    uint64_t flat_total = 0;
    for (size_t i = 0; i < ninst; ++i) {
        const gbrt_instance& in = s->instances[i];
        const uint32_t g = (uint32_t)in.blas_handle;
        if ((in.custom_index_and_mask >> 24) == 0 || g >= s->ngeo || !s->has_range[g]) continue;
        flat_total += s->ranges[g].i_len / 3;
    }
    const bool flatten = !(s->build_flags & GBRT_BUILD_NO_FLATTEN) && flat_total <= GBRT_FLATTEN_MAX_TRIANGLES;
    for (size_t i = 0; i < ninst; ++i) {
        const gbrt_instance& in = s->instances[i];
        DevInstance& d = hinst[i];
        std::memset(&d, 0, sizeof(d));
        std::memcpy(d.xf, in.transform, sizeof(d.xf));
        affine_inverse(d.xf, d.inv);
        d.custom = in.custom_index_and_mask & 0xFFFFFFu;
        d.mask = in.custom_index_and_mask >> 24;
        d.blas_geo = (uint32_t)in.blas_handle;
        if (d.blas_geo >= s->ngeo || d.custom >= s->ngeo)
            return fail(c, GBRT_E_INVALID, "instance " + std::to_string(i) + " references a geometry out of range");
        if (!s->has_range[d.blas_geo])
            return fail(c, GBRT_E_NOT_BUILT, "instance " + std::to_string(i) + " uses a geometry without a BLAS range");
        const gbrt_geo_range& r = s->ranges[d.blas_geo];
        const uint32_t ntri = r.i_len / 3;
        // shading fetches triangles through PrimInfo[custom index]; it must
        // cover every primitive id the BLAS can return
        if (d.custom != d.blas_geo && (!s->has_range[d.custom] || s->ranges[d.custom].i_len < r.i_len))
            return fail(c, GBRT_E_INVALID, "instance " + std::to_string(i) +
                                               ": custom index geometry has fewer triangles than its BLAS");
        d.identity = is_identity(in.transform) && (d.mask & 0xFFu) != 0;
        if ((d.mask & 0xFFu) == 0 || ntri == 0) continue;
        if (!r.opaque) all_opaque = false;
        if (d.identity || flatten) {
            for (uint32_t p = 0; p < ntri; ++p)
                world_items.push_back(make_uint4((uint32_t)i, d.blas_geo, p, r.opaque ? 1u : 0u));
        } else {
            blas_needed[d.blas_geo] = 1;
            tlas_ids.push_back((uint32_t)i);
        }
    }
    // pool sizes
    size_t nnodes = 0, ntris = 0;
    auto add = [&](size_t n) {
        nnodes += n > 1 ? n - 1 : 0;
        ntris += n;
    };
    add(world_items.size());
    std::vector<uint32_t> blas_node_base(s->ngeo, 0), blas_tri_base(s->ngeo, 0);
    for (uint32_t g = 0; g < s->ngeo; ++g) {
        if (!blas_needed[g]) continue;
        blas_node_base[g] = (uint32_t)nnodes;
        blas_tri_base[g] = (uint32_t)ntris;
        add(s->ranges[g].i_len / 3);
    }
    const uint32_t tlas_node_base = (uint32_t)nnodes, tlas_tri_base = (uint32_t)ntris;
    add(tlas_ids.size());
    if (ntris >= (1u << 28)) return fail(c, GBRT_E_INVALID, "scene exceeds 2^28 leaf slots");
    CU(c, s->nodes.alloc(std::max<size_t>(1, nnodes) * sizeof(BNode2)), "cudaMalloc(nodes)");
    CU(c, s->tris.alloc(std::max<size_t>(1, ntris) * sizeof(TriRec)), "cudaMalloc(tris)");
    DevScene& v = s->view;
    v.has_world = 0;
    v.has_tlas = 0;
    v.all_opaque = all_opaque ? 1u : 0u;
    s->all_opaque = all_opaque;
    // instances first: the world build transforms the triangles of flattened ones
    CU(c, upload(s->inst, hinst.data(), hinst.size(), st), "upload(instances)");
    if (hinst.empty()) CU(c, s->inst.alloc(sizeof(DevInstance)), "cudaMalloc");
    // world BVH
    if (!world_items.empty()) {
        CU(c, upload(s->items, world_items.data(), world_items.size(), st), "upload(items)");
        BvhResult r;
        CU(c, build_triangle_bvh(s->vertices.as<gbrt_vertex>(), s->indices.as<uint32_t>(),
                                 s->prims.as<gbrt_priminfo>(), s->items.as<uint4>(), (uint32_t)world_items.size(),
                                 s->nodes.as<BNode2>(), 0, s->tris.as<TriRec>(), 0, &r, st,
                                 s->inst.as<DevInstance>()),
           "build world BVH");
        v.has_world = 1;
        v.world_root = r.root;
        v.world_lo = r.lo;
        v.world_hi = r.hi;
        const size_t nw = world_items.size();
        CU(c, s->cw_nodes.alloc(nw * sizeof(CwNode)), "cudaMalloc(wide nodes)");
        CU(c, s->cw_tris.alloc(nw * sizeof(TriRec)), "cudaMalloc(wide triangles)");
        CU(c, build_triangle_cwbvh(s->vertices.as<gbrt_vertex>(), s->indices.as<uint32_t>(),
                                   s->prims.as<gbrt_priminfo>(), s->items.as<uint4>(), (uint32_t)nw,
                                   s->cw_nodes.as<CwNode>(), s->cw_tris.as<TriRec>(), &s->cw_count, st,
                                   &s->cw_levels, s->inst.as<DevInstance>(), cw_width(s)),
           "build wide world BVH");
        s->nworld = (uint32_t)nw;
        // the tree's SAH cost proxy as built (a refit of unchanged vertices rewrites the same nodes), the
        // reference for the drift check of later refits
        s->cw_sah0 = 0.0;
        s->refits = 0;
        if (s->cw_levels.size() >= 2) {
            CU(c, s->cw_boxes.reserve((size_t)s->cw_count * 2 * sizeof(float4) + 16), "cudaMalloc(refit boxes)");
            CU(c, refit_triangle_cwbvh(s->vertices.as<gbrt_vertex>(), s->indices.as<uint32_t>(),
                                       s->prims.as<gbrt_priminfo>(), s->cw_nodes.as<CwNode>(), s->cw_tris.as<TriRec>(),
                                       s->nworld, s->cw_levels, s->cw_boxes.as<float4>(), st,
                                       s->inst.as<DevInstance>(), &s->cw_sah0),
               "measure wide world BVH");
            s->cw_sah = s->cw_sah0;
        }
    } else {
        s->cw_nodes.release();
        s->cw_tris.release();
        s->cw_count = 0;
        s->cw_levels.clear();
        s->nworld = 0;
    }
    // BLASes + TLAS
    if (!tlas_ids.empty()) {
        std::vector<float4> blo(s->ngeo), bhi(s->ngeo);
        std::vector<int32_t> broot(s->ngeo, 0);
        // 8-wide copies of the BLASes: pools with one slot per triangle
        std::vector<uint32_t> cw_node0(s->ngeo, 0), cw_tri0(s->ngeo, 0);
        size_t cw_slots = 0;
        for (uint32_t g = 0; g < s->ngeo; ++g) {
            if (!blas_needed[g]) continue;
            cw_node0[g] = cw_tri0[g] = (uint32_t)cw_slots;
            cw_slots += s->ranges[g].i_len / 3;
        }
        CU(c, s->blas_cw_nodes.alloc(std::max<size_t>(1, cw_slots) * sizeof(CwNode)), "cudaMalloc(wide BLAS nodes)");
        CU(c, s->blas_cw_tris.alloc(std::max<size_t>(1, cw_slots) * sizeof(TriRec)), "cudaMalloc(wide BLAS tris)");
        DevBuf bitems;
        for (uint32_t g = 0; g < s->ngeo; ++g) {
            if (!blas_needed[g]) continue;
            const uint32_t ntri = s->ranges[g].i_len / 3;
            std::vector<uint4> items(ntri);
            for (uint32_t p = 0; p < ntri; ++p) items[p] = make_uint4(0u, g, p, s->ranges[g].opaque ? 1u : 0u);
            CU(c, upload(bitems, items.data(), items.size(), st), "upload(blas items)");
            BvhResult r;
            CU(c, build_triangle_bvh(s->vertices.as<gbrt_vertex>(), s->indices.as<uint32_t>(),
                                     s->prims.as<gbrt_priminfo>(), bitems.as<uint4>(), ntri, s->nodes.as<BNode2>(),
                                     blas_node_base[g], s->tris.as<TriRec>(), blas_tri_base[g], &r, st),
               "build BLAS");
            broot[g] = r.root;
            blo[g] = r.lo;
            bhi[g] = r.hi;
            uint32_t used = 0;
            CU(c, build_triangle_cwbvh(s->vertices.as<gbrt_vertex>(), s->indices.as<uint32_t>(),
                                       s->prims.as<gbrt_priminfo>(), bitems.as<uint4>(), ntri,
                                       s->blas_cw_nodes.as<CwNode>() + cw_node0[g],
                                       s->blas_cw_tris.as<TriRec>() + cw_tri0[g], &used, st, nullptr, nullptr,
                                       cw_width(s)),
               "build wide BLAS");
        }
        const uint32_t nt = (uint32_t)tlas_ids.size();
        std::vector<float4> ilo(nt), ihi(nt);
        for (uint32_t k = 0; k < nt; ++k) {
            DevInstance& d = hinst[tlas_ids[k]];
            d.blas_root = broot[d.blas_geo];
            d.cw_node0 = cw_node0[d.blas_geo];
            d.cw_tri0 = cw_tri0[d.blas_geo];
            d.has_blas = 1;
            ilo[k] = blo[d.blas_geo];
            ihi[k] = bhi[d.blas_geo];
        }
        CU(c, upload(s->inst, hinst.data(), hinst.size(), st), "upload(instances)");
        DevBuf &d_ids = s->tlas_ids_d, &d_blo = s->tlas_blo, &d_bhi = s->tlas_bhi, &d_lo = s->tlas_lo,
               &d_hi = s->tlas_hi;
        CU(c, upload(d_ids, tlas_ids.data(), nt, st), "upload(tlas ids)");
        CU(c, upload(d_blo, ilo.data(), nt, st), "upload");
        CU(c, upload(d_bhi, ihi.data(), nt, st), "upload");
        CU(c, d_lo.alloc(nt * sizeof(float4)), "cudaMalloc");
        CU(c, d_hi.alloc(nt * sizeof(float4)), "cudaMalloc");
        CU(c, instance_world_boxes(s->inst.as<DevInstance>(), d_ids.as<uint32_t>(), d_blo.as<float4>(),
                                   d_bhi.as<float4>(), nt, d_lo.as<float4>(), d_hi.as<float4>(), st),
           "instance boxes");
        BvhResult r;
        CU(c, build_instance_bvh(d_lo.as<float4>(), d_hi.as<float4>(), d_ids.as<uint32_t>(), nt,
                                 s->nodes.as<BNode2>(), tlas_node_base, s->tris.as<TriRec>(), tlas_tri_base, &r, st),
           "build TLAS");
        s->tlas_node_base = tlas_node_base;
        s->tlas_tri_base = tlas_tri_base;
        v.has_tlas = 1;
        v.tlas_root = r.root;
        v.tlas_lo = r.lo;
        v.tlas_hi = r.hi;
        CU(c, cudaStreamSynchronize(st), "sync after TLAS build");
    } else {
        s->blas_cw_nodes.release();
        s->blas_cw_tris.release();
        CU(c, cudaStreamSynchronize(st), "sync after build");
    }
    s->h_inst = std::move(hinst);
    s->tlas_ids = std::move(tlas_ids);
    s->flattened = false;
    for (const DevInstance& d : s->h_inst) s->flattened = s->flattened || (flatten && !d.identity && (d.mask & 0xFFu));
    refresh_view(s);
    s->built = v.has_world || v.has_tlas;
    return GBRT_OK;
}

// gbrt_tlas_update: the instances keep their geometries, masks and custom
// indices and only their transforms move (the reference's animated frames,
// gltf_viewer main.rs:395-402 -> create_top_as).  Transformed instances merged
// into the world BVH re-transform their triangles: the binary world BVH is
// rebuilt (Morton radix tree, one launch chain) and the wide one refit in
// place, with the refit's drift check; a TLAS is rebuilt over the instances'
// new world boxes, the BLASes untouched.  Anything else changing (a geometry,
// a mask, an instance entering or leaving the world BVH) takes a full build.
int update_instances(gbrt_scene* s, const gbrt_instance* in, uint32_t n) {
    gbrt_ctx* c = s->ctx;
    cudaStream_t st = c->stream;
    bool same = s->h_inst.size() == n;
    for (uint32_t i = 0; same && i < n; ++i) {
        const gbrt_instance& a = s->instances[i];
        const gbrt_instance& b = in[i];
        const uint32_t mask = b.custom_index_and_mask >> 24;
        same = a.custom_index_and_mask == b.custom_index_and_mask && a.blas_handle == b.blas_handle &&
               a.sbt_offset_and_flags == b.sbt_offset_and_flags;
        // without flattening, identity instances live in the world BVH and the others under the TLAS
        if (same && !s->flattened && mask) same = (bool)s->h_inst[i].identity == is_identity(b.transform);
    }
    s->instances.assign(in, in + n);
    if (!same) return build_all(s);
    for (uint32_t i = 0; i < n; ++i) {
        DevInstance& d = s->h_inst[i];
        std::memcpy(d.xf, in[i].transform, sizeof(d.xf));
        affine_inverse(d.xf, d.inv);
        d.identity = is_identity(in[i].transform) && (d.mask & 0xFFu) != 0;
    }
    CU(c, cudaMemcpyAsync(s->inst.p, s->h_inst.data(), n * sizeof(DevInstance), cudaMemcpyHostToDevice, st),
       "upload(instances)");
    DevScene& v = s->view;
    if (v.has_tlas) {
        const uint32_t nt = (uint32_t)s->tlas_ids.size();
        CU(c, instance_world_boxes(s->inst.as<DevInstance>(), s->tlas_ids_d.as<uint32_t>(), s->tlas_blo.as<float4>(),
                                   s->tlas_bhi.as<float4>(), nt, s->tlas_lo.as<float4>(), s->tlas_hi.as<float4>(), st),
           "instance boxes");
        BvhResult r;
        CU(c, build_instance_bvh(s->tlas_lo.as<float4>(), s->tlas_hi.as<float4>(), s->tlas_ids_d.as<uint32_t>(), nt,
                                 s->nodes.as<BNode2>(), s->tlas_node_base, s->tris.as<TriRec>(), s->tlas_tri_base, &r,
                                 st),
           "rebuild TLAS");
        v.tlas_root = r.root;
        v.tlas_lo = r.lo;
        v.tlas_hi = r.hi;
    }
    ++s->instance_updates;
    if (s->flattened) return refit_world(s);
    CU(c, cudaStreamSynchronize(st), "sync after instance update");
    refresh_view(s);
    return GBRT_OK;
}

void fill_stats(gbrt_stats* st, const DeviceCounters& dc, double ms, uint32_t launches) {
    if (!st) return;
    st->rays_camera = dc.camera;
    st->rays_extension = dc.extension;
    st->rays_shadow = dc.shadow;
    st->rays_total = dc.camera + dc.extension + dc.shadow;
    st->hits_shaded = dc.shaded;
    st->device_ms = ms;
    st->kernel_launches = launches;
    st->device_status = dc.status;
    st->node_visits = dc.nodes;
    st->tri_tests = dc.tris;
    for (int k = 0; k < 4; ++k) st->stage_ms[k] = 0.0;
}

int skin_scene(gbrt_scene* s, const gbrt_skin_raw* skins, uint32_t nskin) {
    gbrt_ctx* c = s->ctx;
    DeviceGuard g(c->device);
    cudaStream_t st = c->stream;
    if (!s->skinned) {  // keep the bind-pose vertices (the reference's vertex_buffer)
        CU(c, s->base_vertices.alloc(s->vertices.bytes), "cudaMalloc(base vertices)");
        CU(c, cudaMemcpyAsync(s->base_vertices.p, s->vertices.p, s->vertices.bytes, cudaMemcpyDeviceToDevice, st),
           "copy");
        s->skinned = true;
    }
    CU(c, upload(s->skins, skins, nskin, st), "upload(skins)");
    CU(c, launch_skinning(s->base_vertices.as<gbrt_vertex>(), s->vertices.as<gbrt_vertex>(), s->nv,
                          s->skins.as<gbrt_skin_raw>(), nskin, st),
       "skinning");
    return refit_world(s);
}

constexpr double kRefitDrift = 1.3;

int refit_world(gbrt_scene* s) {
    gbrt_ctx* c = s->ctx;
    DevScene& v = s->view;
    // transformed instances (BLAS boxes feed the TLAS) or no 8-wide copy: full rebuild
    if (v.has_tlas || !v.has_world || !s->cw_count || s->cw_levels.size() < 2) return build_all(s);
    cudaStream_t st = c->stream;
    // binary world BVH: rebuilt (an LBVH over the same items, one launch chain);
    // 8-wide world BVH: refit in place, keeping its topology and slots
    BvhResult r;
    CU(c, build_triangle_bvh(s->vertices.as<gbrt_vertex>(), s->indices.as<uint32_t>(), s->prims.as<gbrt_priminfo>(),
                             s->items.as<uint4>(), s->nworld, s->nodes.as<BNode2>(), 0, s->tris.as<TriRec>(), 0, &r,
                             st, s->inst.as<DevInstance>(), kBvhFast),
       "rebuild world BVH");
    CU(c, s->cw_boxes.reserve((size_t)s->cw_count * 2 * sizeof(float4) + 16), "cudaMalloc(refit boxes)");
    double sah = 0.0;
    CU(c, refit_triangle_cwbvh(s->vertices.as<gbrt_vertex>(), s->indices.as<uint32_t>(), s->prims.as<gbrt_priminfo>(),
                               s->cw_nodes.as<CwNode>(), s->cw_tris.as<TriRec>(), s->nworld, s->cw_levels,
                               s->cw_boxes.as<float4>(), st, s->inst.as<DevInstance>(), &sah),
       "refit wide world BVH");
    ++s->refits;
    s->cw_sah = sah;
    // topology kept through large deformations loses quality: rebuild once the tree's SAH cost proxy has
    // grown by kRefitDrift over the built tree's
    if (s->cw_sah0 > 0.0 && sah > kRefitDrift * s->cw_sah0) {
        ++s->rebuilds;
        return build_all(s);
    }
    v.world_root = r.root;
    v.world_lo = r.lo;
    v.world_hi = r.hi;
    refresh_view(s);
    return GBRT_OK;
}

}  // namespace gbrt_host

extern "C" {

const char* gbrt_version(void) { return "gbrt 0.1 sm_103a"; }

const char* gbrt_last_error(const gbrt_ctx* ctx) { return ctx ? ctx->err.c_str() : g_create_error.c_str(); }

int gbrt_ctx_create(int device, gbrt_ctx** out) {
    if (!out) return fail(nullptr, GBRT_E_INVALID, "out is NULL");
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        cudaGetLastError();
        return fail(nullptr, GBRT_E_NO_DEVICE, "no CUDA device available");
    }
    if (device < 0 || device >= n) return fail(nullptr, GBRT_E_INVALID, "device index out of range");
    gbrt_ctx* c = new (std::nothrow) gbrt_ctx();
    if (!c) return fail(nullptr, GBRT_E_OOM, "host allocation failed");
    c->device = device;
    DeviceGuard g(device);
    auto bail = [&](cudaError_t err, const char* what) {
        std::string m = std::string(what) + ": " + cudaGetErrorString(err);
        gbrt_ctx_destroy(c);
        return fail(nullptr, GBRT_E_CUDA, m);
    };
    if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess) return bail(e, "stream");
    if ((e = cudaEventCreate(&c->ev0)) != cudaSuccess) return bail(e, "event");
    if ((e = cudaStreamCreateWithFlags(&c->side.stream, cudaStreamNonBlocking)) != cudaSuccess) return bail(e, "stream");
    if ((e = cudaEventCreateWithFlags(&c->side.shaded, cudaEventDisableTiming)) != cudaSuccess) return bail(e, "event");
    if ((e = cudaEventCreateWithFlags(&c->side.shadowed, cudaEventDisableTiming)) != cudaSuccess) return bail(e, "event");
    if ((e = cudaEventCreate(&c->ev1)) != cudaSuccess) return bail(e, "event");
    if ((e = cudaEventCreate(&c->tb0)) != cudaSuccess) return bail(e, "event");
    if ((e = cudaEventCreate(&c->tb1)) != cudaSuccess) return bail(e, "event");
    if ((e = c->counters.alloc(sizeof(DeviceCounters))) != cudaSuccess) return bail(e, "counters");
    if ((e = c->trace_work.alloc(256)) != cudaSuccess) return bail(e, "counters");
    float lut[256];
    for (int i = 0; i < 256; ++i) {
        double v = i / 255.0;
        lut[i] = (float)(v <= 0.04045 ? v / 12.92 : std::pow((v + 0.055) / 1.055, 2.4));
    }
    if ((e = init_render_constants(lut)) != cudaSuccess) return bail(e, "constants");
    if ((e = init_wavefront_constants(lut)) != cudaSuccess) return bail(e, "constants");
    if ((e = init_wave_multi_constants(lut)) != cudaSuccess) return bail(e, "constants");
    *out = c;
    return GBRT_OK;
}

int gbrt_ctx_destroy(gbrt_ctx* c) {
    if (!c) return GBRT_OK;
    jobs_shutdown(c);  // finishes the queued jobs, joins the scheduler
    {
        DeviceGuard g(c->device);
        if (c->stream) cudaStreamSynchronize(c->stream);
        c->counters.release();
        c->trace_work.release();
        c->scratch_rays.release();
        c->scratch_hits.release();
        c->scratch_img.release();
        c->scratch_samples.release();
        c->scratch_phits.release();
        c->wf_mem.release();
        c->wf_frame.release();
        stage_timer_free(c->timer);
        wave_ring_free(c->ring);
        if (c->side.stream) cudaStreamSynchronize(c->side.stream);
        if (c->side.shaded) cudaEventDestroy(c->side.shaded);
        if (c->side.shadowed) cudaEventDestroy(c->side.shadowed);
        if (c->side.stream) cudaStreamDestroy(c->side.stream);
        if (c->ev0) cudaEventDestroy(c->ev0);
        if (c->ev1) cudaEventDestroy(c->ev1);
        if (c->tb0) cudaEventDestroy(c->tb0);
        if (c->tb1) cudaEventDestroy(c->tb1);
        if (c->stream) cudaStreamDestroy(c->stream);
    }
    delete c;
    return GBRT_OK;
}

int gbrt_ctx_mem_info(gbrt_ctx* c, uint64_t* free_b, uint64_t* total_b) {
    if (!c || !free_b || !total_b) return fail(c, GBRT_E_INVALID, "NULL argument");
    DeviceGuard g(c->device);
    size_t f = 0, t = 0;
    CU(c, cudaMemGetInfo(&f, &t), "cudaMemGetInfo");
    *free_b = f;
    *total_b = t;
    return GBRT_OK;
}

int gbrt_sync(gbrt_ctx* c) {
    if (!c) return fail(c, GBRT_E_INVALID, "NULL context");
    DeviceGuard g(c->device);
    CU(c, cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    if (c->async_status.p) {
        uint32_t status = 0;
        CU(c, cudaMemcpy(&status, c->async_status.p, 4, cudaMemcpyDeviceToHost), "download status");
        if (status) {
            CU(c, cudaMemset(c->async_status.p, 0, 4), "memset");
            return fail(c, GBRT_E_DEVICE_LIMIT, "an asynchronous frame reported a traversal limit (status " +
                                                    std::to_string(status) + ")");
        }
    }
    return GBRT_OK;
}

int gbrt_scene_create(gbrt_ctx* c, const gbrt_vertex* v, uint32_t nv, const uint32_t* idx, uint32_t ni,
                      const gbrt_priminfo* prims, uint32_t ngeo, const gbrt_material_raw* mats, uint32_t nmat,
                      const gbrt_texture_desc* tex, uint32_t ntex, gbrt_scene** out) {
    if (!c || !out) return fail(c, GBRT_E_INVALID, "NULL argument");
    *out = nullptr;
    if ((nv && !v) || (ni && !idx) || (ngeo && !prims) || (nmat && !mats) || (ntex && !tex))
        return fail(c, GBRT_E_INVALID, "array pointer is NULL for a non-zero count");
    if (ni % 3 != 0) return fail(c, GBRT_E_INVALID, "index count is not a multiple of 3");
    for (uint32_t g = 0; g < ngeo; ++g)
        if (prims[g].material_id >= nmat)
            return fail(c, GBRT_E_INVALID, "geometry " + std::to_string(g) + " references a material out of range");
    DeviceGuard gd(c->device);
    gbrt_scene* s = new (std::nothrow) gbrt_scene();
    if (!s) return fail(c, GBRT_E_OOM, "host allocation failed");
    s->ctx = c;
    s->nv = nv;
    s->ni = ni;
    s->ngeo = ngeo;
    s->nmat = nmat;
    s->ntex = ntex;
    s->h_prims.assign(prims, prims + ngeo);
    s->h_indices.assign(idx, idx + ni);
    s->ranges.assign(ngeo, gbrt_geo_range{0, 0, 0, 1});
    s->has_range.assign(ngeo, 0);
    cudaStream_t st = c->stream;
    auto bail = [&](cudaError_t e, const char* what) {
        delete s;
        return cuda_fail(c, e, what);
    };
    cudaError_t e;
    if ((e = upload(s->vertices, v, nv, st)) != cudaSuccess) return bail(e, "upload(vertices)");
    if ((e = upload(s->indices, idx, ni, st)) != cudaSuccess) return bail(e, "upload(indices)");
    if ((e = upload(s->prims, prims, ngeo, st)) != cudaSuccess) return bail(e, "upload(prims)");
    if ((e = upload(s->mats, mats, nmat, st)) != cudaSuccess) return bail(e, "upload(materials)");
    s->shade_feat = material_features(mats, nmat);
    std::vector<DevTexture> dt(ntex);
    for (uint32_t i = 0; i < ntex; ++i) {
        const gbrt_texture_desc& t = tex[i];
        std::memset(&dt[i], 0, sizeof(DevTexture));
        if (t.format > GBRT_TEX_RGBA32F || t.wrap_s > 2 || t.wrap_t > 2) {
            delete s;
            return fail(c, GBRT_E_INVALID, "texture " + std::to_string(i) + ": bad format or wrap mode");
        }
        const size_t bytes = (size_t)t.width * t.height * texel_bytes(t.format);
        DevBuf* b = new DevBuf();
        s->tex_data.push_back(b);
        if (bytes && t.data) {
            if ((e = b->alloc(bytes)) != cudaSuccess) return bail(e, "cudaMalloc(texture)");
            if ((e = cudaMemcpyAsync(b->p, t.data, bytes, cudaMemcpyHostToDevice, st)) != cudaSuccess)
                return bail(e, "upload(texture)");
            dt[i].data = b->p;
            dt[i].w = t.width;
            dt[i].h = t.height;
        }
        dt[i].format = t.format;
        dt[i].wrap_s = t.wrap_s;
        dt[i].wrap_t = t.wrap_t;
    }
    if ((e = upload(s->tex_descs, dt.data(), dt.size(), st)) != cudaSuccess) return bail(e, "upload(texture descs)");
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return bail(e, "sync");
    refresh_view(s);
    *out = s;
    return GBRT_OK;
}

int gbrt_scene_destroy(gbrt_scene* s) {
    if (!s) return GBRT_OK;
    if (s->jobs_pending.load()) return fail(s->ctx, GBRT_E_BUSY, "jobs that render this scene are unfinished");
    DeviceGuard g(s->ctx->device);
    cudaStreamSynchronize(s->ctx->stream);
    delete s;
    return GBRT_OK;
}

int gbrt_blas_build(gbrt_scene* s, const gbrt_geo_range* r, uint32_t n, uint32_t flags) {
    if (!s) return GBRT_E_INVALID;
    gbrt_ctx* c = s->ctx;
    if (jobs_outstanding(c)) return fail(c, GBRT_E_BUSY, "jobs are running on this context");
    if (n && !r) return fail(c, GBRT_E_INVALID, "ranges is NULL");
    if (flags & ~(GBRT_BUILD_NO_FLATTEN | GBRT_BUILD_WIDTH4)) return fail(c, GBRT_E_INVALID, "unknown build flags");
    s->build_flags = flags;
    for (uint32_t i = 0; i < n; ++i) {
        const gbrt_geo_range& g = r[i];
        if (g.geo_id >= s->ngeo) return fail(c, GBRT_E_INVALID, "geo_id out of range");
        if (g.i_len % 3 != 0) return fail(c, GBRT_E_INVALID, "i_len % 3 != 0");  // acceleration_structures.rs:33
        const gbrt_priminfo& p = s->h_prims[g.geo_id];
        if ((uint64_t)p.i_offset + g.i_len > s->ni) return fail(c, GBRT_E_INVALID, "index range past the index buffer");
        if ((uint64_t)p.v_offset + g.v_len > s->nv) return fail(c, GBRT_E_INVALID, "vertex range past the vertex buffer");
        for (uint32_t k = 0; k < g.i_len; ++k)
            if (s->h_indices[p.i_offset + k] >= g.v_len)
                return fail(c, GBRT_E_INVALID, "geometry " + std::to_string(g.geo_id) + ": index " +
                                                   std::to_string(s->h_indices[p.i_offset + k]) + " >= v_len");
        s->ranges[g.geo_id] = g;
        s->has_range[g.geo_id] = 1;
    }
    s->built = false;
    return GBRT_OK;
}

int gbrt_tlas_build(gbrt_scene* s, const gbrt_instance* in, uint32_t n) {
    if (!s) return GBRT_E_INVALID;
    if (jobs_outstanding(s->ctx)) return fail(s->ctx, GBRT_E_BUSY, "jobs are running on this context");
    if (n && !in) return fail(s->ctx, GBRT_E_INVALID, "instances is NULL");
    DeviceGuard g(s->ctx->device);
    s->instances.assign(in, in + n);
    return build_all(s);
}

int gbrt_tlas_update(gbrt_scene* s, const gbrt_instance* in, uint32_t n) {
    if (!s) return GBRT_E_INVALID;
    gbrt_ctx* c = s->ctx;
    if (jobs_outstanding(c)) return fail(c, GBRT_E_BUSY, "jobs are running on this context");
    if (n && !in) return fail(c, GBRT_E_INVALID, "instances is NULL");
    if (!s->built) return fail(c, GBRT_E_NOT_BUILT, "build the TLAS with gbrt_tlas_build before updating it");
    if (n != s->instances.size()) return fail(c, GBRT_E_INVALID, "instance count differs from the built TLAS");
    DeviceGuard g(c->device);
    return update_instances(s, in, n);
}

int gbrt_skin_and_refit(gbrt_scene* s, const gbrt_skin_raw* skins, uint32_t nskin) {
    if (!s) return GBRT_E_INVALID;
    gbrt_ctx* c = s->ctx;
    if (nskin && !skins) return fail(c, GBRT_E_INVALID, "skins is NULL");
    if (!s->built) return fail(c, GBRT_E_NOT_BUILT, "build the TLAS before skinning");
    if (jobs_outstanding(c)) return fail(c, GBRT_E_BUSY, "jobs are running on this context");
    return skin_scene(s, skins, nskin);
}

int gbrt_lights_set(gbrt_scene* s, const gbrt_light_raw* d, uint32_t nd, const gbrt_light_raw* p, uint32_t np) {
    if (!s) return GBRT_E_INVALID;
    gbrt_ctx* c = s->ctx;
    if (jobs_outstanding(c)) return fail(c, GBRT_E_BUSY, "jobs are running on this context");
    if ((nd && !d) || (np && !p)) return fail(c, GBRT_E_INVALID, "lights pointer is NULL");
    DeviceGuard g(c->device);
    CU(c, upload(s->dlights, d, nd, c->stream), "upload(dlights)");
    CU(c, upload(s->plights, p, np, c->stream), "upload(plights)");
    CU(c, cudaStreamSynchronize(c->stream), "sync");
    s->nd = nd;
    s->np = np;
    refresh_view(s);
    return GBRT_OK;
}

int gbrt_skybox_set(gbrt_scene* s, uint32_t size, const uint8_t* faces) {
    return gbrt_skybox_set_ex(s, size, faces, GBRT_TEX_RGBA8_SRGB);
}

int gbrt_skybox_set_ex(gbrt_scene* s, uint32_t size, const void* faces, uint32_t format) {
    if (!s) return GBRT_E_INVALID;
    gbrt_ctx* c = s->ctx;
    if (format != GBRT_TEX_RGBA8_SRGB && format != GBRT_TEX_RGBA32F)
        return fail(c, GBRT_E_INVALID, "skybox format must be GBRT_TEX_RGBA8_SRGB or GBRT_TEX_RGBA32F");
    if (jobs_outstanding(c)) return fail(c, GBRT_E_BUSY, "jobs are running on this context");
    DeviceGuard g(c->device);
    if (!faces || size == 0) {
        s->sky.release();
        s->sky_size = 0;
    } else {
        const size_t bytes = (size_t)size * size * texel_bytes(format) * 6;
        CU(c, upload(s->sky, static_cast<const uint8_t*>(faces), bytes, c->stream), "upload(skybox)");
        CU(c, cudaStreamSynchronize(c->stream), "sync");
        s->sky_size = size;
    }
    s->sky_format = format;
    refresh_view(s);
    return GBRT_OK;
}

int gbrt_accum_create(gbrt_ctx* c, uint32_t w, uint32_t h, gbrt_accum** out) {
    if (!c || !out || w == 0 || h == 0) return fail(c, GBRT_E_INVALID, "bad accumulation size or NULL argument");
    *out = nullptr;
    DeviceGuard g(c->device);
    gbrt_accum* a = new (std::nothrow) gbrt_accum();
    if (!a) return fail(c, GBRT_E_OOM, "host allocation failed");
    a->ctx = c;
    a->w = w;
    a->h = h;
    cudaError_t e = a->buf.alloc((size_t)w * h * sizeof(float4));
    if (e == cudaSuccess) e = cudaMemsetAsync(a->buf.p, 0, a->buf.bytes, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        delete a;
        return cuda_fail(c, e, "accumulation buffer");
    }
    *out = a;
    return GBRT_OK;
}

int gbrt_accum_reset(gbrt_accum* a) {
    if (!a) return GBRT_E_INVALID;
    if (a->jobs_pending.load()) return fail(a->ctx, GBRT_E_BUSY, "a job writes this accumulation buffer");
    DeviceGuard g(a->ctx->device);
    CU(a->ctx, cudaMemsetAsync(a->buf.p, 0, a->buf.bytes, a->ctx->stream), "memset");
    return GBRT_OK;
}

int gbrt_accum_download(gbrt_accum* a, float* dst) {
    if (!a || !dst) return a ? fail(a->ctx, GBRT_E_INVALID, "dst is NULL") : GBRT_E_INVALID;
    if (a->jobs_pending.load()) return fail(a->ctx, GBRT_E_BUSY, "a job writes this accumulation buffer");
    DeviceGuard g(a->ctx->device);
    CU(a->ctx, cudaMemcpyAsync(dst, a->buf.p, a->buf.bytes, cudaMemcpyDeviceToHost, a->ctx->stream), "download");
    CU(a->ctx, cudaStreamSynchronize(a->ctx->stream), "sync");
    return GBRT_OK;
}

int gbrt_accum_upload(gbrt_accum* a, const float* src) {
    if (!a || !src) return a ? fail(a->ctx, GBRT_E_INVALID, "src is NULL") : GBRT_E_INVALID;
    if (a->jobs_pending.load()) return fail(a->ctx, GBRT_E_BUSY, "a job writes this accumulation buffer");
    DeviceGuard g(a->ctx->device);
    CU(a->ctx, cudaMemcpyAsync(a->buf.p, src, a->buf.bytes, cudaMemcpyHostToDevice, a->ctx->stream), "upload");
    CU(a->ctx, cudaStreamSynchronize(a->ctx->stream), "sync");
    return GBRT_OK;
}

int gbrt_accum_destroy(gbrt_accum* a) {
    if (!a) return GBRT_OK;
    if (a->jobs_pending.load()) return fail(a->ctx, GBRT_E_BUSY, "a job writes this accumulation buffer");
    DeviceGuard g(a->ctx->device);
    cudaStreamSynchronize(a->ctx->stream);
    delete a;
    return GBRT_OK;
}

int gbrt_render_ex(gbrt_scene* s, const gbrt_ubo* ubo, gbrt_accum* acc, uint8_t* out_rgba8, gbrt_stats* stats,
                   const gbrt_render_opts* opts) {
    if (!s) return GBRT_E_INVALID;
    gbrt_ctx* c = s->ctx;
    if (jobs_outstanding(c)) return fail(c, GBRT_E_BUSY, "jobs are running on this context");
    if (!ubo || !acc) return fail(c, GBRT_E_INVALID, "ubo or accumulation buffer is NULL");
    if (!s->built) return fail(c, GBRT_E_NOT_BUILT, "build the BLAS and TLAS before rendering");
    if (acc->ctx != c) return fail(c, GBRT_E_INVALID, "accumulation buffer belongs to another context");
    if (ubo->number_of_samples == 0 || ubo->total_number_of_samples < ubo->number_of_samples)
        return fail(c, GBRT_E_INVALID, "need 0 < number_of_samples <= total_number_of_samples");
    if (opts && opts->mode > GBRT_MODE_WAVEFRONT) return fail(c, GBRT_E_INVALID, "unknown render mode");
    const bool async = opts && (opts->flags & GBRT_RENDER_ASYNC);
    if (async && (opts->sample_radiance || opts->primary_hits || (opts->flags & GBRT_RENDER_STAGE_TIMING)))
        return fail(c, GBRT_E_INVALID, "asynchronous frames have no debug outputs or stage timing");
    DeviceGuard g(c->device);
    cudaStream_t st = c->stream;
    const uint32_t W = acc->w, H = acc->h, ns = ubo->number_of_samples;
    const size_t npix = (size_t)W * H;
    RenderOut out{};
    out.width = W;
    out.height = H;
    out.accum = acc->buf.as<float4>();
    out.counters = c->counters.as<DeviceCounters>();
    if (out_rgba8) {
        CU(c, c->scratch_img.reserve(npix * 4), "cudaMalloc(image)");
        out.rgba8 = c->scratch_img.as<uchar4>();
    }
    if (opts && opts->sample_radiance) {
        CU(c, c->scratch_samples.reserve(npix * ns * 3 * sizeof(float)), "cudaMalloc(samples)");
        out.sample_radiance = c->scratch_samples.as<float>();
    }
    if (opts && opts->primary_hits) {
        CU(c, c->scratch_phits.reserve(npix * ns * sizeof(gbrt_hit)), "cudaMalloc(primary hits)");
        out.primary_hits = c->scratch_phits.as<gbrt_hit>();
    }
    CU(c, cudaMemsetAsync(out.counters, 0, sizeof(DeviceCounters), st), "memset");
    CU(c, cudaEventRecord(c->ev0, st), "event");
    const uint32_t mode = opts ? opts->mode : GBRT_MODE_AUTO;
    const bool wave = (mode == GBRT_MODE_WAVEFRONT || mode == GBRT_MODE_AUTO) && ubo->number_of_bounces <= 31;
    if (mode == GBRT_MODE_WAVEFRONT && !wave) return fail(c, GBRT_E_INVALID, "the wavefront form handles at most 31 bounces");
    uint32_t launches = 1;
    if (wave) {
        const uint64_t paths = (uint64_t)npix * ns;
        const uint32_t cap = (uint32_t)std::min<uint64_t>(paths, kMaxWavePaths);
        CU(c, wavefront_reserve(c, cap, npix), "cudaMalloc(wavefront buffers)");
        const bool timed = opts && (opts->flags & GBRT_RENDER_STAGE_TIMING);
        CU(c, launch_wavefront(s->view, *ubo, out, c->wf, st, timed ? &c->timer : nullptr, nullptr, nullptr,
                               &c->side), "wavefront launch");
        const uint64_t npw = std::min<uint64_t>(npix, cap), k = cap / npw;
        const uint64_t waves = ((npix + npw - 1) / npw) * ((ns + k - 1) / k);
        launches = (uint32_t)(waves * (2 + 3 * ubo->number_of_bounces) + 1);
    } else {
        CU(c, launch_megakernel(s->view, *ubo, out, st), "megakernel launch");
    }
    CU(c, cudaEventRecord(c->ev1, st), "event");
    if (out_rgba8) CU(c, cudaMemcpyAsync(out_rgba8, out.rgba8, npix * 4, cudaMemcpyDeviceToHost, st), "download image");
    if (async) {  // the frame's status joins the context's; gbrt_sync reads it
        if (!c->async_status.p) {
            CU(c, c->async_status.alloc(4), "cudaMalloc(status)");
            CU(c, cudaMemsetAsync(c->async_status.p, 0, 4, st), "memset");
        }
        or_status_kernel<<<1, 1, 0, st>>>(out.counters, c->async_status.as<uint32_t>());
        CU(c, cudaGetLastError(), "status launch");
        if (stats) {
            std::memset(stats, 0, sizeof(*stats));
            stats->kernel_launches = launches;
        }
        return GBRT_OK;
    }
    if (out.sample_radiance)
        CU(c, cudaMemcpyAsync(opts->sample_radiance, out.sample_radiance, npix * ns * 3 * sizeof(float),
                              cudaMemcpyDeviceToHost, st),
           "download samples");
    if (out.primary_hits)
        CU(c, cudaMemcpyAsync(opts->primary_hits, out.primary_hits, npix * ns * sizeof(gbrt_hit),
                              cudaMemcpyDeviceToHost, st),
           "download hits");
    DeviceCounters dc;
    CU(c, cudaMemcpyAsync(&dc, out.counters, sizeof(dc), cudaMemcpyDeviceToHost, st), "download counters");
    CU(c, cudaStreamSynchronize(st), "render");
    float ms = 0.0f;
    CU(c, cudaEventElapsedTime(&ms, c->ev0, c->ev1), "event time");
    fill_stats(stats, dc, ms, launches);
    if (stats && wave && opts && (opts->flags & GBRT_RENDER_STAGE_TIMING))
        CU(c, stage_timer_collect(c->timer, stats->stage_ms), "stage timing");
    if (dc.status) return fail(c, GBRT_E_DEVICE_LIMIT, "a kernel reported a traversal limit (status " +
                                                            std::to_string(dc.status) + ")");
    return GBRT_OK;
}

int gbrt_scene_autotune(gbrt_scene* s, const gbrt_ubo* ubo, uint32_t width, uint32_t height, gbrt_tune_report* rep) {
    if (!s) return GBRT_E_INVALID;
    gbrt_ctx* c = s->ctx;
    if (!ubo || width == 0 || height == 0) return fail(c, GBRT_E_INVALID, "NULL probe UBO or empty probe image");
    if (!s->built) return fail(c, GBRT_E_NOT_BUILT, "build the BLAS and TLAS before tuning");
    if (jobs_outstanding(c)) return fail(c, GBRT_E_BUSY, "jobs are running on this context");
    if (ubo->number_of_bounces > 31 || ubo->number_of_samples == 0)
        return fail(c, GBRT_E_INVALID, "probe needs 1..31 bounces and at least one sample");
    DeviceGuard g(c->device);
    cudaStream_t st = c->stream;
    const size_t npix = (size_t)width * height;
    const uint64_t paths = (uint64_t)npix * ubo->number_of_samples;
    CU(c, wavefront_reserve(c, (uint32_t)std::min<uint64_t>(paths, kMaxWavePaths), npix), "cudaMalloc(wavefront)");
    DevBuf probe;
    CU(c, probe.alloc(npix * sizeof(float4)), "cudaMalloc(probe image)");
    RenderOut out{};
    out.width = width;
    out.height = height;
    out.accum = probe.as<float4>();
    out.counters = c->counters.as<DeviceCounters>();
    gbrt_ubo u = *ubo;
    u.total_number_of_samples = u.number_of_samples;
    // one probe: best of rounds 2 and 3 (the first warms up)
    auto probe_ms = [&](bool binary, double* best) -> int {
        *best = 1e30;
        for (int rep_i = 0; rep_i < 3; ++rep_i) {
            DevScene v = s->view;
            v.prefer_binary = binary ? 1u : 0u;
            CU(c, cudaEventRecord(c->ev0, st), "event");
            CU(c, launch_wavefront(v, u, out, c->wf, st, nullptr, nullptr, nullptr, &c->side), "probe render");
            CU(c, cudaEventRecord(c->ev1, st), "event");
            CU(c, cudaStreamSynchronize(st), "sync");
            float ms = 0.0f;
            CU(c, cudaEventElapsedTime(&ms, c->ev0, c->ev1), "event time");
            if (rep_i > 0) *best = std::min(*best, (double)ms);
        }
        return GBRT_OK;
    };
    const bool has_wide = s->view.cw_nodes != nullptr || !s->view.has_world;
    // ms[layout][sort]: layout 0 binary, 1 4-wide, 2 8-wide
    double ms[3][2] = {{0.0, 0.0}, {0.0, 0.0}, {0.0, 0.0}};
    auto probe_both = [&](int layout) -> int {
        for (int so = 0; so < 2; ++so) {
            s->view.sort_rays = (uint32_t)so;
            const int r = probe_ms(layout == 0, &ms[layout][so]);
            if (r != GBRT_OK) return r;
        }
        return GBRT_OK;
    };
    int rc = probe_both(0);
    if (rc != GBRT_OK) return rc;
    int best_l = 0, best_s = ms[0][1] < ms[0][0] ? 1 : 0;
    if (has_wide) {
        const int l0 = cw_width(s) == 4 ? 1 : 2;
        if ((rc = probe_both(l0)) != GBRT_OK) return rc;
        // the other width: rebuild, probe
        s->build_flags ^= GBRT_BUILD_WIDTH4;
        if ((rc = build_all(s)) != GBRT_OK) return rc;
        if ((rc = probe_both(3 - l0)) != GBRT_OK) return rc;
        for (int l = 1; l < 3; ++l)
            for (int so = 0; so < 2; ++so)
                if (ms[l][so] < ms[best_l][best_s]) {
                    best_l = l;
                    best_s = so;
                }
        // keep the wide BVH at the better width (the binary one is the same either way)
        const int keep = best_l ? best_l : (std::min(ms[1][0], ms[1][1]) < std::min(ms[2][0], ms[2][1]) ? 1 : 2);
        if (keep == l0) {
            s->build_flags ^= GBRT_BUILD_WIDTH4;
            if ((rc = build_all(s)) != GBRT_OK) return rc;
        }
    }
    s->view.prefer_binary = best_l == 0 ? 1u : 0u;
    s->view.sort_rays = (uint32_t)best_s;
    if (rep) {
        rep->ms_binary = ms[0][0];
        rep->ms_wide = ms[2][0];
        rep->ms_wide4 = ms[1][0];
        rep->ms_sorted = ms[best_l][1];
        rep->chosen_width = best_l == 0 ? 2u : (uint32_t)cw_width(s);
        rep->sort_rays = s->view.sort_rays;
    }
    return GBRT_OK;
}

int gbrt_scene_info_get(gbrt_scene* s, gbrt_scene_info* info) {
    if (!s) return GBRT_E_INVALID;
    if (!info) return fail(s->ctx, GBRT_E_INVALID, "NULL info");
    std::memset(info, 0, sizeof(*info));
    info->world_triangles = s->nworld;
    info->wide_nodes = s->cw_count;
    info->wide_width = (uint32_t)cw_width(s);
    info->refits = s->refits;
    info->drift_rebuilds = s->rebuilds;
    info->instance_updates = s->instance_updates;
    info->sah_built = s->cw_sah0;
    info->sah_now = s->cw_sah;
    return GBRT_OK;
}

int gbrt_scene_set_tuning(gbrt_scene* s, uint32_t width, uint32_t sort_rays) {
    if (!s) return GBRT_E_INVALID;
    gbrt_ctx* c = s->ctx;
    if (width != 2 && width != 4 && width != 8) return fail(c, GBRT_E_INVALID, "width must be 2, 4 or 8");
    if (!s->built) return fail(c, GBRT_E_NOT_BUILT, "build the BLAS and TLAS before tuning");
    if (jobs_outstanding(c)) return fail(c, GBRT_E_BUSY, "jobs are running on this context");
    DeviceGuard g(c->device);
    if (width != 2 && (uint32_t)cw_width(s) != width) {
        s->build_flags ^= GBRT_BUILD_WIDTH4;
        const int rc = build_all(s);
        if (rc != GBRT_OK) return rc;
    }
    s->view.prefer_binary = width == 2 ? 1u : 0u;
    s->view.sort_rays = sort_rays ? 1u : 0u;
    return GBRT_OK;
}

int gbrt_render(gbrt_scene* s, const gbrt_ubo* ubo, gbrt_accum* acc, uint8_t* out_rgba8, gbrt_stats* stats) {
    return gbrt_render_ex(s, ubo, acc, out_rgba8, stats, nullptr);
}

int gbrt_trace_rays_device(gbrt_scene* s, const gbrt_ray* d_rays, uint32_t n, uint32_t flags, gbrt_hit* d_hits) {
    if (!s) return GBRT_E_INVALID;
    gbrt_ctx* c = s->ctx;
    if (n && (!d_rays || !d_hits)) return fail(c, GBRT_E_INVALID, "rays or hits is NULL");
    if (!s->built) return fail(c, GBRT_E_NOT_BUILT, "build the BLAS and TLAS before tracing");
    if (jobs_outstanding(c)) return fail(c, GBRT_E_BUSY, "jobs are running on this context");
    DeviceGuard g(c->device);
    CU(c, launch_trace_rays_persistent(s->view, d_rays, n, flags, d_hits, c->trace_work.as<uint32_t>(), nullptr,
                                       c->stream),
       "trace launch");
    return GBRT_OK;
}

int gbrt_trace_rays(gbrt_scene* s, const gbrt_ray* rays, uint32_t n, uint32_t flags, gbrt_hit* hits,
                    gbrt_stats* stats) {
    if (!s) return GBRT_E_INVALID;
    gbrt_ctx* c = s->ctx;
    if (jobs_outstanding(c)) return fail(c, GBRT_E_BUSY, "jobs are running on this context");
    if (n && (!rays || !hits)) return fail(c, GBRT_E_INVALID, "rays or hits is NULL");
    if (!s->built) return fail(c, GBRT_E_NOT_BUILT, "build the BLAS and TLAS before tracing");
    DeviceGuard g(c->device);
    cudaStream_t st = c->stream;
    CU(c, c->scratch_rays.reserve((size_t)std::max(n, 1u) * sizeof(gbrt_ray)), "cudaMalloc(rays)");
    CU(c, c->scratch_hits.reserve((size_t)std::max(n, 1u) * sizeof(gbrt_hit)), "cudaMalloc(hits)");
    DeviceCounters* dcnt = c->counters.as<DeviceCounters>();
    CU(c, cudaMemsetAsync(dcnt, 0, sizeof(DeviceCounters), st), "memset");
    if (n) CU(c, cudaMemcpyAsync(c->scratch_rays.p, rays, n * sizeof(gbrt_ray), cudaMemcpyHostToDevice, st), "upload rays");
    CU(c, cudaEventRecord(c->ev0, st), "event");
    CU(c, launch_trace_rays_persistent(s->view, c->scratch_rays.as<gbrt_ray>(), n, flags,
                                       c->scratch_hits.as<gbrt_hit>(), c->trace_work.as<uint32_t>(), dcnt, st),
       "trace launch");
    CU(c, cudaEventRecord(c->ev1, st), "event");
    if (n) CU(c, cudaMemcpyAsync(hits, c->scratch_hits.p, n * sizeof(gbrt_hit), cudaMemcpyDeviceToHost, st), "download hits");
    DeviceCounters dc;
    CU(c, cudaMemcpyAsync(&dc, dcnt, sizeof(dc), cudaMemcpyDeviceToHost, st), "download counters");
    CU(c, cudaStreamSynchronize(st), "trace");
    float ms = 0.0f;
    CU(c, cudaEventElapsedTime(&ms, c->ev0, c->ev1), "event time");
    dc.camera = n;
    fill_stats(stats, dc, ms, n ? 1 : 0);
    if (dc.status) return fail(c, GBRT_E_DEVICE_LIMIT, "a kernel reported a traversal limit");
    return GBRT_OK;
}

int gbrt_device_alloc(gbrt_ctx* c, uint64_t bytes, void** p) {
    if (!c || !p) return fail(c, GBRT_E_INVALID, "NULL argument");
    DeviceGuard g(c->device);
    CU(c, cudaMalloc(p, bytes), "cudaMalloc");
    return GBRT_OK;
}
int gbrt_device_free(gbrt_ctx* c, void* p) {
    if (!c) return GBRT_E_INVALID;
    DeviceGuard g(c->device);
    CU(c, cudaFree(p), "cudaFree");
    return GBRT_OK;
}
int gbrt_memcpy_h2d(gbrt_ctx* c, void* d, const void* h, uint64_t bytes) {
    if (!c) return GBRT_E_INVALID;
    DeviceGuard g(c->device);
    CU(c, cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, c->stream), "h2d");
    CU(c, cudaStreamSynchronize(c->stream), "sync");
    return GBRT_OK;
}
int gbrt_memcpy_d2h(gbrt_ctx* c, void* h, const void* d, uint64_t bytes) {
    if (!c) return GBRT_E_INVALID;
    DeviceGuard g(c->device);
    CU(c, cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, c->stream), "d2h");
    CU(c, cudaStreamSynchronize(c->stream), "sync");
    return GBRT_OK;
}
int gbrt_timer_begin(gbrt_ctx* c) {
    if (!c) return GBRT_E_INVALID;
    DeviceGuard g(c->device);
    CU(c, cudaEventRecord(c->tb0, c->stream), "event");
    return GBRT_OK;
}
int gbrt_timer_end(gbrt_ctx* c, double* ms) {
    if (!c || !ms) return fail(c, GBRT_E_INVALID, "NULL argument");
    DeviceGuard g(c->device);
    CU(c, cudaEventRecord(c->tb1, c->stream), "event");
    CU(c, cudaEventSynchronize(c->tb1), "event sync");
    float f = 0;
    CU(c, cudaEventElapsedTime(&f, c->tb0, c->tb1), "event time");
    *ms = f;
    return GBRT_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free world-BVH rebuild.
//
// For callers that must not allocate device memory while they run: a frame
// loop that rebuilds the BVH of a deforming mesh every frame (cudaMalloc and
// cudaFree can synchronise the whole device and stall the frame), a host whose
// device memory belongs to another allocator or budget (a Vulkan or engine
// heap, a serving process under a hard memory cap), or code that cannot
// afford to fail with out-of-memory half way through a frame.  The build's
// scratch (Morton keys, radix tree, subtree boxes, sort temporary storage) lives
// in the file-scope array below, which every GPU that loads the library keeps
// until the process exits.
// ---------------------------------------------------------------------------
namespace {

constexpr uint32_t kNoallocMaxTriangles = GBRT_NOALLOC_MAX_TRIANGLES;
constexpr size_t kNoallocScratchBytes = size_t(12) << 20;  // 12 MiB, checked against the layout at set-up
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kMaxDevices] = {};

// Once per device, with that device current: the device address of the
// scratch array (the host-side name of the array is not a device address).
int noalloc_setup(gbrt_ctx* c, void** out) {
    if (c->device < 0 || c->device >= kMaxDevices) return fail(c, GBRT_E_INVALID, "device index too large");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[c->device]) {
        if (bvh_scratch_bytes(kNoallocMaxTriangles) > kNoallocScratchBytes)
            return fail(c, GBRT_E_INVALID, "static build scratch is smaller than the build layout needs");
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(c, e, "cudaGetSymbolAddress(build scratch)");
        g_noalloc_ptr[c->device] = p;
    }
    *out = g_noalloc_ptr[c->device];
    return GBRT_OK;
}

}  // namespace

extern "C" int gbrt_scene_rebuild_noalloc(gbrt_scene* s, const gbrt_vertex* d_vertices) {
    if (!s) return GBRT_E_INVALID;
    gbrt_ctx* c = s->ctx;
    // queued jobs read this scene's BVH and host view from the job thread
    if (jobs_outstanding(c)) return fail(c, GBRT_E_BUSY, "jobs are running on this context");
    if (!s->built) return fail(c, GBRT_E_NOT_BUILT, "build the TLAS with gbrt_tlas_build before rebuilding");
    bool transformed = s->view.has_tlas;  // flattened transformed instances have no TLAS but count too
    for (const gbrt_instance& in : s->instances)
        transformed = transformed || ((in.custom_index_and_mask >> 24) != 0 && !is_identity(in.transform));
    if (transformed)
        return fail(c, GBRT_E_INVALID,
                    "the allocation-free rebuild covers scenes whose instances all have identity transforms");
    if (!s->view.has_world) return fail(c, GBRT_E_NOT_BUILT, "the scene has no world BVH");
    const size_t n = s->items.bytes / sizeof(uint4);
    if (n > kNoallocMaxTriangles)
        return fail(c, GBRT_E_INVALID, "world BVH has " + std::to_string(n) + " triangles; the allocation-free " +
                                           "rebuild handles at most " + std::to_string(kNoallocMaxTriangles));
    DeviceGuard g(c->device);
    void* base = nullptr;
    int rc = noalloc_setup(c, &base);
    if (rc != GBRT_OK) return rc;
    cudaStream_t st = c->stream;
    // From here on the vertices and BVH pools are overwritten in place: after a
    // failure they describe neither the old nor the new geometry, so the scene
    // answers GBRT_E_NOT_BUILT until gbrt_tlas_build builds it again.
    auto broken = [&](cudaError_t e, const char* what) {
        s->built = false;
        return cuda_fail(c, e, what);
    };
    cudaError_t e = cudaSuccess;
    if (d_vertices &&
        (e = cudaMemcpyAsync(s->vertices.p, d_vertices, s->vertices.bytes, cudaMemcpyDeviceToDevice, st)) !=
            cudaSuccess)
        return broken(e, "copy vertices");
    const BuildScratch scratch = bvh_scratch_carve(base, kNoallocMaxTriangles);
    BvhResult r;
    if ((e = build_triangle_bvh_scratch(scratch, s->vertices.as<gbrt_vertex>(), s->indices.as<uint32_t>(),
                                        s->prims.as<gbrt_priminfo>(), s->items.as<uint4>(), (uint32_t)n,
                                        s->nodes.as<BNode2>(), 0, s->tris.as<TriRec>(), 0, &r, st)) != cudaSuccess)
        return broken(e, "allocation-free BVH rebuild");
    // The wide copy of the world BVH keeps its topology and is refit in place
    // into the box buffer reserved at build time (kernels only, no allocation).
    const bool wide = s->cw_count && s->cw_levels.size() >= 2 &&
                      s->cw_boxes.bytes >= (size_t)s->cw_count * 2 * sizeof(float4) + 16;
    double sah = 0.0;
    if (wide && (e = refit_triangle_cwbvh(s->vertices.as<gbrt_vertex>(), s->indices.as<uint32_t>(),
                                          s->prims.as<gbrt_priminfo>(), s->cw_nodes.as<CwNode>(),
                                          s->cw_tris.as<TriRec>(), s->nworld, s->cw_levels, s->cw_boxes.as<float4>(),
                                          st, s->inst.as<DevInstance>(), &sah)) != cudaSuccess)
        return broken(e, "allocation-free refit of the wide BVH");
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return broken(e, "sync after rebuild");
    s->view.world_root = r.root;
    s->view.world_lo = r.lo;
    s->view.world_hi = r.hi;
    if (wide) {
        ++s->refits;
        s->cw_sah = sah;
    } else {  // no wide copy to refit: traversal uses the rebuilt binary BVH
        s->cw_count = 0;
    }
    refresh_view(s);
    return GBRT_OK;
}
