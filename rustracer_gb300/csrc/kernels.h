// kernels.h — host-visible launchers of the device code.
#pragma once
#include <cuda_runtime.h>
#include <vector>
#include "scene.cuh"

namespace gbrt {

struct DeviceCounters {
    unsigned long long camera, extension, shadow, shaded, nodes, tris;
    unsigned int status;
    unsigned int _pad;
};

struct RenderOut {
    uint32_t width, height;
    float4* accum;             // width*height running sums (required)
    uchar4* rgba8;             // tone-mapped image, may be null
    float* sample_radiance;    // [pixel][sample][3], may be null
    gbrt_hit* primary_hits;    // [pixel][sample], may be null
    DeviceCounters* counters;  // required
};

// wavefront.cu: device buffers of the wavefront path tracer, `cap` paths.
// Each job of a wave owns kWfCounters queue lengths and fetch cursors.
constexpr int kWfCounters = 128;
#ifndef GBRT_PID_BITS
#define GBRT_PID_BITS 26
#endif
constexpr uint32_t kPidBits = GBRT_PID_BITS;         // path id bits of a queue entry (segment: the rest)
static_assert(kPidBits <= 26, "queue words keep at least 6 bits of segment index");
constexpr uint32_t kMaxWavePaths = 1u << kPidBits;   // paths per wave
constexpr int kMaxWaveJobs = 32;                     // jobs sharing one wave
constexpr int kMaxWaveSegs = kPidBits <= 24 ? 256 : (1 << (32 - kPidBits));  // (pixels x samples) pieces per wave
struct WfState {
    uint32_t cap;
    float4* ray_o[2];   // extension queues (ping-pong): origin (the path's hit point), RandomSeed in .w
    float4* ray_d[2];   //   direction, path id | segment << kPidBits in .w
    float4* hit;        // t, u, v, instance id
    uint32_t* hit_prim;
    float4* q_tp[2];    // beside the extension queues: the path's throughput, Ray.t
    uint4* q_rng[2];    //   pixel-stream counter, ray-stream counter, ray-stream z
    float4* q_rad[2];   //   radiance, volume_dis
    float4* rad;        // per path, once it has ended: radiance, last Ray.t (the whole way in cache frames)
    float4* tp;         //   throughput, Ray.t, and
    uint4* rng;         //   RNG counters, in frames with a radiance cache (which reads them by path id)
    float4* sh_o;       // shadow queue: origin, tmax
    float4* sh_d;       //   direction, path id
    // the path's radiance (and volume_dis) after this vertex if the shadow ray
    // is blocked / unblocked, and in sh_tp the bits of where it goes (the
    // path's next queue slot | kDstQueue, or its path id if it has ended); in
    // frames with a radiance cache (kShadowDelta) instead emission E +
    // throughput.x / NEE term C + throughput.y, added to the path's radiance by
    // the shadow kernel with throughput.z from sh_tp
    float4* sh_e;
    float4* sh_c;
    float* sh_tp;
    uint32_t* counts;   // kMaxWaveJobs * kWfCounters queue lengths and fetch cursors
    float4* frame_sum;  // per pixel: sum of the frame's samples, last Ray.t (single-frame renders)
};
// WaveJob::flags bit: the job's shadow records hold deltas (sh_e / sh_c).
constexpr uint32_t kShadowDelta = 0x80000000u;
// sh_tp destination bit: the radiance goes to q_rad at that queue slot.
constexpr uint32_t kDstQueue = 0x80000000u;

// One job of a wave: a scene, its UBO and its outputs.  The job's paths are
// the contiguous range [path0, path0 + npaths) of the wave; its queues live
// at the same offsets of the wave's queue arrays.
struct WaveJob {
    DevScene s;
    gbrt_ubo ubo;
    RenderOut out;
    float4* frame_sum;  // per pixel of the job's image
    uint32_t ns;        // samples of the frame (stride of the per-sample outputs)
    uint32_t flags;     // GBRT_RAY_OPAQUE when the UBO says fully_opaque; kShadowDelta
    float tfar;
    uint32_t path0, npaths;
};
// k samples [sample0, sample0 + k) of the pixels [px0, px0 + npw) of a job;
// path path0 + j * npw + i is sample j of pixel px0 + i.
struct WaveSeg {
    uint32_t path0, job, px0, npw, sample0, si0, k, fin0;  // fin0: first thread of wf_finish
};
struct WaveDesc {
    uint32_t njobs, nsegs, npaths, nfin, nb;
    // per stage (extend, shade, shadow): first block of every job, [njobs] = grid size
    uint32_t blk[3][kMaxWaveJobs + 1];
    WaveJob jobs[kMaxWaveJobs];
    WaveSeg segs[kMaxWaveSegs];
};
// Pinned host copies of wave descriptors, reused round-robin; slot i may be
// rewritten once ev[i] (recorded after its upload) has completed.
struct WaveRing {
    static constexpr int kSlots = 4;
    WaveDesc* host = nullptr;
    cudaEvent_t ev[kSlots] = {};
    int next = 0;
    // captured launch sequences of batched waves, per traversal form (with
    // or without kTraceOpaque) and bounce count, valid for the wavefront
    // buffers in graph_state
    cudaGraphExec_t graph[8][32] = {};
    WfState graph_state{};
    // private stream the graphs are captured on: the launch stream is shared
    // with the API calls of other threads, which must not land in a capture
    cudaStream_t cap = nullptr;
};
// Drops the captured graphs (the ring's buffers stay).
void wave_graphs_reset(WaveRing& r);
cudaError_t wave_ring_init(WaveRing& r);
void wave_ring_free(WaveRing& r);
// Waits until the next slot is free and returns it for filling.
cudaError_t wave_acquire(WaveRing& r, WaveDesc** slot);

// Radiance-cache state of a wavefront frame (gbrt_render_nrc).  A path's
// cache vertex is its first hit at bounce >= 1 whose material roughness is
// at least min_roughness.  Render paths stop there and take throughput x
// cache(position); training paths (hash of pixel and sample below
// train_thresh / 65536) trace on and yield one sample: position -> the
// radiance their suffix gathered from that vertex divided by the throughput
// that reached it.
struct NrcWave {
    float4* query;      // [cap] (position, queue word) of stopped render paths, per bounce
    float4* qout;       // [cap] cache output for them
    float4* snap_pos;   // [cap] per path: the training vertex (w = 1 once set)
    float4* snap_rad;   // [cap] radiance before it
    float4* snap_tp;    // [cap] throughput reaching it
    float4* train_pos;  // [train_max] training samples
    float4* train_tgt;
    uint32_t* counts;   // [b] queries of bounce b, [32] training samples
    uint32_t train_max;
    uint32_t train_thresh;
    float min_roughness;
    uint32_t disabled;  // 1: no path stops at the cache (plain path tracing plus training samples)
    uint32_t mode;      // GBRT_NRC_MODE_*: 0 the cache vertex is the first rough hit after the camera hit;
                        // 1 (primary indirect) the camera hit, whose indirect radiance the cache returns
};

// CUDA-event pairs around every wavefront launch, grouped by stage
// (0 extend, 1 shade, 2 shadow, 3 other).  Events are created on demand and
// reused across frames.
struct StageTimer {
    cudaEvent_t* ev = nullptr;  // 2 * capacity events
    int* stage = nullptr;       // stage of each pair
    int capacity = 0, used = 0;
};
size_t wavefront_bytes_per_path();
cudaError_t init_wavefront_constants(const float* srgb_lut);
cudaError_t init_wave_multi_constants(const float* srgb_lut);
// Grows a timer to hold `pairs` event pairs, keeping the pairs recorded so far.
cudaError_t stage_timer_reserve(StageTimer& t, int pairs);
// Fills the per-stage block partition of `w` (blocks in proportion to each
// job's paths, at least one) for the current device.
cudaError_t wave_partition(WaveDesc& w);
// Uploads the slot wave_acquire returned and launches one wave: camera, `w.nb` x
// (extend, shade, shadow), finish.  Launch count: 2 + 3 * w.nb.
cudaError_t launch_wave(WaveRing& ring, const WfState& st, cudaStream_t stream, StageTimer* timer);
// Accumulate + tone map of one finished frame (rgen:132-166).
cudaError_t launch_resolve(const gbrt_ubo& ubo, const RenderOut& out, const float4* frame_sum, cudaStream_t stream);
// A whole frame of one scene: waves of at most st.cap paths, then resolve.
// With `nrc` (and `cache`, the gbrt_nrc to query), paths stop at the radiance
// cache as NrcWave describes.
// A second stream for the shadow stage: shadow(b) runs beside extend(b + 1)
// (they touch disjoint state) and shade(b + 1) waits for it, so each
// launch's tail overlaps the other's work.
struct WfSide {
    cudaStream_t stream = nullptr;
    cudaEvent_t shaded = nullptr, shadowed = nullptr;
};
cudaError_t launch_wavefront(const DevScene& s, const gbrt_ubo& ubo, const RenderOut& out, const WfState& st,
                             cudaStream_t stream, StageTimer* timer = nullptr, const NrcWave* nrc = nullptr,
                             gbrt_nrc* cache = nullptr, const WfSide* side = nullptr);
// Ray queries through the persistent world traversal (8-wide when built);
// `work` is one device word used as the fetch cursor.
cudaError_t launch_trace_rays_persistent(const DevScene& s, const gbrt_ray* rays, uint32_t n, uint32_t flags,
                                         gbrt_hit* hits, uint32_t* work, DeviceCounters* cnt, cudaStream_t st);
// Sums the recorded pairs per stage (call after the stream synchronised).
cudaError_t stage_timer_collect(StageTimer& t, double ms[4]);
void stage_timer_free(StageTimer& t);

// render.cu
cudaError_t init_render_constants(const float* srgb_lut);
cudaError_t launch_megakernel(const DevScene& s, const gbrt_ubo& ubo, const RenderOut& out, cudaStream_t st);
cudaError_t launch_trace_rays(const DevScene& s, const gbrt_ray* rays, uint32_t n, uint32_t flags, gbrt_hit* hits,
                              DeviceCounters* cnt, cudaStream_t st);

// bvh_build.cu -------------------------------------------------------------
// A BVH over n items is written into the scene pools: inner nodes at
// nodes[node_base ...], the items' TriRec slots (in leaf order) at
// tris[tri_base ... tri_base + n).  The root is an inner node index or a
// leaf code.
struct BvhResult {
    int32_t root;
    float4 lo, hi;  // root bounds
};

// Binary-tree construction of the BVH builders: kBvhPloc clusters the items
// (parallel locally-ordered clustering, better trees, a host wait per
// round), kBvhFast splits the Morton order (Karras radix tree, one launch).
constexpr int kBvhFast = 0, kBvhPloc = 1;

// Item descriptors for triangle BVHs: x = instance id (world BVH) or 0,
// y = BLAS geometry id, z = primitive id, w = opaque flag.
// inst (may be null): items whose instance is not an identity one are
// transformed to world space (flattened instances).
cudaError_t build_triangle_bvh(const gbrt_vertex* vertices, const uint32_t* indices, const gbrt_priminfo* prims,
                               const uint4* items, uint32_t n, BNode2* nodes, uint32_t node_base, TriRec* tris,
                               uint32_t tri_base, BvhResult* result_host, cudaStream_t st,
                               const DevInstance* inst = nullptr, int quality = kBvhPloc);

// Scratch of one triangle-BVH build supplied by the caller instead of being
// allocated (every pointer 256-byte aligned, sized for `capacity` items).
struct BuildScratch {
    uint32_t capacity;
    float4 *lo, *hi, *ilo, *ihi;
    uint32_t *morton_in, *morton, *idx_in, *idx, *range_lo, *range_hi, *collapse, *arrive, *cbounds;
    int32_t *left, *right, *parent_i, *parent_l;
    float* cost;
    TriRec* unsorted;
    void* sort_tmp;
    size_t sort_tmp_bytes;
};
// Bytes of radix-sort temporary storage a build over n items needs.
size_t bvh_sort_temp_bytes(uint32_t n);
// Bytes a BuildScratch for `capacity` items takes when carved from one
// 256-byte-aligned block (including the sort temporary storage).
size_t bvh_scratch_bytes(uint32_t capacity);
// Carves a BuildScratch for `capacity` items out of `base` (bvh_scratch_bytes
// bytes, 256-byte aligned).
BuildScratch bvh_scratch_carve(void* base, uint32_t capacity);
// Same build as build_triangle_bvh, with n <= scratch.capacity and no device
// allocation.
cudaError_t build_triangle_bvh_scratch(const BuildScratch& scratch, const gbrt_vertex* vertices,
                                       const uint32_t* indices, const gbrt_priminfo* prims, const uint4* items,
                                       uint32_t n, BNode2* nodes, uint32_t node_base, TriRec* tris,
                                       uint32_t tri_base, BvhResult* result_host, cudaStream_t st);

// Compressed 8-wide BVH over n triangle items: nodes (capacity n, root at 0)
// and their triangles (n slots, node-leaf order); *nodes_used (host) gets
// the node count.  width 4 collapses to at most 4 children per node (same
// node format, so the same traversal).
cudaError_t build_triangle_cwbvh(const gbrt_vertex* vertices, const uint32_t* indices, const gbrt_priminfo* prims,
                                 const uint4* items, uint32_t n, CwNode* nodes, TriRec* tris, uint32_t* nodes_used,
                                 cudaStream_t st, std::vector<uint32_t>* level_starts = nullptr,
                                 const DevInstance* inst = nullptr, int width = 8, int quality = kBvhPloc);
// Refit of an 8-wide BVH built by build_triangle_cwbvh over the same
// triangles: triangle records re-read from the vertices, then every node's
// grid and child boxes recomputed level by level (level_starts: first node
// of each level, last entry = node count).  boxes: scratch of 2 float4 per
// node plus one float.  No host synchronisation unless sah_host is given: it
// then gets the tree's SAH traversal cost proxy, the summed surface area of
// every node's child boxes over the root box's (the expected child-box tests
// of a ray through the root), after a host wait.
cudaError_t refit_triangle_cwbvh(const gbrt_vertex* vertices, const uint32_t* indices, const gbrt_priminfo* prims,
                                 CwNode* nodes, TriRec* tris, uint32_t ntris, const std::vector<uint32_t>& level_starts,
                                 float4* boxes, cudaStream_t st, const DevInstance* inst = nullptr,
                                 double* sah_host = nullptr);

// TLAS over instances: boxes given per instance (lo/hi), the leaf slots carry
// the instance ids.
cudaError_t build_instance_bvh(const float4* lo, const float4* hi, const uint32_t* inst_ids, uint32_t n,
                               BNode2* nodes, uint32_t node_base, TriRec* tris, uint32_t tri_base,
                               BvhResult* result_host, cudaStream_t st, int quality = kBvhPloc);

// Refit: recomputes every inner-node box of a triangle BVH bottom-up from the
// current vertex positions, keeping the topology (used after skinning).
cudaError_t refit_triangle_bvh(const gbrt_vertex* vertices, const uint32_t* indices, const gbrt_priminfo* prims,
                               BNode2* nodes, uint32_t node_base, uint32_t num_inner, TriRec* tris,
                               uint32_t tri_base, uint32_t n, const int32_t* parents, int32_t root,
                               BvhResult* result_host, cudaStream_t st);

// World boxes of transformed instances from their BLAS root bounds.
cudaError_t instance_world_boxes(const DevInstance* inst, const uint32_t* ids, const float4* blas_lo,
                                 const float4* blas_hi, uint32_t n, float4* lo, float4* hi, cudaStream_t st);

// skin.cu
cudaError_t launch_skinning(const gbrt_vertex* vin, gbrt_vertex* vout, uint32_t nv, const gbrt_skin_raw* skins,
                            uint32_t nskin, cudaStream_t st);

}  // namespace gbrt
