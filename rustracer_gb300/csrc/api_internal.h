// api_internal.h -- host-side objects behind the C ABI handles, shared by
// api.cu (the entry points) and jobs.cu (the job scheduler).
#pragma once
#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "kernels.h"
#include "nrc.cuh"

using gbrt::DevScene;
using gbrt::DeviceCounters;
using gbrt::StageTimer;
using gbrt::WaveRing;
using gbrt::WfState;

namespace gbrt_host {

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    cudaError_t alloc(size_t n) {
        if (n == bytes && p) return cudaSuccess;
        release();
        if (n == 0) return cudaSuccess;
        cudaError_t e = cudaMalloc(&p, n);
        if (e == cudaSuccess) bytes = n;
        else p = nullptr;
        return e;
    }
    // grows only
    cudaError_t reserve(size_t n) { return n <= bytes ? cudaSuccess : alloc(n); }
    template <class T>
    T* as() const { return static_cast<T*>(p); }
};


struct JobQueue;  // jobs.cu

}  // namespace gbrt_host

struct gbrt_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, tb0 = nullptr, tb1 = nullptr;
    std::string err;
    gbrt_host::DevBuf counters;
    gbrt_host::DevBuf async_status;  // OR of the status words of frames rendered with GBRT_RENDER_ASYNC
    gbrt_host::DevBuf trace_work;  // fetch cursor of the persistent ray-query kernel
    gbrt_host::DevBuf scratch_rays, scratch_hits, scratch_img, scratch_samples, scratch_phits;
    gbrt_host::DevBuf wf_mem, wf_frame;  // wavefront queues / path state, per-pixel frame sums
    WfState wf{};
    WaveRing ring;
    gbrt::WfSide side;  // shadow-stage stream of single-frame renders
    StageTimer timer;
    std::mutex mu;
    gbrt_host::JobQueue* jobs = nullptr;  // created by the first gbrt_job_submit
    uint64_t jobs_budget = 0;             // gbrt_jobs_configure before the first job
    std::atomic<uint32_t> inject_admit_oom{0};  // gbrt_jobs_inject: admissions still to fail
    uint32_t jobs_policy = 0;
};

struct gbrt_scene {
    gbrt_ctx* ctx = nullptr;
    uint32_t nv = 0, ni = 0, ngeo = 0, nmat = 0, ntex = 0;
    gbrt_host::DevBuf vertices, base_vertices, indices, prims, mats, tex_descs, dlights, plights, sky, skins;
    std::vector<gbrt_host::DevBuf*> tex_data;
    std::vector<gbrt_priminfo> h_prims;
    std::vector<uint32_t> h_indices;     // for range validation
    std::vector<gbrt_geo_range> ranges;  // by geo id
    std::vector<uint8_t> has_range;
    std::vector<gbrt_instance> instances;
    uint32_t nd = 0, np = 0, sky_size = 0, sky_format = GBRT_TEX_RGBA8_SRGB;
    bool skinned = false;
    bool all_opaque = true;
    uint32_t shade_feat = gbrt::kFeatAll;  // material features (kFeat* bits), set at creation
    // acceleration structures
    gbrt_host::DevBuf nodes, tris, inst, items;
    gbrt_host::DevBuf cw_nodes, cw_tris;  // 8-wide world BVH used by the wavefront traversal
    gbrt_host::DevBuf blas_cw_nodes, blas_cw_tris;  // 8-wide BLASes of transformed instances
    std::vector<uint32_t> cw_levels;  // first node of each level of the 8-wide world BVH (for refit)
    gbrt_host::DevBuf cw_boxes;        // refit scratch: float boxes of the 8-wide nodes
    uint32_t nworld = 0;               // triangles in the world BVH
    uint32_t build_flags = 0;          // gbrt_blas_build flags (GBRT_BUILD_NO_FLATTEN, GBRT_BUILD_WIDTH4)
    double cw_sah0 = 0.0;              // SAH cost proxy of the 8-wide world BVH as built (refit drift reference)
    double cw_sah = 0.0;               // ... after the last refit
    uint32_t refits = 0, rebuilds = 0; // refits since the build; full rebuilds forced by refit drift
    // kept by the build for gbrt_tlas_update (transforms only): the device
    // instances as uploaded, the TLAS's instances and BLAS root boxes, and
    // where the TLAS sits in the pools
    std::vector<gbrt::DevInstance> h_inst;
    std::vector<uint32_t> tlas_ids;
    gbrt_host::DevBuf tlas_ids_d, tlas_blo, tlas_bhi, tlas_lo, tlas_hi;
    uint32_t tlas_node_base = 0, tlas_tri_base = 0;
    bool flattened = false;            // transformed instances were merged into the world BVH
    uint32_t instance_updates = 0;     // gbrt_tlas_update calls served incrementally
    uint32_t cw_count = 0;
    bool built = false;
    std::atomic<uint32_t> jobs_pending{0};  // submitted, unfinished jobs that render this scene
    DevScene view{};
    ~gbrt_scene() {
        for (gbrt_host::DevBuf* b : tex_data) delete b;
    }
};

struct gbrt_accum {
    gbrt_ctx* ctx = nullptr;
    uint32_t w = 0, h = 0;
    std::atomic<uint32_t> jobs_pending{0};  // unfinished jobs that write this buffer
    gbrt_host::DevBuf buf;
};

namespace gbrt_host {

int fail(gbrt_ctx* c, int code, const std::string& msg);
int cuda_fail(gbrt_ctx* c, cudaError_t e, const char* what);
#define CU(ctx, x, what)                                        \
    do {                                                        \
        cudaError_t e_ = (x);                                   \
        if (e_ != cudaSuccess) return gbrt_host::cuda_fail(ctx, e_, what); \
    } while (0)

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

// Sizes the wavefront buffers for `cap` paths and `npix` pixels (grow only).
cudaError_t wavefront_reserve(gbrt_ctx* c, uint32_t cap, size_t npix);
// Rebuilds the world BVH, BLASes and TLAS of a scene from its current vertices.
int build_all(gbrt_scene* s);
// Linear-blend skinning of the scene's bind-pose vertices, then refit_world.
int skin_scene(gbrt_scene* s, const gbrt_skin_raw* skins, uint32_t nskin);
void fill_stats(gbrt_stats* st, const DeviceCounters& dc, double ms, uint32_t launches);
// After the vertices moved: the binary world BVH rebuilt and the 8-wide one
// refit in place (topology kept); scenes with transformed instances rebuild
// everything (build_all).
int refit_world(gbrt_scene* s);

// nrc.cu: cache queries and one training step on device arrays (stream-ordered).
cudaError_t nrc_query_device(gbrt_nrc* r, const float4* q, uint32_t n, float4* out, cudaStream_t st);
// Same with the query count read on the device (*n_dev, at most n_max).
cudaError_t nrc_query_counted(gbrt_nrc* r, const float4* q, const uint32_t* n_dev, uint32_t n_max, float4* out,
                              cudaStream_t st);
cudaError_t nrc_train_device(gbrt_nrc* r, const float4* pos, const float4* target, uint32_t n, cudaStream_t st);
const gbrt::NrcView& nrc_view(const gbrt_nrc* r);
// One frame rendered with the cache into out, then its training steps
// (gbrt_render_nrc without the host copies); *what names a failed step.
cudaError_t nrc_frame(gbrt_nrc* r, const DevScene& view, const gbrt_ubo& ubo, const gbrt::RenderOut& out,
                      const WfState& wf, const gbrt_nrc_render_opts& opts, cudaStream_t st, float* loss,
                      const char** what);
// The cache's query status word (0: no tensor-core wait has timed out); waits for st.
uint32_t nrc_status(gbrt_nrc* r, cudaStream_t st);
gbrt_ctx* nrc_ctx(const gbrt_nrc* r);

// jobs.cu: stops the scheduler thread after the queued jobs (ctx destroy).
void jobs_shutdown(gbrt_ctx* c);
// Jobs submitted and not yet finished on this context.
uint32_t jobs_outstanding(const gbrt_ctx* c);

}  // namespace gbrt_host
