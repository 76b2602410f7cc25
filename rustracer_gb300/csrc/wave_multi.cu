// wave_multi.cu — batched waves: up to kMaxWaveJobs jobs (frames of possibly
// different scenes) and kMaxWaveSegs segments share one wavefront.
//
// The wave descriptor lives in constant memory (c_wave, uploaded per wave
// from a pinned ring slot).  The extend / shade / shadow grids are
// partitioned by job in proportion to each job's paths, so every block
// serves one job and reads its scene and UBO with uniform constant loads.
// The job queue (jobs.cu) packs the waves; the kernel bodies are the
// single-frame ones (wavefront.cuh).
#include <algorithm>
#include <cstring>

#include "wavefront.cuh"

namespace gbrt {

__constant__ WaveDesc c_wave;

namespace {

struct MultiWave {
    GB_D uint32_t block_job(int stage) const {
        uint32_t j = 0;
        while (j + 1 < c_wave.njobs && blockIdx.x >= c_wave.blk[stage][j + 1]) ++j;
        return j;
    }
    GB_D uint32_t blk0(int stage, uint32_t j) const { return c_wave.blk[stage][j]; }
    GB_D uint32_t nblk(int stage, uint32_t j) const { return c_wave.blk[stage][j + 1] - c_wave.blk[stage][j]; }
    GB_D const WaveJob& job(uint32_t j) const { return c_wave.jobs[j]; }
    GB_D const WaveSeg& seg(uint32_t i) const { return c_wave.segs[i]; }
    GB_D uint32_t seg_of_path(uint32_t pid) const {  // segments are sorted by path0
        uint32_t lo = 0, hi = c_wave.nsegs;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (c_wave.segs[mid].path0 <= pid) lo = mid;
            else hi = mid;
        }
        return lo;
    }
    GB_D uint32_t seg_of_fin(uint32_t i) const {  // and by fin0
        uint32_t lo = 0, hi = c_wave.nsegs;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (c_wave.segs[mid].fin0 <= i) lo = mid;
            else hi = mid;
        }
        return lo;
    }
    GB_D uint32_t npaths() const { return c_wave.npaths; }
    GB_D uint32_t nfin() const { return c_wave.nfin; }
};

}  // namespace

// camera and finish loop over the wave with a fixed grid, so that one
// captured graph serves every wave of the same bounce count
__global__ void __launch_bounds__(128) wfm_camera(WfState st) {
    for (uint32_t base = blockIdx.x * blockDim.x; base < c_wave.npaths; base += gridDim.x * blockDim.x)
        camera_body(MultiWave{}, st, base + threadIdx.x);
}
// A block starts on its own job's queue and then helps the other jobs'
// queues (their fetch cursors are shared), so blocks of jobs that finish
// early do not idle while a costlier job still has rays.
template <int kMode>
__global__ void __launch_bounds__(128, trace_minb(kMode)) wfm_extend(WfState st, uint32_t b) {
    const uint32_t own = MultiWave{}.block_job(0), nj = c_wave.njobs;
    for (uint32_t t = 0; t < nj; ++t) extend_body<kMode>(MultiWave{}, st, b, own + t < nj ? own + t : own + t - nj);
}
__global__ void __launch_bounds__(kShadeThreads, kShadeMinBlocks) wfm_shade(WfState st, uint32_t b) { shade_body(MultiWave{}, st, b); }
template <int kMode>
__global__ void __launch_bounds__(128, trace_minb(kMode)) wfm_shadow(WfState st, uint32_t b) {
    const uint32_t own = MultiWave{}.block_job(2), nj = c_wave.njobs;
    for (uint32_t t = 0; t < nj; ++t) shadow_body<kMode>(MultiWave{}, st, b, own + t < nj ? own + t : own + t - nj);
}
__global__ void __launch_bounds__(128) wfm_finish(WfState st) {
    for (uint32_t base = blockIdx.x * blockDim.x; base < c_wave.nfin; base += gridDim.x * blockDim.x)
        finish_body(MultiWave{}, st, base + threadIdx.x);
}

// --- host side ---------------------------------------------------------------
cudaError_t init_wave_multi_constants(const float* srgb_lut) {
    return cudaMemcpyToSymbol(c_srgb_lut, srgb_lut, 256 * sizeof(float));
}

namespace {
struct Grid {
    int dev = -1;
    int extend = 0, shade = 0, shadow = 0;
};
Grid g_grid;

cudaError_t grids(Grid& g) {
    int dev;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (g.dev == dev) return cudaSuccess;
    int sms = 0, be = 0, bs = 0, bh = 0;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&be, wfm_extend<kTraceWide>, 128, 0)) != cudaSuccess) return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bs, wfm_shade, kShadeThreads, 0)) != cudaSuccess) return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bh, wfm_shadow<kTraceWide>, 128, 0)) != cudaSuccess) return e;
    g.extend = sms * (be > 0 ? be : 1);
    g.shade = sms * (bs > 0 ? bs : 1);
    g.shadow = sms * (bh > 0 ? bh : 1);
    g.dev = dev;
    return cudaSuccess;
}
}  // namespace

cudaError_t wave_ring_init(WaveRing& r) {
    if (r.host) return cudaSuccess;
    cudaError_t e = cudaMallocHost(&r.host, sizeof(WaveDesc) * WaveRing::kSlots);
    if (e != cudaSuccess) {
        r.host = nullptr;
        return e;
    }
    for (int i = 0; i < WaveRing::kSlots; ++i) {
        if ((e = cudaEventCreateWithFlags(&r.ev[i], cudaEventDisableTiming)) != cudaSuccess) {
            wave_ring_free(r);
            return e;
        }
    }
    if ((e = cudaStreamCreateWithFlags(&r.cap, cudaStreamNonBlocking)) != cudaSuccess) {
        r.cap = nullptr;
        wave_ring_free(r);
        return e;
    }
    r.next = 0;
    return cudaSuccess;
}

void wave_ring_free(WaveRing& r) {
    wave_graphs_reset(r);
    for (int i = 0; i < WaveRing::kSlots; ++i) {
        if (r.ev[i]) {
            cudaEventSynchronize(r.ev[i]);
            cudaEventDestroy(r.ev[i]);
        }
        r.ev[i] = nullptr;
    }
    if (r.host) cudaFreeHost(r.host);
    r.host = nullptr;
    if (r.cap) cudaStreamDestroy(r.cap);
    r.cap = nullptr;
}

cudaError_t wave_acquire(WaveRing& r, WaveDesc** slot) {
    cudaError_t e = wave_ring_init(r);
    if (e != cudaSuccess) return e;
    if ((e = cudaEventSynchronize(r.ev[r.next])) != cudaSuccess) return e;  // its last upload has run
    *slot = &r.host[r.next];
    return cudaSuccess;
}

cudaError_t wave_partition(WaveDesc& w) {
    cudaError_t e = grids(g_grid);
    if (e != cudaSuccess) return e;
    // exactly the stage's full grid, in proportion to each job's paths (at
    // least one block each), so that the launches of every wave are alike
    const int full[3] = {g_grid.extend, g_grid.shade, g_grid.shadow};
    for (int k = 0; k < 3; ++k) {
        const uint32_t total = std::max<uint32_t>((uint32_t)full[k], w.njobs);
        uint32_t n[kMaxWaveJobs], sum = 0, big = 0;
        for (uint32_t j = 0; j < w.njobs; ++j) {
            const uint64_t share = (uint64_t)total * w.jobs[j].npaths / (w.npaths ? w.npaths : 1);
            n[j] = share > 0 ? (uint32_t)share : 1u;
            sum += n[j];
            if (n[j] > n[big]) big = j;
        }
        n[big] = n[big] + total - sum;  // the remainder (either sign) to the largest job
        uint32_t acc = 0;
        for (uint32_t j = 0; j < w.njobs; ++j) {
            w.blk[k][j] = acc;
            acc += n[j];
        }
        w.blk[k][w.njobs] = acc;
    }
    return cudaSuccess;
}

namespace {

int wave_mode(const WaveDesc& w) {
    int mode = kTraceWide;  // the most general form any job's scene needs
    for (uint32_t j = 0; j < w.njobs; ++j) {
        const int m = trace_mode(w.jobs[j].s);
        if (m == kTraceBinary) mode = kTraceBinary;
        else if (m == kTraceWideTlas && mode == kTraceWide) mode = kTraceWideTlas;
    }
    // the alpha test is compiled out when no job of the wave can need it
    bool opaque = true;
    for (uint32_t j = 0; j < w.njobs; ++j)
        opaque = opaque && (w.jobs[j].s.all_opaque || (w.jobs[j].flags & GBRT_RAY_OPAQUE));
    return mode | (opaque ? kTraceOpaque : 0);
}

// The launches of one batched wave with `nb` bounces in traversal form
// `mode`; every grid is fixed, the wave itself is read from c_wave.
cudaError_t enqueue_wave(const WfState& st, int mode, uint32_t nb, cudaStream_t stream, StageTimer* timer) {
    cudaError_t e = cudaMemsetAsync(st.counts, 0, (size_t)kMaxWaveJobs * kWfCounters * sizeof(uint32_t), stream);
    if (e != cudaSuccess) return e;
    auto tb = [&](int stage) {
        if (timer) {
            timer->stage[timer->used] = stage;
            cudaEventRecord(timer->ev[2 * timer->used], stream);
        }
    };
    auto te = [&]() {
        if (timer) cudaEventRecord(timer->ev[2 * timer->used++ + 1], stream);
    };
    const int flat = 4 * g_grid.shade;  // grid-stride kernels
    tb(3);
    wfm_camera<<<flat, 128, 0, stream>>>(st);
    te();
    for (uint32_t b = 0; b < nb; ++b) {
        tb(0);
        GBRT_TRACE_LAUNCH(wfm_extend, g_grid.extend, stream, st, b);
        te();
        tb(1);
        wfm_shade<<<g_grid.shade, kShadeThreads, 0, stream>>>(st, b);
        te();
        tb(2);
        GBRT_TRACE_LAUNCH(wfm_shadow, g_grid.shadow, stream, st, b);
        te();
    }
    tb(3);
    wfm_finish<<<flat, 128, 0, stream>>>(st);
    te();
    return cudaGetLastError();
}

}  // namespace

void wave_graphs_reset(WaveRing& r) {
    for (auto& row : r.graph)
        for (auto& g : row)
            if (g) {
                cudaGraphExecDestroy(g);
                g = nullptr;
            }
    r.graph_state = WfState{};
}

cudaError_t launch_wave(WaveRing& ring, const WfState& st, cudaStream_t stream, StageTimer* timer) {
    const WaveDesc& w = ring.host[ring.next];
    if (w.nb > kMaxBounces || w.njobs == 0 || w.njobs > kMaxWaveJobs || w.nsegs == 0 || w.nsegs > kMaxWaveSegs ||
        w.npaths > st.cap || w.npaths > kMaxWavePaths)
        return cudaErrorInvalidValue;
    for (int k = 0; k < 3; ++k)
        if (w.blk[k][w.njobs] != (uint32_t)(k == 0 ? g_grid.extend : k == 1 ? g_grid.shade : g_grid.shadow))
            return cudaErrorInvalidValue;  // wave_partition fills the grids these launches use
    cudaError_t e = cudaMemcpyToSymbolAsync(c_wave, &w, sizeof(WaveDesc), 0, cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) return e;
    if ((e = cudaEventRecord(ring.ev[ring.next], stream)) != cudaSuccess) return e;
    ring.next = (ring.next + 1) % WaveRing::kSlots;
    const int mode = wave_mode(w);
    if (timer) {
        if ((e = stage_timer_reserve(*timer, timer->used + 2 + 3 * (int)w.nb + 1)) != cudaSuccess) return e;
        return enqueue_wave(st, mode, w.nb, stream, timer);
    }
    // one CUDA graph per (traversal form, bounce count), captured on first use
    // and replayed for every later wave; rebuilt when the wavefront buffers move
    if (std::memcmp(&ring.graph_state, &st, sizeof(WfState)) != 0) {
        wave_graphs_reset(ring);
        ring.graph_state = st;
    }
    cudaGraphExec_t& exec = ring.graph[mode][w.nb];
    if (!exec) {
        cudaGraph_t graph = nullptr;
        if ((e = cudaStreamBeginCapture(ring.cap, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) return e;
        const cudaError_t ee = enqueue_wave(st, mode, w.nb, ring.cap, nullptr);
        e = cudaStreamEndCapture(ring.cap, &graph);
        if (ee != cudaSuccess) e = ee;
        if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            exec = nullptr;
            return e;
        }
    }
    return cudaGraphLaunch(exec, stream);
}

}  // namespace gbrt
