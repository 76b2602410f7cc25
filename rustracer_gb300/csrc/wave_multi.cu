// wave_multi.cu — batched waves: up to kMaxWaveJobs jobs (frames of possibly
// different scenes) and kMaxWaveSegs segments share one wavefront.
//
// The wave descriptor lives in constant memory (c_wave, uploaded per wave
// from a pinned ring slot).  The extend / shade / shadow grids are
// partitioned by job in proportion to each job's paths, so every block
// serves one job and reads its scene and UBO with uniform constant loads.
// The job queue (jobs.cu) packs the waves; the kernel bodies are the
// single-frame ones (wavefront.cuh).
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

__global__ void __launch_bounds__(128) wfm_camera(WfState st) { camera_body(MultiWave{}, st); }
template <int kMode>
__global__ void __launch_bounds__(128, trace_minb(kMode)) wfm_extend(WfState st, uint32_t b) {
    extend_body<kMode>(MultiWave{}, st, b);
}
__global__ void __launch_bounds__(128) wfm_shade(WfState st, uint32_t b) { shade_body(MultiWave{}, st, b); }
template <int kMode>
__global__ void __launch_bounds__(128, trace_minb(kMode)) wfm_shadow(WfState st, uint32_t b) {
    shadow_body<kMode>(MultiWave{}, st, b);
}
__global__ void __launch_bounds__(128) wfm_finish(WfState st) { finish_body(MultiWave{}, st); }

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
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bs, wfm_shade, 128, 0)) != cudaSuccess) return e;
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
    r.next = 0;
    return cudaSuccess;
}

void wave_ring_free(WaveRing& r) {
    for (int i = 0; i < WaveRing::kSlots; ++i) {
        if (r.ev[i]) {
            cudaEventSynchronize(r.ev[i]);
            cudaEventDestroy(r.ev[i]);
        }
        r.ev[i] = nullptr;
    }
    if (r.host) cudaFreeHost(r.host);
    r.host = nullptr;
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
    const int full[3] = {g_grid.extend, g_grid.shade, g_grid.shadow};
    for (int k = 0; k < 3; ++k) {
        uint32_t acc = 0;
        for (uint32_t j = 0; j < w.njobs; ++j) {
            w.blk[k][j] = acc;
            const uint64_t share = ((uint64_t)full[k] * w.jobs[j].npaths + w.npaths / 2) / (w.npaths ? w.npaths : 1);
            acc += share > 0 ? (uint32_t)share : 1u;
        }
        w.blk[k][w.njobs] = acc;
    }
    return cudaSuccess;
}

cudaError_t launch_wave(WaveRing& ring, const WfState& st, cudaStream_t stream, StageTimer* timer) {
    const WaveDesc& w = ring.host[ring.next];
    if (w.nb > kMaxBounces || w.njobs == 0 || w.njobs > kMaxWaveJobs || w.nsegs == 0 || w.nsegs > kMaxWaveSegs ||
        w.npaths > st.cap || w.npaths > kMaxWavePaths)
        return cudaErrorInvalidValue;
    cudaError_t e = cudaMemcpyToSymbolAsync(c_wave, &w, sizeof(WaveDesc), 0, cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) return e;
    if ((e = cudaEventRecord(ring.ev[ring.next], stream)) != cudaSuccess) return e;
    ring.next = (ring.next + 1) % WaveRing::kSlots;
    if ((e = cudaMemsetAsync(st.counts, 0, (size_t)w.njobs * kWfCounters * sizeof(uint32_t), stream)) != cudaSuccess)
        return e;
    int mode = kTraceWide;  // the most general form any job's scene needs
    for (uint32_t j = 0; j < w.njobs; ++j) {
        const int m = trace_mode(w.jobs[j].s);
        if (m == kTraceBinary) mode = kTraceBinary;
        else if (m == kTraceWideTlas && mode == kTraceWide) mode = kTraceWideTlas;
    }
    if (timer && (e = stage_timer_reserve(*timer, timer->used + 2 + 3 * (int)w.nb + 1)) != cudaSuccess) return e;
    auto tb = [&](int stage) {
        if (timer) {
            timer->stage[timer->used] = stage;
            cudaEventRecord(timer->ev[2 * timer->used], stream);
        }
    };
    auto te = [&]() {
        if (timer) cudaEventRecord(timer->ev[2 * timer->used++ + 1], stream);
    };
    tb(3);
    wfm_camera<<<(w.npaths + 127) / 128, 128, 0, stream>>>(st);
    te();
    for (uint32_t b = 0; b < w.nb; ++b) {
        tb(0);
        if (mode == kTraceWide) wfm_extend<kTraceWide><<<w.blk[0][w.njobs], 128, 0, stream>>>(st, b);
        else if (mode == kTraceWideTlas) wfm_extend<kTraceWideTlas><<<w.blk[0][w.njobs], 128, 0, stream>>>(st, b);
        else wfm_extend<kTraceBinary><<<w.blk[0][w.njobs], 128, 0, stream>>>(st, b);
        te();
        tb(1);
        wfm_shade<<<w.blk[1][w.njobs], 128, 0, stream>>>(st, b);
        te();
        tb(2);
        if (mode == kTraceWide) wfm_shadow<kTraceWide><<<w.blk[2][w.njobs], 128, 0, stream>>>(st, b);
        else if (mode == kTraceWideTlas) wfm_shadow<kTraceWideTlas><<<w.blk[2][w.njobs], 128, 0, stream>>>(st, b);
        else wfm_shadow<kTraceBinary><<<w.blk[2][w.njobs], 128, 0, stream>>>(st, b);
        te();
    }
    tb(3);
    wfm_finish<<<(w.nfin + 127) / 128, 128, 0, stream>>>(st);
    te();
    return cudaGetLastError();
}

}  // namespace gbrt
