// wavefront.cu — single-frame wavefront path tracing (gbrt_render_ex).
//
// A frame is traced in waves of at most `cap` paths (one path = one pixel
// sample): k samples of a pixel range per wave, pixel ranges outer, samples
// inner, then one resolve (accumulate + tone map).  The wave -- one job, one
// segment -- travels as a __grid_constant__ kernel parameter, so the scene
// pointers the traversal reads every step are constant-bank operands.  The
// kernel bodies are in wavefront.cuh; the batched form is wave_multi.cu.
#include "wavefront.cuh"

namespace gbrt_host {
cudaError_t nrc_query_counted(gbrt_nrc* r, const float4* q, const uint32_t* n_dev, uint32_t n_max, float4* out,
                              cudaStream_t st);
}

namespace gbrt {

namespace {

// One job and one segment; every block serves it.
struct SingleWave {
    WaveJob J;
    WaveSeg S;
    GB_D uint32_t block_job(int) const { return 0; }
    GB_D uint32_t blk0(int, uint32_t) const { return 0; }
    GB_D uint32_t nblk(int, uint32_t) const { return gridDim.x; }
    GB_D const WaveJob& job(uint32_t) const { return J; }
    GB_D const WaveSeg& seg(uint32_t) const { return S; }
    GB_D uint32_t seg_of_path(uint32_t) const { return 0; }
    GB_D uint32_t seg_of_fin(uint32_t) const { return 0; }
    GB_D uint32_t npaths() const { return S.k * S.npw; }
    GB_D uint32_t nfin() const { return S.npw; }
};

}  // namespace

__global__ void __launch_bounds__(128) wf_camera(const __grid_constant__ SingleWave w, WfState st) {
    camera_body(w, st, blockIdx.x * blockDim.x + threadIdx.x);
}
template <int kMode>
__global__ void __launch_bounds__(128, trace_minb(kMode))
    wf_extend(const __grid_constant__ SingleWave w, WfState st, uint32_t b) {
    extend_body<kMode>(w, st, b, 0u);
}
// kFeat: the material features compiled in (kFeatAll, or 0 for scenes
// without textures, specular-glossiness or debug shading, whose smaller body
// runs at more resident blocks).
template <uint32_t kFeat>
__global__ void __launch_bounds__(kFeat ? kShadeThreads : kShadePlainThreads,
                                  kFeat ? kShadeMinBlocks : kShadePlainMinBlocks)
    wf_shade(const __grid_constant__ SingleWave w, WfState st, uint32_t b) {
    shade_body<SingleWave, false, kFeat>(w, st, b);
}
template <int kMode>
__global__ void __launch_bounds__(128, trace_minb(kMode))
    wf_shadow(const __grid_constant__ SingleWave w, WfState st, uint32_t b) {
    shadow_body<kMode>(w, st, b, 0u);
}
__global__ void __launch_bounds__(128) wf_finish(const __grid_constant__ SingleWave w, WfState st) {
    finish_body(w, st, blockIdx.x * blockDim.x + threadIdx.x);
}

// Radiance-cache forms of shade and finish, and the step that adds
// throughput x cache output to the paths that stopped at bounce b.
__global__ void __launch_bounds__(kShadeThreads, kShadeMinBlocks) wf_shade_nrc(const __grid_constant__ SingleWave w, WfState st, uint32_t b,
                                                    const __grid_constant__ NrcWave nrc) {
    shade_body<SingleWave, true>(w, st, b, &nrc);
}
__global__ void __launch_bounds__(128) wf_finish_nrc(const __grid_constant__ SingleWave w, WfState st,
                                                     const __grid_constant__ NrcWave nrc) {
    finish_body<SingleWave, true>(w, st, blockIdx.x * blockDim.x + threadIdx.x, &nrc);
}
__global__ void __launch_bounds__(256) wf_nrc_apply(WfState st, NrcWave nrc, uint32_t b) {
    const uint32_t n = nrc.counts[b];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 L = nrc.qout[i];
        const uint32_t pid = __float_as_uint(L.w) & kPidMask;
        // primary-indirect mode: the cache returns the camera hit's indirect radiance itself
        const float4 tp = nrc.mode == 1u ? f4(1.0f, 1.0f, 1.0f, 0.0f) : st.tp[pid], r = st.rad[pid];
        st.rad[pid] = f4(r.x + tp.x * fmaxf(L.x, 0.0f), r.y + tp.y * fmaxf(L.y, 0.0f), r.z + tp.z * fmaxf(L.z, 0.0f),
                         r.w);
    }
}

// rgen:132-166: accumulate, tone map, write the image.
__global__ void __launch_bounds__(128) wf_resolve(gbrt_ubo ubo, RenderOut out, const float4* frame_sum) {
    const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= out.width * out.height) return;
    const float4 fs = frame_sum[pix];
    const bool accumulate = ubo.number_of_samples != ubo.total_number_of_samples;
    const float4 prev = accumulate ? out.accum[pix] : f4(0.0f, 0.0f, 0.0f, 0.0f);
    const float3 acc = f3(prev) + f3(fs);
    out.accum[pix] = f4(acc, 0.0f);
    float3 c = tonemap(ubo.tone_mapping_mode, acc / float(ubo.total_number_of_samples));
    if (ubo.mapping == 4u) c = f3(fminf((ubo.heatmap_scale - fmaxf(fs.w, 0.001f)) / ubo.heatmap_scale, 1.0f));
    if (out.rgba8) out.rgba8[pix] = make_uchar4(to_unorm8(c.x), to_unorm8(c.y), to_unorm8(c.z), 255);
}

// --- host side ---------------------------------------------------------------
cudaError_t init_wavefront_constants(const float* srgb_lut) {
    return cudaMemcpyToSymbol(c_srgb_lut, srgb_lut, 256 * sizeof(float));
}

namespace {
struct Grid {
    int dev = -1;
    int extend = 0, shade = 0, shade_plain = 0, shadow = 0;
};
Grid g_grid;

cudaError_t grids(Grid& g) {
    int dev;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (g.dev == dev) return cudaSuccess;
    int sms = 0, be = 0, bs = 0, bh = 0;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&be, wf_extend<kTraceWide>, 128, 0)) != cudaSuccess) return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bs, wf_shade<kFeatAll>, kShadeThreads, 0)) != cudaSuccess)
        return e;
    int bp = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bp, wf_shade<0u>, kShadePlainThreads, 0)) != cudaSuccess)
        return e;
    g.shade_plain = sms * (bp > 0 ? bp : 1);
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bh, wf_shadow<kTraceWide>, 128, 0)) != cudaSuccess) return e;
    g.extend = sms * (be > 0 ? be : 1);
    g.shade = sms * (bs > 0 ? bs : 1);
    g.shadow = sms * (bh > 0 ? bh : 1);
    g.dev = dev;
    return cudaSuccess;
}
}  // namespace

size_t wavefront_bytes_per_path() { return 4 * 16 + 16 + 4 + 4 * 16 + 4 * 16 + 4; }

cudaError_t stage_timer_reserve(StageTimer& t, int pairs) {
    if (pairs <= t.capacity) return cudaSuccess;
    if (pairs < 2 * t.capacity) pairs = 2 * t.capacity;
    cudaEvent_t* ev = new cudaEvent_t[2 * pairs];
    int* stage = new int[pairs];
    for (int i = 0; i < 2 * t.capacity; ++i) ev[i] = t.ev[i];
    for (int i = 0; i < t.capacity; ++i) stage[i] = t.stage[i];  // pairs already recorded this frame
    for (int i = t.capacity; i < pairs; ++i) stage[i] = 3;
    for (int i = 2 * t.capacity; i < 2 * pairs; ++i) {
        cudaError_t e = cudaEventCreate(&ev[i]);
        if (e != cudaSuccess) {
            for (int k = 2 * t.capacity; k < i; ++k) cudaEventDestroy(ev[k]);
            delete[] ev;
            delete[] stage;
            return e;
        }
    }
    delete[] t.ev;
    delete[] t.stage;
    t.ev = ev;
    t.stage = stage;
    t.capacity = pairs;
    return cudaSuccess;
}

void stage_timer_free(StageTimer& t) {
    for (int i = 0; i < 2 * t.capacity; ++i) cudaEventDestroy(t.ev[i]);
    delete[] t.ev;
    delete[] t.stage;
    t = StageTimer{};
}

cudaError_t stage_timer_collect(StageTimer& t, double ms[4]) {
    for (int k = 0; k < 4; ++k) ms[k] = 0.0;
    for (int i = 0; i < t.used; ++i) {
        float f = 0.0f;
        cudaError_t e = cudaEventElapsedTime(&f, t.ev[2 * i], t.ev[2 * i + 1]);
        if (e != cudaSuccess) return e;
        ms[t.stage[i] & 3] += f;
    }
    return cudaSuccess;
}

cudaError_t launch_resolve(const gbrt_ubo& ubo, const RenderOut& out, const float4* frame_sum, cudaStream_t stream) {
    const uint32_t npix = out.width * out.height;
    wf_resolve<<<(npix + 127) / 128, 128, 0, stream>>>(ubo, out, frame_sum);
    return cudaGetLastError();
}

cudaError_t launch_wavefront(const DevScene& s, const gbrt_ubo& ubo, const RenderOut& out, const WfState& st,
                             cudaStream_t stream, StageTimer* timer, const NrcWave* nrc, gbrt_nrc* cache,
                             const WfSide* side) {
    // the overlap needs the stages' own events off and leaves the cache form serial
    // (its apply step updates the radiance the shadow stage also updates)
    if (timer || nrc) side = nullptr;
    if (ubo.number_of_bounces > kMaxBounces) return cudaErrorInvalidValue;
    cudaError_t e = grids(g_grid);
    if (e != cudaSuccess) return e;
    const uint32_t W = out.width, H = out.height, npix = W * H, ns = ubo.number_of_samples;
    const uint32_t sbase = ubo.total_number_of_samples - ns, nb = ubo.number_of_bounces;
    const uint32_t cap = st.cap < kMaxWavePaths ? st.cap : kMaxWavePaths;
    if ((e = cudaMemsetAsync(st.frame_sum, 0, (size_t)npix * sizeof(float4), stream)) != cudaSuccess) return e;
    if (timer) timer->used = 0;
    auto tb = [&](int stage) {
        if (timer) {
            timer->stage[timer->used] = stage;
            cudaEventRecord(timer->ev[2 * timer->used], stream);
        }
    };
    auto te = [&]() {
        if (timer) cudaEventRecord(timer->ev[2 * timer->used++ + 1], stream);
    };
    SingleWave w;
    WaveJob& J = w.J;
    J.s = s;
    J.ubo = ubo;
    J.out = out;
    J.frame_sum = st.frame_sum;
    J.ns = ns;
    // a radiance cache adds to the radiance between shade and shadow (wf_nrc_apply), so the shadow
    // records then hold deltas that the shadow kernel adds
    J.flags = (ubo.fully_opaque ? GBRT_RAY_OPAQUE : 0u) | (nrc ? kShadowDelta : 0u);
    J.tfar = ubo.orthographic_fov_dis > 0.0f ? 100000.0f : 10000.0f;
    J.path0 = 0;
    const int mode = trace_mode(s) | (s.all_opaque || ubo.fully_opaque ? kTraceOpaque : 0);
    // the shade form: the scene's material features and this frame's debug settings
    const uint32_t feat = s.shade_feat | (ubo.mapping != 0u || ubo.debug == 1u ? kFeatDebug : 0u);
    // waves: k samples of a pixel range, k * npw <= cap
    for (uint32_t px0 = 0; px0 < npix;) {
        const uint32_t npw = npix - px0 < cap ? npix - px0 : cap;
        const uint32_t kmax = cap / npw;
        for (uint32_t s0 = 0; s0 < ns;) {
            const uint32_t k = ns - s0 < kmax ? ns - s0 : kmax;
            J.npaths = k * npw;
            w.S = WaveSeg{0u, 0u, px0, npw, sbase + s0, s0, k, 0u};
            if (timer && (e = stage_timer_reserve(*timer, timer->used + 3 + 4 * (int)nb)) != cudaSuccess) return e;
            if ((e = cudaMemsetAsync(st.counts, 0, kWfCounters * sizeof(uint32_t), stream)) != cudaSuccess) return e;
            if (nrc) {
                if ((e = cudaMemsetAsync(nrc->counts, 0, 32 * sizeof(uint32_t), stream)) != cudaSuccess) return e;
                if ((e = cudaMemsetAsync(nrc->snap_pos, 0, (size_t)J.npaths * sizeof(float4), stream)) != cudaSuccess)
                    return e;
            }
            tb(3);
            wf_camera<<<(J.npaths + 127) / 128, 128, 0, stream>>>(w, st);
            te();
            for (uint32_t b = 0; b < nb; ++b) {
                tb(0);
                GBRT_TRACE_LAUNCH(wf_extend, g_grid.extend, stream, w, st, b);
                te();
                if (side && b > 0 && (e = cudaStreamWaitEvent(stream, side->shadowed, 0)) != cudaSuccess) return e;
                tb(1);
                if (nrc) wf_shade_nrc<<<g_grid.shade, kShadeThreads, 0, stream>>>(w, st, b, *nrc);
                else if (feat == 0u) wf_shade<0u><<<g_grid.shade_plain, kShadePlainThreads, 0, stream>>>(w, st, b);
                else wf_shade<kFeatAll><<<g_grid.shade, kShadeThreads, 0, stream>>>(w, st, b);
                te();
                if (nrc && !nrc->disabled && (nrc->mode == 1u ? b == 0 : b >= 1)) {  // queries of the paths that stopped here
                    tb(3);
                    if ((e = gbrt_host::nrc_query_counted(cache, nrc->query, nrc->counts + b, J.npaths, nrc->qout,
                                                          stream)) != cudaSuccess)
                        return e;
                    wf_nrc_apply<<<g_grid.shade, 256, 0, stream>>>(st, *nrc, b);
                    te();
                }
                tb(2);
                cudaStream_t ss = stream;
                if (side) {
                    if ((e = cudaEventRecord(side->shaded, stream)) != cudaSuccess) return e;
                    if ((e = cudaStreamWaitEvent(side->stream, side->shaded, 0)) != cudaSuccess) return e;
                    ss = side->stream;
                }
                GBRT_TRACE_LAUNCH(wf_shadow, g_grid.shadow, ss, w, st, b);
                if (side && (e = cudaEventRecord(side->shadowed, ss)) != cudaSuccess) return e;
                te();
            }
            if (side && (e = cudaStreamWaitEvent(stream, side->shadowed, 0)) != cudaSuccess) return e;
            tb(3);
            if (nrc) wf_finish_nrc<<<(npw + 127) / 128, 128, 0, stream>>>(w, st, *nrc);
            else wf_finish<<<(npw + 127) / 128, 128, 0, stream>>>(w, st);
            te();
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
            s0 += k;
        }
        px0 += npw;
    }
    if (timer && (e = stage_timer_reserve(*timer, timer->used + 1)) != cudaSuccess) return e;
    tb(3);
    e = launch_resolve(ubo, out, st.frame_sum, stream);
    te();
    return e;
}

}  // namespace gbrt
