// wavefront.cu — the wavefront form of the path tracer.
//
// A frame is traced in waves of at most `cap` paths (one path = one pixel
// sample).  Per wave: camera -> for each bounce { extend (closest hit) ->
// shade (closest-hit / miss shaders, Russian roulette, next ray, NEE shadow
// record) -> shadow (any-hit) } -> finish (per-pixel sums in sample order),
// and after the last wave one resolve (accumulate + tone map).  Each stage is
// a small kernel, so the instruction working set fits the cache and lanes of
// a warp run the same stage; queues between stages are compacted with warp
// ballots (one atomic per warp).  Results are bit-identical to the megakernel:
// the same device functions run in the same order per path, the NEE term is
// added as (E + C) after the shadow test like RayTracing.rchit:346-349.
#include "hitgroup.cuh"
#include "kernels.h"
#include "persistent.cuh"

namespace gbrt {

namespace {

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

// Warp-aggregated queue append: every lane of the warp calls it; lanes with
// want == true get consecutive slots.
__device__ __forceinline__ uint32_t warp_append(uint32_t* counter, bool want) {
    const uint32_t mask = __ballot_sync(0xFFFFFFFFu, want);
    uint32_t base = 0;
    if (lane_id() == 0 && mask) base = atomicAdd(counter, (uint32_t)__popc(mask));
    base = __shfl_sync(0xFFFFFFFFu, base, 0);
    return base + __popc(mask & ((1u << lane_id()) - 1u));
}

// Per-warp dynamic fetch of 32 consecutive queue slots.
__device__ __forceinline__ uint32_t warp_fetch(uint32_t* work) {
    uint32_t base = 0;
    if (lane_id() == 0) base = atomicAdd(work, 32u);
    return __shfl_sync(0xFFFFFFFFu, base, 0);
}

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
    return v;
}

}  // namespace

// Counter slots inside WfState::counts (reset at the start of every wave).
constexpr int kQueue = 0;     // [kQueue + b]: extension-queue length at bounce b
constexpr int kShadow = 32;   // [kShadow + b]: shadow-queue length at bounce b
constexpr int kWorkExt = 64;  // [kWorkExt + b]: fetch cursor of extend(b)
constexpr int kWorkSh = 96;   // [kWorkSh + b]: fetch cursor of shadow(b)
constexpr int kMaxBounces = 31;

struct WfParams {
    WfState st;
    uint32_t W, H;
    uint32_t px0, npw;  // pixel range of the wave
    uint32_t sample0;   // global sample index of the wave's first sample
    uint32_t si0;       // frame-local index of that sample
    uint32_t ns;        // samples in the frame (debug-output stride)
    uint32_t npaths;
    float tfar;
    uint32_t flags;     // GBRT_RAY_OPAQUE when the UBO says fully_opaque
    RenderOut out;
};

__device__ __forceinline__ void path_coords(const WfParams& p, uint32_t pid, uint32_t& pix, uint32_t& x, uint32_t& y,
                                            uint32_t& j) {
    j = pid / p.npw;
    pix = p.px0 + (pid - j * p.npw);
    y = pix / p.W;
    x = pix - y * p.W;
}

// rgen:32-80 for every path of the wave: seeds (D1), camera ray, path state.
__global__ void __launch_bounds__(128) wf_camera(gbrt_ubo ubo, WfParams p) {
    const uint32_t pid = blockIdx.x * blockDim.x + threadIdx.x;
    if (pid == 0) p.st.counts[kQueue] = p.npaths;
    if (pid >= p.npaths) return;
    uint32_t pix, x, y, j;
    path_coords(p, pid, pix, x, y, j);
    const uint32_t sample = p.sample0 + j;
    uint32_t seed = tea16(tea16(x, y), sample);
    uint4 rng = make_uint4(x, y, sample, 0u);
    float3 o, d;
    float tfar;
    camera_ray(ubo, x, y, p.W, p.H, rng, seed, o, d, tfar);
    p.st.ray_o[0][pid] = f4(o, 0.0f);
    p.st.ray_d[0][pid] = f4(d, __uint_as_float(pid));
    p.st.tp[pid] = f4(1.0f, 1.0f, 1.0f, 0.0f);             // throughput, Ray.t = 0
    p.st.rad[pid] = f4(0.0f, 0.0f, 0.0f, -1.0f);           // radiance, volume_dis = -1
    p.st.hp[pid] = f4(0.0f, 0.0f, 0.0f, __uint_as_float(seed));  // hitPoint, RandomSeed
    p.st.rng[pid] = make_uint4(rng.w, 0u, tea16(sample, 0x9E3779B9u), 0u);
}

// traceRayEXT for the extension queue of bounce b (closest hit).
template <bool kWide>
__global__ void __launch_bounds__(128) wf_extend(DevScene s, WfParams p, uint32_t b) {
    const uint32_t n = p.st.counts[kQueue + b];
    const float4* __restrict__ ro = p.st.ray_o[b & 1];
    const float4* __restrict__ rd = p.st.ray_d[b & 1];
    TraceStats ts{0, 0, 0};
    world_trace<false, kWide>(
        s, n, &p.st.counts[kWorkExt + b], p.flags, ts,
        [&](uint32_t q, float3& o, float3& d, float& tmin, float& tmax, AnyCtx& ctx) {
            const float4 o4 = ro[q], d4 = rd[q];
            uint32_t pix, x, y, j;
            path_coords(p, __float_as_uint(d4.w), pix, x, y, j);
            o = f3(o4);
            d = f3(d4);
            tmin = 0.001f;
            tmax = p.tfar;
            ctx = AnyCtx{x, y, p.sample0 + j, b};
        },
        [&](uint32_t q, bool hit, const Hit& h) {
            p.st.hit[q] = f4(hit ? h.t : -1.0f, h.u, h.v, __uint_as_float(hit ? h.inst : 0xFFFFFFFFu));
            p.st.hit_prim[q] = h.prim;
            if (b == 0 && p.out.primary_hits) {
                uint32_t pix, x, y, j;
                path_coords(p, __float_as_uint(rd[q].w), pix, x, y, j);
                gbrt_hit g;
                g.t = hit ? h.t : -1.0f;
                g.u = hit ? h.u : 0.0f;
                g.v = hit ? h.v : 0.0f;
                g.instance_id = hit ? h.inst : 0xFFFFFFFFu;
                g.primitive_id = hit ? h.prim : 0xFFFFFFFFu;
                g.custom_index = hit ? s.inst[h.inst].custom : 0xFFFFFFFFu;
                p.out.primary_hits[(size_t)pix * p.ns + p.si0 + j] = g;
            }
        });
    const unsigned long long nodes = warp_sum<unsigned long long>(ts.nodes);
    const unsigned long long tris = warp_sum<unsigned long long>(ts.tris);
    uint32_t stat = ts.status;
    for (int o = 16; o > 0; o >>= 1) stat |= __shfl_down_sync(0xFFFFFFFFu, stat, o);
    if (lane_id() == 0) {
        atomicAdd(&p.out.counters->nodes, nodes);
        atomicAdd(&p.out.counters->tris, tris);
        if (stat) atomicOr(&p.out.counters->status, stat);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (b == 0) atomicAdd(&p.out.counters->camera, (unsigned long long)n);
        else atomicAdd(&p.out.counters->extension, (unsigned long long)n);
    }
}

// Closest-hit / miss shading and the rest of rgen's bounce loop
// (RayTracing.rgen:94-128) for the extension queue of bounce b.
__global__ void __launch_bounds__(128) wf_shade(DevScene s, gbrt_ubo ubo, WfParams p, uint32_t b) {
    const uint32_t n = p.st.counts[kQueue + b];
    const float4* __restrict__ rd = p.st.ray_d[b & 1];
    float4* no = p.st.ray_o[(b + 1) & 1];
    float4* nd = p.st.ray_d[(b + 1) & 1];
    const uint32_t nb = ubo.number_of_bounces;
    PathStats ps{0, 0, 0, 0, 0};
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < n; base += stride) {
        const uint32_t q = base + lane_id();
        const bool active = q < n;
        bool cont = false, shadow = false;
        float3 nxt_o = f3(0.0f), nxt_d = f3(0.0f), so = f3(0.0f), sd = f3(0.0f), sc = f3(0.0f), se = f3(0.0f);
        float3 tp_before = f3(0.0f);
        float stmax = 0.0f;
        uint32_t pid = 0;
        if (active) {
            const float4 d4 = rd[q];
            const float3 d = f3(d4);
            pid = __float_as_uint(d4.w);
            uint32_t pix, x, y, j;
            path_coords(p, pid, pix, x, y, j);
            const float4 h4 = p.st.hit[q];
            const float4 tp4 = p.st.tp[pid], rad4 = p.st.rad[pid], hp4 = p.st.hp[pid];
            uint4 rg = p.st.rng[pid];
            Payload R;
            R.hitValue = R.scatterDir = R.emittance = f3(0.0f);
            R.needScatter = 0;
            R.hitPoint = f3(hp4);
            R.RandomSeed = __float_as_uint(hp4.w);
            R.t = tp4.w;
            R.volume_dis = rad4.w;
            R.rngState = make_uint4(x, y, rg.z, rg.y);
            const uint32_t inst = __float_as_uint(h4.w);
            if (inst != 0xFFFFFFFFu) {
                Hit h;
                h.t = h4.x;
                h.u = h4.y;
                h.v = h4.z;
                h.inst = inst;
                h.prim = p.st.hit_prim[q];
                h.bgeo = 0;
                closest_hit(s, ubo, R, h, d, ps, [&](float3 o_, float3 d_, float t_, float3 C) {
                    shadow = true;
                    so = o_;
                    sd = d_;
                    stmax = t_;
                    sc = C;
                });
            } else {
                miss_shader(s, ubo, R, d);
            }
            float3 tp = f3(tp4);
            float3 rad = f3(rad4);
            tp_before = tp;
            se = R.emittance;
            if (!shadow) rad += tp * R.emittance;
            cont = b + 1 != nb;
            if (cont && b > 3u) {  // Russian roulette, rgen:108-118
                uint4 prng = make_uint4(x, y, p.sample0 + j, rg.x);
                const float pr = clampf(luminance(tp), 0.01f, 0.95f);
                if (pr < pcg_rand(prng)) cont = false;
                else tp /= pr;
                rg.x = prng.w;
            }
            if (cont) {
                tp *= R.hitValue;
                if (!R.needScatter || R.t < 0.0f) cont = false;
            }
            p.st.tp[pid] = f4(tp, R.t);
            p.st.rad[pid] = f4(rad, R.volume_dis);
            p.st.hp[pid] = f4(R.hitPoint, __uint_as_float(R.RandomSeed));
            p.st.rng[pid] = make_uint4(rg.x, R.rngState.w, rg.z, 0u);
            nxt_o = R.hitPoint;
            nxt_d = R.scatterDir;
        }
        const uint32_t slot = warp_append(&p.st.counts[kQueue + b + 1], cont);
        if (cont) {
            no[slot] = f4(nxt_o, 0.0f);
            nd[slot] = f4(nxt_d, __uint_as_float(pid));
        }
        const uint32_t sslot = warp_append(&p.st.counts[kShadow + b], shadow);
        if (shadow) {
            p.st.sh_o[sslot] = f4(so, stmax);
            p.st.sh_d[sslot] = f4(sd, __uint_as_float(pid));
            p.st.sh_e[sslot] = f4(se, tp_before.x);
            p.st.sh_c[sslot] = f4(sc, tp_before.y);
            p.st.sh_tp[sslot] = tp_before.z;
        }
    }
    const unsigned long long hs = warp_sum<unsigned long long>(ps.shaded);
    if (lane_id() == 0 && hs) atomicAdd(&p.out.counters->shaded, hs);
}

// Any-hit shadow rays of bounce b (castShadowRay, RayTracing.rchit:35-59),
// then the deferred radiance update radiance += tp * (E [+ C if unoccluded]).
template <bool kWide>
__global__ void __launch_bounds__(128) wf_shadow(DevScene s, WfParams p, uint32_t b) {
    const uint32_t n = p.st.counts[kShadow + b];
    TraceStats ts{0, 0, 0};
    const uint32_t flags = GBRT_RAY_TERMINATE_ON_FIRST | p.flags;
    world_trace<true, kWide>(
        s, n, &p.st.counts[kWorkSh + b], flags, ts,
        [&](uint32_t q, float3& o, float3& d, float& tmin, float& tmax, AnyCtx& ctx) {
            const float4 o4 = p.st.sh_o[q], d4 = p.st.sh_d[q];
            uint32_t pix, x, y, j;
            path_coords(p, __float_as_uint(d4.w), pix, x, y, j);
            o = f3(o4);
            d = f3(d4);
            tmin = 0.1f;
            tmax = o4.w;
            ctx = AnyCtx{x, y, p.sample0 + j, b | 0x100u};
        },
        [&](uint32_t q, bool occluded, const Hit&) {
            const float4 d4 = p.st.sh_d[q], e4 = p.st.sh_e[q], c4 = p.st.sh_c[q];
            const float tpz = p.st.sh_tp[q];
            const uint32_t pid = __float_as_uint(d4.w);
            float3 e = f3(e4);
            if (!occluded) e += f3(c4);
            const float4 r = p.st.rad[pid];
            const float3 rad = f3(r) + f3(e4.w, c4.w, tpz) * e;
            p.st.rad[pid] = f4(rad, r.w);
        });
    const unsigned long long nodes = warp_sum<unsigned long long>(ts.nodes);
    const unsigned long long tris = warp_sum<unsigned long long>(ts.tris);
    uint32_t stat = ts.status;
    for (int o = 16; o > 0; o >>= 1) stat |= __shfl_down_sync(0xFFFFFFFFu, stat, o);
    if (lane_id() == 0) {
        atomicAdd(&p.out.counters->nodes, nodes);
        atomicAdd(&p.out.counters->tris, tris);
        if (stat) atomicOr(&p.out.counters->status, stat);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&p.out.counters->shadow, (unsigned long long)n);
}

// Per pixel of the wave: add its samples' radiance to the frame sum in
// sample order (the megakernel's per-pixel order), keep the last Ray.t.
__global__ void __launch_bounds__(128) wf_finish(WfParams p, uint32_t k) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.npw) return;
    const uint32_t pix = p.px0 + i;
    float4 acc = p.st.frame_sum[pix];
    float3 sum = f3(acc);
    float last_t = acc.w;
    for (uint32_t j = 0; j < k; ++j) {
        const uint32_t pid = i + j * p.npw;
        const float3 r = f3(p.st.rad[pid]);
        if (p.out.sample_radiance) {
            float* sr = p.out.sample_radiance + ((size_t)pix * p.ns + p.si0 + j) * 3;
            sr[0] = r.x;
            sr[1] = r.y;
            sr[2] = r.z;
        }
        sum += r;
        last_t = p.st.tp[pid].w;
    }
    p.st.frame_sum[pix] = f4(sum, last_t);
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
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&be, wf_extend<true>, 128, 0)) != cudaSuccess) return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bs, wf_shade, 128, 0)) != cudaSuccess) return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bh, wf_shadow<true>, 128, 0)) != cudaSuccess) return e;
    g.extend = sms * (be > 0 ? be : 1);
    g.shade = sms * (bs > 0 ? bs : 1);
    g.shadow = sms * (bh > 0 ? bh : 1);
    g.dev = dev;
    return cudaSuccess;
}
}  // namespace

size_t wavefront_bytes_per_path() { return 4 * 16 + 16 + 4 + 4 * 16 + 4 * 16 + 4; }

namespace {
cudaError_t timer_grow(StageTimer& t, int pairs) {
    if (pairs <= t.capacity) return cudaSuccess;
    cudaEvent_t* ev = new cudaEvent_t[2 * pairs];
    int* stage = new int[pairs];
    for (int i = 0; i < 2 * t.capacity; ++i) ev[i] = t.ev[i];
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
}  // namespace

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
        ms[t.stage[i]] += f;
    }
    return cudaSuccess;
}

cudaError_t launch_wavefront(const DevScene& s, const gbrt_ubo& ubo, const RenderOut& out, const WfState& st,
                             cudaStream_t stream, StageTimer* timer) {
    if (ubo.number_of_bounces > kMaxBounces) return cudaErrorInvalidValue;
    cudaError_t e = grids(g_grid);
    if (e != cudaSuccess) return e;
    const uint32_t W = out.width, H = out.height, npix = W * H, ns = ubo.number_of_samples;
    const uint32_t sbase = ubo.total_number_of_samples - ns;
    if ((e = cudaMemsetAsync(st.frame_sum, 0, (size_t)npix * sizeof(float4), stream)) != cudaSuccess) return e;
    WfParams p;
    p.st = st;
    p.W = W;
    p.H = H;
    p.ns = ns;
    p.tfar = ubo.orthographic_fov_dis > 0.0f ? 100000.0f : 10000.0f;
    p.flags = ubo.fully_opaque ? GBRT_RAY_OPAQUE : 0u;
    p.out = out;
    const uint32_t nb = ubo.number_of_bounces;
    if (timer) {
        const uint64_t npw0 = npix < st.cap ? npix : st.cap, k0 = st.cap / npw0;
        const uint64_t waves = ((npix + npw0 - 1) / npw0) * ((ns + k0 - 1) / k0);
        if ((e = timer_grow(*timer, (int)(waves * (2 + 3 * nb) + 1))) != cudaSuccess) return e;
        timer->used = 0;
    }
    auto tb = [&](int stage) {
        if (timer) {
            timer->stage[timer->used] = stage;
            cudaEventRecord(timer->ev[2 * timer->used], stream);
        }
    };
    auto te = [&]() {
        if (timer) cudaEventRecord(timer->ev[2 * timer->used++ + 1], stream);
    };
    // waves: k samples of a pixel range, k * npw <= cap
    for (uint32_t px0 = 0; px0 < npix;) {
        const uint32_t npw = npix - px0 < st.cap ? npix - px0 : st.cap;
        const uint32_t kmax = st.cap / npw;
        for (uint32_t s0 = 0; s0 < ns;) {
            const uint32_t k = ns - s0 < kmax ? ns - s0 : kmax;
            p.px0 = px0;
            p.npw = npw;
            p.sample0 = sbase + s0;
            p.si0 = s0;
            p.npaths = k * npw;
            if ((e = cudaMemsetAsync(st.counts, 0, kWfCounters * sizeof(uint32_t), stream)) != cudaSuccess) return e;
            tb(3);
            wf_camera<<<(p.npaths + 127) / 128, 128, 0, stream>>>(ubo, p);
            te();
            for (uint32_t b = 0; b < nb; ++b) {
                tb(0);
                if (s.cw_nodes) wf_extend<true><<<g_grid.extend, 128, 0, stream>>>(s, p, b);
                else wf_extend<false><<<g_grid.extend, 128, 0, stream>>>(s, p, b);
                te();
                tb(1);
                wf_shade<<<g_grid.shade, 128, 0, stream>>>(s, ubo, p, b);
                te();
                tb(2);
                if (s.cw_nodes) wf_shadow<true><<<g_grid.shadow, 128, 0, stream>>>(s, p, b);
                else wf_shadow<false><<<g_grid.shadow, 128, 0, stream>>>(s, p, b);
                te();
            }
            tb(3);
            wf_finish<<<(npw + 127) / 128, 128, 0, stream>>>(p, k);
            te();
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
            s0 += k;
        }
        px0 += npw;
    }
    tb(3);
    wf_resolve<<<(npix + 127) / 128, 128, 0, stream>>>(ubo, out, st.frame_sum);
    te();
    return cudaGetLastError();
}

}  // namespace gbrt

namespace gbrt {

// traceRayEXT queries (gbrt_trace_rays) through the persistent traversal of
// the world BVH in the layout the scene carries.
template <bool kAny, bool kWide>
__global__ void __launch_bounds__(128) trace_rays_persistent(DevScene s, const gbrt_ray* rays, uint32_t n,
                                                             uint32_t flags, gbrt_hit* hits, uint32_t* work,
                                                             DeviceCounters* cnt) {
    TraceStats ts{0, 0, 0};
    world_trace<kAny, kWide>(
        s, n, work, flags, ts,
        [&](uint32_t q, float3& o, float3& d, float& tmin, float& tmax, AnyCtx& ctx) {
            const gbrt_ray r = rays[q];
            o = f3(r.org[0], r.org[1], r.org[2]);
            d = f3(r.dir[0], r.dir[1], r.dir[2]);
            tmin = r.tmin;
            tmax = r.tmax;
            ctx = AnyCtx{q, 0u, 0u, 0u};
        },
        [&](uint32_t q, bool hit, const Hit& h) {
            gbrt_hit g;
            g.t = hit ? h.t : -1.0f;
            g.u = hit ? h.u : 0.0f;
            g.v = hit ? h.v : 0.0f;
            g.instance_id = hit ? h.inst : 0xFFFFFFFFu;
            g.primitive_id = hit ? h.prim : 0xFFFFFFFFu;
            g.custom_index = hit ? s.inst[h.inst].custom : 0xFFFFFFFFu;
            hits[q] = g;
        });
    if (cnt) {
        const unsigned long long nodes = warp_sum<unsigned long long>(ts.nodes);
        const unsigned long long tris = warp_sum<unsigned long long>(ts.tris);
        uint32_t stat = ts.status;
        for (int o = 16; o > 0; o >>= 1) stat |= __shfl_down_sync(0xFFFFFFFFu, stat, o);
        if ((threadIdx.x & 31u) == 0) {
            atomicAdd(&cnt->nodes, nodes);
            atomicAdd(&cnt->tris, tris);
            if (stat) atomicOr(&cnt->status, stat);
        }
    }
}

cudaError_t launch_trace_rays_persistent(const DevScene& s, const gbrt_ray* rays, uint32_t n, uint32_t flags,
                                         gbrt_hit* hits, uint32_t* work, DeviceCounters* cnt, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    cudaError_t e = grids(g_grid);
    if (e != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(work, 0, sizeof(uint32_t), st)) != cudaSuccess) return e;
    const uint32_t need = (n + 127) / 128;
    const uint32_t grid = need < (uint32_t)g_grid.extend ? need : (uint32_t)g_grid.extend;
    const bool any = flags & GBRT_RAY_TERMINATE_ON_FIRST;
    if (s.cw_nodes) {
        if (any) trace_rays_persistent<true, true><<<grid, 128, 0, st>>>(s, rays, n, flags, hits, work, cnt);
        else trace_rays_persistent<false, true><<<grid, 128, 0, st>>>(s, rays, n, flags, hits, work, cnt);
    } else {
        if (any) trace_rays_persistent<true, false><<<grid, 128, 0, st>>>(s, rays, n, flags, hits, work, cnt);
        else trace_rays_persistent<false, false><<<grid, 128, 0, st>>>(s, rays, n, flags, hits, work, cnt);
    }
    return cudaGetLastError();
}

}  // namespace gbrt
