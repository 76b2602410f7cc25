// render.cu — the path-tracing megakernel (RayTracing.rgen + .rchit + .rmiss
// + shadow rays in one kernel) and the ray-query kernel.
//
// Launch shape: one thread per pixel, 8x16 pixel blocks (a warp covers an
// 8x4 tile, so primary rays of a warp are coherent); each thread runs the
// frame's samples in order, which keeps the per-pixel sum in the same order
// as the oracle.  Every sample seeds its own RNG streams from (pixel, global
// sample index) -- documented deviation D1 -- so samples are independent.
#include "hitgroup.cuh"
#include "kernels.h"

namespace gbrt {

GB_D float3 trace_path(const DevScene& s, const gbrt_ubo& ubo, uint32_t x, uint32_t y, uint32_t W, uint32_t H,
                       uint32_t sample, PathStats& ps, TraceStats& ts, gbrt_hit* primary, float& last_t) {
    Payload R;
    R.hitValue = R.hitPoint = R.scatterDir = R.emittance = f3(0.0f);
    R.needScatter = 0;
    R.RandomSeed = tea16(tea16(x, y), sample);  // D1
    uint4 rng = make_uint4(x, y, sample, 0u);
    R.rngState = make_uint4(x, y, tea16(sample, 0x9E3779B9u), 0u);
    float3 radiance = f3(0.0f);
    float3 o, d;
    float tFar;
    camera_ray(ubo, x, y, W, H, rng, R.RandomSeed, o, d, tFar);
    float3 throughput = f3(1.0f);
    R.t = 0.0f;
    R.volume_dis = -1.0f;
    const uint32_t flags = ubo.fully_opaque ? GBRT_RAY_OPAQUE : 0u;
    for (uint32_t b = 0; b < ubo.number_of_bounces; b++) {
        if (b == 0) ps.camera++; else ps.extension++;
        Hit h;
        const AnyCtx ctx{x, y, sample, b};
        const bool hit = trace_scene<false>(s, o, d, 0.001f, tFar, flags, ctx, h, ts);
        if (b == 0 && primary) {
            primary->t = hit ? h.t : -1.0f;
            primary->u = hit ? h.u : 0.0f;
            primary->v = hit ? h.v : 0.0f;
            primary->instance_id = hit ? h.inst : 0xFFFFFFFFu;
            primary->primitive_id = hit ? h.prim : 0xFFFFFFFFu;
            primary->custom_index = hit ? s.inst[h.inst].custom : 0xFFFFFFFFu;
        }
        if (hit) {
            closest_hit(s, ubo, R, h, d, ps, [&](float3 so, float3 sd, float stmax, float3 C) {
                Hit sh;
                const AnyCtx sctx{x, y, sample, b | 0x100u};
                if (!trace_scene<true>(s, so, sd, 0.1f, stmax, GBRT_RAY_TERMINATE_ON_FIRST | flags, sctx, sh, ts))
                    R.emittance += C;
            });
        }
        else miss_shader(s, ubo, R, d);
        const float3 hitColor = R.hitValue;
        const float t = R.t;
        const bool scattered = R.needScatter != 0;
        radiance += throughput * R.emittance;
        R.emittance = f3(0.0f);
        if (b + 1 == ubo.number_of_bounces) break;
        if (b > 3u) {  // Russian roulette after MIN_BOUNCES, rgen:15,108-118
            const float p = clampf(luminance(throughput), 0.01f, 0.95f);
            if (p < pcg_rand(rng)) break;
            throughput /= p;
        }
        throughput *= hitColor;
        if (!scattered || t < 0.0f) break;
        o = R.hitPoint;
        d = R.scatterDir;
    }
    last_t = R.t;
    return radiance;
}

__global__ void __launch_bounds__(128) pt_megakernel(DevScene s, gbrt_ubo ubo, RenderOut out) {
    const uint32_t x = blockIdx.x * 8 + (threadIdx.x & 7);
    const uint32_t y = blockIdx.y * 16 + (threadIdx.x >> 3);
    PathStats ps{0, 0, 0, 0, 0};
    TraceStats ts{0, 0, 0};
    const bool active = x < out.width && y < out.height;
    if (active) {
        const uint32_t ns = ubo.number_of_samples;
        const uint32_t sbase = ubo.total_number_of_samples - ns;
        const size_t pix = (size_t)y * out.width + x;
        float3 sum = f3(0.0f);
        float last_t = 0.0f;
        for (uint32_t si = 0; si < ns; ++si) {
            gbrt_hit* ph = out.primary_hits ? out.primary_hits + pix * ns + si : nullptr;
            const float3 r = trace_path(s, ubo, x, y, out.width, out.height, sbase + si, ps, ts, ph, last_t);
            if (out.sample_radiance) {
                float* sr = out.sample_radiance + (pix * ns + si) * 3;
                sr[0] = r.x;
                sr[1] = r.y;
                sr[2] = r.z;
            }
            sum += r;
        }
        // accumulation + tone map, rgen:132-166
        const bool accumulate = ubo.number_of_samples != ubo.total_number_of_samples;
        float4 prev = accumulate ? out.accum[pix] : f4(0.0f, 0.0f, 0.0f, 0.0f);
        const float3 acc = f3(prev) + sum;
        out.accum[pix] = f4(acc, 0.0f);
        float3 c = tonemap(ubo.tone_mapping_mode, acc / float(ubo.total_number_of_samples));
        if (ubo.mapping == 4u)  // DISTANCE
            c = f3(fminf((ubo.heatmap_scale - fmaxf(last_t, 0.001f)) / ubo.heatmap_scale, 1.0f));
        if (out.rgba8)
            out.rgba8[pix] = make_uchar4(to_unorm8(c.x), to_unorm8(c.y), to_unorm8(c.z), 255);
    }
    // per-warp reduction of the counters, one atomic per warp and counter
    unsigned long long cam = ps.camera, ext = ps.extension, sh = ps.shadow, hs = ps.shaded;
    unsigned long long nodes = ts.nodes, tris = ts.tris;
    uint32_t st = ts.status;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        cam += __shfl_down_sync(0xFFFFFFFFu, cam, o);
        ext += __shfl_down_sync(0xFFFFFFFFu, ext, o);
        sh += __shfl_down_sync(0xFFFFFFFFu, sh, o);
        hs += __shfl_down_sync(0xFFFFFFFFu, hs, o);
        nodes += __shfl_down_sync(0xFFFFFFFFu, nodes, o);
        tris += __shfl_down_sync(0xFFFFFFFFu, tris, o);
        st |= __shfl_down_sync(0xFFFFFFFFu, st, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&out.counters->camera, cam);
        atomicAdd(&out.counters->extension, ext);
        atomicAdd(&out.counters->shadow, sh);
        atomicAdd(&out.counters->shaded, hs);
        atomicAdd(&out.counters->nodes, nodes);
        atomicAdd(&out.counters->tris, tris);
        if (st) atomicOr(&out.counters->status, st);
    }
}

template <bool kAny>
__global__ void __launch_bounds__(128) trace_rays_kernel(DevScene s, const gbrt_ray* rays, uint32_t n,
                                                         uint32_t flags, gbrt_hit* hits, DeviceCounters* cnt) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    TraceStats ts{0, 0, 0};
    if (i < n) {
        const gbrt_ray r = rays[i];
        Hit h;
        const AnyCtx ctx{i, 0u, 0u, 0u};
        const bool hit = trace_scene<kAny>(s, f3(r.org[0], r.org[1], r.org[2]), f3(r.dir[0], r.dir[1], r.dir[2]),
                                           r.tmin, r.tmax, flags, ctx, h, ts);
        gbrt_hit o;
        o.t = hit ? h.t : -1.0f;
        o.u = hit ? h.u : 0.0f;
        o.v = hit ? h.v : 0.0f;
        o.instance_id = hit ? h.inst : 0xFFFFFFFFu;
        o.primitive_id = hit ? h.prim : 0xFFFFFFFFu;
        o.custom_index = hit ? s.inst[h.inst].custom : 0xFFFFFFFFu;
        hits[i] = o;
    }
    if (cnt) {
        unsigned long long nodes = ts.nodes, tris = ts.tris;
        uint32_t st = ts.status;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            nodes += __shfl_down_sync(0xFFFFFFFFu, nodes, o);
            tris += __shfl_down_sync(0xFFFFFFFFu, tris, o);
            st |= __shfl_down_sync(0xFFFFFFFFu, st, o);
        }
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(&cnt->nodes, nodes);
            atomicAdd(&cnt->tris, tris);
            if (st) atomicOr(&cnt->status, st);
        }
    }
}

// --- host launchers --------------------------------------------------------
cudaError_t init_render_constants(const float* srgb_lut) {
    return cudaMemcpyToSymbol(c_srgb_lut, srgb_lut, 256 * sizeof(float));
}

cudaError_t launch_megakernel(const DevScene& s, const gbrt_ubo& ubo, const RenderOut& out, cudaStream_t st) {
    dim3 grid((out.width + 7) / 8, (out.height + 15) / 16);
    pt_megakernel<<<grid, 128, 0, st>>>(s, ubo, out);
    return cudaGetLastError();
}

cudaError_t launch_trace_rays(const DevScene& s, const gbrt_ray* rays, uint32_t n, uint32_t flags, gbrt_hit* hits,
                              DeviceCounters* cnt, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    const uint32_t blocks = (n + 127) / 128;
    if (flags & GBRT_RAY_TERMINATE_ON_FIRST)
        trace_rays_kernel<true><<<blocks, 128, 0, st>>>(s, rays, n, flags, hits, cnt);
    else
        trace_rays_kernel<false><<<blocks, 128, 0, st>>>(s, rays, n, flags, hits, cnt);
    return cudaGetLastError();
}

}  // namespace gbrt
