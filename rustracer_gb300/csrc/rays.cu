// rays.cu — gbrt_trace_rays: ray queries through the persistent world
// traversal (8-wide when the scene carries it).
#include "wavefront.cuh"

namespace gbrt {

// traceRayEXT queries (gbrt_trace_rays) through the persistent traversal of
// the world BVH in the layout the scene carries.
template <bool kAny, int kMode>
__global__ void __launch_bounds__(128) trace_rays_persistent(DevScene s, const gbrt_ray* rays, uint32_t n,
                                                             uint32_t flags, gbrt_hit* hits, uint32_t* work,
                                                             DeviceCounters* cnt) {
    TraceStats ts{0, 0, 0};
    world_trace<kAny, kMode>(
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
    static int dev_cached = -1, resident = 0;  // blocks of the persistent kernel that fit the GPU
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev != dev_cached) {
        int sms = 0, per = 0;
        if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, trace_rays_persistent<false, kTraceWideTlas>, 128, 0)) !=
            cudaSuccess)
            return e;
        resident = sms * (per > 0 ? per : 1);
        dev_cached = dev;
    }
    if ((e = cudaMemsetAsync(work, 0, sizeof(uint32_t), st)) != cudaSuccess) return e;
    const uint32_t need = (n + 127) / 128;
    const uint32_t grid = need < (uint32_t)resident ? need : (uint32_t)resident;
    const bool any = flags & GBRT_RAY_TERMINATE_ON_FIRST;
    // ray queries use the 8-wide form with the TLAS (it skips the TLAS of
    // scenes without one), or the binary form where the scene needs it
    if (trace_mode(s) != kTraceBinary) {
        if (any) trace_rays_persistent<true, kTraceWideTlas><<<grid, 128, 0, st>>>(s, rays, n, flags, hits, work, cnt);
        else trace_rays_persistent<false, kTraceWideTlas><<<grid, 128, 0, st>>>(s, rays, n, flags, hits, work, cnt);
    } else {
        if (any) trace_rays_persistent<true, kTraceBinary><<<grid, 128, 0, st>>>(s, rays, n, flags, hits, work, cnt);
        else trace_rays_persistent<false, kTraceBinary><<<grid, 128, 0, st>>>(s, rays, n, flags, hits, work, cnt);
    }
    return cudaGetLastError();
}

}  // namespace gbrt
