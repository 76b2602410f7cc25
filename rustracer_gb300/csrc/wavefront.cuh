// wavefront.cuh — device code of the wavefront path tracer, shared by the
// single-frame kernels (wavefront.cu: the wave is one job and one segment,
// passed as a kernel parameter) and the batched kernels (wave_multi.cu: up to
// kMaxWaveJobs jobs and kMaxWaveSegs segments in constant memory).
//
// A wave is traced as camera -> for each bounce { extend (closest hit) ->
// shade (closest-hit / miss shaders, Russian roulette, next ray, NEE shadow
// record) -> shadow (any-hit) } -> finish (per-pixel sums in sample order).
// Each stage is a small kernel, so the instruction working set fits the cache
// and lanes of a warp run the same stage; queues between stages are compacted
// with warp ballots (one atomic per warp).  Results are bit-identical to the
// megakernel: the same device functions run in the same order per path, the
// NEE term is added as (E + C) after the shadow test like
// RayTracing.rchit:346-349.
//
// A wave view W gives the kernels: block_job(stage) (the job a block serves),
// blk0 / nblk (that job's blocks), job(j), seg(i), seg_of_path(pid),
// seg_of_fin(i), npaths(), nfin().
#pragma once
#include "hitgroup.cuh"
#include "kernels.h"
#include "persistent.cuh"

// Resident 128-thread blocks per SM the traversal kernels (extend, shadow)
// are compiled for: 7 gives them 72 registers (a few dozen bytes of spills)
// at 28 warps per SM.  The traversal waits on dependent node loads, so warps
// pay more than registers: on the icosphere frame with the clustered BVH,
// 4 / 5 / 6 / 7 / 8 blocks gave 3472 / 3768 / 4046 / 4159 / 4134 Mrays/s.
#ifndef GBRT_TRACE_MINB
#define GBRT_TRACE_MINB 7
#endif
// Same bound for every traversal form.
constexpr int trace_minb(int) { return GBRT_TRACE_MINB; }

// Launches traversal kernel K in the form `mode` (trace_mode, with
// kTraceOpaque when nothing in the launch can need the alpha test).
#define GBRT_TRACE_LAUNCH(K, grid, strm, ...)                                                       \
    switch (mode) {                                                                                 \
        case kTraceWide: K<kTraceWide><<<grid, 128, 0, strm>>>(__VA_ARGS__); break;                 \
        case kTraceWideTlas: K<kTraceWideTlas><<<grid, 128, 0, strm>>>(__VA_ARGS__); break;         \
        case kTraceBinary: K<kTraceBinary><<<grid, 128, 0, strm>>>(__VA_ARGS__); break;             \
        case kTraceWide | kTraceOpaque: K<kTraceWide | kTraceOpaque><<<grid, 128, 0, strm>>>(__VA_ARGS__); break; \
        case kTraceWideTlas | kTraceOpaque:                                                         \
            K<kTraceWideTlas | kTraceOpaque><<<grid, 128, 0, strm>>>(__VA_ARGS__);                  \
            break;                                                                                  \
        default: K<kTraceBinary | kTraceOpaque><<<grid, 128, 0, strm>>>(__VA_ARGS__); break;        \
    }

// With the ray-sort key, shadow rays are grouped by octant too; shade blocks
// of 256 threads make the groups twice as long (icosphere frame: 3719 Mrays/s
// with neither, 3748 with both).
#ifndef GBRT_SHADE_THREADS
#define GBRT_SHADE_THREADS 256
#endif

namespace gbrt {

// 2 blocks of 256: at most 128 registers, no spills.  Sweep on the icosphere
// frame: (256, 2) 3768 Mrays/s; (256, 3) 3677 and (128, 6) 3659 with 80
// registers and spills; (256, 1) let ptxas take more registers, one block per
// SM, 3010.
#ifndef GBRT_SHADE_MINB
#define GBRT_SHADE_MINB 2
#endif
// The form without textures, specular-glossiness and debug shading fits 80
// registers: 2 blocks of 384 threads (24 warps per SM).  Icosphere frame,
// threads x blocks: 128 x 6 4627, 192 x 4 4656, 256 x 3 4609, 384 x 2 4689
// Mrays/s (larger blocks make longer octant-grouped runs of rays and the
// barrier of the grouped append waits on fewer partial blocks).
#ifndef GBRT_SHADE_PLAIN_THREADS
#define GBRT_SHADE_PLAIN_THREADS 384
#endif
#ifndef GBRT_SHADE_PLAIN_MINB
#define GBRT_SHADE_PLAIN_MINB 2
#endif
constexpr int kShadeThreads = GBRT_SHADE_THREADS;  // block size of the shade kernels
constexpr int kShadeMinBlocks = GBRT_SHADE_MINB;   // resident blocks per SM the shade kernels are compiled for
// ... and of the form without textures, specular-glossiness and debug shading
constexpr int kShadePlainThreads = GBRT_SHADE_PLAIN_THREADS;
constexpr int kShadePlainMinBlocks = GBRT_SHADE_PLAIN_MINB;

GB_D uint32_t lane_id() { return threadIdx.x & 31u; }

// Warp-aggregated queue append: every lane of the warp calls it; lanes with
// want == true get consecutive slots.
GB_D uint32_t warp_append(uint32_t* counter, bool want) {
    const uint32_t mask = __ballot_sync(0xFFFFFFFFu, want);
    uint32_t base = 0;
    if (lane_id() == 0 && mask) base = atomicAdd(counter, (uint32_t)__popc(mask));
    base = __shfl_sync(0xFFFFFFFFu, base, 0);
    return base + __popc(mask & ((1u << lane_id()) - 1u));
}

// Block-wide appends to two queues (the extension and the shadow queue)
// grouped by a 3-bit key (the ray's direction octant): each queue gets one
// contiguous range per block, key 0 first, so a warp that later takes
// consecutive entries sees rays of few octants.  Order within a key is
// unspecified (every consumer indexes path state by the path id the entry
// carries).  Every thread of the block calls it.  Two barriers per call: the
// 34-word work areas `cur` and `nxt` alternate between calls, and each call
// clears the bins of the next one's area between its barriers (the caller
// clears both before the first call).
GB_D uint32_t group_rank(bool want, uint32_t key, uint32_t* bins) {
    const uint32_t peers = __match_any_sync(0xFFFFFFFFu, want ? key : 8u);
    const uint32_t leader = __ffs(peers) - 1u;
    uint32_t base = 0;
    if (want && lane_id() == leader) base = atomicAdd(&bins[key], (uint32_t)__popc(peers));
    base = __shfl_sync(0xFFFFFFFFu, base, leader);
    return base + __popc(peers & ((1u << lane_id()) - 1u));
}

GB_D void block_append2_by_key(uint32_t* counter_a, bool want_a, uint32_t key_a, uint32_t* counter_b, bool want_b,
                               uint32_t key_b, uint32_t* cur, uint32_t* nxt, uint32_t& slot_a, uint32_t& slot_b) {
    // cur: [0, 8) queue a's bins, [8, 16) queue b's, [16, 32) their offsets, [32, 34) their bases
    const uint32_t ra = group_rank(want_a, key_a, cur), rb = group_rank(want_b, key_b, cur + 8);
    __syncthreads();
    if (threadIdx.x < 2) {  // thread 0: queue a, thread 1: queue b
        const uint32_t q = threadIdx.x;
        uint32_t tot = 0;
        for (int k = 0; k < 8; ++k) {
            cur[16 + 8 * q + k] = tot;
            tot += cur[8 * q + k];
        }
        cur[32 + q] = tot ? atomicAdd(q ? counter_b : counter_a, tot) : 0u;
    } else if (threadIdx.x < 18) {
        nxt[threadIdx.x - 2] = 0;  // nobody reads nxt between the previous call's first barrier and here
    }
    __syncthreads();
    slot_a = want_a ? cur[32] + cur[16 + key_a] + ra : 0u;
    slot_b = want_b ? cur[33] + cur[24 + key_b] + rb : 0u;
}

GB_D uint32_t octant_of(float3 d) { return (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u); }

template <class T>
GB_D T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
    return v;
}

// Counter slots of one job inside WfState::counts (reset at the start of
// every wave).
constexpr int kQueue = 0;     // [kQueue + b]: extension-queue length at bounce b
constexpr int kShadow = 32;   // [kShadow + b]: shadow-queue length at bounce b
constexpr int kWorkExt = 64;  // [kWorkExt + b]: fetch cursor of extend(b)
constexpr int kWorkSh = 96;   // [kWorkSh + b]: fetch cursor of shadow(b)
constexpr int kMaxBounces = 31;
constexpr uint32_t kPidMask = kMaxWavePaths - 1u;

struct PathXY {
    uint32_t pid, pix, x, y, j;  // wave path, pixel, coordinates, sample within the segment
    const WaveSeg* sg;
};

// Decodes a queue word (path id | segment << kPidBits) of a job with image width W.
template <class Wv>
GB_D PathXY decode_path(const Wv& w, uint32_t word, uint32_t W) {
    PathXY r;
    r.pid = word & kPidMask;
    r.sg = &w.seg(word >> kPidBits);
    const uint32_t local = r.pid - r.sg->path0;
    r.j = local / r.sg->npw;
    r.pix = r.sg->px0 + (local - r.j * r.sg->npw);
    r.y = r.pix / W;
    r.x = r.pix - r.y * W;
    return r;
}

GB_D void flush_trace_stats(const TraceStats& ts, DeviceCounters* c) {
    const unsigned long long nodes = warp_sum<unsigned long long>(ts.nodes);
    const unsigned long long tris = warp_sum<unsigned long long>(ts.tris);
    uint32_t stat = ts.status;
    for (int o = 16; o > 0; o >>= 1) stat |= __shfl_down_sync(0xFFFFFFFFu, stat, o);
    if (lane_id() == 0) {
        atomicAdd(&c->nodes, nodes);
        atomicAdd(&c->tris, tris);
        if (stat) atomicOr(&c->status, stat);
    }
}

// rgen:32-80 for every path of the wave: seeds (D1), camera ray, path state.
// Job j's first queue is its paths in order, at the paths' own positions.
template <class Wv>
GB_D void camera_body(const Wv& w, const WfState& st, uint32_t pid) {
    if (pid >= w.npaths()) return;
    const uint32_t si = w.seg_of_path(pid);
    const WaveSeg& sg = w.seg(si);
    const WaveJob& J = w.job(sg.job);
    if (pid == J.path0) st.counts[sg.job * kWfCounters + kQueue] = J.npaths;
    const uint32_t W = J.out.width;
    const uint32_t local = pid - sg.path0, j = local / sg.npw, pix = sg.px0 + (local - j * sg.npw);
    const uint32_t y = pix / W, x = pix - y * W;
    const uint32_t sample = sg.sample0 + j;
    uint32_t seed = tea16(tea16(x, y), sample);
    uint4 rng = make_uint4(x, y, sample, 0u);
    float3 o, d;
    float tfar;
    camera_ray(J.ubo, x, y, W, J.out.height, rng, seed, o, d, tfar);
    // .w of the origin: RandomSeed after the aperture draws.  The rest of the
    // path state starts from values that shade of bounce 0 sets itself
    // (initial_state), so it is not written here unless no bounce runs.
    st.ray_o[0][pid] = f4(o, __uint_as_float(seed));
    st.ray_d[0][pid] = f4(d, __uint_as_float(pid | si << kPidBits));
    if (J.ubo.number_of_bounces == 0u) {  // wf_finish reads radiance and Ray.t
        st.tp[pid] = f4(1.0f, 1.0f, 1.0f, 0.0f);
        st.rad[pid] = f4(0.0f, 0.0f, 0.0f, 0.0f);
    }
}

// The path state a camera ray starts with: throughput 1 (Ray.t = 0),
// radiance 0 (volume_dis = -1), hitPoint 0 with the RandomSeed the camera
// left in the origin's .w, the pixel stream's counter after the camera's
// anti-aliasing draws and the ray stream's seed (RayTracing.rgen:32-48, D1).
GB_D void initial_state(const gbrt_ubo& ubo, float seed_bits, uint32_t sample, float4& tp, float4& rad, float4& hp,
                        uint4& rg) {
    tp = f4(1.0f, 1.0f, 1.0f, 0.0f);
    rad = f4(0.0f, 0.0f, 0.0f, -1.0f);
    hp = f4(0.0f, 0.0f, 0.0f, seed_bits);
    rg = make_uint4(ubo.antialiasing ? 2u : 0u, 0u, tea16(sample, 0x9E3779B9u), 0u);
}

// traceRayEXT for the extension queue of bounce b (closest hit).
template <int kMode, class Wv>
GB_D void extend_body(const Wv& w, const WfState& st, uint32_t b, uint32_t jb) {
    const WaveJob& J = w.job(jb);
    uint32_t* cnt = st.counts + jb * kWfCounters;
    const uint32_t n = cnt[kQueue + b], R = J.path0;
    const float4* __restrict__ ro = st.ray_o[b & 1] + R;
    const float4* __restrict__ rd = st.ray_d[b & 1] + R;
    TraceStats ts{0, 0, 0};
    // the any-hit context (pixel and sample of a BLEND draw) is only read when an alpha test can run
    const bool alpha = !(J.flags & GBRT_RAY_OPAQUE) && !J.s.all_opaque;
    world_trace<false, kMode>(
        J.s, n, &cnt[kWorkExt + b], J.flags, ts,
        [&](uint32_t q, float3& o, float3& d, float& tmin, float& tmax, AnyCtx& ctx) {
            const float4 o4 = ro[q], d4 = rd[q];
            o = f3(o4);
            d = f3(d4);
            tmin = 0.001f;
            tmax = J.tfar;
            if (alpha) {
                const PathXY P = decode_path(w, __float_as_uint(d4.w), J.out.width);
                ctx = AnyCtx{P.x, P.y, P.sg->sample0 + P.j, b};
            }
        },
        [&](uint32_t q, bool hit, const Hit& h) {
            st.hit[R + q] = f4(hit ? h.t : -1.0f, h.u, h.v, __uint_as_float(hit ? h.inst : 0xFFFFFFFFu));
            st.hit_prim[R + q] = h.prim;
            if (b == 0 && J.out.primary_hits) {
                const PathXY P = decode_path(w, __float_as_uint(rd[q].w), J.out.width);
                gbrt_hit g;
                g.t = hit ? h.t : -1.0f;
                g.u = hit ? h.u : 0.0f;
                g.v = hit ? h.v : 0.0f;
                g.instance_id = hit ? h.inst : 0xFFFFFFFFu;
                g.primitive_id = hit ? h.prim : 0xFFFFFFFFu;
                g.custom_index = hit ? J.s.inst[h.inst].custom : 0xFFFFFFFFu;
                J.out.primary_hits[(size_t)P.pix * J.ns + P.sg->si0 + P.j] = g;
            }
        });
    flush_trace_stats(ts, J.out.counters);
    if (blockIdx.x == w.blk0(0, jb) && threadIdx.x == 0) {
        if (b == 0) atomicAdd(&J.out.counters->camera, (unsigned long long)n);
        else atomicAdd(&J.out.counters->extension, (unsigned long long)n);
    }
}

// Closest-hit / miss shading and the rest of rgen's bounce loop
// (RayTracing.rgen:94-128) for the extension queue of bounce b.
// Material roughness of a hit as the radiance cache sees it (factor only:
// metallic-roughness roughness, or 1 - glossiness for specular-glossiness).
GB_D float hit_roughness(const DevScene& s, uint32_t inst) {
    const gbrt_priminfo pi = s.prims[s.inst[inst].custom];
    const gbrt_material_raw& m = s.mats[pi.material_id];
    return m.workflow == 1u ? 1.0f - m.sg_specular_glossiness_factor[3] : m.roughness_factor;
}

GB_D uint32_t nrc_train_hash(uint32_t pix, uint32_t sample) {
    uint32_t h = pix * 0x9E3779B1u ^ (sample + 0x7F4A7C15u) * 0x85EBCA77u;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    return h & 0xFFFFu;
}

template <class Wv, bool kNrc = false, uint32_t kFeat = kFeatAll>
GB_D void shade_body(const Wv& w, const WfState& st, uint32_t b, const NrcWave* nrc = nullptr) {
    const uint32_t jb = w.block_job(1);
    const WaveJob& J = w.job(jb);
    const DevScene& s = J.s;
    const gbrt_ubo& ubo = J.ubo;
    uint32_t* cnt = st.counts + jb * kWfCounters;
    const uint32_t n = cnt[kQueue + b], R = J.path0;
    const float4* __restrict__ rd = st.ray_d[b & 1] + R;
    float4* no = st.ray_o[(b + 1) & 1] + R;
    float4* nd = st.ray_d[(b + 1) & 1] + R;
    const uint32_t nb = ubo.number_of_bounces;
    PathStats ps{0, 0, 0, 0, 0};
    const uint32_t blk0 = w.blk0(1, jb), nblk = w.nblk(1, jb);
    const uint32_t stride = nblk * blockDim.x;
    const bool sort_rays = s.sort_rays != 0u;
    __shared__ uint32_t s_key[2][34];
    uint32_t parity = 0;
    if (sort_rays) {  // block-uniform
        if (threadIdx.x < 68) (&s_key[0][0])[threadIdx.x] = 0;
        __syncthreads();
    }
    // block-uniform trip count (block_append2_by_key synchronises the block)
    for (uint32_t cbase = (blockIdx.x - blk0) * blockDim.x; cbase < n; cbase += stride) {
        const uint32_t q = cbase + threadIdx.x;
        const bool active = q < n;
        bool cont = false, shadow = false;
        float3 nxt_o = f3(0.0f), nxt_d = f3(0.0f), so = f3(0.0f), sd = f3(0.0f), sc = f3(0.0f), se = f3(0.0f);
        float3 tp_before = f3(0.0f);
        float stmax = 0.0f;
        uint32_t word = 0, nseed = 0;
        // radiance after this vertex with the shadow ray blocked / not; throughput, radiance and RNG
        // counters for the next bounce's queue
        float4 sh_blocked = make_float4(0.0f, 0.0f, 0.0f, 0.0f), sh_lit = sh_blocked;
        float4 q_tp_next = sh_blocked, q_rad_next = sh_blocked;
        uint4 q_rng_next = make_uint4(0u, 0u, 0u, 0u);
        if (active) {
            const float4 d4 = rd[q];
            const float3 d = f3(d4);
            word = __float_as_uint(d4.w);
            const PathXY P = decode_path(w, word, J.out.width);
            const uint32_t pid = P.pid;
            const float4 h4 = st.hit[R + q];
            float4 tp4, rad4, hp4;
            uint4 rg;
            if (b == 0u) {
                initial_state(ubo, st.ray_o[0][R + q].w, P.sg->sample0 + P.j, tp4, rad4, hp4, rg);
            } else {  // the hit point is this ray's origin, which carries RandomSeed
                tp4 = kNrc ? st.tp[pid] : st.q_tp[b & 1][R + q];
                rad4 = kNrc ? st.rad[pid] : st.q_rad[b & 1][R + q];
                hp4 = st.ray_o[b & 1][R + q];
                rg = kNrc ? st.rng[pid] : st.q_rng[b & 1][R + q];
            }
            Payload Rp;
            Rp.hitValue = Rp.scatterDir = Rp.emittance = f3(0.0f);
            Rp.needScatter = 0;
            Rp.hitPoint = f3(hp4);
            Rp.RandomSeed = __float_as_uint(hp4.w);
            Rp.t = tp4.w;
            Rp.volume_dis = rad4.w;
            Rp.rngState = make_uint4(P.x, P.y, rg.z, rg.y);
            const uint32_t inst = __float_as_uint(h4.w);
            bool cached = false;  // a render path stopping at the radiance cache
            bool stop_after = false;  // primary-indirect mode: shade this camera hit, then stop at the cache
            if constexpr (kNrc) {
                const bool train = nrc_train_hash(P.pix, P.sg->sample0 + P.j) < nrc->train_thresh;
                if (nrc->mode == 1u) {
                    // camera hit: render paths take the cache's indirect radiance after shading it;
                    // training paths mark the vertex (w = 2) and record the radiance gathered so far
                    // at the next bounce (after this vertex's emission and shadow-tested NEE)
                    if (b == 0u && inst != 0xFFFFFFFFu && hit_roughness(s, inst) >= nrc->min_roughness) {
                        const float3 o = f3(st.ray_o[0][R + q]);
                        const float3 x = f3(fmaf(h4.x, d.x, o.x), fmaf(h4.x, d.y, o.y), fmaf(h4.x, d.z, o.z));
                        if (train) {
                            nrc->snap_pos[pid] = f4(x, 2.0f);
                            nrc->snap_tp[pid] = f4(1.0f, 1.0f, 1.0f, 0.0f);
                        } else if (!nrc->disabled) {
                            stop_after = true;
                            const uint32_t k = atomicAdd(&nrc->counts[0], 1u);
                            nrc->query[k] = f4(x, __uint_as_float(word));
                        }
                    } else if (b == 1u && train && nrc->snap_pos[pid].w == 2.0f) {
                        nrc->snap_pos[pid].w = 1.0f;
                        nrc->snap_rad[pid] = rad4;
                    }
                } else if (b >= 1u && inst != 0xFFFFFFFFu && (train || !nrc->disabled) &&
                    hit_roughness(s, inst) >= nrc->min_roughness) {
                    const float3 o = f3(st.ray_o[b & 1][R + q]);
                    const float3 x = f3(fmaf(h4.x, d.x, o.x), fmaf(h4.x, d.y, o.y), fmaf(h4.x, d.z, o.z));
                    if (train) {
                        if (nrc->snap_pos[pid].w == 0.0f) {
                            nrc->snap_pos[pid] = f4(x, 1.0f);
                            nrc->snap_rad[pid] = rad4;
                            nrc->snap_tp[pid] = tp4;
                        }
                    } else {
                        cached = true;
                        const uint32_t k = atomicAdd(&nrc->counts[b], 1u);
                        nrc->query[k] = f4(x, __uint_as_float(word));
                    }
                }
            }
            if (cached) {
            } else if (inst != 0xFFFFFFFFu) {
                Hit h;
                h.t = h4.x;
                h.u = h4.y;
                h.v = h4.z;
                h.inst = inst;
                h.prim = st.hit_prim[R + q];
                h.bgeo = 0;
                closest_hit<kFeat>(s, ubo, Rp, h, d, ps, [&](float3 o_, float3 d_, float t_, float3 C) {
                    shadow = true;
                    so = o_;
                    sd = d_;
                    stmax = t_;
                    sc = C;
                });
            } else {
                miss_shader(s, ubo, Rp, d);
            }
            if (!cached) {
            float3 tp = f3(tp4);
            float3 rad = f3(rad4);
            tp_before = tp;
            se = Rp.emittance;
            if (!shadow) rad += tp * Rp.emittance;
            cont = b + 1 != nb;
            if (cont && b > 3u) {  // Russian roulette, rgen:108-118
                uint4 prng = make_uint4(P.x, P.y, P.sg->sample0 + P.j, rg.x);
                const float pr = clampf(luminance(tp), 0.01f, 0.95f);
                if (pr < pcg_rand(prng)) cont = false;
                else tp /= pr;
                rg.x = prng.w;
            }
            if (cont) {
                tp *= Rp.hitValue;
                if (!Rp.needScatter || Rp.t < 0.0f) cont = false;
            }
            if (stop_after) cont = false;
            // .w of the radiance: volume_dis while the path goes on, its last Ray.t once it has
            // ended (wf_finish reads it); frames with a radiance cache keep Ray.t in tp
            const float rad_w = (kNrc || cont) ? Rp.volume_dis : Rp.t;
            if (kNrc || (!shadow && !cont)) {
                st.rad[pid] = f4(rad, rad_w);
            } else if (!shadow) {
                q_rad_next = f4(rad, rad_w);
            } else {  // the shadow kernel writes the radiance: E + C when the light is visible (rchit:338-350)
                sh_blocked = f4(rad + tp_before * se, rad_w);
                sh_lit = f4(rad + tp_before * (se + sc), rad_w);
            }
            if constexpr (kNrc) {
                st.tp[pid] = f4(tp, Rp.t);
                if (cont) st.rng[pid] = make_uint4(rg.x, Rp.rngState.w, rg.z, 0u);  // read again only by a next bounce
            } else {  // written beside the next extension ray, in queue order
                q_tp_next = f4(tp, Rp.t);
                q_rng_next = make_uint4(rg.x, Rp.rngState.w, rg.z, 0u);
            }
            nxt_o = Rp.hitPoint;
            nxt_d = Rp.scatterDir;
            nseed = Rp.RandomSeed;
            }
        }
        uint32_t slot, sslot;
        if (sort_rays) {
            block_append2_by_key(&cnt[kQueue + b + 1], cont, octant_of(nxt_d), &cnt[kShadow + b], shadow,
                                 octant_of(sd), s_key[parity], s_key[parity ^ 1u], slot, sslot);
            parity ^= 1u;
        } else {
            slot = warp_append(&cnt[kQueue + b + 1], cont);
            sslot = warp_append(&cnt[kShadow + b], shadow);
        }
        if (cont) {
            no[slot] = f4(nxt_o, __uint_as_float(nseed));
            if constexpr (!kNrc) {
                st.q_tp[(b + 1) & 1][R + slot] = q_tp_next;
                st.q_rng[(b + 1) & 1][R + slot] = q_rng_next;
                if (!shadow) st.q_rad[(b + 1) & 1][R + slot] = q_rad_next;
            }
            nd[slot] = f4(nxt_d, __uint_as_float(word));
        }
        if (shadow) {
            st.sh_o[R + sslot] = f4(so, stmax);
            st.sh_d[R + sslot] = f4(sd, __uint_as_float(word));
            if constexpr (kNrc) {
                st.sh_e[R + sslot] = f4(se, tp_before.x);
                st.sh_c[R + sslot] = f4(sc, tp_before.y);
                st.sh_tp[R + sslot] = tp_before.z;
            } else {
                st.sh_e[R + sslot] = sh_blocked;
                st.sh_c[R + sslot] = sh_lit;
                st.sh_tp[R + sslot] = __uint_as_float(cont ? slot | kDstQueue : word & kPidMask);
            }
        }
    }
    const unsigned long long hs = warp_sum<unsigned long long>(ps.shaded);
    if (lane_id() == 0 && hs) atomicAdd(&J.out.counters->shaded, hs);
}

// Any-hit shadow rays of bounce b (castShadowRay, RayTracing.rchit:35-59),
// then the deferred radiance update radiance += tp * (E [+ C if unoccluded]).
template <int kMode, class Wv>
GB_D void shadow_body(const Wv& w, const WfState& st, uint32_t b, uint32_t jb) {
    const WaveJob& J = w.job(jb);
    uint32_t* cnt = st.counts + jb * kWfCounters;
    const uint32_t n = cnt[kShadow + b], R = J.path0;
    const float4* __restrict__ so = st.sh_o + R;
    const float4* __restrict__ sd = st.sh_d + R;
    TraceStats ts{0, 0, 0};
    const uint32_t flags = GBRT_RAY_TERMINATE_ON_FIRST | J.flags;
    const bool alpha = !(J.flags & GBRT_RAY_OPAQUE) && !J.s.all_opaque;
    world_trace<true, kMode>(
        J.s, n, &cnt[kWorkSh + b], flags, ts,
        [&](uint32_t q, float3& o, float3& d, float& tmin, float& tmax, AnyCtx& ctx) {
            const float4 o4 = so[q], d4 = sd[q];
            o = f3(o4);
            d = f3(d4);
            tmin = 0.1f;
            tmax = o4.w;
            if (alpha) {
                const PathXY P = decode_path(w, __float_as_uint(d4.w), J.out.width);
                ctx = AnyCtx{P.x, P.y, P.sg->sample0 + P.j, b | 0x100u};
            }
        },
        [&](uint32_t q, bool occluded, const Hit&) {
            if (!(J.flags & kShadowDelta)) {  // the record holds both outcomes and where they go
                const uint32_t dst = __float_as_uint(st.sh_tp[R + q]);
                const float4 v = occluded ? st.sh_e[R + q] : st.sh_c[R + q];
                if (dst & kDstQueue) st.q_rad[(b + 1) & 1][R + (dst & ~kDstQueue)] = v;
                else st.rad[dst] = v;
                return;
            }
            const uint32_t pid = __float_as_uint(sd[q].w) & kPidMask;
            const float4 e4 = st.sh_e[R + q], c4 = st.sh_c[R + q];
            const float tpz = st.sh_tp[R + q];
            float3 e = f3(e4);
            if (!occluded) e += f3(c4);
            const float4 r = st.rad[pid];
            const float3 rad = f3(r) + f3(e4.w, c4.w, tpz) * e;
            st.rad[pid] = f4(rad, r.w);
        });
    flush_trace_stats(ts, J.out.counters);
    if (blockIdx.x == w.blk0(2, jb) && threadIdx.x == 0)
        atomicAdd(&J.out.counters->shadow, (unsigned long long)n);
}

// Per pixel of every segment: add its samples' radiance to the job's frame
// sum in sample order (the megakernel's per-pixel order), keep the last Ray.t.
template <class Wv, bool kNrc = false>
GB_D void finish_body(const Wv& w, const WfState& st, uint32_t i, const NrcWave* nrc = nullptr) {
    if (i >= w.nfin()) return;
    const WaveSeg& sg = w.seg(w.seg_of_fin(i));
    const WaveJob& J = w.job(sg.job);
    const uint32_t li = i - sg.fin0, pix = sg.px0 + li;
    float4 acc = J.frame_sum[pix];
    float3 sum = f3(acc);
    float last_t = acc.w;
    for (uint32_t j = 0; j < sg.k; ++j) {
        const uint32_t pid = sg.path0 + li + j * sg.npw;
        const float4 r4 = st.rad[pid];
        const float3 r = f3(r4);
        if (J.out.sample_radiance) {
            float* sr = J.out.sample_radiance + ((size_t)pix * J.ns + sg.si0 + j) * 3;
            sr[0] = r.x;
            sr[1] = r.y;
            sr[2] = r.z;
        }
        sum += r;
        last_t = kNrc ? st.tp[pid].w : r4.w;
        if constexpr (kNrc) {  // training sample: suffix radiance / throughput at the vertex
            const float4 sp = nrc->snap_pos[pid];
            if (sp.w != 0.0f) {
                // w = 2: a marked camera hit whose path ended there: no indirect radiance
                const float3 r0 = sp.w == 2.0f ? r : f3(nrc->snap_rad[pid]), t0 = f3(nrc->snap_tp[pid]);
                const float3 dr = r - r0;
                const float3 tg = f3(t0.x > 0.0f ? dr.x / t0.x : 0.0f, t0.y > 0.0f ? dr.y / t0.y : 0.0f,
                                     t0.z > 0.0f ? dr.z / t0.z : 0.0f);
                const uint32_t k = atomicAdd(&nrc->counts[32], 1u);
                if (k < nrc->train_max) {
                    nrc->train_pos[k] = f4(f3(sp), 1.0f);
                    nrc->train_tgt[k] = f4(tg, 0.0f);
                }
            }
        }
    }
    J.frame_sum[pix] = f4(sum, last_t);
}

}  // namespace gbrt
