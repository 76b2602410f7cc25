// persistent.cuh — persistent-lane traversal of the world BVH with ray
// refill (after Aila & Laine 2009, "Understanding the Efficiency of Ray
// Traversal on GPUs").
//
// Every lane owns one ray at a time.  Each outer iteration a lane descends
// inner nodes until it reaches a leaf (or its stack empties), then tests that
// leaf's triangles (while-while).  A lane whose ray finished goes idle; once
// at least kRefill lanes of the warp are idle they take new rays from the
// queue together (one atomic per warp).  The warp therefore no longer waits
// for its longest ray, which is what kept SIMT efficiency low when a warp
// traced a fixed group of 32 rays.  The stack holds (node, entry distance)
// pairs so entries behind the current closest hit are dropped when popped.
//
// Scenes with transformed instances finish each ray with the two-level pass
// of trace.cuh after the world BVH (same exactness rules).
#pragma once
#include "trace.cuh"

namespace gbrt {

constexpr int kEmpty = 0x7FFFFFFF;  // "stack exhausted"
// icosphere frame (8-wide, clustered BVH, 7 blocks per SM): 4 / 8 / 12 / 16 /
// 20 / 24 idle lanes gave 4034 / 4174 / 4225 / 4288 / 4262 / 4183 Mrays/s
// Entries of the 8-wide traversal stack kept in shared memory (0: the whole
// stack in local memory, which stays in L1).  Icosphere frame: 4254 Mrays/s
// with 0, 4258 with 8, 4256 with 16 (noise), so L1 keeps its capacity for
// nodes and triangles.
#ifndef GBRT_CW_SMEM_STACK
#define GBRT_CW_SMEM_STACK 0
#endif
#ifndef GBRT_REFILL
#define GBRT_REFILL 16
#endif
constexpr uint32_t kRefill = GBRT_REFILL;  // idle lanes that trigger a refill

// Loader: bool load(uint32_t q, float3& o, float3& d, float& tmin, float& tmax, AnyCtx& ctx)
// Finisher: void finish(uint32_t q, bool hit, const Hit& h)
template <bool kAny, bool kAlpha, class Loader, class Finisher>
GB_D void persistent_trace(const DevScene& s, uint32_t n, uint32_t* work, uint32_t flags, TraceStats& ts,
                           Loader&& load, Finisher&& finish) {
    const uint32_t lane = threadIdx.x & 31u;
    const bool test_alpha = kAlpha && !(flags & GBRT_RAY_OPAQUE) && !s.all_opaque;
    int stack_node[kStack];
    float stack_t[kStack];
    bool has = false, exhausted = false;
    uint32_t q = 0;
    TRay r;
    Hit best;
    float best_det = 1.0f;  // any-hit queries: best.u, best.v hold V, W of the world hit until the ray is done
    AnyCtx ctx{0, 0, 0, 0};
    float tmin = 0.0f, tmax = 0.0f;
    int cur = kEmpty, sp = 0;
    uint32_t iter = 0;
    for (;;) {
        if (!exhausted) {
            const uint32_t idle = __ballot_sync(0xFFFFFFFFu, !has);
            if (__popc(idle) >= (int)kRefill) {
                uint32_t base = 0;
                if (lane == 0) base = atomicAdd(work, (uint32_t)__popc(idle));
                base = __shfl_sync(0xFFFFFFFFu, base, 0);
                if (base + __popc(idle) >= n) exhausted = true;
                if (!has) {
                    q = base + __popc(idle & ((1u << lane) - 1u));
                    if (q < n) {
                        float3 o, d;
                        load(q, o, d, tmin, tmax, ctx);
                        best.t = tmax;
                        best.u = best.v = 0.0f;
                        best_det = 1.0f;
                        best.inst = best.prim = best.bgeo = 0xFFFFFFFFu;
                        iter = 0;
                        if (d.x == 0.0f && d.y == 0.0f && d.z == 0.0f) {
                            finish(q, false, best);
                        } else {
                            has = true;
                            setup_ray(r, o, d);
                            sp = 0;
                            cur = kEmpty;
                            float tn;
                            if (s.has_world && box_hit(r, s.world_lo.x, s.world_hi.x, s.world_lo.y, s.world_hi.y,
                                                       s.world_lo.z, s.world_hi.z, tmin, best.t, tn))
                                cur = s.world_root;
                        }
                    }
                }
            }
        }
        if (!__any_sync(0xFFFFFFFFu, has)) {
            if (exhausted) break;
            continue;
        }
        if (!has) continue;
        // --- descend to a leaf ------------------------------------------------
        int leaf = 0;
        while (cur != kEmpty) {
            if (++iter > kMaxIter) {
                ts.status |= GBRT_STATUS_ITER_LIMIT;
                cur = kEmpty;
                break;
            }
            if (cur < 0) {  // leaf: take it, resume from the stack afterwards
                leaf = cur;
                cur = kEmpty;
                while (sp > 0) {
                    --sp;
                    if (stack_t[sp] <= best.t) {
                        cur = stack_node[sp];
                        break;
                    }
                }
                break;
            }
            const BNode2* nd = s.nodes + cur;
            const float4 a = __ldg(&nd->lxy), b = __ldg(&nd->rxy), z = __ldg(&nd->lrz);
            const int4 c = __ldg(&nd->c);
            ts.nodes++;
            float tn0, tn1;
            const bool h0 = box_hit(r, a.x, a.y, a.z, a.w, z.x, z.y, tmin, best.t, tn0);
            const bool h1 = box_hit(r, b.x, b.y, b.z, b.w, z.z, z.w, tmin, best.t, tn1);
            if (h0 && h1) {
                const bool swap = tn1 < tn0;
                if (sp < kStack) {
                    stack_node[sp] = swap ? c.x : c.y;
                    stack_t[sp] = swap ? tn0 : tn1;
                    ++sp;
                } else {
                    ts.status |= GBRT_STATUS_STACK_OVERFLOW;
                }
                cur = swap ? c.y : c.x;
            } else if (h0) {
                cur = c.x;
            } else if (h1) {
                cur = c.y;
            } else {
                cur = kEmpty;
                while (sp > 0) {
                    --sp;
                    if (stack_t[sp] <= best.t) {
                        cur = stack_node[sp];
                        break;
                    }
                }
            }
        }
        // --- test the leaf ------------------------------------------------------
        bool done = false;
        if (leaf != 0) {
            const uint32_t first = leaf_first(leaf), count = leaf_count(leaf);
            for (uint32_t i = 0; i < count; ++i) {
                const TriRec* tr = s.tris + first + i;
                const float4 pa = __ldg(&tr->a), pb = __ldg(&tr->b), pc = __ldg(&tr->c);
                ts.tris++;
                // any-hit queries keep V, W and det of the hit and divide once the ray is done (if
                // their caller reads u, v at all); closest-hit queries divide per accepted hit
                float t, u, v, det = 1.0f;
                if constexpr (kAny) {
                    if (!isect_tri_t(r, f3(pa), f3(pb), f3(pc), tmin, best.t, t, u, v, det)) continue;
                } else {
                    if (!isect_tri(r, f3(pa), f3(pb), f3(pc), tmin, best.t, t, u, v)) continue;
                }
                const uint32_t inst = __float_as_uint(pa.w);
                const uint32_t prim = __float_as_uint(pb.w);
                const uint32_t gw = __float_as_uint(pc.w);
                if (!closer(t, inst, prim, best)) continue;
                if (test_alpha && !(gw >> 31) &&
                    anyhit_ignore(s, s.inst[inst].custom, prim, inst, kAny ? __fdiv_rn(u, det) : u,
                                  kAny ? __fdiv_rn(v, det) : v, ctx))
                    continue;
                best.t = t;
                best.u = u;
                best.v = v;
                best_det = det;
                best.inst = inst;
                best.prim = prim;
                best.bgeo = gw & 0x7FFFFFFFu;
                if (kAny) {
                    done = true;
                    break;
                }
            }
        }
        if (!done && cur == kEmpty) done = true;
        if (done) {
            if constexpr (kAny) {
                best.u = __fdiv_rn(best.u, best_det);
                best.v = __fdiv_rn(best.v, best_det);
            }
            if (s.has_tlas && !(kAny && best.inst != 0xFFFFFFFFu)) {
                // transformed instances: finish the ray with the two-level pass
                trace_tlas<kAny>(s, r, r.o, r.d, tmin, best, test_alpha, ctx, ts);
            }
            finish(q, best.inst != 0xFFFFFFFFu, best);
            has = false;
        }
    }
}

}  // namespace gbrt

namespace gbrt {

// Persistent-lane traversal of the 8-wide world BVH; same interface and
// refill policy as persistent_trace.
template <bool kAny, bool kTlas, bool kAlpha, class Loader, class Finisher>
GB_D void persistent_trace_cw(const DevScene& s, uint32_t n, uint32_t* work, uint32_t flags, TraceStats& ts,
                              Loader&& load, Finisher&& finish) {
    const uint32_t lane = threadIdx.x & 31u;
    const bool test_alpha = kAlpha && !(flags & GBRT_RAY_OPAQUE) && !s.all_opaque;
#if GBRT_CW_SMEM_STACK
    // the top kSmemStack entries of each lane's stack in shared memory ([entry][thread]: a warp's accesses
    // to one depth are consecutive 8-byte words), deeper ones in local memory; every traversal kernel
    // runs 128-thread blocks (its launch bound)
    constexpr int kSmemStack = GBRT_CW_SMEM_STACK;
    __shared__ uint2 s_stack[kSmemStack][128];
    uint2 stack[kCwStack - kSmemStack];
    auto push = [&](uint2 v, int i) {
        if (i < kSmemStack) s_stack[i][threadIdx.x] = v;
        else stack[i - kSmemStack] = v;
    };
    auto pop = [&](int i) { return i < kSmemStack ? s_stack[i][threadIdx.x] : stack[i - kSmemStack]; };
#else
    uint2 stack[kCwStack];
    auto push = [&](uint2 v, int i) { stack[i] = v; };
    auto pop = [&](int i) { return stack[i]; };
#endif
    bool has = false, exhausted = false;
    uint32_t q = 0, oct = 0;
    TRay r;
    Hit best;
    float best_det = 1.0f;  // any-hit queries: best.u, best.v hold V, W of the world hit until the ray is done
    AnyCtx ctx{0, 0, 0, 0};
    float tmin = 0.0f, tmax = 0.0f;
    uint2 ng = make_uint2(0, 0);
    int sp = 0;
    uint32_t iter = 0;
    for (;;) {
        if (!exhausted) {
            const uint32_t idle = __ballot_sync(0xFFFFFFFFu, !has);
            if (__popc(idle) >= (int)kRefill) {
                uint32_t base = 0;
                if (lane == 0) base = atomicAdd(work, (uint32_t)__popc(idle));
                base = __shfl_sync(0xFFFFFFFFu, base, 0);
                if (base + __popc(idle) >= n) exhausted = true;
                if (!has) {
                    q = base + __popc(idle & ((1u << lane) - 1u));
                    if (q < n) {
                        float3 o, d;
                        load(q, o, d, tmin, tmax, ctx);
                        best.t = tmax;
                        best.u = best.v = 0.0f;
                        best_det = 1.0f;
                        best.inst = best.prim = best.bgeo = 0xFFFFFFFFu;
                        iter = 0;
                        if (d.x == 0.0f && d.y == 0.0f && d.z == 0.0f) {
                            finish(q, false, best);
                        } else {
                            has = true;
                            setup_ray(r, o, d);
                            oct = (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u);
                            sp = 0;
                            // virtual parent: one inner child (the root, node 0) in slot 0
                            ng = s.has_world ? make_uint2(0u, (1u << (24u + oct)) | 1u) : make_uint2(0u, 0u);
                        }
                    }
                }
            }
        }
        if (!__any_sync(0xFFFFFFFFu, has)) {
            if (exhausted) break;
            continue;
        }
        if (!has) continue;
        bool done = false;
        while (!(ng.y & 0xFF000000u) && sp > 0) ng = pop(--sp);
        if (!(ng.y & 0xFF000000u)) {
            done = true;
        } else if (++iter > kMaxIter) {
            ts.status |= GBRT_STATUS_ITER_LIMIT;
            done = true;
        } else {
            const uint32_t bit = __ffs(ng.y & 0xFF000000u) - 1u;
            ng.y &= ~(1u << bit);
            const uint32_t slot = (bit - 24u) ^ oct;
            const uint32_t child = ng.x + __popc((ng.y & 0xFFu) & ((1u << slot) - 1u));
            if (ng.y & 0xFF000000u) {
                if (sp < kCwStack) push(ng, sp++);
                else ts.status |= GBRT_STATUS_STACK_OVERFLOW;
            }
            uint32_t cb, tb, im;
            const uint32_t hm = cw_intersect(s.cw_nodes, child, r, oct, tmin, best.t, cb, tb, im);
            ts.nodes++;
            ng = make_uint2(cb, (hm & 0xFF000000u) | im);
            uint32_t tri_bits = hm & 0x00FFFFFFu;
            while (tri_bits) {
                const uint32_t tbit = __ffs(tri_bits) - 1u;
                tri_bits &= tri_bits - 1u;
                const TriRec* tr = s.cw_tris + tb + tbit;
                const float4 pa = __ldg(&tr->a), pb = __ldg(&tr->b), pc = __ldg(&tr->c);
                ts.tris++;
                // any-hit queries keep V, W and det of the hit and divide once the ray is done (if
                // their caller reads u, v at all); closest-hit queries divide per accepted hit
                float t, u, v, det = 1.0f;
                if constexpr (kAny) {
                    if (!isect_tri_t(r, f3(pa), f3(pb), f3(pc), tmin, best.t, t, u, v, det)) continue;
                } else {
                    if (!isect_tri(r, f3(pa), f3(pb), f3(pc), tmin, best.t, t, u, v)) continue;
                }
                const uint32_t inst = __float_as_uint(pa.w);
                const uint32_t prim = __float_as_uint(pb.w);
                const uint32_t gw = __float_as_uint(pc.w);
                if (!closer(t, inst, prim, best)) continue;
                if (test_alpha && !(gw >> 31) &&
                    anyhit_ignore(s, s.inst[inst].custom, prim, inst, kAny ? __fdiv_rn(u, det) : u,
                                  kAny ? __fdiv_rn(v, det) : v, ctx))
                    continue;
                best.t = t;
                best.u = u;
                best.v = v;
                best_det = det;
                best.inst = inst;
                best.prim = prim;
                best.bgeo = gw & 0x7FFFFFFFu;
                if (kAny) {
                    done = true;
                    break;
                }
            }
        }
        if (done) {
            if constexpr (kAny) {
                best.u = __fdiv_rn(best.u, best_det);
                best.v = __fdiv_rn(best.v, best_det);
            }
            if constexpr (kTlas) {
                if (s.has_tlas && !(kAny && best.inst != 0xFFFFFFFFu))
                    trace_tlas<kAny, true>(s, r, r.o, r.d, tmin, best, test_alpha, ctx, ts);
            }
            finish(q, best.inst != 0xFFFFFFFFu, best);
            has = false;
        }
    }
}

// Traversal forms of a world query (chosen per launch by trace_mode):
//   kTraceBinary  binary world BVH, binary BLASes (scenes without 8-wide nodes)
//   kTraceWide    8-wide world BVH, no transformed instances
//   kTraceWideTlas 8-wide world BVH, then the TLAS with 8-wide BLASes
// Keeping the TLAS code out of the common form keeps its registers free.
// A form | kTraceOpaque is compiled without the any-hit alpha test, for
// launches where no geometry can need it (all-opaque scenes or frames); the
// code it leaves out cost the 8-wide traversal kernels spills.
constexpr int kTraceBinary = 0, kTraceWide = 1, kTraceWideTlas = 2, kTraceOpaque = 4;

template <bool kAny, int kMode, class Loader, class Finisher>
GB_D void world_trace(const DevScene& s, uint32_t n, uint32_t* work, uint32_t flags, TraceStats& ts, Loader&& load,
                      Finisher&& finish) {
    constexpr int kForm = kMode & 3;
    constexpr bool kAlpha = !(kMode & kTraceOpaque);
    if constexpr (kForm == kTraceBinary) persistent_trace<kAny, kAlpha>(s, n, work, flags, ts, load, finish);
    else persistent_trace_cw<kAny, kForm == kTraceWideTlas, kAlpha>(s, n, work, flags, ts, load, finish);
}

// The form a scene needs: binary when it has a world BVH without its
// 8-wide copy (after gbrt_scene_rebuild_noalloc) or when the autotuner chose
// it, else 8-wide, with the TLAS when it has transformed instances.
inline int trace_mode(const DevScene& s) {
    if (s.prefer_binary || (s.has_world && !s.cw_nodes)) return kTraceBinary;
    return s.has_tlas ? kTraceWideTlas : kTraceWide;
}

}  // namespace gbrt
