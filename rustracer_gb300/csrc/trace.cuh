// trace.cuh — software traceRayEXT for GB300 (no RT cores): BVH2
// traversal with a per-thread short stack, the watertight FP32 triangle test
// and the alpha-tested any-hit of RayTracing.rahit / RayTracing.shadow.rahit.
//
// Exactness contract with the CPU oracle: the triangle test and the ray
// transform into instance space use explicitly rounded operations in the same
// order as the oracle, so a ray returns the same (t, u, v, instance,
// primitive) whatever BVH was built.  Box tests only need to be conservative
// (Ize 2013 robust slab test).  Ties in t go to the smaller instance id, then
// the smaller primitive id.
#pragma once
#include <float.h>
#include "shade.cuh"


namespace gbrt {

constexpr int kStack = 64;
constexpr uint32_t kMaxIter = 1u << 22;  // per query; hitting it sets GBRT_STATUS_ITER_LIMIT

struct TRay {
    float3 o, d, inv;
    int kx, ky, kz;
    float Sx, Sy, Sz;
};

GB_D float sel3(float3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

// Woop, Benthin, Wald 2013: the axis of largest |d| becomes z (first maximum
// wins); x/y swap when d.z < 0 to keep the winding.
GB_D void setup_ray(TRay& r, float3 o, float3 d) {
    r.o = o;
    r.d = d;
    r.inv.x = d.x != 0.0f ? __fdiv_rn(1.0f, d.x) : copysignf(FLT_MAX, d.x);
    r.inv.y = d.y != 0.0f ? __fdiv_rn(1.0f, d.y) : copysignf(FLT_MAX, d.y);
    r.inv.z = d.z != 0.0f ? __fdiv_rn(1.0f, d.z) : copysignf(FLT_MAX, d.z);
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    r.kz = (ax >= ay && ax >= az) ? 0 : (ay >= az ? 1 : 2);
    r.kx = r.kz + 1 == 3 ? 0 : r.kz + 1;
    r.ky = r.kx + 1 == 3 ? 0 : r.kx + 1;
    float dz = sel3(d, r.kz);
    if (dz < 0.0f) { int t = r.kx; r.kx = r.ky; r.ky = t; }
    r.Sx = __fdiv_rn(sel3(d, r.kx), dz);
    r.Sy = __fdiv_rn(sel3(d, r.ky), dz);
    r.Sz = __fdiv_rn(1.0f, dz);
}

// Watertight ray-triangle test (FP32, IEEE round-to-nearest, no contraction
// except the six projections, which are explicit FMAs on both sides), up to
// the distance: on a hit in [tmin, tmax] it returns t and the unnormalised
// barycentrics V, W and their sum det with U; the barycentrics of the hit
// are u = V / det, v = W / det (isect_tri), which a traversal loop divides
// out only for the hit it keeps.
GB_D bool isect_tri_t(const TRay& r, float3 p0, float3 p1, float3 p2, float tmin, float tmax, float& t_out,
                      float& V_out, float& W_out, float& det_out) {
    float3 A = f3(sub_rn(p0.x, r.o.x), sub_rn(p0.y, r.o.y), sub_rn(p0.z, r.o.z));
    float3 B = f3(sub_rn(p1.x, r.o.x), sub_rn(p1.y, r.o.y), sub_rn(p1.z, r.o.z));
    float3 C = f3(sub_rn(p2.x, r.o.x), sub_rn(p2.y, r.o.y), sub_rn(p2.z, r.o.z));
    const float Akz = sel3(A, r.kz), Bkz = sel3(B, r.kz), Ckz = sel3(C, r.kz);
    const float Ax = __fmaf_rn(-r.Sx, Akz, sel3(A, r.kx));
    const float Ay = __fmaf_rn(-r.Sy, Akz, sel3(A, r.ky));
    const float Bx = __fmaf_rn(-r.Sx, Bkz, sel3(B, r.kx));
    const float By = __fmaf_rn(-r.Sy, Bkz, sel3(B, r.ky));
    const float Cx = __fmaf_rn(-r.Sx, Ckz, sel3(C, r.kx));
    const float Cy = __fmaf_rn(-r.Sy, Ckz, sel3(C, r.ky));
    float U = sub_rn(mul_rn(Cx, By), mul_rn(Cy, Bx));
    float V = sub_rn(mul_rn(Ax, Cy), mul_rn(Ay, Cx));
    float W = sub_rn(mul_rn(Bx, Ay), mul_rn(By, Ax));
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = __double2float_rn(__dsub_rn(__dmul_rn((double)Cx, (double)By), __dmul_rn((double)Cy, (double)Bx)));
        V = __double2float_rn(__dsub_rn(__dmul_rn((double)Ax, (double)Cy), __dmul_rn((double)Ay, (double)Cx)));
        W = __double2float_rn(__dsub_rn(__dmul_rn((double)Bx, (double)Ay), __dmul_rn((double)By, (double)Ax)));
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = add_rn(add_rn(U, V), W);
    if (det == 0.0f) return false;
    const float Az = mul_rn(r.Sz, Akz), Bz = mul_rn(r.Sz, Bkz), Cz = mul_rn(r.Sz, Ckz);
    const float T = add_rn(add_rn(mul_rn(U, Az), mul_rn(V, Bz)), mul_rn(W, Cz));
    const float t = __fdiv_rn(T, det);
    if (!(t >= tmin && t <= tmax)) return false;
    t_out = t;
    V_out = V;
    W_out = W;
    det_out = det;
    return true;
}
GB_D bool isect_tri(const TRay& r, float3 p0, float3 p1, float3 p2, float tmin, float tmax, float& t_out,
                    float& u_out, float& v_out) {
    float V, W, det;
    if (!isect_tri_t(r, p0, p1, p2, tmin, tmax, t_out, V, W, det)) return false;
    u_out = __fdiv_rn(V, det);
    v_out = __fdiv_rn(W, det);
    return true;
}

// Robust slab test against [lo, hi]; returns the entry distance in tn.
GB_D bool box_hit(const TRay& r, float lox, float hix, float loy, float hiy, float loz, float hiz, float tmin,
                  float tcur, float& tn) {
    const float up = 1.0000003576278687f;  // 1 + 2*gamma(3), gamma(n) = n*2^-24 / (1 - n*2^-24)
    float t0x = (lox - r.o.x) * r.inv.x, t1x = (hix - r.o.x) * r.inv.x;
    float t0y = (loy - r.o.y) * r.inv.y, t1y = (hiy - r.o.y) * r.inv.y;
    float t0z = (loz - r.o.z) * r.inv.z, t1z = (hiz - r.o.z) * r.inv.z;
    float n = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fmaxf(fminf(t0z, t1z), tmin));
    float f = fminf(fminf(fmaxf(t0x, t1x) * up, fmaxf(t0y, t1y) * up), fminf(fmaxf(t0z, t1z) * up, tcur));
    tn = n;
    return n <= f * up;
}

struct Hit {
    float t, u, v;
    uint32_t inst, prim, bgeo;
};

GB_D bool closer(float t, uint32_t inst, uint32_t prim, const Hit& b) {
    if (t < b.t) return true;
    if (t > b.t) return false;
    return inst < b.inst || (inst == b.inst && prim < b.prim);
}

// Identifies one any-hit draw (documented deviation D3).
struct AnyCtx {
    uint32_t px, py, sample, tag;
};

// testOpacityAnyHit, RayTracing.rahit:44-104 / RayTracing.shadow.rahit:44-104.
// Only the alpha channel decides, so only it is computed; every operation is
// rounded like the CPU oracle's.  Returns true when the hit is ignored.
GB_D bool anyhit_ignore(const DevScene& s, uint32_t custom, uint32_t prim, uint32_t inst, float u, float v,
                        const AnyCtx& c) {
    const gbrt_priminfo pi = s.prims[custom];
    const gbrt_material_raw& mat = s.mats[pi.material_id];
    const uint32_t alpha_mode = mat.alpha_mode;
    if (alpha_mode == 1u) return false;  // OPAQUE
    const uint32_t io = pi.i_offset + 3u * prim;
    const gbrt_vertex& v0 = s.vertices[pi.v_offset + s.indices[io]];
    const gbrt_vertex& v1 = s.vertices[pi.v_offset + s.indices[io + 1]];
    const gbrt_vertex& v2 = s.vertices[pi.v_offset + s.indices[io + 2]];
    const float b0 = sub_rn(sub_rn(1.0f, u), v);
    auto mixc = [&](float a, float b, float cc) { return add_rn(add_rn(mul_rn(a, b0), mul_rn(b, u)), mul_rn(cc, v)); };
    const float ca = mixc(v0.color[3], v1.color[3], v2.color[3]);
    auto uvset = [&](int coord) {
        if (coord == 0) return make_float2(mixc(v0.uv0[0], v1.uv0[0], v2.uv0[0]), mixc(v0.uv0[1], v1.uv0[1], v2.uv0[1]));
        if (coord == 1) return make_float2(mixc(v0.uv1[0], v1.uv1[0], v2.uv1[0]), mixc(v0.uv1[1], v1.uv1[1], v2.uv1[1]));
        return make_float2(0.0f, 0.0f);
    };
    float opacity;
    if (mat.workflow == 1u) {  // SPECULAR_GLOSS_WORKFLOW
        float da = mat.sg_diffuse_factor[3];
        if (mat.sg_diffuse_texture.index >= 0)
            da = mul_rn(da, texture(s, mat.sg_diffuse_texture.index, uvset(mat.sg_diffuse_texture.coord)).w);
        opacity = mul_rn(ca, da);
    } else {
        opacity = mul_rn(ca, mat.base_color[3]);
        if (mat.base_color_texture.index >= 0)
            opacity = mul_rn(opacity, texture(s, mat.base_color_texture.index, uvset(mat.base_color_texture.coord)).w);
    }
    if (alpha_mode == 2u) return opacity < mat.alpha_cutoff;  // MASK
    const float uu = u2f(pcg4d(make_uint4(c.px, c.py, c.sample, blend_hash(inst, prim, c.tag))).x);
    return opacity <= uu;  // BLEND
}

struct TraceStats {
    uint32_t nodes, tris, status;
};

// Traverses one BVH of the pool from `root` (inner node index or leaf code).
// inst_override >= 0: every triangle belongs to that instance (BLAS of a
// transformed instance).  Returns true when a terminate-on-first query found
// a hit.
template <bool kTerminateOnFirst>
GB_D bool traverse_bvh(const DevScene& s, int root, const TRay& r, float tmin, Hit& best, bool test_alpha,
                       const AnyCtx& ctx, TraceStats& st, int inst_override) {
    int stack[kStack];
    int sp = 0;
    int cur = root;
    uint32_t iter = 0;
    for (;;) {
        if (++iter > kMaxIter) {
            st.status |= GBRT_STATUS_ITER_LIMIT;
            return false;
        }
        if (cur >= 0) {
            const BNode2* n = s.nodes + cur;
            const float4 a = __ldg(&n->lxy), b = __ldg(&n->rxy), z = __ldg(&n->lrz);
            const int4 c = __ldg(&n->c);
            st.nodes++;
            float tn0, tn1;
            const bool h0 = box_hit(r, a.x, a.y, a.z, a.w, z.x, z.y, tmin, best.t, tn0);
            const bool h1 = box_hit(r, b.x, b.y, b.z, b.w, z.z, z.w, tmin, best.t, tn1);
            if (h0 && h1) {
                int nearc = c.x, farc = c.y;
                if (tn1 < tn0) { nearc = c.y; farc = c.x; }
                if (sp < kStack) stack[sp++] = farc;
                else st.status |= GBRT_STATUS_STACK_OVERFLOW;
                cur = nearc;
                continue;
            }
            if (h0) { cur = c.x; continue; }
            if (h1) { cur = c.y; continue; }
        } else {
            const uint32_t first = leaf_first(cur), count = leaf_count(cur);
            for (uint32_t i = 0; i < count; ++i) {
                const TriRec* tr = s.tris + first + i;
                const float4 pa = __ldg(&tr->a), pb = __ldg(&tr->b), pc = __ldg(&tr->c);
                st.tris++;
                float t, u, v;
                if (!isect_tri(r, f3(pa), f3(pb), f3(pc), tmin, best.t, t, u, v)) continue;
                const uint32_t inst = inst_override >= 0 ? (uint32_t)inst_override : __float_as_uint(pa.w);
                const uint32_t prim = __float_as_uint(pb.w);
                const uint32_t gw = __float_as_uint(pc.w);
                if (!closer(t, inst, prim, best)) continue;
                if (test_alpha && !(gw >> 31) &&
                    anyhit_ignore(s, s.inst[inst].custom, prim, inst, u, v, ctx))
                    continue;
                best.t = t;
                best.u = u;
                best.v = v;
                best.inst = inst;
                best.prim = prim;
                best.bgeo = gw & 0x7FFFFFFFu;
                if (kTerminateOnFirst) return true;
            }
        }
        if (sp == 0) return false;
        cur = stack[--sp];
    }
}

constexpr int kCwStack = 32;

// Byte k of an 8-byte group (lo word = bytes 0..3) as the float
// 1 + q * 2^-15, in one byte permute: result bytes (from low) = 0x00, q, 0x80,
// 0x3F, i.e. 0x3F80qq00.
GB_D float cw_q(uint32_t lo, uint32_t hi, int k) {
    const uint32_t w = k < 4 ? lo : hi;
    return __uint_as_float(__byte_perm(w, 0x3F800000u, 0x7604u | ((uint32_t)(k & 3) << 4)));
}

// Intersects the 8 children of wide node `node`: returns the hit mask (bits
// 24 + (slot ^ oct) for inner children, triangle bits 0..23 for leaves) and
// the node's child base, triangle base and inner-slot mask.
GB_D uint32_t cw_intersect(const CwNode* nodes, uint32_t node, const TRay& r, uint32_t oct, float tmin, float tmax,
                           uint32_t& child_base, uint32_t& tri_base, uint32_t& imask) {
    const uint4* np = reinterpret_cast<const uint4*>(nodes + node);
    const uint4 w0 = __ldg(np), w1 = __ldg(np + 1), w2 = __ldg(np + 2), w3 = __ldg(np + 3), w4 = __ldg(np + 4);
    child_base = w1.x;
    tri_base = w1.y;
    imask = w0.w >> 24;
    // per axis: t = o + q * s = fma(1 + q 2^-15, 2^15 s, o - 2^15 s).  An axis the
    // ray is parallel to (d = 0) gives (-inf, +inf) and the origin must lie
    // inside that child's slab instead.
    const float scx = __uint_as_float((w0.w & 0xFFu) << 23);
    const float scy = __uint_as_float(((w0.w >> 8) & 0xFFu) << 23);
    const float scz = __uint_as_float(((w0.w >> 16) & 0xFFu) << 23);
    const float px = __uint_as_float(w0.x), py = __uint_as_float(w0.y), pz = __uint_as_float(w0.z);
    const bool zx = r.d.x == 0.0f, zy = r.d.y == 0.0f, zz = r.d.z == 0.0f;
    const float Sx = zx ? 0.0f : 32768.0f * (scx * r.inv.x);
    const float Sy = zy ? 0.0f : 32768.0f * (scy * r.inv.y);
    const float Sz = zz ? 0.0f : 32768.0f * (scz * r.inv.z);
    const float Ox = (px - r.o.x) * r.inv.x - Sx, Oy = (py - r.o.y) * r.inv.y - Sy, Oz = (pz - r.o.z) * r.inv.z - Sz;
    const float Oxn = zx ? -INFINITY : Ox, Oxf = zx ? INFINITY : Ox;
    const float Oyn = zy ? -INFINITY : Oy, Oyf = zy ? INFINITY : Oy;
    const float Ozn = zz ? -INFINITY : Oz, Ozf = zz ? INFINITY : Oz;
    const bool parallel = zx || zy || zz;
    // near / far planes per axis by direction sign
    const bool nx = r.inv.x < 0.0f, ny = r.inv.y < 0.0f, nz = r.inv.z < 0.0f;
    const uint32_t lnx0 = nx ? w3.z : w2.x, lnx1 = nx ? w3.w : w2.y, lfx0 = nx ? w2.x : w3.z, lfx1 = nx ? w2.y : w3.w;
    const uint32_t lny0 = ny ? w4.x : w2.z, lny1 = ny ? w4.y : w2.w, lfy0 = ny ? w2.z : w4.x, lfy1 = ny ? w2.w : w4.y;
    const uint32_t lnz0 = nz ? w4.z : w3.x, lnz1 = nz ? w4.w : w3.y, lfz0 = nz ? w3.x : w4.z, lfz1 = nz ? w3.y : w4.w;
    uint32_t hits = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const uint32_t meta = ((k < 4 ? w1.z : w1.w) >> (8 * (k & 3))) & 0xFFu;
        const float tnx = fmaf(cw_q(lnx0, lnx1, k), Sx, Oxn), tfx = fmaf(cw_q(lfx0, lfx1, k), Sx, Oxf);
        const float tny = fmaf(cw_q(lny0, lny1, k), Sy, Oyn), tfy = fmaf(cw_q(lfy0, lfy1, k), Sy, Oyf);
        const float tnz = fmaf(cw_q(lnz0, lnz1, k), Sz, Ozn), tfz = fmaf(cw_q(lfz0, lfz1, k), Sz, Ozf);
        const float tn = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, tmin));
        const float tf = fminf(fminf(tfx, tfy), fminf(tfz, tmax));
        bool inside = true;
        if (parallel) {  // decoded slab of each parallel axis must contain the origin
            auto in = [&](bool z, uint32_t lo0, uint32_t lo1, uint32_t hi0, uint32_t hi1, float p, float sc, float o) {
                if (!z) return true;
                const float ql = (cw_q(lo0, lo1, k) - 1.0f) * 32768.0f, qh = (cw_q(hi0, hi1, k) - 1.0f) * 32768.0f;
                return o >= p + ql * sc && o <= p + qh * sc;
            };
            inside = in(zx, w2.x, w2.y, w3.z, w3.w, px, scx, r.o.x) && in(zy, w2.z, w2.w, w4.x, w4.y, py, scy, r.o.y) &&
                     in(zz, w3.x, w3.y, w4.z, w4.w, pz, scz, r.o.z);
        }
        // empty slots (meta 0) contribute no bit
        const uint32_t low = meta & 0x1Fu;
        const uint32_t bits = low >= 24u ? (1u << (24u + ((uint32_t)k ^ oct))) : ((meta >> 5) << low);
        hits |= (tn <= tf && inside) ? bits : 0u;
    }
    return hits;
}

// Stack traversal of one 8-wide BLAS (nodes / tris: its own arrays, root at
// node 0) for a ray already in object space; hits report instance `inst`.
// Returns true when kTerminateOnFirst and a hit was accepted.
//
// Out of line on purpose: inlined next to the world traversal's own 8-wide
// loop, the second copy of the node decode made the TLAS kernels 1.8x slower
// (32 instanced scenes: 232 vs 425 Mrays/s on GB300), while the call costs
// little -- it runs once per instance a ray reaches.
template <bool kTerminateOnFirst>
__device__ __noinline__ bool traverse_cw(const DevScene& s, const CwNode* nodes, const TriRec* tris, const TRay& r, float tmin,
                      Hit& best, bool test_alpha, const AnyCtx& ctx, TraceStats& ts, uint32_t inst) {
    const uint32_t oct = (r.d.x < 0.0f ? 1u : 0u) | (r.d.y < 0.0f ? 2u : 0u) | (r.d.z < 0.0f ? 4u : 0u);
    uint2 stack[kCwStack];
    int sp = 0;
    uint2 ng = make_uint2(0u, (1u << (24u + oct)) | 1u);  // virtual parent of the root
    uint32_t iter = 0;
    for (;;) {
        while (!(ng.y & 0xFF000000u) && sp > 0) ng = stack[--sp];
        if (!(ng.y & 0xFF000000u)) return false;
        if (++iter > kMaxIter) {
            ts.status |= GBRT_STATUS_ITER_LIMIT;
            return false;
        }
        const uint32_t bit = __ffs(ng.y & 0xFF000000u) - 1u;
        ng.y &= ~(1u << bit);
        const uint32_t slot = (bit - 24u) ^ oct;
        const uint32_t child = ng.x + __popc((ng.y & 0xFFu) & ((1u << slot) - 1u));
        if (ng.y & 0xFF000000u) {
            if (sp < kCwStack) stack[sp++] = ng;
            else ts.status |= GBRT_STATUS_STACK_OVERFLOW;
        }
        uint32_t cb, tb, im;
        const uint32_t hm = cw_intersect(nodes, child, r, oct, tmin, best.t, cb, tb, im);
        ts.nodes++;
        ng = make_uint2(cb, (hm & 0xFF000000u) | im);
        uint32_t tri_bits = hm & 0x00FFFFFFu;
        while (tri_bits) {
            const uint32_t tbit = __ffs(tri_bits) - 1u;
            tri_bits &= tri_bits - 1u;
            const TriRec* tr = tris + tb + tbit;
            const float4 pa = __ldg(&tr->a), pb = __ldg(&tr->b), pc = __ldg(&tr->c);
            ts.tris++;
            float t, u, v;
            if (!isect_tri(r, f3(pa), f3(pb), f3(pc), tmin, best.t, t, u, v)) continue;
            const uint32_t prim = __float_as_uint(pb.w);
            const uint32_t gw = __float_as_uint(pc.w);
            if (!closer(t, inst, prim, best)) continue;
            if (test_alpha && !(gw >> 31) && anyhit_ignore(s, s.inst[inst].custom, prim, inst, u, v, ctx)) continue;
            best.t = t;
            best.u = u;
            best.v = v;
            best.inst = inst;
            best.prim = prim;
            best.bgeo = gw & 0x7FFFFFFFu;
            if (kTerminateOnFirst) return true;
        }
    }
}

// The TLAS part of a query: transformed instances, each BLAS traversed in
// object space with the world-to-object transform applied unfused (like the
// oracle), updating `best`.  Returns true when a terminate-on-first query
// found a hit.  kCwBlas: the BLASes are traversed in their 8-wide form
// (built for every BLAS), else in the binary form.
template <bool kTerminateOnFirst, bool kCwBlas = false>
GB_D bool trace_tlas(const DevScene& s, const TRay& r, float3 o, float3 d, float tmin, Hit& best, bool test_alpha,
                     const AnyCtx& ctx, TraceStats& st) {
    {
        float tn;
        if (box_hit(r, s.tlas_lo.x, s.tlas_hi.x, s.tlas_lo.y, s.tlas_hi.y, s.tlas_lo.z, s.tlas_hi.z, tmin, best.t,
                    tn)) {
            // TLAS leaves are leaf codes over the instance-id array stored in
            // the .a.w lanes of TriRec slots (see the build).
            int stack[16];
            int sp = 0;
            int cur = s.tlas_root;
            for (;;) {
                if (cur >= 0) {
                    const BNode2* n = s.nodes + cur;
                    const float4 a = __ldg(&n->lxy), b = __ldg(&n->rxy), z = __ldg(&n->lrz);
                    const int4 c = __ldg(&n->c);
                    st.nodes++;
                    float tn0, tn1;
                    const bool h0 = box_hit(r, a.x, a.y, a.z, a.w, z.x, z.y, tmin, best.t, tn0);
                    const bool h1 = box_hit(r, b.x, b.y, b.z, b.w, z.z, z.w, tmin, best.t, tn1);
                    if (h0 && h1) {
                        if (sp < 16) stack[sp++] = c.y;
                        else st.status |= GBRT_STATUS_STACK_OVERFLOW;
                        cur = c.x;
                        continue;
                    }
                    if (h0) { cur = c.x; continue; }
                    if (h1) { cur = c.y; continue; }
                } else {
                    const uint32_t first = leaf_first(cur), count = leaf_count(cur);
                    for (uint32_t i = 0; i < count; ++i) {
                        const uint32_t ii = __float_as_uint(__ldg(&s.tris[first + i].a).w);
                        const DevInstance& in = s.inst[ii];
                        if ((in.mask & 0xFFu) == 0u || !in.has_blas) continue;
                        TRay orr;
                        setup_ray(orr, xform34_rn(in.inv, o, 1.0f), xform34_rn(in.inv, d, 0.0f));
                        if constexpr (kCwBlas) {
                            if (traverse_cw<kTerminateOnFirst>(s, s.blas_cw_nodes + in.cw_node0,
                                                               s.blas_cw_tris + in.cw_tri0, orr, tmin, best,
                                                               test_alpha, ctx, st, ii))
                                return true;
                        } else {
                            if (traverse_bvh<kTerminateOnFirst>(s, in.blas_root, orr, tmin, best, test_alpha, ctx,
                                                                st, (int)ii))
                                return true;
                        }
                    }
                }
                if (sp == 0) break;
                cur = stack[--sp];
            }
        }
    }
    return best.inst != 0xFFFFFFFFu;
}

// Full query: the merged world BVH, then the TLAS over transformed instances.
template <bool kTerminateOnFirst>
GB_D bool trace_scene(const DevScene& s, float3 o, float3 d, float tmin, float tmax, uint32_t flags,
                      const AnyCtx& ctx, Hit& best, TraceStats& st) {
    best.t = tmax;
    best.u = best.v = 0.0f;
    best.inst = best.prim = best.bgeo = 0xFFFFFFFFu;
    if (d.x == 0.0f && d.y == 0.0f && d.z == 0.0f) return false;
    const bool test_alpha = !(flags & GBRT_RAY_OPAQUE) && !s.all_opaque;
    TRay r;
    setup_ray(r, o, d);
    if (s.has_world) {
        float tn;
        if (box_hit(r, s.world_lo.x, s.world_hi.x, s.world_lo.y, s.world_hi.y, s.world_lo.z, s.world_hi.z, tmin,
                    best.t, tn)) {
            if (traverse_bvh<kTerminateOnFirst>(s, s.world_root, r, tmin, best, test_alpha, ctx, st, -1))
                return true;
        }
    }
    if (s.has_tlas) trace_tlas<kTerminateOnFirst>(s, r, o, d, tmin, best, test_alpha, ctx, st);
    return best.inst != 0xFFFFFFFFu;
}

}  // namespace gbrt
