// bvh_build.cu — GPU BVH construction.
//
// 30-bit Morton codes of the item centroids and a CUB radix sort, then a
// binary tree: by default parallel locally-ordered clustering
// (ploc_build.inc), or, for fast rebuilds, the linear BVH of Karras 2012
// ("Maximizing Parallelism in the Construction of BVHs, Octrees, and k-d
// Trees": one thread per inner node finds its key range and split); then one
// bottom-up pass (atomic arrival counters) that computes the boxes
// and the SAH cost of every subtree and collapses subtrees of at most
// kMaxLeaf items into leaves when that lowers the SAH cost.  The result is
// written in the traversal layout (BNode2 with both child boxes; leaves as
// codes over a contiguous range of TriRec slots in Morton order).
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>
#include <cstring>
#include <utility>
#include <float.h>
#include "kernels.h"

namespace gbrt {

namespace {

#ifndef GBRT_SAH_TRAVERSE
#define GBRT_SAH_TRAVERSE 1.2f
#endif
constexpr float kCostTraverse = GBRT_SAH_TRAVERSE;  // SAH cost of an inner node relative to one triangle test
constexpr float kCostTri = 1.0f;

__device__ __forceinline__ uint32_t expand_bits(uint32_t v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

// float <-> order-preserving uint for atomic min/max of bounds
__device__ __forceinline__ uint32_t f2o(float f) {
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float o2f(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

struct Scratch {
    float4* lo;           // [n] item boxes
    float4* hi;
    uint32_t* morton_in;  // [n]
    uint32_t* morton;     // [n] sorted
    uint32_t* idx_in;     // [n]
    uint32_t* idx;        // [n] sorted item index
    int32_t* left;        // [n-1] inner children: >= 0 inner, < 0 ~leaf(sorted position)
    int32_t* right;
    int32_t* parent_i;    // [n-1] parent of inner node (-1 root)
    int32_t* parent_l;    // [n] parent of leaf
    uint32_t* range_lo;   // [n-1]
    uint32_t* range_hi;
    float4* ilo;          // [n-1] inner boxes
    float4* ihi;
    float* cost;          // [n-1] SAH cost (area-weighted)
    uint32_t* collapse;   // [n-1] 1 = becomes a leaf
    uint32_t* arrive;     // [n-1]
    uint32_t* cbounds;    // 6 order-encoded centroid bounds
    void* cub_tmp;
    size_t cub_bytes;
};

// Item i's triangle (world space when `inst` is given and the item's
// instance is a flattened transformed one), its box and TriRec.
__global__ void tri_boxes_kernel(const gbrt_vertex* V, const uint32_t* I, const gbrt_priminfo* P, const uint4* items,
                                 uint32_t n, float4* lo, float4* hi, TriRec* unsorted, uint32_t* cb,
                                 const DevInstance* inst) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float3 c = f3(0.0f);
    bool ok = i < n;
    if (ok) {
        const uint4 it = items[i];
        const gbrt_priminfo pi = P[it.y];
        const uint32_t io = pi.i_offset + 3u * it.z;
        const float* a = V[pi.v_offset + I[io]].pos;
        const float* b = V[pi.v_offset + I[io + 1]].pos;
        const float* d = V[pi.v_offset + I[io + 2]].pos;
        float3 p0 = f3(a[0], a[1], a[2]), p1 = f3(b[0], b[1], b[2]), p2 = f3(d[0], d[1], d[2]);
        if (inst && !inst[it.x].identity) {
            const float* xf = inst[it.x].xf;
            p0 = xform34_rn(xf, p0, 1.0f);
            p1 = xform34_rn(xf, p1, 1.0f);
            p2 = xform34_rn(xf, p2, 1.0f);
        }
        const float3 l = fmin3(fmin3(p0, p1), p2), h = fmax3(fmax3(p0, p1), p2);
        lo[i] = f4(l, 0.0f);
        hi[i] = f4(h, 0.0f);
        TriRec r;
        r.a = f4(p0, __uint_as_float(it.x));
        r.b = f4(p1, __uint_as_float(it.z));
        r.c = f4(p2, __uint_as_float(it.y | (it.w ? 0x80000000u : 0u)));
        unsorted[i] = r;
        c = (l + h) * 0.5f;
    }
    // centroid bounds: warp reduce then atomics
    float mnx = ok ? c.x : FLT_MAX, mny = ok ? c.y : FLT_MAX, mnz = ok ? c.z : FLT_MAX;
    float mxx = ok ? c.x : -FLT_MAX, mxy = ok ? c.y : -FLT_MAX, mxz = ok ? c.z : -FLT_MAX;
    for (int o = 16; o > 0; o >>= 1) {
        mnx = fminf(mnx, __shfl_down_sync(0xFFFFFFFFu, mnx, o));
        mny = fminf(mny, __shfl_down_sync(0xFFFFFFFFu, mny, o));
        mnz = fminf(mnz, __shfl_down_sync(0xFFFFFFFFu, mnz, o));
        mxx = fmaxf(mxx, __shfl_down_sync(0xFFFFFFFFu, mxx, o));
        mxy = fmaxf(mxy, __shfl_down_sync(0xFFFFFFFFu, mxy, o));
        mxz = fmaxf(mxz, __shfl_down_sync(0xFFFFFFFFu, mxz, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(cb + 0, f2o(mnx));
        atomicMin(cb + 1, f2o(mny));
        atomicMin(cb + 2, f2o(mnz));
        atomicMax(cb + 3, f2o(mxx));
        atomicMax(cb + 4, f2o(mxy));
        atomicMax(cb + 5, f2o(mxz));
    }
}

__global__ void box_centroid_bounds_kernel(const float4* lo, const float4* hi, uint32_t n, uint32_t* cb) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool ok = i < n;
    float3 c = ok ? (f3(lo[i]) + f3(hi[i])) * 0.5f : f3(0.0f);
    float mnx = ok ? c.x : FLT_MAX, mny = ok ? c.y : FLT_MAX, mnz = ok ? c.z : FLT_MAX;
    float mxx = ok ? c.x : -FLT_MAX, mxy = ok ? c.y : -FLT_MAX, mxz = ok ? c.z : -FLT_MAX;
    for (int o = 16; o > 0; o >>= 1) {
        mnx = fminf(mnx, __shfl_down_sync(0xFFFFFFFFu, mnx, o));
        mny = fminf(mny, __shfl_down_sync(0xFFFFFFFFu, mny, o));
        mnz = fminf(mnz, __shfl_down_sync(0xFFFFFFFFu, mnz, o));
        mxx = fmaxf(mxx, __shfl_down_sync(0xFFFFFFFFu, mxx, o));
        mxy = fmaxf(mxy, __shfl_down_sync(0xFFFFFFFFu, mxy, o));
        mxz = fmaxf(mxz, __shfl_down_sync(0xFFFFFFFFu, mxz, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(cb + 0, f2o(mnx));
        atomicMin(cb + 1, f2o(mny));
        atomicMin(cb + 2, f2o(mnz));
        atomicMax(cb + 3, f2o(mxx));
        atomicMax(cb + 4, f2o(mxy));
        atomicMax(cb + 5, f2o(mxz));
    }
}

__global__ void morton_kernel(const float4* lo, const float4* hi, uint32_t n, const uint32_t* cb, uint32_t* codes,
                              uint32_t* idx) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float3 mn = f3(o2f(cb[0]), o2f(cb[1]), o2f(cb[2]));
    const float3 mx = f3(o2f(cb[3]), o2f(cb[4]), o2f(cb[5]));
    const float3 ext = mx - mn;
    const float3 c = (f3(lo[i]) + f3(hi[i])) * 0.5f;
    auto q = [](float v, float m, float e) {
        float t = e > 0.0f ? (v - m) / e : 0.5f;
        return (uint32_t)fminf(fmaxf(t * 1024.0f, 0.0f), 1023.0f);
    };
    const uint32_t x = q(c.x, mn.x, ext.x), y = q(c.y, mn.y, ext.y), z = q(c.z, mn.z, ext.z);
    codes[i] = (expand_bits(x) << 2) | (expand_bits(y) << 1) | expand_bits(z);
    idx[i] = i;
}

__device__ __forceinline__ int delta(const uint32_t* k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    const uint32_t a = k[i], b = k[j];
    if (a == b) return 32 + __clz((uint32_t)i ^ (uint32_t)j);
    return __clz(a ^ b);
}

// Karras 2012, Figure 4: one thread per inner node.
__global__ void karras_kernel(const uint32_t* k, int n, int32_t* left, int32_t* right, int32_t* parent_i,
                              int32_t* parent_l, uint32_t* rlo, uint32_t* rhi) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int d = (delta(k, n, i, i + 1) - delta(k, n, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = delta(k, n, i, i - d);
    int lmax = 2;
    while (delta(k, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (delta(k, n, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = delta(k, n, i, j);
    int s = 0;
    int t = l;
    do {
        t = (t + 1) >> 1;
        if (delta(k, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    const int gamma = i + s * d + min(d, 0);
    const int lo = min(i, j), hi = max(i, j);
    int32_t lc, rc;
    if (lo == gamma) { lc = ~gamma; parent_l[gamma] = i; } else { lc = gamma; parent_i[gamma] = i; }
    if (hi == gamma + 1) { rc = ~(gamma + 1); parent_l[gamma + 1] = i; } else { rc = gamma + 1; parent_i[gamma + 1] = i; }
    left[i] = lc;
    right[i] = rc;
    rlo[i] = (uint32_t)lo;
    rhi[i] = (uint32_t)hi;
    if (i == 0) parent_i[0] = -1;
}

__device__ __forceinline__ float half_area(float3 l, float3 h) {
    const float3 e = fmax3(h - l, f3(0.0f));
    return e.x * e.y + e.y * e.z + e.z * e.x;
}

// Bottom-up: one thread per leaf climbs while it is the second child to
// arrive at a node.  Child data is read with L1-bypassing loads.
__global__ void bottom_up_kernel(int n, const uint32_t* idx, const float4* lo, const float4* hi,
                                 const int32_t* left, const int32_t* right, const int32_t* parent_i,
                                 const int32_t* parent_l, const uint32_t* rlo, const uint32_t* rhi, float4* ilo,
                                 float4* ihi, float* cost, uint32_t* collapse, uint32_t* arrive, uint32_t max_leaf,
                                 float cost_traverse) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int p = parent_l[i];
    while (p >= 0) {
        __threadfence();
        if (atomicAdd(&arrive[p], 1u) == 0u) return;  // the sibling will finish p
        __threadfence();
        float3 bl[2], bh[2];
        float c[2];
        const int32_t ch[2] = {__ldcg(&left[p]), __ldcg(&right[p])};
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            if (ch[k] < 0) {
                const uint32_t item = __ldcg(&idx[~ch[k]]);
                bl[k] = f3(__ldcg(&lo[item]));
                bh[k] = f3(__ldcg(&hi[item]));
                c[k] = kCostTri * half_area(bl[k], bh[k]);
            } else {
                bl[k] = f3(__ldcg(&ilo[ch[k]]));
                bh[k] = f3(__ldcg(&ihi[ch[k]]));
                c[k] = __ldcg(&cost[ch[k]]);
            }
        }
        const float3 l = fmin3(bl[0], bl[1]), h = fmax3(bh[0], bh[1]);
        const float a = half_area(l, h);
        const uint32_t count = rhi[p] - rlo[p] + 1u;
        const float split = cost_traverse * a + c[0] + c[1];
        const float as_leaf = kCostTri * a * (float)count;
        const bool col = count <= max_leaf && as_leaf <= split;
        ilo[p] = f4(l, 0.0f);
        ihi[p] = f4(h, 0.0f);
        cost[p] = col ? as_leaf : split;
        collapse[p] = col ? 1u : 0u;
        p = parent_i[p];
    }
}

// Writes the traversal nodes.  Inner node p of the radix tree becomes pool
// node node_base + p; a child that is a radix-tree leaf or a collapsed inner
// node becomes a leaf code over its contiguous sorted range.
__global__ void emit_nodes_kernel(int n, const uint32_t* idx, const float4* lo, const float4* hi,
                                  const int32_t* left, const int32_t* right, const uint32_t* rlo,
                                  const uint32_t* rhi, const float4* ilo, const float4* ihi,
                                  const uint32_t* collapse, BNode2* nodes, uint32_t node_base, uint32_t tri_base) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n - 1) return;
    float3 bl[2], bh[2];
    int code[2];
    const int32_t ch[2] = {left[p], right[p]};
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        if (ch[k] < 0) {
            const uint32_t item = idx[~ch[k]];
            bl[k] = f3(lo[item]);
            bh[k] = f3(hi[item]);
            code[k] = leaf_code(tri_base + (uint32_t)~ch[k], 1u);
        } else {
            bl[k] = f3(ilo[ch[k]]);
            bh[k] = f3(ihi[ch[k]]);
            code[k] = collapse[ch[k]] ? leaf_code(tri_base + rlo[ch[k]], rhi[ch[k]] - rlo[ch[k]] + 1u)
                                      : (int)(node_base + ch[k]);
        }
    }
    BNode2 o;
    o.lxy = f4(bl[0].x, bh[0].x, bl[0].y, bh[0].y);
    o.rxy = f4(bl[1].x, bh[1].x, bl[1].y, bh[1].y);
    o.lrz = f4(bl[0].z, bh[0].z, bl[1].z, bh[1].z);
    o.c = make_int4(code[0], code[1], 0, 0);
    nodes[node_base + p] = o;
}

__global__ void gather_tris_kernel(const uint32_t* idx, uint32_t n, const TriRec* unsorted, TriRec* tris,
                                   uint32_t tri_base) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) tris[tri_base + i] = unsorted[idx[i]];
}

__global__ void gather_inst_kernel(const uint32_t* idx, uint32_t n, const uint32_t* ids, TriRec* tris,
                                   uint32_t tri_base) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        TriRec r;
        r.a = f4(0.0f, 0.0f, 0.0f, __uint_as_float(ids[idx[i]]));
        r.b = f4(0.0f, 0.0f, 0.0f, 0.0f);
        r.c = f4(0.0f, 0.0f, 0.0f, 0.0f);
        tris[tri_base + i] = r;
    }
}

__global__ void init_bounds_kernel(uint32_t* cb) {
    if (threadIdx.x < 3) cb[threadIdx.x] = 0xFFFFFFFFu;
    else if (threadIdx.x < 6) cb[threadIdx.x] = 0u;
}

#define CK(x)                                   \
    do {                                        \
        cudaError_t e_ = (x);                   \
        if (e_ != cudaSuccess) return e_;       \
    } while (0)

inline uint32_t blocks(uint32_t n, uint32_t b = 256) { return (n + b - 1) / b; }

// Allocates the scratch of one build (stream-ordered).
cudaError_t scratch_alloc(Scratch& s, uint32_t n, cudaStream_t st) {
    std::memset(&s, 0, sizeof(s));
    const size_t m = n > 1 ? n - 1 : 1;
    CK(cudaMallocAsync((void**)&s.lo, n * sizeof(float4), st));
    CK(cudaMallocAsync((void**)&s.hi, n * sizeof(float4), st));
    CK(cudaMallocAsync((void**)&s.morton_in, n * sizeof(uint32_t), st));
    CK(cudaMallocAsync((void**)&s.morton, n * sizeof(uint32_t), st));
    CK(cudaMallocAsync((void**)&s.idx_in, n * sizeof(uint32_t), st));
    CK(cudaMallocAsync((void**)&s.idx, n * sizeof(uint32_t), st));
    CK(cudaMallocAsync((void**)&s.left, m * sizeof(int32_t), st));
    CK(cudaMallocAsync((void**)&s.right, m * sizeof(int32_t), st));
    CK(cudaMallocAsync((void**)&s.parent_i, m * sizeof(int32_t), st));
    CK(cudaMallocAsync((void**)&s.parent_l, n * sizeof(int32_t), st));
    CK(cudaMallocAsync((void**)&s.range_lo, m * sizeof(uint32_t), st));
    CK(cudaMallocAsync((void**)&s.range_hi, m * sizeof(uint32_t), st));
    CK(cudaMallocAsync((void**)&s.ilo, m * sizeof(float4), st));
    CK(cudaMallocAsync((void**)&s.ihi, m * sizeof(float4), st));
    CK(cudaMallocAsync((void**)&s.cost, m * sizeof(float), st));
    CK(cudaMallocAsync((void**)&s.collapse, m * sizeof(uint32_t), st));
    CK(cudaMallocAsync((void**)&s.arrive, m * sizeof(uint32_t), st));
    CK(cudaMallocAsync((void**)&s.cbounds, 8 * sizeof(uint32_t), st));
    CK(cub::DeviceRadixSort::SortPairs(nullptr, s.cub_bytes, s.morton_in, s.morton, s.idx_in, s.idx, (int)n, 0, 30,
                                       st));
    CK(cudaMallocAsync(&s.cub_tmp, s.cub_bytes ? s.cub_bytes : 16, st));
    return cudaSuccess;
}

void scratch_free(Scratch& s, cudaStream_t st) {
    void* ptrs[] = {s.lo, s.hi, s.morton_in, s.morton, s.idx_in, s.idx, s.left, s.right, s.parent_i,
                    s.parent_l, s.range_lo, s.range_hi, s.ilo, s.ihi, s.cost, s.collapse, s.arrive, s.cbounds,
                    s.cub_tmp};
    for (void* p : ptrs)
        if (p) cudaFreeAsync(p, st);
}

}  // namespace

#include "ploc_build.inc"

namespace {

// Morton codes, sort, binary tree (PLOC clustering, or the Karras radix tree
// when quality is kBvhFast) and the bottom-up pass (boxes, SAH costs, leaf
// collapse with at most max_leaf items, an inner node costing cost_traverse
// triangle tests per unit of area).  Item boxes in s.lo/hi and centroid
// bounds in s.cbounds must be ready.
cudaError_t radix_tree(Scratch& s, uint32_t n, uint32_t max_leaf, cudaStream_t st, int quality,
                       float cost_traverse = kCostTraverse) {
    morton_kernel<<<blocks(n), 256, 0, st>>>(s.lo, s.hi, n, s.cbounds, s.morton_in, s.idx_in);
    CK(cudaGetLastError());
    CK(cub::DeviceRadixSort::SortPairs(s.cub_tmp, s.cub_bytes, s.morton_in, s.morton, s.idx_in, s.idx, (int)n, 0,
                                       30, st));
    if (n > 1) {
        cudaError_t pe = quality == kBvhPloc ? ploc_tree(s, n, st) : cudaErrorNotReady;
        if (pe != cudaSuccess && pe != cudaErrorNotReady) return pe;
        if (pe == cudaErrorNotReady) {  // radix tree (asked for, or clustering did not converge)
            karras_kernel<<<blocks(n - 1), 256, 0, st>>>(s.morton, (int)n, s.left, s.right, s.parent_i, s.parent_l,
                                                        s.range_lo, s.range_hi);
            CK(cudaGetLastError());
        }
        CK(cudaMemsetAsync(s.arrive, 0, (n - 1) * sizeof(uint32_t), st));
        bottom_up_kernel<<<blocks(n), 256, 0, st>>>((int)n, s.idx, s.lo, s.hi, s.left, s.right, s.parent_i,
                                                   s.parent_l, s.range_lo, s.range_hi, s.ilo, s.ihi, s.cost,
                                                   s.collapse, s.arrive, max_leaf, cost_traverse);
        CK(cudaGetLastError());
    }
    return cudaSuccess;
}

// Common tail: radix tree with leaves of up to kMaxLeaf items, emit BNode2.
cudaError_t build_common(Scratch& s, uint32_t n, BNode2* nodes, uint32_t node_base, uint32_t tri_base,
                         BvhResult* res, cudaStream_t st, int quality) {
    CK(radix_tree(s, n, kMaxLeaf, st, quality));
    if (n > 1) {
        emit_nodes_kernel<<<blocks(n - 1), 256, 0, st>>>((int)n, s.idx, s.lo, s.hi, s.left, s.right, s.range_lo,
                                                        s.range_hi, s.ilo, s.ihi, s.collapse, nodes, node_base,
                                                        tri_base);
        CK(cudaGetLastError());
    }
    // root: inner node 0 (or a leaf if it collapsed / n == 1)
    float4 rl, rh;
    uint32_t col = 0;
    if (n > 1) {
        CK(cudaMemcpyAsync(&rl, s.ilo, sizeof(float4), cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(&rh, s.ihi, sizeof(float4), cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(&col, s.collapse, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    } else {
        CK(cudaMemcpyAsync(&rl, s.lo, sizeof(float4), cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(&rh, s.hi, sizeof(float4), cudaMemcpyDeviceToHost, st));
    }
    CK(cudaStreamSynchronize(st));
    res->lo = rl;
    res->hi = rh;
    if (n == 1) res->root = leaf_code(tri_base, 1u);
    else if (col) res->root = leaf_code(tri_base, n);
    else res->root = (int32_t)node_base;
    return cudaSuccess;
}

}  // namespace

cudaError_t build_triangle_bvh(const gbrt_vertex* vertices, const uint32_t* indices, const gbrt_priminfo* prims,
                               const uint4* items, uint32_t n, BNode2* nodes, uint32_t node_base, TriRec* tris,
                               uint32_t tri_base, BvhResult* res, cudaStream_t st, const DevInstance* inst,
                               int quality) {
    if (n == 0) return cudaErrorInvalidValue;
    Scratch s;
    cudaError_t e = scratch_alloc(s, n, st);
    TriRec* unsorted = nullptr;
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&unsorted, n * sizeof(TriRec), st);
    if (e == cudaSuccess) {
        init_bounds_kernel<<<1, 32, 0, st>>>(s.cbounds);
        tri_boxes_kernel<<<blocks(n), 256, 0, st>>>(vertices, indices, prims, items, n, s.lo, s.hi, unsorted,
                                                    s.cbounds, inst);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = build_common(s, n, nodes, node_base, tri_base, res, st, quality);
    if (e == cudaSuccess) {
        gather_tris_kernel<<<blocks(n), 256, 0, st>>>(s.idx, n, unsorted, tris, tri_base);
        e = cudaGetLastError();
    }
    if (unsorted) cudaFreeAsync(unsorted, st);
    scratch_free(s, st);
    return e;
}

cudaError_t build_instance_bvh(const float4* lo, const float4* hi, const uint32_t* ids, uint32_t n, BNode2* nodes,
                               uint32_t node_base, TriRec* tris, uint32_t tri_base, BvhResult* res,
                               cudaStream_t st, int quality) {
    if (n == 0) return cudaErrorInvalidValue;
    Scratch s;
    cudaError_t e = scratch_alloc(s, n, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s.lo, lo, n * sizeof(float4), cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s.hi, hi, n * sizeof(float4), cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) {
        init_bounds_kernel<<<1, 32, 0, st>>>(s.cbounds);
        box_centroid_bounds_kernel<<<blocks(n), 256, 0, st>>>(s.lo, s.hi, n, s.cbounds);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = build_common(s, n, nodes, node_base, tri_base, res, st, quality);
    if (e == cudaSuccess) {
        gather_inst_kernel<<<blocks(n), 256, 0, st>>>(s.idx, n, ids, tris, tri_base);
        e = cudaGetLastError();
    }
    scratch_free(s, st);
    return e;
}

size_t bvh_sort_temp_bytes(uint32_t n) {
    size_t bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, bytes, (const uint32_t*)nullptr, (uint32_t*)nullptr,
                                    (const uint32_t*)nullptr, (uint32_t*)nullptr, (int)n, 0, 30);
    return bytes;
}

namespace {
inline size_t al256(size_t x) { return (x + 255) & ~size_t(255); }
}  // namespace

size_t bvh_scratch_bytes(uint32_t cap) {
    const size_t n = cap, m = cap > 1 ? cap - 1 : 1;
    return 4 * al256(n * sizeof(float4)) + 4 * al256(n * sizeof(uint32_t)) + 2 * al256(m * sizeof(uint32_t)) +
           2 * al256(m * sizeof(uint32_t)) + al256(32) + 4 * al256(n * sizeof(int32_t)) +
           al256(m * sizeof(float)) + al256(n * sizeof(TriRec)) + al256(bvh_sort_temp_bytes(cap));
}

BuildScratch bvh_scratch_carve(void* base, uint32_t cap) {
    const size_t n = cap, m = cap > 1 ? cap - 1 : 1;
    char* p = static_cast<char*>(base);
    auto take = [&](size_t bytes) {
        void* r = p;
        p += al256(bytes);
        return r;
    };
    BuildScratch s;
    s.capacity = cap;
    s.lo = (float4*)take(n * sizeof(float4));
    s.hi = (float4*)take(n * sizeof(float4));
    s.ilo = (float4*)take(n * sizeof(float4));
    s.ihi = (float4*)take(n * sizeof(float4));
    s.morton_in = (uint32_t*)take(n * sizeof(uint32_t));
    s.morton = (uint32_t*)take(n * sizeof(uint32_t));
    s.idx_in = (uint32_t*)take(n * sizeof(uint32_t));
    s.idx = (uint32_t*)take(n * sizeof(uint32_t));
    s.range_lo = (uint32_t*)take(m * sizeof(uint32_t));
    s.range_hi = (uint32_t*)take(m * sizeof(uint32_t));
    s.collapse = (uint32_t*)take(m * sizeof(uint32_t));
    s.arrive = (uint32_t*)take(m * sizeof(uint32_t));
    s.cbounds = (uint32_t*)take(32);
    s.left = (int32_t*)take(n * sizeof(int32_t));
    s.right = (int32_t*)take(n * sizeof(int32_t));
    s.parent_i = (int32_t*)take(n * sizeof(int32_t));
    s.parent_l = (int32_t*)take(n * sizeof(int32_t));
    s.cost = (float*)take(m * sizeof(float));
    s.unsorted = (TriRec*)take(n * sizeof(TriRec));
    s.sort_tmp_bytes = bvh_sort_temp_bytes(cap);
    s.sort_tmp = take(s.sort_tmp_bytes);
    return s;
}

cudaError_t build_triangle_bvh_scratch(const BuildScratch& bs, const gbrt_vertex* vertices, const uint32_t* indices,
                                       const gbrt_priminfo* prims, const uint4* items, uint32_t n, BNode2* nodes,
                                       uint32_t node_base, TriRec* tris, uint32_t tri_base, BvhResult* res,
                                       cudaStream_t st) {
    if (n == 0 || n > bs.capacity) return cudaErrorInvalidValue;
    Scratch s;
    std::memset(&s, 0, sizeof(s));
    s.lo = bs.lo;
    s.hi = bs.hi;
    s.morton_in = bs.morton_in;
    s.morton = bs.morton;
    s.idx_in = bs.idx_in;
    s.idx = bs.idx;
    s.left = bs.left;
    s.right = bs.right;
    s.parent_i = bs.parent_i;
    s.parent_l = bs.parent_l;
    s.range_lo = bs.range_lo;
    s.range_hi = bs.range_hi;
    s.ilo = bs.ilo;
    s.ihi = bs.ihi;
    s.cost = bs.cost;
    s.collapse = bs.collapse;
    s.arrive = bs.arrive;
    s.cbounds = bs.cbounds;
    s.cub_tmp = bs.sort_tmp;
    s.cub_bytes = bvh_sort_temp_bytes(n);  // the sort of n items needs no more than the capacity's size
    if (s.cub_bytes > bs.sort_tmp_bytes) return cudaErrorInvalidValue;
    init_bounds_kernel<<<1, 32, 0, st>>>(s.cbounds);
    tri_boxes_kernel<<<blocks(n), 256, 0, st>>>(vertices, indices, prims, items, n, s.lo, s.hi, bs.unsorted,
                                                s.cbounds, nullptr);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = build_common(s, n, nodes, node_base, tri_base, res, st, kBvhFast);  // no allocation
    if (e == cudaSuccess) {
        gather_tris_kernel<<<blocks(n), 256, 0, st>>>(s.idx, n, bs.unsorted, tris, tri_base);
        e = cudaGetLastError();
    }
    return e;
}

// World box of a transformed instance: the 8 transformed corners of its BLAS
// root box, widened by a relative 1e-6 of the box size plus 1e-6 of the
// largest coordinate so float rounding of the transform cannot make it
// smaller than the exact image.
__global__ void inst_boxes_kernel(const DevInstance* inst, const uint32_t* ids, const float4* blo,
                                  const float4* bhi, uint32_t n, float4* lo, float4* hi) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const DevInstance& in = inst[ids[i]];
    const float4 l = blo[i], h = bhi[i];
    float3 mn = f3(FLT_MAX), mx = f3(-FLT_MAX);
    for (int c = 0; c < 8; ++c) {
        const float3 p = f3((c & 1) ? h.x : l.x, (c & 2) ? h.y : l.y, (c & 4) ? h.z : l.z);
        const float3 q = f3(in.xf[0] * p.x + in.xf[1] * p.y + in.xf[2] * p.z + in.xf[3],
                            in.xf[4] * p.x + in.xf[5] * p.y + in.xf[6] * p.z + in.xf[7],
                            in.xf[8] * p.x + in.xf[9] * p.y + in.xf[10] * p.z + in.xf[11]);
        mn = fmin3(mn, q);
        mx = fmax3(mx, q);
    }
    const float3 ext = mx - mn;
    const float m = fmaxf(fmaxf(fmaxf(fabsf(mn.x), fabsf(mn.y)), fmaxf(fabsf(mn.z), fabsf(mx.x))),
                          fmaxf(fabsf(mx.y), fabsf(mx.z)));
    const float pad = 1e-6f * (fmaxf(fmaxf(ext.x, ext.y), ext.z) + m) + 1e-30f;
    lo[i] = f4(mn - pad, 0.0f);
    hi[i] = f4(mx + pad, 0.0f);
}

cudaError_t instance_world_boxes(const DevInstance* inst, const uint32_t* ids, const float4* blas_lo,
                                 const float4* blas_hi, uint32_t n, float4* lo, float4* hi, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    inst_boxes_kernel<<<blocks(n), 256, 0, st>>>(inst, ids, blas_lo, blas_hi, n, lo, hi);
    return cudaGetLastError();
}

}  // namespace gbrt

namespace gbrt {
#include "cwbvh_build.inc"
}  // namespace gbrt
