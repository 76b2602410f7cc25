// nrc.cu — kernels of the neural radiance cache (layout in nrc.cuh).
//
// * nrc_infer_kernel: queries (the path tracer's hot use): FP16 hash-grid
//   gather, then the MLP on tensor cores (mma.sync m16n8k16, BF16 inputs,
//   FP32 accumulation).  A warp takes 32 queries; the encoding is written to
//   shared memory once and read back as A fragments, and every later layer's
//   A fragments are the previous layer's accumulators after ReLU and BF16
//   packing, so activations never leave registers.  Weights (BF16, rows
//   padded by 8 to spread the shared-memory banks) are loaded once per block.
// * nrc_train_kernel: one thread per training sample, FP32: encoding from
//   the FP32 master table, forward, relative L2 loss (y - t)^2 / (sg(y)^2 +
//   0.01) averaged over samples and channels, backward to the encoding; the
//   table gradient is scattered with atomics, activations and pre-activation
//   gradients are stored for
// * nrc_wgrad_kernel: dW_l = sum over samples of dZ_{l+1} H_l^T, split over
//   the batch, atomics into the FP32 gradient;
// * nrc_adam_grid_kernel / nrc_adam_mlp_kernel: Adam on the FP32 masters,
//   rewriting the FP16 / BF16 copies the queries read.
#include <cmath>
#include <cstring>
#include <new>
#include <random>
#include <vector>

#include "api_internal.h"
#include "nrc.cuh"

using namespace gbrt;

namespace gbrt {

namespace {

constexpr int kActStride = kNrcIn + kNrcHiddenLayers * kNrcHidden;    // 352: H0 | H1..H5
constexpr int kGradStride = kNrcHiddenLayers * kNrcHidden + 8;        // 328: dZ1..dZ5 | dY (3, padded)
constexpr int kPadK = 8;                                               // BF16 row padding

// offsets of layer l in the padded BF16 copy
__host__ __device__ constexpr int bf16_off(int l) {
    return l == 0 ? 0 : kNrcHidden * (kNrcIn + kPadK) + (l - 1) * kNrcHidden * (kNrcHidden + kPadK);
}
constexpr int kBf16Padded = bf16_off(5) + 8 * (kNrcHidden + kPadK);  // 21568
__host__ __device__ constexpr int f32_off(int l) { return l == 0 ? 0 : kNrcWh + (l - 1) * kNrcHidden * kNrcHidden; }
__host__ __device__ constexpr int in_dim(int l) { return l == 0 ? kNrcIn : kNrcHidden; }
__host__ __device__ constexpr int out_dim(int l) { return l == 5 ? kNrcOut : kNrcHidden; }

GB_D void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

GB_D uint32_t pack_bf16(float lo, float hi) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&h);
}

// One layer on a warp's 32 rows: acc[m][nt] = A[m] (32 x K) * W^T (K x 8*NT).
template <int K, int NT>
GB_D void mlp_layer(const __nv_bfloat16* w, const uint32_t (&a)[2][4][4], float (&acc)[2][8][4], int g, int t) {
#pragma unroll
    for (int m = 0; m < 2; ++m)
#pragma unroll
        for (int n = 0; n < NT; ++n) acc[m][n][0] = acc[m][n][1] = acc[m][n][2] = acc[m][n][3] = 0.0f;
#pragma unroll
    for (int ks = 0; ks < K / 16; ++ks) {
#pragma unroll
        for (int n = 0; n < NT; ++n) {
            const __nv_bfloat16* row = w + (n * 8 + g) * (K + kPadK) + ks * 16 + t * 2;
            const uint32_t b0 = *reinterpret_cast<const uint32_t*>(row);
            const uint32_t b1 = *reinterpret_cast<const uint32_t*>(row + 8);
            mma_bf16(acc[0][n], a[0][ks], b0, b1);
            mma_bf16(acc[1][n], a[1][ks], b0, b1);
        }
    }
}

// Accumulators of a 64-wide layer -> ReLU -> A fragments of the next layer.
GB_D void relu_to_a(const float (&acc)[2][8][4], uint32_t (&a)[2][4][4]) {
#pragma unroll
    for (int m = 0; m < 2; ++m)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            a[m][j][0] = pack_bf16(fmaxf(acc[m][2 * j][0], 0.0f), fmaxf(acc[m][2 * j][1], 0.0f));
            a[m][j][1] = pack_bf16(fmaxf(acc[m][2 * j][2], 0.0f), fmaxf(acc[m][2 * j][3], 0.0f));
            a[m][j][2] = pack_bf16(fmaxf(acc[m][2 * j + 1][0], 0.0f), fmaxf(acc[m][2 * j + 1][1], 0.0f));
            a[m][j][3] = pack_bf16(fmaxf(acc[m][2 * j + 1][2], 0.0f), fmaxf(acc[m][2 * j + 1][3], 0.0f));
        }
}

}  // namespace

// FP16 encoding of one point (32 features).
GB_D void nrc_encode_h(const NrcView& v, float3 p, float (&x)[kNrcIn]) {
#pragma unroll
    for (int l = 0; l < kNrcLevels; ++l) {
        float f0 = 0.0f, f1 = 0.0f;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            uint32_t idx;
            float w;
            nrc_corner(v, l, p, c, idx, w);
            const float2 e = __half22float2(v.grid_h[idx]);
            f0 = fmaf(w, e.x, f0);
            f1 = fmaf(w, e.y, f1);
        }
        x[2 * l] = f0;
        x[2 * l + 1] = f1;
    }
}

constexpr int kInferWarps = 4;
constexpr int kInRow = kNrcIn + kPadK;  // 40 BF16 per input row
constexpr size_t kInferSmem = (size_t)kBf16Padded * 2 + (size_t)kInferWarps * 32 * kInRow * 2;

// q[i] = (position, payload); out[i] = (radiance, payload)
__global__ void __launch_bounds__(128) nrc_infer_kernel(NrcView v, const float4* __restrict__ q, uint32_t n,
                                                        float4* __restrict__ out, const uint32_t* n_dev) {
    if (n_dev) n = min(n, *n_dev);
    if (blockIdx.x * kInferWarps * 32u >= n) return;  // no queries for this block: skip the weight copy
    extern __shared__ __align__(16) unsigned char smem[];
    __nv_bfloat16* sw = reinterpret_cast<__nv_bfloat16*>(smem);
    __nv_bfloat16* sin_all = sw + kBf16Padded;
    {
        const uint4* src = reinterpret_cast<const uint4*>(v.mlp_h);
        uint4* dst = reinterpret_cast<uint4*>(sw);
        for (int i = threadIdx.x; i < kBf16Padded / 8; i += blockDim.x) dst[i] = src[i];
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    __nv_bfloat16* sin = sin_all + warp * 32 * kInRow;
    for (uint32_t base = (blockIdx.x * kInferWarps + warp) * 32u; base < n;
         base += gridDim.x * kInferWarps * 32u) {
        const uint32_t i = base + lane;
        {
            float x[kNrcIn];
            const float4 qi = i < n ? q[i] : f4(0.0f, 0.0f, 0.0f, 0.0f);
            nrc_encode_h(v, nrc_normalise(v, f3(qi)), x);
#pragma unroll
            for (int k = 0; k < kNrcIn; k += 2)
                *reinterpret_cast<uint32_t*>(sin + lane * kInRow + k) = pack_bf16(x[k], x[k + 1]);
        }
        __syncwarp();
        uint32_t a[2][4][4];
#pragma unroll
        for (int m = 0; m < 2; ++m)
#pragma unroll
            for (int ks = 0; ks < 2; ++ks) {
                const __nv_bfloat16* r0 = sin + (m * 16 + g) * kInRow + ks * 16 + t * 2;
                const __nv_bfloat16* r1 = r0 + 8 * kInRow;
                a[m][ks][0] = *reinterpret_cast<const uint32_t*>(r0);
                a[m][ks][1] = *reinterpret_cast<const uint32_t*>(r1);
                a[m][ks][2] = *reinterpret_cast<const uint32_t*>(r0 + 8);
                a[m][ks][3] = *reinterpret_cast<const uint32_t*>(r1 + 8);
            }
        __syncwarp();
        float acc[2][8][4];
        mlp_layer<kNrcIn, 8>(sw + bf16_off(0), a, acc, g, t);
        relu_to_a(acc, a);
#pragma unroll
        for (int l = 1; l < kNrcHiddenLayers; ++l) {
            mlp_layer<kNrcHidden, 8>(sw + bf16_off(l), a, acc, g, t);
            relu_to_a(acc, a);
        }
        mlp_layer<kNrcHidden, 1>(sw + bf16_off(5), a, acc, g, t);
        // output columns 0..2: lanes t = 0 (cols 0, 1) and t = 1 (col 2)
#pragma unroll
        for (int m = 0; m < 2; ++m)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const uint32_t row = base + m * 16 + g + h * 8;
                if (row < n) {
                    float* o = reinterpret_cast<float*>(out + row);
                    if (t == 0) {
                        o[0] = acc[m][0][2 * h];
                        o[1] = acc[m][0][2 * h + 1];
                    } else if (t == 1) {
                        o[2] = acc[m][0][2 * h];
                        o[3] = q[row].w;
                    }
                }
            }
    }
}

// ---------------------------------------------------------------------------
// Queries on the 5th-generation tensor cores (tcgen05).  A CTA of 128 threads
// takes 128 queries per step: thread i encodes query i into row i of the A
// tile (shared memory, BF16, K-major canonical layout without swizzle: 8x8
// core matrices of 128 B, K-adjacent ones 128 B apart, 8-row groups K*16 B
// apart); one elected thread issues the layer's tcgen05.mma (M = 128, N = 64
// or 16, K = 16 per instruction) with the FP32 accumulator in tensor memory
// (64 columns), commits to an mbarrier, and every warp reads its 32 rows back
// with tcgen05.ld, applies ReLU, and writes them as the next layer's A tile.
// Weights stay in shared memory in the same layout for the whole kernel.
// Every wait is bounded: on a timeout the kernel records kTcTimeout in
// *status and stops issuing work.

constexpr uint32_t kTcTimeout = 1u;
constexpr int kTcRows = 128;
// BF16 weights in core-matrix layout: layer l occupies out_l x in_l (W5 padded to 16 rows)
__host__ __device__ constexpr int tc_w_off(int l) {  // in elements
    return l == 0 ? 0 : kNrcHidden * kNrcIn + (l - 1) * kNrcHidden * kNrcHidden;
}
constexpr int kTcWElems = tc_w_off(5) + 16 * kNrcHidden;                    // 19,456
constexpr size_t kTcSmem = (size_t)kTcWElems * 2 + (size_t)kTcRows * kNrcHidden * 2 + 64;

// byte offset of element (row, k) in a K-major no-swizzle tile with K columns
GB_D uint32_t tc_core_off(uint32_t row, uint32_t k, uint32_t K) {
    return ((row >> 3) * (K >> 3) + (k >> 3)) * 128u + (row & 7u) * 16u + (k & 7u) * 2u;
}

// Shared-memory matrix descriptor: start >> 4 (bits 0-13), leading (K)
// byte offset >> 4 (16-29), stride (8-row group) byte offset >> 4 (32-45),
// version 1 (46-47), no swizzle (61-63 = 0).
GB_D uint64_t tc_smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), BF16
// A and B (7-9 = 1, 10-12 = 1), both K-major, N >> 3 at bits 17-22, M >> 4 at
// bits 24-28.
__host__ __device__ constexpr uint32_t tc_idesc(uint32_t M, uint32_t N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

GB_D void tc_mma(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.u32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

GB_D bool tc_wait(uint32_t mbar, uint32_t phase) {
    for (uint32_t it = 0; it < (1u << 22); ++it) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(mbar), "r"(phase)
            : "memory");
        if (done) return true;
    }
    return false;
}

#define TC_LD16(base, v)                                                                                        \
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, " \
                 "[%16];\n"                                                                                     \
                 : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),          \
                   "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),      \
                   "=r"(v[14]), "=r"(v[15])                                                                     \
                 : "r"(base))

__global__ void __launch_bounds__(128, 1) nrc_infer_tc_kernel(NrcView v, const float4* __restrict__ q, uint32_t n,
                                                              float4* __restrict__ out, const uint32_t* n_dev,
                                                              const __nv_bfloat16* __restrict__ wtc,
                                                              uint32_t* status) {
    extern __shared__ __align__(16) unsigned char smem_tc[];
    unsigned char* sw = smem_tc;                             // weights
    unsigned char* sa = smem_tc + (size_t)kTcWElems * 2;     // A tile, 128 x 64 BF16
    uint64_t* mbar = reinterpret_cast<uint64_t*>(sa + kTcRows * kNrcHidden * 2);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 1);
    if (n_dev) n = min(n, *n_dev);
    if (blockIdx.x * kTcRows >= n) return;  // no tile for this block: skip the weight copy and the allocation
    const uint32_t tid = threadIdx.x, warp = tid >> 5;
    {  // weights are pre-arranged in core-matrix order by the host
        const uint4* src = reinterpret_cast<const uint4*>(wtc);
        uint4* dst = reinterpret_cast<uint4*>(sw);
        for (int i = tid; i < kTcWElems / 8; i += blockDim.x) dst[i] = src[i];
    }
    const uint32_t sw_s = (uint32_t)__cvta_generic_to_shared(sw), sa_s = (uint32_t)__cvta_generic_to_shared(sa);
    const uint32_t mbar_s = (uint32_t)__cvta_generic_to_shared(mbar);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mbar_s));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        const uint32_t dst = (uint32_t)__cvta_generic_to_shared(tslot);
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 64;\n" ::"r"(dst));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *tslot;
    const uint32_t tlane = tmem + ((warp * 32u) << 16);  // this warp's 32 lanes
    uint32_t phase = 0;
    bool ok = true;
    for (uint32_t base = blockIdx.x * kTcRows; base < n && ok; base += gridDim.x * kTcRows) {
        const uint32_t i = base + tid;
        {
            float x[kNrcIn];
            const float4 qi = i < n ? q[i] : f4(0.0f, 0.0f, 0.0f, 0.0f);
            nrc_encode_h(v, nrc_normalise(v, f3(qi)), x);
#pragma unroll
            for (int k = 0; k < kNrcIn; k += 8) {
                uint4 pk;
                pk.x = pack_bf16(x[k], x[k + 1]);
                pk.y = pack_bf16(x[k + 2], x[k + 3]);
                pk.z = pack_bf16(x[k + 4], x[k + 5]);
                pk.w = pack_bf16(x[k + 6], x[k + 7]);
                *reinterpret_cast<uint4*>(sa + tc_core_off(tid, k, kNrcIn)) = pk;
            }
        }
        float y[3] = {0.0f, 0.0f, 0.0f};
        for (int l = 0; l < 6 && ok; ++l) {
            const uint32_t K = l == 0 ? kNrcIn : kNrcHidden, N = l == 5 ? 16 : kNrcHidden;
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            __syncthreads();
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            if (tid == 0) {
                const uint32_t wbase = sw_s + (uint32_t)tc_w_off(l) * 2u;
                for (uint32_t ks = 0; ks < K / 16; ++ks) {
                    const uint64_t ad = tc_smem_desc(sa_s + ks * 256u, 128u, K * 16u);
                    const uint64_t bd = tc_smem_desc(wbase + ks * 256u, 128u, K * 16u);
                    tc_mma(tmem, ad, bd, tc_idesc(kTcRows, N), ks);
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                    mbar_s)
                             : "memory");
            }
            ok = __syncthreads_and(tc_wait(mbar_s, phase) ? 1 : 0) != 0;  // uniform across the CTA
            phase ^= 1u;
            if (!ok) break;
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            if (l < 5) {
#pragma unroll
                for (int c = 0; c < kNrcHidden; c += 16) {
                    uint32_t r[16];
                    TC_LD16(tlane + (uint32_t)c, r);
                    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
                    for (int k = 0; k < 16; k += 8) {
                        uint4 pk;
                        pk.x = pack_bf16(fmaxf(__uint_as_float(r[k]), 0.0f), fmaxf(__uint_as_float(r[k + 1]), 0.0f));
                        pk.y = pack_bf16(fmaxf(__uint_as_float(r[k + 2]), 0.0f), fmaxf(__uint_as_float(r[k + 3]), 0.0f));
                        pk.z = pack_bf16(fmaxf(__uint_as_float(r[k + 4]), 0.0f), fmaxf(__uint_as_float(r[k + 5]), 0.0f));
                        pk.w = pack_bf16(fmaxf(__uint_as_float(r[k + 6]), 0.0f), fmaxf(__uint_as_float(r[k + 7]), 0.0f));
                        *reinterpret_cast<uint4*>(sa + tc_core_off(tid, c + k, kNrcHidden)) = pk;
                    }
                }
            } else {
                uint32_t r[16];
                TC_LD16(tlane, r);
                asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
                y[0] = __uint_as_float(r[0]);
                y[1] = __uint_as_float(r[1]);
                y[2] = __uint_as_float(r[2]);
            }
        }
        if (ok && i < n) out[i] = f4(y[0], y[1], y[2], q[i].w);
    }
    if (!ok) {
        if (status && tid == 0) atomicOr(status, kTcTimeout);
        tc_wait(mbar_s, phase ^ 1u);  // give the MMAs still in flight (bounded) time before the columns are freed
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 64;\n" ::"r"(tmem));
}

// FP32 masters -> BF16 weights in the core-matrix order of the tcgen05
// kernel (W5 padded to 16 rows with zeros).
__global__ void nrc_tc_weights_kernel(const float* __restrict__ w, __nv_bfloat16* __restrict__ wtc) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= kTcWElems) return;
    int l = 0;
    while (l < 5 && e >= tc_w_off(l + 1)) ++l;
    const int K = l == 0 ? kNrcIn : kNrcHidden;
    const int local = e - tc_w_off(l);
    // invert tc_core_off: 128-B core matrices of 8 rows x 8 elements
    const int cm = local / 64, within = local % 64;
    const int kc = cm % (K / 8), rg = cm / (K / 8);
    const int row = rg * 8 + within / 8, k = kc * 8 + within % 8;
    const int O = l == 5 ? kNrcOut : kNrcHidden;
    const float x = row < O ? w[f32_off(l) + row * K + k] : 0.0f;
    wtc[e] = __float2bfloat16_rn(x);
}

struct NrcGrad {
    float* grid;  // [levels * table * 2]
    float* mlp;   // [kNrcMlpParams]
    float* act;   // [n][kActStride]
    float* dz;    // [n][kGradStride]
    float* loss;  // one word
};

constexpr size_t kTrainSmem = (size_t)kNrcMlpParams * 4;

__global__ void __launch_bounds__(128) nrc_train_kernel(NrcView v, NrcGrad gr, const float4* __restrict__ pos,
                                                        const float4* __restrict__ target, uint32_t n, float inv_n) {
    extern __shared__ float swf[];
    for (int i = threadIdx.x; i < kNrcMlpParams; i += blockDim.x) swf[i] = v.mlp_w[i];
    __syncthreads();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float loss = 0.0f;
    if (i < n) {
        float* A = gr.act + (size_t)i * kActStride;
        float* D = gr.dz + (size_t)i * kGradStride;
        const float3 p = nrc_normalise(v, f3(pos[i]));
        float x[kNrcIn];
#pragma unroll
        for (int l = 0; l < kNrcLevels; ++l) {
            float f0 = 0.0f, f1 = 0.0f;
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                uint32_t idx;
                float w;
                nrc_corner(v, l, p, c, idx, w);
                f0 = fmaf(w, v.grid_w[2 * idx], f0);
                f1 = fmaf(w, v.grid_w[2 * idx + 1], f1);
            }
            x[2 * l] = f0;
            x[2 * l + 1] = f1;
        }
        for (int k = 0; k < kNrcIn; ++k) A[k] = x[k];
        float h[kNrcHidden];
        for (int o = 0; o < kNrcHidden; ++o) {
            float s = 0.0f;
#pragma unroll
            for (int k = 0; k < kNrcIn; ++k) s = fmaf(swf[o * kNrcIn + k], x[k], s);
            h[o] = fmaxf(s, 0.0f);
            A[kNrcIn + o] = h[o];
        }
        for (int l = 1; l < kNrcHiddenLayers; ++l) {
            const float* W = swf + f32_off(l);
            float hn[kNrcHidden];
            for (int o = 0; o < kNrcHidden; ++o) {
                float s = 0.0f;
#pragma unroll
                for (int k = 0; k < kNrcHidden; ++k) s = fmaf(W[o * kNrcHidden + k], h[k], s);
                hn[o] = fmaxf(s, 0.0f);
            }
            for (int o = 0; o < kNrcHidden; ++o) {
                h[o] = hn[o];
                A[kNrcIn + l * kNrcHidden + o] = hn[o];
            }
        }
        const float4 tg = target[i];
        const float tc[3] = {tg.x, tg.y, tg.z};
        float dy[3];
        for (int c = 0; c < 3; ++c) {
            float y = 0.0f;
#pragma unroll
            for (int k = 0; k < kNrcHidden; ++k) y = fmaf(swf[kNrcW5 + c * kNrcHidden + k], h[k], y);
            const float d = y - tc[c], den = y * y + 0.01f;
            loss += d * d / den;
            dy[c] = 2.0f * d / den * (inv_n / 3.0f);
            D[5 * kNrcHidden + c] = dy[c];
        }
        // backward: dZ5 = (W5^T dy) * [H5 > 0]
        float dz[kNrcHidden];
        for (int k = 0; k < kNrcHidden; ++k) {
            const float s = swf[kNrcW5 + k] * dy[0] + swf[kNrcW5 + kNrcHidden + k] * dy[1] +
                            swf[kNrcW5 + 2 * kNrcHidden + k] * dy[2];
            dz[k] = h[k] > 0.0f ? s : 0.0f;
            D[4 * kNrcHidden + k] = dz[k];
        }
        // hidden layers l = 4..1: dZ_l = (W_l^T dZ_{l+1}) * [H_l > 0]
        for (int l = kNrcHiddenLayers - 1; l >= 1; --l) {
            const float* W = swf + f32_off(l);
            const float* Hl = A + kNrcIn + (l - 1) * kNrcHidden;
            float dp[kNrcHidden];
            for (int k = 0; k < kNrcHidden; ++k) {
                float s = 0.0f;
#pragma unroll 8
                for (int o = 0; o < kNrcHidden; ++o) s = fmaf(W[o * kNrcHidden + k], dz[o], s);
                dp[k] = Hl[k] > 0.0f ? s : 0.0f;
            }
            for (int k = 0; k < kNrcHidden; ++k) {
                dz[k] = dp[k];
                D[(l - 1) * kNrcHidden + k] = dp[k];
            }
        }
        // encoding gradient dH0 = W0^T dZ1, scattered to the table corners
        float dx[kNrcIn];
        for (int k = 0; k < kNrcIn; ++k) {
            float s = 0.0f;
#pragma unroll 8
            for (int o = 0; o < kNrcHidden; ++o) s = fmaf(swf[o * kNrcIn + k], dz[o], s);
            dx[k] = s;
        }
        for (int l = 0; l < kNrcLevels; ++l)
            for (int c = 0; c < 8; ++c) {
                uint32_t idx;
                float w;
                nrc_corner(v, l, p, c, idx, w);
                atomicAdd(&gr.grid[2 * idx], w * dx[2 * l]);
                atomicAdd(&gr.grid[2 * idx + 1], w * dx[2 * l + 1]);
            }
    }
    for (int o = 16; o > 0; o >>= 1) loss += __shfl_down_sync(0xFFFFFFFFu, loss, o);
    if ((threadIdx.x & 31) == 0 && loss != 0.0f) atomicAdd(gr.loss, loss * inv_n / 3.0f);
}

// dW_l[o][k] = sum_m D[m][dz of layer l's output o] * A[m][input k of layer l];
// block (split, layer), 256 threads, samples [split*chunk, ...) in tiles of 32.
__global__ void __launch_bounds__(256) nrc_wgrad_kernel(const float* __restrict__ act, const float* __restrict__ dz,
                                                        uint32_t n, uint32_t chunk, float* grad) {
    const int l = blockIdx.y;
    const int K = in_dim(l), O = out_dim(l);
    const int aoff = l == 0 ? 0 : kNrcIn + (l - 1) * kNrcHidden;
    const int doff = l == 5 ? 5 * kNrcHidden : l * kNrcHidden;
    __shared__ float sa[32][kNrcHidden + 1], sd[32][kNrcHidden + 1];
    float accv[16];
    for (int e = 0; e < 16; ++e) accv[e] = 0.0f;
    const uint32_t m0 = blockIdx.x * chunk, m1 = min(n, m0 + chunk);
    for (uint32_t mb = m0; mb < m1; mb += 32) {
        for (int e = threadIdx.x; e < 32 * kNrcHidden; e += blockDim.x) {
            const int r = e / kNrcHidden, c = e % kNrcHidden;
            const uint32_t m = mb + r;
            sa[r][c] = (m < m1 && c < K) ? act[(size_t)m * kActStride + aoff + c] : 0.0f;
            sd[r][c] = (m < m1 && c < O) ? dz[(size_t)m * kGradStride + doff + c] : 0.0f;
        }
        __syncthreads();
        for (int e = 0; e < 16; ++e) {
            const int idx = threadIdx.x + e * 256;  // (o, k) flattened, o * 64 + k
            const int o = idx >> 6, k = idx & 63;
            float s = accv[e];
#pragma unroll 8
            for (int r = 0; r < 32; ++r) s = fmaf(sd[r][o], sa[r][k], s);
            accv[e] = s;
        }
        __syncthreads();
    }
    for (int e = 0; e < 16; ++e) {
        const int idx = threadIdx.x + e * 256;
        const int o = idx >> 6, k = idx & 63;
        if (o < O && k < K && accv[e] != 0.0f) atomicAdd(&grad[f32_off(l) + o * K + k], accv[e]);
    }
}

// ---------------------------------------------------------------------------
// Training on tensor cores (the default; GBRT_NRC_TRAIN_FP32 keeps the FP32
// kernels above).  BF16 operands, FP32 accumulation, mma.sync m16n8k16:
// * nrc_train_tc_kernel: a warp takes 32 samples: FP32 encoding from the
//   master table (lane = sample), the forward pass layer by layer as in the
//   queries (accumulators -> ReLU -> BF16 A fragments in registers), the loss
//   and dL/dy in FP32, then the backward pass dH_l = dZ_{l+1} W_l on the
//   tensor cores with the transposed BF16 weights, the ReLU masks read back
//   from the stored activations; the encoding gradient is scattered into the
//   table gradient with float2 atomics.  Activations H_0..H_5 and
//   pre-activation gradients dZ_1..dZ_5, dY are written in BF16, sample-major;
// * nrc_wgrad_tc_kernel: dW_l = dZ_{l+1}^T H_l over the batch, split-K over
//   samples: tiles of 64 samples staged in shared memory, operands loaded
//   transposed with ldmatrix.trans, partial sums added with atomics.
// The float64 oracle reproduces these roundings (oracle/nrc_ref.py, bf16).
// ---------------------------------------------------------------------------
constexpr int kTActStride = kNrcIn + kNrcHiddenLayers * kNrcHidden;  // 352 BF16: H0 | H1..H5
constexpr int kTGradStride = kNrcHiddenLayers * kNrcHidden + 16;     // 336 BF16: dZ1..dZ5 | dY (3, padded to 16)
__host__ __device__ constexpr int bwd_out_pad(int l) { return l == 5 ? 16 : kNrcHidden; }
// transposed BF16 weights W_l^T [in][out padded + 8], layer offsets
__host__ __device__ constexpr int bwd_off(int l) {
    return l == 0 ? 0 : bwd_off(l - 1) + in_dim(l - 1) * (bwd_out_pad(l - 1) + kPadK);
}
constexpr int kBwdElems = bwd_off(6);  // 22272
constexpr int kTrainWarps = 4;
constexpr int kXRow = kNrcIn + 1;  // FP32 row of the encoding-gradient staging tile
constexpr size_t kTrainTcSmem =
    (size_t)(kBf16Padded + kBwdElems) * 2 + (size_t)kTrainWarps * 32 * kXRow * 4;

// Every element of the transposed copy, zero in the padding (the dY
// padding columns multiply it).
__global__ void nrc_bwd_weights_kernel(const float* __restrict__ w, __nv_bfloat16* __restrict__ wt) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= kBwdElems) return;
    int l = 0;
    while (l < 5 && e >= bwd_off(l + 1)) ++l;
    const int row = (e - bwd_off(l)) / (bwd_out_pad(l) + kPadK), col = (e - bwd_off(l)) % (bwd_out_pad(l) + kPadK);
    const float x = col < out_dim(l) ? w[f32_off(l) + col * in_dim(l) + row] : 0.0f;  // W_l[o = col][k = row]
    wt[e] = __float2bfloat16_rn(x);
}

// The 16 x (8 NT) accumulators of rows m*16 + {g, g + 8} as BF16 A-fragment
// words, stored at row-major BF16 offset `col0` of each sample's row.
GB_D void store_frag_rows(uint32_t* dst_row0, uint32_t base, uint32_t n, int stride_words, int col0,
                          const uint32_t (&a)[2][4][4], int nk, int g, int t) {
#pragma unroll
    for (int m = 0; m < 2; ++m)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const uint32_t row = base + m * 16 + g + h * 8;
            if (row >= n) continue;
            uint32_t* r = dst_row0 + (size_t)row * stride_words + col0 / 2;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                if (j >= nk) break;
                r[j * 8 + t] = a[m][j][h];          // cols 16 j + 2 t, + 1
                r[j * 8 + 4 + t] = a[m][j][2 + h];  // cols 16 j + 8 + 2 t, + 1
            }
        }
}

// dZ = dH * [H > 0] in the accumulator layout, H read back as BF16 pairs
// from the stored activations (rows past n: H = 0), then packed as A
// fragments.
GB_D void mask_to_a(const float (&acc)[2][8][4], const uint32_t* act_row0, uint32_t base, uint32_t n, int hcol0,
                    uint32_t (&a)[2][4][4], int g, int t) {
#pragma unroll
    for (int m = 0; m < 2; ++m) {
        uint32_t hw[2][8];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const uint32_t row = base + m * 16 + g + h * 8;
            const uint32_t* r = act_row0 + (size_t)row * (kTActStride / 2) + hcol0 / 2;
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) hw[h][nt] = row < n ? r[nt * 4 + t] : 0u;
        }
        float d[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                // BF16 halves: low 16 bits = col 2t, high = col 2t + 1; positive iff > 0
                const uint32_t lo = hw[h][nt] & 0xFFFFu, hi = hw[h][nt] >> 16;
                d[nt][2 * h] = (lo != 0u && !(lo & 0x8000u)) ? acc[m][nt][2 * h] : 0.0f;
                d[nt][2 * h + 1] = (hi != 0u && !(hi & 0x8000u)) ? acc[m][nt][2 * h + 1] : 0.0f;
            }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            a[m][j][0] = pack_bf16(d[2 * j][0], d[2 * j][1]);
            a[m][j][1] = pack_bf16(d[2 * j][2], d[2 * j][3]);
            a[m][j][2] = pack_bf16(d[2 * j + 1][0], d[2 * j + 1][1]);
            a[m][j][3] = pack_bf16(d[2 * j + 1][2], d[2 * j + 1][3]);
        }
    }
}

struct NrcTcGrad {
    float* grid;            // [levels * table * 2]
    float* loss;            // one word
    uint32_t* act;          // [n][kTActStride / 2] BF16 pairs
    uint32_t* dz;           // [n][kTGradStride / 2] BF16 pairs
};

__global__ void __launch_bounds__(kTrainWarps * 32)
    nrc_train_tc_kernel(NrcView v, NrcTcGrad gr, const __nv_bfloat16* __restrict__ wbwd, const float4* __restrict__ pos,
                        const float4* __restrict__ target, uint32_t n, float inv_n) {
    extern __shared__ __align__(16) unsigned char smem[];
    __nv_bfloat16* swf = reinterpret_cast<__nv_bfloat16*>(smem);  // forward weights, padded rows
    __nv_bfloat16* swb = swf + kBf16Padded;                        // transposed weights
    float* sx_all = reinterpret_cast<float*>(swb + kBwdElems);
    {
        const uint4* src = reinterpret_cast<const uint4*>(v.mlp_h);
        uint4* dst = reinterpret_cast<uint4*>(swf);
        for (int i = threadIdx.x; i < kBf16Padded / 8; i += blockDim.x) dst[i] = src[i];
        src = reinterpret_cast<const uint4*>(wbwd);
        dst = reinterpret_cast<uint4*>(swb);
        for (int i = threadIdx.x; i < kBwdElems / 8; i += blockDim.x) dst[i] = src[i];
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    float* sx = sx_all + warp * 32 * kXRow;
    __nv_bfloat16* sin = reinterpret_cast<__nv_bfloat16*>(sx);  // the BF16 encoding tile shares it (32 x 40)
    float loss = 0.0f;
    for (uint32_t base = (blockIdx.x * kTrainWarps + warp) * 32u; base < n; base += gridDim.x * kTrainWarps * 32u) {
        const uint32_t i = base + lane;
        float3 p = f3(0.0f);
        {  // encoding from the FP32 master table, lane = sample
            float x[kNrcIn];
            if (i < n) {
                p = nrc_normalise(v, f3(pos[i]));
#pragma unroll
                for (int l = 0; l < kNrcLevels; ++l) {
                    float f0 = 0.0f, f1 = 0.0f;
#pragma unroll
                    for (int c = 0; c < 8; ++c) {
                        uint32_t idx;
                        float w;
                        nrc_corner(v, l, p, c, idx, w);
                        const float2 e = reinterpret_cast<const float2*>(v.grid_w)[idx];
                        f0 = fmaf(w, e.x, f0);
                        f1 = fmaf(w, e.y, f1);
                    }
                    x[2 * l] = f0;
                    x[2 * l + 1] = f1;
                }
            } else {
#pragma unroll
                for (int k = 0; k < kNrcIn; ++k) x[k] = 0.0f;
            }
            uint32_t* arow = i < n ? gr.act + (size_t)i * (kTActStride / 2) : nullptr;
#pragma unroll
            for (int k = 0; k < kNrcIn; k += 2) {
                const uint32_t pk = pack_bf16(x[k], x[k + 1]);
                *reinterpret_cast<uint32_t*>(sin + lane * kInRow + k) = pk;
                if (arow) arow[k / 2] = pk;
            }
        }
        __syncwarp();
        uint32_t a[2][4][4];
#pragma unroll
        for (int m = 0; m < 2; ++m)
#pragma unroll
            for (int ks = 0; ks < 2; ++ks) {
                const __nv_bfloat16* r0 = sin + (m * 16 + g) * kInRow + ks * 16 + t * 2;
                const __nv_bfloat16* r1 = r0 + 8 * kInRow;
                a[m][ks][0] = *reinterpret_cast<const uint32_t*>(r0);
                a[m][ks][1] = *reinterpret_cast<const uint32_t*>(r1);
                a[m][ks][2] = *reinterpret_cast<const uint32_t*>(r0 + 8);
                a[m][ks][3] = *reinterpret_cast<const uint32_t*>(r1 + 8);
            }
        __syncwarp();
        // forward
        float acc[2][8][4];
#pragma unroll 1
        for (int l = 0; l < kNrcHiddenLayers; ++l) {
            if (l == 0) mlp_layer<kNrcIn, 8>(swf + bf16_off(0), a, acc, g, t);
            else mlp_layer<kNrcHidden, 8>(swf + bf16_off(l), a, acc, g, t);
            relu_to_a(acc, a);
            store_frag_rows(gr.act, base, n, kTActStride / 2, kNrcIn + l * kNrcHidden, a, 4, g, t);
        }
        mlp_layer<kNrcHidden, 1>(swf + bf16_off(5), a, acc, g, t);
        // loss and dL/dy (columns 0..2 of the output tile: t = 0 holds 0, 1; t = 1 holds 2)
        uint32_t ady[2][4][4];
#pragma unroll
        for (int m = 0; m < 2; ++m) {
            float dy[4];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const uint32_t row = base + m * 16 + g + h * 8;
                const float4 tg = (row < n && t < 2) ? target[row] : f4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    const int col = 2 * t + q;
                    float d = 0.0f;
                    if (row < n && col < kNrcOut) {
                        const float y = acc[m][0][2 * h + q];
                        const float tc = col == 0 ? tg.x : (col == 1 ? tg.y : tg.z);
                        const float dd = y - tc, den = y * y + 0.01f;
                        loss += dd * dd / den;
                        d = 2.0f * dd / den * (inv_n / 3.0f);
                    }
                    dy[2 * h + q] = d;
                }
            }
            ady[m][0][0] = pack_bf16(dy[0], dy[1]);
            ady[m][0][1] = pack_bf16(dy[2], dy[3]);
            ady[m][0][2] = 0u;
            ady[m][0][3] = 0u;
        }
        store_frag_rows(gr.dz, base, n, kTGradStride / 2, kNrcHiddenLayers * kNrcHidden, ady, 1, g, t);
        // backward: dH5 = dY W5, dZ5 = dH5 * [H5 > 0]
        mlp_layer<16, 8>(swb + bwd_off(5), ady, acc, g, t);
        mask_to_a(acc, gr.act, base, n, kNrcIn + 4 * kNrcHidden, a, g, t);
        store_frag_rows(gr.dz, base, n, kTGradStride / 2, 4 * kNrcHidden, a, 4, g, t);
#pragma unroll 1
        for (int l = kNrcHiddenLayers - 1; l >= 1; --l) {  // dZ_l = (dZ_{l+1} W_l) * [H_l > 0]
            mlp_layer<kNrcHidden, 8>(swb + bwd_off(l), a, acc, g, t);
            mask_to_a(acc, gr.act, base, n, kNrcIn + (l - 1) * kNrcHidden, a, g, t);
            store_frag_rows(gr.dz, base, n, kTGradStride / 2, (l - 1) * kNrcHidden, a, 4, g, t);
        }
        // encoding gradient dX = dZ1 W0 (32 columns), to lane = sample through shared memory
        mlp_layer<kNrcHidden, 4>(swb + bwd_off(0), a, acc, g, t);
        __syncwarp();
#pragma unroll
        for (int m = 0; m < 2; ++m)
#pragma unroll
            for (int nt = 0; nt < 4; ++nt)
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    float* r = sx + (m * 16 + g + h * 8) * kXRow + nt * 8 + 2 * t;
                    r[0] = acc[m][nt][2 * h];
                    r[1] = acc[m][nt][2 * h + 1];
                }
        __syncwarp();
        if (i < n) {
            const float* dx = sx + lane * kXRow;
#pragma unroll 1
            for (int l = 0; l < kNrcLevels; ++l)
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                    uint32_t idx;
                    float w;
                    nrc_corner(v, l, p, c, idx, w);
                    atomicAdd(reinterpret_cast<float2*>(gr.grid) + idx, make_float2(w * dx[2 * l], w * dx[2 * l + 1]));
                }
        }
        __syncwarp();
    }
    for (int o = 16; o > 0; o >>= 1) loss += __shfl_down_sync(0xFFFFFFFFu, loss, o);
    if (lane == 0 && loss != 0.0f) atomicAdd(gr.loss, loss * inv_n / 3.0f);
}

GB_D void ldsm_x4_trans(uint32_t (&r)[4], const void* p) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}

constexpr int kWgTile = 64;              // samples per shared-memory tile
constexpr int kWgRow = kNrcHidden + 8;   // padded BF16 row (144 B: ldmatrix rows hit distinct banks)

// dW_l[o][k] += sum over the block's samples of dZ[m][o] H[m][k]; block =
// (sample split, layer), 4 warps, warp w owns rows o in [16 w, 16 w + 16).
__global__ void __launch_bounds__(128) nrc_wgrad_tc_kernel(const uint32_t* __restrict__ act,
                                                          const uint32_t* __restrict__ dz, uint32_t n, uint32_t chunk,
                                                          float* grad) {
    const int l = blockIdx.y;
    const int K = in_dim(l), O = out_dim(l), Opad = bwd_out_pad(l);
    const int aoff = l == 0 ? 0 : kNrcIn + (l - 1) * kNrcHidden;     // BF16 column of H_l
    const int doff = l == 5 ? kNrcHiddenLayers * kNrcHidden : l * kNrcHidden;  // BF16 column of dZ_{l+1}
    __shared__ __align__(16) __nv_bfloat16 sa[kWgTile][kWgRow], sd[kWgTile][kWgRow];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const bool active = warp * 16 < Opad;
    float acc[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
    const uint32_t m0 = blockIdx.x * chunk, m1 = min(n, m0 + chunk);
    for (uint32_t mb = m0; mb < m1; mb += kWgTile) {
        // stage 64 samples: H_l (K columns) and dZ (Opad columns), 16-byte pieces
        for (int e = threadIdx.x; e < kWgTile * 8; e += blockDim.x) {
            const int r = e >> 3, c8 = (e & 7) * 8;
            const uint32_t m = mb + r;
            uint4 va = make_uint4(0u, 0u, 0u, 0u), vd = va;
            if (m < m1) {
                if (c8 < K) va = *reinterpret_cast<const uint4*>(act + (size_t)m * (kTActStride / 2) + (aoff + c8) / 2);
                if (c8 < Opad) vd = *reinterpret_cast<const uint4*>(dz + (size_t)m * (kTGradStride / 2) + (doff + c8) / 2);
            }
            *reinterpret_cast<uint4*>(&sa[r][c8]) = va;
            *reinterpret_cast<uint4*>(&sd[r][c8]) = vd;
        }
        __syncthreads();
        if (active) {
#pragma unroll
            for (int ks = 0; ks < kWgTile / 16; ++ks) {
                // A = dZ^T (rows o, cols m): 8x8 blocks (m0, o0), (m0, o0+8), (m0+8, o0), (m0+8, o0+8)
                const int mi = lane & 7, mat = lane >> 3;
                uint32_t af[4];
                ldsm_x4_trans(af, &sd[ks * 16 + (mat >> 1) * 8 + mi][warp * 16 + (mat & 1) * 8]);
                const uint32_t afr[4] = {af[0], af[1], af[2], af[3]};
#pragma unroll
                for (int np = 0; np < 4; ++np) {
                    if (np * 16 >= K) break;
                    // B = H (rows m, cols k): blocks (m0, k0), (m0+8, k0), (m0, k0+8), (m0+8, k0+8)
                    uint32_t bf[4];
                    ldsm_x4_trans(bf, &sa[ks * 16 + (mat & 1) * 8 + mi][np * 16 + (mat >> 1) * 8]);
                    mma_bf16(acc[2 * np], afr, bf[0], bf[1]);
                    mma_bf16(acc[2 * np + 1], afr, bf[2], bf[3]);
                }
            }
        }
        __syncthreads();
    }
    if (!active) return;
    float* gw = grad + f32_off(l);
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const int k = nt * 8 + 2 * t;
        if (k >= K) break;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int o = warp * 16 + g + 8 * h;
            if (o >= O) continue;
            if (acc[nt][2 * h] != 0.0f) atomicAdd(gw + o * K + k, acc[nt][2 * h]);
            if (acc[nt][2 * h + 1] != 0.0f) atomicAdd(gw + o * K + k + 1, acc[nt][2 * h + 1]);
        }
    }
}

struct AdamCfg {
    float lr, b1, b2, eps, c1, c2;  // c1 = 1 / (1 - b1^t), c2 = 1 / (1 - b2^t)
};

GB_D float adam_one(float& w, float g, float& m, float& v, const AdamCfg& a) {
    m = a.b1 * m + (1.0f - a.b1) * g;
    v = a.b2 * v + (1.0f - a.b2) * g * g;
    w = w - a.lr * (m * a.c1) / (sqrtf(v * a.c2) + a.eps);
    return w;
}

// Adam over the table: thread i updates entry i (both features) and its
// half2 copy.
__global__ void nrc_adam_grid_kernel(float2* w, const float2* g, float2* m, float2* v, uint32_t n, AdamCfg a,
                                     __half2* grid_h) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float2 wi = w[i], mi = m[i], vi = v[i];
    const float2 gi = g[i];
    adam_one(wi.x, gi.x, mi.x, vi.x, a);
    adam_one(wi.y, gi.y, mi.y, vi.y, a);
    w[i] = wi;
    m[i] = mi;
    v[i] = vi;
    grid_h[i] = __floats2half2_rn(wi.x, wi.y);
}

// Adam over the MLP and its padded BF16 copy.
__global__ void nrc_adam_mlp_kernel(float* w, const float* g, float* m, float* v, AdamCfg a, __nv_bfloat16* mlp_h) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kNrcMlpParams) return;
    float wi = w[i], mi = m[i], vi = v[i];
    adam_one(wi, g[i], mi, vi, a);
    w[i] = wi;
    m[i] = mi;
    v[i] = vi;
    int l = 0;
    while (l < 5 && i >= f32_off(l + 1)) ++l;
    const int K = in_dim(l), r = (i - f32_off(l)) / K, c = (i - f32_off(l)) % K;
    mlp_h[bf16_off(l) + r * (K + kPadK) + c] = __float2bfloat16_rn(wi);
}

// FP16 / BF16 copies of the masters (after init or a parameter upload).
__global__ void nrc_copy_kernel(const float* grid_w, uint32_t ngrid2, __half2* grid_h, const float* mlp_w,
                                __nv_bfloat16* mlp_h) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ngrid2) grid_h[i] = __floats2half2_rn(grid_w[2 * i], grid_w[2 * i + 1]);
    if (i < (uint32_t)kNrcMlpParams) {
        int l = 0;
        while (l < 5 && (int)i >= f32_off(l + 1)) ++l;
        const int K = in_dim(l), r = ((int)i - f32_off(l)) / K, c = ((int)i - f32_off(l)) % K;
        mlp_h[bf16_off(l) + r * (K + kPadK) + c] = __float2bfloat16_rn(mlp_w[i]);
    }
}

}  // namespace gbrt

// --- host side ---------------------------------------------------------------
using gbrt_host::DevBuf;
using gbrt_host::DeviceGuard;
using gbrt_host::fail;
using gbrt_host::jobs_outstanding;

struct gbrt_nrc {
    gbrt_ctx* ctx = nullptr;
    DevBuf f_query, f_qout, f_snap_pos, f_snap_rad, f_snap_tp, f_train_pos, f_train_tgt, f_counts;
    uint32_t f_cap = 0, f_train_max = 0;
    gbrt_nrc_config cfg{};
    NrcView view{};
    uint32_t nentries = 0;  // levels * table
    DevBuf grid_w, grid_h, grid_g, grid_m, grid_v;
    DevBuf mlp_w, mlp_h, mlp_g, mlp_m, mlp_v;
    DevBuf act, dz, loss, io_a, io_b;
    DevBuf mlp_tc, status;  // BF16 weights in tcgen05 core-matrix order; query status word
    DevBuf mlp_bt;          // transposed BF16 weights of the tensor-core backward pass
    uint32_t step = 0;
    int infer_blocks = 0, tc_blocks = 0, train_blocks = 0;
};

namespace {

int nrc_setup_view(gbrt_nrc* r) {
    const gbrt_nrc_config& c = r->cfg;
    NrcView& v = r->view;
    v.table = 1u << c.log2_table;
    for (int l = 0; l < kNrcLevels; ++l) {
        const double s = (double)c.base_resolution * std::pow((double)c.growth, (double)l) - 1.0;
        v.lv[l].scale = (float)s;
        const double res = std::ceil((double)(float)s) + 2.0;
        v.lv[l].res = res * res * res <= (double)v.table ? (uint32_t)res : 0u;
    }
    v.lo = make_float3(c.box_lo[0], c.box_lo[1], c.box_lo[2]);
    v.inv_ext = make_float3(1.0f / (c.box_hi[0] - c.box_lo[0]), 1.0f / (c.box_hi[1] - c.box_lo[1]),
                            1.0f / (c.box_hi[2] - c.box_lo[2]));
    v.grid_w = r->grid_w.as<float>();
    v.grid_h = r->grid_h.as<__half2>();
    v.mlp_w = r->mlp_w.as<float>();
    v.mlp_h = r->mlp_h.as<__nv_bfloat16>();
    return GBRT_OK;
}

cudaError_t nrc_refresh_copies(gbrt_nrc* r, cudaStream_t st) {
    const uint32_t n = std::max<uint32_t>(r->nentries, kNrcMlpParams);
    nrc_copy_kernel<<<(n + 255) / 256, 256, 0, st>>>(r->grid_w.as<float>(), r->nentries, r->grid_h.as<__half2>(),
                                                     r->mlp_w.as<float>(), r->mlp_h.as<__nv_bfloat16>());
    nrc_tc_weights_kernel<<<(kTcWElems + 255) / 256, 256, 0, st>>>(r->mlp_w.as<float>(), r->mlp_tc.as<__nv_bfloat16>());
    nrc_bwd_weights_kernel<<<(kBwdElems + 255) / 256, 256, 0, st>>>(r->mlp_w.as<float>(), r->mlp_bt.as<__nv_bfloat16>());
    return cudaGetLastError();
}

bool train_fp32(const gbrt_nrc* r) { return (r->cfg.flags & GBRT_NRC_TRAIN_FP32) != 0; }

cudaError_t nrc_reserve_batch(gbrt_nrc* r, uint32_t n) {
    const size_t a = train_fp32(r) ? (size_t)n * kActStride * 4 : (size_t)n * kTActStride * 2;
    const size_t d = train_fp32(r) ? (size_t)n * kGradStride * 4 : (size_t)n * kTGradStride * 2;
    cudaError_t e = r->act.reserve(a);
    if (e == cudaSuccess) e = r->dz.reserve(d);
    return e;
}

// Gradients of the mean loss over n samples (device arrays) into grid_g / mlp_g.
cudaError_t nrc_gradients(gbrt_nrc* r, const float4* pos, const float4* target, uint32_t n, cudaStream_t st) {
    cudaError_t e = nrc_reserve_batch(r, n);
    if (e != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(r->grid_g.p, 0, r->grid_g.bytes, st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(r->mlp_g.p, 0, r->mlp_g.bytes, st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(r->loss.p, 0, 4, st)) != cudaSuccess) return e;
    if (!train_fp32(r)) {
        NrcTcGrad g{r->grid_g.as<float>(), r->loss.as<float>(), r->act.as<uint32_t>(), r->dz.as<uint32_t>()};
        const uint32_t tiles = (n + 31) / 32;
        const uint32_t blocks = std::min<uint32_t>((tiles + kTrainWarps - 1) / kTrainWarps, (uint32_t)r->train_blocks);
        nrc_train_tc_kernel<<<blocks, kTrainWarps * 32, kTrainTcSmem, st>>>(
            r->view, g, r->mlp_bt.as<__nv_bfloat16>(), pos, target, n, 1.0f / (float)n);
        // 512-sample chunks: 768 blocks for a 2^16 batch, about 5 per SM
        const uint32_t chunk = 512, splits = (n + chunk - 1) / chunk;
        nrc_wgrad_tc_kernel<<<dim3(splits, 6), 128, 0, st>>>(r->act.as<uint32_t>(), r->dz.as<uint32_t>(), n, chunk,
                                                             r->mlp_g.as<float>());
        return cudaGetLastError();
    }
    NrcGrad g{r->grid_g.as<float>(), r->mlp_g.as<float>(), r->act.as<float>(), r->dz.as<float>(), r->loss.as<float>()};
    nrc_train_kernel<<<(n + 127) / 128, 128, kTrainSmem, st>>>(r->view, g, pos, target, n, 1.0f / (float)n);
    const uint32_t chunk = 1024, splits = (n + chunk - 1) / chunk;
    nrc_wgrad_kernel<<<dim3(splits, 6), 256, 0, st>>>(r->act.as<float>(), r->dz.as<float>(), n, chunk,
                                                      r->mlp_g.as<float>());
    return cudaGetLastError();
}

cudaError_t nrc_adam(gbrt_nrc* r, cudaStream_t st) {
    ++r->step;
    AdamCfg a;
    a.b1 = 0.9f;
    a.b2 = 0.99f;
    a.eps = 1e-15f;
    a.c1 = (float)(1.0 / (1.0 - std::pow(0.9, (double)r->step)));
    a.c2 = (float)(1.0 / (1.0 - std::pow(0.99, (double)r->step)));
    a.lr = r->cfg.learning_rate;
    const uint32_t ne = r->nentries;
    nrc_adam_grid_kernel<<<(ne + 255) / 256, 256, 0, st>>>(r->grid_w.as<float2>(), r->grid_g.as<float2>(),
                                                          r->grid_m.as<float2>(), r->grid_v.as<float2>(), ne, a,
                                                          r->grid_h.as<__half2>());
    nrc_adam_mlp_kernel<<<(kNrcMlpParams + 255) / 256, 256, 0, st>>>(r->mlp_w.as<float>(), r->mlp_g.as<float>(),
                                                                     r->mlp_m.as<float>(), r->mlp_v.as<float>(), a,
                                                                     r->mlp_h.as<__nv_bfloat16>());
    nrc_tc_weights_kernel<<<(kTcWElems + 255) / 256, 256, 0, st>>>(r->mlp_w.as<float>(), r->mlp_tc.as<__nv_bfloat16>());
    nrc_bwd_weights_kernel<<<(kBwdElems + 255) / 256, 256, 0, st>>>(r->mlp_w.as<float>(), r->mlp_bt.as<__nv_bfloat16>());
    return cudaGetLastError();
}

}  // namespace

namespace gbrt_host {

namespace {
// Shared-memory opt-in of the two kernels above 48 KB and the query grid.
cudaError_t nrc_kernel_setup(gbrt_nrc* r) {
    if (!r->infer_blocks) {
        cudaError_t e = cudaFuncSetAttribute(nrc_infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)kInferSmem);
        if (e != cudaSuccess) return e;
        e = cudaFuncSetAttribute(nrc_train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTrainSmem);
        if (e != cudaSuccess) return e;
        e = cudaFuncSetAttribute(nrc_train_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTrainTcSmem);
        if (e != cudaSuccess) return e;
        int sms = 0, per = 0, dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, nrc_infer_kernel, 128, kInferSmem);
        r->infer_blocks = sms * std::max(per, 1);
        int per_train = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_train, nrc_train_tc_kernel, kTrainWarps * 32, kTrainTcSmem);
        r->train_blocks = sms * std::max(per_train, 1);
        e = cudaFuncSetAttribute(nrc_infer_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem);
        if (e != cudaSuccess) return e;
        cudaFuncSetAttribute(nrc_infer_tc_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
        // CTAs per SM by shared memory (the occupancy query has reported 1 for this
        // kernel where the launch fits 4), at most 4 x 64 tensor-memory columns
        int smem_sm = 0, smem_rsv = 0, per_tc = 0;
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
        cudaDeviceGetAttribute(&smem_rsv, cudaDevAttrReservedSharedMemoryPerBlock, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_tc, nrc_infer_tc_kernel, 128, kTcSmem);
        per_tc = std::max(per_tc, smem_sm / (int)(kTcSmem + (size_t)smem_rsv));
        r->tc_blocks = sms * std::max(std::min(per_tc, 4), 1);
    }
    return cudaSuccess;
}
}  // namespace

cudaError_t nrc_query_device(gbrt_nrc* r, const float4* q, uint32_t n, float4* out, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    cudaError_t e = nrc_kernel_setup(r);
    if (e != cudaSuccess) return e;
    if (!(r->cfg.flags & GBRT_NRC_QUERY_MMA_SYNC)) {
        const uint32_t need = (n + kTcRows - 1) / kTcRows;
        nrc_infer_tc_kernel<<<std::min<uint32_t>(need, (uint32_t)r->tc_blocks), 128, kTcSmem, st>>>(
            r->view, q, n, out, nullptr, r->mlp_tc.as<__nv_bfloat16>(), r->status.as<uint32_t>());
        return cudaGetLastError();
    }
    const uint32_t need = (n + kInferWarps * 32 - 1) / (kInferWarps * 32);
    nrc_infer_kernel<<<std::min<uint32_t>(need, (uint32_t)r->infer_blocks), 128, kInferSmem, st>>>(r->view, q, n, out,
                                                                                                   nullptr);
    return cudaGetLastError();
}

cudaError_t nrc_query_counted(gbrt_nrc* r, const float4* q, const uint32_t* n_dev, uint32_t n_max, float4* out,
                              cudaStream_t st) {
    cudaError_t e = nrc_kernel_setup(r);
    if (e != cudaSuccess) return e;
    if (!(r->cfg.flags & GBRT_NRC_QUERY_MMA_SYNC))
        nrc_infer_tc_kernel<<<r->tc_blocks, 128, kTcSmem, st>>>(r->view, q, n_max, out, n_dev,
                                                                r->mlp_tc.as<__nv_bfloat16>(),
                                                                r->status.as<uint32_t>());
    else
        nrc_infer_kernel<<<r->infer_blocks, 128, kInferSmem, st>>>(r->view, q, n_max, out, n_dev);
    return cudaGetLastError();
}

cudaError_t nrc_train_device(gbrt_nrc* r, const float4* pos, const float4* target, uint32_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    cudaError_t e = nrc_kernel_setup(r);
    if (e == cudaSuccess) e = nrc_gradients(r, pos, target, n, st);
    if (e == cudaSuccess) e = nrc_adam(r, st);
    return e;
}

const NrcView& nrc_view(const gbrt_nrc* r) { return r->view; }

}  // namespace gbrt_host

using gbrt_host::nrc_query_device;

extern "C" {

int gbrt_nrc_create(gbrt_ctx* c, const gbrt_nrc_config* cfg, gbrt_nrc** out) {
    if (!c || !cfg || !out) return fail(c, GBRT_E_INVALID, "NULL argument");
    *out = nullptr;
    if (cfg->log2_table < 8 || cfg->log2_table > 24 || cfg->base_resolution < 2 || !(cfg->growth >= 1.0f) ||
        !(cfg->learning_rate > 0.0f))
        return fail(c, GBRT_E_INVALID, "bad radiance-cache configuration");
    for (int k = 0; k < 3; ++k)
        if (!(cfg->box_hi[k] > cfg->box_lo[k])) return fail(c, GBRT_E_INVALID, "empty radiance-cache box");
    DeviceGuard g(c->device);
    auto r = new (std::nothrow) gbrt_nrc();
    if (!r) return fail(c, GBRT_E_OOM, "host allocation failed");
    r->ctx = c;
    r->cfg = *cfg;
    r->nentries = (uint32_t)kNrcLevels << cfg->log2_table;
    const size_t ng = (size_t)r->nentries * 2;
    cudaError_t e = cudaSuccess;
    for (DevBuf* b : {&r->grid_w, &r->grid_g, &r->grid_m, &r->grid_v})
        if (e == cudaSuccess) e = b->alloc(ng * 4);
    if (e == cudaSuccess) e = r->grid_h.alloc(ng * 2);
    for (DevBuf* b : {&r->mlp_w, &r->mlp_g, &r->mlp_m, &r->mlp_v})
        if (e == cudaSuccess) e = b->alloc(kNrcMlpParams * 4);
    if (e == cudaSuccess) e = r->mlp_h.alloc(kBf16Padded * 2);
    if (e == cudaSuccess) e = r->mlp_tc.alloc(kTcWElems * 2);
    if (e == cudaSuccess) e = r->mlp_bt.alloc(kBwdElems * 2);
    if (e == cudaSuccess) e = r->status.alloc(4);
    if (e == cudaSuccess) e = r->loss.alloc(4);
    if (e != cudaSuccess) {
        delete r;
        return gbrt_host::cuda_fail(c, e, "radiance-cache buffers");
    }
    nrc_setup_view(r);
    // seeded init: table U(-1e-4, 1e-4), weights U(-sqrt(6 / fan_in), +)
    std::mt19937_64 rng(cfg->seed);
    std::uniform_real_distribution<float> u01(0.0f, 1.0f);
    std::vector<float> hw(ng);
    for (auto& x : hw) x = (u01(rng) * 2.0f - 1.0f) * 1e-4f;
    std::vector<float> hm(kNrcMlpParams);
    for (int l = 0; l < 6; ++l) {
        const float b = std::sqrt(6.0f / (float)in_dim(l));
        for (int i = 0; i < in_dim(l) * out_dim(l); ++i) hm[f32_off(l) + i] = (u01(rng) * 2.0f - 1.0f) * b;
    }
    cudaStream_t st = c->stream;
    e = cudaMemcpyAsync(r->grid_w.p, hw.data(), ng * 4, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(r->mlp_w.p, hm.data(), kNrcMlpParams * 4, cudaMemcpyHostToDevice, st);
    for (DevBuf* b : {&r->grid_m, &r->grid_v, &r->mlp_m, &r->mlp_v})
        if (e == cudaSuccess) e = cudaMemsetAsync(b->p, 0, b->bytes, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(r->mlp_h.p, 0, r->mlp_h.bytes, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(r->status.p, 0, 4, st);
    if (e == cudaSuccess) e = nrc_refresh_copies(r, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        delete r;
        return gbrt_host::cuda_fail(c, e, "radiance-cache init");
    }
    *out = r;
    return GBRT_OK;
}

int gbrt_nrc_destroy(gbrt_nrc* r) {
    if (!r) return GBRT_OK;
    if (jobs_outstanding(r->ctx)) return fail(r->ctx, GBRT_E_BUSY, "jobs are running on this context");
    DeviceGuard g(r->ctx->device);
    cudaStreamSynchronize(r->ctx->stream);
    delete r;
    return GBRT_OK;
}

int gbrt_nrc_params(gbrt_nrc* r, float* mlp, float* grid, int upload) {
    if (!r) return GBRT_E_INVALID;
    gbrt_ctx* c = r->ctx;
    if (jobs_outstanding(c)) return fail(c, GBRT_E_BUSY, "jobs are running on this context");
    DeviceGuard g(c->device);
    cudaStream_t st = c->stream;
    const size_t ng = (size_t)r->nentries * 2 * 4;
    const cudaMemcpyKind k = upload ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost;
    if (mlp) CU(c, cudaMemcpyAsync(upload ? r->mlp_w.p : mlp, upload ? (void*)mlp : r->mlp_w.p, kNrcMlpParams * 4, k, st), "params");
    if (grid) CU(c, cudaMemcpyAsync(upload ? r->grid_w.p : grid, upload ? (void*)grid : r->grid_w.p, ng, k, st), "params");
    if (upload) CU(c, nrc_refresh_copies(r, st), "copies");
    CU(c, cudaStreamSynchronize(st), "sync");
    return GBRT_OK;
}

int gbrt_nrc_query(gbrt_nrc* r, const float* pos4, uint32_t n, float* out4) {
    if (!r) return GBRT_E_INVALID;
    gbrt_ctx* c = r->ctx;
    if (jobs_outstanding(c)) return fail(c, GBRT_E_BUSY, "jobs are running on this context");
    if (n && (!pos4 || !out4)) return fail(c, GBRT_E_INVALID, "NULL argument");
    DeviceGuard g(c->device);
    cudaStream_t st = c->stream;
    CU(c, r->io_a.reserve((size_t)n * 16), "cudaMalloc");
    CU(c, r->io_b.reserve((size_t)n * 16), "cudaMalloc");
    CU(c, cudaMemcpyAsync(r->io_a.p, pos4, (size_t)n * 16, cudaMemcpyHostToDevice, st), "upload");
    CU(c, nrc_query_device(r, r->io_a.as<float4>(), n, r->io_b.as<float4>(), st), "query");
    CU(c, cudaMemcpyAsync(out4, r->io_b.p, (size_t)n * 16, cudaMemcpyDeviceToHost, st), "download");
    uint32_t status = 0;
    CU(c, cudaMemcpyAsync(&status, r->status.p, 4, cudaMemcpyDeviceToHost, st), "download");
    CU(c, cudaStreamSynchronize(st), "sync");
    if (status) return fail(c, GBRT_E_DEVICE_LIMIT, "a tensor-core wait of the cache query timed out");
    return GBRT_OK;
}

int gbrt_nrc_query_device(gbrt_nrc* r, const float* pos4_dev, uint32_t n, float* out4_dev, float* device_ms) {
    if (!r) return GBRT_E_INVALID;
    gbrt_ctx* c = r->ctx;
    if (jobs_outstanding(c)) return fail(c, GBRT_E_BUSY, "jobs are running on this context");
    if (n && (!pos4_dev || !out4_dev)) return fail(c, GBRT_E_INVALID, "NULL argument");
    if (((uintptr_t)pos4_dev | (uintptr_t)out4_dev) & 15u) return fail(c, GBRT_E_INVALID, "buffers must be 16-byte aligned");
    DeviceGuard g(c->device);
    cudaStream_t st = c->stream;
    CU(c, cudaEventRecord(c->ev0, st), "event");
    if (n) CU(c, nrc_query_device(r, reinterpret_cast<const float4*>(pos4_dev), n, reinterpret_cast<float4*>(out4_dev), st),
              "query");
    CU(c, cudaEventRecord(c->ev1, st), "event");
    uint32_t status = 0;
    CU(c, cudaMemcpyAsync(&status, r->status.p, 4, cudaMemcpyDeviceToHost, st), "download");
    CU(c, cudaStreamSynchronize(st), "sync");
    if (device_ms) CU(c, cudaEventElapsedTime(device_ms, c->ev0, c->ev1), "event time");
    if (status) return fail(c, GBRT_E_DEVICE_LIMIT, "a tensor-core wait of the cache query timed out");
    return GBRT_OK;
}

int gbrt_nrc_train(gbrt_nrc* r, const float* pos4, const float* target4, uint32_t n, int step, float* loss,
                   float* grad_mlp, float* grad_grid) {
    if (!r) return GBRT_E_INVALID;
    gbrt_ctx* c = r->ctx;
    if (jobs_outstanding(c)) return fail(c, GBRT_E_BUSY, "jobs are running on this context");
    if (n == 0 || !pos4 || !target4) return fail(c, GBRT_E_INVALID, "empty batch or NULL argument");
    DeviceGuard g(c->device);
    cudaStream_t st = c->stream;
    CU(c, r->io_a.reserve((size_t)n * 16), "cudaMalloc");
    CU(c, r->io_b.reserve((size_t)n * 16), "cudaMalloc");
    CU(c, cudaMemcpyAsync(r->io_a.p, pos4, (size_t)n * 16, cudaMemcpyHostToDevice, st), "upload");
    CU(c, cudaMemcpyAsync(r->io_b.p, target4, (size_t)n * 16, cudaMemcpyHostToDevice, st), "upload");
    CU(c, gbrt_host::nrc_kernel_setup(r), "radiance-cache kernel setup");
    CU(c, nrc_gradients(r, r->io_a.as<float4>(), r->io_b.as<float4>(), n, st), "gradients");
    if (grad_mlp) CU(c, cudaMemcpyAsync(grad_mlp, r->mlp_g.p, kNrcMlpParams * 4, cudaMemcpyDeviceToHost, st), "download");
    if (grad_grid)
        CU(c, cudaMemcpyAsync(grad_grid, r->grid_g.p, (size_t)r->nentries * 8, cudaMemcpyDeviceToHost, st), "download");
    if (loss) CU(c, cudaMemcpyAsync(loss, r->loss.p, 4, cudaMemcpyDeviceToHost, st), "download");
    if (step) CU(c, nrc_adam(r, st), "adam");
    CU(c, cudaStreamSynchronize(st), "sync");
    return GBRT_OK;
}

}  // extern "C"

namespace gbrt_host {

// One frame with the cache on stream st: traces into out (its accumulation,
// image and counters) with the wavefront buffers of wf (frame_sum sized for
// out, cap paths per wave), then runs opts.train_steps Adam steps on the
// frame's training samples.  Host-synchronises once, for the number of
// training samples.  *what names the failed step.
cudaError_t nrc_frame(gbrt_nrc* r, const DevScene& view, const gbrt_ubo& ubo, const RenderOut& out, const WfState& wf,
                      const gbrt_nrc_render_opts& opts, cudaStream_t st, float* loss, const char** what) {
    const uint64_t paths = (uint64_t)out.width * out.height * ubo.number_of_samples;
    const uint32_t cap = (uint32_t)std::min<uint64_t>(std::min<uint64_t>(paths, wf.cap), kMaxWavePaths);
    const uint32_t tmax = std::max<uint32_t>(opts.train_samples, 1u) * 2u;  // room for the hash's spread
    cudaError_t e = cudaSuccess;
    *what = "cudaMalloc(cache frame buffers)";
    if (r->f_cap < cap) {
        for (DevBuf* b : {&r->f_query, &r->f_qout, &r->f_snap_pos, &r->f_snap_rad, &r->f_snap_tp})
            if ((e = b->alloc((size_t)cap * sizeof(float4))) != cudaSuccess) return e;
        r->f_cap = cap;
    }
    if (r->f_train_max < tmax) {
        if ((e = r->f_train_pos.alloc((size_t)tmax * sizeof(float4))) != cudaSuccess) return e;
        if ((e = r->f_train_tgt.alloc((size_t)tmax * sizeof(float4))) != cudaSuccess) return e;
        r->f_train_max = tmax;
    }
    if ((e = r->f_counts.reserve(64 * sizeof(uint32_t))) != cudaSuccess) return e;
    NrcWave nw{};
    nw.query = r->f_query.as<float4>();
    nw.qout = r->f_qout.as<float4>();
    nw.snap_pos = r->f_snap_pos.as<float4>();
    nw.snap_rad = r->f_snap_rad.as<float4>();
    nw.snap_tp = r->f_snap_tp.as<float4>();
    nw.train_pos = r->f_train_pos.as<float4>();
    nw.train_tgt = r->f_train_tgt.as<float4>();
    nw.counts = r->f_counts.as<uint32_t>();
    nw.train_max = r->f_train_max;
    const double frac = std::min(1.0, (double)opts.train_samples / (double)paths);
    nw.train_thresh = (uint32_t)std::min(65536.0, std::ceil(frac * 65536.0));
    nw.min_roughness = opts.min_roughness;
    nw.disabled = opts.disabled ? 1u : 0u;
    nw.mode = opts.mode;
    WfState w = wf;
    w.cap = cap;
    *what = "wavefront launch";
    if ((e = cudaMemsetAsync(nw.counts + 32, 0, sizeof(uint32_t), st)) != cudaSuccess) return e;
    if ((e = launch_wavefront(view, ubo, out, w, st, nullptr, &nw, r)) != cudaSuccess) return e;
    uint32_t ntrain = 0;
    *what = "training sample count";
    if ((e = cudaMemcpyAsync(&ntrain, nw.counts + 32, 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
    ntrain = std::min(ntrain, nw.train_max);
    *what = "cache training";
    for (uint32_t k = 0; k < opts.train_steps && ntrain > 0; ++k)
        if ((e = nrc_train_device(r, nw.train_pos, nw.train_tgt, ntrain, st)) != cudaSuccess) return e;
    if (loss) {
        *loss = 0.0f;  // loss of the last step
        if (ntrain > 0 && opts.train_steps)
            if ((e = cudaMemcpyAsync(loss, r->loss.p, 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
    }
    *what = "";
    return cudaSuccess;
}

uint32_t nrc_status(gbrt_nrc* r, cudaStream_t st) {
    uint32_t v = 0;
    if (cudaMemcpyAsync(&v, r->status.p, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return ~0u;
    return v;
}

gbrt_ctx* nrc_ctx(const gbrt_nrc* r) { return r->ctx; }

}  // namespace gbrt_host

extern "C" int gbrt_render_nrc(gbrt_scene* s, gbrt_nrc* r, const gbrt_ubo* ubo, gbrt_accum* acc, uint8_t* out_rgba8,
                               gbrt_stats* stats, const gbrt_nrc_render_opts* opts, float* loss) {
    using namespace gbrt_host;
    if (!s || !r) return GBRT_E_INVALID;
    gbrt_ctx* c = s->ctx;
    if (!ubo || !acc || !opts) return fail(c, GBRT_E_INVALID, "NULL argument");
    if (r->ctx != c || acc->ctx != c) return fail(c, GBRT_E_INVALID, "cache or accumulation of another context");
    if (!s->built) return fail(c, GBRT_E_NOT_BUILT, "build the BLAS and TLAS before rendering");
    if (jobs_outstanding(c)) return fail(c, GBRT_E_BUSY, "jobs are running on this context");
    if (ubo->number_of_samples == 0 || ubo->total_number_of_samples < ubo->number_of_samples)
        return fail(c, GBRT_E_INVALID, "need 0 < number_of_samples <= total_number_of_samples");
    if (ubo->number_of_bounces > 31) return fail(c, GBRT_E_INVALID, "the wavefront form handles at most 31 bounces");
    if (opts->mode > GBRT_NRC_MODE_PRIMARY_INDIRECT) return fail(c, GBRT_E_INVALID, "unknown radiance-cache mode");
    DeviceGuard g(c->device);
    cudaStream_t st = c->stream;
    const uint32_t W = acc->w, H = acc->h, ns = ubo->number_of_samples;
    const size_t npix = (size_t)W * H;
    const uint64_t paths = (uint64_t)npix * ns;
    const uint32_t cap = (uint32_t)std::min<uint64_t>(paths, kMaxWavePaths);
    CU(c, wavefront_reserve(c, cap, npix), "cudaMalloc(wavefront buffers)");
    RenderOut out{};
    out.width = W;
    out.height = H;
    out.accum = acc->buf.as<float4>();
    out.counters = c->counters.as<DeviceCounters>();
    if (out_rgba8) {
        CU(c, c->scratch_img.reserve(npix * 4), "cudaMalloc(image)");
        out.rgba8 = c->scratch_img.as<uchar4>();
    }
    CU(c, cudaMemsetAsync(out.counters, 0, sizeof(DeviceCounters), st), "memset");
    CU(c, cudaEventRecord(c->ev0, st), "event");
    float lsum = 0.0f;
    const char* what = "";
    CU(c, nrc_frame(r, s->view, *ubo, out, c->wf, *opts, st, &lsum, &what), what);
    CU(c, cudaEventRecord(c->ev1, st), "event");
    if (out_rgba8) CU(c, cudaMemcpyAsync(out_rgba8, out.rgba8, npix * 4, cudaMemcpyDeviceToHost, st), "download image");
    DeviceCounters dc;
    CU(c, cudaMemcpyAsync(&dc, out.counters, sizeof(dc), cudaMemcpyDeviceToHost, st), "download counters");
    CU(c, cudaStreamSynchronize(st), "render");
    float ms = 0.0f;
    CU(c, cudaEventElapsedTime(&ms, c->ev0, c->ev1), "event time");
    fill_stats(stats, dc, ms, 0);
    if (loss) *loss = lsum;
    if (dc.status) return fail(c, GBRT_E_DEVICE_LIMIT, "a kernel reported a traversal limit");
    if (nrc_status(r, st)) return fail(c, GBRT_E_DEVICE_LIMIT, "a tensor-core wait of the cache query timed out");
    return GBRT_OK;
}
