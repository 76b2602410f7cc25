// nrc.cuh — the neural radiance cache (hash-grid encoding + 5x64 MLP):
// parameter layout and the encoding shared by inference, training and the
// path tracer.
//
// Encoding: multiresolution hash grid (Mueller et al. 2022) over the position
// normalised to the scene box: 16 levels, 2^log2_table entries of 2 features
// per level; level l has scale s_l = base * growth^l - 1, a point p in
// [0,1]^3 maps to g = p * s_l + 0.5, its cell floor(g) and trilinear weights
// from g - floor(g); a level with (ceil(s_l) + 2)^3 <= table entries is
// indexed densely (x + y r + z r^2, r = ceil(s_l) + 2), the others by the
// spatial hash (x * 1) ^ (y * 2654435761) ^ (z * 805459861) mod table.
// MLP: 32 -> 64 -> 64 -> 64 -> 64 -> 64 -> 3, ReLU after the five hidden
// layers, no biases, linear output; weights W_l stored [out][in].
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "vec.cuh"

namespace gbrt {

constexpr int kNrcLevels = 16;
constexpr int kNrcFeat = 2;
constexpr int kNrcIn = kNrcLevels * kNrcFeat;  // 32
constexpr int kNrcHidden = 64;
constexpr int kNrcHiddenLayers = 5;
constexpr int kNrcOut = 3;
// FP32 master weights: W0 [64][32], W1..W4 [64][64], W5 [3][64]
constexpr int kNrcW0 = 0;
constexpr int kNrcWh = kNrcHidden * kNrcIn;                      // first 64x64 layer
constexpr int kNrcW5 = kNrcWh + 4 * kNrcHidden * kNrcHidden;     // 18432
constexpr int kNrcMlpParams = kNrcW5 + kNrcOut * kNrcHidden;     // 18624
// BF16 inference copy: same order, W5 padded to [8][64]
constexpr int kNrcMlpBf16 = kNrcW5 + 8 * kNrcHidden;             // 18944

struct NrcLevel {
    float scale;
    uint32_t res;    // dense resolution (ceil(scale) + 2) or 0 = hashed
};

struct NrcView {
    NrcLevel lv[kNrcLevels];
    uint32_t table;      // entries per level (power of two)
    float3 lo, inv_ext;  // scene box: p01 = (x - lo) * inv_ext
    const float* grid_w;          // FP32 master table [level][entry][2]
    const __half2* grid_h;        // FP16 copy for inference
    const float* mlp_w;           // FP32 master weights
    const __nv_bfloat16* mlp_h;   // BF16 copy for inference (tensor cores)
};

GB_D uint32_t nrc_index(const NrcView& v, int l, uint32_t x, uint32_t y, uint32_t z) {
    const uint32_t r = v.lv[l].res;
    if (r) return x + y * r + z * r * r;
    return (x ^ (y * 2654435761u) ^ (z * 805459861u)) & (v.table - 1u);
}

// Corner c (bit 0 = x, 1 = y, 2 = z) of level l for the normalised point p:
// entry index and trilinear weight.
GB_D void nrc_corner(const NrcView& v, int l, float3 p, int c, uint32_t& idx, float& w) {
    const float s = v.lv[l].scale;
    const float gx = fmaf(p.x, s, 0.5f), gy = fmaf(p.y, s, 0.5f), gz = fmaf(p.z, s, 0.5f);
    const float fx = floorf(gx), fy = floorf(gy), fz = floorf(gz);
    const float tx = gx - fx, ty = gy - fy, tz = gz - fz;
    const uint32_t x = (uint32_t)(int)fx + (c & 1), y = (uint32_t)(int)fy + ((c >> 1) & 1),
                   z = (uint32_t)(int)fz + ((c >> 2) & 1);
    w = ((c & 1) ? tx : 1.0f - tx) * (((c >> 1) & 1) ? ty : 1.0f - ty) * (((c >> 2) & 1) ? tz : 1.0f - tz);
    idx = (uint32_t)l * v.table + nrc_index(v, l, x, y, z);
}

GB_D float3 nrc_normalise(const NrcView& v, float3 x) {
    float3 p = f3((x.x - v.lo.x) * v.inv_ext.x, (x.y - v.lo.y) * v.inv_ext.y, (x.z - v.lo.z) * v.inv_ext.z);
    p.x = fminf(fmaxf(p.x, 0.0f), 1.0f);
    p.y = fminf(fmaxf(p.y, 0.0f), 1.0f);
    p.z = fminf(fmaxf(p.z, 0.0f), 1.0f);
    return p;
}

}  // namespace gbrt
