// skin.cu — linear-blend skinning, shaders/AnimationCompute.comp:14-39.
//
// One thread per vertex (the reference dispatches vertex_count/256+1 groups of
// 256, crates/examples/gltf_viewer/src/compute_unit.rs:43).  The blended
// matrix is formed like the shader: w.x*B[j.x] + w.y*B[j.y] + w.z*B[j.z] +
// w.w*B[j.w], then pos = M*(p,1), normal = normalize(M*(n,0)), tangent.xyz =
// normalize(M*(t.xyz,0)) keeping tangent.w.  Every operation is rounded on its
// own (no fused multiply-add), so skinned positions -- and the hits on them --
// are bit-identical to the CPU oracle's.
#include "kernels.h"

namespace gbrt {

namespace {
GB_D float4 mat4_mul_exact(const float* m, float4 v) {
    float r[4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
        r[i] = add_rn(add_rn(add_rn(mul_rn(m[i], v.x), mul_rn(m[4 + i], v.y)), mul_rn(m[8 + i], v.z)),
                      mul_rn(m[12 + i], v.w));
    return make_float4(r[0], r[1], r[2], r[3]);
}
GB_D float rsqrt_exact(float d) { return __fdiv_rn(1.0f, __fsqrt_rn(d)); }
}  // namespace

__global__ void __launch_bounds__(256) skin_kernel(const gbrt_vertex* __restrict__ vin, gbrt_vertex* __restrict__ vout,
                                                   uint32_t nv, const gbrt_skin_raw* __restrict__ skins,
                                                   uint32_t nskin) {
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= nv) return;
    gbrt_vertex v = vin[g];
    const int si = v.skin_index;
    if (si >= 0 && (uint32_t)si < nskin) {
        const gbrt_skin_raw& sk = skins[si];
        const float w[4] = {v.weights[0], v.weights[1], v.weights[2], v.weights[3]};
        const uint32_t j[4] = {v.joints[0] & 255u, v.joints[1] & 255u, v.joints[2] & 255u, v.joints[3] & 255u};
        float m[16];
#pragma unroll
        for (int k = 0; k < 16; ++k)
            m[k] = add_rn(add_rn(add_rn(mul_rn(w[0], sk.joints[j[0]][k]), mul_rn(w[1], sk.joints[j[1]][k])),
                                 mul_rn(w[2], sk.joints[j[2]][k])),
                          mul_rn(w[3], sk.joints[j[3]][k]));
        const float4 p = mat4_mul_exact(m, f4(v.pos[0], v.pos[1], v.pos[2], 1.0f));
        v.pos[0] = p.x;
        v.pos[1] = p.y;
        v.pos[2] = p.z;
        const float4 n4 = mat4_mul_exact(m, f4(v.normal[0], v.normal[1], v.normal[2], 0.0f));
        const float ns = rsqrt_exact(add_rn(add_rn(mul_rn(n4.x, n4.x), mul_rn(n4.y, n4.y)), mul_rn(n4.z, n4.z)));
        v.normal[0] = mul_rn(n4.x, ns);
        v.normal[1] = mul_rn(n4.y, ns);
        v.normal[2] = mul_rn(n4.z, ns);
        const float tw = v.tangent[3];
        const float4 t4 = mat4_mul_exact(m, f4(v.tangent[0], v.tangent[1], v.tangent[2], 0.0f));
        const float ts = rsqrt_exact(
            add_rn(add_rn(add_rn(mul_rn(t4.x, t4.x), mul_rn(t4.y, t4.y)), mul_rn(t4.z, t4.z)), mul_rn(t4.w, t4.w)));
        v.tangent[0] = mul_rn(t4.x, ts);
        v.tangent[1] = mul_rn(t4.y, ts);
        v.tangent[2] = mul_rn(t4.z, ts);
        v.tangent[3] = tw;
    }
    vout[g] = v;
}

cudaError_t launch_skinning(const gbrt_vertex* vin, gbrt_vertex* vout, uint32_t nv, const gbrt_skin_raw* skins,
                            uint32_t nskin, cudaStream_t st) {
    if (nv == 0) return cudaSuccess;
    skin_kernel<<<(nv + 255) / 256, 256, 0, st>>>(vin, vout, nv, skins, nskin);
    return cudaGetLastError();
}

}  // namespace gbrt
