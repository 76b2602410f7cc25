// skin.cu — linear-blend skinning, shaders/AnimationCompute.comp:14-39.
//
// One thread per vertex (the reference dispatches vertex_count/256+1 groups of
// 256, crates/examples/gltf_viewer/src/compute_unit.rs:43).  The blended
// matrix is formed like the shader: w.x*B[j.x] + w.y*B[j.y] + w.z*B[j.z] +
// w.w*B[j.w], then pos = M*(p,1), normal = normalize(M*(n,0)), tangent.xyz =
// normalize(M*(t.xyz,0)) keeping tangent.w.
#include "kernels.h"

namespace gbrt {

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
            m[k] = w[0] * sk.joints[j[0]][k] + w[1] * sk.joints[j[1]][k] + w[2] * sk.joints[j[2]][k] +
                   w[3] * sk.joints[j[3]][k];
        const float4 p = mat4_mul(m, f4(v.pos[0], v.pos[1], v.pos[2], 1.0f));
        v.pos[0] = p.x;
        v.pos[1] = p.y;
        v.pos[2] = p.z;
        const float3 n = normalize3(f3(mat4_mul(m, f4(v.normal[0], v.normal[1], v.normal[2], 0.0f))));
        v.normal[0] = n.x;
        v.normal[1] = n.y;
        v.normal[2] = n.z;
        const float tw = v.tangent[3];
        const float4 t = normalize4(mat4_mul(m, f4(v.tangent[0], v.tangent[1], v.tangent[2], 0.0f)));
        v.tangent[0] = t.x;
        v.tangent[1] = t.y;
        v.tangent[2] = t.z;
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
