// vec.cuh — float2/3/4 arithmetic for device code.
//
// Shading code may let the compiler fuse multiply-adds.  Code whose result
// must match the CPU bit for bit (triangle test, alpha test, texture
// filtering on the any-hit path) uses the *_rn helpers at the bottom, which
// are never contracted.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define GB_HD __host__ __device__ __forceinline__
#define GB_D __device__ __forceinline__

GB_HD float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
GB_HD float3 f3(float s) { return make_float3(s, s, s); }
GB_HD float3 f3(float4 a) { return make_float3(a.x, a.y, a.z); }
GB_HD float4 f4(float x, float y, float z, float w) { return make_float4(x, y, z, w); }
GB_HD float4 f4(float3 a, float w) { return make_float4(a.x, a.y, a.z, w); }

GB_HD float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
GB_HD float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
GB_HD float3 operator*(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
GB_HD float3 operator/(float3 a, float3 b) { return f3(a.x / b.x, a.y / b.y, a.z / b.z); }
GB_HD float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
GB_HD float3 operator*(float s, float3 a) { return f3(s * a.x, s * a.y, s * a.z); }
GB_HD float3 operator/(float3 a, float s) { return f3(a.x / s, a.y / s, a.z / s); }
GB_HD float3 operator/(float s, float3 a) { return f3(s / a.x, s / a.y, s / a.z); }
GB_HD float3 operator+(float3 a, float s) { return f3(a.x + s, a.y + s, a.z + s); }
GB_HD float3 operator-(float3 a, float s) { return f3(a.x - s, a.y - s, a.z - s); }
GB_HD float3 operator-(float s, float3 a) { return f3(s - a.x, s - a.y, s - a.z); }
GB_HD float3 operator-(float3 a) { return f3(-a.x, -a.y, -a.z); }
GB_HD float3& operator+=(float3& a, float3 b) { a = a + b; return a; }
GB_HD float3& operator*=(float3& a, float3 b) { a = a * b; return a; }
GB_HD float3& operator*=(float3& a, float s) { a = a * s; return a; }
GB_HD float3& operator/=(float3& a, float s) { a = a / s; return a; }
GB_HD float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
GB_HD float3 cross(float3 a, float3 b) {
    return f3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
GB_HD float3 fmin3(float3 a, float3 b) { return f3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)); }
GB_HD float3 fmax3(float3 a, float3 b) { return f3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)); }
GB_HD float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
GB_HD float3 clamp3(float3 a, float lo, float hi) { return f3(clampf(a.x, lo, hi), clampf(a.y, lo, hi), clampf(a.z, lo, hi)); }
GB_HD float mixf(float x, float y, float a) { return x * (1.0f - a) + y * a; }
GB_HD float3 mix3(float3 x, float3 y, float a) { return x * (1.0f - a) + y * a; }
GB_HD float len3(float3 a) { return sqrtf(dot(a, a)); }
GB_HD float3 normalize3(float3 a) { return a * (1.0f / sqrtf(dot(a, a))); }
GB_HD float4 operator*(float4 a, float4 b) { return f4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
GB_HD float4 operator*(float4 a, float s) { return f4(a.x * s, a.y * s, a.z * s, a.w * s); }
GB_HD float4 operator+(float4 a, float4 b) { return f4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
GB_HD float4 normalize4(float4 a) {
    float s = 1.0f / sqrtf(a.x * a.x + a.y * a.y + a.z * a.z + a.w * a.w);
    return a * s;
}
GB_HD float luminance(float3 c) { return dot(c, f3(0.2126f, 0.7152f, 0.0722f)); }
GB_HD float3 reflect3(float3 I, float3 N) { return I - 2.0f * dot(N, I) * N; }
GB_HD float3 refract3(float3 I, float3 N, float eta) {
    float d = dot(N, I);
    float k = 1.0f - eta * eta * (1.0f - d * d);
    if (k < 0.0f) return f3(0.0f);
    return eta * I - (eta * d + sqrtf(k)) * N;
}
GB_HD bool is_zero3(float3 a) { return a.x == 0.0f && a.y == 0.0f && a.z == 0.0f; }

// column-major mat4 * vec4, summed left to right
GB_HD float4 mat4_mul(const float* m, float4 v) {
    return f4(m[0] * v.x + m[4] * v.y + m[8] * v.z + m[12] * v.w,
              m[1] * v.x + m[5] * v.y + m[9] * v.z + m[13] * v.w,
              m[2] * v.x + m[6] * v.y + m[10] * v.z + m[14] * v.w,
              m[3] * v.x + m[7] * v.y + m[11] * v.z + m[15] * v.w);
}

#ifdef __CUDACC__
// --- never-contracted arithmetic ------------------------------------------
GB_D float mul_rn(float a, float b) { return __fmul_rn(a, b); }
GB_D float add_rn(float a, float b) { return __fadd_rn(a, b); }
GB_D float sub_rn(float a, float b) { return __fsub_rn(a, b); }
// column-major mat4 * vec4, unfused, summed left to right
GB_D float4 mat4_mul_rn(const float* m, float4 v) {
    float r[4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
        r[i] = add_rn(add_rn(add_rn(mul_rn(m[i], v.x), mul_rn(m[4 + i], v.y)), mul_rn(m[8 + i], v.z)),
                      mul_rn(m[12 + i], v.w));
    return make_float4(r[0], r[1], r[2], r[3]);
}
GB_D float dot3_rn(float3 a, float3 b) { return add_rn(add_rn(mul_rn(a.x, b.x), mul_rn(a.y, b.y)), mul_rn(a.z, b.z)); }
// normalize(v) = v * (1 / sqrt(dot(v, v))), every step IEEE-rounded
GB_D float3 normalize3_rn(float3 v) {
    const float s = __fdiv_rn(1.0f, __fsqrt_rn(dot3_rn(v, v)));
    return make_float3(mul_rn(v.x, s), mul_rn(v.y, s), mul_rn(v.z, s));
}
// row-major 3x4 transform of (v, w), ((a*x + b*y) + c*z) + d*w, unfused
GB_D float3 xform34_rn(const float* T, float3 v, float w) {
    float3 r;
    r.x = add_rn(add_rn(add_rn(mul_rn(T[0], v.x), mul_rn(T[1], v.y)), mul_rn(T[2], v.z)), mul_rn(T[3], w));
    r.y = add_rn(add_rn(add_rn(mul_rn(T[4], v.x), mul_rn(T[5], v.y)), mul_rn(T[6], v.z)), mul_rn(T[7], w));
    r.z = add_rn(add_rn(add_rn(mul_rn(T[8], v.x), mul_rn(T[9], v.y)), mul_rn(T[10], v.z)), mul_rn(T[11], w));
    return r;
}
#endif
