// oracle/glsl.h — the subset of GLSL 4.60 value semantics that rustracer's
// shaders use, as plain C++17, so that the shader code in oracle.cpp can be
// written statement by statement like the GLSL it restates.
//
// TEST INFRASTRUCTURE ONLY.  This directory is the CPU oracle that the tests,
// the smoke check and bench.py's CPU-baseline leg compare the CUDA path with.
// Nothing in the shipped library includes, links or calls it.
//
// Rules followed (GLSL 4.60 spec, ch. 8): componentwise arithmetic; mix(x,y,a)
// = x*(1-a)+y*a; normalize(x) = x * inversesqrt(dot(x,x)) with inversesqrt
// computed as 1/sqrt; reflect/refract as defined in 8.5; matrices are
// column-major.  The oracle is compiled with -ffp-contract=off so that no
// multiply-add is fused unless written as std::fma.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <algorithm>

namespace glsl {

// Parity diagnostics (the ORC_DIAG build of the oracle only): every dot
// product, length, refraction root and normalised vector passes through
// diag_round, which moves it by a few ulps in nudge mode -- the size of the
// differences that fused multiply-adds and approximate square roots make on
// the GPU.  Without ORC_DIAG it is the identity.
#ifdef ORC_DIAG
float diag_round(float r);
#else
inline float diag_round(float r) { return r; }
#endif

struct vec2 {
    float x, y;
    vec2() : x(0), y(0) {}
    explicit vec2(float s) : x(s), y(s) {}
    vec2(float a, float b) : x(a), y(b) {}
    float& operator[](int i) { return i == 0 ? x : y; }
    float operator[](int i) const { return i == 0 ? x : y; }
};
struct vec3 {
    float x, y, z;
    vec3() : x(0), y(0), z(0) {}
    explicit vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    vec3(vec2 a, float c) : x(a.x), y(a.y), z(c) {}
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
struct vec4 {
    float x, y, z, w;
    vec4() : x(0), y(0), z(0), w(0) {}
    explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    vec4(vec3 a, float d) : x(a.x), y(a.y), z(a.z), w(d) {}
    vec4(vec2 a, float c, float d) : x(a.x), y(a.y), z(c), w(d) {}
    vec3 xyz() const { return vec3(x, y, z); }
    vec3 rgb() const { return vec3(x, y, z); }
    vec2 xy() const { return vec2(x, y); }
    vec2 zw() const { return vec2(z, w); }
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
};
struct uvec4 {
    uint32_t x, y, z, w;
    uvec4() : x(0), y(0), z(0), w(0) {}
    uvec4(uint32_t a, uint32_t b, uint32_t c, uint32_t d) : x(a), y(b), z(c), w(d) {}
};

// ---- vec2 ----
inline vec2 operator+(vec2 a, vec2 b) { return vec2(a.x + b.x, a.y + b.y); }
inline vec2 operator-(vec2 a, vec2 b) { return vec2(a.x - b.x, a.y - b.y); }
inline vec2 operator*(vec2 a, vec2 b) { return vec2(a.x * b.x, a.y * b.y); }
inline vec2 operator/(vec2 a, vec2 b) { return vec2(a.x / b.x, a.y / b.y); }
inline vec2 operator*(vec2 a, float s) { return vec2(a.x * s, a.y * s); }
inline vec2 operator*(float s, vec2 a) { return vec2(s * a.x, s * a.y); }
inline vec2 operator+(vec2 a, float s) { return vec2(a.x + s, a.y + s); }
inline vec2 operator-(vec2 a, float s) { return vec2(a.x - s, a.y - s); }
inline float dot(vec2 a, vec2 b) { return a.x * b.x + a.y * b.y; }

// ---- vec3 ----
inline vec3 operator+(vec3 a, vec3 b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(vec3 a, vec3 b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(vec3 a, vec3 b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator/(vec3 a, vec3 b) { return vec3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline vec3 operator*(vec3 a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator*(float s, vec3 a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator/(vec3 a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
inline vec3 operator+(vec3 a, float s) { return vec3(a.x + s, a.y + s, a.z + s); }
inline vec3 operator-(vec3 a, float s) { return vec3(a.x - s, a.y - s, a.z - s); }
inline vec3 operator-(float s, vec3 a) { return vec3(s - a.x, s - a.y, s - a.z); }
inline vec3 operator/(float s, vec3 a) { return vec3(s / a.x, s / a.y, s / a.z); }
inline vec3 operator-(vec3 a) { return vec3(-a.x, -a.y, -a.z); }
inline vec3& operator+=(vec3& a, vec3 b) { a = a + b; return a; }
inline vec3& operator*=(vec3& a, vec3 b) { a = a * b; return a; }
inline vec3& operator*=(vec3& a, float s) { a = a * s; return a; }
inline vec3& operator/=(vec3& a, float s) { a = a / s; return a; }
inline bool operator==(vec3 a, vec3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
inline bool operator!=(vec3 a, vec3 b) { return !(a == b); }
inline float dot(vec3 a, vec3 b) { return diag_round(a.x * b.x + a.y * b.y + a.z * b.z); }
inline vec3 cross(vec3 a, vec3 b) {
    return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
inline float inversesqrt(float x) { return 1.0f / std::sqrt(x); }
inline float length(vec3 a) { return diag_round(std::sqrt(dot(a, a))); }
inline vec3 normalize(vec3 a) {
    const vec3 r = a * inversesqrt(dot(a, a));
    return vec3(diag_round(r.x), diag_round(r.y), diag_round(r.z));
}
inline vec3 min(vec3 a, vec3 b) { return vec3(std::min(a.x, b.x), std::min(a.y, b.y), std::min(a.z, b.z)); }
inline vec3 max(vec3 a, vec3 b) { return vec3(std::max(a.x, b.x), std::max(a.y, b.y), std::max(a.z, b.z)); }
inline vec3 mix(vec3 x, vec3 y, float a) { return x * (1.0f - a) + y * a; }
inline vec3 exp(vec3 a) { return vec3(std::exp(a.x), std::exp(a.y), std::exp(a.z)); }
inline vec3 log(vec3 a) { return vec3(std::log(a.x), std::log(a.y), std::log(a.z)); }
inline vec3 pow(vec3 a, vec3 b) { return vec3(std::pow(a.x, b.x), std::pow(a.y, b.y), std::pow(a.z, b.z)); }
inline vec3 clamp(vec3 a, float lo, float hi) {
    return vec3(std::min(std::max(a.x, lo), hi), std::min(std::max(a.y, lo), hi),
                std::min(std::max(a.z, lo), hi));
}
inline vec3 reflect(vec3 I, vec3 N) { return I - 2.0f * dot(N, I) * N; }
inline vec3 refract(vec3 I, vec3 N, float eta) {
    float d = dot(N, I);
    float k = 1.0f - eta * eta * (1.0f - d * d);
    if (k < 0.0f) return vec3(0.0f);
    return eta * I - (eta * d + diag_round(std::sqrt(k))) * N;
}

// ---- vec4 ----
inline vec4 operator+(vec4 a, vec4 b) { return vec4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline vec4 operator*(vec4 a, vec4 b) { return vec4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
inline vec4 operator*(vec4 a, float s) { return vec4(a.x * s, a.y * s, a.z * s, a.w * s); }
inline vec4 operator*(float s, vec4 a) { return a * s; }
inline vec4 operator-(vec4 a, float s) { return vec4(a.x - s, a.y - s, a.z - s, a.w - s); }
inline vec4& operator*=(vec4& a, vec4 b) { a = a * b; return a; }
inline float dot(vec4 a, vec4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
inline vec4 normalize(vec4 a) { return a * inversesqrt(dot(a, a)); }

// ---- scalar helpers ----
inline float clamp(float x, float lo, float hi) { return std::min(std::max(x, lo), hi); }
inline float mix(float x, float y, float a) { return x * (1.0f - a) + y * a; }
inline float uintBitsToFloat(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
inline uint32_t floatBitsToUint(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
inline int32_t floatBitsToInt(float f) { int32_t u; std::memcpy(&u, &f, 4); return u; }
inline float intBitsToFloat(int32_t u) { float f; std::memcpy(&f, &u, 4); return f; }

// mat4, column-major: m[c*4 + r].  (mat4 * vec4)[r] = sum_c m[c*4+r]*v[c],
// summed left to right.
inline vec4 mul(const float* m, vec4 v) {
    vec4 r;
    for (int i = 0; i < 4; ++i)
        r[i] = m[0 * 4 + i] * v.x + m[1 * 4 + i] * v.y + m[2 * 4 + i] * v.z + m[3 * 4 + i] * v.w;
    return r;
}
// mat4x3 given as a row-major 3x4 (VkTransformMatrixKHR): (M * v)[r] =
// T[r*4+0]*x + T[r*4+1]*y + T[r*4+2]*z + T[r*4+3]*w.
inline vec3 mul34(const float* T, vec4 v) {
    vec3 r;
    for (int i = 0; i < 3; ++i)
        r[i] = T[i * 4 + 0] * v.x + T[i * 4 + 1] * v.y + T[i * 4 + 2] * v.z + T[i * 4 + 3] * v.w;
    return r;
}

}  // namespace glsl
