// oracle/oracle.cpp — scalar C++17 restatement of rustracer's ray-tracing
// shaders and a reference binned-SAH BVH2, used as the parity oracle and the
// timed CPU baseline.
//
// TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and
// bench.py's CPU-baseline leg load this code.  The CUDA library never links
// it and never falls back to it.
//
// Parity status: UNPINNED.  The reference runs these shaders on a Vulkan
// ray-tracing driver, which cannot run here, and ships no golden vectors;
// traversal and the triangle test live inside the driver.  Every function
// below cites the GLSL (paths relative to
// crates/examples/gltf_viewer/shaders/ unless stated) that it follows
// statement by statement.  GLSL float literals are written with an f suffix
// so that no expression is promoted to double.
//
// Deviations applied identically here and in the CUDA kernels:
//  D1 seeds: per sample s (global sample index) the pixel stream is
//     initRNG(px, size, s), the ray stream initRNG(px, size, TEA(s,
//     0x9E3779B9)) and RandomSeed = TEA(TEA(x, y), s), replacing clockARB()
//     and frame_count (RayTracing.rgen:32-40).
//  D2 closest-hit ties (equal FP32 t) go to the smaller instance id, then the
//     smaller primitive id.
//  D3 BLEND any-hit draws u = uintToFloat(pcg4d(uvec4(px, py, s,
//     blend_hash(instance, prim, tag))).x) instead of consuming the shared
//     rngState in traversal order (RayTracing.rahit:101).
//  D4 textures are filtered in software (bilinear, no mips); cube faces are
//     filtered with clamp-to-edge inside the selected face.
//  D5 the debug==1 legacy branch and the HEAT mapping are outside the parity
//     contract (HEAT renders as RENDER here).
#include "oracle.h"
#include "glsl.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

using namespace glsl;

namespace {

// ---------------------------------------------------------------------------
// Parity diagnostics (not shader semantics), compiled into the ORC_DIAG build
// (liboracle_diag.so) that the tests use; the timed CPU baseline
// (liboracle.so) carries none of it.
//
// A GPU sample can leave the 1e-4 band around the oracle's sample when its
// path meets a decision whose operands sit so close to the threshold that
// ulp-level differences in the arithmetic before it (CUDA's sin/cos/pow/exp/
// log against libm's, approximate divisions and square roots, fused
// multiply-adds) take the other side, or when the
// path amplifies those ulps continuously (a GGX lobe evaluated near its peak
// cancels 1 - NdotH^2).  Per sample the oracle records:
//  - margin[0]: the smallest |operand - threshold| of the decisions taken:
//    Russian roulette (rgen:108-118), BRDF lobe choice (rchit:357-366), RIS
//    acceptance (rchit:109), the light's back-face skip (rchit:98), front-face
//    and outward-normal sides (rchit:189-193), TIR (PBR.glsl:689-692), the
//    facing tests of the indirect sample (PBR.glsl:656) and of the NEE BRDF
//    (PBR.glsl:539-540,737), the rotation's pole case (PBR.glsl:365),
//    MASK/BLEND opacity tests of secondary rays (rahit:98,102), the
//    directional light's side in the miss shader (rmiss:22) and the sky's
//    cube-face choice;
//  - margin[1]: the smallest barycentric coordinate of any secondary hit
//    (distance to the triangle's nearest edge, where a ray nudged by an ulp
//    can hit the neighbour or miss).
// Every operand here is a uniform random number, a probability, a cosine or
// a barycentric, all of unit scale, so the margins are absolute.  Decisions
// between integer-exact quantities (the uniform light pick) come out the same
// on both sides and are not logged.  In nudge mode every transcendental
// result, shading division and square root, dot product, length and
// normalised vector component is moved by +-k ulps
// (sign drawn from a per-sample counter hash): samples that then leave the
// 1e-4 band are ill-conditioned at the ulp level.
// ---------------------------------------------------------------------------
struct SampleDiag {
    float margin[2];
    uint32_t nudge_ulps;
    uint32_t nudge_state;
};
#ifdef ORC_DIAG
thread_local SampleDiag* g_diag = nullptr;
inline void note_margin(float m) {
    if (g_diag) g_diag->margin[0] = std::min(g_diag->margin[0], std::fabs(m));
}
inline void note_edge(float m) {
    if (g_diag) g_diag->margin[1] = std::min(g_diag->margin[1], std::fabs(m));
}
inline float nudged(float r) {
    if (!g_diag || !g_diag->nudge_ulps || !std::isfinite(r)) return r;
    uint32_t h = g_diag->nudge_state = g_diag->nudge_state * 747796405u + 2891336453u;
    h = ((h >> ((h >> 28u) + 4u)) ^ h) * 277803737u;
    const float to = (h >> 31) ? INFINITY : -INFINITY;
    for (uint32_t k = 0; k < g_diag->nudge_ulps; ++k) r = std::nextafter(r, to);
    return r;
}
#else
constexpr SampleDiag* g_diag = nullptr;
inline void note_margin(float) {}
inline void note_edge(float) {}
inline float nudged(float r) { return r; }
#endif
// The shaders' transcendentals, nudged in diagnostics mode.
inline float t_pow(float a, float b) { return nudged(std::pow(a, b)); }
inline float t_sin(float a) { return nudged(std::sin(a)); }
inline float t_cos(float a) { return nudged(std::cos(a)); }
inline vec3 t_exp(vec3 a) { return vec3(nudged(std::exp(a.x)), nudged(std::exp(a.y)), nudged(std::exp(a.z))); }
inline vec3 t_log(vec3 a) { return vec3(nudged(std::log(a.x)), nudged(std::log(a.y)), nudged(std::log(a.z))); }
// The shaders' divisions and square roots, nudged in diagnostics mode like the
// transcendentals: the CUDA shading kernels compute them in approximate forms
// (within 2 ulps).
inline float dv(float a, float b) { return nudged(a / b); }
inline vec3 dv(vec3 a, float b) { return vec3(dv(a.x, b), dv(a.y, b), dv(a.z, b)); }
inline float sq(float a) { return nudged(std::sqrt(a)); }
// Seed of a sample's nudge signs (mixed with the nudge argument: its size in
// the low 16 bits, a draw index above them, so each size and draw has its
// own signs).
inline uint32_t nudge_seed(uint32_t x, uint32_t y, uint32_t s) { return (x * 73856093u) ^ (y * 19349663u) ^ (s * 83492791u) ^ 0x5bd1e995u; }

// ---------------------------------------------------------------------------
// lib/Random.glsl
// ---------------------------------------------------------------------------
// InitRandomSeed, Random.glsl:12-25 (TEA, 16 rounds).
uint32_t InitRandomSeed(uint32_t val0, uint32_t val1) {
    uint32_t v0 = val0, v1 = val1, s0 = 0;
    for (uint32_t n = 0; n < 16; n++) {
        s0 += 0x9e3779b9u;
        v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + s0) ^ ((v1 >> 5) + 0xc8013ea4u);
        v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + s0) ^ ((v0 >> 5) + 0x7e95761eu);
    }
    return v0;
}
// RandomInt / RandomFloat, Random.glsl:27-42.
uint32_t RandomInt(uint32_t& seed) { return (seed = 1664525u * seed + 1013904223u); }
float RandomFloat(uint32_t& seed) {
    return (float(RandomInt(seed) & 0x00FFFFFFu) / float(0x01000000));
}
// RandomInUnitDisk / RandomInUnitSphere, Random.glsl:44-66.  The vec2/vec3
// constructor arguments are evaluated left to right (GLSL 4.60 5.10).
vec2 RandomInUnitDisk(uint32_t& seed) {
    for (;;) {
        float a = RandomFloat(seed);
        float b = RandomFloat(seed);
        const vec2 p = 2.0f * vec2(a, b) - 1.0f;
        if (dot(p, p) < 1.0f) return p;
    }
}
vec3 RandomInUnitSphere(uint32_t& seed) {
    for (;;) {
        float a = RandomFloat(seed);
        float b = RandomFloat(seed);
        float c = RandomFloat(seed);
        const vec3 p = 2.0f * vec3(a, b, c) - 1.0f;
        if (dot(p, p) < 1.0f) return p;
    }
}
// uintToFloat, Random.glsl:70-72.
float uintToFloat(uint32_t x) { return uintBitsToFloat(0x3f800000u | (x >> 9)) - 1.0f; }
// initRNG, Random.glsl:75-77.
uvec4 initRNG(uint32_t px, uint32_t py, uint32_t frame) { return uvec4(px, py, frame, 0u); }
// pcg4d, Random.glsl:81-98.
uvec4 pcg4d(uvec4 v) {
    v.x = v.x * 1664525u + 1013904223u;
    v.y = v.y * 1664525u + 1013904223u;
    v.z = v.z * 1664525u + 1013904223u;
    v.w = v.w * 1664525u + 1013904223u;
    v.x += v.y * v.w;
    v.y += v.z * v.x;
    v.z += v.x * v.y;
    v.w += v.y * v.z;
    v.x ^= v.x >> 16u;
    v.y ^= v.y >> 16u;
    v.z ^= v.z >> 16u;
    v.w ^= v.w >> 16u;
    v.x += v.y * v.w;
    v.y += v.z * v.x;
    v.z += v.x * v.y;
    v.w += v.y * v.z;
    return v;
}
// rand, Random.glsl:102-105.
float rand(uvec4& s) {
    s.w++;
    return uintToFloat(pcg4d(s).x);
}
// jenkinsHash / hashAndColor, Random.glsl:108-125.
uint32_t jenkinsHash(uint32_t x) {
    x += x << 10;
    x ^= x >> 6;
    x += x << 3;
    x ^= x >> 11;
    x += x << 15;
    return x;
}
vec3 hashAndColor(uint32_t i) {
    uint32_t hash = jenkinsHash(i);
    float r = float((hash >> 0) & 0xFFu) / 255.0f;
    float g = float((hash >> 8) & 0xFFu) / 255.0f;
    float b = float((hash >> 16) & 0xFFu) / 255.0f;
    return vec3(r, g, b);
}
// D3: stateless key of one BLEND any-hit draw.
uint32_t blend_hash(uint32_t instance, uint32_t prim, uint32_t tag) {
    return jenkinsHash(jenkinsHash(jenkinsHash(tag) ^ instance) ^ prim);
}

// ---------------------------------------------------------------------------
// lib/PBR.glsl (GGX + Frostbite diffuse configuration, PBR.glsl:56-165)
// ---------------------------------------------------------------------------
constexpr uint32_t DIFFUSE_TYPE = 1, SPECULAR_TYPE = 2, TRANSMISSION_TYPE = 3;
constexpr float PI = 3.141592653589f;
const float ONE_OVER_PI = (1.0f / PI);
const float TWO_PI = (2.0f * PI);
constexpr float OURSIDE_IOR = 1.0f;

struct BrdfData {
    vec3 specularF0, diffuseReflectance, specularF90;
    float roughness, alpha, alphaSquared;
    vec3 F;
    vec3 V, N, H, L;
    float NdotL, NdotV, LdotH, NdotH, VdotH;
    bool Vbackfacing, Lbackfacing;
};

struct MaterialBrdf {
    vec3 baseColor;
    float metallic, roughness, ior, transmission;
    bool use_spec;
    float specular_factor;
    vec3 specular_color_factor, dielectricSpecularF0, dielectricSpecularF90, F0, F90, c_diff;
    bool frontFace;
    vec3 attenuation_color;
    float attenuation_distance;
    bool volume;
    float t_diff;
};

float Schlick(const float cosine, const float refractionIndex) {  // PBR.glsl:48-53
    float r0 = dv(1.0f - refractionIndex, 1.0f + refractionIndex);
    r0 *= r0;
    return r0 + (1.0f - r0) * t_pow(1.0f - cosine, 5.0f);
}

void matBuild(MaterialBrdf& m) {  // PBR.glsl:195-206
    float factor = dv(m.ior - OURSIDE_IOR, m.ior + OURSIDE_IOR);
    m.dielectricSpecularF0 = min(factor * factor * m.specular_color_factor, vec3(1.0f)) * m.specular_factor;
    m.dielectricSpecularF90 = m.specular_color_factor;
    m.F0 = mix(m.dielectricSpecularF0, m.baseColor, m.metallic);
    m.F90 = mix(m.dielectricSpecularF90, vec3(1.0f), m.metallic);
    m.c_diff = mix(m.baseColor, vec3(0.0f), m.metallic);
}

float saturate(float x) { return clamp(x, 0.0f, 1.0f); }  // PBR.glsl:212
float luminance(vec3 rgb) { return dot(rgb, vec3(0.2126f, 0.7152f, 0.0722f)); }  // :221-224

vec3 evalFresnel(vec3 f0, float f90, float NdotS) {  // PBR.glsl:228-243
    return f0 + (f90 - f0) * t_pow(1.0f - NdotS, 5.0f);
}

float Smith_G_a(float alpha, float NdotS) {  // PBR.glsl:248-250
    return dv(NdotS, std::max(0.00001f, alpha) * sq(1.0f - std::min(0.99999f, NdotS * NdotS)));
}
float Smith_G_Lambda_GGX(float a) {  // PBR.glsl:253-255
    return (-1.0f + sq(1.0f + dv(1.0f, a * a))) * 0.5f;
}
float Smith_G2_Height_Correlated(float alpha, float NdotL, float NdotV) {  // :258-262
    float aL = Smith_G_a(alpha, NdotL);
    float aV = Smith_G_a(alpha, NdotV);
    return dv(1.0f, 1.0f + Smith_G_Lambda_GGX(aL) + Smith_G_Lambda_GGX(aV));
}
float GGX_D(float alphaSquared, float NdotH) {  // PBR.glsl:286-289
    float b = ((alphaSquared - 1.0f) * NdotH * NdotH + 1.0f);
    return dv(alphaSquared, PI * b * b);
}
vec3 evalMicrofacet(const BrdfData& d) {  // PBR.glsl:292-303
    float D = GGX_D(std::max(0.00001f, d.alphaSquared), d.NdotH);
    float G2 = Smith_G2_Height_Correlated(d.alpha, d.NdotL, d.NdotV);
    return dv(d.F * G2 * D, 4.0f * d.NdotL * d.NdotV) * d.NdotL;
}
float shadowedF90(const vec3 F90) { return std::min(1.0f, luminance(F90)); }  // :312-322

struct BRDFProb { float specular, diffuse, transmission; };
BRDFProb getBrdfProbability(const MaterialBrdf& mat, vec3 V, vec3 shadingNormal) {  // :324-358
    float specularF0 = luminance(mat.F0);
    float diffuseReflectance = luminance(mat.c_diff);
    float Fresnel = saturate(luminance(evalFresnel(vec3(specularF0), shadowedF90(mat.F90),
                                                   std::max(0.0f, dot(V, shadingNormal)))));
    float specular = Fresnel * mat.specular_factor;
    float penetration = diffuseReflectance * (1.0f - mat.specular_factor * Fresnel);
    float diffuse = penetration * (1.0f - mat.transmission);
    float transmission = penetration * mat.transmission;
    float sum = std::max(0.0001f, (specular + diffuse + transmission));
    float p = dv(specular, sum);
    p = clamp(p, 0.001f, 0.9f);
    float d = (1.0f - p) * (1.0f - mat.transmission);
    float t = (1.0f - p) * mat.transmission;
    sum = p + d + t;
    p = dv(p, sum);
    d = dv(d, sum);
    t = dv(t, sum);
    return {p, d, t};
}

vec4 getRotationToZAxis(vec3 v) {  // PBR.glsl:362-368
    note_margin(v.z + 0.99999f);
    if (v.z < -0.99999f) return vec4(1.0f, 0.0f, 0.0f, 0.0f);
    return normalize(vec4(v.y, -v.x, 0.0f, 1.0f + v.z));
}
vec3 rotatePoint(vec4 q, vec3 v) {  // PBR.glsl:373-376
    const vec3 qAxis = vec3(q.x, q.y, q.z);
    return 2.0f * dot(qAxis, v) * qAxis + (q.w * q.w - dot(qAxis, qAxis)) * v +
           2.0f * q.w * cross(qAxis, v);
}
vec4 invertRotation(vec4 q) { return vec4(-q.x, -q.y, -q.z, q.w); }  // PBR.glsl:580-583

vec3 sampleHemisphere(vec2 u) {  // PBR.glsl:381-394
    float a = sq(u.x);
    float b = TWO_PI * u.y;
    return vec3(a * t_cos(b), a * t_sin(b), sq(1.0f - u.x));
}

vec3 sampleGGXVNDF(vec3 Ve, vec2 alpha2D, vec2 u) {  // PBR.glsl:413-436
    vec3 Vh = normalize(vec3(alpha2D.x * Ve.x, alpha2D.y * Ve.y, Ve.z));
    float lensq = Vh.x * Vh.x + Vh.y * Vh.y;
    vec3 T1 = lensq > 0.0f ? vec3(-Vh.y, Vh.x, 0.0f) * nudged(inversesqrt(lensq)) : vec3(1.0f, 0.0f, 0.0f);
    vec3 T2 = cross(Vh, T1);
    float r = sq(u.x);
    float phi = TWO_PI * u.y;
    float t1 = r * t_cos(phi);
    float t2 = r * t_sin(phi);
    float s = 0.5f * (1.0f + Vh.z);
    t2 = mix(sq(1.0f - t1 * t1), t2, s);
    vec3 Nh = t1 * T1 + t2 * T2 + sq(std::max(0.0f, 1.0f - t1 * t1 - t2 * t2)) * Vh;
    return normalize(vec3(alpha2D.x * Nh.x, alpha2D.y * Nh.y, std::max(0.0f, Nh.z)));
}

float Smith_G1_GGX(float alpha, float NdotS, float alphaSquared, float NdotSSquared) {  // :446-448
    (void)alpha;
    (void)NdotS;
    return dv(2.0f, sq(dv((alphaSquared * (1.0f - NdotSSquared)) + NdotSSquared, NdotSSquared)) + 1.0f);
}
float Smith_G2_Over_G1_Height_Correlated(float alpha, float alphaSquared, float NdotL, float NdotV) {  // :470-474
    float G1V = Smith_G1_GGX(alpha, NdotV, alphaSquared, NdotV * NdotV);
    float G1L = Smith_G1_GGX(alpha, NdotL, alphaSquared, NdotL * NdotL);
    return dv(G1L, G1V + G1L - G1V * G1L);
}
float frostbiteDisneyDiffuse(const BrdfData& d) {  // PBR.glsl:486-496
    float energyBias = 0.5f * d.roughness;
    float energyFactor = mix(1.0f, 1.0f / 1.51f, d.roughness);
    float FD90MinusOne = energyBias + 2.0f * d.LdotH * d.LdotH * d.roughness - 1.0f;
    float FDL = 1.0f + (FD90MinusOne * t_pow(1.0f - d.NdotL, 5.0f));
    float FDV = 1.0f + (FD90MinusOne * t_pow(1.0f - d.NdotV, 5.0f));
    return FDL * FDV * energyFactor;
}
vec3 evalFrostbiteDisneyDiffuse(const BrdfData& d) {  // PBR.glsl:516-518
    return d.diffuseReflectance * (frostbiteDisneyDiffuse(d) * ONE_OVER_PI * d.NdotL);
}

BrdfData prepareBRDFData(vec3 N, vec3 L, vec3 V, const MaterialBrdf& m) {  // PBR.glsl:527-564
    BrdfData d;
    d.V = V;
    d.N = N;
    d.H = normalize(L + V);
    d.L = L;
    // data.Ht (PBR.glsl:535) only feeds specular_btdf, which nothing calls.
    float NdotL = dot(N, L);
    float NdotV = dot(N, V);
    d.Vbackfacing = (NdotV <= 0.0f);
    d.Lbackfacing = (NdotL <= 0.0f);
    d.NdotL = std::min(std::max(0.00001f, NdotL), 1.0f);
    d.NdotV = std::min(std::max(0.00001f, NdotV), 1.0f);
    d.LdotH = saturate(dot(L, d.H));
    d.NdotH = saturate(dot(N, d.H));
    d.VdotH = saturate(dot(V, d.H));
    d.specularF0 = m.F0;
    d.specularF90 = m.F90;
    d.diffuseReflectance = m.c_diff;
    d.roughness = m.roughness;
    d.alpha = m.roughness * m.roughness;
    d.alphaSquared = d.alpha * d.alpha;
    d.F = evalFresnel(d.specularF0, shadowedF90(m.F90), d.VdotH);
    return d;
}

vec3 sampleSpecularMicrofacet(vec3 Vlocal, float alpha, float alphaSquared, vec3 specularF0, vec2 u,
                              vec3& weight, vec3 specularF90) {  // PBR.glsl:587-616
    vec3 Hlocal;
    if (alpha == 0.0f) {
        Hlocal = vec3(0.0f, 0.0f, 1.0f);
    } else {
        Hlocal = sampleGGXVNDF(Vlocal, vec2(alpha, alpha), u);
    }
    vec3 Llocal = reflect(-Vlocal, Hlocal);
    float HdotL = std::max(0.00001f, std::min(1.0f, dot(Hlocal, Llocal)));
    const vec3 Nlocal = vec3(0.0f, 0.0f, 1.0f);
    float NdotL = std::max(0.00001f, std::min(1.0f, dot(Nlocal, Llocal)));
    float NdotV = std::max(0.00001f, std::min(1.0f, dot(Nlocal, Vlocal)));
    (void)std::max(0.00001f, std::min(1.0f, dot(Nlocal, Hlocal)));  // NdotH, unused by the weight
    vec3 F = evalFresnel(specularF0, shadowedF90(specularF90), HdotL);
    weight = F * Smith_G2_Over_G1_Height_Correlated(alpha, alphaSquared, NdotL, NdotV);
    return Llocal;
}

bool evalIndirectCombinedBRDF(vec2 u, vec3 shadingNormal, vec3 geometryNormal, vec3 V,
                              const MaterialBrdf& material, const uint32_t brdfType,
                              vec3& rayDirection, vec3& sampleWeight, float& volume_dis) {  // :649-729
    note_margin(dot(geometryNormal, V));
    if (dot(geometryNormal, V) < 0.0f) return false;
    vec4 qRotationToZ = getRotationToZAxis(shadingNormal);
    vec3 Vlocal = rotatePoint(qRotationToZ, V);
    const vec3 Nlocal = vec3(0.0f, 0.0f, 1.0f);
    vec3 rayDirectionLocal = vec3(0.0f, 0.0f, 0.0f);
    if (brdfType == DIFFUSE_TYPE) {
        rayDirectionLocal = sampleHemisphere(u);
        const BrdfData data = prepareBRDFData(Nlocal, rayDirectionLocal, Vlocal, material);
        sampleWeight = (1.0f - material.specular_factor * data.F) * data.diffuseReflectance *
                       frostbiteDisneyDiffuse(data);
        sampleWeight *= (1.0f - material.transmission);
    } else if (brdfType == SPECULAR_TYPE) {
        const BrdfData data = prepareBRDFData(Nlocal, vec3(0.0f, 0.0f, 1.0f), Vlocal, material);
        rayDirectionLocal = sampleSpecularMicrofacet(Vlocal, data.alpha, data.alphaSquared, data.specularF0,
                                                     u, sampleWeight, data.specularF90);
        sampleWeight *= material.specular_factor;
    } else if (brdfType == TRANSMISSION_TYPE) {
        if (material.volume) {
            const float refraction_ratio = material.frontFace ? dv(1.0f, material.ior) : material.ior;
            const float dn = dot(Nlocal, -Vlocal);
            note_margin(1.0f - refraction_ratio * refraction_ratio * (1.0f - dn * dn));  // refract's k
            const vec3 refracted = refract(-Vlocal, Nlocal, refraction_ratio);
            if (refracted == vec3(0.0f)) {
                sampleWeight = vec3(0.0f);
                return false;
            }
            rayDirectionLocal = refracted;
        } else {
            rayDirectionLocal = -Vlocal;
        }
        const BrdfData data = prepareBRDFData(Nlocal, rayDirectionLocal, Vlocal, material);
        sampleWeight = max(vec3(0.0f), data.diffuseReflectance * material.transmission);
        if (!material.frontFace && material.volume) {
            float dis = volume_dis;
            volume_dis = -1.0f;
            vec3 sigma = dv(t_log(material.attenuation_color), material.attenuation_distance);
            vec3 attenuation = t_exp(sigma * dis);
            sampleWeight *= min(attenuation, vec3(1.0f));
        }
    }
    if (luminance(sampleWeight) == 0.0f) return false;
    rayDirection = normalize(rotatePoint(invertRotation(qRotationToZ), rayDirectionLocal));
    return true;
}

vec3 evalCombinedBRDF(vec3 N, vec3 L, vec3 V, const MaterialBrdf& material) {  // PBR.glsl:731-745
    const BrdfData data = prepareBRDFData(N, L, V, material);
    note_margin(dot(N, L));
    note_margin(dot(N, V));
    if (data.Vbackfacing || data.Lbackfacing) return vec3(0.0f, 0.0f, 0.0f);
    vec3 specular = evalMicrofacet(data);
    vec3 diffuse = evalFrostbiteDisneyDiffuse(data);
    return diffuse + specular;
}

// ---------------------------------------------------------------------------
// lib/Material.glsl, lib/PunctualLight.glsl, lib/Tonemapping.glsl
// ---------------------------------------------------------------------------
constexpr uint32_t SPECULAR_GLOSS_WORKFLOW = 1;
constexpr float c_MinRoughness = 0.04f;
float convertMetallic(vec3 diffuse, vec3 specular, float maxSpecular) {  // Material.glsl:78-89
    float perceivedDiffuse = sq(0.299f * diffuse.x * diffuse.x + 0.587f * diffuse.y * diffuse.y +
                                       0.114f * diffuse.z * diffuse.z);
    float perceivedSpecular = sq(0.299f * specular.x * specular.x + 0.587f * specular.y * specular.y +
                                        0.114f * specular.z * specular.z);
    if (perceivedSpecular < c_MinRoughness) return 0.0f;
    float a = c_MinRoughness;
    float b = dv(perceivedDiffuse * (1.0f - maxSpecular), 1.0f - c_MinRoughness) + perceivedSpecular -
              2.0f * c_MinRoughness;
    float c = c_MinRoughness - perceivedSpecular;
    float D = std::max(b * b - 4.0f * a * c, 0.0f);
    return clamp(dv(-b + sq(D), 2.0f * a), 0.0f, 1.0f);
}

constexpr uint32_t POINT_LIGHT = 1;
vec3 getLightIntensityAtPoint(const gbrt_light_raw& light, float distance) {  // PunctualLight.glsl:17-30
    vec3 color = light.intensity * vec3(light.color[0], light.color[1], light.color[2]);
    if (light.kind == POINT_LIGHT) {
        const float radius = 0.5f;
        const float radiusSquared = radius * radius;
        const float distanceSquared = distance * distance;
        const float attenuation =
            dv(2.0f, distanceSquared + radiusSquared + distance * sq(distanceSquared + radiusSquared));
        return color * attenuation;
    }
    return color;
}

const float INV_GAMMA = 1.0f / 2.2f;  // Tonemapping.glsl:6-7
vec3 LINEARtoSRGB(vec3 c) { return pow(c, vec3(INV_GAMMA)); }
vec3 toneMapUncharted2Impl(vec3 color) {  // Tonemapping.glsl:15-23
    const float A = 0.15f, B = 0.50f, C = 0.10f, D = 0.20f, E = 0.02f, F = 0.30f;
    return ((color * (A * color + C * B) + D * E) / (color * (A * color + B) + D * F)) - E / F;
}
vec3 toneMapUncharted(vec3 color) {  // Tonemapping.glsl:25-30
    const float W = 11.2f;
    color = toneMapUncharted2Impl(color * 2.0f);
    vec3 whiteScale = 1.0f / toneMapUncharted2Impl(vec3(W));
    return LINEARtoSRGB(color * whiteScale);
}
vec3 toneMapHejlRichard(vec3 color) {  // Tonemapping.glsl:34-37
    color = max(vec3(0.0f), color - vec3(0.004f));
    return (color * (6.2f * color + 0.5f)) / (color * (6.2f * color + 1.7f) + 0.06f);
}
vec3 toneMapACES(vec3 color) {  // Tonemapping.glsl:41-48
    const float A = 2.51f, B = 0.03f, C = 2.43f, D = 0.59f, E = 0.14f;
    return LINEARtoSRGB(clamp((color * (A * color + B)) / (color * (C * color + D) + E), 0.0f, 1.0f));
}
vec3 defaultToneMap(vec3 color) {  // Tonemapping.glsl:50-53
    color = color / (color + 1.0f);
    return LINEARtoSRGB(color);
}
vec3 tonemap(uint32_t mode, vec3 radiance) {  // RayTracing.rgen:137-149
    if (mode == 0) return defaultToneMap(radiance);
    if (mode == 1) return toneMapUncharted(radiance);
    if (mode == 2) return toneMapHejlRichard(radiance);
    if (mode == 3) return toneMapACES(radiance);
    return LINEARtoSRGB(radiance);
}

// Heatmap.glsl is only used by the HEAT mapping (D5).

// ---------------------------------------------------------------------------
// lib/RayTracingCommons.glsl
// ---------------------------------------------------------------------------
constexpr uint32_t RENDER = 0, HEAT = 1, INSTANCE = 2, TRIANGLE = 3, DISTANCE = 4, ALBEDO = 5,
                   METALLIC = 6, ROUGHNESS = 7, NORMAL = 8, TANGENT = 9, TRANSMISSION = 10, GEO_ID = 11;

struct MixVertex {
    vec3 pos, normal;
    vec4 tangent, color, uv0And1;
    int32_t skin_index;
};

inline vec3 vpos(const gbrt_vertex& v) { return vec3(v.pos[0], v.pos[1], v.pos[2]); }
inline vec3 vnormal(const gbrt_vertex& v) { return vec3(v.normal[0], v.normal[1], v.normal[2]); }
inline vec4 v4(const float* f) { return vec4(f[0], f[1], f[2], f[3]); }

template <class V>
V Mix3(V a, V b, V c, vec3 bc) { return a * bc.x + b * bc.y + c * bc.z; }  // Commons.glsl:32-45

vec2 getUV(vec4 uv0And1, int32_t index) {  // Commons.glsl:65-72
    if (index == 0) return uv0And1.xy();
    if (index == 1) return uv0And1.zw();
    return vec2(0.0f);
}

vec3 getMixVertexAndGeoNormal(const gbrt_vertex& v0, const gbrt_vertex& v1, const gbrt_vertex& v2,
                              vec2 attrs, MixVertex& m) {  // Commons.glsl:82-97
    const vec3 bc = vec3(1.0f - attrs.x - attrs.y, attrs.x, attrs.y);
    vec4 uv_0(v0.uv0[0], v0.uv0[1], v0.uv1[0], v0.uv1[1]);
    vec4 uv_1(v1.uv0[0], v1.uv0[1], v1.uv1[0], v1.uv1[1]);
    vec4 uv_2(v2.uv0[0], v2.uv0[1], v2.uv1[0], v2.uv1[1]);
    m.uv0And1 = Mix3(uv_0, uv_1, uv_2, bc);
    m.pos = Mix3(vpos(v0), vpos(v1), vpos(v2), bc);
    m.color = Mix3(v4(v0.color), v4(v1.color), v4(v2.color), bc);
    m.normal = normalize(Mix3(normalize(vnormal(v0)), normalize(vnormal(v1)), normalize(vnormal(v2)), bc));
    m.tangent = normalize(Mix3(v4(v0.tangent), v4(v1.tangent), v4(v2.tangent), bc));
    m.skin_index = v0.skin_index;
    // calculate_geo_normal, Commons.glsl:75-80
    vec3 p0 = vpos(v0), p1 = vpos(v1), p2 = vpos(v2);
    vec3 e1 = p2 - p0;
    vec3 e0 = p1 - p0;
    return cross(e0, e1);
}

vec3 offset_ray(const vec3 p, const vec3 n) {  // Commons.glsl:103-119
    const float origin = 1.0f / 32.0f;
    const float float_scale = 1.0f / 65536.0f;
    const float int_scale = 256.0f;
    int32_t ofx = int32_t(n.x * int_scale), ofy = int32_t(n.y * int_scale), ofz = int32_t(n.z * int_scale);
    auto add = [](float f, int32_t o) {  // two's-complement wrap like the GPU
        return intBitsToFloat(int32_t(uint32_t(floatBitsToInt(f)) + uint32_t(o)));
    };
    vec3 p_i = vec3(add(p.x, (p.x < 0.0f) ? -ofx : ofx), add(p.y, (p.y < 0.0f) ? -ofy : ofy),
                    add(p.z, (p.z < 0.0f) ? -ofz : ofz));
    return vec3(std::fabs(p.x) < origin ? p.x + float_scale * n.x : p_i.x,
                std::fabs(p.y) < origin ? p.y + float_scale * n.y : p_i.y,
                std::fabs(p.z) < origin ? p.z + float_scale * n.z : p_i.z);
}

// ---------------------------------------------------------------------------
// Textures (D4): bilinear, no mips, Vulkan wrap rules; sRGB decoded per
// texel before filtering (Vulkan spec 16.3 / 16.7).
// ---------------------------------------------------------------------------
float g_srgb_lut[256];
struct LutInit {
    LutInit() {
        for (int i = 0; i < 256; ++i) {
            double c = i / 255.0;
            g_srgb_lut[i] = (float)(c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4));
        }
    }
} g_lut_init;

float half_to_float(uint16_t h) {
    uint32_t s = (h >> 15) & 1u, e = (h >> 10) & 31u, m = h & 1023u;
    float f;
    if (e == 0) f = std::ldexp((float)m, -24);
    else if (e == 31) f = m ? std::numeric_limits<float>::quiet_NaN() : std::numeric_limits<float>::infinity();
    else f = std::ldexp((float)(m | 1024u), (int)e - 25);
    return s ? -f : f;
}

struct Texture {
    uint32_t w = 0, h = 0, format = 0, wrap_s = 0, wrap_t = 0;
    std::vector<uint8_t> data;
};

int wrap_index(int i, int n, uint32_t mode) {
    if (mode == GBRT_WRAP_CLAMP_TO_EDGE) return std::min(std::max(i, 0), n - 1);
    if (mode == GBRT_WRAP_MIRRORED_REPEAT) {
        int m = ((i % (2 * n)) + 2 * n) % (2 * n);
        return m < n ? m : 2 * n - 1 - m;
    }
    return ((i % n) + n) % n;
}

vec4 fetch(const Texture& t, int x, int y) {
    size_t k = (size_t)y * t.w + (size_t)x;
    if (t.format == GBRT_TEX_RGBA32F) {
        float f[4];
        std::memcpy(f, t.data.data() + 16 * k, 16);
        return vec4(f[0], f[1], f[2], f[3]);
    }
    if (t.format == GBRT_TEX_RGBA16F) {
        const uint16_t* p = reinterpret_cast<const uint16_t*>(t.data.data()) + 4 * k;
        return vec4(half_to_float(p[0]), half_to_float(p[1]), half_to_float(p[2]), half_to_float(p[3]));
    }
    const uint8_t* p = t.data.data() + 4 * k;
    if (t.format == GBRT_TEX_RGBA8_SRGB)
        return vec4(g_srgb_lut[p[0]], g_srgb_lut[p[1]], g_srgb_lut[p[2]], float(p[3]) / 255.0f);
    return vec4(float(p[0]) / 255.0f, float(p[1]) / 255.0f, float(p[2]) / 255.0f, float(p[3]) / 255.0f);
}

vec4 lerp4(vec4 a, vec4 b, float f) { return a * (1.0f - f) + b * f; }

vec4 sample_bilinear(const Texture& t, vec2 uv) {
    float x = uv.x * float(t.w) - 0.5f;
    float y = uv.y * float(t.h) - 0.5f;
    float fx = std::floor(x), fy = std::floor(y);
    float ax = x - fx, ay = y - fy;
    int i0 = (int)fx, j0 = (int)fy;
    int xa = wrap_index(i0, t.w, t.wrap_s), xb = wrap_index(i0 + 1, t.w, t.wrap_s);
    int ya = wrap_index(j0, t.h, t.wrap_t), yb = wrap_index(j0 + 1, t.h, t.wrap_t);
    vec4 top = lerp4(fetch(t, xa, ya), fetch(t, xb, ya), ax);
    vec4 bot = lerp4(fetch(t, xa, yb), fetch(t, xb, yb), ax);
    return lerp4(top, bot, ay);
}

// ---------------------------------------------------------------------------
// Scene, BVH2 and traversal
// ---------------------------------------------------------------------------
struct Aabb {
    float lo[3] = {INFINITY, INFINITY, INFINITY};
    float hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    void grow(const float* p) {
        for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], p[k]); hi[k] = std::max(hi[k], p[k]); }
    }
    void grow(const Aabb& b) {
        for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], b.lo[k]); hi[k] = std::max(hi[k], b.hi[k]); }
    }
    float area() const {
        float d[3];
        for (int k = 0; k < 3; ++k) d[k] = std::max(0.0f, hi[k] - lo[k]);
        return 2.0f * (d[0] * d[1] + d[1] * d[2] + d[2] * d[0]);
    }
};

struct BNode {
    Aabb box;
    int32_t first;  // inner: index of the left child (right = first + 1); leaf: first ref
    int32_t count;  // 0 = inner
};

struct Bvh {
    std::vector<BNode> nodes;
    std::vector<uint32_t> refs;  // leaf order -> primitive reference
    std::vector<float> pos;      // world BVH: 9 floats (3 vertices) per primitive reference
};

// Binned SAH BVH2 (16 bins, leaf <= 4 refs, traversal cost 1, test cost 1).
void build_bvh(const std::vector<Aabb>& boxes, Bvh& out) {
    const int NB = 16, MAXLEAF = 4;
    size_t n = boxes.size();
    out.nodes.clear();
    out.refs.resize(n);
    for (size_t i = 0; i < n; ++i) out.refs[i] = (uint32_t)i;
    std::vector<float> cen(3 * n);
    for (size_t i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) cen[3 * i + k] = 0.5f * (boxes[i].lo[k] + boxes[i].hi[k]);
    struct Task { int node; int begin, end; };
    out.nodes.push_back(BNode{});
    std::vector<Task> stack{{0, 0, (int)n}};
    while (!stack.empty()) {
        Task t = stack.back();
        stack.pop_back();
        Aabb bb, cb;
        for (int i = t.begin; i < t.end; ++i) {
            bb.grow(boxes[out.refs[i]]);
            cb.grow(&cen[3 * out.refs[i]]);
        }
        int cnt = t.end - t.begin;
        out.nodes[t.node].box = bb;
        auto make_leaf = [&] { out.nodes[t.node].first = t.begin; out.nodes[t.node].count = cnt; };
        if (cnt <= 1) { make_leaf(); continue; }
        float best_cost = INFINITY;
        int best_axis = -1, best_split = -1;
        for (int ax = 0; ax < 3; ++ax) {
            float ext = cb.hi[ax] - cb.lo[ax];
            if (!(ext > 0.0f)) continue;
            Aabb bin[NB];
            int bc[NB] = {0};
            float scale = NB / ext;
            for (int i = t.begin; i < t.end; ++i) {
                int b = std::min(NB - 1, (int)((cen[3 * out.refs[i] + ax] - cb.lo[ax]) * scale));
                bin[b].grow(boxes[out.refs[i]]);
                bc[b]++;
            }
            float la[NB], ra[NB];
            int lc[NB], rc[NB];
            Aabb acc;
            int c = 0;
            for (int b = 0; b < NB - 1; ++b) { acc.grow(bin[b]); c += bc[b]; la[b] = acc.area(); lc[b] = c; }
            acc = Aabb();
            c = 0;
            for (int b = NB - 1; b > 0; --b) { acc.grow(bin[b]); c += bc[b]; ra[b - 1] = acc.area(); rc[b - 1] = c; }
            for (int b = 0; b < NB - 1; ++b) {
                if (lc[b] == 0 || rc[b] == 0) continue;
                float cost = la[b] * lc[b] + ra[b] * rc[b];
                if (cost < best_cost) { best_cost = cost; best_axis = ax; best_split = b; }
            }
        }
        float parea = bb.area();
        float split_cost = 1.0f + (parea > 0.0f ? best_cost / parea : (float)cnt);
        if (best_axis < 0) {
            if (cnt <= MAXLEAF) { make_leaf(); continue; }
            // all centroids coincide: split by index
            int mid = t.begin + cnt / 2;
            int l = (int)out.nodes.size();
            out.nodes[t.node].first = l;
            out.nodes[t.node].count = 0;
            out.nodes.push_back(BNode{});
            out.nodes.push_back(BNode{});
            stack.push_back({l, t.begin, mid});
            stack.push_back({l + 1, mid, t.end});
            continue;
        }
        if (cnt <= MAXLEAF && (float)cnt <= split_cost) { make_leaf(); continue; }
        float scale = NB / (cb.hi[best_axis] - cb.lo[best_axis]);
        auto mid_it = std::partition(out.refs.begin() + t.begin, out.refs.begin() + t.end, [&](uint32_t r) {
            int b = std::min(NB - 1, (int)((cen[3 * r + best_axis] - cb.lo[best_axis]) * scale));
            return b <= best_split;
        });
        int mid = (int)(mid_it - out.refs.begin());
        int l = (int)out.nodes.size();
        out.nodes[t.node].first = l;
        out.nodes[t.node].count = 0;
        out.nodes.push_back(BNode{});
        out.nodes.push_back(BNode{});
        stack.push_back({l, t.begin, mid});
        stack.push_back({l + 1, mid, t.end});
    }
}

struct Instance {
    float xf[12];     // object-to-world, row-major 3x4
    float inv[12];    // world-to-object
    uint32_t custom;  // geometry id
    uint32_t mask;
    uint32_t blas;    // geometry id of the BLAS
    bool identity;
};

// World-to-object transform of an instance: adjugate inverse of the 3x3
// part in double, translation -R^-1 t, each rounded once to float.  The CUDA
// library computes the same expression.
void affine_inverse(const float* m, float* inv) {
    double a00 = m[0], a01 = m[1], a02 = m[2], a10 = m[4], a11 = m[5], a12 = m[6];
    double a20 = m[8], a21 = m[9], a22 = m[10];
    double t0 = m[3], t1 = m[7], t2 = m[11];
    double det = a00 * (a11 * a22 - a12 * a21) - a01 * (a10 * a22 - a12 * a20) + a02 * (a10 * a21 - a11 * a20);
    double r[9] = {(a11 * a22 - a12 * a21) / det, (a02 * a21 - a01 * a22) / det, (a01 * a12 - a02 * a11) / det,
                   (a12 * a20 - a10 * a22) / det, (a00 * a22 - a02 * a20) / det, (a02 * a10 - a00 * a12) / det,
                   (a10 * a21 - a11 * a20) / det, (a01 * a20 - a00 * a21) / det, (a00 * a11 - a01 * a10) / det};
    for (int i = 0; i < 3; ++i) {
        inv[i * 4 + 0] = (float)r[i * 3 + 0];
        inv[i * 4 + 1] = (float)r[i * 3 + 1];
        inv[i * 4 + 2] = (float)r[i * 3 + 2];
        inv[i * 4 + 3] = (float)(-(r[i * 3 + 0] * t0 + r[i * 3 + 1] * t1 + r[i * 3 + 2] * t2));
    }
}

}  // namespace

struct orc_scene {
    std::vector<gbrt_vertex> base_vertices;  // as uploaded
    std::vector<gbrt_vertex> vertices;       // what shaders read (skinned if orc_skin ran)
    std::vector<uint32_t> indices;
    std::vector<gbrt_priminfo> prims;
    std::vector<gbrt_material_raw> mats;
    std::vector<Texture> textures;
    std::vector<gbrt_light_raw> dlights, plights;
    uint32_t sky_size = 0;
    std::vector<Texture> sky_faces;  // +X,-X,+Y,-Y,+Z,-Z
    // BLAS per geometry
    std::vector<gbrt_geo_range> ranges;  // indexed by geo id
    std::vector<uint8_t> geo_opaque;
    std::vector<Bvh> blas;               // per geo id (built lazily for non-identity use)
    std::vector<char> blas_needed;
    // TLAS
    std::vector<Instance> inst;
    Bvh world;                           // merged BVH over identity-instance (and flattened) triangles
    uint32_t build_flags = 0;            // GBRT_BUILD_NO_FLATTEN
    bool flattened = false;
    std::vector<uint64_t> world_refs;    // (instance << 32) | prim
    Bvh tlas;                            // over entries: 0 = world (if any), then instances
    std::vector<int32_t> tlas_entries;   // -1 = world BVH, else instance index
    bool built = false;
};

namespace {

// --- triangle fetch -------------------------------------------------------
inline void tri_vertices(const orc_scene& s, uint32_t geo, uint32_t prim, const float*& p0, const float*& p1,
                         const float*& p2) {
    const gbrt_priminfo& pi = s.prims[geo];
    uint32_t io = pi.i_offset + 3 * prim;
    p0 = s.vertices[pi.v_offset + s.indices[io]].pos;
    p1 = s.vertices[pi.v_offset + s.indices[io + 1]].pos;
    p2 = s.vertices[pi.v_offset + s.indices[io + 2]].pos;
}

// --- rays -----------------------------------------------------------------
template <typename T>
struct TRay {
    T o[3], d[3], inv[3];
    int kx, ky, kz;
    T Sx, Sy, Sz;
};

template <typename T>
void setup_ray(TRay<T>& r, const float* o, const float* d) {
    for (int k = 0; k < 3; ++k) {
        r.o[k] = (T)o[k];
        r.d[k] = (T)d[k];
        r.inv[k] = d[k] != 0.0f ? (T)1 / (T)d[k] : std::copysign(std::numeric_limits<T>::max(), (T)d[k]);
    }
    // Woop, Benthin, Wald 2013, "Watertight Ray/Triangle Intersection": the
    // dimension with the largest |d| becomes z (first maximum wins).
    T ax = std::fabs(r.d[0]), ay = std::fabs(r.d[1]), az = std::fabs(r.d[2]);
    r.kz = (ax >= ay && ax >= az) ? 0 : (ay >= az ? 1 : 2);
    r.kx = r.kz + 1 == 3 ? 0 : r.kz + 1;
    r.ky = r.kx + 1 == 3 ? 0 : r.kx + 1;
    if (r.d[r.kz] < 0) std::swap(r.kx, r.ky);
    r.Sx = r.d[r.kx] / r.d[r.kz];
    r.Sy = r.d[r.ky] / r.d[r.kz];
    r.Sz = (T)1 / r.d[r.kz];
}

// Watertight test.  FP32: the projections are fused multiply-adds, the edge
// functions, det and T are unfused, t = T/det, u = V/det, v = W/det, all
// IEEE round-to-nearest; an exactly zero edge function is recomputed in
// double.  Returns false on a miss or t outside [tmin, tmax].
template <typename T>
bool intersect_tri(const TRay<T>& r, const float* p0, const float* p1, const float* p2, T tmin, T tmax,
                   T& t_out, float& u_out, float& v_out) {
    T A[3], B[3], C[3];
    for (int k = 0; k < 3; ++k) {
        A[k] = (T)p0[k] - r.o[k];
        B[k] = (T)p1[k] - r.o[k];
        C[k] = (T)p2[k] - r.o[k];
    }
    T Ax = std::fma(-r.Sx, A[r.kz], A[r.kx]);
    T Ay = std::fma(-r.Sy, A[r.kz], A[r.ky]);
    T Bx = std::fma(-r.Sx, B[r.kz], B[r.kx]);
    T By = std::fma(-r.Sy, B[r.kz], B[r.ky]);
    T Cx = std::fma(-r.Sx, C[r.kz], C[r.kx]);
    T Cy = std::fma(-r.Sy, C[r.kz], C[r.ky]);
    T U = Cx * By - Cy * Bx;
    T V = Ax * Cy - Ay * Cx;
    T W = Bx * Ay - By * Ax;
    if (sizeof(T) == 4 && (U == 0 || V == 0 || W == 0)) {
        double CxBy = (double)Cx * (double)By, CyBx = (double)Cy * (double)Bx;
        U = (T)(CxBy - CyBx);
        double AxCy = (double)Ax * (double)Cy, AyCx = (double)Ay * (double)Cx;
        V = (T)(AxCy - AyCx);
        double BxAy = (double)Bx * (double)Ay, ByAx = (double)By * (double)Ax;
        W = (T)(BxAy - ByAx);
    }
    if ((U < 0 || V < 0 || W < 0) && (U > 0 || V > 0 || W > 0)) return false;
    T det = U + V + W;
    if (det == 0) return false;
    T Az = r.Sz * A[r.kz];
    T Bz = r.Sz * B[r.kz];
    T Cz = r.Sz * C[r.kz];
    T Tn = U * Az + V * Bz + W * Cz;
    T t = Tn / det;
    if (!(t >= tmin && t <= tmax)) return false;
    t_out = t;
    u_out = (float)(V / det);
    v_out = (float)(W / det);
    return true;
}

// Robust slab test (Ize 2013): far distances are scaled by 1 + 2*gamma(3)
// and the comparison against the current closest t is widened the same way,
// so no box holding a hit at t <= tcur is culled.
template <typename T>
bool box_hit(const TRay<T>& r, const Aabb& b, T tmin, T tcur) {
    const T eps = std::numeric_limits<T>::epsilon() * (T)0.5;
    const T g3 = 3 * eps / (1 - 3 * eps);
    const T up = 1 + 2 * g3;
    T tn = tmin, tf = tcur;
    for (int k = 0; k < 3; ++k) {
        T t0 = ((T)b.lo[k] - r.o[k]) * r.inv[k];
        T t1 = ((T)b.hi[k] - r.o[k]) * r.inv[k];
        if (t0 > t1) std::swap(t0, t1);
        tn = std::max(tn, t0);
        tf = std::min(tf, t1 * up);
    }
    return tn <= tf * up;
}

struct TraceCtx {  // identifies any-hit draws (D3)
    uint32_t px, py, sample, tag;
};

struct Counters {
    uint64_t nodes = 0, tris = 0;
};

// testOpacityAnyHit, RayTracing.rahit:44-104 (and the identical
// RayTracing.shadow.rahit:44-104).  Returns true when the candidate is
// transparent (ignoreIntersectionEXT).
bool anyhit_ignore(const orc_scene& s, uint32_t geo, uint32_t prim, uint32_t instance, float u, float v,
                   const TraceCtx& ctx);

struct HitT {
    double t;
    float u, v;
    uint32_t inst, prim, geo;
};

inline bool closer(double t, uint32_t inst, uint32_t prim, const HitT& best) {  // D2
    if (t < best.t) return true;
    if (t > best.t) return false;
    return inst < best.inst || (inst == best.inst && prim < best.prim);
}

// Visits a BVH whose refs resolve through `resolve`.  Returns true when the
// traversal must stop (terminate-on-first hit found).
template <typename T, typename Resolve>
bool traverse_bvh(const orc_scene& s, const Bvh& bvh, const TRay<T>& r, T tmin, HitT& best, uint32_t flags,
                  const TraceCtx& ctx, Counters& cnt, Resolve resolve, bool& found) {
    if (bvh.nodes.empty()) return false;
    int stack[128];
    int sp = 0;
    if (!box_hit(r, bvh.nodes[0].box, tmin, (T)best.t)) return false;
    stack[sp++] = 0;
    while (sp > 0) {
        const BNode& n = bvh.nodes[stack[--sp]];
        if (n.count > 0) {
            for (int i = 0; i < n.count; ++i) {
                uint32_t inst, prim, bgeo, geo;
                const uint32_t ref = bvh.refs[n.first + i];
                resolve(ref, inst, prim, bgeo, geo);
                const float *p0, *p1, *p2;
                if (!bvh.pos.empty()) {  // stored (world-space) triangle
                    p0 = &bvh.pos[9 * (size_t)ref];
                    p1 = p0 + 3;
                    p2 = p0 + 6;
                } else {
                    tri_vertices(s, bgeo, prim, p0, p1, p2);
                }
                cnt.tris++;
                T t;
                float u, v;
                if (!intersect_tri(r, p0, p1, p2, tmin, (T)best.t, t, u, v)) continue;
                if (!closer((double)t, inst, prim, best)) continue;
                if (!(flags & GBRT_RAY_OPAQUE) && !s.geo_opaque[bgeo] &&
                    anyhit_ignore(s, geo, prim, inst, u, v, ctx))
                    continue;
                best = HitT{(double)t, u, v, inst, prim, geo};
                found = true;
                if (flags & GBRT_RAY_TERMINATE_ON_FIRST) return true;
            }
            continue;
        }
        cnt.nodes++;
        const BNode& l = bvh.nodes[n.first];
        const BNode& rr = bvh.nodes[n.first + 1];
        bool hl = box_hit(r, l.box, tmin, (T)best.t);
        bool hr = box_hit(r, rr.box, tmin, (T)best.t);
        if (hl && hr) {
            // nearer child first
            T cl = 0, cr = 0;
            for (int k = 0; k < 3; ++k) {
                cl += ((T)(l.box.lo[k] + l.box.hi[k]) * (T)0.5 - r.o[k]) * r.d[k];
                cr += ((T)(rr.box.lo[k] + rr.box.hi[k]) * (T)0.5 - r.o[k]) * r.d[k];
            }
            if (sp + 2 > 128) return false;
            if (cl <= cr) { stack[sp++] = n.first + 1; stack[sp++] = n.first; }
            else { stack[sp++] = n.first; stack[sp++] = n.first + 1; }
        } else if (hl) {
            stack[sp++] = n.first;
        } else if (hr) {
            stack[sp++] = n.first + 1;
        }
    }
    return false;
}

// traceRayEXT over TLAS -> BLAS.  Identity instances live in the merged world
// BVH; the rest are intersected in object space with the ray transformed by
// the instance's world-to-object matrix (unfused, left to right).
template <typename T>
bool trace(const orc_scene& s, const float* o, const float* d, float tmin, float tmax, uint32_t flags,
           const TraceCtx& ctx, HitT& best, Counters& cnt) {
    best = HitT{(double)tmax, 0, 0, ~0u, ~0u, ~0u};
    if (!s.built) return false;
    if (d[0] == 0.0f && d[1] == 0.0f && d[2] == 0.0f) return false;
    TRay<T> wr;
    setup_ray(wr, o, d);
    bool found = false;
    const Bvh& tl = s.tlas;
    if (tl.nodes.empty()) return false;
    int stack[128];
    int sp = 0;
    if (!box_hit(wr, tl.nodes[0].box, (T)tmin, (T)best.t)) return false;
    stack[sp++] = 0;
    while (sp > 0) {
        const BNode& n = tl.nodes[stack[--sp]];
        if (n.count > 0) {
            for (int i = 0; i < n.count; ++i) {
                int32_t e = s.tlas_entries[tl.refs[n.first + i]];
                bool stop;
                if (e < 0) {
                    stop = traverse_bvh<T>(s, s.world, wr, (T)tmin, best, flags, ctx, cnt,
                                           [&](uint32_t ref, uint32_t& inst, uint32_t& prim, uint32_t& bgeo,
                                               uint32_t& geo) {
                                               uint64_t wref = s.world_refs[ref];
                                               inst = (uint32_t)(wref >> 32);
                                               prim = (uint32_t)wref;
                                               bgeo = s.inst[inst].blas;
                                               geo = s.inst[inst].custom;
                                           },
                                           found);
                } else {
                    const Instance& in = s.inst[e];
                    if ((in.mask & 0xFFu) == 0) continue;
                    vec3 oo = mul34(in.inv, vec4(o[0], o[1], o[2], 1.0f));
                    vec3 dd = mul34(in.inv, vec4(d[0], d[1], d[2], 0.0f));
                    float of[3] = {oo.x, oo.y, oo.z}, df[3] = {dd.x, dd.y, dd.z};
                    TRay<T> orr;
                    setup_ray(orr, of, df);
                    uint32_t ie = (uint32_t)e;
                    uint32_t g = in.custom, bg = in.blas;
                    stop = traverse_bvh<T>(s, s.blas[in.blas], orr, (T)tmin, best, flags, ctx, cnt,
                                           [&](uint32_t ref, uint32_t& inst, uint32_t& prim, uint32_t& bgeo,
                                               uint32_t& geo) {
                                               inst = ie;
                                               prim = ref;
                                               bgeo = bg;
                                               geo = g;
                                           },
                                           found);
                }
                if (stop) return true;
            }
            continue;
        }
        cnt.nodes++;
        const BNode& l = tl.nodes[n.first];
        const BNode& rr = tl.nodes[n.first + 1];
        bool hl = box_hit(wr, l.box, (T)tmin, (T)best.t);
        bool hr = box_hit(wr, rr.box, (T)tmin, (T)best.t);
        if (sp + 2 > 128) break;
        if (hl) stack[sp++] = n.first;
        if (hr) stack[sp++] = n.first + 1;
    }
    return found;
}

vec4 texture(const orc_scene& s, int32_t index, vec2 uv) {
    if (index < 0 || (size_t)index >= s.textures.size() || s.textures[index].w == 0) return vec4(1.0f);
    return sample_bilinear(s.textures[index], uv);
}

bool anyhit_ignore(const orc_scene& s, uint32_t geo, uint32_t prim, uint32_t instance, float u, float v,
                   const TraceCtx& ctx) {
    const gbrt_priminfo& primInfo = s.prims[geo];
    const gbrt_material_raw& mat = s.mats[primInfo.material_id];
    if (mat.alpha_mode == 1u) return false;  // OPAQUE
    const uint32_t io = primInfo.i_offset + 3 * prim;
    const gbrt_vertex& v0 = s.vertices[primInfo.v_offset + s.indices[io]];
    const gbrt_vertex& v1 = s.vertices[primInfo.v_offset + s.indices[io + 1]];
    const gbrt_vertex& v2 = s.vertices[primInfo.v_offset + s.indices[io + 2]];
    MixVertex mix_vertex;
    getMixVertexAndGeoNormal(v0, v1, v2, vec2(u, v), mix_vertex);
    vec4 uv0And1 = mix_vertex.uv0And1;
    const vec4 baseColor = v4(mat.base_color);
    vec4 color4 = mix_vertex.color * baseColor;
    if (mat.base_color_texture.index >= 0)
        color4 *= texture(s, mat.base_color_texture.index, getUV(uv0And1, mat.base_color_texture.coord));
    float opacity = color4.w;
    if (mat.workflow == SPECULAR_GLOSS_WORKFLOW) {
        vec4 diffuse_factor = v4(mat.sg_diffuse_factor);
        if (mat.sg_diffuse_texture.index >= 0)
            diffuse_factor *= texture(s, mat.sg_diffuse_texture.index, getUV(uv0And1, mat.sg_diffuse_texture.coord));
        color4 = mix_vertex.color * diffuse_factor;
        opacity = color4.w;
    }
    if (mat.alpha_mode == 2u) {  // MASK
        if (ctx.tag != 0u) note_margin(opacity - mat.alpha_cutoff);  // camera rays are bit-exact
        return (opacity < mat.alpha_cutoff);
    }
    uvec4 key(ctx.px, ctx.py, ctx.sample, blend_hash(instance, prim, ctx.tag));  // D3
    float uu = uintToFloat(pcg4d(key).x);
    if (ctx.tag != 0u) note_margin(opacity - uu);
    return (opacity <= uu);
}

// Cube map lookup (Vulkan face selection, clamp-to-edge bilinear, D4).
vec3 sample_sky(const orc_scene& s, vec3 d) {
    if (s.sky_size == 0) return vec3(0.0f);
    float ax = std::fabs(d.x), ay = std::fabs(d.y), az = std::fabs(d.z);
    {  // face choice: distance between the largest and the second largest axis
        const float hi = std::max(ax, std::max(ay, az)), lo = std::min(ax, std::min(ay, az));
        note_margin(hi - (ax + ay + az - hi - lo));
    }
    int face;
    float sc, tc, ma;
    if (ax >= ay && ax >= az) {
        ma = ax;
        if (d.x >= 0.0f) { face = 0; sc = -d.z; tc = -d.y; } else { face = 1; sc = d.z; tc = -d.y; }
    } else if (ay >= az) {
        ma = ay;
        if (d.y >= 0.0f) { face = 2; sc = d.x; tc = d.z; } else { face = 3; sc = d.x; tc = -d.z; }
    } else {
        ma = az;
        if (d.z >= 0.0f) { face = 4; sc = d.x; tc = -d.y; } else { face = 5; sc = -d.x; tc = -d.y; }
    }
    float su = 0.5f * (dv(sc, ma) + 1.0f);
    float sv = 0.5f * (dv(tc, ma) + 1.0f);
    return sample_bilinear(s.sky_faces[face], vec2(su, sv)).xyz();
}

// RayPayload, RayTracingCommons.glsl:11-24.
struct RayPayload {
    vec3 hitValue, hitPoint;
    float t;
    vec3 scatterDirection;
    bool needScatter;
    uint32_t RandomSeed;
    vec3 emittance;
    uvec4 rngState;
    float volume_dis;
};

struct FrameCtx {
    const orc_scene* s;
    const gbrt_ubo* ubo;
    uint32_t px, py, sample, bounce;
    int fp64;
    Counters* cnt;
    uint64_t shadow_rays = 0, shaded = 0;
};

template <typename T>
bool trace_any(FrameCtx& f, const float* o, const float* d, float tmin, float tmax, uint32_t flags, HitT& h,
               uint32_t tag) {
    TraceCtx tc{f.px, f.py, f.sample, tag};
    return trace<T>(*f.s, o, d, tmin, tmax, flags, tc, h, *f.cnt);
}

bool trace_ray(FrameCtx& f, const float* o, const float* d, float tmin, float tmax, uint32_t flags, HitT& h,
               uint32_t tag) {
    return f.fp64 ? trace_any<double>(f, o, d, tmin, tmax, flags, h, tag)
                  : trace_any<float>(f, o, d, tmin, tmax, flags, h, tag);
}

// RayTracing.rmiss:14-45.
void miss_shader(FrameCtx& f, RayPayload& Ray, const float* dir) {
    const orc_scene& s = *f.s;
    vec3 light_acc = vec3(0.0f);
    vec3 ray_direction = normalize(vec3(dir[0], dir[1], dir[2]));
    if (Ray.t != 0.0f) {
        for (size_t i = 0; i < s.dlights.size(); i++) {
            const gbrt_light_raw& li = s.dlights[i];
            float cos = dot(normalize(vec3(li.transform[0], li.transform[1], li.transform[2])), ray_direction);
            note_margin(cos);
            if (cos < 0.0f) light_acc += -cos * vec3(li.color[0], li.color[1], li.color[2]) * li.intensity;
        }
    }
    if (f.ubo->has_sky) {
        const vec3 skyColor = sample_sky(s, ray_direction);
        light_acc += skyColor + light_acc;
    } else {
        light_acc += vec3(0.01f);
    }
    Ray.hitValue = vec3(0.0f);
    Ray.needScatter = false;
    Ray.emittance = light_acc;
    if (s.dlights.empty()) Ray.emittance = vec3(0.0f);
    Ray.t = -1.0f;
}

// castShadowRay, RayTracing.rchit:35-59; misses run shadow.rmiss:10-13.
bool castShadowRay(FrameCtx& f, vec3 hitPosition, vec3 directionToLight, float tMax) {
    const float o[3] = {hitPosition.x, hitPosition.y, hitPosition.z};
    const float d[3] = {directionToLight.x, directionToLight.y, directionToLight.z};
    uint32_t flags = GBRT_RAY_TERMINATE_ON_FIRST;
    if (f.ubo->fully_opaque) flags |= GBRT_RAY_OPAQUE;
    f.shadow_rays++;
    HitT h;
    bool shadow = trace_ray(f, o, d, 0.1f, tMax, flags, h, f.bounce | 0x100u);
    return !shadow;
}

// sampleLightUniform / sampleLightRIS, RayTracing.rchit:62-122.
bool sampleLightUniform(const orc_scene& s, uvec4& rngState, gbrt_light_raw& light, float& w) {
    uint32_t light_num = (uint32_t)s.plights.size();
    if (light_num == 0) return false;
    uint32_t idx = std::min(light_num - 1, (uint32_t)(rand(rngState) * float(light_num)));
    light = s.plights[idx];
    w = float(light_num);
    return true;
}
bool sampleLightRIS(const orc_scene& s, uvec4& rngState, vec3 hitPosition, vec3 surfaceNormal,
                    gbrt_light_raw& selectedSample, float& lightSampleWeight) {
    uint32_t light_num = (uint32_t)s.plights.size();
    if (light_num == 0) return false;
    float totalWeights = 0.0f;
    float samplePdfG = 0.0f;
    uint32_t candidates_num = std::min(light_num, 3u);
    for (uint32_t i = 0; i < candidates_num; i++) {
        const gbrt_light_raw& li = s.plights[i];
        if (luminance(vec3(li.color[0], li.color[1], li.color[2]) * li.intensity) < 0.1f) continue;
        float candidateWeight;
        gbrt_light_raw candidate;
        if (sampleLightUniform(s, rngState, candidate, candidateWeight)) {
            vec3 lightVector = vec3(candidate.transform[0], candidate.transform[1], candidate.transform[2]) -
                               hitPosition;
            vec3 L = normalize(lightVector);
            note_margin(dot(surfaceNormal, L) - 0.00001f);
            if (dot(surfaceNormal, L) < 0.00001f) continue;
            float candidatePdfG = luminance(getLightIntensityAtPoint(candidate, length(lightVector)));
            const float candidateRISWeight = candidatePdfG * candidateWeight;
            totalWeights += candidateRISWeight;
            const float accept = rand(rngState);
            const float acceptRatio = dv(candidateRISWeight, totalWeights);
            note_margin(accept - acceptRatio);
            if (accept < acceptRatio) {
                selectedSample = candidate;
                samplePdfG = candidatePdfG;
            }
        }
    }
    if (totalWeights == 0.0f) return false;
    lightSampleWeight = dv(dv(totalWeights, float(3)), samplePdfG);
    return true;
}

vec3 normal_transform(const float* o2w, vec3 n) { return normalize(mul34(o2w, vec4(n, 0.0f))); }  // rchit:28-30

// RayTracing.rchit:136-477.
void closest_hit(FrameCtx& f, RayPayload& Ray, const HitT& hit, const float* wdir) {
    const orc_scene& s = *f.s;
    const gbrt_ubo& ubo = *f.ubo;
    f.shaded++;
    static const float ident[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
    const float* o2w = s.inst[hit.inst].identity ? ident : s.inst[hit.inst].xf;
    const gbrt_priminfo& primInfo = s.prims[hit.geo];
    const gbrt_material_raw& mat = s.mats[primInfo.material_id];
    vec3 last_hit = Ray.hitPoint;
    Ray.t = (float)hit.t;
    const uint32_t vertexOffset = primInfo.v_offset;
    const uint32_t indexOffset = primInfo.i_offset + (3 * hit.prim);
    const gbrt_vertex& v0 = s.vertices[vertexOffset + s.indices[indexOffset]];
    const gbrt_vertex& v1 = s.vertices[vertexOffset + s.indices[indexOffset + 1]];
    const gbrt_vertex& v2 = s.vertices[vertexOffset + s.indices[indexOffset + 2]];
    const vec2 HitAttributes(hit.u, hit.v);
    MixVertex mix_vertex;
    vec3 geo_normal = normal_transform(o2w, getMixVertexAndGeoNormal(v0, v1, v2, HitAttributes, mix_vertex));
    vec3 pos = mix_vertex.pos;
    vec3 origin = mul34(o2w, vec4(pos, 1.0f));
    vec4 uv0And1 = mix_vertex.uv0And1;
    const vec4 baseColor = v4(mat.base_color);
    vec4 color4 = mix_vertex.color * baseColor;
    if (mat.base_color_texture.index >= 0)
        color4 *= texture(s, mat.base_color_texture.index, getUV(uv0And1, mat.base_color_texture.coord));
    vec3 color = color4.rgb();
    Ray.needScatter = false;
    Ray.hitPoint = pos;
    vec3 normal = mix_vertex.normal;
    if (mat.normal_texture.index >= 0) {
        vec3 normal_t = normalize(
            texture(s, mat.normal_texture.index, getUV(uv0And1, mat.normal_texture.coord)).xyz() * 2.0f - 1.0f);
        // getNormal, rchit:124-129
        vec3 tangent_mix = mix_vertex.tangent.xyz();
        vec3 tangent = normalize((tangent_mix - dot(tangent_mix, normal) * normal));
        vec3 b = normalize(cross(normal, tangent) * mix_vertex.tangent.w);
        normal = tangent * normal_t.x + b * normal_t.y + normal * normal_t.z;
    }
    normal = normal_transform(o2w, normal);
    const vec3 V = -normalize(vec3(wdir[0], wdir[1], wdir[2]));
    const float cos = dot(V, geo_normal);
    const bool frontFace = cos >= 0.0f;
    geo_normal = frontFace ? geo_normal : -geo_normal;
    const vec3 outwardNormal = dot(geo_normal, normal) < 0.0f ? -normal : normal;
    if (f.bounce) {  // camera rays are bit-exact
        note_margin(cos);
        note_margin(dot(geo_normal, normal));
    }

    vec3 emittance = vec3(mat.emissive_factor[0], mat.emissive_factor[1], mat.emissive_factor[2]);
    if (mat.emissive_texture.index >= 0)
        emittance *= texture(s, mat.emissive_texture.index, getUV(uv0And1, mat.emissive_texture.coord)).rgb();

    float metallic = mat.metallic_factor;
    float roughness = mat.roughness_factor;
    if (mat.metallic_roughness_texture.index >= 0) {
        vec4 mr = texture(s, mat.metallic_roughness_texture.index, getUV(uv0And1, mat.metallic_roughness_texture.coord));
        roughness *= mr.y;
        metallic *= mr.z;
    }
    vec3 specular_factor_workflow = vec3(1.0f);
    if (mat.workflow == SPECULAR_GLOSS_WORKFLOW) {
        vec4 diffuse_factor = v4(mat.sg_diffuse_factor);
        vec4 specular_glossiness_factor = v4(mat.sg_specular_glossiness_factor);
        if (mat.sg_diffuse_texture.index >= 0)
            diffuse_factor *= texture(s, mat.sg_diffuse_texture.index, getUV(uv0And1, mat.sg_diffuse_texture.coord));
        if (mat.sg_specular_glossiness_texture.index >= 0)
            specular_glossiness_factor *= texture(s, mat.sg_specular_glossiness_texture.index,
                                                  getUV(uv0And1, mat.sg_specular_glossiness_texture.coord));
        specular_factor_workflow = specular_glossiness_factor.rgb();
        float glossiness_factor = specular_glossiness_factor.w;
        roughness = 1.0f - glossiness_factor;
        float maxSpecular = std::max(std::max(specular_factor_workflow.x, specular_factor_workflow.y),
                                     specular_factor_workflow.z);
        color = mix_vertex.color.rgb() * diffuse_factor.rgb();
        metallic = convertMetallic(color, specular_factor_workflow, maxSpecular);
    }
    float transmission_factor = 0.0f;
    if (mat.transmission_exist) {
        transmission_factor = mat.transmission_factor;
        if (mat.transmission_texture.index >= 0)
            transmission_factor *=
                texture(s, mat.transmission_texture.index, getUV(uv0And1, mat.transmission_texture.coord)).x;
    }
    uint32_t mapping = ubo.mapping;
    if (mat.unlit) mapping = ALBEDO;
    switch (mapping) {  // rchit:258-286
        case ALBEDO: Ray.emittance = color; return;
        case TRIANGLE: Ray.emittance = vec3(1.0f - hit.u - hit.v, hit.u, hit.v); return;
        case INSTANCE: Ray.emittance = hashAndColor(hit.inst); return;
        case METALLIC: Ray.emittance = vec3(metallic); return;
        case ROUGHNESS: Ray.emittance = vec3(roughness); return;
        case NORMAL: Ray.emittance = (outwardNormal + 1.0f) / 2.0f; return;
        case TANGENT: Ray.emittance = (normal_transform(o2w, mix_vertex.tangent.xyz()) + 1.0f) / 2.0f; return;
        case TRANSMISSION: Ray.emittance = vec3(transmission_factor); return;
        case GEO_ID: Ray.emittance = hashAndColor(hit.geo); return;
        default: break;
    }
    float spec_factor = mat.specular_factor;
    vec3 spec_color_factor = vec3(mat.specular_color_factor[0], mat.specular_color_factor[1], mat.specular_color_factor[2]);
    if (mat.specular_texture.index >= 0)
        spec_factor *= texture(s, mat.specular_texture.index, getUV(uv0And1, mat.specular_texture.coord)).w;
    if (mat.specular_color_texture.index >= 0)
        spec_color_factor *=
            texture(s, mat.specular_color_texture.index, getUV(uv0And1, mat.specular_color_texture.coord)).rgb();
    const float ior = mat.ior;

    Ray.hitPoint = origin;
    uint32_t seed = Ray.RandomSeed;
    uvec4 rngState = Ray.rngState;
    Ray.emittance = emittance * ubo.exposure;
    Ray.needScatter = false;
    uint32_t brdfType = 0;
    vec3 throughput = vec3(1.0f);
    MaterialBrdf matbrdf;
    matbrdf.baseColor = color;
    matbrdf.metallic = metallic;
    matbrdf.roughness = roughness;
    matbrdf.ior = mat.volume_exists ? ior : 1.0f;
    matbrdf.transmission = transmission_factor;
    matbrdf.specular_factor = spec_factor;
    matbrdf.specular_color_factor = spec_color_factor;
    matbrdf.use_spec = mat.specular_exist != 0;
    matbrdf.frontFace = frontFace;
    matBuild(matbrdf);
    if (mat.workflow == SPECULAR_GLOSS_WORKFLOW) {
        float maxSpecular = std::max(std::max(specular_factor_workflow.x, specular_factor_workflow.y),
                                     specular_factor_workflow.z);
        matbrdf.c_diff = color * (1.0f - maxSpecular);
        matbrdf.F0 = specular_factor_workflow;
    }
    matbrdf.attenuation_color = vec3(mat.attenuation_color[0], mat.attenuation_color[1], mat.attenuation_color[2]);
    matbrdf.attenuation_distance = mat.attenuation_distance;
    matbrdf.volume = mat.volume_exists != 0;
    float displacement = length(origin - last_hit);
    matbrdf.t_diff = displacement;

    gbrt_light_raw light{};
    float light_weight = 0.0f;
    if (sampleLightRIS(s, rngState, origin, geo_normal, light, light_weight)) {  // rchit:338-350
        vec3 light_vec = vec3(light.transform[0], light.transform[1], light.transform[2]) - origin;
        float light_distance = length(light_vec);
        light_vec = normalize(light_vec);
        if (castShadowRay(f, origin, light_vec, light_distance)) {
            Ray.emittance += evalCombinedBRDF(outwardNormal, light_vec, V, matbrdf) * light_weight *
                             light.intensity * vec3(light.color[0], light.color[1], light.color[2]);
        }
    }

    if (metallic == 1.0f && roughness == 0.0f) {  // rchit:352-395
        brdfType = SPECULAR_TYPE;
    } else {
        BRDFProb prob = getBrdfProbability(matbrdf, V, outwardNormal);
        float randfloat = rand(rngState);
        note_margin(randfloat - prob.specular);
        note_margin(randfloat - (prob.specular + prob.diffuse));
        if (randfloat < prob.specular) {
            brdfType = SPECULAR_TYPE;
            throughput /= prob.specular;
            if (Ray.volume_dis >= 0.0f) Ray.volume_dis += displacement;
        } else if (randfloat >= prob.specular && randfloat <= prob.specular + prob.diffuse) {
            brdfType = DIFFUSE_TYPE;
            throughput /= prob.diffuse;
            if (Ray.volume_dis >= 0.0f) Ray.volume_dis += displacement;
        } else {
            brdfType = TRANSMISSION_TYPE;
            if (mat.volume_exists) {
                if (Ray.volume_dis >= 0.0f) Ray.volume_dis += displacement;
                else if (frontFace) Ray.volume_dis = 0.0f;
            }
            throughput /= prob.transmission;
        }
    }
    if (brdfType == TRANSMISSION_TYPE) origin = offset_ray(origin, -geo_normal);
    vec3 brdfWeight(0.0f);
    float ua = rand(rngState);
    float ub = rand(rngState);
    vec2 u = vec2(ua, ub);
    vec3 direction(0.0f);
    Ray.needScatter = evalIndirectCombinedBRDF(u, outwardNormal, geo_normal, V, matbrdf, brdfType, direction,
                                               brdfWeight, Ray.volume_dis);
    throughput *= brdfWeight;
    Ray.hitPoint = origin;
    Ray.scatterDirection = direction;
    Ray.hitValue = throughput;

    if (ubo.debug == 1) {  // rchit:437-474 (legacy; D5)
        vec3 wd = vec3(wdir[0], wdir[1], wdir[2]);
        if (matbrdf.transmission > 0.0f) {
            const float refraction_ratio = frontFace ? dv(1.0f, ior) : ior;
            const float cos_theta = std::fabs(cos);
            const vec3 refracted = refract(wd, outwardNormal, refraction_ratio);
            const float reflectProb = refracted != vec3(0.0f) ? Schlick(cos_theta, refraction_ratio) : 1.0f;
            Ray.hitValue = color;
            Ray.needScatter = true;
            if (RandomFloat(seed) < reflectProb) Ray.scatterDirection = reflect(wd, normal);
            else Ray.scatterDirection = refracted;
        } else if (length(emittance) < 0.01f && roughness == 1.0f) {
            const bool isScattered = dot(wd, geo_normal) < 0.0f;
            const vec3 scatter = normalize(vec3(outwardNormal + RandomInUnitSphere(seed)));
            Ray.needScatter = isScattered;
            Ray.scatterDirection = scatter;
            Ray.hitValue = isScattered ? color : vec3(0.0f);
        } else if (metallic > 0.0f) {
            vec3 reflected = reflect(wd, outwardNormal);
            const bool isScattered = dot(reflected, geo_normal) > 0.0f;
            Ray.needScatter = isScattered;
            Ray.hitValue = isScattered ? color : vec3(0.0f);
            Ray.scatterDirection = reflected + 0.08f * RandomInUnitSphere(seed);
        }
    }
    Ray.RandomSeed = seed;
    Ray.rngState = rngState;
}

constexpr float tMinC = 0.001f, tMaxC = 10000.0f;  // lib/Camera.glsl:2-3

// One sample of RayTracing.rgen:49-130 for pixel (x, y); returns its radiance.
template <typename Acc>
vec3 raygen_sample(FrameCtx& f, uint32_t x, uint32_t y, uint32_t W, uint32_t H, uint32_t s, gbrt_hit* primary,
                   uint64_t& cam, uint64_t& ext, float& last_t) {
    const gbrt_ubo& ubo = *f.ubo;
    RayPayload Ray;
    Ray.hitValue = vec3(0.0f);
    Ray.hitPoint = vec3(0.0f);
    Ray.scatterDirection = vec3(0.0f);
    Ray.needScatter = false;
    Ray.emittance = vec3(0.0f);
    // D1 seeds (replacing rgen:32-40)
    Ray.RandomSeed = InitRandomSeed(InitRandomSeed(x, y), s);
    uvec4 rngState = initRNG(x, y, s);
    Ray.rngState = initRNG(x, y, InitRandomSeed(s, 0x9E3779B9u));
    f.sample = s;
    Acc radiance[3] = {0, 0, 0};

    vec2 pixel;
    const vec2 pixelCenter = vec2(float(x), float(y)) + vec2(0.5f);
    if (ubo.antialiasing) {
        float ra = rand(rngState);
        float rb = rand(rngState);
        vec2 offset = vec2(ra, rb) - 0.5f;
        pixel = pixelCenter + offset;
    } else {
        pixel = pixelCenter;
    }
    const vec2 uv = (pixel / vec2(float(W), float(H))) * 2.0f - 1.0f;
    vec2 offset = ubo.aperture / 2.0f * RandomInUnitDisk(Ray.RandomSeed);
    vec4 origin = mul(ubo.model_view_inverse, vec4(offset, 0.0f, 1.0f));
    vec4 target = mul(ubo.projection_inverse, vec4(uv.x, uv.y, 1.0f, 1.0f));
    vec4 direction = mul(ubo.model_view_inverse,
                         vec4(normalize(target.xyz() * ubo.focus_distance - vec3(offset, 0.0f)), 0.0f));
    float tFar = tMaxC;
    if (ubo.orthographic_fov_dis > 0.0f) {
        vec2 new_uv = (1.0f + ubo.orthographic_fov_dis) * uv;
        origin = vec4(new_uv.x, -new_uv.y, 0.0f, 1.0f);
        origin = mul(ubo.model_view_inverse, origin);
        direction = vec4(0.0f, 0.0f, -1.0f, 0.0f);
        direction = mul(ubo.model_view_inverse, direction);
        tFar = 10.0f * tMaxC;
    }
    vec3 throughput = vec3(1.0f);
    Ray.t = 0.0f;
    Ray.volume_dis = -1.0f;
    uint32_t rayFlags = 0;
    if (ubo.fully_opaque) rayFlags |= GBRT_RAY_OPAQUE;
    for (uint32_t b = 0; b < ubo.number_of_bounces; b++) {
        f.bounce = b;
        const float o[3] = {origin.x, origin.y, origin.z};
        const float d[3] = {direction.x, direction.y, direction.z};
        if (b == 0) cam++; else ext++;
        HitT h;
        bool hit = trace_ray(f, o, d, tMinC, tFar, rayFlags, h, b);
        if (b == 0 && primary) {
            primary->t = hit ? (float)h.t : -1.0f;
            primary->u = hit ? h.u : 0.0f;
            primary->v = hit ? h.v : 0.0f;
            primary->instance_id = hit ? h.inst : ~0u;
            primary->primitive_id = hit ? h.prim : ~0u;
            primary->custom_index = hit ? h.geo : ~0u;
        }
        if (hit && b) note_edge(std::min(std::min(h.u, h.v), 1.0f - h.u - h.v));
        if (hit) closest_hit(f, Ray, h, d);
        else miss_shader(f, Ray, d);
        const vec3 hitColor = Ray.hitValue;
        const float t = Ray.t;
        const bool isScattered = Ray.needScatter;
        vec3 add = throughput * Ray.emittance;
        radiance[0] += add.x;
        radiance[1] += add.y;
        radiance[2] += add.z;
        Ray.emittance = vec3(0.0f);
        if (b + 1 == ubo.number_of_bounces) break;
        if (b > 3u) {  // MIN_BOUNCES, rgen:15,108-118
            float rrProbability = clamp(luminance(throughput), 0.01f, 0.95f);
            float prop = rand(rngState);
            note_margin(rrProbability - prop);
            if (rrProbability < prop) break;
            throughput /= rrProbability;
        }
        throughput *= hitColor;
        if (!isScattered || t < 0.0f) break;
        origin = vec4(Ray.hitPoint, 1.0f);
        direction = vec4(Ray.scatterDirection, 0.0f);
    }
    last_t = Ray.t;
    return vec3((float)radiance[0], (float)radiance[1], (float)radiance[2]);
}

void rebuild(orc_scene& s) {
    size_t ngeo = s.ranges.size();
    // per-geo BLAS (only for geometries referenced by non-identity instances)
    s.blas.assign(ngeo, Bvh());
    for (size_t g = 0; g < ngeo; ++g) {
        if (!s.blas_needed.size() || !s.blas_needed[g]) continue;
        uint32_t ntri = s.ranges[g].i_len / 3;
        std::vector<Aabb> boxes(ntri);
        for (uint32_t p = 0; p < ntri; ++p) {
            const float *p0, *p1, *p2;
            tri_vertices(s, (uint32_t)g, p, p0, p1, p2);
            boxes[p].grow(p0); boxes[p].grow(p1); boxes[p].grow(p2);
        }
        build_bvh(boxes, s.blas[g]);
    }
    // merged world BVH over identity instances, and over transformed ones too
    // when the flattened scene has at most GBRT_FLATTEN_MAX_TRIANGLES
    // triangles (their vertices transformed once, mul34 unfused), unless the
    // build asked for GBRT_BUILD_NO_FLATTEN -- the rule of the library's build
    uint64_t flat_total = 0;
    for (size_t i = 0; i < s.inst.size(); ++i)
        if ((s.inst[i].mask & 0xFFu) != 0) flat_total += s.ranges[s.inst[i].blas].i_len / 3;
    s.flattened = !(s.build_flags & GBRT_BUILD_NO_FLATTEN) && flat_total <= GBRT_FLATTEN_MAX_TRIANGLES;
    s.world_refs.clear();
    std::vector<Aabb> wboxes;
    std::vector<float> wpos;
    for (size_t i = 0; i < s.inst.size(); ++i) {
        const Instance& in = s.inst[i];
        if (!in.identity && !(s.flattened && (in.mask & 0xFFu) != 0)) continue;
        uint32_t g = in.blas;
        uint32_t ntri = s.ranges[g].i_len / 3;
        for (uint32_t p = 0; p < ntri; ++p) {
            const float* pv[3];
            tri_vertices(s, g, p, pv[0], pv[1], pv[2]);
            Aabb b;
            for (int k = 0; k < 3; ++k) {
                float q[3] = {pv[k][0], pv[k][1], pv[k][2]};
                if (!in.identity) {
                    vec3 w = mul34(in.xf, vec4(q[0], q[1], q[2], 1.0f));
                    q[0] = w.x;
                    q[1] = w.y;
                    q[2] = w.z;
                }
                b.grow(q);
                wpos.insert(wpos.end(), q, q + 3);
            }
            wboxes.push_back(b);
            s.world_refs.push_back(((uint64_t)i << 32) | p);
        }
    }
    s.world = Bvh();
    if (!wboxes.empty()) build_bvh(wboxes, s.world);
    s.world.pos = std::move(wpos);
    // TLAS entries
    s.tlas_entries.clear();
    std::vector<Aabb> tboxes;
    if (!s.world.nodes.empty()) { s.tlas_entries.push_back(-1); tboxes.push_back(s.world.nodes[0].box); }
    for (size_t i = 0; i < s.inst.size(); ++i) {
        if (s.inst[i].identity || s.flattened) continue;
        const Bvh& b = s.blas[s.inst[i].blas];
        if (b.nodes.empty()) continue;
        Aabb ob = b.nodes[0].box, wb;
        for (int c = 0; c < 8; ++c) {
            float p[3] = {(c & 1) ? ob.hi[0] : ob.lo[0], (c & 2) ? ob.hi[1] : ob.lo[1], (c & 4) ? ob.hi[2] : ob.lo[2]};
            vec3 q = mul34(s.inst[i].xf, vec4(p[0], p[1], p[2], 1.0f));
            float qq[3] = {q.x, q.y, q.z};
            wb.grow(qq);
        }
        // one ulp of slack on each side: world boxes are computed in float
        for (int k = 0; k < 3; ++k) {
            wb.lo[k] = std::nextafter(wb.lo[k], -INFINITY);
            wb.hi[k] = std::nextafter(wb.hi[k], INFINITY);
        }
        s.tlas_entries.push_back((int32_t)i);
        tboxes.push_back(wb);
    }
    s.tlas = Bvh();
    if (!tboxes.empty()) build_bvh(tboxes, s.tlas);
    s.built = !tboxes.empty();
}

inline uint8_t to_unorm8(float c) {  // float -> UNORM8, round to nearest
    c = std::min(std::max(c, 0.0f), 1.0f);
    return (uint8_t)std::floor(c * 255.0f + 0.5f);
}

}  // namespace

// ===========================================================================
// C API
// ===========================================================================
extern "C" {

orc_scene* orc_scene_create(const gbrt_vertex* v, uint32_t nv, const uint32_t* idx, uint32_t ni,
                            const gbrt_priminfo* prims, uint32_t ngeo, const gbrt_material_raw* mats,
                            uint32_t nmat, const gbrt_texture_desc* tex, uint32_t ntex) {
    orc_scene* s = new orc_scene();
    s->base_vertices.assign(v, v + nv);
    s->vertices = s->base_vertices;
    s->indices.assign(idx, idx + ni);
    s->prims.assign(prims, prims + ngeo);
    s->mats.assign(mats, mats + nmat);
    s->textures.resize(ntex);
    for (uint32_t i = 0; i < ntex; ++i) {
        Texture& t = s->textures[i];
        t.w = tex[i].width;
        t.h = tex[i].height;
        t.format = tex[i].format;
        t.wrap_s = tex[i].wrap_s;
        t.wrap_t = tex[i].wrap_t;
        size_t bytes = (size_t)t.w * t.h * (t.format == GBRT_TEX_RGBA32F ? 16 : t.format == GBRT_TEX_RGBA16F ? 8 : 4);
        if (tex[i].data && bytes) {
            const uint8_t* p = static_cast<const uint8_t*>(tex[i].data);
            t.data.assign(p, p + bytes);
        } else {
            t.w = t.h = 0;
        }
    }
    return s;
}

void orc_scene_destroy(orc_scene* s) { delete s; }

int orc_blas_build(orc_scene* s, const gbrt_geo_range* r, uint32_t n) {
    uint32_t ngeo = (uint32_t)s->prims.size();
    s->ranges.assign(ngeo, gbrt_geo_range{0, 0, 0, 1});
    s->geo_opaque.assign(ngeo, 1);
    for (uint32_t i = 0; i < n; ++i) {
        if (r[i].geo_id >= ngeo || r[i].i_len % 3 != 0) return GBRT_E_INVALID;
        s->ranges[r[i].geo_id] = r[i];
        s->geo_opaque[r[i].geo_id] = r[i].opaque ? 1 : 0;
    }
    return GBRT_OK;
}

int orc_build_flags(orc_scene* s, uint32_t flags) {
    s->build_flags = flags;
    return GBRT_OK;
}

int orc_tlas_build(orc_scene* s, const gbrt_instance* in, uint32_t n) {
    s->inst.resize(n);
    s->blas_needed.assign(s->prims.size(), 0);
    for (uint32_t i = 0; i < n; ++i) {
        Instance& I = s->inst[i];
        std::memcpy(I.xf, in[i].transform, sizeof(I.xf));
        I.custom = in[i].custom_index_and_mask & 0xFFFFFFu;
        I.mask = in[i].custom_index_and_mask >> 24;
        I.blas = (uint32_t)in[i].blas_handle;
        if (I.blas >= s->prims.size() || I.custom >= s->prims.size()) return GBRT_E_INVALID;
        static const float id[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
        I.identity = std::memcmp(I.xf, id, sizeof(id)) == 0 && (I.mask & 0xFFu) != 0;
        affine_inverse(I.xf, I.inv);
        if (!I.identity) s->blas_needed[I.blas] = 1;
    }
    rebuild(*s);
    return GBRT_OK;
}

int orc_lights_set(orc_scene* s, const gbrt_light_raw* d, uint32_t nd, const gbrt_light_raw* p, uint32_t np) {
    s->dlights.assign(d, d + nd);
    s->plights.assign(p, p + np);
    return GBRT_OK;
}

int orc_skybox_set(orc_scene* s, uint32_t face_size, const uint8_t* faces) {
    return orc_skybox_set_ex(s, face_size, faces, GBRT_TEX_RGBA8_SRGB);
}

// Cube faces as RGBA8 sRGB (the reference's decoded JPEG faces) or linear
// RGBA32F (an HDR extension of the GB300 library).
int orc_skybox_set_ex(orc_scene* s, uint32_t face_size, const void* faces_v, uint32_t format) {
    if (format != GBRT_TEX_RGBA8_SRGB && format != GBRT_TEX_RGBA32F) return GBRT_E_INVALID;
    const uint8_t* faces = static_cast<const uint8_t*>(faces_v);
    s->sky_size = faces ? face_size : 0;
    s->sky_faces.clear();
    if (!faces) return GBRT_OK;
    size_t fb = (size_t)face_size * face_size * (format == GBRT_TEX_RGBA32F ? 16 : 4);
    s->sky_faces.resize(6);
    for (int f = 0; f < 6; ++f) {
        Texture& t = s->sky_faces[f];
        t.w = t.h = face_size;
        t.format = format;
        t.wrap_s = t.wrap_t = GBRT_WRAP_CLAMP_TO_EDGE;
        t.data.assign(faces + f * fb, faces + (f + 1) * fb);
    }
    return GBRT_OK;
}

// AnimationCompute.comp:14-39.
int orc_skin(orc_scene* s, const gbrt_skin_raw* skins, uint32_t nskin) {
    for (size_t i = 0; i < s->base_vertices.size(); ++i) {
        gbrt_vertex v = s->base_vertices[i];
        int skin_index = v.skin_index;
        if (skin_index >= 0) {
            if ((uint32_t)skin_index >= nskin) return GBRT_E_INVALID;
            const gbrt_skin_raw& skin = skins[skin_index];
            float m[16];
            const float w[4] = {v.weights[0], v.weights[1], v.weights[2], v.weights[3]};
            for (int k = 0; k < 16; ++k) {
                m[k] = w[0] * skin.joints[v.joints[0] & 255][k] + w[1] * skin.joints[v.joints[1] & 255][k] +
                       w[2] * skin.joints[v.joints[2] & 255][k] + w[3] * skin.joints[v.joints[3] & 255][k];
            }
            vec4 pos = mul(m, vec4(v.pos[0], v.pos[1], v.pos[2], 1.0f));
            v.pos[0] = pos.x; v.pos[1] = pos.y; v.pos[2] = pos.z;
            vec3 nn = normalize(mul(m, vec4(v.normal[0], v.normal[1], v.normal[2], 0.0f)).xyz());
            v.normal[0] = nn.x; v.normal[1] = nn.y; v.normal[2] = nn.z;
            float tw = v.tangent[3];
            vec4 tt = normalize(mul(m, vec4(v.tangent[0], v.tangent[1], v.tangent[2], 0.0f)));
            v.tangent[0] = tt.x; v.tangent[1] = tt.y; v.tangent[2] = tt.z; v.tangent[3] = tw;
        }
        s->vertices[i] = v;
    }
    if (!s->inst.empty()) rebuild(*s);
    return GBRT_OK;
}

int orc_get_vertices(orc_scene* s, gbrt_vertex* out, uint32_t nv) {
    if (nv != s->vertices.size()) return GBRT_E_INVALID;
    std::memcpy(out, s->vertices.data(), sizeof(gbrt_vertex) * nv);
    return GBRT_OK;
}

int orc_trace(orc_scene* s, const gbrt_ray* rays, uint32_t n, uint32_t flags, gbrt_hit* hits, int fp64,
              int nthreads, orc_stats* st) {
    auto t0 = std::chrono::steady_clock::now();
    uint64_t nodes = 0, tris = 0;
    int used = 1;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel reduction(+ : nodes, tris)
    {
#pragma omp single
        used = omp_get_num_threads();
#pragma omp for schedule(dynamic, 256)
#endif
        for (int64_t i = 0; i < (int64_t)n; ++i) {
            Counters c;
            HitT h;
            TraceCtx ctx{(uint32_t)i, 0, 0, 0};
            bool hit = fp64 ? trace<double>(*s, rays[i].org, rays[i].dir, rays[i].tmin, rays[i].tmax, flags, ctx, h, c)
                            : trace<float>(*s, rays[i].org, rays[i].dir, rays[i].tmin, rays[i].tmax, flags, ctx, h, c);
            gbrt_hit& o = hits[i];
            o.t = hit ? (float)h.t : -1.0f;
            o.u = hit ? h.u : 0.0f;
            o.v = hit ? h.v : 0.0f;
            o.instance_id = hit ? h.inst : ~0u;
            o.primitive_id = hit ? h.prim : ~0u;
            o.custom_index = hit ? h.geo : ~0u;
            nodes += c.nodes;
            tris += c.tris;
        }
#ifdef _OPENMP
    }
#endif
    if (st) {
        std::memset(st, 0, sizeof(*st));
        st->node_visits = nodes;
        st->tri_tests = tris;
        st->rays_camera = n;
        st->threads = (uint32_t)used;
        st->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    return GBRT_OK;
}

int orc_render(orc_scene* s, const gbrt_ubo* ubo, uint32_t W, uint32_t H, uint32_t row0, uint32_t row1,
               float* accum, uint8_t* out, float* sample_radiance, gbrt_hit* primary_hits, int fp64, int nthreads,
               orc_stats* st) {
    return orc_render_diag(s, ubo, W, H, row0, row1, accum, out, sample_radiance, primary_hits, nullptr, 0, fp64,
                           nthreads, st);
}

int orc_render_diag(orc_scene* s, const gbrt_ubo* ubo, uint32_t W, uint32_t H, uint32_t row0, uint32_t row1,
                    float* accum, uint8_t* out, float* sample_radiance, gbrt_hit* primary_hits, float* sample_margins,
                    uint32_t nudge_ulps, int fp64, int nthreads, orc_stats* st) {
    if (!s->built) return GBRT_E_NOT_BUILT;
    if (row1 > H || row0 > row1) return GBRT_E_INVALID;
#ifndef ORC_DIAG
    if (sample_margins || nudge_ulps) return GBRT_E_INVALID;  // diagnostics live in liboracle_diag.so
#endif
    auto t0 = std::chrono::steady_clock::now();
    const uint32_t ns = ubo->number_of_samples;
    const uint32_t sbase = ubo->total_number_of_samples - ns;
    uint64_t cam = 0, ext = 0, shadow = 0, shaded = 0, nodes = 0, tris = 0;
    int used = 1;
    const int64_t npix = (int64_t)(row1 - row0) * W;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel reduction(+ : cam, ext, shadow, shaded, nodes, tris)
    {
#pragma omp single
        used = omp_get_num_threads();
#pragma omp for schedule(dynamic, 16)
#endif
        for (int64_t k = 0; k < npix; ++k) {
            uint32_t y = row0 + (uint32_t)(k / W), x = (uint32_t)(k % W);
            size_t pix = (size_t)y * W + x;
            Counters c;
            FrameCtx f{s, ubo, x, y, 0, 0, fp64, &c};
            float rad_f[3] = {0, 0, 0};
            double rad_d[3] = {0, 0, 0};
            float last_t = 0.0f;
            for (uint32_t si = 0; si < ns; ++si) {
                gbrt_hit* ph = primary_hits ? &primary_hits[pix * ns + si] : nullptr;
                SampleDiag diag{{INFINITY, INFINITY}, nudge_ulps & 0xFFFFu,
                                nudge_seed(x, y, sbase + si) ^ (nudge_ulps * 0x9E3779B9u)};
#ifdef ORC_DIAG
                g_diag = (sample_margins || nudge_ulps) ? &diag : nullptr;
#endif
                vec3 r = fp64 ? raygen_sample<double>(f, x, y, W, H, sbase + si, ph, cam, ext, last_t)
                              : raygen_sample<float>(f, x, y, W, H, sbase + si, ph, cam, ext, last_t);
#ifdef ORC_DIAG
                g_diag = nullptr;
#endif
                if (sample_margins) {
                    sample_margins[(pix * ns + si) * 2] = diag.margin[0];
                    sample_margins[(pix * ns + si) * 2 + 1] = diag.margin[1];
                }
                if (sample_radiance) {
                    float* sr = &sample_radiance[(pix * ns + si) * 3];
                    sr[0] = r.x; sr[1] = r.y; sr[2] = r.z;
                }
                rad_f[0] += r.x; rad_f[1] += r.y; rad_f[2] += r.z;
                rad_d[0] += r.x; rad_d[1] += r.y; rad_d[2] += r.z;
            }
            shadow += f.shadow_rays;
            shaded += f.shaded;
            nodes += c.nodes;
            tris += c.tris;
            // rgen:132-166
            const bool accumulate = ubo->number_of_samples != ubo->total_number_of_samples;
            vec3 prev = (accumulate && accum) ? vec3(accum[4 * pix], accum[4 * pix + 1], accum[4 * pix + 2]) : vec3(0.0f);
            vec3 accumulated = fp64 ? vec3((float)((double)prev.x + rad_d[0]), (float)((double)prev.y + rad_d[1]),
                                           (float)((double)prev.z + rad_d[2]))
                                    : prev + vec3(rad_f[0], rad_f[1], rad_f[2]);
            vec3 radiance = accumulated / float(ubo->total_number_of_samples);
            vec3 color = tonemap(ubo->tone_mapping_mode, radiance);
            if (ubo->mapping == DISTANCE)
                color = vec3(std::min((ubo->heatmap_scale - std::max(last_t, tMinC)) / ubo->heatmap_scale, 1.0f));
            if (accum) {
                accum[4 * pix] = accumulated.x;
                accum[4 * pix + 1] = accumulated.y;
                accum[4 * pix + 2] = accumulated.z;
                accum[4 * pix + 3] = 0.0f;
            }
            if (out) {
                out[4 * pix] = to_unorm8(color.x);
                out[4 * pix + 1] = to_unorm8(color.y);
                out[4 * pix + 2] = to_unorm8(color.z);
                out[4 * pix + 3] = 255;
            }
        }
#ifdef _OPENMP
    }
#endif
    if (st) {
        st->rays_camera = cam;
        st->rays_extension = ext;
        st->rays_shadow = shadow;
        st->hits_shaded = shaded;
        st->node_visits = nodes;
        st->tri_tests = tris;
        st->threads = (uint32_t)used;
        st->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    return GBRT_OK;
}

void orc_pcg4d(const uint32_t in[4], uint32_t out[4]) {
    uvec4 r = pcg4d(uvec4(in[0], in[1], in[2], in[3]));
    out[0] = r.x; out[1] = r.y; out[2] = r.z; out[3] = r.w;
}
uint32_t orc_tea(uint32_t a, uint32_t b) { return InitRandomSeed(a, b); }
float orc_rand(uint32_t st[4]) {
    uvec4 s(st[0], st[1], st[2], st[3]);
    float r = rand(s);
    st[0] = s.x; st[1] = s.y; st[2] = s.z; st[3] = s.w;
    return r;
}
float orc_random_float(uint32_t* seed) { return RandomFloat(*seed); }
void orc_eval_combined_brdf(const float N[3], const float L[3], const float V[3], const float bc[3], float metallic,
                            float roughness, float ior, float out[3]) {
    MaterialBrdf m{};
    m.baseColor = vec3(bc[0], bc[1], bc[2]);
    m.metallic = metallic;
    m.roughness = roughness;
    m.ior = ior;
    m.transmission = 0.0f;
    m.specular_factor = 1.0f;
    m.specular_color_factor = vec3(1.0f);
    m.frontFace = true;
    matBuild(m);
    vec3 r = evalCombinedBRDF(vec3(N[0], N[1], N[2]), vec3(L[0], L[1], L[2]), vec3(V[0], V[1], V[2]), m);
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}
void orc_tonemap(uint32_t mode, const float in[3], float out[3]) {
    vec3 r = tonemap(mode, vec3(in[0], in[1], in[2]));
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}
void orc_offset_ray(const float p[3], const float n[3], float out[3]) {
    vec3 r = offset_ray(vec3(p[0], p[1], p[2]), vec3(n[0], n[1], n[2]));
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}
void orc_sample_texture(orc_scene* s, int32_t index, float u, float v, float out[4]) {
    vec4 r = texture(*s, index, vec2(u, v));
    out[0] = r.x; out[1] = r.y; out[2] = r.z; out[3] = r.w;
}
void orc_sample_skybox(orc_scene* s, const float dir[3], float out[3]) {
    vec3 r = sample_sky(*s, vec3(dir[0], dir[1], dir[2]));
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}
uint32_t orc_blend_hash(uint32_t instance, uint32_t prim, uint32_t tag) { return blend_hash(instance, prim, tag); }

}  // extern "C"

#ifdef ORC_DIAG
float glsl::diag_round(float r) { return nudged(r); }
#endif
