// shade.cuh — device restatement of rustracer's shader libraries:
// Random.glsl (RNG), PBR.glsl (GGX + Frostbite diffuse), Material.glsl,
// PunctualLight.glsl, Tonemapping.glsl and RayTracingCommons.glsl helpers.
// Paths are relative to crates/examples/gltf_viewer/shaders/.
#pragma once
#include <cuda_fp16.h>
#include "scene.cuh"

namespace gbrt {

// ---------------------------------------------------------------------------
// Random.glsl
// ---------------------------------------------------------------------------
GB_HD uint32_t tea16(uint32_t v0, uint32_t v1) {  // InitRandomSeed, Random.glsl:12-25
    uint32_t s0 = 0;
#pragma unroll
    for (uint32_t n = 0; n < 16; n++) {
        s0 += 0x9e3779b9u;
        v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + s0) ^ ((v1 >> 5) + 0xc8013ea4u);
        v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + s0) ^ ((v0 >> 5) + 0x7e95761eu);
    }
    return v0;
}
GB_HD uint32_t lcg_next(uint32_t& seed) { return (seed = 1664525u * seed + 1013904223u); }  // :27-31
GB_HD float lcg_float(uint32_t& seed) {                                                  // :33-42
    return float(lcg_next(seed) & 0x00FFFFFFu) / float(0x01000000);
}
GB_HD float2 unit_disk(uint32_t& seed) {  // RandomInUnitDisk, :44-54
    for (;;) {
        float a = lcg_float(seed);
        float b = lcg_float(seed);
        float px = 2.0f * a - 1.0f, py = 2.0f * b - 1.0f;
        if (px * px + py * py < 1.0f) return make_float2(px, py);
    }
}
GB_HD float3 unit_sphere(uint32_t& seed) {  // RandomInUnitSphere, :56-66
    for (;;) {
        float a = lcg_float(seed);
        float b = lcg_float(seed);
        float c = lcg_float(seed);
        float3 p = f3(2.0f * a - 1.0f, 2.0f * b - 1.0f, 2.0f * c - 1.0f);
        if (dot(p, p) < 1.0f) return p;
    }
}
GB_HD float u2f(uint32_t x) {  // uintToFloat, :70-72
#ifdef __CUDA_ARCH__
    return __uint_as_float(0x3f800000u | (x >> 9)) - 1.0f;
#else
    union { uint32_t u; float f; } c;
    c.u = 0x3f800000u | (x >> 9);
    return c.f - 1.0f;
#endif
}
GB_HD uint4 pcg4d(uint4 v) {  // Random.glsl:81-98
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
// rand, Random.glsl:102-105.  Only .x of pcg4d is used, but all four lanes
// feed it through the two mixing rounds.
GB_HD float pcg_rand(uint4& s) {
    s.w++;
    return u2f(pcg4d(s).x);
}
GB_HD uint32_t jenkins(uint32_t x) {  // Random.glsl:108-115
    x += x << 10;
    x ^= x >> 6;
    x += x << 3;
    x ^= x >> 11;
    x += x << 15;
    return x;
}
GB_HD float3 hash_color(uint32_t i) {  // hashAndColor, Random.glsl:119-125
    uint32_t h = jenkins(i);
    return f3(float(h & 0xFFu) / 255.0f, float((h >> 8) & 0xFFu) / 255.0f, float((h >> 16) & 0xFFu) / 255.0f);
}
// Stateless key of a BLEND any-hit draw (documented deviation D3).
GB_HD uint32_t blend_hash(uint32_t instance, uint32_t prim, uint32_t tag) {
    return jenkins(jenkins(jenkins(tag) ^ instance) ^ prim);
}

// ---------------------------------------------------------------------------
// PBR.glsl
// ---------------------------------------------------------------------------
constexpr uint32_t DIFFUSE_TYPE = 1, SPECULAR_TYPE = 2, TRANSMISSION_TYPE = 3;
#define GB_PI 3.141592653589f
#define GB_ONE_OVER_PI (1.0f / GB_PI)
#define GB_TWO_PI (2.0f * GB_PI)

struct MatBrdf {  // MaterialBrdf, PBR.glsl:173-193 (fields the math reads)
    float3 baseColor;
    float metallic, roughness, ior, transmission, specular_factor;
    float3 specular_color_factor, F0, F90, c_diff;
    bool frontFace, volume;
    float3 attenuation_color;
    float attenuation_distance;
};

struct BrdfData {  // PBR.glsl:13-45
    float3 specularF0, diffuseReflectance, F;
    float roughness, alpha, alphaSquared;
    float NdotL, NdotV, LdotH, NdotH, VdotH;
    bool Vbackfacing, Lbackfacing;
};

GB_D float schlick(float cosine, float refractionIndex) {  // PBR.glsl:48-53
    float r0 = (1.0f - refractionIndex) / (1.0f + refractionIndex);
    r0 *= r0;
    return r0 + (1.0f - r0) * powf(1.0f - cosine, 5.0f);
}
GB_D void mat_build(MatBrdf& m) {  // matBuild, PBR.glsl:195-206
    float factor = (m.ior - 1.0f) / (m.ior + 1.0f);
    m.F0 = fmin3(factor * factor * m.specular_color_factor, f3(1.0f)) * m.specular_factor;  // dielectric F0
    float3 dF90 = m.specular_color_factor;
    m.F0 = mix3(m.F0, m.baseColor, m.metallic);
    m.F90 = mix3(dF90, f3(1.0f), m.metallic);
    m.c_diff = mix3(m.baseColor, f3(0.0f), m.metallic);
}
GB_D float saturatef(float x) { return clampf(x, 0.0f, 1.0f); }
GB_D float3 fresnel(float3 f0, float f90, float NdotS) {  // evalFresnelSchlick, :228-231
    return f0 + (f90 - f0) * powf(1.0f - NdotS, 5.0f);
}
GB_D float smith_g_a(float alpha, float NdotS) {  // :248-250
    return NdotS / (fmaxf(0.00001f, alpha) * sqrtf(1.0f - fminf(0.99999f, NdotS * NdotS)));
}
GB_D float smith_lambda_ggx(float a) { return (-1.0f + sqrtf(1.0f + (1.0f / (a * a)))) * 0.5f; }  // :253-255
GB_D float smith_g2_hc(float alpha, float NdotL, float NdotV) {  // :258-262
    float aL = smith_g_a(alpha, NdotL);
    float aV = smith_g_a(alpha, NdotV);
    return 1.0f / (1.0f + smith_lambda_ggx(aL) + smith_lambda_ggx(aV));
}
GB_D float ggx_d(float a2, float NdotH) {  // :286-289
    float b = ((a2 - 1.0f) * NdotH * NdotH + 1.0f);
    return a2 / (GB_PI * b * b);
}
GB_D float3 eval_microfacet(const BrdfData& d) {  // :292-303
    float D = ggx_d(fmaxf(0.00001f, d.alphaSquared), d.NdotH);
    float G2 = smith_g2_hc(d.alpha, d.NdotL, d.NdotV);
    return ((d.F * G2 * D) / (4.0f * d.NdotL * d.NdotV)) * d.NdotL;
}
GB_D float shadowed_f90(float3 F90) { return fminf(1.0f, luminance(F90)); }  // :312-322

struct BrdfProb { float specular, diffuse, transmission; };
GB_D BrdfProb brdf_probability(const MatBrdf& m, float3 V, float3 N) {  // getBrdfProbability, :324-358
    float specularF0 = luminance(m.F0);
    float diffuseReflectance = luminance(m.c_diff);
    float Fr = saturatef(luminance(fresnel(f3(specularF0), shadowed_f90(m.F90), fmaxf(0.0f, dot(V, N)))));
    float specular = Fr * m.specular_factor;
    float penetration = diffuseReflectance * (1.0f - m.specular_factor * Fr);
    float diffuse = penetration * (1.0f - m.transmission);
    float transmission = penetration * m.transmission;
    float sum = fmaxf(0.0001f, (specular + diffuse + transmission));
    float p = clampf(specular / sum, 0.001f, 0.9f);
    float d = (1.0f - p) * (1.0f - m.transmission);
    float t = (1.0f - p) * m.transmission;
    sum = p + d + t;
    return BrdfProb{p / sum, d / sum, t / sum};
}
GB_D float4 rotation_to_z(float3 v) {  // getRotationToZAxis, :362-368
    if (v.z < -0.99999f) return f4(1.0f, 0.0f, 0.0f, 0.0f);
    return normalize4(f4(v.y, -v.x, 0.0f, 1.0f + v.z));
}
GB_D float3 rotate_point(float4 q, float3 v) {  // :373-376
    const float3 a = f3(q.x, q.y, q.z);
    return 2.0f * dot(a, v) * a + (q.w * q.w - dot(a, a)) * v + 2.0f * q.w * cross(a, v);
}
// sampleGGXVNDF, :413-436, given the polar sample t1 = sqrt(u.x) cos(2 pi u.y),
// t2 = sqrt(u.x) sin(2 pi u.y) (eval_indirect draws it once for both lobes).
GB_D float3 sample_ggx_vndf_polar(float3 Ve, float alpha, float t1, float t2) {
    float3 Vh = normalize3(f3(alpha * Ve.x, alpha * Ve.y, Ve.z));
    float lensq = Vh.x * Vh.x + Vh.y * Vh.y;
    float3 T1 = lensq > 0.0f ? f3(-Vh.y, Vh.x, 0.0f) * (1.0f / sqrtf(lensq)) : f3(1.0f, 0.0f, 0.0f);
    float3 T2 = cross(Vh, T1);
    float s = 0.5f * (1.0f + Vh.z);
    t2 = mixf(sqrtf(1.0f - t1 * t1), t2, s);
    float3 Nh = t1 * T1 + t2 * T2 + sqrtf(fmaxf(0.0f, 1.0f - t1 * t1 - t2 * t2)) * Vh;
    return normalize3(f3(alpha * Nh.x, alpha * Nh.y, fmaxf(0.0f, Nh.z)));
}
GB_D float smith_g1_ggx(float a2, float NdotS2) {  // Smith_G1_GGX(alpha, NdotS, a2, NdotS2), :446-448
    return 2.0f / (sqrtf(((a2 * (1.0f - NdotS2)) + NdotS2) / NdotS2) + 1.0f);
}
GB_D float g2_over_g1(float a2, float NdotL, float NdotV) {  // :470-474
    float G1V = smith_g1_ggx(a2, NdotV * NdotV);
    float G1L = smith_g1_ggx(a2, NdotL * NdotL);
    return G1L / (G1V + G1L - G1V * G1L);
}
GB_D float frostbite_diffuse(const BrdfData& d) {  // frostbiteDisneyDiffuse, :486-496
    float energyBias = 0.5f * d.roughness;
    float energyFactor = mixf(1.0f, 1.0f / 1.51f, d.roughness);
    float FD90MinusOne = energyBias + 2.0f * d.LdotH * d.LdotH * d.roughness - 1.0f;
    float FDL = 1.0f + (FD90MinusOne * powf(1.0f - d.NdotL, 5.0f));
    float FDV = 1.0f + (FD90MinusOne * powf(1.0f - d.NdotV, 5.0f));
    return FDL * FDV * energyFactor;
}
GB_D BrdfData prepare_brdf(float3 N, float3 L, float3 V, const MatBrdf& m) {  // prepareBRDFData, :527-564
    BrdfData d;
    float3 H = normalize3(L + V);
    float NdotL = dot(N, L);
    float NdotV = dot(N, V);
    d.Vbackfacing = (NdotV <= 0.0f);
    d.Lbackfacing = (NdotL <= 0.0f);
    d.NdotL = fminf(fmaxf(0.00001f, NdotL), 1.0f);
    d.NdotV = fminf(fmaxf(0.00001f, NdotV), 1.0f);
    d.LdotH = saturatef(dot(L, H));
    d.NdotH = saturatef(dot(N, H));
    d.VdotH = saturatef(dot(V, H));
    d.specularF0 = m.F0;
    d.diffuseReflectance = m.c_diff;
    d.roughness = m.roughness;
    d.alpha = m.roughness * m.roughness;
    d.alphaSquared = d.alpha * d.alpha;
    d.F = fresnel(d.specularF0, shadowed_f90(m.F90), d.VdotH);
    return d;
}
GB_D float3 eval_combined_brdf(float3 N, float3 L, float3 V, const MatBrdf& m) {  // :731-745
    const BrdfData d = prepare_brdf(N, L, V, m);
    if (d.Vbackfacing || d.Lbackfacing) return f3(0.0f);
    float3 specular = eval_microfacet(d);
    float3 diffuse = d.diffuseReflectance * (frostbite_diffuse(d) * GB_ONE_OVER_PI * d.NdotL);
    return diffuse + specular;
}
// evalIndirectCombinedBRDF, PBR.glsl:649-729 (with sampleSpecularMicrofacet,
// :587-616).  The vector written to dir is only meaningful on true.
GB_D bool eval_indirect(float2 u, float3 N, float3 Ng, float3 V, const MatBrdf& m, uint32_t type, float3& dir,
                        float3& weight, float& volume_dis) {
    if (dot(Ng, V) < 0.0f) return false;
    float4 q = rotation_to_z(N);
    float3 Vl = rotate_point(q, V);
    const float3 Nl = f3(0.0f, 0.0f, 1.0f);
    float3 Ll = f3(0.0f);
    if (type == DIFFUSE_TYPE || type == SPECULAR_TYPE) {
        // Both lobes start from the same polar sample of u (sampleHemisphere :381-394 and
        // sampleGGXVNDF :413-436 both take sqrt(u.x) and the angle 2 pi u.y) and from
        // prepareBRDFData, at the sampled direction for the diffuse lobe and at the normal for
        // the specular one; computing those once keeps the lanes of a warp together whichever
        // lobe each path chose.
        const bool diffuse = type == DIFFUSE_TYPE;
        const float ru = sqrtf(u.x);
        float su, cu;
        sincosf(GB_TWO_PI * u.y, &su, &cu);
        const float t1 = ru * cu, t2 = ru * su;
        if (diffuse) Ll = f3(t1, t2, sqrtf(1.0f - u.x));
        const BrdfData d = prepare_brdf(Nl, diffuse ? Ll : Nl, Vl, m);
        if (diffuse) {
            weight = (1.0f - m.specular_factor * d.F) * d.diffuseReflectance * frostbite_diffuse(d);
            weight *= (1.0f - m.transmission);
        } else {  // sampleSpecularMicrofacet, :587-616
            float3 Hl = d.alpha == 0.0f ? f3(0.0f, 0.0f, 1.0f) : sample_ggx_vndf_polar(Vl, d.alpha, t1, t2);
            Ll = reflect3(-Vl, Hl);
            float HdotL = fmaxf(0.00001f, fminf(1.0f, dot(Hl, Ll)));
            float NdotL = fmaxf(0.00001f, fminf(1.0f, Ll.z));
            float NdotV = fmaxf(0.00001f, fminf(1.0f, Vl.z));
            float3 F = fresnel(d.specularF0, shadowed_f90(m.F90), HdotL);
            weight = F * g2_over_g1(d.alphaSquared, NdotL, NdotV);
            weight *= m.specular_factor;
        }
    } else if (type == TRANSMISSION_TYPE) {
        if (m.volume) {
            const float eta = m.frontFace ? 1.0f / m.ior : m.ior;
            const float3 refr = refract3(-Vl, Nl, eta);
            if (is_zero3(refr)) {
                weight = f3(0.0f);
                return false;
            }
            Ll = refr;
        } else {
            Ll = -Vl;
        }
        weight = fmax3(f3(0.0f), m.c_diff * m.transmission);
        if (!m.frontFace && m.volume) {
            float dis = volume_dis;
            volume_dis = -1.0f;
            float3 sigma = f3(logf(m.attenuation_color.x), logf(m.attenuation_color.y), logf(m.attenuation_color.z)) /
                           m.attenuation_distance;
            float3 s = sigma * dis;
            float3 att = f3(expf(s.x), expf(s.y), expf(s.z));
            weight *= fmin3(att, f3(1.0f));
        }
    }
    if (luminance(weight) == 0.0f) return false;
    dir = normalize3(rotate_point(f4(-q.x, -q.y, -q.z, q.w), Ll));
    return true;
}

// ---------------------------------------------------------------------------
// Material.glsl, PunctualLight.glsl, Tonemapping.glsl
// ---------------------------------------------------------------------------
GB_D float convert_metallic(float3 diffuse, float3 specular, float maxSpecular) {  // Material.glsl:78-89
    float pd = sqrtf(0.299f * diffuse.x * diffuse.x + 0.587f * diffuse.y * diffuse.y + 0.114f * diffuse.z * diffuse.z);
    float ps = sqrtf(0.299f * specular.x * specular.x + 0.587f * specular.y * specular.y +
                     0.114f * specular.z * specular.z);
    if (ps < 0.04f) return 0.0f;
    float a = 0.04f;
    float b = pd * (1.0f - maxSpecular) / (1.0f - 0.04f) + ps - 2.0f * 0.04f;
    float c = 0.04f - ps;
    float D = fmaxf(b * b - 4.0f * a * c, 0.0f);
    return clampf((-b + sqrtf(D)) / (2.0f * a), 0.0f, 1.0f);
}
GB_D float3 light_intensity_at(const gbrt_light_raw& l, float dist) {  // PunctualLight.glsl:17-30
    float3 color = l.intensity * f3(l.color[0], l.color[1], l.color[2]);
    if (l.kind == 1u) {
        const float r2 = 0.25f;
        const float d2 = dist * dist;
        return color * (2.0f / (d2 + r2 + dist * sqrtf(d2 + r2)));
    }
    return color;
}
GB_HD float3 pow3(float3 c, float e) { return f3(powf(c.x, e), powf(c.y, e), powf(c.z, e)); }
GB_HD float3 uncharted_impl(float3 c) {  // Tonemapping.glsl:15-23
    const float A = 0.15f, B = 0.50f, C = 0.10f, D = 0.20f, E = 0.02f, F = 0.30f;
    return ((c * (A * c + C * B) + D * E) / (c * (A * c + B) + D * F)) - E / F;
}
GB_HD float3 tonemap(uint32_t mode, float3 c) {  // RayTracing.rgen:137-149 + Tonemapping.glsl
    const float inv_gamma = 1.0f / 2.2f;
    if (mode == 0) return pow3(c / (c + 1.0f), inv_gamma);
    if (mode == 1) {
        float3 x = uncharted_impl(c * 2.0f);
        float3 white = 1.0f / uncharted_impl(f3(11.2f));
        return pow3(x * white, inv_gamma);
    }
    if (mode == 2) {
        c = fmax3(f3(0.0f), c - f3(0.004f));
        return (c * (6.2f * c + 0.5f)) / (c * (6.2f * c + 1.7f) + 0.06f);
    }
    if (mode == 3) {
        const float A = 2.51f, B = 0.03f, C = 2.43f, D = 0.59f, E = 0.14f;
        return pow3(clamp3((c * (A * c + B)) / (c * (C * c + D) + E), 0.0f, 1.0f), inv_gamma);
    }
    return pow3(c, inv_gamma);
}
GB_HD uint8_t to_unorm8(float c) { return (uint8_t)floorf(clampf(c, 0.0f, 1.0f) * 255.0f + 0.5f); }

// offset_ray, RayTracingCommons.glsl:103-119.
GB_D float3 offset_ray(float3 p, float3 n) {
    const float origin = 1.0f / 32.0f, float_scale = 1.0f / 65536.0f, int_scale = 256.0f;
    int ox = (int)(n.x * int_scale), oy = (int)(n.y * int_scale), oz = (int)(n.z * int_scale);
    float px = __int_as_float(__float_as_int(p.x) + ((p.x < 0.0f) ? -ox : ox));
    float py = __int_as_float(__float_as_int(p.y) + ((p.y < 0.0f) ? -oy : oy));
    float pz = __int_as_float(__float_as_int(p.z) + ((p.z < 0.0f) ? -oz : oz));
    return f3(fabsf(p.x) < origin ? p.x + float_scale * n.x : px, fabsf(p.y) < origin ? p.y + float_scale * n.y : py,
              fabsf(p.z) < origin ? p.z + float_scale * n.z : pz);
}

// ---------------------------------------------------------------------------
// Texture sampling (software bilinear, no mips, Vulkan wrap rules; sRGB
// decoded per texel through a 256-entry table computed on the host).
// Arithmetic is unfused so the any-hit alpha test matches the CPU exactly.
// ---------------------------------------------------------------------------
static __constant__ float c_srgb_lut[256];  // filled per translation unit by its init function

GB_D int wrap_idx(int i, int n, uint32_t mode) {
    if (mode == GBRT_WRAP_CLAMP_TO_EDGE) return min(max(i, 0), n - 1);
    if (mode == GBRT_WRAP_MIRRORED_REPEAT) {
        int m = ((i % (2 * n)) + 2 * n) % (2 * n);
        return m < n ? m : 2 * n - 1 - m;
    }
    return ((i % n) + n) % n;
}
GB_D float half_bits_to_float(uint16_t h) { return __half2float(__ushort_as_half(h)); }
GB_D float4 tex_fetch(const DevTexture& t, int x, int y) {
    size_t k = (size_t)y * t.w + (size_t)x;
    if (t.format == GBRT_TEX_RGBA32F) return __ldg(reinterpret_cast<const float4*>(t.data) + k);
    if (t.format == GBRT_TEX_RGBA16F) {
        uint2 raw = __ldg(reinterpret_cast<const uint2*>(t.data) + k);
        return f4(half_bits_to_float(raw.x & 0xFFFF), half_bits_to_float(raw.x >> 16),
                  half_bits_to_float(raw.y & 0xFFFF), half_bits_to_float(raw.y >> 16));
    }
    uchar4 p = __ldg(reinterpret_cast<const uchar4*>(t.data) + k);
    if (t.format == GBRT_TEX_RGBA8_SRGB)
        return f4(c_srgb_lut[p.x], c_srgb_lut[p.y], c_srgb_lut[p.z], __fdiv_rn((float)p.w, 255.0f));
    return f4(__fdiv_rn((float)p.x, 255.0f), __fdiv_rn((float)p.y, 255.0f), __fdiv_rn((float)p.z, 255.0f),
              __fdiv_rn((float)p.w, 255.0f));
}
GB_D float lerp_rn(float a, float b, float f) { return add_rn(mul_rn(a, sub_rn(1.0f, f)), mul_rn(b, f)); }
GB_D float4 lerp4_rn(float4 a, float4 b, float f) {
    return f4(lerp_rn(a.x, b.x, f), lerp_rn(a.y, b.y, f), lerp_rn(a.z, b.z, f), lerp_rn(a.w, b.w, f));
}
GB_D float4 sample_tex2d(const DevTexture& t, float u, float v) {
    float x = sub_rn(mul_rn(u, (float)t.w), 0.5f);
    float y = sub_rn(mul_rn(v, (float)t.h), 0.5f);
    float fx = floorf(x), fy = floorf(y);
    float ax = sub_rn(x, fx), ay = sub_rn(y, fy);
    int i0 = (int)fx, j0 = (int)fy;
    int xa = wrap_idx(i0, t.w, t.wrap_s), xb = wrap_idx(i0 + 1, t.w, t.wrap_s);
    int ya = wrap_idx(j0, t.h, t.wrap_t), yb = wrap_idx(j0 + 1, t.h, t.wrap_t);
    float4 top = lerp4_rn(tex_fetch(t, xa, ya), tex_fetch(t, xb, ya), ax);
    float4 bot = lerp4_rn(tex_fetch(t, xa, yb), tex_fetch(t, xb, yb), ax);
    return lerp4_rn(top, bot, ay);
}
GB_D float4 texture(const DevScene& s, int idx, float2 uv) {
    if (idx < 0 || (uint32_t)idx >= s.ntex || s.tex[idx].w == 0) return f4(1.0f, 1.0f, 1.0f, 1.0f);
    return sample_tex2d(s.tex[idx], uv.x, uv.y);
}
GB_D float2 get_uv(float4 uv01, int index) {  // getUV, Commons.glsl:65-72
    if (index == 0) return make_float2(uv01.x, uv01.y);
    if (index == 1) return make_float2(uv01.z, uv01.w);
    return make_float2(0.0f, 0.0f);
}
// Cube map (Vulkan face selection; bilinear clamped inside the face).
GB_D float3 sample_sky(const DevScene& s, float3 d) {
    if (s.sky_size == 0) return f3(0.0f);
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
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
    DevTexture t;
    const size_t texel = s.sky_format == GBRT_TEX_RGBA32F ? 16u : 4u;
    t.data = static_cast<const unsigned char*>(s.sky) + (size_t)face * s.sky_size * s.sky_size * texel;
    t.w = t.h = s.sky_size;
    t.format = s.sky_format;
    t.wrap_s = t.wrap_t = GBRT_WRAP_CLAMP_TO_EDGE;
    float4 r = sample_tex2d(t, 0.5f * (sc / ma + 1.0f), 0.5f * (tc / ma + 1.0f));
    return f3(r.x, r.y, r.z);
}

}  // namespace gbrt
