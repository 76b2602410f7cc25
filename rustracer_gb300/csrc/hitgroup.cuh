// hitgroup.cuh — the reference's hit group on the device: ray payload,
// miss shader (RayTracing.rmiss), RIS light sampling and closest-hit shading
// (RayTracing.rchit), and the camera ray of RayTracing.rgen, shared by the
// megakernel and the wavefront kernels.
#pragma once
#include "trace.cuh"

namespace gbrt {

struct Payload {  // RayPayload, RayTracingCommons.glsl:11-24
    float3 hitValue, hitPoint, scatterDir, emittance;
    float t, volume_dis;
    uint32_t needScatter;
    uint32_t RandomSeed;
    uint4 rngState;
};

struct PathStats {
    uint32_t camera, extension, shadow, shaded, status;
};

GB_D float3 normal_xform(const float* T, float3 n) {  // normal_transform, RayTracing.rchit:28-30
    return normalize3(f3(T[0] * n.x + T[1] * n.y + T[2] * n.z, T[4] * n.x + T[5] * n.y + T[6] * n.z,
                         T[8] * n.x + T[9] * n.y + T[10] * n.z));
}
GB_D float3 point_xform(const float* T, float3 p) {
    return f3(T[0] * p.x + T[1] * p.y + T[2] * p.z + T[3], T[4] * p.x + T[5] * p.y + T[6] * p.z + T[7],
              T[8] * p.x + T[9] * p.y + T[10] * p.z + T[11]);
}
GB_D float3 ldg3(const float* p) { return f3(__ldg(p), __ldg(p + 1), __ldg(p + 2)); }
GB_D float4 ldg4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }

// RayTracing.rmiss:14-45.
GB_D void miss_shader(const DevScene& s, const gbrt_ubo& ubo, Payload& R, float3 dir) {
    float3 acc = f3(0.0f);
    const float3 rd = normalize3(dir);
    if (R.t != 0.0f) {
        for (uint32_t i = 0; i < s.nd; i++) {
            const gbrt_light_raw& li = s.dlights[i];
            const float c = dot(normalize3(f3(li.transform[0], li.transform[1], li.transform[2])), rd);
            if (c < 0.0f) acc += -c * f3(li.color[0], li.color[1], li.color[2]) * li.intensity;
        }
    }
    if (ubo.has_sky) {
        const float3 sky = sample_sky(s, rd);
        acc += sky + acc;
    } else {
        acc += f3(0.01f);
    }
    R.hitValue = f3(0.0f);
    R.needScatter = 0;
    R.emittance = s.nd == 0 ? f3(0.0f) : acc;
    R.t = -1.0f;
}

// sampleLightUniform + sampleLightRIS, RayTracing.rchit:62-122.
GB_D bool sample_light_ris(const DevScene& s, uint4& rng, float3 P, float3 Ng, gbrt_light_raw& sel, float& w) {
    const uint32_t n = s.np;
    if (n == 0) return false;
    float total = 0.0f, pdf_sel = 0.0f;
    const uint32_t cand = n < 3u ? n : 3u;
    for (uint32_t i = 0; i < cand; i++) {
        const gbrt_light_raw& li = s.plights[i];
        if (luminance(f3(li.color[0], li.color[1], li.color[2]) * li.intensity) < 0.1f) continue;
        const uint32_t idx = min(n - 1, (uint32_t)(pcg_rand(rng) * float(n)));
        const gbrt_light_raw& c = s.plights[idx];
        const float3 lv = f3(c.transform[0], c.transform[1], c.transform[2]) - P;
        const float3 L = normalize3(lv);
        if (dot(Ng, L) < 0.00001f) continue;
        const float pdfG = luminance(light_intensity_at(c, len3(lv)));
        const float ris = pdfG * float(n);
        total += ris;
        if (pcg_rand(rng) < (ris / total)) {
            sel = c;
            pdf_sel = pdfG;
        }
    }
    if (total == 0.0f) return false;
    w = (total / 3.0f) / pdf_sel;
    return true;
}

// RayTracing.rchit:136-477 for the hit h of a ray with world direction wdir.
// shadow(origin, dir, tmax, C) handles the NEE shadow ray: it must add C to
// R.emittance when the light is unoccluded (the megakernel traces it at once,
// the wavefront defers it to the any-hit kernel).  kFeat (kFeat* bits) lists
// the material features compiled in; the caller picks a form that covers the
// scene's DevScene::shade_feat and the frame's debug settings.
template <uint32_t kFeat = kFeatAll, class ShadowFn>
GB_D void closest_hit(const DevScene& s, const gbrt_ubo& ubo, Payload& R, const Hit& h, float3 wdir, PathStats& ps,
                      ShadowFn&& shadow) {
    constexpr bool kTex = (kFeat & kFeatTextures) != 0;
    constexpr bool kVol = (kFeat & kFeatVolume) != 0;
    ps.shaded++;
    const DevInstance& in = s.inst[h.inst];
    const uint32_t custom = in.custom;
    float T[12];
    if (in.identity) {
#pragma unroll
        for (int k = 0; k < 12; ++k) T[k] = (k % 5 == 0) ? 1.0f : 0.0f;
    } else {
#pragma unroll
        for (int k = 0; k < 12; ++k) T[k] = in.xf[k];
    }
    const gbrt_priminfo pi = s.prims[custom];
    const gbrt_material_raw& mat = s.mats[pi.material_id];
    const float3 last_hit = R.hitPoint;
    R.t = h.t;
    const uint32_t io = pi.i_offset + 3u * h.prim;
    const gbrt_vertex* v0 = s.vertices + pi.v_offset + s.indices[io];
    const gbrt_vertex* v1 = s.vertices + pi.v_offset + s.indices[io + 1];
    const gbrt_vertex* v2 = s.vertices + pi.v_offset + s.indices[io + 2];
    // getMixVertexAndGeoNormal, RayTracingCommons.glsl:82-97
    const float b0 = 1.0f - h.u - h.v, b1 = h.u, b2 = h.v;
    const float4 uv0 = f4(__ldg(&v0->uv0[0]), __ldg(&v0->uv0[1]), __ldg(&v0->uv1[0]), __ldg(&v0->uv1[1]));
    const float4 uv1 = f4(__ldg(&v1->uv0[0]), __ldg(&v1->uv0[1]), __ldg(&v1->uv1[0]), __ldg(&v1->uv1[1]));
    const float4 uv2 = f4(__ldg(&v2->uv0[0]), __ldg(&v2->uv0[1]), __ldg(&v2->uv1[0]), __ldg(&v2->uv1[1]));
    const float4 uv01 = uv0 * b0 + uv1 * b1 + uv2 * b2;
    // pos and normal are the first two 16-byte fields of the 128-byte vertex: one vector load each
    const float3 p0 = f3(ldg4(v0->pos)), p1 = f3(ldg4(v1->pos)), p2 = f3(ldg4(v2->pos));
    const float3 pos = p0 * b0 + p1 * b1 + p2 * b2;
    const float4 col = ldg4(v0->color) * b0 + ldg4(v1->color) * b1 + ldg4(v2->color) * b2;
    float3 normal = normalize3(normalize3(f3(ldg4(v0->normal))) * b0 + normalize3(f3(ldg4(v1->normal))) * b1 +
                               normalize3(f3(ldg4(v2->normal))) * b2);
    const float4 tangent = normalize4(ldg4(v0->tangent) * b0 + ldg4(v1->tangent) * b1 + ldg4(v2->tangent) * b2);
    float3 Ng = normal_xform(T, cross(p1 - p0, p2 - p0));
    float3 origin = point_xform(T, pos);

    float4 color4 = col * f4(mat.base_color[0], mat.base_color[1], mat.base_color[2], mat.base_color[3]);
    if (kTex && mat.base_color_texture.index >= 0)
        color4 = color4 * texture(s, mat.base_color_texture.index, get_uv(uv01, mat.base_color_texture.coord));
    float3 color = f3(color4);
    R.needScatter = 0;
    R.hitPoint = pos;
    if (kTex && mat.normal_texture.index >= 0) {  // getNormal, rchit:124-129,180-185
        const float4 tn = texture(s, mat.normal_texture.index, get_uv(uv01, mat.normal_texture.coord));
        const float3 nt = normalize3(f3(tn) * 2.0f - 1.0f);
        const float3 tm = f3(tangent);
        const float3 tg = normalize3(tm - dot(tm, normal) * normal);
        const float3 bt = normalize3(cross(normal, tg) * tangent.w);
        normal = tg * nt.x + bt * nt.y + normal * nt.z;
    }
    normal = normal_xform(T, normal);
    const float3 V = -normalize3(wdir);
    const float cosv = dot(V, Ng);
    const bool frontFace = cosv >= 0.0f;
    Ng = frontFace ? Ng : -Ng;
    const float3 N = dot(Ng, normal) < 0.0f ? -normal : normal;  // outwardNormal

    float3 emittance = f3(mat.emissive_factor[0], mat.emissive_factor[1], mat.emissive_factor[2]);
    if (kTex && mat.emissive_texture.index >= 0)
        emittance *= f3(texture(s, mat.emissive_texture.index, get_uv(uv01, mat.emissive_texture.coord)));
    float metallic = mat.metallic_factor, roughness = mat.roughness_factor;
    if (kTex && mat.metallic_roughness_texture.index >= 0) {
        const float4 mr = texture(s, mat.metallic_roughness_texture.index,
                                  get_uv(uv01, mat.metallic_roughness_texture.coord));
        roughness *= mr.y;
        metallic *= mr.z;
    }
    float3 spec_wf = f3(1.0f);
    const bool sg = (kFeat & kFeatSpecGloss) && mat.workflow == 1u;
    if (sg) {  // rchit:216-239
        float4 df = ldg4(mat.sg_diffuse_factor);
        float4 sgf = ldg4(mat.sg_specular_glossiness_factor);
        if (kTex && mat.sg_diffuse_texture.index >= 0)
            df = df * texture(s, mat.sg_diffuse_texture.index, get_uv(uv01, mat.sg_diffuse_texture.coord));
        if (kTex && mat.sg_specular_glossiness_texture.index >= 0)
            sgf = sgf * texture(s, mat.sg_specular_glossiness_texture.index,
                                get_uv(uv01, mat.sg_specular_glossiness_texture.coord));
        spec_wf = f3(sgf);
        roughness = 1.0f - sgf.w;
        const float maxs = fmaxf(fmaxf(spec_wf.x, spec_wf.y), spec_wf.z);
        color = f3(col) * f3(df);
        metallic = convert_metallic(color, spec_wf, maxs);
    }
    float transmission = 0.0f;
    if (mat.transmission_exist) {
        transmission = mat.transmission_factor;
        if (kTex && mat.transmission_texture.index >= 0)
            transmission *= texture(s, mat.transmission_texture.index, get_uv(uv01, mat.transmission_texture.coord)).x;
    }
    uint32_t mapping = (kFeat & kFeatDebug) ? ubo.mapping : 0u;
    if ((kFeat & kFeatDebug) && mat.unlit) mapping = 5u;  // ALBEDO
    switch (mapping) {  // rchit:258-286
        case 5: R.emittance = color; return;
        case 3: R.emittance = f3(1.0f - h.u - h.v, h.u, h.v); return;
        case 2: R.emittance = hash_color(h.inst); return;
        case 6: R.emittance = f3(metallic); return;
        case 7: R.emittance = f3(roughness); return;
        case 8: R.emittance = (N + 1.0f) / 2.0f; return;
        case 9: R.emittance = (normal_xform(T, f3(tangent)) + 1.0f) / 2.0f; return;
        case 10: R.emittance = f3(transmission); return;
        case 11: R.emittance = hash_color(custom); return;
        default: break;
    }
    float spec_factor = mat.specular_factor;
    float3 spec_color = f3(mat.specular_color_factor[0], mat.specular_color_factor[1], mat.specular_color_factor[2]);
    if (kTex && mat.specular_texture.index >= 0)
        spec_factor *= texture(s, mat.specular_texture.index, get_uv(uv01, mat.specular_texture.coord)).w;
    if (kTex && mat.specular_color_texture.index >= 0)
        spec_color *= f3(texture(s, mat.specular_color_texture.index, get_uv(uv01, mat.specular_color_texture.coord)));

    R.hitPoint = origin;
    uint32_t seed = R.RandomSeed;
    uint4 rng = R.rngState;
    R.emittance = emittance * ubo.exposure;
    R.needScatter = 0;
    float3 throughput = f3(1.0f);
    MatBrdf m;
    m.baseColor = color;
    m.metallic = metallic;
    m.roughness = roughness;
    m.ior = mat.volume_exists ? mat.ior : 1.0f;
    m.transmission = transmission;
    m.specular_factor = spec_factor;
    m.specular_color_factor = spec_color;
    m.frontFace = frontFace;
    mat_build(m);
    if (sg) {
        const float maxs = fmaxf(fmaxf(spec_wf.x, spec_wf.y), spec_wf.z);
        m.c_diff = color * (1.0f - maxs);
        m.F0 = spec_wf;
    }
    m.attenuation_color = f3(mat.attenuation_color[0], mat.attenuation_color[1], mat.attenuation_color[2]);
    m.attenuation_distance = mat.attenuation_distance;
    m.volume = kVol && mat.volume_exists != 0;
    const float displacement = len3(origin - last_hit);

    gbrt_light_raw light;
    float lw;
    if (sample_light_ris(s, rng, origin, Ng, light, lw)) {  // rchit:338-350
        float3 lv = f3(light.transform[0], light.transform[1], light.transform[2]) - origin;
        const float ld = len3(lv);
        lv = normalize3(lv);
        ps.shadow++;
        shadow(origin, lv, ld,
               eval_combined_brdf(N, lv, V, m) * lw * light.intensity * f3(light.color[0], light.color[1], light.color[2]));
    }
    uint32_t type;
    if (metallic == 1.0f && roughness == 0.0f) {  // rchit:352-395
        type = SPECULAR_TYPE;
    } else {
        const BrdfProb p = brdf_probability(m, V, N);
        const float r = pcg_rand(rng);
        if (r < p.specular) {
            type = SPECULAR_TYPE;
            throughput /= p.specular;
            if (R.volume_dis >= 0.0f) R.volume_dis += displacement;
        } else if (r >= p.specular && r <= p.specular + p.diffuse) {
            type = DIFFUSE_TYPE;
            throughput /= p.diffuse;
            if (R.volume_dis >= 0.0f) R.volume_dis += displacement;
        } else {
            type = TRANSMISSION_TYPE;
            if (kVol && mat.volume_exists) {
                if (R.volume_dis >= 0.0f) R.volume_dis += displacement;
                else if (frontFace) R.volume_dis = 0.0f;
            }
            throughput /= p.transmission;
        }
    }
    if (type == TRANSMISSION_TYPE) origin = offset_ray(origin, -Ng);
    float3 w = f3(0.0f), dir = f3(0.0f);
    const float ua = pcg_rand(rng);
    const float ub = pcg_rand(rng);
    R.needScatter = eval_indirect(make_float2(ua, ub), N, Ng, V, m, type, dir, w, R.volume_dis) ? 1u : 0u;
    throughput *= w;
    R.hitPoint = origin;
    R.scatterDir = dir;
    R.hitValue = throughput;
    if ((kFeat & kFeatDebug) && ubo.debug == 1u) {  // rchit:437-474 (legacy branch, D5)
        if (m.transmission > 0.0f) {
            const float eta = frontFace ? 1.0f / mat.ior : mat.ior;
            const float3 refr = refract3(wdir, N, eta);
            const float rp = !is_zero3(refr) ? schlick(fabsf(cosv), eta) : 1.0f;
            R.hitValue = color;
            R.needScatter = 1;
            R.scatterDir = lcg_float(seed) < rp ? reflect3(wdir, normal) : refr;
        } else if (len3(emittance) < 0.01f && roughness == 1.0f) {
            const bool sc = dot(wdir, Ng) < 0.0f;
            const float3 d = normalize3(N + unit_sphere(seed));
            R.needScatter = sc;
            R.scatterDir = d;
            R.hitValue = sc ? color : f3(0.0f);
        } else if (metallic > 0.0f) {
            const float3 rf = reflect3(wdir, N);
            const bool sc = dot(rf, Ng) > 0.0f;
            R.needScatter = sc;
            R.hitValue = sc ? color : f3(0.0f);
            R.scatterDir = rf + 0.08f * unit_sphere(seed);
        }
    }
    R.RandomSeed = seed;
    R.rngState = rng;
}

// One sample of RayTracing.rgen:49-130; returns its radiance.

// Camera ray of RayTracing.rgen:52-75 for pixel (x, y) and global sample
// index `sample` (documented deviation D1 seeds).  Rounded step by step like
// the oracle, so primary rays -- and their hits -- are bit-identical.
// Advances the pixel stream `rng` (anti-aliasing draws) and RandomSeed
// (aperture disk draws).
GB_D void camera_ray(const gbrt_ubo& ubo, uint32_t x, uint32_t y, uint32_t W, uint32_t H, uint4& rng,
                     uint32_t& RandomSeed, float3& o, float3& d, float& tFar) {
    float2 pixel = make_float2(add_rn(float(x), 0.5f), add_rn(float(y), 0.5f));
    if (ubo.antialiasing) {
        const float ra = pcg_rand(rng);
        const float rb = pcg_rand(rng);
        pixel.x = add_rn(pixel.x, sub_rn(ra, 0.5f));
        pixel.y = add_rn(pixel.y, sub_rn(rb, 0.5f));
    }
    const float2 uv = make_float2(sub_rn(mul_rn(__fdiv_rn(pixel.x, float(W)), 2.0f), 1.0f),
                                  sub_rn(mul_rn(__fdiv_rn(pixel.y, float(H)), 2.0f), 1.0f));
    const float2 disk = unit_disk(RandomSeed);
    const float half_ap = __fdiv_rn(ubo.aperture, 2.0f);
    const float2 off = make_float2(mul_rn(half_ap, disk.x), mul_rn(half_ap, disk.y));
    float4 origin = mat4_mul_rn(ubo.model_view_inverse, f4(off.x, off.y, 0.0f, 1.0f));
    const float4 target = mat4_mul_rn(ubo.projection_inverse, f4(uv.x, uv.y, 1.0f, 1.0f));
    const float3 tv = f3(sub_rn(mul_rn(target.x, ubo.focus_distance), off.x),
                         sub_rn(mul_rn(target.y, ubo.focus_distance), off.y),
                         sub_rn(mul_rn(target.z, ubo.focus_distance), 0.0f));
    float4 direction = mat4_mul_rn(ubo.model_view_inverse, f4(normalize3_rn(tv), 0.0f));
    tFar = 10000.0f;
    if (ubo.orthographic_fov_dis > 0.0f) {
        const float k = add_rn(1.0f, ubo.orthographic_fov_dis);
        origin = mat4_mul_rn(ubo.model_view_inverse, f4(mul_rn(k, uv.x), -mul_rn(k, uv.y), 0.0f, 1.0f));
        direction = mat4_mul_rn(ubo.model_view_inverse, f4(0.0f, 0.0f, -1.0f, 0.0f));
        tFar = 10.0f * 10000.0f;
    }
    o = f3(origin);
    d = f3(direction);
}

}  // namespace gbrt
