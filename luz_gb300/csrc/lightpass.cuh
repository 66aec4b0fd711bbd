// lightpass.cuh — the deferred light pass of one lit pixel (light.frag main), shared
// by the light pass kernel (lightpass.cu) and the batched frame kernel (batch.cu).
#pragma once
#include "internal.cuh"
#include "raygen.cuh"
#include "shadowmap.cuh"

namespace luz {

struct LightParams {
    const float4* surf;          // compacted lit pixels: (fragPos, pixel), (N, x | y << 16)
    const uint4* surf_mat;       // beside them: (albedo, material, emission, pixel) words
    const uint32_t* lit_count;
    const uint32_t* albedo;
    const float4* normal;
    const uint32_t* material;
    const uint32_t* emission;
    const uint32_t* shadow_bits;
    const uint32_t* ao_bits;
    const float* ao_denoised;
    const float4* denoised;      // kCompose: filtered (shadow ratio rgb, AO)
    float4* signal;              // kSplit: (S rgb, AO)
    float4* unshadowed;          // kSplit: written (U rgb, lit shadow fraction); kCompose: read
    const luz_light* lights;
    const uint32_t* light_slot;
    uint32_t light_count;
    uint32_t words;
    uint32_t ao_samples;
    int shadow_type;
    const DevShadowLight* shadow_lights;   // LUZ_SHADOW_MAP: per light, shadow_count of them
    uint32_t shadow_count;
    float cam[3];
    float ambient[3];
    float ambient_intensity;
    uint32_t width, height;
    float4* out;
    const float* srgb_lut;       // pow(i / 255, 2.2), i = 0..255: the albedo decode of light.frag:172
};

// The Cook-Torrance terms of light.frag:17-45 (DistributionGGX, GeometrySchlickGGX,
// GeometrySmith) are evaluated inline in light_pass_kernel, their quotients folded into
// one division per light: D * G / (4 NdotV NdotL + 1e-4) =
// a2 NdotV NdotL / (pi dd^2 gv gl (4 NdotV NdotL + 1e-4)).
constexpr float kInvPi = 1.0f / kPi;

// light.frag:47-49; pow(x, 5.0) evaluated as x^4 * x.
__device__ __forceinline__ V3 fresnel_schlick(float cos_theta, V3 F0) {
    float x = clamp01(1.0f - cos_theta);
    float x2 = x * x;
    float p5 = (x2 * x2) * x;
    return F0 + (V3{1.0f, 1.0f, 1.0f} - F0) * p5;
}

__device__ __forceinline__ float unorm8_to_float(uint32_t b) { return (float)b / 255.0f; }

// kCoherent: the planes were written earlier in the same launch (the batch frame
// kernel): read through L2, not the non-coherent read-only path.
template <bool kCoherent = false>
__device__ __forceinline__ uint32_t bit_at(const uint32_t* __restrict__ planes, uint32_t plane,
                                           uint32_t words, uint32_t pix) {
    const uint32_t* p = planes + (size_t)plane * words + (pix >> 5);
    return ((kCoherent ? __ldcg(p) : __ldg(p)) >> (pix & 31)) & 1u;
}

// Modes of the light pass. kPlain: light.frag main with the ray-traced shadow factors
// and AO from the bit planes. kDenoisedAo: the same with AO from the denoised plane.
// kSplit (the denoiser's input pass): the direct light twice, shadowed as light.frag
// sums it (S) and unshadowed (U, every shadow factor 0), written as (S, AO) and
// (U, unoccluded fraction of the shadow samples); no light-plane write. kCompose: the frame from the filtered
// shadow ratio R and AO: ambient * AO + U * R + emission.
enum : int { kPlain = 0, kDenoisedAo = 1, kSplit = 2, kCompose = 3 };

// light.frag main (light.frag:171-235) for lit pixel t of the compacted list, in mode
// kMode; lights: the frame's lights (a shared-memory copy or the device array).
// kCoherent: the G-buffer planes, the lit-pixel list and the hit/miss planes were
// written earlier in the same launch (the batch frame kernel) and are read through L2.
template <int kMode, bool kCoherent = false>
__device__ __forceinline__ void light_pass_pixel(const LightParams& P, const luz_light* lights, uint32_t t) {
    const V3 amb = V3{P.ambient[0], P.ambient[1], P.ambient[2]};
    // lit pixel t: fragPos is the G-buffer pass's DepthToWorld of this pixel
    // (light.frag:186), N its normal
    const float4* sp = P.surf + 2 * (size_t)t;
    const float4 s0 = kCoherent ? __ldcg(sp) : __ldg(sp), s1 = kCoherent ? __ldcg(sp + 1) : __ldg(sp + 1);
    const uint32_t pix = __float_as_uint(s0.w);
    const V3 N = V3{s1.x, s1.y, s1.z};
    // the pixel's G-buffer words, one 16-B record in list order
    const uint4 gw = kCoherent ? __ldcg(P.surf_mat + t) : __ldg(P.surf_mat + t);
    const uint32_t a8 = gw.x, m8 = gw.y, e8 = gw.z;
    V3 albedo = V3{__ldg(P.srgb_lut + (a8 & 0xFF)), __ldg(P.srgb_lut + ((a8 >> 8) & 0xFF)),
                     __ldg(P.srgb_lut + ((a8 >> 16) & 0xFF))};
    float roughness = unorm8_to_float(m8 & 0xFF);
    float metallic = unorm8_to_float((m8 >> 8) & 0xFF);
    float occlusion = unorm8_to_float((m8 >> 16) & 0xFF);
    V3 emission = V3{unorm8_to_float(e8 & 0xFF), unorm8_to_float((e8 >> 8) & 0xFF),
                     unorm8_to_float((e8 >> 16) & 0xFF)};
    const V3 p = V3{s0.x, s0.y, s0.z};
    V3 cam = V3{P.cam[0], P.cam[1], P.cam[2]};
    V3 V = normalize(cam - p);
    V3 F0 = V3{0.04f, 0.04f, 0.04f} * (1.0f - metallic) + albedo * metallic;
    V3 Lo = V3{0.0f, 0.0f, 0.0f};
    V3 Lu = V3{0.0f, 0.0f, 0.0f};   // kSplit: unshadowed direct light
    uint32_t hits_all = 0, slots_all = 0;   // kSplit: occluded shadow samples over all lights
    float shadow_sum = 0.0f;                // kSplit: sum of the shadow factors (other shadow types)
    // per-pixel parts of the Cook-Torrance terms (light.frag:17-49, 210-229)
    const float a = roughness * roughness, a2 = a * a;
    const float r1 = roughness + 1.0f, k = (r1 * r1) / 8.0f;
    const float NdotV = fmax_(dot(N, V), 0.0f);
    const float gv = NdotV * (1.0f - k) + k;                 // GeometrySchlickGGX(NdotV) denominator
    const V3 diffuse_albedo = albedo * ((1.0f - metallic) * kInvPi);
    // EvaluateShadow's origin (light.frag:138-139), used by the 2D shadow maps
    const V3 shadow_origin = p + N * fmax_(length(p - cam) * 0.01f, 0.05f);
    for (uint32_t i = 0; i < (kMode == kCompose ? 0u : P.light_count); ++i) {
        const luz_light& lt = lights[i];
        const V3 L = light_vector(lt, p);                    // light.frag:194-198
        const float attenuation = light_attenuation(lt, p, L);   // light.frag:199-208
        // EvaluateShadow (light.frag:137-169): ray-traced factor = hits / samples.
        float shadow = 1.0f;
        if (P.shadow_type == LUZ_SHADOW_RAYTRACING) {
            int ns = lt.num_shadow_samples;
            if (ns <= 0) {
                shadow = 0.0f;
            } else {
                uint32_t first = P.light_slot[i];
                uint32_t hits = 0;
                for (int s = 0; s < ns; ++s) hits += bit_at<kCoherent>(P.shadow_bits, first + s, P.words, pix);
                shadow = (float)hits / (float)ns;
                if constexpr (kMode == kSplit) {
                    hits_all += hits;
                    slots_all += (uint32_t)ns;
                }
            }
        } else if (P.shadow_type == LUZ_SHADOW_MAP && i < P.shadow_count && P.shadow_lights[i].faces) {
            shadow = shadow_map_factor(P.shadow_lights[i], p, shadow_origin);   // light.frag:147-164
        }
        if constexpr (kMode == kSplit) shadow_sum += shadow;
        V3 color = V3{lt.color[0], lt.color[1], lt.color[2]};
        V3 radiance = ((color * lt.intensity) * attenuation) * (1.0f - shadow);
        V3 H = normalize(V + L);
        const float NdotH = fmax_(dot(N, H), 0.0f);
        const float NdotL = fmax_(dot(N, L), 0.0f);
        const float dd = NdotH * NdotH * (a2 - 1.0f) + 1.0f;
        const float gl = NdotL * (1.0f - k) + k;
        V3 F = fresnel_schlick(clamp01(dot(H, V)), F0);
        // D * G / (4 NdotV NdotL + 1e-4) with D = a2 / (pi dd^2) and
        // G = NdotV NdotL / (gv gl), as one quotient
        const float spec_scale = (a2 * (NdotV * NdotL)) /
                                 ((kPi * dd * dd) * (gv * gl) * ((4.0f * NdotV) * NdotL + 0.0001f));
        V3 spec = F * spec_scale;
        V3 diffuse = (V3{1.0f, 1.0f, 1.0f} - F) * diffuse_albedo;
        Lo = Lo + (diffuse + spec) * radiance * NdotL;
        if constexpr (kMode == kSplit) Lu = Lu + (diffuse + spec) * ((color * lt.intensity) * attenuation) * NdotL;
    }
    float ao;
    if constexpr (kMode == kCompose) {
        const float4 d = P.denoised[pix], u = P.unshadowed[pix];
        Lo = V3{u.x * d.x, u.y * d.y, u.z * d.z};
        ao = d.w;
    } else if constexpr (kMode == kDenoisedAo) {
        ao = P.ao_denoised[pix];
    } else if (P.ao_samples == 0) {
        ao = 1.0f;
    } else {
        uint32_t misses = 0;
        for (uint32_t s = 0; s < P.ao_samples; ++s) misses += bit_at<kCoherent>(P.ao_bits, s, P.words, pix);
        ao = (float)misses / (float)P.ao_samples;
    }
    if constexpr (kMode == kSplit) {
        // the denoiser's shadow feature: the unoccluded fraction of all shadow samples of
        // the pixel (1 - hits / samples; with other shadow types 1 - the mean shadow factor)
        float lit_fraction = 1.0f;
        if (P.shadow_type == LUZ_SHADOW_RAYTRACING) {
            if (slots_all) lit_fraction = 1.0f - (float)hits_all / (float)slots_all;
        } else if (P.light_count) {
            lit_fraction = 1.0f - shadow_sum / (float)P.light_count;
        }
        P.signal[pix] = make_float4(Lo.x, Lo.y, Lo.z, ao);
        P.unshadowed[pix] = make_float4(Lu.x, Lu.y, Lu.z, lit_fraction);
        return;
    }
    V3 ambient = (((amb * P.ambient_intensity) * albedo) * occlusion) * ao;
    V3 c = (ambient + Lo) + emission;
    P.out[pix] = make_float4(c.x, c.y, c.z, 1.0f);
}


}  // namespace luz
