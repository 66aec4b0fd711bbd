// lightpass.cu — the deferred light pass: light.frag main (light.frag:171-235) over
// the G-buffer planes and the visibility bit planes. Thread t shades the t-th lit
// pixel of the compacted list the G-buffer pass wrote (world position and normal;
// every lane of a warp runs the same light loop). The pass that compacted that list
// wrote the background colour of the unlit pixels.
#include <cstring>

#include "internal.cuh"
#include "raygen.cuh"
#include "shadowmap.cuh"

namespace luz {

// pow(i/255, 2.2) for the albedo decode of light.frag:172, filled by the host.
__constant__ float c_srgb_lut[256];

luz_status upload_srgb_lut(luz_ctx* ctx, const float* lut) {
    LUZ_CUDA(ctx, cudaMemcpyToSymbol(c_srgb_lut, lut, 256 * sizeof(float)));
    return LUZ_OK;
}

struct LightParams {
    const float4* surf;          // compacted lit pixels: (fragPos, pixel), (N, x | y << 16)
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

__device__ __forceinline__ uint32_t bit_at(const uint32_t* __restrict__ planes, uint32_t plane,
                                           uint32_t words, uint32_t pix) {
    return (__ldg(planes + (size_t)plane * words + (pix >> 5)) >> (pix & 31)) & 1u;
}

// Modes of the light pass. kPlain: light.frag main with the ray-traced shadow factors
// and AO from the bit planes. kDenoisedAo: the same with AO from the denoised plane.
// kSplit (the denoiser's input pass): the direct light twice, shadowed as light.frag
// sums it (S) and unshadowed (U, every shadow factor 0), written as (S, AO) and
// (U, unoccluded fraction of the shadow samples); no light-plane write. kCompose: the frame from the filtered
// shadow ratio R and AO: ambient * AO + U * R + emission.
enum : int { kPlain = 0, kDenoisedAo = 1, kSplit = 2, kCompose = 3 };

template <int kMode>
__global__ void __launch_bounds__(256) light_pass_kernel(LightParams P) {
    extern __shared__ luz_light s_lights[];
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t lit = *P.lit_count;
    const V3 amb = V3{P.ambient[0], P.ambient[1], P.ambient[2]};
    // the background (light.frag:178-181) was written by the lit-list pass
    if (blockIdx.x * blockDim.x >= lit) return;   // no lit pixel in this block
    for (uint32_t i = threadIdx.x; i < P.light_count; i += blockDim.x) s_lights[i] = P.lights[i];
    __syncthreads();
    if (t >= lit) return;
    // lit pixel t: fragPos is the G-buffer pass's DepthToWorld of this pixel
    // (light.frag:186), N its normal
    const float4 s0 = __ldg(P.surf + 2 * (size_t)t), s1 = __ldg(P.surf + 2 * (size_t)t + 1);
    const uint32_t pix = __float_as_uint(s0.w);
    const V3 N = V3{s1.x, s1.y, s1.z};
    uint32_t a8 = P.albedo[pix], m8 = P.material[pix], e8 = P.emission[pix];
    V3 albedo = V3{c_srgb_lut[a8 & 0xFF], c_srgb_lut[(a8 >> 8) & 0xFF], c_srgb_lut[(a8 >> 16) & 0xFF]};
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
        const luz_light& lt = s_lights[i];
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
                for (int s = 0; s < ns; ++s) hits += bit_at(P.shadow_bits, first + s, P.words, pix);
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
        for (uint32_t s = 0; s < P.ao_samples; ++s) misses += bit_at(P.ao_bits, s, P.words, pix);
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

// AO value per pixel (mean of the miss bits; 0 for background pixels).
__global__ void __launch_bounds__(256) ao_resolve_kernel(const float4* normal, const uint32_t* ao_bits,
                                                         uint32_t words, uint32_t samples,
                                                         uint32_t pixels, float* ao) {
    uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= pixels) return;
    float4 nn = normal[pix];
    if (length(V3{nn.x, nn.y, nn.z}) == 0.0f) { ao[pix] = 0.0f; return; }
    if (samples == 0) { ao[pix] = 1.0f; return; }
    uint32_t misses = 0;
    for (uint32_t s = 0; s < samples; ++s) misses += bit_at(ao_bits, s, words, pix);
    ao[pix] = (float)misses / (float)samples;
}


luz_status launch_light_pass(luz_ctx* ctx, luz_frame* f, int mode) {
    if (mode < kPlain || mode > kCompose) return set_error(ctx, LUZ_ERR_INVALID, "unknown light pass mode");
    luz_status st = ensure_lit_list(ctx, f);
    if (st != LUZ_OK) return st;
    LightParams P;
    P.surf = f->surf;
    P.lit_count = f->lit_count;
    P.albedo = f->albedo;
    P.normal = f->normal;
    P.material = f->material;
    P.emission = f->emission;
    P.shadow_bits = f->shadow_bits;
    P.ao_bits = f->ao_bits;
    P.ao_denoised = f->ao_denoised;
    P.denoised = f->denoised;
    P.signal = f->signal;
    P.unshadowed = f->unshadowed;
    P.lights = f->d_lights;
    P.light_slot = f->d_light_slot;
    P.light_count = f->light_count;
    P.words = f->words;
    P.ao_samples = f->ao_samples;
    P.shadow_type = f->h_scene.shadow_type;
    P.shadow_lights = f->d_shadow_lights;
    P.shadow_count = f->shadow_light_count;
    memcpy(P.cam, f->h_scene.cam_pos, 12);
    memcpy(P.ambient, f->h_scene.ambient_light_color, 12);
    P.ambient_intensity = f->h_scene.ambient_light_intensity;
    P.width = f->width;
    P.height = f->height;
    P.out = f->light;
    size_t smem = (size_t)f->light_count * sizeof(luz_light);
    void (*kernels[4])(LightParams) = {light_pass_kernel<kPlain>, light_pass_kernel<kDenoisedAo>,
                                       light_pass_kernel<kSplit>, light_pass_kernel<kCompose>};
    static size_t attr_bytes[4] = {48 * 1024, 48 * 1024, 48 * 1024, 48 * 1024};
    if (smem > attr_bytes[mode]) {
        LUZ_CUDA(ctx, cudaFuncSetAttribute(kernels[mode], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr_bytes[mode] = smem;
    }
    uint32_t blocks = (f->pixels + 255) / 256;
    prof_begin(ctx, LUZ_KERNEL_LIGHT_PASS);
    kernels[mode]<<<blocks, 256, smem, ctx->stream>>>(P);
    prof_end(ctx);
    LUZ_LAUNCHED(ctx, "light_pass_kernel");
    return LUZ_OK;
}

luz_status launch_ao_resolve(luz_ctx* ctx, luz_frame* f) {
    uint32_t blocks = (f->pixels + 255) / 256;
    ao_resolve_kernel<<<blocks, 256, 0, ctx->stream>>>(f->normal, f->ao_bits, f->words,
                                                      f->ao_samples, f->pixels, f->ao);
    LUZ_LAUNCHED(ctx, "ao_resolve_kernel");
    return LUZ_OK;
}

}  // namespace luz
