// raygen.cuh — shadow and AO ray generation of light.frag, bit-identical to the CPU
// oracle (FMA contraction off, IEEE division and square root, GLSL operation order).
#pragma once
#include "internal.cuh"

namespace luz {

// The light vector L of light.frag main (light.frag:194-198), which both the shadow
// ray and the light pass's max(dot(N, L), 0) use.
__device__ __forceinline__ V3 light_vector(const luz_light& lt, V3 p) {
    V3 lpos = V3{lt.position[0], lt.position[1], lt.position[2]};
    V3 ldir = V3{lt.direction[0], lt.direction[1], lt.direction[2]};
    V3 L = normalize(lpos - p);
    if (lt.type == LUZ_LIGHT_DIRECTIONAL) L = normalize(-ldir);
    return L;
}

// Attenuation of light.frag main (light.frag:196-208) given L = light_vector(lt, p):
// 1 for directional lights, 1/d^2 for point lights, times the cone term for spots.
__device__ __forceinline__ float light_attenuation(const luz_light& lt, V3 p, V3 L) {
    V3 lpos = V3{lt.position[0], lt.position[1], lt.position[2]};
    V3 ldir = V3{lt.direction[0], lt.direction[1], lt.direction[2]};
    float attenuation = 1.0f;
    if (lt.type == LUZ_LIGHT_SPOT) {
        float dist = length(lpos - p);
        attenuation = 1.0f / (dist * dist);
        float theta = dot(L, normalize(-ldir));
        float epsilon = lt.inner_angle - lt.outer_angle;
        attenuation *= clamp01((theta - lt.outer_angle) / epsilon);
    } else if (lt.type == LUZ_LIGHT_POINT) {
        float dist = length(lpos - p);
        attenuation = 1.0f / (dist * dist);
    }
    return attenuation;
}

// True when the light pass's contribution of this light cannot depend on its shadow
// factor s: it adds ((kD * albedo / pi + spec) * radiance) * max(dot(N, L), 0) with
// radiance = ((color * intensity) * attenuation) * (1 - s) (light.frag:209-226). If
// the weight max(dot(N, L), 0) is 0 (dot <= 0 or NaN), or every channel of
// (color * intensity) * attenuation is +-0 (radiance +-0 for every s in [0, 1]), the
// sum takes the same value for every s (a +-0 term leaves Lo unchanged, a non-finite
// factor gives NaN either way).
__device__ __forceinline__ bool shadow_has_no_effect(const luz_light& lt, V3 p, V3 N, V3 L) {
    if (!(dot(N, L) > 0.0f)) return true;
    const float a = light_attenuation(lt, p, L);
    const V3 c = (V3{lt.color[0], lt.color[1], lt.color[2]} * lt.intensity) * a;
    return c.x == 0.0f && c.y == 0.0f && c.z == 0.0f;
}

// EvaluateShadow (light.frag:137-146) + TraceShadowRay (light.frag:86-109) for one
// sample, given L = light_vector(lt, p): origin, direction and tMax of the shadow
// ray; tMin is 0.001.
__device__ __forceinline__ void shadow_ray(const luz_light& lt, V3 p, V3 N, V3 cam, float rx,
                                           float ry, V3 L, V3& O, V3& dir, float& tmax) {
    V3 lpos = V3{lt.position[0], lt.position[1], lt.position[2]};
    V3 ldir = V3{lt.direction[0], lt.direction[1], lt.direction[2]};
    float bias = fmax_(length(p - cam) * 0.01f, 0.05f);
    O = p + N * bias;
    float dist = length(lpos - p);
    V3 Lv = (lt.type == LUZ_LIGHT_DIRECTIONAL) ? (ldir * dot(ldir, L)) * dist : L * dist;
    V3 T = normalize(cross(Lv, V3{0.0f, 1.0f, 0.0f}));
    V3 B = normalize(cross(T, Lv));
    float dx, dy;
    disk_sample(rx, ry, lt.radius, &dx, &dy);
    tmax = length(Lv);
    dir = normalize((Lv + dx * T) + dy * B);
}

// TraceAORays (light.frag:111-135) for one sample, with the AO origin of
// light.frag:229-230 (bias without the 0.05 floor).
__device__ __forceinline__ void ao_ray(V3 p, V3 N, V3 cam, float rx, float ry, V3& O, V3& dir) {
    float bias = length(p - cam) * 0.01f;
    O = p + N * bias;
    V3 T = fabsf(N.z) > 0.5f ? V3{0.0f, -N.z, N.y} : V3{-N.y, N.x, 0.0f};
    V3 B = cross(N, T);
    V3 h = hemisphere_sample(rx, ry);
    dir = (T * h.x + B * h.y) + N * h.z;
}

__device__ __forceinline__ void sample_rg(const uint8_t* __restrict__ bn, uint32_t bn_size,
                                          int sampler, uint32_t px, uint32_t py, int i, int frame,
                                          uint32_t stream, float* rx, float* ry) {
    if (sampler == LUZ_SAMPLER_STRATIFIED) {
        stratified_rg(px, py, i, frame, stream, rx, ry);
    } else {
        uint32_t tx = px % bn_size, ty = py % bn_size;
        uint32_t w = __ldg(reinterpret_cast<const uint32_t*>(bn) + ty * bn_size + tx);
        blue_noise_rg(w & 0xFF, (w >> 8) & 0xFF, i, frame, rx, ry);
    }
}

}  // namespace luz
