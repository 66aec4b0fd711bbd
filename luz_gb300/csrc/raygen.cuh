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
