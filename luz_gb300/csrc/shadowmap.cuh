// shadowmap.cuh — shadow-map lookups of light.frag's EvaluateShadow (light.frag:147-165),
// shared by the light pass. Maps are sampled with the reference's sampler written out
// (bilinear; repeat addressing for 2D maps; cube faces clamp to their edges).
#pragma once
#include "internal.cuh"

namespace luz {

__device__ __forceinline__ uint32_t sm_wrap(float f, uint32_t n) { return repeat_index(f, n); }

__device__ __forceinline__ uint32_t sm_clamp(float f, uint32_t n) {
    if (!(f > 0.0f)) return 0u;
    if (f >= (float)(n - 1)) return n - 1;
    return (uint32_t)f;
}

// Bilinear depth of one face; repeat = 2D maps, else clamp to edge.
__device__ __forceinline__ float sm_sample(const float* __restrict__ face, uint32_t res, float u, float v,
                                           bool repeat) {
    float x = u * (float)res - 0.5f, y = v * (float)res - 0.5f;
    if (!isfinite(x)) x = 0.0f;
    if (!isfinite(y)) y = 0.0f;
    float fx = floorf(x), fy = floorf(y);
    float ax = x - fx, ay = y - fy, bx = 1.0f - ax, by = 1.0f - ay;
    uint32_t x0, x1, y0, y1;
    if (repeat) {
        x0 = sm_wrap(fx, res);
        y0 = sm_wrap(fy, res);
        x1 = x0 + 1 == res ? 0u : x0 + 1;
        y1 = y0 + 1 == res ? 0u : y0 + 1;
    } else {
        x0 = sm_clamp(fx, res);
        y0 = sm_clamp(fy, res);
        x1 = sm_clamp(fx + 1.0f, res);
        y1 = sm_clamp(fy + 1.0f, res);
    }
    float c00 = __ldg(face + (size_t)y0 * res + x0), c10 = __ldg(face + (size_t)y0 * res + x1);
    float c01 = __ldg(face + (size_t)y1 * res + x0), c11 = __ldg(face + (size_t)y1 * res + x1);
    return (c00 * bx + c10 * ax) * by + (c01 * bx + c11 * ax) * ay;
}

// Cube-map face and (s, t) of a direction (Vulkan's cube face selection table; ties go
// to x, then y).
__device__ __forceinline__ void cube_face(V3 d, uint32_t& face, float& s, float& t) {
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z), ma, sc, tc;
    if (ax >= ay && ax >= az) {
        face = d.x >= 0.0f ? 0u : 1u;
        ma = ax;
        sc = d.x >= 0.0f ? -d.z : d.z;
        tc = -d.y;
    } else if (ay >= az) {
        face = d.y >= 0.0f ? 2u : 3u;
        ma = ay;
        sc = d.x;
        tc = d.y >= 0.0f ? d.z : -d.z;
    } else {
        face = d.z >= 0.0f ? 4u : 5u;
        ma = az;
        sc = d.z >= 0.0f ? d.x : -d.x;
        tc = -d.y;
    }
    if (ma == 0.0f) {
        face = 0;
        s = t = 0.5f;
        return;
    }
    s = 0.5f * (sc / ma + 1.0f);
    t = 0.5f * (tc / ma + 1.0f);
}

// EvaluateShadow's map branch: 1 = in shadow.
__device__ __forceinline__ float shadow_map_factor(const DevShadowLight& S, V3 frag, V3 origin) {
    if (S.faces == 6) {
        V3 d = frag - V3{S.position[0], S.position[1], S.position[2]};
        uint32_t face;
        float s, t;
        cube_face(d, face, s, t);
        float depth = sm_sample(S.map + (size_t)face * S.res * S.res, S.res, s, t, false);
        return length(d) - 0.05f >= depth * S.z_far ? 1.0f : 0.0f;
    }
    float p4[4] = {origin.x, origin.y, origin.z, 1.0f}, fl[4];
    mat4_mul_vec4(S.view_proj0, p4, fl);
    float depth = sm_sample(S.map, S.res, fl[0] * 0.5f + 0.5f, fl[1] * 0.5f + 0.5f, true);
    return fl[2] >= depth ? 1.0f : 0.0f;
}

}  // namespace luz
