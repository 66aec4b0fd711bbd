// ref_shim.hpp — the GLSL environment that the reference's light pass shader
// (source/Shaders/light.frag, utils.glsl) expects, restated for a CPU build under
// glm, so that the shader's own functions can run here as a check of the oracle.
//
// TEST INFRASTRUCTURE: used only by the oracle/_ref recipe (oracle/ref_shaders.py).
// Ray queries call back into the oracle's BVH traversal; textures are the
// G-buffer planes sampled at texel centres.
#pragma once
#define GLM_FORCE_RADIANS
#define GLM_FORCE_DEPTH_ZERO_TO_ONE
#define GLM_ENABLE_EXPERIMENTAL
#include <glm/glm.hpp>
#include <cmath>
#include <cstdint>
#include <cstring>

#define LUZ_ENGINE 1
using namespace glm;
#include "LuzCommon.h"

// GLSL evaluates unsuffixed literals in single precision.
#undef PI
#define PI 3.14159265359f
#undef LUZ_PI
#define LUZ_PI 3.14159265359f
#undef GOLDEN_RATIO
#define GOLDEN_RATIO 2.118033988749895f
#define LIGHT_TYPE_POINT 0
#define LIGHT_TYPE_DIRECTIONAL 2
#define LIGHT_TYPE_SPOT 1

namespace refshim {

// texture kinds: 0 = RGBA8 UNORM, 1 = RGBA32F, 2 = R32F. filter 0: the texel under the
// coordinate (full-screen passes read texel centres); 1: the reference's sampler,
// bilinear with repeat addressing (VulkanWrapper.cpp:2429-2454), in the oracle's
// arithmetic — the one part of the post-processing passes this shim defines itself.
struct sampler2D {
    const void* data = nullptr;
    int w = 1, h = 1, kind = 0, filter = 0;
};
// A cube shadow map: six R32F faces of res x res texels (+x, -x, +y, -y, +z, -z).
struct samplerCube {
    const float* faces = nullptr;
    int res = 1;
};

inline vec4 fetch(const sampler2D& s, int x, int y) {
    x = x < 0 ? 0 : (x >= s.w ? s.w - 1 : x);
    y = y < 0 ? 0 : (y >= s.h ? s.h - 1 : y);
    size_t i = (size_t)y * s.w + x;
    if (!s.data) return vec4(0.0f);
    if (s.kind == 0) {
        const uint8_t* p = (const uint8_t*)s.data + 4 * i;
        return vec4(p[0] / 255.0f, p[1] / 255.0f, p[2] / 255.0f, p[3] / 255.0f);
    }
    if (s.kind == 1) {
        const float* p = (const float*)s.data + 4 * i;
        return vec4(p[0], p[1], p[2], p[3]);
    }
    return vec4(((const float*)s.data)[i], 0.0f, 0.0f, 1.0f);
}

struct rayQueryEXT {
    vec3 o, d;
    float tmin = 0.0f, tmax = 0.0f;
    int proceeded = 0, hit = 0;
};

// Any-hit callback: (user, origin, tmin, direction, tmax) -> 1 on a hit.
using AnyHitFn = int (*)(const void* user, const float* o, const float* d, float tmin, float tmax, int closest,
                         int brute, float* t_out);

struct Env {
    AnyHitFn anyhit = nullptr;
    const void* user = nullptr;
    // optional ray log: 8 floats per ray (o, tmin, d, tmax)
    float* ray_log = nullptr;
    uint64_t ray_log_cap = 0, ray_count = 0;
};
extern Env g_env;

}  // namespace refshim

using refshim::rayQueryEXT;
using refshim::sampler2D;
using refshim::samplerCube;

inline int wrap_texel(float f, int n) {
    float m = std::fmod(f, (float)n);
    if (m < 0.0f) m += (float)n;
    int i = (int)m;
    return i < n ? i : 0;
}
inline vec4 texture(const sampler2D& s, vec2 uv) {
    if (s.filter == 0) return refshim::fetch(s, (int)std::floor(uv.x * s.w), (int)std::floor(uv.y * s.h));
    float x = uv.x * (float)s.w - 0.5f, y = uv.y * (float)s.h - 0.5f;
    if (!std::isfinite(x)) x = 0.0f;
    if (!std::isfinite(y)) y = 0.0f;
    float fx = std::floor(x), fy = std::floor(y);
    float ax = x - fx, ay = y - fy, bx = 1.0f - ax, by = 1.0f - ay;
    int x0 = wrap_texel(fx, s.w), y0 = wrap_texel(fy, s.h);
    int x1 = x0 + 1 == s.w ? 0 : x0 + 1, y1 = y0 + 1 == s.h ? 0 : y0 + 1;
    vec4 c00 = refshim::fetch(s, x0, y0), c10 = refshim::fetch(s, x1, y0);
    vec4 c01 = refshim::fetch(s, x0, y1), c11 = refshim::fetch(s, x1, y1);
    vec4 r;
    for (int k = 0; k < 4; ++k) r[k] = (c00[k] * bx + c10[k] * ax) * by + (c01[k] * bx + c11[k] * ax) * ay;
    return r;
}
// Storage image of the compute passes (RGBA32F).
struct image2D {
    float* data = nullptr;
    int w = 1, h = 1;
};
inline void imageStore(image2D& im, ivec2 p, vec4 v) {
    if (!im.data || p.x < 0 || p.y < 0 || p.x >= im.w || p.y >= im.h) return;
    float* o = im.data + 4 * ((size_t)p.y * im.w + p.x);
    o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
}
// Cube-map lookup for the shadow maps: the face of the major axis of the direction
// (ties to x, then y) with the face coordinates of Vulkan's cube-face table, then
// bilinear filtering clamped to the face's edges (the reference's sampler is linear;
// edge texels are not blended across faces here).
inline vec4 texture(const samplerCube& s, vec3 d) {
    if (!s.faces) return vec4(0.0f);
    const float ax = std::fabs(d.x), ay = std::fabs(d.y), az = std::fabs(d.z);
    int face;
    float ma, sc, tc;
    if (ax >= ay && ax >= az) {
        face = d.x >= 0.0f ? 0 : 1; ma = ax; sc = d.x >= 0.0f ? -d.z : d.z; tc = -d.y;
    } else if (ay >= az) {
        face = d.y >= 0.0f ? 2 : 3; ma = ay; sc = d.x; tc = d.y >= 0.0f ? d.z : -d.z;
    } else {
        face = d.z >= 0.0f ? 4 : 5; ma = az; sc = d.z >= 0.0f ? d.x : -d.x; tc = -d.y;
    }
    float u = 0.5f, v = 0.5f;
    if (ma != 0.0f) {
        u = 0.5f * (sc / ma + 1.0f);
        v = 0.5f * (tc / ma + 1.0f);
    } else {
        face = 0;
    }
    const int n = s.res;
    const float* f = s.faces + (size_t)face * n * n;
    float x = u * (float)n - 0.5f, y = v * (float)n - 0.5f;
    if (!std::isfinite(x)) x = 0.0f;
    if (!std::isfinite(y)) y = 0.0f;
    const float fx = std::floor(x), fy = std::floor(y);
    const float wx = x - fx, wy = y - fy;
    auto clampi = [n](float c) { return c <= 0.0f ? 0 : (c >= (float)(n - 1) ? n - 1 : (int)c); };
    const int x0 = clampi(fx), x1 = clampi(fx + 1.0f), y0 = clampi(fy), y1 = clampi(fy + 1.0f);
    const float c00 = f[(size_t)y0 * n + x0], c10 = f[(size_t)y0 * n + x1];
    const float c01 = f[(size_t)y1 * n + x0], c11 = f[(size_t)y1 * n + x1];
    return vec4((c00 * (1.0f - wx) + c10 * wx) * (1.0f - wy) + (c01 * (1.0f - wx) + c11 * wx) * wy, 0.0f, 0.0f, 1.0f);
}
inline ivec2 textureSize(const sampler2D& s, int) { return ivec2(s.w, s.h); }
inline vec4 texelFetch(const sampler2D& s, ivec2 p, int) { return refshim::fetch(s, p.x, p.y); }

struct TlasHandle {};
static const TlasHandle tlas_dummy{};
constexpr unsigned gl_RayFlagsTerminateOnFirstHitEXT = 4u;
constexpr int gl_RayQueryCommittedIntersectionNoneEXT = 0;

inline void rayQueryInitializeEXT(rayQueryEXT& q, const TlasHandle&, unsigned, unsigned, vec3 o, float tmin, vec3 d,
                                  float tmax) {
    q.o = o;
    q.d = d;
    q.tmin = tmin;
    q.tmax = tmax;
    q.proceeded = 0;
    q.hit = 0;
}
inline bool rayQueryProceedEXT(rayQueryEXT& q) {
    if (!q.proceeded) {
        q.proceeded = 1;
        float o[3] = {q.o.x, q.o.y, q.o.z}, d[3] = {q.d.x, q.d.y, q.d.z};
        refshim::Env& e = refshim::g_env;
        if (e.ray_log && e.ray_count < e.ray_log_cap) {
            float* r = e.ray_log + 8 * e.ray_count;
            r[0] = o[0]; r[1] = o[1]; r[2] = o[2]; r[3] = q.tmin;
            r[4] = d[0]; r[5] = d[1]; r[6] = d[2]; r[7] = q.tmax;
        }
        e.ray_count++;
        q.hit = e.anyhit ? e.anyhit(e.user, o, d, q.tmin, q.tmax, 0, 0, nullptr) : 0;
    }
    return false;   // the committed result is final: TerminateOnFirstHit, opaque geometry
}
inline int rayQueryGetIntersectionTypeEXT(rayQueryEXT& q, bool) { return q.hit ? 1 : 0; }
