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

// texture kinds: 0 = RGBA8 UNORM, 1 = RGBA32F, 2 = R32F
struct sampler2D {
    const void* data = nullptr;
    int w = 1, h = 1, kind = 0;
};
struct samplerCube {};

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

inline vec4 texture(const sampler2D& s, vec2 uv) {
    return refshim::fetch(s, (int)std::floor(uv.x * s.w), (int)std::floor(uv.y * s.h));
}
inline vec4 texture(const samplerCube&, vec3) { return vec4(0.0f); }
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
