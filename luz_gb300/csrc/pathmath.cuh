// pathmath.cuh — arithmetic of the visibility / lighting path, shared by the host
// side of the library and the sm_103a kernels.
//
// Every function here is evaluated with FMA contraction disabled (nvcc -fmad=false,
// g++ -ffp-contract=off), IEEE division and square root, and a fixed operation
// order, so that a ray built on the device is bit-identical to the same ray built
// by a CPU that follows the same steps. Hit/miss masks can only be bit-exact if the
// rays are.
#pragma once
#include <stdint.h>
#include <math.h>

#if defined(__CUDACC__)
#define LUZ_HD __host__ __device__ __forceinline__
#else
#define LUZ_HD inline
#endif

namespace luz {

// Constants of source/Shaders/LuzCommon.h:10-12, as GLSL evaluates them: unsuffixed
// GLSL literals are single precision.
constexpr float kPi = 3.14159265359f;
constexpr float kGoldenRatio = 2.118033988749895f;
constexpr float kTwoPiHemisphere = 6.283f;   // light.frag:65 uses the literal 6.283

struct V3 {
    float x, y, z;
};

LUZ_HD V3 v3(float x, float y, float z) { return V3{x, y, z}; }
LUZ_HD V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
LUZ_HD V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
LUZ_HD V3 operator*(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }
LUZ_HD V3 operator*(float s, V3 a) { return V3{s * a.x, s * a.y, s * a.z}; }
LUZ_HD V3 operator*(V3 a, V3 b) { return V3{a.x * b.x, a.y * b.y, a.z * b.z}; }
LUZ_HD V3 operator/(V3 a, float s) { return V3{a.x / s, a.y / s, a.z / s}; }
LUZ_HD V3 operator-(V3 a) { return V3{-a.x, -a.y, -a.z}; }
// GLSL dot: (x*x' + y*y') + z*z'
LUZ_HD float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
LUZ_HD V3 cross(V3 a, V3 b) {
    return V3{a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
LUZ_HD float length(V3 a) { return sqrtf(dot(a, a)); }
// normalize(v) = v * (1 / length(v)): one IEEE division, as glm's
// x * inversesqrt(dot(x, x)) form (the reciprocal here correctly rounded).
LUZ_HD V3 normalize(V3 a) {
    float inv = 1.0f / length(a);
    return V3{a.x * inv, a.y * inv, a.z * inv};
}
// min/max by comparison (not fminf/fmaxf): identical results for signed zeros and
// NaN on every compiler, which the byte-exact BVH comparison relies on.
LUZ_HD float fmin_(float a, float b) { return a < b ? a : b; }
LUZ_HD float fmax_(float a, float b) { return a > b ? a : b; }

// Repeat addressing (the reference's sampler, VulkanWrapper.cpp:2429-2454) of an
// integer-valued float texel coordinate f (a floor result) into [0, n): the same
// value as fmodf(f, n) (+ n when negative), without the division for |f| < n, which
// covers every coordinate of a texture coordinate in [-1, 2).
LUZ_HD uint32_t repeat_index(float f, uint32_t n) {
    const float nf = (float)n;
    if (f >= 0.0f && f < nf) return (uint32_t)f;
    if (f < 0.0f && f >= -nf) return (uint32_t)(f + nf);   // exact: integers below 2^24
    float m = fmodf(f, nf);
    if (m < 0.0f) m += nf;
    uint32_t i = (uint32_t)m;
    return i < n ? i : 0u;
}
LUZ_HD float clamp01(float x) { return fmin_(fmax_(x, 0.0f), 1.0f); }
LUZ_HD float fract_(float x) { return x - floorf(x); }
LUZ_HD bool finite3(V3 a) { return isfinite(a.x) && isfinite(a.y) && isfinite(a.z); }

// ---------------------------------------------------------------- sine / cosine
// The project's own sincos, used wherever the path needs cos/sin (DiskSample,
// HemisphereSample, scene generators). Method: Cody–Waite argument reduction by
// pi/2 with a three-part split of pi/2 (W. J. Cody and W. Waite, "Software Manual
// for the Elementary Functions", 1980), then the Taylor series of sin and cos on
// |r| <= pi/4 truncated after the r^9 and r^10 terms (truncation error below
// 2e-9). Coefficients are the rounded reciprocals of factorials, 1/n!.
// Valid for |x| < 2^11 * pi/2; error against a correctly rounded result is a few
// ulp of 1.0 (checked against libm in the tests).
constexpr float kTwoOverPi = 0x1.45f306p-1f;
constexpr float kPio2Hi = 0x1.92p+0f;        // 8 significant bits: k*hi exact
constexpr float kPio2Mid = 0x1.fb5p-12f;     // 13 significant bits: k*mid exact
constexpr float kPio2Lo = 0x1.110b46p-26f;
constexpr float kS3 = -1.0f / 6.0f, kS5 = 1.0f / 120.0f, kS7 = -1.0f / 5040.0f,
                kS9 = 1.0f / 362880.0f;
constexpr float kC2 = -0.5f, kC4 = 1.0f / 24.0f, kC6 = -1.0f / 720.0f, kC8 = 1.0f / 40320.0f,
                kC10 = -1.0f / 3628800.0f;

LUZ_HD void sincos_(float x, float* s, float* c) {
    float k = rintf(x * kTwoOverPi);
    float r = x - k * kPio2Hi;
    r = r - k * kPio2Mid;
    r = r - k * kPio2Lo;
    float r2 = r * r;
    float sp = r + r * (r2 * (kS3 + r2 * (kS5 + r2 * (kS7 + r2 * kS9))));
    float cp = 1.0f + r2 * (kC2 + r2 * (kC4 + r2 * (kC6 + r2 * (kC8 + r2 * kC10))));
    int q = ((int)k) & 3;
    float ss, cc;
    if (q == 0) { ss = sp; cc = cp; }
    else if (q == 1) { ss = cp; cc = -sp; }
    else if (q == 2) { ss = -sp; cc = -cp; }
    else { ss = -cp; cc = sp; }
    *s = ss;
    *c = cc;
}

// ---------------------------------------------------------------- samplers
// DiskSample, light.frag:57-61.
LUZ_HD void disk_sample(float rx, float ry, float radius, float* dx, float* dy) {
    float point_radius = radius * sqrtf(rx);
    float point_angle = ry * 2.0f * kPi;
    float s, c;
    sincos_(point_angle, &s, &c);
    *dx = point_radius * c;
    *dy = point_radius * s;
}

// HemisphereSample, light.frag:63-69 (cosine-weighted).
LUZ_HD V3 hemisphere_sample(float rx, float ry) {
    float r = sqrtf(rx);
    float theta = kTwoPiHemisphere * ry;
    float s, c;
    sincos_(theta, &s, &c);
    return V3{r * c, r * s, sqrtf(fmax_(0.0f, 1.0f - rx))};
}

// BlueNoiseSample(i).rg, light.frag:71-75: fract(texel + GOLDEN_RATIO*(128*i + frame%128)).
// texel_r/g are the UNORM8 texel bytes of the substitute texture at
// (x mod size, y mod size). frame%128 follows GLSL int % (truncating).
LUZ_HD void blue_noise_rg(uint32_t texel_r, uint32_t texel_g, int i, int frame, float* rx,
                          float* ry) {
    float offs = kGoldenRatio * (float)(128 * i + frame % 128);
    *rx = fract_((float)texel_r / 255.0f + offs);
    *ry = fract_((float)texel_g / 255.0f + offs);
}

// Stratified sequence: R2 (the 2-D Kronecker sequence of the plastic number,
// M. Roberts 2018) in 32-bit fixed point, so that sample i of 1024+ stays exact.
// The 64 pixels of an 8x8 block share one Cranley–Patterson rotation and take
// interleaved points of one sequence (sample i of in-block pixel j is point 64 i + j):
// the single samples of neighbouring pixels are stratified over the hemisphere,
// which is what a spatial filter over 1-sample estimates needs.
constexpr uint32_t kR2a = 0xC13FA9A9u;   // 2^32 / plastic number
constexpr uint32_t kR2b = 0x91E10DA5u;   // 2^32 / plastic number^2
LUZ_HD uint32_t hash32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352du;
    x ^= x >> 15; x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}
LUZ_HD void stratified_rg(uint32_t px, uint32_t py, int i, int frame, uint32_t stream,
                          float* rx, float* ry) {
    uint32_t h = hash32((px >> 3) * 0x9E3779B1u ^ hash32((py >> 3) + 0x632BE5ABu * (uint32_t)(frame + 1)) ^
                        (stream * 0x85EBCA77u));
    uint32_t h2 = hash32(h ^ 0x27D4EB2Fu);
    uint32_t k = (uint32_t)i * 64u + (((py & 7u) << 3) | (px & 7u));
    uint32_t ux = h + k * kR2a;
    uint32_t uy = h2 + k * kR2b;
    *rx = (float)(ux >> 8) * (1.0f / 16777216.0f);
    *ry = (float)(uy >> 8) * (1.0f / 16777216.0f);
}

// ---------------------------------------------------------------- matrices
// 4x4 column-major (glm layout: m[c*4 + r]); GLSL mat*vec sums j = 0..3 left to right.
LUZ_HD void mat4_mul_vec4(const float* m, const float v[4], float out[4]) {
    for (int r = 0; r < 4; ++r) {
        out[r] = m[0 * 4 + r] * v[0] + m[1 * 4 + r] * v[1] + m[2 * 4 + r] * v[2] +
                 m[3 * 4 + r] * v[3];
    }
}

// DepthToWorld, source/Shaders/utils.glsl:1-7.
LUZ_HD V3 depth_to_world(const float* inverse_proj, const float* inverse_view, float u,
                         float v, float depth) {
    float clip[4] = {u * 2.0f - 1.0f, v * 2.0f - 1.0f, depth, 1.0f};
    float view[4];
    mat4_mul_vec4(inverse_proj, clip, view);
    float w = view[3];
    view[0] = view[0] / w;
    view[1] = view[1] / w;
    view[2] = view[2] / w;
    view[3] = view[3] / w;
    float world[4];
    mat4_mul_vec4(inverse_view, view, world);
    return V3{world[0], world[1], world[2]};
}

// Pixel-centre texture coordinate of the full-screen pass (light.vert: uv origin top-left).
LUZ_HD float pixel_uv(uint32_t x, uint32_t extent) {
    return ((float)x + 0.5f) / (float)extent;
}

// Affine 3x4 row-major [R | t]: inverse [R^-1 | -R^-1 t] by cofactors, fixed order.
LUZ_HD void affine_inverse(const float m[12], float out[12]) {
    float a = m[0], b = m[1], c = m[2], d = m[4], e = m[5], f = m[6], g = m[8], h = m[9],
          k = m[10];
    float c00 = e * k - f * h;
    float c01 = f * g - d * k;
    float c02 = d * h - e * g;
    float det = a * c00 + b * c01 + c * c02;
    float inv = 1.0f / det;
    float r00 = c00 * inv, r01 = (c * h - b * k) * inv, r02 = (b * f - c * e) * inv;
    float r10 = c01 * inv, r11 = (a * k - c * g) * inv, r12 = (c * d - a * f) * inv;
    float r20 = c02 * inv, r21 = (b * g - a * h) * inv, r22 = (a * e - b * d) * inv;
    float tx = m[3], ty = m[7], tz = m[11];
    out[0] = r00; out[1] = r01; out[2] = r02; out[3] = -(r00 * tx + r01 * ty + r02 * tz);
    out[4] = r10; out[5] = r11; out[6] = r12; out[7] = -(r10 * tx + r11 * ty + r12 * tz);
    out[8] = r20; out[9] = r21; out[10] = r22; out[11] = -(r20 * tx + r21 * ty + r22 * tz);
}

LUZ_HD V3 xform_point(const float m[12], V3 p) {
    return V3{m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3],
              m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
              m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]};
}
LUZ_HD V3 xform_dir(const float m[12], V3 d) {
    return V3{m[0] * d.x + m[1] * d.y + m[2] * d.z, m[4] * d.x + m[5] * d.y + m[6] * d.z,
              m[8] * d.x + m[9] * d.y + m[10] * d.z};
}

// ---------------------------------------------------------------- Morton codes
LUZ_HD uint32_t expand_bits10(uint32_t v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}
LUZ_HD uint32_t quantize10(float c, float lo, float ext) {
    float n = ext > 0.0f ? (c - lo) / ext : 0.0f;
    float q = fmin_(fmax_(n * 1024.0f, 0.0f), 1023.0f);
    return (uint32_t)q;
}
// 30-bit Morton code of a box centre within the centroid bounds [cmin, cmin+ext].
LUZ_HD uint32_t morton30(V3 lo, V3 hi, V3 cmin, V3 ext) {
    float cx = (lo.x + hi.x) * 0.5f, cy = (lo.y + hi.y) * 0.5f, cz = (lo.z + hi.z) * 0.5f;
    uint32_t x = quantize10(cx, cmin.x, ext.x);
    uint32_t y = quantize10(cy, cmin.y, ext.y);
    uint32_t z = quantize10(cz, cmin.z, ext.z);
    return (expand_bits10(x) << 2) | (expand_bits10(y) << 1) | expand_bits10(z);
}

// Padding of an instance's world box (object-space hits are found with a ray
// transformed to object space; the world box must still contain them).
LUZ_HD float box_pad(float lo, float hi) {
    float m = fmax_(fabsf(lo), fabsf(hi));
    return m * 0x1p-14f + (hi - lo) * 0x1p-16f + 0x1p-60f;
}

}  // namespace luz
