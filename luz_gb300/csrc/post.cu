// post.cu — the passes after the light pass: temporal anti-aliasing (taa.comp), the
// luminance histogram and its average (histogram.comp, histogramAverage.comp) and the
// compose / tone-mapping pass (present.frag) into a headless BGRA8 image.
//
// The reference samples its images through one sampler (linear filtering, repeat
// addressing, a single mip level: VulkanWrapper.cpp:2429-2454); `texture()` here is
// that bilinear filter written out in IEEE single precision, so the device and the
// CPU oracle produce the same bits.
#include <algorithm>
#include <cstring>

#include "internal.cuh"

namespace luz {

// GLSL min/max/clamp (GLSL 4.60 §8.3: min(x, y) = y < x ? y : x).
__device__ __forceinline__ float gmin(float x, float y) { return y < x ? y : x; }
__device__ __forceinline__ float gmax(float x, float y) { return x < y ? y : x; }
__device__ __forceinline__ float4 gmin4(float4 a, float4 b) {
    return make_float4(gmin(a.x, b.x), gmin(a.y, b.y), gmin(a.z, b.z), gmin(a.w, b.w));
}
__device__ __forceinline__ float4 gmax4(float4 a, float4 b) {
    return make_float4(gmax(a.x, b.x), gmax(a.y, b.y), gmax(a.z, b.z), gmax(a.w, b.w));
}
__device__ __forceinline__ float4 add4(float4 a, float4 b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
__device__ __forceinline__ float4 sub4(float4 a, float4 b) { return make_float4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
__device__ __forceinline__ float4 mul4(float4 a, float s) { return make_float4(a.x * s, a.y * s, a.z * s, a.w * s); }
__device__ __forceinline__ float4 div4(float4 a, float s) { return make_float4(a.x / s, a.y / s, a.z / s, a.w / s); }
__device__ __forceinline__ bool anynan4(float4 a) { return isnan(a.x) || isnan(a.y) || isnan(a.z) || isnan(a.w); }

// ---------------------------------------------------------------- sampling
__device__ __forceinline__ uint32_t wrap_texel(float f, uint32_t n) { return repeat_index(f, n); }

struct Bilinear {
    uint32_t x0, x1, y0, y1;
    float ax, ay, bx, by;
};

__device__ __forceinline__ Bilinear bilinear(float u, float v, uint32_t w, uint32_t h) {
    float x = u * (float)w - 0.5f, y = v * (float)h - 0.5f;
    if (!isfinite(x)) x = 0.0f;
    if (!isfinite(y)) y = 0.0f;
    float fx = floorf(x), fy = floorf(y);
    Bilinear b;
    b.ax = x - fx;
    b.ay = y - fy;
    b.bx = 1.0f - b.ax;
    b.by = 1.0f - b.ay;
    b.x0 = wrap_texel(fx, w);
    b.y0 = wrap_texel(fy, h);
    b.x1 = b.x0 + 1 == w ? 0u : b.x0 + 1;
    b.y1 = b.y0 + 1 == h ? 0u : b.y0 + 1;
    return b;
}

__device__ __forceinline__ float lerp2(float c00, float c10, float c01, float c11, const Bilinear& b) {
    return (c00 * b.bx + c10 * b.ax) * b.by + (c01 * b.bx + c11 * b.ax) * b.ay;
}

__device__ __forceinline__ float4 sample4(const float4* __restrict__ img, uint32_t w, uint32_t h, float u, float v) {
    Bilinear b = bilinear(u, v, w, h);
    float4 c00 = __ldg(img + (size_t)b.y0 * w + b.x0), c10 = __ldg(img + (size_t)b.y0 * w + b.x1);
    float4 c01 = __ldg(img + (size_t)b.y1 * w + b.x0), c11 = __ldg(img + (size_t)b.y1 * w + b.x1);
    return make_float4(lerp2(c00.x, c10.x, c01.x, c11.x, b), lerp2(c00.y, c10.y, c01.y, c11.y, b),
                       lerp2(c00.z, c10.z, c01.z, c11.z, b), lerp2(c00.w, c10.w, c01.w, c11.w, b));
}

__device__ __forceinline__ float sample1(const float* __restrict__ img, uint32_t w, uint32_t h, float u, float v) {
    Bilinear b = bilinear(u, v, w, h);
    return lerp2(__ldg(img + (size_t)b.y0 * w + b.x0), __ldg(img + (size_t)b.y0 * w + b.x1),
                 __ldg(img + (size_t)b.y1 * w + b.x0), __ldg(img + (size_t)b.y1 * w + b.x1), b);
}

// ---------------------------------------------------------------- TAA (taa.comp)
// A 16x16 block of pixels stages a 20x20 tile of the light image and of the depth
// (texel origin - 2, wrapped with the sampler's repeat addressing): every tap of
// find_closest_3x3, get_motion_vector and get_neighbor_3x3 lies at an offset of -1, 0
// or +1 pixel, whose bilinear footprint spans texels x - 2 .. x + 2. Tile slot t of a
// row holds texel wrap(origin + t), so the footprint's texels wrap(fx), wrap(fx + 1)
// sit in slots fx - origin and fx - origin + 1: the same values, the same arithmetic.
// The history sample follows the motion vector and reads global memory.
constexpr int kTaaTile = 16, kTaaSpan = kTaaTile + 4;

__device__ __forceinline__ int taa_slot(int f, int origin) { return min(max(f - origin, 0), kTaaSpan - 2); }

// One axis of bilinear(): the footprint's first tile slot and the two weights. The
// taps of a pixel share three u and three v positions, so a 3x3 neighbourhood needs
// three of each (the same operations bilinear() performs per tap).
struct TapAxis {
    int slot;
    float a, b;
};
__device__ __forceinline__ TapAxis tap_axis(float u, uint32_t n, int origin) {
    float x = u * (float)n - 0.5f;
    if (!isfinite(x)) x = 0.0f;
    const float f = floorf(x);
    TapAxis t;
    t.a = x - f;
    t.b = 1.0f - t.a;
    t.slot = taa_slot((int)f, origin);
    return t;
}
__device__ __forceinline__ float tap1(const float* tile, TapAxis X, TapAxis Y) {
    const float* r0 = tile + Y.slot * kTaaSpan + X.slot;
    return (r0[0] * X.b + r0[1] * X.a) * Y.b + (r0[kTaaSpan] * X.b + r0[kTaaSpan + 1] * X.a) * Y.a;
}
__device__ __forceinline__ float4 tap4(const float4* tile, TapAxis X, TapAxis Y) {
    const float4* r0 = tile + Y.slot * kTaaSpan + X.slot;
    const float4 c00 = r0[0], c10 = r0[1], c01 = r0[kTaaSpan], c11 = r0[kTaaSpan + 1];
    return make_float4((c00.x * X.b + c10.x * X.a) * Y.b + (c01.x * X.b + c11.x * X.a) * Y.a,
                       (c00.y * X.b + c10.y * X.a) * Y.b + (c01.y * X.b + c11.y * X.a) * Y.a,
                       (c00.z * X.b + c10.z * X.a) * Y.b + (c01.z * X.b + c11.z * X.a) * Y.a,
                       (c00.w * X.b + c10.w * X.a) * Y.b + (c01.w * X.b + c11.w * X.a) * Y.a);
}

struct TaaParams {
    const float4* input;     // this frame's light image
    const float4* history;   // last frame's TAA output
    const float* depth;
    float4* output;
    uint32_t w, h;
    int reconstruct;
    float inverse_proj[16], inverse_view[16], view_proj[16], prev_view_proj[16];
    float jitter[2], prev_jitter[2];
};

// utils.glsl: MitchellFilter with B = C = 1/3, evaluated at any distance.
__device__ __forceinline__ float mitchell(float x) {
    const float B = 1.0f / 3.0f, C = 1.0f / 3.0f;
    float x2 = x * x;
    float x3 = x2 * x;
    return (6.0f - 2.0f * B) * x3 - (6.0f - 2.0f * B - 3.0f * C) * x2 + 1.0f;
}

__device__ __forceinline__ float luminance(float r, float g, float b) {
    return r * 0.2127f + g * 0.7152f + b * 0.0722f;
}

// taa.comp:16-26 (get_motion_vector): screen-space motion of the surface at (u, v),
// given the depth sampled there.
__device__ __forceinline__ void motion_at(const TaaParams& P, float u, float v, float depth, float& mx, float& my) {
    V3 wp = depth_to_world(P.inverse_proj, P.inverse_view, u, v, depth);
    float p4[4] = {wp.x, wp.y, wp.z, 1.0f}, prev[4], cur[4];
    mat4_mul_vec4(P.prev_view_proj, p4, prev);
    mat4_mul_vec4(P.view_proj, p4, cur);
    float px = prev[0] / prev[3], py = prev[1] / prev[3];
    float cx = cur[0] / cur[3], cy = cur[1] / cur[3];
    mx = ((cx - P.jitter[0]) - (px - P.prev_jitter[0])) * 0.5f;
    my = ((cy - P.jitter[1]) - (py - P.prev_jitter[1])) * 0.5f;
}

// taa.comp:134-157 (clip_aabb, vec4 form).
__device__ __forceinline__ float4 clip_aabb(float mnx, float mny, float mnz, float mxx, float mxy, float mxz, float4 p,
                                           float4 q) {
    float4 r = sub4(q, p);
    float rmaxx = mxx - p.x, rmaxy = mxy - p.y, rmaxz = mxz - p.z;
    float rminx = mnx - p.x, rminy = mny - p.y, rminz = mnz - p.z;
    const float eps = 0.00000001f;
    if (r.x > rmaxx + eps) r = mul4(r, rmaxx / r.x);
    if (r.y > rmaxy + eps) r = mul4(r, rmaxy / r.y);
    if (r.z > rmaxz + eps) r = mul4(r, rmaxz / r.z);
    if (r.x < rminx - eps) r = mul4(r, rminx / r.x);
    if (r.y < rminy - eps) r = mul4(r, rminy / r.y);
    if (r.z < rminz - eps) r = mul4(r, rminz / r.z);
    return add4(p, r);
}

__global__ void __launch_bounds__(256) taa_kernel(TaaParams P) {
    __shared__ float4 s_light[kTaaSpan * kTaaSpan];
    __shared__ float s_depth[kTaaSpan * kTaaSpan];
    const int ox = (int)(blockIdx.x * kTaaTile) - 2, oy = (int)(blockIdx.y * kTaaTile) - 2;
    for (int i = threadIdx.x; i < kTaaSpan * kTaaSpan; i += blockDim.x) {
        const uint32_t tx = repeat_index((float)(ox + i % kTaaSpan), P.w);
        const uint32_t ty = repeat_index((float)(oy + i / kTaaSpan), P.h);
        s_light[i] = __ldg(P.input + (size_t)ty * P.w + tx);
        s_depth[i] = __ldg(P.depth + (size_t)ty * P.w + tx);
    }
    __syncthreads();
    uint32_t x = blockIdx.x * kTaaTile + (threadIdx.x & 15), y = blockIdx.y * kTaaTile + (threadIdx.x >> 4);
    if (x >= P.w || y >= P.h) return;
    const float su = ((float)x + 0.5f) / (float)P.w, sv = ((float)y + 0.5f) / (float)P.h;
    // the three u and v of the 3x3 taps (uv -/+ 1/size, one component at a time as the
    // GLSL vec2 arithmetic does; find_closest_3x3 and get_neighbor_3x3 use the same)
    const float du = 1.0f / (float)P.w, dv = 1.0f / (float)P.h;
    const float us[3] = {su - du, su, su + du}, vs[3] = {sv - dv, sv, sv + dv};
    TapAxis ax[3], ay[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        ax[k] = tap_axis(us[k], P.w, ox);
        ay[k] = tap_axis(vs[k], P.h, oy);
    }
    // find_closest_3x3 (taa.comp:111-132); the motion vector's depth sample at the
    // chosen tap is that tap's depth (taa.comp:16-26)
    int bi = 0, bj = 0;
    float best_z = 0.0f;
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const float z = tap1(s_depth, ax[i], ay[j]);
            if ((i == 0 && j == 0) || best_z > z) { bi = i; bj = j; best_z = z; }
        }
    const float cu = su + du * (float)(bi - 1), cv = sv + dv * (float)(bj - 1);
    float mx, my;
    motion_at(P, cu, cv, best_z, mx, my);
    const float hu = su - mx, hv = sv - my;
    float4 hist = sample4(P.history, P.w, P.h, hu, hv);
    // get_neighbor_3x3 (taa.comp:28-93)
    float4 c[9];
    const float mw[3] = {mitchell(sqrtf(2.0f)), mitchell(1.0f), mitchell(0.0f)};   // |d| = sqrt2, 1, 0
#pragma unroll
    for (int k = 0; k < 9; ++k) c[k] = tap4(s_light, ax[k % 3], ay[k / 3]);
    // order tl tc tr ml mc mr bl bc br = c[0..8]
    float4 cmin = gmin4(c[0], gmin4(c[1], gmin4(c[2], gmin4(c[3], gmin4(c[4], gmin4(c[5], gmin4(c[6], gmin4(c[7], c[8]))))))));
    float4 cmax = gmax4(c[0], gmax4(c[1], gmax4(c[2], gmax4(c[3], gmax4(c[4], gmax4(c[5], gmax4(c[6], gmax4(c[7], c[8]))))))));
    float4 cavg = c[0];
    for (int k = 1; k < 9; ++k) cavg = add4(cavg, c[k]);
    cavg = div4(cavg, 9.0f);
    float4 cmin5 = gmin4(c[1], gmin4(c[3], gmin4(c[4], gmin4(c[5], c[7]))));
    float4 cmax5 = gmax4(c[1], gmax4(c[3], gmax4(c[4], gmax4(c[5], c[7]))));
    float4 cavg5 = div4(add4(add4(add4(add4(c[1], c[3]), c[4]), c[5]), c[7]), 5.0f);
    cmin = mul4(add4(cmin, cmin5), 0.5f);
    cmax = mul4(add4(cmax, cmax5), 0.5f);
    cavg = mul4(add4(cavg, cavg5), 0.5f);
    float4 src = make_float4(0.f, 0.f, 0.f, 0.f);
    if (P.reconstruct == 1) {
        float wsum = 0.0f;
        for (int k = 0; k < 9; ++k) {
            int dx = k % 3 - 1, dy = k / 3 - 1;
            float wgt = mw[(dx != 0) + (dy != 0) == 2 ? 0 : ((dx != 0) + (dy != 0) == 1 ? 1 : 2)];
            src = add4(src, mul4(c[k], wgt));
            wsum += wgt;
        }
        src = div4(src, wsum);
    }
    if (P.reconstruct == 0 || anynan4(src)) src = c[4];   // the centre tap is texture(input, uv)
    float4 out;
    if (hu > 1.0f || hv > 1.0f || hu < 0.0f || hv < 0.0f) {
        out = src;
    } else {
        float4 cl = gmin4(gmax4(cavg, cmin), cmax);   // clamp(cavg, cmin, cmax)
        hist = clip_aabb(cmin.x, cmin.y, cmin.z, cmax.x, cmax.y, cmax.z, cl, hist);
        float sw = 0.05f, hw = 1.0f - sw;
        // anti_flicker (taa.comp:159-166)
        float rs = 1.0f / (gmax(gmax(src.x, src.y), src.z) + 1.0f);
        float rh = 1.0f / (gmax(gmax(hist.x, hist.y), hist.z) + 1.0f);
        float ls = luminance(src.x * rs, src.y * rs, src.z * rs);
        float lh = luminance(hist.x * rh, hist.y * rh, hist.z * rh);
        sw *= 1.0f / (1.0f + ls);
        hw *= 1.0f / (1.0f + lh);
        out = div4(add4(mul4(src, sw), mul4(hist, hw)), gmax(sw + hw, 0.0000001f));
        if (anynan4(out)) out = src;
    }
    P.output[(size_t)y * P.w + x] = out;
}

luz_status launch_taa(luz_ctx* ctx, luz_frame* f, int reconstruct) {
    TaaParams P;
    P.input = f->light;
    P.history = f->taa;
    P.depth = f->depth;
    P.output = f->taa_next;
    P.w = f->width;
    P.h = f->height;
    P.reconstruct = reconstruct;
    const luz_scene& s = f->h_scene;
    memcpy(P.inverse_proj, s.inverse_proj, 64);
    memcpy(P.inverse_view, s.inverse_view, 64);
    memcpy(P.view_proj, s.view_proj, 64);
    memcpy(P.prev_view_proj, s.prev_view_proj, 64);
    memcpy(P.jitter, s.jitter, 8);
    memcpy(P.prev_jitter, s.prev_jitter, 8);
    dim3 grid((f->width + kTaaTile - 1) / kTaaTile, (f->height + kTaaTile - 1) / kTaaTile);
    prof_begin(ctx, LUZ_KERNEL_TAA);
    taa_kernel<<<grid, 256, 0, ctx->stream>>>(P);
    prof_end(ctx);
    LUZ_LAUNCHED(ctx, "taa_kernel");
    std::swap(f->taa, f->taa_next);   // the output is the next frame's history
    return LUZ_OK;
}

// ---------------------------------------------------------------- luminance histogram
// histogram.comp / histogramAverage.comp with the constants of
// DeferredRenderer::LuminanceHistogramPass (DeferredRenderer.cpp:447-466): 256 bins of
// log2 luminance over [-10, 2], bin 0 for luminance below 1e-6.
constexpr float kHistMinLog = -10.0f;
constexpr float kHistOneOverLog = 1.0f / 12.0f;

__device__ __forceinline__ uint32_t histogram_bin(float r, float g, float b) {
    float lum = r * 0.2127f + g * 0.7152f + b * 0.0722f;
    if (lum < 0.000001f) return 0u;
    float t = (log2f(lum) - kHistMinLog) * kHistOneOverLog;
    t = gmin(gmax(t, 0.0f), 1.0f);
    return (uint32_t)(t * 254.0f + 1.0f);
}

__global__ void __launch_bounds__(256) histogram_kernel(const float4* __restrict__ img, uint32_t n,
                                                        uint32_t* __restrict__ bins) {
    __shared__ uint32_t s_bins[256];
    s_bins[threadIdx.x] = 0u;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 c = __ldg(img + i);
        atomicAdd(&s_bins[histogram_bin(c.x, c.y, c.z)], 1u);
    }
    __syncthreads();
    if (s_bins[threadIdx.x]) atomicAdd(bins + threadIdx.x, s_bins[threadIdx.x]);
}

// out: bins[256] | weighted sum, log average, average luminance, adapted luminance
// (floats); state[0] holds the adapted luminance across frames.
__global__ void __launch_bounds__(256) histogram_average_kernel(const uint32_t* __restrict__ bins, uint32_t n,
                                                                float delta_time, float* state, uint32_t* out) {
    __shared__ float s[256];
    const uint32_t i = threadIdx.x;
    const float count = (float)bins[i];
    s[i] = count * (float)i;
    __syncthreads();
    for (uint32_t k = 128; k > 0; k >>= 1) {   // the reference's halving reduction
        if (i < k) s[i] += s[i + k];
        __syncthreads();
    }
    out[i] = bins[i];
    if (i == 0) {
        float weighted_log_average = (s[0] / gmax((float)n - count, 1.0f)) - 1.0f;
        float average = exp2f(((weighted_log_average / 254.0f) * kHistOneOverLog) + kHistMinLog);
        float last = state[0];
        float adapted = last + (average - last) * (1.0f - expf(-delta_time * 1.1f));
        state[0] = adapted;
        float* o = reinterpret_cast<float*>(out + 256);
        o[0] = s[0];
        o[1] = weighted_log_average;
        o[2] = average;
        o[3] = adapted;
    }
}

// ---------------------------------------------------------------- compose (present.frag)
struct ComposeParams {
    const float4* light;     // the light (or TAA) image
    const uint32_t* albedo;
    const float4* normal;
    const uint32_t* material;
    const uint32_t* emission;
    const float* depth;
    uint32_t* out;           // BGRA8 UNORM (the reference's compose format)
    uint32_t w, h;
    int image_type;
};

__device__ __forceinline__ float4 unorm4(uint32_t c) {
    return make_float4((float)(c & 255u) / 255.0f, (float)((c >> 8) & 255u) / 255.0f,
                       (float)((c >> 16) & 255u) / 255.0f, (float)(c >> 24) / 255.0f);
}

__device__ __forceinline__ float4 sample_rgba8(const uint32_t* __restrict__ img, uint32_t w, uint32_t h, float u,
                                               float v) {
    Bilinear b = bilinear(u, v, w, h);
    float4 c00 = unorm4(__ldg(img + (size_t)b.y0 * w + b.x0)), c10 = unorm4(__ldg(img + (size_t)b.y0 * w + b.x1));
    float4 c01 = unorm4(__ldg(img + (size_t)b.y1 * w + b.x0)), c11 = unorm4(__ldg(img + (size_t)b.y1 * w + b.x1));
    return make_float4(lerp2(c00.x, c10.x, c01.x, c11.x, b), lerp2(c00.y, c10.y, c01.y, c11.y, b),
                       lerp2(c00.z, c10.z, c01.z, c11.z, b), lerp2(c00.w, c10.w, c01.w, c11.w, b));
}

__device__ __forceinline__ float aces(float x) {
    const float a = 2.51f, b = 0.03f, c = 2.43f, d = 0.59f, e = 0.14f;
    x = (x * (a * x + b)) / (x * (c * x + d) + e);
    return powf(x, 1.0f / 2.2f);
}

__device__ __forceinline__ uint32_t unorm8c(float x) {
    x = gmin(gmax(x, 0.0f), 1.0f);   // NaN -> 0 (UNORM conversion of a NaN)
    return (uint32_t)(x * 255.0f + 0.5f);
}

__global__ void __launch_bounds__(256) compose_kernel(ComposeParams P) {
    uint32_t x = blockIdx.x * 16 + (threadIdx.x & 15), y = blockIdx.y * 16 + (threadIdx.x >> 4);
    if (x >= P.w || y >= P.h) return;
    float tu = ((float)x + 0.5f) / (float)P.w, tv = ((float)y + 0.5f) / (float)P.h;
    int type = P.image_type;
    float fu = tu, fv = tv;
    if (type == 6) {   // 3 x 2 grid of the six views (present.frag:44-67)
        fu = tu * 3.0f;
        fv = tv * 2.0f;
        if (tv < 0.5f) {
            if (tu < 1.0f / 3.0f) type = 0;
            else if (tu < 2.0f / 3.0f) { type = 1; fu -= 1.0f; }
            else { type = 2; fu -= 2.0f; }
        } else {
            fv -= 1.0f;
            if (tu < 1.0f / 3.0f) type = 3;
            else if (tu < 2.0f / 3.0f) { type = 4; fu -= 1.0f; }
            else { type = 5; fu -= 2.0f; }
        }
        fu = 1.0f / 6.0f + fu * 2.0f / 3.0f;
    }
    float4 v;
    switch (type) {
        case 1: v = sample_rgba8(P.albedo, P.w, P.h, fu, fv); break;
        case 2: v = sample4(P.normal, P.w, P.h, fu, fv); break;
        case 3: v = sample_rgba8(P.material, P.w, P.h, fu, fv); break;
        case 4: v = sample_rgba8(P.emission, P.w, P.h, fu, fv); break;
        case 5: { float d = sample1(P.depth, P.w, P.h, fu, fv); v = make_float4(d, 0.f, 0.f, 1.f); break; }
        default: v = sample4(P.light, P.w, P.h, fu, fv); break;
    }
    if (type == 0) {
        v = make_float4(aces(v.x), aces(v.y), aces(v.z), 1.0f);   // no debug overlay: debugColor.a = 0
    } else if (type == 2) {
        v = make_float4((v.x + 1.0f) / 2.0f, (v.y + 1.0f) / 2.0f, (v.z + 1.0f) / 2.0f, (v.w + 1.0f) / 2.0f);
    } else if (type == 5) {
        const float nearp = 0.01f, farp = 5.0f;   // LinearizeDepth
        float l = (2.0f * nearp) / (farp + nearp - v.x * (farp - nearp));
        v = make_float4(l, l, l, l);
    }
    P.out[(size_t)y * P.w + x] = unorm8c(v.z) | (unorm8c(v.y) << 8) | (unorm8c(v.x) << 16) | (255u << 24);
}

}  // namespace luz

extern "C" luz_status luz_luminance_histogram(luz_ctx* ctx, luz_frame* f, int32_t source, float delta_time,
                                              luz_histogram* out) {
    using namespace luz;
    if (!ctx || !f || !out) return LUZ_ERR_INVALID;
    const float4* img = source ? f->taa : f->light;
    cudaStream_t st = ctx->stream;
    LUZ_CUDA(ctx, cudaMemsetAsync(f->hist, 0, 256 * 4, st));
    uint32_t blocks = std::min<uint32_t>((f->pixels + 255) / 256, (uint32_t)ctx->sm_count * 8);
    histogram_kernel<<<blocks, 256, 0, st>>>(img, f->pixels, f->hist);
    LUZ_LAUNCHED(ctx, "histogram_kernel");
    histogram_average_kernel<<<1, 256, 0, st>>>(f->hist, f->pixels, delta_time, f->hist_state, f->hist + 256);
    LUZ_LAUNCHED(ctx, "histogram_average_kernel");
    static_assert(sizeof(luz_histogram) == 260 * 4, "luz_histogram layout");
    LUZ_CUDA(ctx, cudaMemcpyAsync(out, f->hist + 256, sizeof(luz_histogram), cudaMemcpyDeviceToHost, st));
    LUZ_CUDA(ctx, cudaStreamSynchronize(st));
    return LUZ_OK;
}

extern "C" luz_status luz_compose(luz_ctx* ctx, luz_frame* f, int32_t source, int32_t image_type) {
    using namespace luz;
    if (!ctx || !f || image_type < 0 || image_type > 6) return LUZ_ERR_INVALID;
    ComposeParams P;
    P.light = source ? f->taa : f->light;
    P.albedo = f->albedo;
    P.normal = f->normal;
    P.material = f->material;
    P.emission = f->emission;
    P.depth = f->depth;
    P.out = f->compose;
    P.w = f->width;
    P.h = f->height;
    P.image_type = image_type;
    dim3 grid((f->width + 15) / 16, (f->height + 15) / 16);
    compose_kernel<<<grid, 256, 0, ctx->stream>>>(P);
    LUZ_LAUNCHED(ctx, "compose_kernel");
    return LUZ_OK;
}

extern "C" luz_status luz_taa(luz_ctx* ctx, luz_frame* f, int32_t reconstruct) {
    if (!ctx || !f) return LUZ_ERR_INVALID;
    return luz::launch_taa(ctx, f, reconstruct ? 1 : 0);
}

extern "C" luz_status luz_taa_reset(luz_ctx* ctx, luz_frame* f) {
    if (!ctx || !f) return LUZ_ERR_INVALID;
    LUZ_CUDA(ctx, cudaMemsetAsync(f->taa, 0, (size_t)f->pixels * 16, ctx->stream));
    return LUZ_OK;
}
