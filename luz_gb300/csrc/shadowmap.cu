// shadowmap.cu — the shadow-map pass (shadowMap.vert/.geom/.frag, DeferredRenderer::
// ShadowMapPass, DeferredRenderer.cpp:268-292) as a CUDA depth rasteriser.
//
// Every triangle of every TLAS instance is transformed by its model matrix and the
// light's view-projection (six cube faces for point lights). Cube faces use a
// perspective with near 0, so triangles are clipped against w >= kNearW first; the
// orthographic maps of the other lights need no clipping (w = 1) and discard
// fragments whose depth leaves [0, 1]. Rasterisation samples pixel centres with edge
// functions in single precision and a top-left rule on shared edges; front faces
// (counter-clockwise in framebuffer space) are culled as the reference's pipeline
// does. Depth: the interpolated NDC z for 2D maps, |light - fragment| / zFar for cube
// faces with the world position interpolated perspective-correctly. The depth test
// LESS is an atomic minimum over the depth bits (non-negative floats order like their
// bits), so the result does not depend on the order fragments arrive in.
//
// One thread per (triangle, face) rasterises its triangle when the screen bounding
// box is small; larger triangles go to a queue that one CTA per triangle drains.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "internal.cuh"

namespace luz {

constexpr float kNearW = 1e-5f;
constexpr uint32_t kSmallBox = 256;          // pixels a single thread rasterises
constexpr uint32_t kBigQueue = 1u << 18;     // queued large triangles per launch

struct RVert {   // screen x, y, NDC z, 1/w, world position
    float x, y, z, iw, wx, wy, wz;
};

struct BigTri {
    RVert v[3];
    uint32_t face;
    uint32_t pad[3];
};

struct RasterParams {
    const DevInstanceInput* inst;
    const uint32_t* tri_offset;   // per instance: first triangle (exclusive prefix), n+1 entries
    uint32_t ninst, total_tris, faces, res;
    float vp[6][16];
    float light[3];
    float inv_zfar;
    uint32_t* map;                // faces * res * res depth bits
    BigTri* big;
    uint32_t* big_count;
    uint32_t* status;
};

__device__ __forceinline__ float edge(const RVert& a, const RVert& b, float px, float py) {
    return (b.x - a.x) * (py - a.y) - (b.y - a.y) * (px - a.x);
}
__device__ __forceinline__ bool top_left(const RVert& a, const RVert& b) {
    float dy = b.y - a.y, dx = b.x - a.x;
    return dy > 0.0f || (dy == 0.0f && dx < 0.0f);
}

// Fragment at pixel (px, py) of a back-facing screen triangle; writes the depth.
__device__ __forceinline__ void fragment(const RasterParams& P, const RVert* v, float area2, uint32_t face,
                                         uint32_t px, uint32_t py) {
    float sx = (float)px + 0.5f, sy = (float)py + 0.5f;
    float e0 = edge(v[1], v[2], sx, sy), e1 = edge(v[2], v[0], sx, sy), e2 = edge(v[0], v[1], sx, sy);
    bool in0 = e0 > 0.0f || (e0 == 0.0f && top_left(v[1], v[2]));
    bool in1 = e1 > 0.0f || (e1 == 0.0f && top_left(v[2], v[0]));
    bool in2 = e2 > 0.0f || (e2 == 0.0f && top_left(v[0], v[1]));
    if (!(in0 && in1 && in2)) return;
    float b0 = e0 / area2, b1 = e1 / area2, b2 = e2 / area2;
    float depth;
    if (P.faces == 6) {
        float w0 = b0 * v[0].iw, w1 = b1 * v[1].iw, w2 = b2 * v[2].iw;
        float iw = (w0 + w1) + w2;
        float fx = ((w0 * v[0].wx + w1 * v[1].wx) + w2 * v[2].wx) / iw;
        float fy = ((w0 * v[0].wy + w1 * v[1].wy) + w2 * v[2].wy) / iw;
        float fz = ((w0 * v[0].wz + w1 * v[1].wz) + w2 * v[2].wz) / iw;
        float dx = P.light[0] - fx, dy = P.light[1] - fy, dz = P.light[2] - fz;
        depth = sqrtf(dx * dx + dy * dy + dz * dz) * P.inv_zfar;
    } else {
        depth = (b0 * v[0].z + b1 * v[1].z) + b2 * v[2].z;
    }
    if (!(depth >= 0.0f && depth < 1.0f)) return;   // nothing below the clear value passes LESS
    atomicMin(P.map + (size_t)face * P.res * P.res + (size_t)py * P.res + px, __float_as_uint(depth));
}

struct Box {
    uint32_t x0, y0, x1, y1;   // inclusive
    bool empty;
};

__device__ __forceinline__ Box screen_box(const RVert* v, uint32_t res) {
    float mnx = fminf(fminf(v[0].x, v[1].x), v[2].x), mxx = fmaxf(fmaxf(v[0].x, v[1].x), v[2].x);
    float mny = fminf(fminf(v[0].y, v[1].y), v[2].y), mxy = fmaxf(fmaxf(v[0].y, v[1].y), v[2].y);
    Box b;
    // pixel centres px + 0.5 inside [mn, mx]
    float lx = fmaxf(floorf(mnx - 0.5f), 0.0f), ly = fmaxf(floorf(mny - 0.5f), 0.0f);
    float hx = fminf(ceilf(mxx - 0.5f), (float)res - 1.0f), hy = fminf(ceilf(mxy - 0.5f), (float)res - 1.0f);
    b.empty = !(lx <= hx && ly <= hy);
    if (b.empty) return b;
    b.x0 = (uint32_t)lx;
    b.y0 = (uint32_t)ly;
    b.x1 = (uint32_t)hx;
    b.y1 = (uint32_t)hy;
    return b;
}

// Framebuffer-space orientation of the Vulkan rule: a = -1/2 sum(x_i y_i+1 - x_i+1 y_i),
// front-facing (counter-clockwise) when a > 0. Returns the edge-function area (2x the
// standard signed area, = -2a) of a triangle to rasterise, 0 when culled.
__device__ __forceinline__ float raster_area(const RVert* v) {
    float s = (v[0].x * v[1].y - v[1].x * v[0].y) + (v[1].x * v[2].y - v[2].x * v[1].y) +
              (v[2].x * v[0].y - v[0].x * v[2].y);
    float a = -0.5f * s;
    if (!(a < 0.0f)) return 0.0f;   // front face (culled), degenerate or NaN
    return (v[1].x - v[0].x) * (v[2].y - v[0].y) - (v[1].y - v[0].y) * (v[2].x - v[0].x);
}

__device__ __forceinline__ void raster_tri(const RasterParams& P, const RVert* v, uint32_t face) {
    float area2 = raster_area(v);
    if (!(area2 > 0.0f)) return;
    Box b = screen_box(v, P.res);
    if (b.empty) return;
    uint32_t pixels = (b.x1 - b.x0 + 1) * (b.y1 - b.y0 + 1);
    if (pixels <= kSmallBox) {
        for (uint32_t py = b.y0; py <= b.y1; ++py)
            for (uint32_t px = b.x0; px <= b.x1; ++px) fragment(P, v, area2, face, px, py);
        return;
    }
    uint32_t slot = atomicAdd(P.big_count, 1u);
    if (slot >= kBigQueue) {
        atomicOr(P.status, (uint32_t)LUZ_DEV_RASTER_OVERFLOW);
        return;
    }
    BigTri& t = P.big[slot];
    t.v[0] = v[0];
    t.v[1] = v[1];
    t.v[2] = v[2];
    t.face = face;
}

__device__ __forceinline__ void clip_to_screen(const RasterParams& P, const float c[4], const float w[3], RVert& o) {
    float iw = 1.0f / c[3];
    o.x = (c[0] * iw * 0.5f + 0.5f) * (float)P.res;
    o.y = (c[1] * iw * 0.5f + 0.5f) * (float)P.res;
    o.z = c[2] * iw;
    o.iw = iw;
    o.wx = w[0];
    o.wy = w[1];
    o.wz = w[2];
}

__global__ void __launch_bounds__(256) shadow_raster_kernel(RasterParams P) {
    uint64_t item = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (item >= (uint64_t)P.total_tris * P.faces) return;
    uint32_t face = (uint32_t)(item % P.faces), tri = (uint32_t)(item / P.faces);
    uint32_t lo = 0, hi = P.ninst - 1;
    while (lo < hi) {   // instance of the triangle
        uint32_t mid = (lo + hi + 1) >> 1;
        if (P.tri_offset[mid] <= tri) lo = mid; else hi = mid - 1;
    }
    const DevInstanceInput& I = P.inst[lo];
    uint32_t local = tri - P.tri_offset[lo];
    const float* m = I.o2w;
    float clip[3][4], world[3][3];
    for (int k = 0; k < 3; ++k) {
        const float* p = I.vertices[I.indices[3 * local + k]].position;
        // modelMat * vec4(p, 1) (shadowMap.vert), then viewProj[face] * world (shadowMap.geom)
        for (int r = 0; r < 3; ++r) world[k][r] = m[r * 4 + 0] * p[0] + m[r * 4 + 1] * p[1] + m[r * 4 + 2] * p[2] + m[r * 4 + 3];
        float w4[4] = {world[k][0], world[k][1], world[k][2], 1.0f};
        mat4_mul_vec4(P.vp[face], w4, clip[k]);
    }
    if (P.faces != 6) {
        RVert v[3];
        for (int k = 0; k < 3; ++k) clip_to_screen(P, clip[k], world[k], v[k]);
        raster_tri(P, v, face);
        return;
    }
    // Sutherland-Hodgman against w >= kNearW, attributes linear in clip space
    float pc[4][4], pw[4][3];
    int n = 0;
    for (int k = 0; k < 3; ++k) {
        const int j = (k + 1) % 3;
        const bool ink = clip[k][3] >= kNearW, inj = clip[j][3] >= kNearW;
        if (ink) {
            for (int q = 0; q < 4; ++q) pc[n][q] = clip[k][q];
            for (int q = 0; q < 3; ++q) pw[n][q] = world[k][q];
            ++n;
        }
        if (ink != inj) {
            float t = (kNearW - clip[k][3]) / (clip[j][3] - clip[k][3]);
            for (int q = 0; q < 4; ++q) pc[n][q] = clip[k][q] + (clip[j][q] - clip[k][q]) * t;
            for (int q = 0; q < 3; ++q) pw[n][q] = world[k][q] + (world[j][q] - world[k][q]) * t;
            ++n;
        }
    }
    if (n < 3) return;
    RVert sv[4];
    for (int k = 0; k < n; ++k) clip_to_screen(P, pc[k], pw[k], sv[k]);
    RVert t0[3] = {sv[0], sv[1], sv[2]};
    raster_tri(P, t0, face);
    if (n == 4) {
        RVert t1[3] = {sv[0], sv[2], sv[3]};
        raster_tri(P, t1, face);
    }
}

__global__ void __launch_bounds__(256) shadow_raster_big_kernel(RasterParams P) {
    const uint32_t count = min(*P.big_count, kBigQueue);
    for (uint32_t i = blockIdx.x; i < count; i += gridDim.x) {
        BigTri t = P.big[i];
        float area2 = raster_area(t.v);
        Box b = screen_box(t.v, P.res);
        if (!(area2 > 0.0f) || b.empty) continue;
        uint32_t wdt = b.x1 - b.x0 + 1, pixels = wdt * (b.y1 - b.y0 + 1);
        for (uint32_t k = threadIdx.x; k < pixels; k += blockDim.x)
            fragment(P, t.v, area2, t.face, b.x0 + k % wdt, b.y0 + k / wdt);
    }
}

__global__ void fill_kernel(uint32_t* p, size_t n, uint32_t v) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) p[i] = v;
}

}  // namespace luz

using namespace luz;

static luz_status frame_render_shadow_maps_body(luz_ctx* ctx, luz_frame* f, const luz_tlas* t,
                                                const luz_shadow_light* lights, uint32_t count,
                                                uint32_t res) {
    if (!ctx || !f || !t || (count && !lights) || res == 0 || res > 8192) return LUZ_ERR_INVALID;
    cudaStream_t st = ctx->stream;
    LUZ_CUDA(ctx, cudaStreamSynchronize(st));
    // layout: one arena with every light's faces
    std::vector<size_t> off(count);
    std::vector<uint32_t> faces(count);
    size_t total = 0;
    for (uint32_t l = 0; l < count; ++l) {
        faces[l] = lights[l].faces;
        if (faces[l] != 0 && faces[l] != 1 && faces[l] != 6)
            return set_error(ctx, LUZ_ERR_INVALID, "shadow light " + std::to_string(l) + ": faces must be 0, 1 or 6");
        off[l] = total;
        total += (size_t)faces[l] * res * res;
    }
    if (total * 4 > f->shadow_maps_bytes || !f->d_shadow_maps) {
        if (f->d_shadow_maps) cudaFree(f->d_shadow_maps);
        f->d_shadow_maps = nullptr;
        f->shadow_maps_bytes = 0;
        LUZ_CUDA(ctx, cudaMalloc(&f->d_shadow_maps, std::max(total, (size_t)1) * 4));
        f->shadow_maps_bytes = std::max(total, (size_t)1) * 4;
    }
    if (f->d_shadow_lights) cudaFree(f->d_shadow_lights);
    f->d_shadow_lights = nullptr;
    LUZ_CUDA(ctx, cudaMalloc(&f->d_shadow_lights, std::max(count, 1u) * sizeof(DevShadowLight)));
    std::vector<DevShadowLight> table(std::max(count, 1u));
    for (uint32_t l = 0; l < count; ++l) {
        DevShadowLight& d = table[l];
        d.map = f->d_shadow_maps + off[l];
        memcpy(d.view_proj0, lights[l].view_proj[0], 64);
        memcpy(d.position, lights[l].position, 12);
        d.z_far = lights[l].z_far;
        d.faces = faces[l];
        d.res = res;
    }
    LUZ_CUDA(ctx, cudaMemcpy(f->d_shadow_lights, table.data(), std::max(count, 1u) * sizeof(DevShadowLight),
                             cudaMemcpyHostToDevice));
    f->shadow_light_count = count;
    f->shadow_res = res;
    f->h_shadow_offset = off;
    f->h_shadow_faces = faces;
    if (total) {
        fill_kernel<<<ctx->sm_count * 4, 256, 0, st>>>((uint32_t*)f->d_shadow_maps, total, 0x3F800000u);   // 1.0f
        LUZ_LAUNCHED(ctx, "fill_kernel");
    }
    // instances of the TLAS (object-to-world rows, vertex / index buffers)
    uint32_t ninst = t->count;
    if (ninst == 0 || total == 0) return LUZ_OK;
    std::vector<uint32_t> tri_off(ninst + 1, 0);
    for (uint32_t i = 0; i < ninst; ++i) tri_off[i + 1] = tri_off[i] + t->h_input[i].blas_prims;
    const uint32_t total_tris = tri_off[ninst];
    if (total_tris == 0) return LUZ_OK;
    uint32_t* d_tri_off = nullptr;
    BigTri* d_big = nullptr;
    uint32_t* d_big_count = nullptr;
    auto cleanup = [&]() {
        if (d_tri_off) cudaFree(d_tri_off);
        if (d_big) cudaFree(d_big);
        if (d_big_count) cudaFree(d_big_count);
    };
    if (cudaMalloc(&d_tri_off, (ninst + 1) * 4) != cudaSuccess || cudaMalloc(&d_big, kBigQueue * sizeof(BigTri)) != cudaSuccess ||
        cudaMalloc(&d_big_count, 4) != cudaSuccess) {
        cleanup();
        return set_error(ctx, LUZ_ERR_OOM, "shadow-map raster buffers");
    }
    LUZ_CUDA(ctx, cudaMemcpy(d_tri_off, tri_off.data(), (ninst + 1) * 4, cudaMemcpyHostToDevice));
    luz_status result = LUZ_OK;
    for (uint32_t l = 0; l < count && result == LUZ_OK; ++l) {
        if (!faces[l]) continue;
        RasterParams P;
        P.inst = t->d_input;
        P.tri_offset = d_tri_off;
        P.ninst = ninst;
        P.total_tris = total_tris;
        P.faces = faces[l];
        P.res = res;
        memcpy(P.vp, lights[l].view_proj, sizeof(P.vp));
        memcpy(P.light, lights[l].position, 12);
        P.inv_zfar = 1.0f / lights[l].z_far;
        P.map = (uint32_t*)(f->d_shadow_maps + off[l]);
        P.big = d_big;
        P.big_count = d_big_count;
        P.status = ctx->d_status;
        cudaMemsetAsync(d_big_count, 0, 4, st);
        uint64_t items = (uint64_t)total_tris * faces[l];
        shadow_raster_kernel<<<(uint32_t)((items + 255) / 256), 256, 0, st>>>(P);
        if (check_launch(ctx, "shadow_raster_kernel") != LUZ_OK) { result = LUZ_ERR_CUDA; break; }
        ctx->launches++;
        shadow_raster_big_kernel<<<ctx->sm_count * 2, 256, 0, st>>>(P);
        if (check_launch(ctx, "shadow_raster_big_kernel") != LUZ_OK) { result = LUZ_ERR_CUDA; break; }
        ctx->launches++;
    }
    cudaError_t e = cudaStreamSynchronize(st);
    cleanup();
    if (result != LUZ_OK) return result;
    if (e != cudaSuccess) return cuda_error(ctx, e, "shadow-map rasterisation");
    return LUZ_OK;
}

extern "C" luz_status luz_frame_render_shadow_maps(luz_ctx* ctx, luz_frame* f, const luz_tlas* t,
                                                   const luz_shadow_light* lights, uint32_t count,
                                                   uint32_t res) {
    return guarded(ctx, [&] { return frame_render_shadow_maps_body(ctx, f, t, lights, count, res); });
}

extern "C" luz_status luz_frame_read_shadow_map(luz_ctx* ctx, luz_frame* f, uint32_t light, float* dst, size_t bytes) {
    if (!ctx || !f || !dst || light >= f->shadow_light_count) return LUZ_ERR_INVALID;
    size_t n = (size_t)f->h_shadow_faces[light] * f->shadow_res * f->shadow_res;
    if (bytes < n * 4) return set_error(ctx, LUZ_ERR_INVALID, "short buffer for the shadow map");
    LUZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (n) LUZ_CUDA(ctx, cudaMemcpy(dst, f->d_shadow_maps + f->h_shadow_offset[light], n * 4, cudaMemcpyDeviceToHost));
    return LUZ_OK;
}
