// gbuffer.cuh — the G-buffer pass of one pixel (primary closest hit, material and
// texture maps, the reference's formats), shared by the G-buffer kernel (trace.cu) and
// the batched frame kernel (batch.cu).
#pragma once
#include "raygen.cuh"
#include "traverse.cuh"

namespace luz {

__device__ __forceinline__ uint32_t unorm8(float x) {
    return (uint32_t)(clamp01(x) * 255.0f + 0.5f);
}
__device__ __forceinline__ uint32_t pack_unorm8(float r, float g, float b, float a) {
    return unorm8(r) | (unorm8(g) << 8) | (unorm8(b) << 16) | (unorm8(a) << 24);
}

// Block-wide exclusive scan (256 threads).
__device__ __forceinline__ uint32_t block_excl(uint32_t v, uint32_t* s_tmp /*8*/) {
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_tmp[warp] = x;
    __syncthreads();
    uint32_t pre = 0;
    for (int w = 0; w < warp; ++w) pre += s_tmp[w];
    __syncthreads();
    return pre + x - v;
}


// ---------------------------------------------------------------- textures
// Bilinear sample with repeat addressing of one RGBA8 UNORM level (the reference's
// sampler, VulkanWrapper.cpp:2429-2454): texel centres at (i + 0.5) / size, weights
// from the fractional part, texels as c / 255.
__device__ __forceinline__ uint32_t tex_wrap(float f, uint32_t n) { return repeat_index(f, n); }

__device__ __forceinline__ float4 tex_texel(const DevTexture& t, uint32_t x, uint32_t y) {
    uint32_t c = __ldg(t.texels + (size_t)y * t.width + x);
    return make_float4((float)(c & 255u) / 255.0f, (float)((c >> 8) & 255u) / 255.0f,
                       (float)((c >> 16) & 255u) / 255.0f, (float)(c >> 24) / 255.0f);
}

__device__ __forceinline__ float4 tex_sample(const DevTexture& t, float u, float v) {
    float x = u * (float)t.width - 0.5f, y = v * (float)t.height - 0.5f;
    if (!isfinite(x)) x = 0.0f;
    if (!isfinite(y)) y = 0.0f;
    float fx = floorf(x), fy = floorf(y);
    float ax = x - fx, ay = y - fy;
    uint32_t x0 = tex_wrap(fx, t.width), y0 = tex_wrap(fy, t.height);
    uint32_t x1 = x0 + 1 == t.width ? 0u : x0 + 1, y1 = y0 + 1 == t.height ? 0u : y0 + 1;
    float4 c00 = tex_texel(t, x0, y0), c10 = tex_texel(t, x1, y0), c01 = tex_texel(t, x0, y1),
           c11 = tex_texel(t, x1, y1);
    float bx = 1.0f - ax, by = 1.0f - ay;
    float4 r;
    r.x = (c00.x * bx + c10.x * ax) * by + (c01.x * bx + c11.x * ax) * ay;
    r.y = (c00.y * bx + c10.y * ax) * by + (c01.y * bx + c11.y * ax) * ay;
    r.z = (c00.z * bx + c10.z * ax) * by + (c01.z * bx + c11.z * ax) * ay;
    r.w = (c00.w * bx + c10.w * ax) * by + (c01.w * bx + c11.w * ax) * ay;
    return r;
}

// ---------------------------------------------------------------- G-buffer
struct GbufParams {
    const float4* tlas_nodes;
    uint32_t tlas_node_count;
    const DevInstance* instances;
    uint32_t instance_count;
    const DevShadeInstance* shade;
    const luz_model* models;
    const uint8_t* model_skip;
    uint32_t model_count;
    uint32_t width, height;
    float inverse_proj[16], inverse_view[16], view_proj[16];
    float cam[3];
    uint32_t* albedo;
    float4* normal;
    uint32_t* material;
    uint32_t* emission;
    float* depth;
    uint2* primary_hit;
    uint32_t* hit_instance;   // input index of the hit instance (~0 = miss)
    uint32_t* status;
    const DevTexture* textures;
    uint32_t texture_count;
};

// Texcoord of a hit: the vertex texcoords weighted by the barycentrics.
__device__ __forceinline__ void hit_uv(const DevShadeInstance& S, uint32_t prim, float b0, float b1, float b2,
                                       float& u, float& v) {
    const luz_vertex& v0 = S.vertices[S.indices[3 * prim]];
    const luz_vertex& v1 = S.vertices[S.indices[3 * prim + 1]];
    const luz_vertex& v2 = S.vertices[S.indices[3 * prim + 2]];
    u = (v0.texcoord[0] * b0 + v1.texcoord[0] * b1) + v2.texcoord[0] * b2;
    v = (v0.texcoord[1] * b0 + v1.texcoord[1] * b1) + v2.texcoord[1] * b2;
}

// opaque.frag:29-34: albedo = color * colorMap; discarded below 0.5. Holds the few
// inputs it needs by value: taking the address of the pass's parameter block would move
// the whole block to local memory and every access of the pass with it.
struct AlphaTest {
    const luz_model* models;
    uint32_t model_count;
    const DevTexture* textures;
    uint32_t texture_count;
    const DevShadeInstance* shade;
    __device__ __forceinline__ bool operator()(uint32_t input, uint32_t custom, uint32_t prim, float b0, float b1,
                                               float b2) const {
        if (custom >= model_count) return true;
        const luz_model& m = models[custom];
        if (m.color_map < 0 || (uint32_t)m.color_map >= texture_count) return !(m.color[3] < 0.5f);
        float u, v;
        hit_uv(shade[input], prim, b0, b1, b2, u, v);
        float a = m.color[3] * tex_sample(textures[m.color_map], u, v).w;
        return !(a < 0.5f);
    }
};

// What gbuffer_shade wrote: the normal (xyz) and depth (w), and the albedo, material
// and emission words (a miss: normal 0, depth 1 and zero words).
struct GbufPixel {
    float4 nd;
    uint32_t albedo, material, emission;
};

// The primary ray of pixel (x, y) and its closest hit.
struct GbufRay {
    V3 cam, dir;
    ClosestHit h;
};

// opaque.vert:21-31 + opaque.frag:21-58 at pixel (x, y), in two parts so that a caller
// can end a thread whose ray missed (an early exit: a miss path that rejoins the hit
// path at the end of one inlined function made the G-buffer kernel 9 % slower).
// gbuffer_trace traces the pixel-centre ray; on a miss it writes the miss values of
// every plane and returns false. gbuffer_shade evaluates the hit and writes the planes.
// Params: GbufParams (by value) where G is a kernel parameter, const GbufParams& where
// it sits in device memory.
template <typename Params>
__device__ __forceinline__ bool gbuffer_trace(Params G, uint32_t x, uint32_t y, GbufRay& r) {
    const uint32_t pix = y * G.width + x;
    TlasView T{G.tlas_nodes, G.instances, G.instance_count};
    float u = pixel_uv(x, G.width), v = pixel_uv(y, G.height);
    r.cam = V3{G.cam[0], G.cam[1], G.cam[2]};
    V3 target = depth_to_world(G.inverse_proj, G.inverse_view, u, v, 1.0f);
    r.dir = normalize(target - r.cam);
    uint32_t err = 0;
    const float inf = __int_as_float(0x7f800000);
    bool hit = trace_ray<true, false, AlphaTest>(T, r.cam, r.dir, 0.0f, inf, 0xFFu, G.model_skip, G.model_count, &r.h,
                                                 err, nullptr,
                                                 AlphaTest{G.models, G.model_count, G.textures, G.texture_count, G.shade});
    if (err) atomicOr(G.status, err);
    if (!hit) {
        G.albedo[pix] = 0u;
        G.normal[pix] = make_float4(0.f, 0.f, 0.f, 0.f);
        G.material[pix] = 0u;
        G.emission[pix] = 0u;
        G.depth[pix] = 1.0f;
        G.primary_hit[pix] = make_uint2(0xFFFFFFFFu, 0xFFFFFFFFu);
        G.hit_instance[pix] = 0xFFFFFFFFu;
    }
    return hit;
}

template <typename Params>
__device__ __forceinline__ GbufPixel gbuffer_shade(Params G, uint32_t x, uint32_t y, const GbufRay& r) {
    const uint32_t pix = y * G.width + x;
    const ClosestHit& h = r.h;
    const V3 cam = r.cam, dir = r.dir;
    uint32_t err = 0;
    V3 p = cam + dir * h.t;
    float pw[4] = {p.x, p.y, p.z, 1.0f}, clip[4];
    mat4_mul_vec4(G.view_proj, pw, clip);
    float depth = clip[2] / clip[3];
    // ModelBlock (default of GPUScene.cpp:19-30 when the custom index has no model).
    float color[4] = {1.f, 1.f, 1.f, 1.f}, em[4] = {0.f, 0.f, 0.f, 1.f};
    float metallic = 0.0f, roughness = 0.5f, occlusion = 1.0f;
    int32_t maps[5] = {-1, -1, -1, -1, -1};   // color, metallic-roughness, ao, normal, emission
    if (h.custom < G.model_count) {
        const luz_model& m = G.models[h.custom];
        for (int k = 0; k < 4; ++k) color[k] = m.color[k];
        for (int k = 0; k < 3; ++k) em[k] = m.emission[k];
        metallic = m.metallic;
        roughness = m.roughness;
        maps[0] = m.color_map;
        maps[1] = m.metallic_roughness_map;
        maps[2] = m.ao_map;
        maps[3] = m.normal_map;
        maps[4] = m.emission_map;
        for (int k = 0; k < 5; ++k)
            if (maps[k] >= 0 && (uint32_t)maps[k] >= G.texture_count) {
                err |= LUZ_DEV_BAD_INDEX;
                maps[k] = -1;
            }
    }
    const DevShadeInstance& S = G.shade[h.inst_input];
    uint32_t i0 = S.indices[3 * h.prim], i1 = S.indices[3 * h.prim + 1], i2 = S.indices[3 * h.prim + 2];
    const float* nm = S.normal_mat;
    // opaque.vert:26-30 per vertex: normal and tangent by transpose(inverse(model)),
    // tangent made orthogonal to the normal, bitangent = cross(N, T) * w.
    V3 nv[3], tv[3], bv[3];
    uint32_t ids[3] = {i0, i1, i2};
    const bool tbn = maps[3] >= 0;
    for (int k = 0; k < 3; ++k) {
        const luz_vertex& vx = S.vertices[ids[k]];
        const float* n = vx.normal;
        V3 t = V3{nm[0] * n[0] + nm[1] * n[1] + nm[2] * n[2], nm[3] * n[0] + nm[4] * n[1] + nm[5] * n[2],
                  nm[6] * n[0] + nm[7] * n[1] + nm[8] * n[2]};
        nv[k] = normalize(t);
        if (tbn) {
            const float* g = vx.tangent;
            V3 tg = V3{nm[0] * g[0] + nm[1] * g[1] + nm[2] * g[2], nm[3] * g[0] + nm[4] * g[1] + nm[5] * g[2],
                       nm[6] * g[0] + nm[7] * g[1] + nm[8] * g[2]};
            tg = normalize(tg);
            tv[k] = normalize(tg - nv[k] * dot(tg, nv[k]));
            bv[k] = cross(nv[k], tv[k]) * g[3];
        }
    }
    V3 Ni = (nv[0] * h.b0 + nv[1] * h.b1) + nv[2] * h.b2;
    V3 N = normalize(Ni);
    // opaque.frag:29-51
    float uv[2] = {0.0f, 0.0f};
    if (maps[0] >= 0 || maps[1] >= 0 || maps[2] >= 0 || maps[3] >= 0 || maps[4] >= 0)
        hit_uv(S, h.prim, h.b0, h.b1, h.b2, uv[0], uv[1]);
    if (maps[0] >= 0) {
        float4 c = tex_sample(G.textures[maps[0]], uv[0], uv[1]);
        color[0] *= c.x; color[1] *= c.y; color[2] *= c.z; color[3] *= c.w;
    }
    if (maps[1] >= 0) {
        float4 c = tex_sample(G.textures[maps[1]], uv[0], uv[1]);
        roughness *= c.y;
        metallic *= c.z;
    }
    if (maps[2] >= 0) occlusion = tex_sample(G.textures[maps[2]], uv[0], uv[1]).x;
    if (maps[4] >= 0) {
        float4 c = tex_sample(G.textures[maps[4]], uv[0], uv[1]);
        em[0] *= c.x; em[1] *= c.y; em[2] *= c.z; em[3] *= c.w;
    }
    if (tbn) {
        float4 c = tex_sample(G.textures[maps[3]], uv[0], uv[1]);
        V3 ti = (tv[0] * h.b0 + tv[1] * h.b1) + tv[2] * h.b2;
        V3 bi = (bv[0] * h.b0 + bv[1] * h.b1) + bv[2] * h.b2;
        bool flat_t = ti.x == 0.0f && ti.y == 0.0f && ti.z == 0.0f;
        bool white = c.x == 1.0f && c.y == 1.0f && c.z == 1.0f;
        if (!flat_t && !white) {
            V3 ns = normalize(V3{c.x * 2.0f - 1.0f, c.y * 2.0f - 1.0f, c.z * 2.0f - 1.0f});
            N = normalize((ti * ns.x + bi * ns.y) + Ni * ns.z);
        }
    }
    if (err) atomicOr(G.status, err);
    const GbufPixel out{make_float4(N.x, N.y, N.z, depth), pack_unorm8(color[0], color[1], color[2], color[3]),
                        pack_unorm8(roughness, metallic, occlusion, 1.0f), pack_unorm8(em[0], em[1], em[2], em[3])};
    G.albedo[pix] = out.albedo;
    G.normal[pix] = make_float4(N.x, N.y, N.z, 1.0f);
    G.material[pix] = out.material;
    G.emission[pix] = out.emission;
    G.depth[pix] = depth;
    G.primary_hit[pix] = make_uint2(h.custom, h.prim);
    G.hit_instance[pix] = h.inst_input;
    return out;
}

}  // namespace luz
