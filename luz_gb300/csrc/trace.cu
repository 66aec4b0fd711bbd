// trace.cu — primary-ray G-buffer and the compaction of lit pixels (the inputs of
// the visibility kernel in visibility.cu).
#include <algorithm>
#include <cstddef>
#include <cstring>

#include "raygen.cuh"
#include "traverse.cuh"

namespace luz {

constexpr int kSmemTlasNodes = 1024;   // 64 KB of TLAS top levels per CTA

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

__device__ __forceinline__ void stage_tlas(const float4* __restrict__ g, uint32_t node_count,
                                           float4* s, uint32_t& staged) {
    staged = min(node_count, (uint32_t)kSmemTlasNodes);
    for (uint32_t i = threadIdx.x; i < staged * kNodeF4; i += blockDim.x) s[i] = __ldg(g + i);
    __syncthreads();
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
    uint32_t* status;
};

// opaque.vert:21-31 + opaque.frag:21-58 evaluated at the closest hit of the
// pixel-centre ray. 16x16 pixel tiles per CTA.
__global__ void __launch_bounds__(256) gbuffer_kernel(GbufParams G) {
    extern __shared__ float4 s_nodes[];
    uint32_t staged;
    stage_tlas(G.tlas_nodes, G.tlas_node_count, s_nodes, staged);
    uint32_t tiles_x = (G.width + 15) / 16;
    uint32_t tx = blockIdx.x % tiles_x, ty = blockIdx.x / tiles_x;
    uint32_t x = tx * 16 + (threadIdx.x & 15), y = ty * 16 + (threadIdx.x >> 4);
    if (x >= G.width || y >= G.height) return;
    uint32_t pix = y * G.width + x;
    TlasView T{G.tlas_nodes, s_nodes, staged, G.instances, G.instance_count};
    float u = pixel_uv(x, G.width), v = pixel_uv(y, G.height);
    V3 cam = V3{G.cam[0], G.cam[1], G.cam[2]};
    V3 target = depth_to_world(G.inverse_proj, G.inverse_view, u, v, 1.0f);
    V3 dir = normalize(target - cam);
    ClosestHit h;
    uint32_t err = 0;
    const float inf = __int_as_float(0x7f800000);
    bool hit = trace_ray<true>(T, cam, dir, 0.0f, inf, 0xFFu, G.model_skip, G.model_count, &h, err);
    if (err) atomicOr(G.status, err);
    if (!hit) {
        G.albedo[pix] = 0u;
        G.normal[pix] = make_float4(0.f, 0.f, 0.f, 0.f);
        G.material[pix] = 0u;
        G.emission[pix] = 0u;
        G.depth[pix] = 1.0f;
        G.primary_hit[pix] = make_uint2(0xFFFFFFFFu, 0xFFFFFFFFu);
        return;
    }
    V3 p = cam + dir * h.t;
    float pw[4] = {p.x, p.y, p.z, 1.0f}, clip[4];
    mat4_mul_vec4(G.view_proj, pw, clip);
    float depth = clip[2] / clip[3];
    // ModelBlock (default of GPUScene.cpp:19-30 when the custom index has no model).
    float color[4] = {1.f, 1.f, 1.f, 1.f}, em[3] = {0.f, 0.f, 0.f};
    float metallic = 0.0f, roughness = 0.5f;
    if (h.custom < G.model_count) {
        const luz_model& m = G.models[h.custom];
        for (int k = 0; k < 4; ++k) color[k] = m.color[k];
        for (int k = 0; k < 3; ++k) em[k] = m.emission[k];
        metallic = m.metallic;
        roughness = m.roughness;
    }
    const DevShadeInstance& S = G.shade[h.inst_input];
    uint32_t i0 = S.indices[3 * h.prim], i1 = S.indices[3 * h.prim + 1], i2 = S.indices[3 * h.prim + 2];
    const float* nm = S.normal_mat;
    V3 nv[3];
    uint32_t ids[3] = {i0, i1, i2};
    for (int k = 0; k < 3; ++k) {
        const float* n = S.vertices[ids[k]].normal;
        V3 t = V3{nm[0] * n[0] + nm[1] * n[1] + nm[2] * n[2], nm[3] * n[0] + nm[4] * n[1] + nm[5] * n[2],
                  nm[6] * n[0] + nm[7] * n[1] + nm[8] * n[2]};
        nv[k] = normalize(t);
    }
    V3 N = normalize((nv[0] * h.b0 + nv[1] * h.b1) + nv[2] * h.b2);
    G.albedo[pix] = pack_unorm8(color[0], color[1], color[2], color[3]);
    G.normal[pix] = make_float4(N.x, N.y, N.z, 1.0f);
    G.material[pix] = pack_unorm8(roughness, metallic, 1.0f, 1.0f);
    G.emission[pix] = pack_unorm8(em[0], em[1], em[2], 1.0f);
    G.depth[pix] = depth;
    G.primary_hit[pix] = make_uint2(h.custom, h.prim);
}

// ---------------------------------------------------------------- lit-pixel compaction
// A pixel is lit when length(N) != 0 (light.frag:178). Chunks of 1024 pixels;
// the compacted order is the pixel order.
constexpr int kChunk = 1024;

__device__ __forceinline__ bool pixel_lit(const float4* normal, uint32_t pix, uint32_t n) {
    if (pix >= n) return false;
    float4 v = normal[pix];
    return !(length(V3{v.x, v.y, v.z}) == 0.0f);
}

__global__ void __launch_bounds__(256) lit_count_kernel(const float4* normal, uint32_t n,
                                                        uint32_t* chunk_counts) {
    __shared__ uint32_t s_tmp[8];
    uint32_t base = blockIdx.x * kChunk + threadIdx.x * 4;
    uint32_t c = 0;
    for (int k = 0; k < 4; ++k) c += pixel_lit(normal, base + k, n);
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xFFFFFFFFu, c, o);
    if ((threadIdx.x & 31) == 0) s_tmp[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < 8; ++w) t += s_tmp[w];
        chunk_counts[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(1024) lit_scan_kernel(uint32_t* chunk_counts, uint32_t chunks,
                                                        uint32_t* total) {
    __shared__ uint32_t s_warp[32];
    __shared__ uint32_t s_carry;
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    for (uint32_t base = 0; base < chunks; base += 1024) {
        uint32_t i = base + threadIdx.x;
        uint32_t v = i < chunks ? chunk_counts[i] : 0u;
        uint32_t x = v;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) s_warp[warp] = x;
        __syncthreads();
        uint32_t pre = 0, all = 0;
        for (int w = 0; w < 32; ++w) {
            if (w < warp) pre += s_warp[w];
            all += s_warp[w];
        }
        uint32_t carry = s_carry;
        if (i < chunks) chunk_counts[i] = carry + pre + x - v;
        __syncthreads();
        if (threadIdx.x == 0) s_carry = carry + all;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = s_carry;
}

__global__ void __launch_bounds__(256) lit_write_kernel(const float4* normal, const float* depth,
                                                        uint32_t width, uint32_t height,
                                                        const uint32_t* chunk_offsets,
                                                        const float* inverse_proj,
                                                        const float* inverse_view, float4* surf) {
    __shared__ uint32_t s_tmp[8];
    __shared__ float s_ip[16], s_iv[16];
    if (threadIdx.x < 16) { s_ip[threadIdx.x] = inverse_proj[threadIdx.x]; s_iv[threadIdx.x] = inverse_view[threadIdx.x]; }
    __syncthreads();
    uint32_t n = width * height;
    uint32_t base = blockIdx.x * kChunk + threadIdx.x * 4;
    bool lit[4];
    uint32_t c = 0;
    for (int k = 0; k < 4; ++k) { lit[k] = pixel_lit(normal, base + k, n); c += lit[k]; }
    uint32_t pos = chunk_offsets[blockIdx.x] + block_excl(c, s_tmp);
    for (int k = 0; k < 4; ++k) {
        if (!lit[k]) continue;
        uint32_t pix = base + k;
        uint32_t x = pix % width, y = pix / width;
        V3 p = depth_to_world(s_ip, s_iv, pixel_uv(x, width), pixel_uv(y, height), depth[pix]);
        float4 nn = normal[pix];
        surf[2 * (size_t)pos] = make_float4(p.x, p.y, p.z, __uint_as_float(pix));
        surf[2 * (size_t)pos + 1] = make_float4(nn.x, nn.y, nn.z, 0.f);
        ++pos;
    }
}

// ---------------------------------------------------------------- host launchers
luz_status launch_gbuffer(luz_ctx* ctx, luz_frame* f, const luz_tlas* t) {
    GbufParams G;
    G.tlas_nodes = t->nodes;
    G.tlas_node_count = t->count ? t->node_count : 0;
    G.instances = t->instances;
    G.instance_count = t->count;
    G.shade = t->shade;
    G.models = f->d_models;
    G.model_skip = f->d_model_skip;
    G.model_count = f->model_count;
    G.width = f->width;
    G.height = f->height;
    memcpy(G.inverse_proj, f->h_scene.inverse_proj, 64);
    memcpy(G.inverse_view, f->h_scene.inverse_view, 64);
    memcpy(G.view_proj, f->h_scene.view_proj, 64);
    memcpy(G.cam, f->h_scene.cam_pos, 12);
    G.albedo = f->albedo;
    G.normal = f->normal;
    G.material = f->material;
    G.emission = f->emission;
    G.depth = f->depth;
    G.primary_hit = f->primary_hit;
    G.status = ctx->d_status;
    uint32_t tiles = ((f->width + 15) / 16) * ((f->height + 15) / 16);
    static bool attr_set = false;
    if (!attr_set) {
        LUZ_CUDA(ctx, cudaFuncSetAttribute(gbuffer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           kSmemTlasNodes * 64));
        attr_set = true;
    }
    size_t smem = (size_t)std::min<uint32_t>(G.tlas_node_count, kSmemTlasNodes) * 64;
    gbuffer_kernel<<<tiles, 256, smem, ctx->stream>>>(G);
    LUZ_LAUNCHED(ctx, "gbuffer_kernel");
    // compaction of lit pixels
    uint32_t chunks = (f->pixels + kChunk - 1) / kChunk;
    lit_count_kernel<<<chunks, 256, 0, ctx->stream>>>(f->normal, f->pixels, f->block_counts);
    LUZ_LAUNCHED(ctx, "lit_count_kernel");
    lit_scan_kernel<<<1, 1024, 0, ctx->stream>>>(f->block_counts, chunks, f->lit_count);
    LUZ_LAUNCHED(ctx, "lit_scan_kernel");
    lit_write_kernel<<<chunks, 256, 0, ctx->stream>>>(f->normal, f->depth, f->width, f->height,
                                                      f->block_counts,
                                                      (const float*)((const char*)f->d_scene + offsetof(luz_scene, inverse_proj)),
                                                      (const float*)((const char*)f->d_scene + offsetof(luz_scene, inverse_view)),
                                                      f->surf);
    LUZ_LAUNCHED(ctx, "lit_write_kernel");
    return LUZ_OK;
}

}  // namespace luz
