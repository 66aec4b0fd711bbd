// trace.cu — primary-ray G-buffer and the compaction of lit pixels (the inputs of
// the visibility kernel in visibility.cu).
#include <algorithm>
#include <cstddef>
#include <cstring>

#include "gbuffer.cuh"

namespace luz {

const float4* tlas_leaf_boxes(const luz_tlas* t);

// 8x8 pixels per CTA of 64 threads, 16 CTAs per SM (64 registers): measured at
// 1080p 0.65 ms against 0.75 ms for 16x16-pixel CTAs with the TLAS top staged in
// shared memory (L1 holds it as well, and the CTAs retire at a finer grain).
constexpr uint32_t kGbTile = 8;
constexpr int kGbMinBlocks = 16;

// ---------------------------------------------------------------- tile candidate lists
// Primary rays of one 8x8 tile leave the camera inside the cone of the tile's four
// corner-pixel rays (the pixel targets on the far plane are a projective image of the
// pixel grid, so the corner pixels bound them). A TLAS leaf whose box lies outside
// that cone, or behind the camera, cannot be hit by any of the tile's rays: the
// G-buffer traces a tile whose list of remaining leaves has at most kGbFineMax entries
// through those leaves only (nearest box first), a tile with none as all misses, and
// any other tile through the TLAS. Lists are built per frame in two levels: 64x64-pixel
// coarse tiles test every leaf, 8x8 tiles test their coarse tile's list. The closest
// hit, ties broken by (instance, primitive), is the same over any superset of the
// instances the rays reach, so the planes are bit for bit those of the full traversal.
constexpr uint32_t kGbCoarse = 64;
constexpr uint32_t kGbCoarseMax = 255;    // coarse list: count + 255 leaves
constexpr uint32_t kGbFineMax = 15;       // fine list: count + 15 leaves
constexpr uint32_t kGbListAll = 0xFFFFFFFFu;   // count: trace through the TLAS
// The coarse lists test every leaf per 64x64 tile: above this many instances every
// tile traces through the TLAS.
constexpr uint32_t kGbListMaxInstances = 65536;

// The cone of the primary rays of the pixels [x0, x1] x [y0, y1]: four planes through
// the camera spanned by adjacent corner rays and the plane normal to the centre ray,
// normals pointing inside. ok = false when a corner ray is not finite or not within 90
// degrees of the centre ray (no cone to cull with).
struct PixelCone {
    V3 n[5];
    bool ok;
};

template <typename Params>
__device__ __forceinline__ V3 pixel_ray_dir(const Params& G, V3 cam, uint32_t x, uint32_t y) {
    return normalize(depth_to_world(G.inverse_proj, G.inverse_view, pixel_uv(x, G.width), pixel_uv(y, G.height), 1.0f) -
                     cam);
}

template <typename Params>
__device__ __forceinline__ PixelCone pixel_cone(const Params& G, V3 cam, uint32_t x0, uint32_t y0, uint32_t x1,
                                                uint32_t y1) {
    PixelCone c;
    const V3 d00 = pixel_ray_dir(G, cam, x0, y0), d10 = pixel_ray_dir(G, cam, x1, y0),
             d01 = pixel_ray_dir(G, cam, x0, y1), d11 = pixel_ray_dir(G, cam, x1, y1);
    const V3 dc = normalize(d00 + d10 + d01 + d11);
    c.ok = finite3(d00) && finite3(d10) && finite3(d01) && finite3(d11) && finite3(dc) && dot(d00, dc) > 0.0f &&
           dot(d10, dc) > 0.0f && dot(d01, dc) > 0.0f && dot(d11, dc) > 0.0f;
    c.n[0] = cross(d00, d10);
    c.n[1] = cross(d10, d11);
    c.n[2] = cross(d11, d01);
    c.n[3] = cross(d01, d00);
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (dot(c.n[k], dc) < 0.0f) c.n[k] = V3{-c.n[k].x, -c.n[k].y, -c.n[k].z};
    c.n[4] = dc;
    return c;
}

// True when the box lies on the outer side of one of the cone's planes by more than
// 2^-12 x |n|_1 x (|p - cam|_1 + |hi - lo|_1), p the box corner farthest along n: a
// margin far above the rounding of the corner rays and of these products. A NaN box is
// kept; an empty (inverted) box is culled or kept.
__device__ __forceinline__ bool box_outside_cone(const PixelCone& c, V3 cam, float4 lo, float4 hi) {
    const float ext = (fabsf(hi.x - lo.x) + fabsf(hi.y - lo.y)) + fabsf(hi.z - lo.z);
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        const V3 n = c.n[k];
        const V3 p = V3{(n.x >= 0.0f ? hi.x : lo.x) - cam.x, (n.y >= 0.0f ? hi.y : lo.y) - cam.y,
                        (n.z >= 0.0f ? hi.z : lo.z) - cam.z};
        const float v = (n.x * p.x + n.y * p.y) + n.z * p.z;
        const float m = 0x1p-12f * ((fabsf(n.x) + fabsf(n.y)) + fabsf(n.z)) *
                        (((fabsf(p.x) + fabsf(p.y)) + fabsf(p.z)) + ext);
        if (v < -m) return true;
    }
    return false;
}

// One block of 256 threads per 64x64-pixel coarse tile: the leaves (in index order)
// whose boxes the tile's cone does not cull; kGbListAll past kGbCoarseMax.
__global__ void __launch_bounds__(256) gb_coarse_kernel(GbufParams G, const float4* __restrict__ leaf_box, uint32_t n,
                                                        uint32_t* __restrict__ coarse) {
    __shared__ uint32_t s_warp[8];
    const uint32_t cx = (G.width + kGbCoarse - 1) / kGbCoarse;
    const uint32_t tx = blockIdx.x % cx, ty = blockIdx.x / cx;
    const uint32_t x0 = tx * kGbCoarse, y0 = ty * kGbCoarse;
    const uint32_t x1 = min(x0 + kGbCoarse, G.width) - 1, y1 = min(y0 + kGbCoarse, G.height) - 1;
    const V3 cam = V3{G.cam[0], G.cam[1], G.cam[2]};
    const PixelCone c = pixel_cone(G, cam, x0, y0, x1, y1);
    uint32_t* list = coarse + (size_t)blockIdx.x * (kGbCoarseMax + 1);
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    uint32_t total = 0;
    for (uint32_t base = 0; c.ok && base < n; base += blockDim.x) {
        const uint32_t j = base + tid;
        const bool keep = j < n && !box_outside_cone(c, cam, leaf_box[2 * j], leaf_box[2 * j + 1]);
        const uint32_t bal = __ballot_sync(0xFFFFFFFFu, keep);
        if (lane == 0) s_warp[warp] = __popc(bal);
        __syncthreads();
        uint32_t off = total, sum = 0;
        for (uint32_t w = 0; w < blockDim.x / 32; ++w) {
            if (w < warp) off += s_warp[w];
            sum += s_warp[w];
        }
        const uint32_t pos = off + __popc(bal & ((1u << lane) - 1u));
        if (keep && pos < kGbCoarseMax) list[1 + pos] = j;
        total += sum;
        __syncthreads();
    }
    if (tid == 0) list[0] = c.ok && total <= kGbCoarseMax ? total : kGbListAll;
}

// One block of 64 threads per coarse tile, one thread per 8x8 tile inside it: the
// coarse list's leaves its own cone does not cull, nearest box (from the camera) first.
__global__ void __launch_bounds__(64) gb_fine_kernel(GbufParams G, const float4* __restrict__ leaf_box,
                                                     const uint32_t* __restrict__ coarse, uint32_t* __restrict__ fine) {
    __shared__ float4 s_box[2 * kGbCoarseMax];
    __shared__ uint32_t s_leaf[kGbCoarseMax];
    const uint32_t cx = (G.width + kGbCoarse - 1) / kGbCoarse;
    const uint32_t ctx_ = blockIdx.x % cx, cty = blockIdx.x / cx;
    const uint32_t* cl = coarse + (size_t)blockIdx.x * (kGbCoarseMax + 1);
    const uint32_t cn = cl[0];
    const uint32_t nc = cn == kGbListAll ? 0u : cn;
    for (uint32_t k = threadIdx.x; k < nc; k += blockDim.x) {
        const uint32_t j = cl[1 + k];
        s_leaf[k] = j;
        s_box[2 * k] = leaf_box[2 * j];
        s_box[2 * k + 1] = leaf_box[2 * j + 1];
    }
    __syncthreads();
    const uint32_t per = kGbCoarse / kGbTile;
    const uint32_t fx = ctx_ * per + threadIdx.x % per, fy = cty * per + threadIdx.x / per;
    const uint32_t x0 = fx * kGbTile, y0 = fy * kGbTile;
    if (x0 >= G.width || y0 >= G.height) return;
    const uint32_t tiles_x = (G.width + kGbTile - 1) / kGbTile;
    uint32_t* list = fine + ((size_t)fy * tiles_x + fx) * (kGbFineMax + 1);
    if (cn == kGbListAll) {
        list[0] = kGbListAll;
        return;
    }
    const uint32_t x1 = min(x0 + kGbTile, G.width) - 1, y1 = min(y0 + kGbTile, G.height) - 1;
    const V3 cam = V3{G.cam[0], G.cam[1], G.cam[2]};
    const PixelCone c = pixel_cone(G, cam, x0, y0, x1, y1);
    if (!c.ok) {
        list[0] = kGbListAll;
        return;
    }
    uint32_t cnt = 0, leaf[kGbFineMax];
    float dist[kGbFineMax];
    for (uint32_t k = 0; k < nc; ++k) {
        const float4 lo = s_box[2 * k], hi = s_box[2 * k + 1];
        if (box_outside_cone(c, cam, lo, hi)) continue;
        if (cnt == kGbFineMax) { ++cnt; break; }
        // insertion by the distance from the camera to the box
        const float ex = fmaxf(fmaxf(lo.x - cam.x, cam.x - hi.x), 0.0f);
        const float ey = fmaxf(fmaxf(lo.y - cam.y, cam.y - hi.y), 0.0f);
        const float ez = fmaxf(fmaxf(lo.z - cam.z, cam.z - hi.z), 0.0f);
        const float d = (ex * ex + ey * ey) + ez * ez;
        uint32_t q = cnt++;
        while (q > 0 && dist[q - 1] > d) {
            dist[q] = dist[q - 1];
            leaf[q] = leaf[q - 1];
            --q;
        }
        dist[q] = d;
        leaf[q] = s_leaf[k];
    }
    if (cnt > kGbFineMax) {
        list[0] = kGbListAll;
        return;
    }
    list[0] = cnt;
    for (uint32_t k = 0; k < cnt; ++k) list[1 + k] = leaf[k];
}

// The G-buffer pass: kGbTile x kGbTile pixel tiles per CTA, one pixel per thread. The
// steps are those of gbuffer_trace and gbuffer_shade (gbuffer.cuh, which the batch frame
// kernel calls over its scenes' parameters in device memory), written out here over the
// kernel's own parameter block: the same steps through the shared functions measured
// 9 % slower at 1080p (0.673 vs 0.616 ms) with the parameter block passed by value or by
// reference. The batch tests check that the two give the same planes bit for bit.
__global__ void __launch_bounds__(kGbTile * kGbTile, kGbMinBlocks) gbuffer_kernel(GbufParams G,
                                                                                   const uint32_t* __restrict__ lists) {
    uint32_t tiles_x = (G.width + kGbTile - 1) / kGbTile;
    uint32_t tx = blockIdx.x % tiles_x, ty = blockIdx.x / tiles_x;
    uint32_t x = tx * kGbTile + (threadIdx.x % kGbTile), y = ty * kGbTile + (threadIdx.x / kGbTile);
    if (x >= G.width || y >= G.height) return;
    uint32_t pix = y * G.width + x;
    uint32_t err = 0;

    // The tile's candidate leaves (none: every ray misses; kGbListAll: the TLAS).
    const uint32_t* list = lists + (size_t)blockIdx.x * (kGbFineMax + 1);
    const uint32_t cnt = __ldg(list);
    TlasView T{G.tlas_nodes, G.instances, G.instance_count};
    float u = pixel_uv(x, G.width), v = pixel_uv(y, G.height);
    V3 cam = V3{G.cam[0], G.cam[1], G.cam[2]};
    V3 target = depth_to_world(G.inverse_proj, G.inverse_view, u, v, 1.0f);
    V3 dir = normalize(target - cam);
    ClosestHit h;
    const float inf = __int_as_float(0x7f800000);
    bool hit = trace_ray<true, false, AlphaTest>(T, cam, dir, 0.0f, inf, 0xFFu, G.model_skip, G.model_count, &h,
                                                 err, nullptr,
                                                 AlphaTest{G.models, G.model_count, G.textures, G.texture_count, G.shade},
                                                 list + 1, cnt == kGbListAll ? -1 : (int)cnt);
    if (err) atomicOr(G.status, err);
    if (!hit) {
        G.albedo[pix] = 0u;
        G.normal[pix] = make_float4(0.f, 0.f, 0.f, 0.f);
        G.material[pix] = 0u;
        G.emission[pix] = 0u;
        G.depth[pix] = 1.0f;
        G.primary_hit[pix] = make_uint2(0xFFFFFFFFu, 0xFFFFFFFFu);
        G.hit_instance[pix] = 0xFFFFFFFFu;
        return;
    }

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
    G.albedo[pix] = pack_unorm8(color[0], color[1], color[2], color[3]);
    G.normal[pix] = make_float4(N.x, N.y, N.z, 1.0f);
    G.material[pix] = pack_unorm8(roughness, metallic, occlusion, 1.0f);
    G.emission[pix] = pack_unorm8(em[0], em[1], em[2], em[3]);
    G.depth[pix] = depth;
    G.primary_hit[pix] = make_uint2(h.custom, h.prim);
    G.hit_instance[pix] = h.inst_input;
}

// ---------------------------------------------------------------- lit-pixel compaction
// A pixel is lit when length(N) != 0 (light.frag:178). The list follows a tiled
// order of the image — kLitTile x kLitTile pixel tiles in row order, pixels in row
// order inside a tile — so the 32 rays a warp takes at once (32 neighbouring items of
// one light) start from a compact patch of pixels rather than a 32-pixel row.
// Chunks of 1024 positions of that order.
constexpr int kChunk = 1024;
constexpr uint32_t kLitTile = 4;   // measured at 1080p: 4x4 3.85 ms, 8x8 3.88, 16x16 3.94, rows 4.24

// Pixel at position o of the tiled order, or ~0u past the image.
__device__ __forceinline__ uint32_t tiled_pixel(uint32_t o, uint32_t width, uint32_t height) {
    const uint32_t tiles_x = (width + kLitTile - 1) / kLitTile;
    const uint32_t tile = o / (kLitTile * kLitTile), w = o % (kLitTile * kLitTile);
    const uint32_t x = (tile % tiles_x) * kLitTile + w % kLitTile, y = (tile / tiles_x) * kLitTile + w / kLitTile;
    return (x < width && y < height) ? y * width + x : ~0u;
}

__device__ __forceinline__ bool pixel_lit(const float4* normal, uint32_t pix) {
    if (pix == ~0u) return false;
    float4 v = normal[pix];
    return !(length(V3{v.x, v.y, v.z}) == 0.0f);
}

__global__ void __launch_bounds__(256) lit_count_kernel(const float4* normal, uint32_t width, uint32_t height,
                                                        uint32_t* chunk_counts) {
    __shared__ uint32_t s_tmp[8];
    uint32_t base = blockIdx.x * kChunk + threadIdx.x * 4;
    uint32_t c = 0;
    for (int k = 0; k < 4; ++k) c += pixel_lit(normal, tiled_pixel(base + k, width, height));
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

// Also writes light.frag's background colour (light.frag:178-181: ambient colour x
// intensity, alpha 1) into the light plane at every unlit pixel, so the light pass
// touches lit pixels only, and packs each lit pixel's albedo, material and emission
// words beside it, so that the light pass reads its G-buffer inputs as 16-B records in
// list order.
__global__ void __launch_bounds__(256) lit_write_kernel(const float4* normal, const float* depth,
                                                        const uint32_t* albedo, const uint32_t* material,
                                                        const uint32_t* emission,
                                                        uint32_t width, uint32_t height,
                                                        const uint32_t* chunk_offsets,
                                                        const float* inverse_proj,
                                                        const float* inverse_view, const float* ambient,
                                                        float4* surf, uint4* surf_mat, float4* light) {
    __shared__ uint32_t s_tmp[8];
    __shared__ float s_ip[16], s_iv[16];
    __shared__ float4 s_bg;
    if (threadIdx.x < 16) { s_ip[threadIdx.x] = inverse_proj[threadIdx.x]; s_iv[threadIdx.x] = inverse_view[threadIdx.x]; }
    if (threadIdx.x == 0) {
        // ambient = (ambientLightColor, ambientLightIntensity), the first 16 B of the scene block
        const V3 c = V3{ambient[0], ambient[1], ambient[2]} * ambient[3];
        s_bg = make_float4(c.x, c.y, c.z, 1.0f);
    }
    __syncthreads();
    uint32_t base = blockIdx.x * kChunk + threadIdx.x * 4;
    bool lit[4];
    uint32_t px[4];
    uint32_t c = 0;
    for (int k = 0; k < 4; ++k) {
        px[k] = tiled_pixel(base + k, width, height);
        lit[k] = pixel_lit(normal, px[k]);
        c += lit[k];
    }
    uint32_t pos = chunk_offsets[blockIdx.x] + block_excl(c, s_tmp);
    for (int k = 0; k < 4; ++k) {
        if (!lit[k]) {
            if (px[k] != ~0u) light[px[k]] = s_bg;
            continue;
        }
        uint32_t pix = px[k];
        uint32_t x = pix % width, y = pix / width;
        V3 p = depth_to_world(s_ip, s_iv, pixel_uv(x, width), pixel_uv(y, height), depth[pix]);
        float4 nn = normal[pix];
        surf[2 * (size_t)pos] = make_float4(p.x, p.y, p.z, __uint_as_float(pix));
        surf[2 * (size_t)pos + 1] = make_float4(nn.x, nn.y, nn.z, __uint_as_float(x | (y << 16)));
        surf_mat[pos] = make_uint4(albedo[pix], material[pix], emission[pix], pix);
        ++pos;
    }
}

// ---------------------------------------------------------------- host launchers
luz_status launch_lit_compaction(luz_ctx* ctx, luz_frame* f);

// Inputs of the G-buffer pass of frame f over TLAS t.
luz_status make_gbuf_params(luz_ctx* ctx, luz_frame* f, const luz_tlas* t, GbufParams& G) {
    // 4-wide nodes; node_count (the binary count) bounds the 4-wide count and the
    // nodes4 buffer, so staging that many stays inside it.
    G.tlas_nodes = t->nodes4;
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
    G.hit_instance = f->hit_instance;
    G.status = ctx->d_status;
    G.textures = f->d_textures;
    G.texture_count = f->texture_count;
    if (f->max_map_index >= (int32_t)f->texture_count)
        return set_error(ctx, LUZ_ERR_INVALID, "a ModelBlock map index is beyond the frame's textures");
    return LUZ_OK;
}

luz_status launch_gbuffer(luz_ctx* ctx, luz_frame* f, const luz_tlas* t) {
    GbufParams G;
    luz_status st = make_gbuf_params(ctx, f, t, G);
    if (st != LUZ_OK) return st;
    uint32_t tiles = ((f->width + kGbTile - 1) / kGbTile) * ((f->height + kGbTile - 1) / kGbTile);
    const uint32_t coarse = ((f->width + kGbCoarse - 1) / kGbCoarse) * ((f->height + kGbCoarse - 1) / kGbCoarse);
    prof_begin(ctx, LUZ_KERNEL_GBUFFER);
    if (t->count > kGbListMaxInstances) {   // every tile through the TLAS (count word kGbListAll)
        LUZ_CUDA(ctx, cudaMemsetAsync(f->gb_fine, 0xFF, (size_t)tiles * (kGbFineMax + 1) * 4, ctx->stream));
    } else if (t->count > 0) {
        const float4* leaf_box = tlas_leaf_boxes(t);
        gb_coarse_kernel<<<coarse, 256, 0, ctx->stream>>>(G, leaf_box, t->count, f->gb_coarse);
        LUZ_LAUNCHED(ctx, "gb_coarse_kernel");
        gb_fine_kernel<<<coarse, 64, 0, ctx->stream>>>(G, leaf_box, f->gb_coarse, f->gb_fine);
        LUZ_LAUNCHED(ctx, "gb_fine_kernel");
    } else {
        LUZ_CUDA(ctx, cudaMemsetAsync(f->gb_fine, 0, (size_t)tiles * (kGbFineMax + 1) * 4, ctx->stream));
    }
    gbuffer_kernel<<<tiles, kGbTile * kGbTile, 0, ctx->stream>>>(G, f->gb_fine);
    prof_end(ctx);
    LUZ_LAUNCHED(ctx, "gbuffer_kernel");
    return launch_lit_compaction(ctx, f);
}

// Compaction of the lit pixels (length(N) != 0) of the normal plane into the
// (fragPos, pixel), (N, x | y << 16) list that ray generation and the light pass read.
uint32_t lit_chunks(uint32_t width, uint32_t height) {
    const uint64_t positions = (uint64_t)((width + kLitTile - 1) / kLitTile) * ((height + kLitTile - 1) / kLitTile) *
                               kLitTile * kLitTile;
    return (uint32_t)((positions + kChunk - 1) / kChunk);
}

luz_status launch_lit_compaction(luz_ctx* ctx, luz_frame* f) {
    uint32_t chunks = lit_chunks(f->width, f->height);
    lit_count_kernel<<<chunks, 256, 0, ctx->stream>>>(f->normal, f->width, f->height, f->block_counts);
    LUZ_LAUNCHED(ctx, "lit_count_kernel");
    lit_scan_kernel<<<1, 1024, 0, ctx->stream>>>(f->block_counts, chunks, f->lit_count);
    LUZ_LAUNCHED(ctx, "lit_scan_kernel");
    lit_write_kernel<<<chunks, 256, 0, ctx->stream>>>(f->normal, f->depth, f->albedo, f->material, f->emission,
                                                      f->width, f->height,
                                                      f->block_counts,
                                                      (const float*)((const char*)f->d_scene + offsetof(luz_scene, inverse_proj)),
                                                      (const float*)((const char*)f->d_scene + offsetof(luz_scene, inverse_view)),
                                                      (const float*)((const char*)f->d_scene + offsetof(luz_scene, ambient_light_color)),
                                                      f->surf, f->surf_mat, f->light);
    LUZ_LAUNCHED(ctx, "lit_write_kernel");
    f->surf_valid = true;
    return LUZ_OK;
}

// Rebuilds the lit-pixel list when the planes or scene constants it came from were
// replaced since the last G-buffer pass (luz_frame_write, luz_frame_upload).
luz_status ensure_lit_list(luz_ctx* ctx, luz_frame* f) {
    return f->surf_valid ? LUZ_OK : launch_lit_compaction(ctx, f);
}

}  // namespace luz
