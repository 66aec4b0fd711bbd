// batch.cu — many independent scenes of uneven size rendered as one unit. The frame
// kernel (batch_frame_kernel) runs a whole frame of every scene in ONE persistent
// launch: the per-frame TLAS builds, the clearing of the hit/miss planes, the G-buffer
// tiles with their lit-pixel compaction, the shadow/AO traversal of all scenes' rays and
// the light passes, ordered by tickets from a few counters and per-scene flags, every
// wait bounded. Recordable as one CUDA graph (a memset of the counters and the kernel)
// and replayed with a single launch; a launch-shape autotuner. The staged form (every
// TLAS build, G-buffer and light pass its own launch around one visibility launch)
// remains for scenes the frame kernel does not take. (No counterpart in the reference,
// which renders one scene per frame.)
#include <algorithm>
#include <cstddef>
#include <cstring>
#include <vector>

#include "gbuffer.cuh"
#include "lbvh_device.cuh"
#include "lightpass.cuh"
#include "vis_trace.cuh"

namespace luz {
luz_status pack_tlas_input(luz_ctx* ctx, luz_tlas* t, const luz_instance* inst, uint32_t n);
luz_status launch_tlas_build(luz_ctx* ctx, luz_tlas* t);
luz_status launch_gbuffer(luz_ctx* ctx, luz_frame* f, const luz_tlas* t);
luz_status launch_light_pass(luz_ctx* ctx, luz_frame* f, int mode);
luz_status make_gbuf_params(luz_ctx* ctx, luz_frame* f, const luz_tlas* t, GbufParams& G);
LightParams make_light_params(luz_ctx* ctx, luz_frame* f);
TlasBuildArgs tlas_build_args(luz_tlas* t);

// ---------------------------------------------------------------- frame kernel
constexpr uint32_t kFrameTile = 16;                   // G-buffer item: 16x16 pixels, one per thread
constexpr uint32_t kClearWords = 16384;               // clear item: 64 KB of a hit/miss plane
constexpr uint32_t kFrameWaitIters = 1u << 22;        // polls (128 ns apart) before a wait gives up
constexpr size_t kFrameSmem = kStackBytes + kColdBytes;   // traversal stacks + cold ray state
constexpr uint32_t kFrameMaxLights = (uint32_t)(kFrameSmem / sizeof(luz_light));
static_assert(kVisThreads == kFrameTile * kFrameTile, "a G-buffer item is one pixel per thread");
static_assert(kFrameSmem >= kFusedTlasMax * sizeof(unsigned long long), "TLAS sort keys fit the shared memory");

// Per-scene inputs of the frame kernel.
struct FrameScene {
    TlasBuildArgs tlas;      // n = 0: no instances
    GbufParams gb;
    LightParams lp;          // plain light pass
    uint32_t* lit_count;
    float4* surf;            // compacted lit pixels (fragPos, pixel), (N, x | y << 16)
    uint4* surf_mat;         // beside them: (albedo, material, emission, pixel)
    float ambient[4];        // ambientLightColor, ambientLightIntensity
    uint32_t tiles_x;        // 16x16 G-buffer tiles per row
};

struct ClearItem {
    uint32_t* p;             // 16-B aligned
    uint32_t words;
};

// Counters of one frame (zeroed before every launch), followed by one "TLAS built"
// flag per scene.
struct FrameCtl {
    uint32_t ticket;                 // prologue tickets handed out (TLAS, clear, G-buffer)
    uint32_t prologue_done;          // prologue items finished
    uint32_t ready;                  // ray offsets published
    uint32_t light_ticket;           // light-pass tickets handed out
    unsigned long long rays;         // ray items handed out
    unsigned long long resolved;     // ray items finished
    unsigned long long total_rays;
    uint32_t light_items;
    uint32_t abort;                  // a wait gave up: every later wait gives up at once
};

struct FrameArgs {
    const FrameScene* fs;
    const SceneVis* vis;
    const uint32_t* tile_off;        // [scenes + 1] G-buffer items before scene s
    const ClearItem* clears;
    FrameCtl* ctl;
    uint32_t* tlas_done;             // [scenes]
    unsigned long long* offsets;     // [scenes + 1] ray items before scene s (published)
    uint32_t* light_off;             // [scenes + 1] light-pass items before scene s (published)
    uint32_t scenes, clear_items, prologue_items;
    VisCommon C;
    unsigned long long* stats;
};

__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_u32(uint32_t* p, uint32_t v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Polls until *p >= target; false when the wait gave up (LUZ_DEV_BATCH_QUEUE) or an
// earlier wait of the launch did (abort), so that one failure does not make every
// later wait run to its limit.
__device__ __noinline__ bool wait_u32(const uint32_t* p, uint32_t target, uint32_t* abort) {
    for (uint32_t i = 0; i < kFrameWaitIters; ++i) {
        if (ld_acquire_u32(p) >= target) return true;
        if (ld_acquire_u32(abort)) return false;
        __nanosleep(128);
    }
    atomicExch(abort, 1u);
    return false;
}
__device__ __noinline__ bool wait_u64(const unsigned long long* p, unsigned long long target, uint32_t* abort) {
    for (uint32_t i = 0; i < kFrameWaitIters; ++i) {
        if (ld_acquire_u64(p) >= target) return true;
        if (ld_acquire_u32(abort)) return false;
        __nanosleep(128);
    }
    atomicExch(abort, 1u);
    return false;
}

// Largest s < n with off[s] <= x (off ascending, off[0] = 0).
template <typename T>
__device__ __forceinline__ uint32_t find_item(const T* off, uint32_t n, T x) {
    uint32_t lo = 0, hi = n - 1;
    while (lo < hi) {
        uint32_t mid = (lo + hi + 1) >> 1;
        if (off[mid] <= x) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Run by one thread once every prologue item has finished: the ray and light-pass
// item offsets of every scene from its lit-pixel count, then the release of `ready`
// (not after a failed wait: every scene's TLAS and G-buffer must be complete).
__device__ __noinline__ void publish_offsets(const FrameArgs& A) {
    __threadfence();
    if (ld_acquire_u32(&A.ctl->abort)) return;   // a wait gave up: the waiters of `ready` give up too
    unsigned long long acc = 0;
    uint32_t lacc = 0;
    for (uint32_t s = 0; s < A.scenes; ++s) {
        A.offsets[s] = acc;
        A.light_off[s] = lacc;
        const uint32_t lit = ld_acquire_u32(A.fs[s].lit_count);
        acc += (unsigned long long)lit * (A.vis[s].shadow_slots + A.vis[s].ao_samples);
        lacc += (lit + kVisThreads - 1) / kVisThreads;
    }
    A.offsets[A.scenes] = acc;
    A.light_off[A.scenes] = lacc;
    A.ctl->total_rays = acc;
    A.ctl->light_items = lacc;
    __threadfence();
    st_release_u32(&A.ctl->ready, 1u);
}

// The G-buffer item g of scene F: a 16x16-pixel tile, thread t at pixel t % 16 of 4x4
// sub-tile t / 16 (sub-tiles in row order), so that the lit pixels it appends to the
// scene's list keep the 4x4-patch order the traversal's warps like. Writes every
// G-buffer plane, the background colour of light.frag:178-181 at the unlit pixels, and
// appends the lit pixels (length(N) != 0, light.frag:178) with their DepthToWorld
// position (light.frag:186) and G-buffer words to the list; the list's order between tiles is the order
// the tiles finish, and no output depends on it.
__device__ __noinline__ void frame_gbuffer_item(const FrameScene& F, uint32_t k, uint32_t* s_tmp,
                                                uint32_t* s_base) {
    const uint32_t tid = threadIdx.x;
    const uint32_t tx = k % F.tiles_x, ty = k / F.tiles_x;
    const uint32_t sub = tid >> 4, w = tid & 15u;
    const uint32_t x = tx * kFrameTile + (sub & 3u) * 4u + (w & 3u);
    const uint32_t y = ty * kFrameTile + (sub >> 2) * 4u + (w >> 2);
    const uint32_t width = F.gb.width, height = F.gb.height;
    const bool inside = x < width && y < height;
    GbufPixel gp{make_float4(0.f, 0.f, 0.f, 1.f), 0u, 0u, 0u};
    if (inside) {
        GbufRay ray;
        if (gbuffer_trace<const GbufParams&>(F.gb, x, y, ray)) gp = gbuffer_shade<const GbufParams&>(F.gb, x, y, ray);
    }
    const float4 nd = gp.nd;
    const bool lit = inside && !(length(V3{nd.x, nd.y, nd.z}) == 0.0f);
    const uint32_t rank = block_excl(lit ? 1u : 0u, s_tmp);
    if (tid == 0) {
        uint32_t total = 0;
        for (int q = 0; q < kVisThreads / 32; ++q) total += s_tmp[q];
        *s_base = total ? atomicAdd(F.lit_count, total) : 0u;
    }
    __syncthreads();
    if (!inside) return;
    const uint32_t pix = y * width + x;
    if (lit) {
        const uint32_t pos = *s_base + rank;
        const V3 p = depth_to_world(F.gb.inverse_proj, F.gb.inverse_view, pixel_uv(x, width), pixel_uv(y, height),
                                    nd.w);
        F.surf[2 * (size_t)pos] = make_float4(p.x, p.y, p.z, __uint_as_float(pix));
        F.surf[2 * (size_t)pos + 1] = make_float4(nd.x, nd.y, nd.z, __uint_as_float(x | (y << 16)));
        F.surf_mat[pos] = make_uint4(gp.albedo, gp.material, gp.emission, pix);
    } else {
        const V3 c = V3{F.ambient[0], F.ambient[1], F.ambient[2]} * F.ambient[3];
        F.lp.out[pix] = make_float4(c.x, c.y, c.z, 1.0f);
    }
}

// The TLAS build item of scene F (its own call: the build's registers stay out of the
// traversal loop's allocation).
__device__ __noinline__ void frame_tlas_item(const FrameScene& F, unsigned long long* s_keys, uint32_t* s_bounds,
                                             uint32_t* status) {
    if (threadIdx.x == 0) *F.lit_count = 0u;
    if (F.tlas.n > 0) tlas_build_block<const TlasBuildArgs&>(F.tlas, s_keys, s_bounds, status);
}

// Light-pass item: lit pixels [c * 256, c * 256 + 256) of scene F, lights staged in
// shared memory.
__device__ __noinline__ void frame_light_item(const FrameScene& F, uint32_t c, luz_light* s_lights) {
    for (uint32_t i = threadIdx.x; i < F.lp.light_count; i += kVisThreads) s_lights[i] = F.lp.lights[i];
    __syncthreads();
    const uint32_t t = c * kVisThreads + threadIdx.x;
    if (t < ld_acquire_u32(F.lit_count)) light_pass_pixel<kPlain, true>(F.lp, s_lights, t);
}

// Phase 2 of the frame kernel for one warp: lanes refill from the counter over the
// rays of all scenes (item g of scene s with offsets[s] <= g < offsets[s+1]), each
// lane carrying its scene's TLAS and outputs; the items the warp took are added to
// `resolved` when it leaves.
template <bool kStats>
__device__ __forceinline__ void frame_trace(const FrameArgs& A, unsigned long long total, float4* smem,
                                         uint32_t& err) {
    const uint32_t tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    uint32_t* s_stack = reinterpret_cast<uint32_t*>(smem) + warp * (kSmemStack * 32) + lane;
    const Cold c{reinterpret_cast<float*>(reinterpret_cast<uint32_t*>(smem) + kVisThreads * kSmemStack) + tid};
    int lstack[kLocalStack];
    const uint32_t full = 0xFFFFFFFFu, lt_mask = (1u << lane) - 1u;
    uint32_t rays = 0;
    uint32_t taken = 0;   // items this warp took (a warp takes far fewer than 2^32)
    TraceCounters cnt{0, 0, 0, 0};
    LaneRay r{};
    bool active = false, exhausted = false;
    for (;;) {
        uint32_t idle = __ballot_sync(full, !active);
        if (!exhausted && __popc(idle) >= (int)A.C.refill) {
            int leader = __ffs(idle) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(&A.ctl->rays, (unsigned long long)__popc(idle));
            base = __shfl_sync(full, base, leader);
            if (base + __popc(idle) >= total) exhausted = true;
            if (base < total) taken += (uint32_t)min(total - base, (unsigned long long)__popc(idle));
            if (!active) {
                const unsigned long long item = base + __popc(idle & lt_mask);
                if (item < total) {
                    const uint32_t s = find_item<unsigned long long>(A.offsets, A.scenes, item);
                    const SceneVis& S = A.vis[s];
                    const uint32_t lit = *S.lit_count;   // final since `ready`
                    const unsigned long long local = item - A.offsets[s];
                    const uint32_t slot = (uint32_t)(local / lit);
                    const uint32_t j = (uint32_t)(local - (unsigned long long)slot * lit);
                    active = setup_ray<true>(r, c, S, A.C, slot, j);
                    if (kStats && active) ++rays;
                }
            }
        }
        if (exhausted && __ballot_sync(full, active) == 0) break;
        run_steps<kStats, false>(r, c, active, nullptr, 0u, r.tlas, r.insts, s_stack, lstack, A.C.steps,
                                 A.C.step_cap, err, cnt);
    }
    // every lane's bit-plane writes are ordered before the warp's count of resolved items
    __threadfence();
    __syncwarp();
    if (lane == 0 && taken) atomicAdd(&A.ctl->resolved, (unsigned long long)taken);
    if (kStats) flush_stats(A.stats, rays, cnt);
}

// One frame of every scene. Phases, each fed by tickets so that an item only waits on
// items handed out before it (every wait ends, whichever CTAs are resident):
//   1. prologue, one item per CTA at a time: the TLAS build of each scene (tickets
//      0..S-1; a scene's lit count is zeroed there), the clearing of the hit/miss
//      planes in 64-KB items, then the G-buffer tiles (each waits for its scene's
//      TLAS). The CTA that finishes the last prologue item publishes the ray offsets.
//   2. traversal: after `ready`, the warps of every CTA refill their lanes from one
//      counter over the rays of all scenes (visibility_batch_kernel's loop); a warp
//      that leaves the loop adds the items it took to `resolved`.
//   3. light passes: 256 lit pixels per item, after every ray item is resolved.
template <bool kStats>
__global__ void __launch_bounds__(kVisThreads, LUZ_VIS_MIN_BLOCKS) batch_frame_kernel(FrameArgs A) {
    extern __shared__ float4 smem[];
    __shared__ uint32_t s_item, s_base, s_ok, s_tmp[kVisThreads / 32], s_bounds[6];
    __shared__ unsigned long long s_total;
    __shared__ uint32_t s_light_items;
    const uint32_t tid = threadIdx.x;
    uint32_t err = 0;

    // ---- 1. prologue
    for (;;) {
        if (tid == 0) s_item = atomicAdd(&A.ctl->ticket, 1u);
        __syncthreads();
        const uint32_t item = s_item;
        if (item >= A.prologue_items) break;
        if (item < A.scenes) {
            frame_tlas_item(A.fs[item], reinterpret_cast<unsigned long long*>(smem), s_bounds, A.C.status);
            __syncthreads();
            if (tid == 0) {
                __threadfence();
                st_release_u32(A.tlas_done + item, 1u);
            }
        } else if (item < A.scenes + A.clear_items) {
            const ClearItem c = A.clears[item - A.scenes];
            // 16-B stores where the item is 16-B aligned (plane bases and 64-KB steps are)
            const uint32_t n4 = (reinterpret_cast<uintptr_t>(c.p) & 15u) ? 0u : c.words >> 2;
            uint4* p4 = reinterpret_cast<uint4*>(c.p);
            for (uint32_t i = tid; i < n4; i += kVisThreads) p4[i] = make_uint4(0u, 0u, 0u, 0u);
            for (uint32_t i = (n4 << 2) + tid; i < c.words; i += kVisThreads) c.p[i] = 0u;
        } else {
            const uint32_t g = item - A.scenes - A.clear_items;
            const uint32_t s = find_item<uint32_t>(A.tile_off, A.scenes, g);
            if (tid == 0) s_ok = wait_u32(A.tlas_done + s, 1u, &A.ctl->abort);
            __syncthreads();
            if (s_ok) frame_gbuffer_item(A.fs[s], g - A.tile_off[s], s_tmp, &s_base);
            else err |= LUZ_DEV_BATCH_QUEUE;   // no trace through a TLAS that may not be built
        }
        __syncthreads();
        if (tid == 0) {
            __threadfence();
            if (atomicAdd(&A.ctl->prologue_done, 1u) + 1u == A.prologue_items) publish_offsets(A);
        }
    }

    // ---- 2. traversal
    if (tid == 0) {
        s_ok = wait_u32(&A.ctl->ready, 1u, &A.ctl->abort);
        s_total = ld_acquire_u64(&A.ctl->total_rays);
        s_light_items = ld_acquire_u32(&A.ctl->light_items);
    }
    __syncthreads();
    if (!s_ok) {
        if (tid == 0) atomicOr(A.C.status, (uint32_t)LUZ_DEV_BATCH_QUEUE);
        return;
    }
    frame_trace<kStats>(A, s_total, smem, err);

    // ---- 3. light passes
    __syncthreads();
    luz_light* s_lights = reinterpret_cast<luz_light*>(smem);
    bool resolved = false;
    for (;;) {
        if (tid == 0) {
            s_item = atomicAdd(&A.ctl->light_ticket, 1u);
            s_ok = 1u;
            if (s_item < s_light_items && !resolved) {
                s_ok = wait_u64(&A.ctl->resolved, s_total, &A.ctl->abort);
                resolved = true;
            }
        }
        __syncthreads();
        const uint32_t item = s_item;
        if (item >= s_light_items) break;
        if (!s_ok) {
            err |= LUZ_DEV_BATCH_QUEUE;
            break;
        }
        const uint32_t s = find_item<uint32_t>(A.light_off, A.scenes, item);
        frame_light_item(A.fs[s], item - A.light_off[s], s_lights);
        __syncthreads();
    }
    if (err) atomicOr(A.C.status, err);
}

}  // namespace luz

struct luz_batch {
    luz_ctx* ctx = nullptr;
    std::vector<luz_tlas*> tlas;
    std::vector<luz_frame*> frames;
    std::vector<luz::SceneVis> h_scenes;
    luz::SceneVis* d_scenes = nullptr;
    unsigned long long* d_offsets = nullptr;
    unsigned long long* d_work = nullptr;
    unsigned long long* d_stats = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int frame_index = 0;
    // frame kernel
    bool fusable = false;            // every scene fits the frame kernel
    bool fused = false;              // renders run the frame kernel
    luz::FrameScene* d_fs = nullptr;
    uint32_t* d_tile_off = nullptr;
    luz::ClearItem* d_clears = nullptr;
    void* d_ctl = nullptr;           // FrameCtl + one flag per scene
    size_t ctl_bytes = 0;
    uint32_t* d_light_off = nullptr;
    uint32_t clear_items = 0, tile_items = 0;
};

namespace luz {

static luz_status set_frame_index(luz_ctx* ctx, luz_batch* b, int frame_index) {
    // The sampler frame index lives in the per-scene records (fixed inside a graph).
    if (frame_index != b->frame_index) {
        for (auto& s : b->h_scenes) s.frame = frame_index;
        LUZ_CUDA(ctx, cudaMemcpyAsync(b->d_scenes, b->h_scenes.data(), b->h_scenes.size() * sizeof(SceneVis),
                                      cudaMemcpyHostToDevice, ctx->stream));
        b->frame_index = frame_index;
    }
    return LUZ_OK;
}

// The frame kernel of the batch: the counters cleared, then one persistent launch.
static luz_status launch_frame(luz_ctx* ctx, luz_batch* b, bool stats) {
    cudaStream_t st = ctx->stream;
    LUZ_CUDA(ctx, cudaMemsetAsync(b->d_ctl, 0, b->ctl_bytes, st));
    if (stats) LUZ_CUDA(ctx, cudaMemsetAsync(b->d_stats, 0, 5 * sizeof(unsigned long long), st));
    FrameCtl* ctl = reinterpret_cast<FrameCtl*>(b->d_ctl);
    FrameArgs A;
    A.fs = b->d_fs;
    A.vis = b->d_scenes;
    A.tile_off = b->d_tile_off;
    A.clears = b->d_clears;
    A.ctl = ctl;
    A.tlas_done = reinterpret_cast<uint32_t*>(ctl + 1);
    A.offsets = b->d_offsets;
    A.light_off = b->d_light_off;
    A.scenes = (uint32_t)b->frames.size();
    A.clear_items = b->clear_items;
    A.prologue_items = A.scenes + b->clear_items + b->tile_items;
    A.C = make_vis_common(ctx, &ctl->rays);
    A.stats = stats ? b->d_stats : nullptr;
    const uint32_t grid = (uint32_t)ctx->sm_count * vis_tuning(ctx).ctas_per_sm;
    prof_begin(ctx, LUZ_KERNEL_BATCH_FRAME);
    if (stats) batch_frame_kernel<true><<<grid, kVisThreads, kFrameSmem, st>>>(A);
    else batch_frame_kernel<false><<<grid, kVisThreads, kFrameSmem, st>>>(A);
    prof_end(ctx);
    LUZ_LAUNCHED(ctx, stats ? "batch_frame_kernel<stats>" : "batch_frame_kernel");
    for (auto* f : b->frames) f->surf_valid = true;
    return LUZ_OK;
}

static luz_status batch_record(luz_ctx* ctx, luz_batch* b, int frame_index, bool stats) {
    luz_status s = set_frame_index(ctx, b, frame_index);
    if (s != LUZ_OK) return s;
    if (b->fused) return launch_frame(ctx, b, stats);
    for (size_t i = 0; i < b->frames.size(); ++i) {
        if ((s = launch_tlas_build(ctx, b->tlas[i])) != LUZ_OK) return s;
        if ((s = launch_gbuffer(ctx, b->frames[i], b->tlas[i])) != LUZ_OK) return s;
        if ((s = clear_visibility(ctx, b->frames[i])) != LUZ_OK) return s;
    }
    if ((s = launch_visibility_batch(ctx, b->d_scenes, (uint32_t)b->frames.size(), b->d_offsets, b->d_work,
                                     stats ? b->d_stats : nullptr)) != LUZ_OK)
        return s;
    for (auto* f : b->frames)
        if ((s = launch_light_pass(ctx, f, 0)) != LUZ_OK) return s;
    return LUZ_OK;
}

// Device tables of the frame kernel; leaves b->fusable false when a scene does not fit
// (more than kFusedTlasMax instances or kFrameMaxLights lights).
static luz_status setup_frame_kernel(luz_ctx* ctx, luz_batch* b) {
    const uint32_t n = (uint32_t)b->frames.size();
    for (uint32_t i = 0; i < n; ++i)
        if (b->tlas[i]->count > kFusedTlasMax || b->frames[i]->light_count > kFrameMaxLights) return LUZ_OK;
    std::vector<FrameScene> fs(n);
    std::vector<uint32_t> tile_off(n + 1, 0);
    std::vector<ClearItem> clears;
    for (uint32_t i = 0; i < n; ++i) {
        luz_frame* f = b->frames[i];
        FrameScene& F = fs[i];
        F.tlas = tlas_build_args(b->tlas[i]);
        luz_status s = make_gbuf_params(ctx, f, b->tlas[i], F.gb);
        if (s != LUZ_OK) return s;
        F.lp = make_light_params(ctx, f);
        F.lit_count = f->lit_count;
        F.surf = f->surf;
        F.surf_mat = f->surf_mat;
        memcpy(F.ambient, f->h_scene.ambient_light_color, 12);
        F.ambient[3] = f->h_scene.ambient_light_intensity;
        F.tiles_x = (f->width + kFrameTile - 1) / kFrameTile;
        const uint32_t tiles = F.tiles_x * ((f->height + kFrameTile - 1) / kFrameTile);
        tile_off[i + 1] = tile_off[i] + tiles;
        uint32_t* planes[2] = {f->shadow_bits, f->ao_bits};
        const uint64_t words[2] = {(uint64_t)f->shadow_slots * f->words, (uint64_t)f->ao_samples * f->words};
        for (int k = 0; k < 2; ++k)
            for (uint64_t w0 = 0; w0 < words[k]; w0 += kClearWords)
                clears.push_back(ClearItem{planes[k] + w0, (uint32_t)std::min<uint64_t>(kClearWords, words[k] - w0)});
    }
    b->clear_items = (uint32_t)clears.size();
    b->tile_items = tile_off[n];
    b->ctl_bytes = sizeof(FrameCtl) + (size_t)n * 4;
    cudaError_t e = cudaMalloc(&b->d_fs, n * sizeof(FrameScene));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_tile_off, (n + 1) * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_clears, std::max<size_t>(clears.size(), 1) * sizeof(ClearItem));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_ctl, b->ctl_bytes);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_light_off, (n + 1) * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemcpy(b->d_fs, fs.data(), n * sizeof(FrameScene), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(b->d_tile_off, tile_off.data(), (n + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !clears.empty())
        e = cudaMemcpy(b->d_clears, clears.data(), clears.size() * sizeof(ClearItem), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_error(ctx, e, "batch frame-kernel tables");
    b->fusable = true;
    b->fused = true;
    return LUZ_OK;
}

static void drop_graph(luz_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
}

}  // namespace luz

using namespace luz;

extern "C" {

static luz_status batch_create_body(luz_ctx* ctx, uint32_t count, const luz_batch_scene* scenes, luz_batch** out) {
    if (!ctx || !scenes || !out || count == 0) return LUZ_ERR_INVALID;
    luz_batch* b = new luz_batch();
    b->ctx = ctx;
    auto fail = [&](luz_status s) { luz_batch_destroy(b); return s; };
    for (uint32_t i = 0; i < count; ++i) {
        const luz_batch_scene& d = scenes[i];
        luz_tlas* t = nullptr;
        luz_frame* f = nullptr;
        luz_status s = luz_tlas_create(ctx, std::max(d.instance_count, 1u), &t);
        if (s != LUZ_OK) return fail(s);
        b->tlas.push_back(t);
        if ((s = luz_frame_create(ctx, d.width, d.height, &f)) != LUZ_OK) return fail(s);
        b->frames.push_back(f);
        if ((s = luz_frame_upload(ctx, f, d.scene, d.lights, d.light_count, d.models, d.model_count)) != LUZ_OK)
            return fail(s);
        // Instances are packed once into the TLAS's pinned staging buffer; every render
        // (and the graph) copies them from there.
        if ((s = pack_tlas_input(ctx, t, d.instances, d.instance_count)) != LUZ_OK) return fail(s);
        // The frame kernel rebuilds the TLAS from the device copy of the instances.
        if (t->count)
            LUZ_CUDA(ctx, cudaMemcpy(t->d_input, t->h_input, (size_t)t->count * sizeof(DevInstanceInput),
                                     cudaMemcpyHostToDevice));
        b->h_scenes.push_back(make_scene_vis(f, t, 0));
    }
    cudaError_t e = cudaMalloc(&b->d_scenes, count * sizeof(SceneVis));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_offsets, (count + 1) * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_work, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_stats, 5 * sizeof(unsigned long long));
    if (e == cudaSuccess)
        e = cudaMemcpy(b->d_scenes, b->h_scenes.data(), count * sizeof(SceneVis), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail(cuda_error(ctx, e, "batch allocation"));
    luz_status fs = setup_frame_kernel(ctx, b);
    if (fs != LUZ_OK) return fail(fs);
    *out = b;
    return LUZ_OK;
}

luz_status luz_batch_create(luz_ctx* ctx, uint32_t count, const luz_batch_scene* scenes, luz_batch** out) {
    return guarded(ctx, [&] { return batch_create_body(ctx, count, scenes, out); });
}

void luz_batch_destroy(luz_batch* b) {
    if (!b) return;
    cudaDeviceSynchronize();
    drop_graph(b);
    for (auto* f : b->frames) luz_frame_destroy(f);
    for (auto* t : b->tlas) luz_tlas_destroy(t);
    void* p[] = {b->d_scenes, b->d_offsets, b->d_work, b->d_stats, b->d_fs, b->d_tile_off, b->d_clears, b->d_ctl,
                 b->d_light_off};
    for (void* x : p)
        if (x) cudaFree(x);
    delete b;
}

uint32_t luz_batch_count(const luz_batch* b) { return b ? (uint32_t)b->frames.size() : 0; }

luz_frame* luz_batch_frame(luz_batch* b, uint32_t i) {
    return (b && i < b->frames.size()) ? b->frames[i] : nullptr;
}

luz_status luz_batch_render(luz_ctx* ctx, luz_batch* b, int32_t frame_index) {
    if (!ctx || !b) return LUZ_ERR_INVALID;
    return batch_record(ctx, b, frame_index, false);
}

luz_status luz_batch_stats(luz_ctx* ctx, luz_batch* b, int32_t frame_index, uint64_t out[5]) {
    if (!ctx || !b || !out) return LUZ_ERR_INVALID;
    luz_status s = batch_record(ctx, b, frame_index, true);
    if (s != LUZ_OK) return s;
    LUZ_CUDA(ctx, cudaMemcpyAsync(out, b->d_stats, 5 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                  ctx->stream));
    LUZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return LUZ_OK;
}

luz_status luz_batch_capture(luz_ctx* ctx, luz_batch* b, int32_t frame_index) {
    if (!ctx || !b) return LUZ_ERR_INVALID;
    if (ctx->stream == nullptr)
        return set_error(ctx, LUZ_ERR_INVALID, "capture needs an explicit stream");
    LUZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    drop_graph(b);
    // The frame index is written before capture: the records are then constant.
    if (frame_index != b->frame_index) {
        for (auto& s : b->h_scenes) s.frame = frame_index;
        LUZ_CUDA(ctx, cudaMemcpy(b->d_scenes, b->h_scenes.data(), b->h_scenes.size() * sizeof(SceneVis),
                                 cudaMemcpyHostToDevice));
        b->frame_index = frame_index;
    }
    LUZ_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    luz_status s = batch_record(ctx, b, frame_index, false);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    if (s != LUZ_OK) {
        if (g) cudaGraphDestroy(g);
        return s;
    }
    if (e != cudaSuccess) return cuda_error(ctx, e, "cudaStreamEndCapture");
    b->graph = g;
    e = cudaGraphInstantiate(&b->exec, g, 0);
    if (e != cudaSuccess) { drop_graph(b); return cuda_error(ctx, e, "cudaGraphInstantiate"); }
    return LUZ_OK;
}

luz_status luz_batch_replay(luz_ctx* ctx, luz_batch* b) {
    if (!ctx || !b || !b->exec) return set_error(ctx, LUZ_ERR_INVALID, "no captured graph");
    LUZ_CUDA(ctx, cudaGraphLaunch(b->exec, ctx->stream));
    ctx->launches++;
    return LUZ_OK;
}

// Times the visibility launch of the batch (with the frame kernel: the whole frame
// launch) for each candidate shape and keeps the fastest (median of `reps` launches). Candidates: refill {8,16,32} x steps
// {16,32,64} x CTAs per SM {2,3,4}. Drops a captured graph (its shape is stale).
luz_status luz_batch_autotune(luz_ctx* ctx, luz_batch* b, uint32_t reps, luz_vis_tuning* chosen, float* best_ms) {
    if (!ctx || !b) return LUZ_ERR_INVALID;
    reps = std::max(reps, 1u);
    drop_graph(b);
    luz_status s = batch_record(ctx, b, b->frame_index, false);   // G-buffers and lit counts in place
    if (s != LUZ_OK) return s;
    cudaEvent_t e0, e1;
    LUZ_CUDA(ctx, cudaEventCreate(&e0));
    LUZ_CUDA(ctx, cudaEventCreate(&e1));
    const uint32_t refills[] = {8, 16, 32}, steps[] = {16, 32, 64}, ctas[] = {2, 3, 4};
    const uint32_t base_smem = vis_tuning(ctx).smem_nodes;
    VisTuning best{0, 0, 0, 0, 0};
    float best_t = 3.0e38f;
    for (uint32_t rf : refills)
        for (uint32_t sp : steps)
            for (uint32_t ct : ctas) {
                ctx->vis_tuning = VisTuning{0, rf, sp, ct, 1};
                std::vector<float> ts;
                for (uint32_t r = 0; r <= reps; ++r) {
                    if (!b->fused)
                        for (auto* f : b->frames)
                            if ((s = clear_visibility(ctx, f)) != LUZ_OK) return s;
                    cudaEventRecord(e0, ctx->stream);
                    if (b->fused)
                        s = launch_frame(ctx, b, false);
                    else
                        s = launch_visibility_batch(ctx, b->d_scenes, (uint32_t)b->frames.size(), b->d_offsets,
                                                    b->d_work, nullptr);
                    if (s != LUZ_OK) return s;
                    cudaEventRecord(e1, ctx->stream);
                    LUZ_CUDA(ctx, cudaEventSynchronize(e1));
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, e0, e1);
                    if (r) ts.push_back(ms);   // the first launch warms up
                }
                std::sort(ts.begin(), ts.end());
                float med = ts[ts.size() / 2];
                if (med < best_t) { best_t = med; best = ctx->vis_tuning; }
            }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    // the single-scene TLAS staging size keeps its current value
    best.smem_nodes = base_smem;
    ctx->vis_tuning = best;
    if (chosen) *chosen = luz_vis_tuning{best.smem_nodes, best.refill, best.steps, best.ctas_per_sm};
    if (best_ms) *best_ms = best_t;
    uint32_t bits = 0;
    LUZ_CUDA(ctx, cudaMemcpy(&bits, ctx->d_status, 4, cudaMemcpyDeviceToHost));
    return bits ? set_error(ctx, LUZ_ERR_DEVICE, "device status word raised while tuning") : LUZ_OK;
}

luz_status luz_batch_set_fused(luz_ctx* ctx, luz_batch* b, int32_t on) {
    if (!ctx || !b) return LUZ_ERR_INVALID;
    if (on && !b->fusable)
        return set_error(ctx, LUZ_ERR_LIMIT, "a scene of the batch does not fit the frame kernel");
    if ((on != 0) != b->fused) drop_graph(b);
    b->fused = on != 0;
    return LUZ_OK;
}

int32_t luz_batch_fused(const luz_batch* b) { return b && b->fused ? 1 : 0; }

}  // extern "C"
