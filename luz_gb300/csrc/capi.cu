// capi.cu — the extern "C" entry points of include/luz.h: context, BLAS/TLAS
// handles, frames, uploads and read-back.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "internal.cuh"

namespace luz {
luz_status build_blas_batch(luz_ctx* ctx, uint32_t count, const luz_blas_desc* descs, luz_blas** out);
luz_status tlas_alloc(luz_ctx* ctx, luz_tlas* t);
luz_status build_tlas(luz_ctx* ctx, luz_tlas* t, const luz_instance* inst, uint32_t n);
luz_status launch_gbuffer(luz_ctx* ctx, luz_frame* f, const luz_tlas* t);
luz_status launch_visibility(luz_ctx* ctx, luz_frame* f, const luz_tlas* t, int frame_index,
                             unsigned long long* d_stats);
luz_status frame_lit_count(luz_ctx* ctx, luz_frame* f, uint32_t* count);
luz_status launch_light_pass(luz_ctx* ctx, luz_frame* f, int mode);
uint32_t lit_chunks(uint32_t width, uint32_t height);
luz_status launch_ao_resolve(luz_ctx* ctx, luz_frame* f);

// The process's live contexts: all on one device (per-device setup is cached per
// process), and a new setup generation when the first of them is created.
static std::mutex g_ctx_mutex;
static int g_ctx_live = 0;
static int g_ctx_device = -1;
static std::atomic<uint64_t> g_setup_generation{0};

uint64_t setup_generation() { return g_setup_generation.load(std::memory_order_acquire); }

luz_status set_error(luz_ctx* ctx, luz_status st, const std::string& msg) {
    if (ctx) ctx->last_error = msg;
    return st;
}
luz_status cuda_error(luz_ctx* ctx, cudaError_t e, const char* what) {
    std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    luz_status st = LUZ_ERR_CUDA;
    if (e == cudaErrorMemoryAllocation) st = LUZ_ERR_OOM;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) st = LUZ_ERR_NO_DEVICE;
    return set_error(ctx, st, m);
}
luz_status check_launch(luz_ctx* ctx, const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error(ctx, e, what);
    return LUZ_OK;
}
void prof_begin(luz_ctx* ctx, int32_t kernel) {
    if (!ctx->prof_on) return;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(ctx->stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return;
    while (ctx->prof_pool.size() < ctx->prof_used + 2) {
        cudaEvent_t e = nullptr;
        if (cudaEventCreate(&e) != cudaSuccess) return;
        ctx->prof_pool.push_back(e);
    }
    luz_ctx::ProfRec r{kernel, ctx->prof_pool[ctx->prof_used], nullptr};   // b: set by prof_end
    ctx->prof_used += 2;
    cudaEventRecord(r.a, ctx->stream);
    ctx->prof_recs.push_back(r);
}

void prof_end(luz_ctx* ctx) {
    if (!ctx->prof_on || ctx->prof_recs.empty() || ctx->prof_recs.back().b) return;
    cudaEvent_t b = ctx->prof_pool[ctx->prof_used - 1];
    cudaEventRecord(b, ctx->stream);
    ctx->prof_recs.back().b = b;
}

luz_status ensure_scratch(luz_ctx* ctx, size_t bytes) {
    if (bytes <= ctx->scratch_bytes) return LUZ_OK;
    if (ctx->d_scratch) {
        LUZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        cudaFree(ctx->d_scratch);
        ctx->d_scratch = nullptr;
        ctx->scratch_bytes = 0;
    }
    size_t b = std::max(bytes, (size_t)1 << 20);
    LUZ_CUDA(ctx, cudaMalloc(&ctx->d_scratch, b));
    ctx->scratch_bytes = b;
    return LUZ_OK;
}

static void free_frame_buffers(luz_frame* f) {
    void* ptrs[] = {f->albedo, f->normal, f->material, f->emission, f->depth, f->light,
                    f->primary_hit, f->hit_instance, f->gb_coarse, f->gb_fine, f->shadow_bits, f->ao_bits, f->ao, f->ao_denoised, f->signal,
                    f->unshadowed, f->denoised, f->surf, f->surf_mat,
                    f->features, f->lin_depth, f->taa, f->taa_next, f->compose, f->hist, f->hist_state,
                    f->block_counts, f->lit_count, f->dn_list, f->dn_count, f->d_scene, f->d_lights, f->d_models,
                    f->d_slot_table, f->d_light_slot, f->d_model_skip, f->work_counter, f->d_textures,
                    f->d_texels, f->d_shadow_lights, f->d_shadow_maps, f->rays_a, f->rays_b, f->rays_c, f->beams,
                    f->beam_lists};
    for (void* p : ptrs)
        if (p) cudaFree(p);
}

// (Re)allocates *p for at least `need` elements when `cap` is short; cap is updated.
static luz_status grow(luz_ctx* ctx, void** p, uint32_t& cap, uint32_t need, size_t elem) {
    if (need <= cap && *p) return LUZ_OK;
    uint32_t n = std::max(need, std::max(cap * 2, 16u));
    if (*p) {
        LUZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        cudaFree(*p);
        *p = nullptr;
    }
    LUZ_CUDA(ctx, cudaMalloc(p, (size_t)n * elem));
    cap = n;
    return LUZ_OK;
}

}  // namespace luz

using namespace luz;

extern "C" {

luz_status luz_ctx_create(int device, luz_ctx** out) {
    if (!out) return LUZ_ERR_INVALID;
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) return LUZ_ERR_NO_DEVICE;
    if (device < 0 || device >= n) return LUZ_ERR_INVALID;
    {
        std::lock_guard<std::mutex> lock(g_ctx_mutex);
        if (g_ctx_live > 0 && device != g_ctx_device) return LUZ_ERR_INVALID;   // one device per process
        if (g_ctx_live == 0) {
            g_ctx_device = device;
            g_setup_generation.fetch_add(1, std::memory_order_acq_rel);
        }
        ++g_ctx_live;
    }
    luz_ctx* ctx = new luz_ctx();
    ctx->device = device;
    ctx->registered = true;
    auto fail = [&](luz_status s) { luz_ctx_destroy(ctx); return s; };
    if (cudaSetDevice(device) != cudaSuccess) return fail(LUZ_ERR_CUDA);
    if (cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking) != cudaSuccess)
        return fail(LUZ_ERR_CUDA);
    ctx->stream = ctx->own_stream;
    cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (cudaMalloc(&ctx->d_status, 4) != cudaSuccess) return fail(LUZ_ERR_OOM);
    for (auto& ev : ctx->build_ev)
        if (cudaEventCreate(&ev) != cudaSuccess) return fail(LUZ_ERR_CUDA);
    cudaMemset(ctx->d_status, 0, 4);
    float lut[256];
    for (int i = 0; i < 256; ++i) lut[i] = (float)std::pow((double)((float)i / 255.0f), 2.2);
    if (cudaMalloc(&ctx->d_srgb_lut, sizeof(lut)) != cudaSuccess) return fail(LUZ_ERR_OOM);
    if (cudaMemcpy(ctx->d_srgb_lut, lut, sizeof(lut), cudaMemcpyHostToDevice) != cudaSuccess)
        return fail(LUZ_ERR_CUDA);
    // Default substitute blue noise: a flat mid-grey texel (callers upload the seeded one).
    uint8_t grey[4] = {128, 128, 128, 255};
    if (luz_ctx_set_blue_noise(ctx, grey, 1) != LUZ_OK) return fail(LUZ_ERR_CUDA);
    *out = ctx;
    return LUZ_OK;
}

void luz_ctx_destroy(luz_ctx* ctx) {
    if (!ctx) return;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->d_status) cudaFree(ctx->d_status);
    if (ctx->d_blue_noise) cudaFree(ctx->d_blue_noise);
    if (ctx->d_srgb_lut) cudaFree(ctx->d_srgb_lut);
    if (ctx->d_scratch) cudaFree(ctx->d_scratch);
    if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    for (auto ev : ctx->build_ev)
        if (ev) cudaEventDestroy(ev);
    for (auto ev : ctx->prof_pool) cudaEventDestroy(ev);
    if (ctx->registered) {
        std::lock_guard<std::mutex> lock(g_ctx_mutex);
        --g_ctx_live;
    }
    delete ctx;
}

luz_status luz_ctx_last_blas_build_ms(luz_ctx* ctx, float* device_ms) {
    if (!ctx || !device_ms) return LUZ_ERR_INVALID;
    if (!ctx->build_timed) return set_error(ctx, LUZ_ERR_INVALID, "no BLAS build on this context yet");
    LUZ_CUDA(ctx, cudaEventSynchronize(ctx->build_ev[1]));
    LUZ_CUDA(ctx, cudaEventElapsedTime(device_ms, ctx->build_ev[0], ctx->build_ev[1]));
    return LUZ_OK;
}

luz_status luz_ctx_profile(luz_ctx* ctx, int32_t on) {
    if (!ctx) return LUZ_ERR_INVALID;
    if (on) {
        LUZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));   // the pool's events are free again
        ctx->prof_recs.clear();
        ctx->prof_used = 0;
    }
    ctx->prof_on = on != 0;
    return LUZ_OK;
}

luz_status luz_ctx_profile_read(luz_ctx* ctx, int32_t kernel, float* total_ms, uint32_t* launches) {
    if (!ctx || !total_ms || !launches) return LUZ_ERR_INVALID;
    LUZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    double sum = 0.0;
    uint32_t n = 0;
    for (const auto& r : ctx->prof_recs) {
        if (r.kernel != kernel || !r.b) continue;
        float ms = 0.f;
        LUZ_CUDA(ctx, cudaEventElapsedTime(&ms, r.a, r.b));
        sum += ms;
        ++n;
    }
    *total_ms = (float)sum;
    *launches = n;
    return LUZ_OK;
}

namespace {
// Streams `words` 16-B words of a buffer `reps` times through L2 (ld.global.cg: cached
// in L2 only, so L1 serves none of it); one XOR per block keeps the loads live.
__global__ void __launch_bounds__(512) l2_read_probe_kernel(const uint4* __restrict__ buf, size_t words,
                                                            uint32_t reps, uint32_t* sink) {
    uint32_t x = 0;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (uint32_t r = 0; r < reps; ++r)
        for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < words; i += stride) {
            const uint4 v = __ldcg(buf + i);
            x ^= v.x ^ v.y ^ v.z ^ v.w;
        }
    x = __reduce_xor_sync(0xFFFFFFFFu, x);
    if ((threadIdx.x & 31) == 0 && x == 0x9E3779B9u) atomicXor(sink, x);   // practically never taken
}
}  // namespace

luz_status luz_ctx_probe_l2_read(luz_ctx* ctx, uint64_t bytes, uint32_t reps, float* gbs) {
    if (!ctx || !gbs || bytes < (1u << 20) || reps == 0) return LUZ_ERR_INVALID;
    const size_t words = (size_t)(bytes / 16);
    void* buf = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto run = [&]() -> luz_status {
        LUZ_CUDA(ctx, cudaMalloc(&buf, words * 16 + 256));
        LUZ_CUDA(ctx, cudaMemsetAsync(buf, 0x5A, words * 16 + 256, ctx->stream));
        LUZ_CUDA(ctx, cudaEventCreate(&e0));
        LUZ_CUDA(ctx, cudaEventCreate(&e1));
        uint32_t* sink = (uint32_t*)((char*)buf + words * 16);
        const uint32_t grid = (uint32_t)ctx->sm_count * 4;
        l2_read_probe_kernel<<<grid, 512, 0, ctx->stream>>>((const uint4*)buf, words, 2, sink);   // warm L2
        LUZ_LAUNCHED(ctx, "l2_read_probe_kernel");
        LUZ_CUDA(ctx, cudaEventRecord(e0, ctx->stream));
        l2_read_probe_kernel<<<grid, 512, 0, ctx->stream>>>((const uint4*)buf, words, reps, sink);
        LUZ_LAUNCHED(ctx, "l2_read_probe_kernel");
        LUZ_CUDA(ctx, cudaEventRecord(e1, ctx->stream));
        LUZ_CUDA(ctx, cudaEventSynchronize(e1));
        float ms = 0.f;
        LUZ_CUDA(ctx, cudaEventElapsedTime(&ms, e0, e1));
        *gbs = (float)((double)words * 16.0 * reps / (ms * 1e-3) / 1e9);
        return LUZ_OK;
    };
    const luz_status st = run();
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (buf) {
        cudaStreamSynchronize(ctx->stream);
        cudaFree(buf);
    }
    return st;
}

const char* luz_last_error(const luz_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

luz_status luz_ctx_synchronize(luz_ctx* ctx) {
    if (!ctx) return LUZ_ERR_INVALID;
    LUZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    uint32_t bits = 0;
    LUZ_CUDA(ctx, cudaMemcpy(&bits, ctx->d_status, 4, cudaMemcpyDeviceToHost));
    if (bits) {
        char msg[96];
        snprintf(msg, sizeof(msg), "a kernel raised the device status word (LUZ_DEV_* bits 0x%x)", bits);
        return set_error(ctx, LUZ_ERR_DEVICE, msg);
    }
    return LUZ_OK;
}

luz_status luz_ctx_set_debug_step_cap(luz_ctx* ctx, uint32_t steps) {
    if (!ctx) return LUZ_ERR_INVALID;
    ctx->debug_step_cap = steps;
    return LUZ_OK;
}

luz_status luz_ctx_device_status(luz_ctx* ctx, uint32_t* bits) {
    if (!ctx || !bits) return LUZ_ERR_INVALID;
    LUZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    LUZ_CUDA(ctx, cudaMemcpy(bits, ctx->d_status, 4, cudaMemcpyDeviceToHost));
    LUZ_CUDA(ctx, cudaMemset(ctx->d_status, 0, 4));
    return LUZ_OK;
}

uint64_t luz_ctx_launch_count(const luz_ctx* ctx) { return ctx ? ctx->launches : 0; }

luz_status luz_ctx_set_stream(luz_ctx* ctx, void* stream) {
    if (!ctx) return LUZ_ERR_INVALID;
    LUZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
    return LUZ_OK;
}

luz_status luz_ctx_set_blue_noise(luz_ctx* ctx, const uint8_t* rgba8, uint32_t size) {
    if (!ctx || !rgba8 || size == 0 || size > 4096) return LUZ_ERR_INVALID;
    if (ctx->d_blue_noise) {
        LUZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        cudaFree(ctx->d_blue_noise);
        ctx->d_blue_noise = nullptr;
    }
    LUZ_CUDA(ctx, cudaMalloc(&ctx->d_blue_noise, (size_t)size * size * 4));
    LUZ_CUDA(ctx, cudaMemcpy(ctx->d_blue_noise, rgba8, (size_t)size * size * 4, cudaMemcpyHostToDevice));
    ctx->blue_noise_size = size;
    return LUZ_OK;
}

// ------------------------------------------------------------------ BLAS
luz_status luz_blas_build(luz_ctx* ctx, const luz_blas_desc* desc, luz_blas** out) {
    if (!ctx || !desc || !out) return LUZ_ERR_INVALID;
    return guarded(ctx, [&] { return build_blas_batch(ctx, 1, desc, out); });
}

luz_status luz_blas_build_batch(luz_ctx* ctx, uint32_t count, const luz_blas_desc* descs, luz_blas** out) {
    if (!ctx || !descs || !out || count == 0) return LUZ_ERR_INVALID;
    if (count > (1u << 18)) return set_error(ctx, LUZ_ERR_LIMIT, "more than 2^18 BLAS in one batch");
    return guarded(ctx, [&] { return build_blas_batch(ctx, count, descs, out); });
}

void luz_blas_destroy(luz_blas* b) {
    if (!b) return;
    if (b->arena && --b->arena->refs == 0) {
        cudaDeviceSynchronize();   // the handle may outlive its context: do not touch it
        cudaFree(b->arena->base);
        delete b->arena;
    }
    delete b;
}

uint32_t luz_blas_primitive_count(const luz_blas* b) { return b ? b->prims : 0; }

luz_status luz_blas_memory(const luz_blas* b, luz_memory* out) {
    if (!b || !out) return LUZ_ERR_INVALID;
    *out = b->memory;
    return LUZ_OK;
}

luz_status luz_blas_download_wide(luz_ctx* ctx, const luz_blas* b, void* nodes4) {
    if (!ctx || !b || !nodes4) return LUZ_ERR_INVALID;
    if (!b->nodes4) return set_error(ctx, LUZ_ERR_INVALID, "BLAS has no 4-wide nodes");
    LUZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    uint32_t m = std::max(b->prims, 2u) - 1;
    LUZ_CUDA(ctx, cudaMemcpy(nodes4, b->nodes4, (size_t)m * 128, cudaMemcpyDeviceToHost));
    return LUZ_OK;
}

luz_status luz_blas_download(luz_ctx* ctx, const luz_blas* b, void* nodes, void* tris,
                             uint32_t* morton_sorted, uint32_t* order) {
    if (!ctx || !b) return LUZ_ERR_INVALID;
    LUZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    uint32_t n = b->prims, m = std::max(n, 2u) - 1;
    if (nodes) LUZ_CUDA(ctx, cudaMemcpy(nodes, b->nodes, (size_t)m * 64, cudaMemcpyDeviceToHost));
    if (tris && n) LUZ_CUDA(ctx, cudaMemcpy(tris, b->tris, (size_t)n * 48, cudaMemcpyDeviceToHost));
    if (morton_sorted && n) LUZ_CUDA(ctx, cudaMemcpy(morton_sorted, b->morton, (size_t)n * 4, cudaMemcpyDeviceToHost));
    if (order && n) LUZ_CUDA(ctx, cudaMemcpy(order, b->order, (size_t)n * 4, cudaMemcpyDeviceToHost));
    return LUZ_OK;
}

// ------------------------------------------------------------------ TLAS
luz_status luz_tlas_create(luz_ctx* ctx, uint32_t max_instances, luz_tlas** out) {
    if (!ctx || !out || max_instances == 0) return LUZ_ERR_INVALID;
    if (max_instances > (1u << 24)) return set_error(ctx, LUZ_ERR_LIMIT, "max_instances above 2^24");
    luz_tlas* t = new luz_tlas();
    t->ctx = ctx;
    t->max_instances = max_instances;
    luz_status s = tlas_alloc(ctx, t);
    if (s == LUZ_OK && cudaEventCreateWithFlags(&t->input_copied, cudaEventDisableTiming) != cudaSuccess)
        s = set_error(ctx, LUZ_ERR_CUDA, "cudaEventCreate");
    if (s != LUZ_OK) { luz_tlas_destroy(t); return s; }
    *out = t;
    return LUZ_OK;
}

luz_status luz_tlas_build(luz_ctx* ctx, luz_tlas* t, const luz_instance* inst, uint32_t count) {
    if (!ctx || !t || (count && !inst)) return LUZ_ERR_INVALID;
    // The pinned staging buffer may still be read by the previous build's copy.
    LUZ_CUDA(ctx, cudaEventSynchronize(t->input_copied));
    luz_status s = build_tlas(ctx, t, inst, count);
    if (s != LUZ_OK) return s;
    t->node_count = std::max(count, 2u) - 1;
    LUZ_CUDA(ctx, cudaEventRecord(t->input_copied, ctx->stream));
    return LUZ_OK;
}

void luz_tlas_destroy(luz_tlas* t) {
    if (!t) return;
    cudaDeviceSynchronize();   // the handle may outlive its context: do not touch it
    if (t->nodes) cudaFree(t->nodes);
    if (t->nodes4) cudaFree(t->nodes4);
    if (t->levels) cudaFree(t->levels);
    if (t->instances) cudaFree(t->instances);
    if (t->shade) cudaFree(t->shade);
    if (t->d_input) cudaFree(t->d_input);
    if (t->h_input) cudaFreeHost(t->h_input);
    if (t->morton) cudaFree(t->morton);
    if (t->order) cudaFree(t->order);
    if (t->near) cudaFree(t->near);
    if (t->leaf_of) cudaFree(t->leaf_of);
    if (t->tmp) cudaFree(t->tmp);
    if (t->input_copied) cudaEventDestroy(t->input_copied);
    delete t;
}

luz_status luz_tlas_download(luz_ctx* ctx, const luz_tlas* t, void* nodes, uint32_t* morton_sorted,
                             uint32_t* order, uint32_t* node_count) {
    if (!ctx || !t) return LUZ_ERR_INVALID;
    LUZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    uint32_t n = t->count, m = n ? std::max(n, 2u) - 1 : 0;
    if (node_count) *node_count = m;
    if (nodes && m) LUZ_CUDA(ctx, cudaMemcpy(nodes, t->nodes, (size_t)m * 64, cudaMemcpyDeviceToHost));
    if (morton_sorted && n) LUZ_CUDA(ctx, cudaMemcpy(morton_sorted, t->morton, (size_t)n * 4, cudaMemcpyDeviceToHost));
    if (order && n) LUZ_CUDA(ctx, cudaMemcpy(order, t->order, (size_t)n * 4, cudaMemcpyDeviceToHost));
    return LUZ_OK;
}

luz_status luz_tlas_download_wide(luz_ctx* ctx, const luz_tlas* t, void* nodes4) {
    if (!ctx || !t || !nodes4) return LUZ_ERR_INVALID;
    LUZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    uint32_t n = t->count, m = n ? std::max(n, 2u) - 1 : 0;
    if (m) LUZ_CUDA(ctx, cudaMemcpy(nodes4, t->nodes4, (size_t)m * 128, cudaMemcpyDeviceToHost));
    return LUZ_OK;
}

luz_status luz_tlas_memory(const luz_tlas* t, luz_memory* out) {
    if (!t || !out) return LUZ_ERR_INVALID;
    uint64_t cap = std::max(t->max_instances, 1u), m = std::max<uint64_t>(cap, 2) - 1;
    out->nodes = m * 64;
    out->wide_nodes = m * 128;
    out->leaves = cap * sizeof(DevInstance);
    // level table; per instance: shading record, input record, Morton code and order,
    // near list (4 x uint4) and leaf index; build scratch
    out->other = 66 * 4 + cap * (sizeof(DevShadeInstance) + sizeof(DevInstanceInput) + 8 + 4 * sizeof(uint4) + 4) +
                 t->tmp_bytes;
    return LUZ_OK;
}

// ------------------------------------------------------------------ frame
luz_status luz_frame_create(luz_ctx* ctx, uint32_t width, uint32_t height, luz_frame** out) {
    if (!ctx || !out || width == 0 || height == 0) return LUZ_ERR_INVALID;
    if ((uint64_t)width * height > (1ull << 27))
        return set_error(ctx, LUZ_ERR_LIMIT, "frame larger than 2^27 pixels");
    if (width > 65535 || height > 65535)   // lit-pixel records carry x | y << 16
        return set_error(ctx, LUZ_ERR_LIMIT, "frame wider or taller than 65535 pixels");
    luz_frame* f = new luz_frame();
    f->ctx = ctx;
    f->width = width;
    f->height = height;
    f->pixels = width * height;
    f->words = (f->pixels + 31) / 32;
    size_t P = f->pixels;
    uint32_t chunks = lit_chunks(width, height);
    cudaError_t e = cudaSuccess;
    auto A = [&](void** p, size_t bytes) { if (e == cudaSuccess) e = cudaMalloc(p, std::max(bytes, (size_t)16)); };
    A((void**)&f->albedo, P * 4);
    A((void**)&f->normal, P * 16);
    A((void**)&f->material, P * 4);
    A((void**)&f->emission, P * 4);
    A((void**)&f->depth, P * 4);
    A((void**)&f->light, P * 16);
    A((void**)&f->primary_hit, P * 8);
    A((void**)&f->hit_instance, P * 4);
    A((void**)&f->gb_coarse, (size_t)((width + 63) / 64) * ((height + 63) / 64) * 256 * 4);
    A((void**)&f->gb_fine, (size_t)((width + 7) / 8) * ((height + 7) / 8) * 16 * 4);
    A((void**)&f->ao, P * 4);
    A((void**)&f->ao_denoised, P * 4);
    A((void**)&f->signal, P * 16);
    A((void**)&f->unshadowed, P * 16);
    A((void**)&f->denoised, P * 16);
    A((void**)&f->features, P * 16);
    A((void**)&f->lin_depth, P * 4);
    A((void**)&f->dn_list, P * 4);
    A((void**)&f->dn_count, 4);
    A((void**)&f->taa, P * 16);
    A((void**)&f->taa_next, P * 16);
    A((void**)&f->compose, P * 4);
    A((void**)&f->hist, (256 + 260) * 4);
    A((void**)&f->hist_state, 16);
    A((void**)&f->surf, P * 32);
    A((void**)&f->surf_mat, P * 16);
    A((void**)&f->block_counts, (size_t)chunks * 4);
    A((void**)&f->lit_count, 4);
    A((void**)&f->d_scene, sizeof(luz_scene));
    A((void**)&f->work_counter, 8);
    if (e != cudaSuccess) {
        free_frame_buffers(f);
        delete f;
        return cuda_error(ctx, e, "cudaMalloc(frame)");
    }
    cudaMemset(f->ao_denoised, 0, P * 4);
    cudaMemset(f->signal, 0, P * 16);
    cudaMemset(f->unshadowed, 0, P * 16);
    cudaMemset(f->denoised, 0, P * 16);
    cudaMemset(f->taa, 0, P * 16);
    cudaMemset(f->compose, 0, P * 4);
    cudaMemset(f->hist_state, 0, 16);
    *out = f;
    return LUZ_OK;
}

void luz_frame_destroy(luz_frame* f) {
    if (!f) return;
    cudaDeviceSynchronize();   // the handle may outlive its context: do not touch it
    free_frame_buffers(f);
    delete f;
}

static luz_status frame_upload_body(luz_ctx* ctx, luz_frame* f, const luz_scene* scene, const luz_light* lights,
                                    uint32_t light_count, const luz_model* models, uint32_t model_count) {
    if (!ctx || !f || !scene || (light_count && !lights) || (model_count && !models))
        return LUZ_ERR_INVALID;
    if (scene->ao_num_samples < 0 || scene->ao_num_samples > LUZ_MAX_AO_SAMPLES)
        return set_error(ctx, LUZ_ERR_LIMIT, "ao_num_samples outside [0, LUZ_MAX_AO_SAMPLES]");
    // aoMin is the AO rays' tMin (light.frag:125-126); a ray query's tMin must not be
    // negative (the editor clamps it to [0, 10], Editor.cpp:329).
    if (scene->ao_min < 0.0f) return set_error(ctx, LUZ_ERR_INVALID, "ao_min is negative (a ray query's tMin)");
    if (light_count > 65535) return set_error(ctx, LUZ_ERR_LIMIT, "more than 65535 lights");
    // Shadow slots: Σ numShadowSamples (GPUScene.cpp:248), one bit plane each.
    std::vector<uint32_t> slot_table, light_slot(std::max(light_count, 1u));
    for (uint32_t l = 0; l < light_count; ++l) {
        light_slot[l] = (uint32_t)slot_table.size();
        int ns = scene->shadow_type == LUZ_SHADOW_RAYTRACING ? lights[l].num_shadow_samples : 0;
        if (ns < 0) ns = 0;
        if (slot_table.size() + ns > LUZ_MAX_SHADOW_SLOTS)
            return set_error(ctx, LUZ_ERR_LIMIT, "more than LUZ_MAX_SHADOW_SLOTS shadow samples per pixel");
        for (int s = 0; s < ns; ++s) slot_table.push_back(l | ((uint32_t)s << 16));
    }
    cudaStream_t st = ctx->stream;
    uint32_t shadow_slots = (uint32_t)slot_table.size();
    uint32_t ao = (uint32_t)scene->ao_num_samples;
    uint32_t cap_shadow = f->shadow_planes_cap, cap_ao = f->ao_planes_cap;
    luz_status s;
    if ((s = grow(ctx, (void**)&f->shadow_bits, cap_shadow, std::max(shadow_slots, 1u), (size_t)f->words * 4)) != LUZ_OK) return s;
    if ((s = grow(ctx, (void**)&f->ao_bits, cap_ao, std::max(ao, 1u), (size_t)f->words * 4)) != LUZ_OK) return s;
    f->shadow_planes_cap = cap_shadow;
    f->ao_planes_cap = cap_ao;
    static_assert(sizeof(luz_light) == 64, "luz_light layout");
    static_assert(sizeof(luz_model) == 128, "luz_model layout");
    static_assert(sizeof(luz_vertex) == 48, "luz_vertex layout");
    if (light_count > f->lights_cap || !f->d_lights) {
        uint32_t cap = 0, cap2 = 0;
        if ((s = grow(ctx, (void**)&f->d_lights, cap, std::max(light_count, 1u), sizeof(luz_light))) != LUZ_OK) return s;
        if ((s = grow(ctx, (void**)&f->d_light_slot, cap2, cap, 4)) != LUZ_OK) return s;
        f->lights_cap = cap;
    }
    if (model_count > f->models_cap || !f->d_models) {
        uint32_t cap = 0, cap2 = 0;
        if ((s = grow(ctx, (void**)&f->d_models, cap, std::max(model_count, 1u), sizeof(luz_model))) != LUZ_OK) return s;
        if ((s = grow(ctx, (void**)&f->d_model_skip, cap2, cap, 1)) != LUZ_OK) return s;
        f->models_cap = cap;
    }
    if (!f->d_slot_table) LUZ_CUDA(ctx, cudaMalloc(&f->d_slot_table, (size_t)LUZ_MAX_SHADOW_SLOTS * 4));
    f->h_slot_table = slot_table;
    std::vector<uint8_t> skip(std::max(model_count, 1u), 0);
    int32_t max_map = -1;
    for (uint32_t m = 0; m < model_count; ++m) {
        const luz_model& md = models[m];
        skip[m] = md.color_map >= 0 ? 2 : (md.color[3] < 0.5f ? 1 : 0);
        for (int32_t t : {md.ao_map, md.color_map, md.normal_map, md.emission_map, md.metallic_roughness_map})
            max_map = std::max(max_map, t);
    }
    f->max_map_index = max_map;
    f->h_scene = *scene;
    f->surf_valid = false;   // the lit list's positions come from this scene's matrices
    f->light_count = light_count;
    f->model_count = model_count;
    f->shadow_slots = shadow_slots;
    f->ao_samples = ao;
    LUZ_CUDA(ctx, cudaMemcpyAsync(f->d_scene, scene, sizeof(luz_scene), cudaMemcpyHostToDevice, st));
    if (light_count) {
        LUZ_CUDA(ctx, cudaMemcpyAsync(f->d_lights, lights, (size_t)light_count * sizeof(luz_light), cudaMemcpyHostToDevice, st));
        LUZ_CUDA(ctx, cudaMemcpyAsync(f->d_light_slot, light_slot.data(), (size_t)light_count * 4, cudaMemcpyHostToDevice, st));
    }
    if (shadow_slots)
        LUZ_CUDA(ctx, cudaMemcpyAsync(f->d_slot_table, slot_table.data(), (size_t)shadow_slots * 4, cudaMemcpyHostToDevice, st));
    if (model_count) {
        LUZ_CUDA(ctx, cudaMemcpyAsync(f->d_models, models, (size_t)model_count * sizeof(luz_model), cudaMemcpyHostToDevice, st));
        LUZ_CUDA(ctx, cudaMemcpyAsync(f->d_model_skip, skip.data(), model_count, cudaMemcpyHostToDevice, st));
    }
    // Pageable sources: the copies above are staged before returning; the vectors
    // may go out of scope once the stream has consumed them.
    LUZ_CUDA(ctx, cudaStreamSynchronize(st));
    return LUZ_OK;
}

luz_status luz_frame_upload(luz_ctx* ctx, luz_frame* f, const luz_scene* scene, const luz_light* lights,
                            uint32_t light_count, const luz_model* models, uint32_t model_count) {
    return guarded(ctx, [&] { return frame_upload_body(ctx, f, scene, lights, light_count, models, model_count); });
}

static luz_status frame_set_textures_body(luz_ctx* ctx, luz_frame* f, const luz_texture_desc* tex, uint32_t count) {
    if (!ctx || !f || (count && !tex)) return LUZ_ERR_INVALID;
    size_t total = 0;
    std::vector<size_t> off(count);
    for (uint32_t k = 0; k < count; ++k) {
        if (!tex[k].rgba8 || tex[k].width == 0 || tex[k].height == 0 || tex[k].width > 65536 || tex[k].height > 65536)
            return set_error(ctx, LUZ_ERR_INVALID, "texture " + std::to_string(k) + ": empty or larger than 65536");
        off[k] = total;
        total += ((size_t)tex[k].width * tex[k].height * 4 + 255) & ~(size_t)255;
    }
    LUZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (f->d_textures) { cudaFree(f->d_textures); f->d_textures = nullptr; }
    if (f->d_texels) { cudaFree(f->d_texels); f->d_texels = nullptr; }
    f->texture_count = 0;
    if (!count) return LUZ_OK;
    LUZ_CUDA(ctx, cudaMalloc(&f->d_texels, total));
    LUZ_CUDA(ctx, cudaMalloc(&f->d_textures, (size_t)count * sizeof(DevTexture)));
    std::vector<DevTexture> table(count);
    for (uint32_t k = 0; k < count; ++k) {
        table[k].texels = (const uint32_t*)((char*)f->d_texels + off[k]);
        table[k].width = tex[k].width;
        table[k].height = tex[k].height;
        LUZ_CUDA(ctx, cudaMemcpy((char*)f->d_texels + off[k], tex[k].rgba8, (size_t)tex[k].width * tex[k].height * 4,
                                 cudaMemcpyHostToDevice));
    }
    LUZ_CUDA(ctx, cudaMemcpy(f->d_textures, table.data(), (size_t)count * sizeof(DevTexture), cudaMemcpyHostToDevice));
    f->texture_count = count;
    return LUZ_OK;
}

luz_status luz_frame_set_textures(luz_ctx* ctx, luz_frame* f, const luz_texture_desc* tex, uint32_t count) {
    return guarded(ctx, [&] { return frame_set_textures_body(ctx, f, tex, count); });
}

luz_status luz_gbuffer_primary(luz_ctx* ctx, luz_frame* f, const luz_tlas* t) {
    if (!ctx || !f || !t) return LUZ_ERR_INVALID;
    return launch_gbuffer(ctx, f, t);
}

luz_status luz_trace_visibility(luz_ctx* ctx, luz_frame* f, const luz_tlas* t, int32_t frame_index) {
    if (!ctx || !f || !t) return LUZ_ERR_INVALID;
    return launch_visibility(ctx, f, t, frame_index, nullptr);
}

luz_status luz_frame_set_shadow_cull(luz_frame* f, int32_t enable) {
    if (!f) return LUZ_ERR_INVALID;
    f->shadow_cull = enable != 0;
    return LUZ_OK;
}

luz_status luz_trace_visibility_stats(luz_ctx* ctx, luz_frame* f, const luz_tlas* t, int32_t frame_index,
                                      uint64_t out[5]) {
    if (!ctx || !f || !t || !out) return LUZ_ERR_INVALID;
    unsigned long long* d = nullptr;
    LUZ_CUDA(ctx, cudaMalloc(&d, 5 * sizeof(unsigned long long)));
    luz_status s = LUZ_OK;
    cudaError_t z = cudaMemsetAsync(d, 0, 5 * sizeof(unsigned long long), ctx->stream);   // zero when nothing is traced
    if (z != cudaSuccess) s = cuda_error(ctx, z, "stats clear");
    if (s == LUZ_OK) s = launch_visibility(ctx, f, t, frame_index, d);
    if (s == LUZ_OK) {
        cudaError_t e = cudaMemcpyAsync(out, d, 5 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) s = cuda_error(ctx, e, "stats read-back");
    }
    cudaFree(d);
    return s;
}

luz_status luz_ao_resolve(luz_ctx* ctx, luz_frame* f) {
    if (!ctx || !f) return LUZ_ERR_INVALID;
    return launch_ao_resolve(ctx, f);
}

luz_status luz_frame_lit_count(luz_ctx* ctx, luz_frame* f, uint32_t* count) {
    if (!ctx || !f || !count) return LUZ_ERR_INVALID;
    return frame_lit_count(ctx, f, count);
}

luz_status luz_light_pass(luz_ctx* ctx, luz_frame* f, int32_t mode) {
    if (!ctx || !f) return LUZ_ERR_INVALID;
    // public modes 0, 1, 2 -> plain, denoised AO, composed from the denoiser's output
    if (mode < LUZ_LIGHT_PASS_PLAIN || mode > LUZ_LIGHT_PASS_DENOISED)
        return set_error(ctx, LUZ_ERR_INVALID, "unknown light pass mode");
    return launch_light_pass(ctx, f, mode == LUZ_LIGHT_PASS_DENOISED ? 3 : mode);
}

luz_status luz_render_frame(luz_ctx* ctx, luz_frame* f, luz_tlas* t, const luz_instance* instances,
                            uint32_t instance_count, int32_t frame_index) {
    if (!ctx || !f || !t) return LUZ_ERR_INVALID;
    luz_status s;
    if ((s = luz_tlas_build(ctx, t, instances, instance_count)) != LUZ_OK) return s;
    if ((s = launch_gbuffer(ctx, f, t)) != LUZ_OK) return s;
    if ((s = launch_visibility(ctx, f, t, frame_index, nullptr)) != LUZ_OK) return s;
    return launch_light_pass(ctx, f, 0);
}

size_t luz_frame_plane_bytes(const luz_frame* f, int32_t plane) {
    if (!f) return 0;
    size_t P = f->pixels;
    switch (plane) {
        case LUZ_PLANE_ALBEDO: case LUZ_PLANE_MATERIAL: case LUZ_PLANE_EMISSION: case LUZ_PLANE_DEPTH:
        case LUZ_PLANE_AO: case LUZ_PLANE_AO_DENOISED: case LUZ_PLANE_LIN_DEPTH:
        case LUZ_PLANE_COMPOSE: return P * 4;
        case LUZ_PLANE_NORMAL: case LUZ_PLANE_LIGHT: case LUZ_PLANE_FEATURES: case LUZ_PLANE_TAA:
        case LUZ_PLANE_SIGNAL: case LUZ_PLANE_UNSHADOWED: case LUZ_PLANE_DENOISED: return P * 16;
        case LUZ_PLANE_PRIMARY_HIT: return P * 8;
        case LUZ_PLANE_SHADOW_BITS: return (size_t)f->shadow_slots * f->words * 4;
        case LUZ_PLANE_AO_BITS: return (size_t)f->ao_samples * f->words * 4;
        default: return 0;
    }
}

void* luz_frame_plane_device_ptr(luz_frame* f, int32_t plane) {
    if (!f) return nullptr;
    switch (plane) {
        case LUZ_PLANE_ALBEDO: return f->albedo;
        case LUZ_PLANE_NORMAL: return f->normal;
        case LUZ_PLANE_MATERIAL: return f->material;
        case LUZ_PLANE_EMISSION: return f->emission;
        case LUZ_PLANE_DEPTH: return f->depth;
        case LUZ_PLANE_LIGHT: return f->light;
        case LUZ_PLANE_SHADOW_BITS: return f->shadow_bits;
        case LUZ_PLANE_AO_BITS: return f->ao_bits;
        case LUZ_PLANE_AO: return f->ao;
        case LUZ_PLANE_AO_DENOISED: return f->ao_denoised;
        case LUZ_PLANE_PRIMARY_HIT: return f->primary_hit;
        case LUZ_PLANE_FEATURES: return f->features;
        case LUZ_PLANE_LIN_DEPTH: return f->lin_depth;
        case LUZ_PLANE_TAA: return f->taa;
        case LUZ_PLANE_COMPOSE: return f->compose;
        case LUZ_PLANE_SIGNAL: return f->signal;
        case LUZ_PLANE_UNSHADOWED: return f->unshadowed;
        case LUZ_PLANE_DENOISED: return f->denoised;
        default: return nullptr;
    }
}

luz_status luz_frame_read(luz_ctx* ctx, luz_frame* f, int32_t plane, void* dst, size_t bytes) {
    if (!ctx || !f || !dst) return LUZ_ERR_INVALID;
    size_t need = luz_frame_plane_bytes(f, plane);
    void* src = luz_frame_plane_device_ptr(f, plane);
    if (!src || bytes < need) return set_error(ctx, LUZ_ERR_INVALID, "bad plane or short buffer");
    if (need == 0) return LUZ_OK;
    LUZ_CUDA(ctx, cudaMemcpyAsync(dst, src, need, cudaMemcpyDeviceToHost, ctx->stream));
    LUZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return LUZ_OK;
}

luz_status luz_frame_write(luz_ctx* ctx, luz_frame* f, int32_t plane, const void* src, size_t bytes) {
    if (!ctx || !f || !src) return LUZ_ERR_INVALID;
    size_t need = luz_frame_plane_bytes(f, plane);
    void* dst = luz_frame_plane_device_ptr(f, plane);
    if (!dst || bytes != need) return set_error(ctx, LUZ_ERR_INVALID, "bad plane or size mismatch");
    if (need == 0) return LUZ_OK;
    LUZ_CUDA(ctx, cudaMemcpyAsync(dst, src, need, cudaMemcpyHostToDevice, ctx->stream));
    LUZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    // the lit list comes from the normal, depth, albedo, material and emission planes,
    // and its pass writes the background pixels of the light plane
    if (plane == LUZ_PLANE_NORMAL || plane == LUZ_PLANE_DEPTH || plane == LUZ_PLANE_LIGHT ||
        plane == LUZ_PLANE_ALBEDO || plane == LUZ_PLANE_MATERIAL || plane == LUZ_PLANE_EMISSION)
        f->surf_valid = false;
    return LUZ_OK;
}

}  // extern "C"
