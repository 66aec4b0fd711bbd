// batch.cu — many independent scenes of uneven size rendered as one unit: every TLAS
// build and G-buffer pass, ONE persistent visibility launch over the shadow/AO rays of
// all scenes, every light pass; recordable as one CUDA graph and replayed with a
// single launch; a launch-shape autotuner for the visibility kernel. (No counterpart
// in the reference, which renders one scene per frame.)
#include <algorithm>
#include <cstring>
#include <vector>

#include "visibility.cuh"

namespace luz {
luz_status pack_tlas_input(luz_ctx* ctx, luz_tlas* t, const luz_instance* inst, uint32_t n);
luz_status launch_tlas_build(luz_ctx* ctx, luz_tlas* t);
luz_status launch_gbuffer(luz_ctx* ctx, luz_frame* f, const luz_tlas* t);
luz_status launch_light_pass(luz_ctx* ctx, luz_frame* f, int mode);
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
};

namespace luz {

static luz_status batch_record(luz_ctx* ctx, luz_batch* b, int frame_index, bool stats) {
    // The sampler frame index lives in the per-scene records (fixed inside a graph).
    if (frame_index != b->frame_index) {
        for (auto& s : b->h_scenes) s.frame = frame_index;
        LUZ_CUDA(ctx, cudaMemcpyAsync(b->d_scenes, b->h_scenes.data(), b->h_scenes.size() * sizeof(SceneVis),
                                      cudaMemcpyHostToDevice, ctx->stream));
        b->frame_index = frame_index;
    }
    luz_status s;
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

static void drop_graph(luz_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
}

}  // namespace luz

using namespace luz;

extern "C" {

luz_status luz_batch_create(luz_ctx* ctx, uint32_t count, const luz_batch_scene* scenes, luz_batch** out) {
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
        b->h_scenes.push_back(make_scene_vis(f, t, 0));
    }
    cudaError_t e = cudaMalloc(&b->d_scenes, count * sizeof(SceneVis));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_offsets, (count + 1) * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_work, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_stats, 5 * sizeof(unsigned long long));
    if (e == cudaSuccess)
        e = cudaMemcpy(b->d_scenes, b->h_scenes.data(), count * sizeof(SceneVis), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail(cuda_error(ctx, e, "batch allocation"));
    *out = b;
    return LUZ_OK;
}

void luz_batch_destroy(luz_batch* b) {
    if (!b) return;
    cudaDeviceSynchronize();
    drop_graph(b);
    for (auto* f : b->frames) luz_frame_destroy(f);
    for (auto* t : b->tlas) luz_tlas_destroy(t);
    void* p[] = {b->d_scenes, b->d_offsets, b->d_work, b->d_stats};
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

// Times the visibility launch of the batch for each candidate shape and keeps the
// fastest (median of `reps` launches). Candidates: refill {8,16,32} x steps
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
                    for (auto* f : b->frames)
                        if ((s = clear_visibility(ctx, f)) != LUZ_OK) return s;
                    cudaEventRecord(e0, ctx->stream);
                    s = launch_visibility_batch(ctx, b->d_scenes, (uint32_t)b->frames.size(), b->d_offsets, b->d_work,
                                                nullptr);
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

}  // extern "C"
