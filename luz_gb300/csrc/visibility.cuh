// visibility.cuh — inputs of the visibility kernels, shared with the batch driver.
#pragma once
#include "internal.cuh"

namespace luz {

// Per-scene inputs of the visibility pass (a device array in batch mode).
struct SceneVis {
    const float4* tlas_nodes;
    uint32_t tlas_node_count;
    uint32_t instance_count;
    const DevInstance* instances;
    const float4* surf;
    const uint32_t* lit_count;
    const luz_light* lights;
    const uint32_t* slot_table;
    uint32_t shadow_slots, ao_samples;
    float cam[3];
    float ao_min, ao_max;
    int sampler, frame;
    int cull;                 // leave out shadow rays that cannot change the light pass's output
    uint32_t width, words;
    uint32_t* shadow_bits;
    uint32_t* ao_bits;
    // Short rays (near lists, visibility_kernel only; near_reach = 0 disables them)
    const uint4* near;
    const uint32_t* order;      // TLAS leaf -> instance input index
    const uint32_t* leaf_of;    // instance input index -> TLAS leaf
    const uint32_t* hit_instance;
    float near_reach;
    // Shadow-ray beam lists (visibility_kernel only; null disables them): per group of
    // 32 items, count + 7 TLAS leaves
    const uint32_t* beam_lists;
    const float4* leaf_box;      // TLAS leaf boxes (lo, hi), leaf order
    uint32_t beam_cap;           // leaves a beam list may hold before it falls back
};

struct VisCommon {
    const uint8_t* blue_noise;
    uint32_t bn_size;
    unsigned long long* work_counter;
    uint32_t* status;
    uint32_t refill, steps, smem_nodes;
    uint32_t step_cap;        // traversal steps per ray before it is ended (LUZ_DEV_TRAVERSAL_CAP)
};

// The context's visibility launch shape (the library defaults until one is set).
const VisTuning& vis_tuning(const luz_ctx* ctx);
// Launch-independent inputs of the visibility kernels (blue noise, status word, shape).
VisCommon make_vis_common(luz_ctx* ctx, unsigned long long* work_counter);
SceneVis make_scene_vis(const luz_frame* f, const luz_tlas* t, int frame_index);
// World boxes of the last TLAS build's instances (input order, lo / hi float4 pairs)
// and its leaf boxes (leaf order).
const float4* tlas_instance_boxes(const luz_tlas* t);
const float4* tlas_leaf_boxes(const luz_tlas* t);
luz_status clear_visibility(luz_ctx* ctx, luz_frame* f);
luz_status launch_visibility_batch(luz_ctx* ctx, const SceneVis* d_scenes, uint32_t n,
                                   unsigned long long* d_offsets, unsigned long long* work_counter,
                                   unsigned long long* d_stats);

}  // namespace luz
