// internal.cuh — device records, handle structs and error plumbing of libluz_gb300.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/luz.h"
#include "device_setup.hpp"
#include "pathmath.cuh"

namespace luz {

// ---------------------------------------------------------------- BVH layout
// A BVH node holds the boxes of its two children, 64 B = 4 x float4:
//   n0 = (c0.lo.x, c0.hi.x, c0.lo.y, c0.hi.y)
//   n1 = (c1.lo.x, c1.hi.x, c1.lo.y, c1.hi.y)
//   n2 = (c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z)
//   n3 = (child0, child1, 0, 0) as int bits; child >= 0 is an internal node index,
//        child < 0 is a leaf ~index (a triangle in a BLAS, an instance in a TLAS).
// A triangle is 48 B = 3 x float4: (v0, prim), (v1, 0), (v2, 0) in object space, in
// sorted leaf order; `prim` is the original triangle index as int bits.
constexpr int kNodeF4 = 4;
constexpr int kTriF4 = 3;
constexpr int32_t kEmptyChild = (int32_t)0x80000001;  // child slot with an inverted box
constexpr int32_t kStackMarker = (int32_t)0x80000000; // two-level stack: back to the TLAS
constexpr int kStackSize = 128;

// A 4-wide node (128 B = 8 x float4), the even-depth collapse of the binary tree:
//   f0 lo.x[4], f1 hi.x[4], f2 lo.y[4], f3 hi.y[4], f4 lo.z[4], f5 hi.z[4],
//   f6 child[4] (int bits: >= 0 a 4-wide node, < 0 a leaf ~index, kEmptyChild), f7 0.
constexpr int kNode4F4 = 8;

// Items (rays) per visibility chunk: the ray generation pass writes one chunk of
// 32-B ray records (4 GiB at most; a 1080p frame with 57 rays per pixel fits one
// chunk even when every pixel is lit), the traversal kernel consumes it.
constexpr uint32_t kRayChunk = 1u << 27;

// One TLAS leaf, in sorted (leaf) order. 96 B, 16-B aligned for vector loads.
// sphere: the BLAS's bounding sphere in object space, (centre, radius): the root box
// centre and the square root of the largest squared vertex distance from it (the
// root node's spare word), +inf when that word is not finite.
struct __align__(16) DevInstance {
    float w2o[12];          // world -> object, 3x4 row-major
    float4 sphere;
    uint32_t custom_index;  // instanceCustomIndex = modelRID
    uint32_t mask;
    uint32_t input_index;   // position in the caller's instance array
    uint32_t blas_prims;    // BLAS primitive count
    const float4* nodes4;   // BLAS 4-wide nodes
    const float4* tris;     // BLAS triangles
};
static_assert(sizeof(DevInstance) == 96, "DevInstance layout");

// A frame texture: RGBA8 texels (one u32 each, rows top to bottom).
struct DevTexture {
    const uint32_t* texels;
    uint32_t width, height;
};

// A light's shadow map as the light pass reads it.
struct DevShadowLight {
    const float* map;        // faces * res * res depths
    float view_proj0[16];
    float position[3];
    float z_far;
    uint32_t faces;          // 0 = no map, 1 = 2D, 6 = cube (+x, -x, +y, -y, +z, -z)
    uint32_t res;
};

// Per-instance data used by the G-buffer kernel, in the caller's instance order.
struct DevShadeInstance {
    float normal_mat[9];    // transpose(inverse(model 3x3)), row-major
    float pad0;
    const luz_vertex* vertices;
    const uint32_t* indices;
};

// Host-side instance as uploaded by luz_tlas_build (64 B + pointers).
struct DevInstanceInput {
    float o2w[12];
    const float4* nodes;
    const float4* tris;
    const luz_vertex* vertices;
    const uint32_t* indices;
    uint32_t custom_index;
    uint32_t mask;
    uint32_t blas_prims;
    uint32_t pad;
    const float4* nodes4;
};

// ---------------------------------------------------------------- handles
struct Arena {            // one device allocation shared by a batch of BLAS
    void* base = nullptr;
    int refs = 0;
};

// Launch shape of the visibility kernel (chosen by the autotuner, or defaults).
struct VisTuning {
    uint32_t smem_nodes;    // TLAS nodes staged in shared memory per CTA
    uint32_t refill;        // idle lanes that trigger a refill (1..32)
    uint32_t steps;         // traversal steps between refill checks
    uint32_t ctas_per_sm;
    uint32_t set;           // 0 = use the library defaults
};

}  // namespace luz

struct luz_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    std::string last_error;
    uint32_t* d_status = nullptr;        // device status word (LUZ_DEV_* bits)
    uint64_t launches = 0;
    uint8_t* d_blue_noise = nullptr;     // RGBA8 size*size
    float* d_srgb_lut = nullptr;         // pow(i / 255, 2.2), i = 0..255 (albedo decode)
    uint32_t blue_noise_size = 0;
    // reusable scratch
    void* d_scratch = nullptr;
    size_t scratch_bytes = 0;
    void* h_pinned = nullptr;
    size_t pinned_bytes = 0;
    int sm_count = 0;
    int raygen_blocks = 0;                      // resident ray-generation blocks per SM (0: not queried)
    bool registered = false;                    // counted among the process's live contexts
    luz::VisTuning vis_tuning{0, 0, 0, 0, 0};   // set == 0: library defaults
    uint32_t debug_step_cap = 0;                // traversal steps per ray, 0 = the library's cap
    // device pipeline of the last batched BLAS build (after its host->device copies)
    cudaEvent_t build_ev[2] = {nullptr, nullptr};
    bool build_timed = false;
    // per-kernel timing (luz_ctx_profile): an event pair around each instrumented launch
    bool prof_on = false;
    std::vector<cudaEvent_t> prof_pool;
    size_t prof_used = 0;
    struct ProfRec { int32_t kernel; cudaEvent_t a, b; };
    std::vector<ProfRec> prof_recs;
};

struct luz_blas {
    luz_ctx* ctx = nullptr;
    luz::Arena* arena = nullptr;
    float4* nodes = nullptr;             // max(n-1,1) nodes
    float4* nodes4 = nullptr;            // 4-wide collapse (at most max(n-1,1) nodes)
    float4* tris = nullptr;              // n triangles
    uint32_t* morton = nullptr;          // sorted 30-bit keys (n)
    uint32_t* order = nullptr;           // sorted primitive order (n)
    luz_vertex* vertices = nullptr;      // shading copy of the vertex buffer (48-B stride)
    uint32_t* indices = nullptr;
    uint32_t prims = 0;
    uint32_t vertex_count = 0;
    luz_memory memory{};                 // bytes of this BLAS's slices of the arena
};

struct luz_tlas {
    luz_ctx* ctx = nullptr;
    uint32_t max_instances = 0;
    uint32_t count = 0;
    float4* nodes = nullptr;             // BFS order, max(n-1,1) nodes
    float4* nodes4 = nullptr;            // 4-wide collapse, breadth-first order
    uint32_t* levels = nullptr;          // BFS level table (count, starts)
    luz::DevInstance* instances = nullptr;        // leaf order
    luz::DevShadeInstance* shade = nullptr;       // input order
    luz::DevInstanceInput* d_input = nullptr;
    luz::DevInstanceInput* h_input = nullptr;     // pinned staging
    uint32_t* morton = nullptr;
    uint32_t* order = nullptr;
    uint4* near = nullptr;               // per instance (input order): near list of short rays
    uint32_t* leaf_of = nullptr;         // per instance (input order): its TLAS leaf
    uint32_t node_count = 0;
    cudaEvent_t input_copied = nullptr;           // h_input may be rewritten after this
    // build temporaries
    void* tmp = nullptr;
    size_t tmp_bytes = 0;
};

struct luz_frame {
    luz_ctx* ctx = nullptr;
    uint32_t width = 0, height = 0, pixels = 0, words = 0;  // words per bit plane
    // G-buffer (DeferredRenderer.cpp:175-248 formats)
    uint32_t* albedo = nullptr;     // RGBA8
    float4* normal = nullptr;       // RGBA32F
    uint32_t* material = nullptr;   // RGBA8
    uint32_t* emission = nullptr;   // RGBA8
    float* depth = nullptr;         // F32
    float4* light = nullptr;        // RGBA32F
    uint2* primary_hit = nullptr;
    uint32_t* hit_instance = nullptr;    // input index of the primary hit's instance (~0 = miss)
    uint32_t* gb_coarse = nullptr;       // G-buffer candidate leaves per 64x64 tile (count + 255)
    uint32_t* gb_fine = nullptr;         // and per 8x8 tile (count + 15)
    // visibility
    uint32_t* shadow_bits = nullptr;
    uint32_t* ao_bits = nullptr;
    float* ao = nullptr;
    float* ao_denoised = nullptr;
    bool shadow_cull = true;        // leave out shadow rays that cannot change the image
    float4* signal = nullptr;       // shadowed direct light S (r, g, b) and AO per pixel: denoiser input
    float4* unshadowed = nullptr;   // unshadowed direct light U (r, g, b) and lit shadow fraction per pixel
    float4* denoised = nullptr;     // filtered shadow ratio (r, g, b) and AO
    void* features = nullptr;       // 8 x bf16 per pixel (denoiser input)
    float* lin_depth = nullptr;
    uint32_t* dn_list = nullptr;    // lit pixels in row-major order (x | y << 16), from the features pass
    uint32_t* dn_count = nullptr;   // its length (device counter)
    float4* taa = nullptr;          // TAA output = next frame's history
    float4* taa_next = nullptr;
    uint32_t* compose = nullptr;    // BGRA8 tone-mapped output
    uint32_t* hist = nullptr;       // 256 bins | luz_histogram
    luz::DevShadowLight* d_shadow_lights = nullptr;
    float* d_shadow_maps = nullptr;
    size_t shadow_maps_bytes = 0;
    uint32_t shadow_light_count = 0, shadow_res = 0;
    std::vector<size_t> h_shadow_offset;     // per light: first float of its map
    std::vector<uint32_t> h_shadow_faces;
    float* hist_state = nullptr;    // adapted luminance across frames
    uint32_t shadow_planes_cap = 0, ao_planes_cap = 0;
    uint32_t shadow_slots = 0, ao_samples = 0;
    // compacted lit pixels
    float4* surf = nullptr;         // 2 float4 per lit pixel: (fragPos, pixel), (N, x | y << 16)
    uint4* surf_mat = nullptr;      // 1 uint4 per lit pixel: (albedo, material, emission, pixel) words
    bool surf_valid = false;        // surf / lit_count match the current planes and scene
    uint32_t* block_counts = nullptr;
    uint32_t* lit_count = nullptr;  // device counter
    uint32_t h_lit_count = 0;
    // scene constants
    luz_scene h_scene{};
    luz_scene* d_scene = nullptr;
    luz_light* d_lights = nullptr;
    uint32_t lights_cap = 0, light_count = 0;
    luz_model* d_models = nullptr;
    uint32_t models_cap = 0, model_count = 0;
    uint32_t* d_slot_table = nullptr;  // per shadow slot: light | sample << 16
    std::vector<uint32_t> h_slot_table;
    uint32_t* d_light_slot = nullptr;  // per light: first shadow slot
    uint8_t* d_model_skip = nullptr;   // per model: 1 = discarded by the alpha test, 2 = tested per hit
    int32_t max_map_index = -1;        // largest texture index of the uploaded ModelBlocks
    luz::DevTexture* d_textures = nullptr;
    void* d_texels = nullptr;
    uint32_t texture_count = 0;
    unsigned long long* work_counter = nullptr;
    // generated shadow / AO rays of one chunk (structure of arrays, rays_cap each):
    // (origin, tMax) and (direction, pixel); tMax = -inf marks an item with no ray
    float4* rays_a = nullptr;
    float4* rays_b = nullptr;
    uint32_t* rays_c = nullptr;          // own instance of a ray that starts at its near list
    float4* beams = nullptr;             // per group of 32 items: origin ball, end-point ball
    uint32_t* beam_lists = nullptr;      // per group of 32 items: count + up to 31 TLAS leaves
    uint32_t rays_cap = 0;
};

// ---------------------------------------------------------------- error plumbing
namespace luz {
luz_status set_error(luz_ctx* ctx, luz_status st, const std::string& msg);
luz_status cuda_error(luz_ctx* ctx, cudaError_t e, const char* what);
luz_status ensure_scratch(luz_ctx* ctx, size_t bytes);
luz_status check_launch(luz_ctx* ctx, const char* what);
// The current generation of per-device setup (device_setup.hpp): a new one starts
// when a context is created while no other context of the process is alive.
uint64_t setup_generation();
// Rebuilds the frame's lit-pixel list when its planes or scene constants changed.
luz_status ensure_lit_list(luz_ctx* ctx, luz_frame* f);
// Per-kernel timing: prof_begin records an event before a launch of kernel `kernel`
// (LUZ_KERNEL_*), prof_end one after it, both on the context's stream; nothing when
// profiling is off or the stream is being captured.
void prof_begin(luz_ctx* ctx, int32_t kernel);
void prof_end(luz_ctx* ctx);

// Runs the body of a C entry point that sizes host memory from its inputs: a failed
// host allocation (std::bad_alloc) or another C++ exception becomes a status, as no
// exception may cross the C ABI.
template <class F>
luz_status guarded(luz_ctx* ctx, F&& body) noexcept {
    auto note = [ctx](luz_status st, const char* what) noexcept {
        try {
            if (ctx) ctx->last_error = what;
        } catch (...) {
        }
        return st;
    };
    try {
        return body();
    } catch (const std::bad_alloc&) {
        return note(LUZ_ERR_OOM, "host allocation failed");
    } catch (const std::exception& e) {
        return note(LUZ_ERR_INVALID, e.what());
    } catch (...) {
        return note(LUZ_ERR_INVALID, "unexpected exception");
    }
}
}  // namespace luz

#define LUZ_CUDA(ctx, call)                                          \
    do {                                                             \
        cudaError_t e_ = (call);                                     \
        if (e_ != cudaSuccess) return luz::cuda_error(ctx, e_, #call); \
    } while (0)

#define LUZ_LAUNCHED(ctx, name)                                  \
    do {                                                         \
        (ctx)->launches++;                                       \
        luz_status s_ = luz::check_launch(ctx, name);            \
        if (s_ != LUZ_OK) return s_;                             \
    } while (0)
