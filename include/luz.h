/*
 * luz.h — C ABI of the GB300-native ray-traced visibility and deferred-lighting path.
 *
 * Every entry point replaces one call of the reference renderer's RHI / renderer
 * surface (hadryansalles/Luz); the replaced interface is cited beside each one as
 * file:line within that project. Plain C types only: pointers, sizes, PODs and
 * opaque handles. No exception crosses this boundary; every call returns a
 * luz_status and the context keeps a human-readable message (luz_last_error).
 *
 * Threading: a luz_ctx is thread-compatible (one host thread at a time), like the
 * reference's single global Vulkan context `_ctx` (source/Graphics/VulkanWrapper.cpp).
 * All GPU work of a context is ordered on the context's CUDA stream. Several contexts
 * may be driven from several threads at once; they all use one device (one process
 * per GPU, as the reference runs one Vulkan device per process).
 */
#ifndef LUZ_GB300_H
#define LUZ_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status */
typedef int32_t luz_status;
enum {
    LUZ_OK = 0,
    LUZ_ERR_INVALID = 1,        /* bad argument / handle / size                 */
    LUZ_ERR_CUDA = 2,           /* a CUDA runtime call failed                   */
    LUZ_ERR_OOM = 3,            /* device or host allocation failed             */
    LUZ_ERR_DEVICE = 4,         /* a kernel raised its status word (see below)  */
    LUZ_ERR_LIMIT = 5,          /* a documented size limit was exceeded         */
    LUZ_ERR_NO_DEVICE = 6       /* no CUDA device / driver                      */
};

/* Device status-word bits (luz_ctx_device_status). Kernels never trap; every
 * spin or traversal loop has an iteration cap and sets one of these instead. */
enum {
    LUZ_DEV_SORT_LOOKBACK_TIMEOUT = 1u << 0,
    LUZ_DEV_STACK_OVERFLOW = 1u << 1,
    LUZ_DEV_TRAVERSAL_CAP = 1u << 2,
    LUZ_DEV_KARRAS_RANGE = 1u << 3,
    LUZ_DEV_BATCH_QUEUE = 1u << 4,
    LUZ_DEV_BAD_INDEX = 1u << 5,
    LUZ_DEV_RASTER_OVERFLOW = 1u << 6,
    LUZ_DEV_MMA_WAIT = 1u << 7          /* a tensor-core product did not complete in time */
};

/* ------------------------------------------------------------------ limits */
#define LUZ_MAX_SHADOW_SLOTS 16384  /* Σ_lights numShadowSamples per pixel      */
#define LUZ_MAX_AO_SAMPLES 4096     /* aoNumSamples per pixel                   */
#define LUZ_BLUE_NOISE_SIZE 128     /* substitute blue-noise texture, RGBA8     */

/* Light types and shadow types: source/Shaders/LuzCommon.h:24-29. */
#define LUZ_LIGHT_POINT 0
#define LUZ_LIGHT_SPOT 1
#define LUZ_LIGHT_DIRECTIONAL 2
#define LUZ_SHADOW_DISABLED 0
#define LUZ_SHADOW_RAYTRACING 1
#define LUZ_SHADOW_MAP 2

/* Sample sequences. PARITY reproduces BlueNoiseSample (source/Shaders/light.frag:71-75)
 * over the seeded substitute texture; STRATIFIED is a per-pixel rotated R2 sequence
 * evaluated in 32-bit fixed point, which stays unbiased at 1024+ samples. */
#define LUZ_SAMPLER_PARITY 0
#define LUZ_SAMPLER_STRATIFIED 1

/* ------------------------------------------------------------------ data contract */

/* MeshAsset::MeshVertex, 48 B (source/Resources/AssetManager.hpp:83-91). */
typedef struct luz_vertex {
    float position[3];
    float normal[3];
    float tangent[4];
    float texcoord[2];
} luz_vertex;

/* The fields of LightBlock (source/Shaders/LuzCommon.h:37-50) that the ray-traced
 * light pass reads; 64 B. Angles are radians (GPUScene.cpp:244,246 converts). The
 * shadow-map matrices and volumetric fields (LuzCommon.h:52-60) are not on the path. */
typedef struct luz_light {
    float color[3];
    float intensity;
    float position[3];
    float inner_angle;
    float direction[3];
    float outer_angle;
    int32_t type;
    int32_t num_shadow_samples;
    float radius;
    int32_t shadow_map;
} luz_light;

/* ModelBlock, 128 B (source/Shaders/LuzCommon.h:76-92). model_mat is column-major
 * (glm layout). Texture and buffer RIDs are kept for layout parity; texture maps
 * index luz_frame textures (-1 = none). */
typedef struct luz_model {
    float model_mat[16];
    float color[4];
    float emission[3];
    float metallic;
    float roughness;
    int32_t ao_map;
    int32_t color_map;
    int32_t normal_map;
    int32_t emission_map;
    int32_t metallic_roughness_map;
    int32_t vertex_buffer;
    int32_t index_buffer;
} luz_model;

/* SceneBlock (source/Shaders/LuzCommon.h:94-125) without its fixed
 * `LightBlock lights[LUZ_MAX_LIGHTS]` array: lights travel as a separate array of
 * any length (the reference caps them at 64, LuzCommon.h:20). Matrices column-major. */
typedef struct luz_scene {
    float ambient_light_color[3];
    float ambient_light_intensity;
    float proj[16];
    float view[16];
    float view_proj[16];
    float prev_view_proj[16];
    float inverse_proj[16];
    float inverse_view[16];
    float jitter[2];
    float prev_jitter[2];
    float cam_pos[3];
    int32_t num_lights;
    float ao_min;
    float ao_max;
    float exposure;
    int32_t ao_num_samples;
    int32_t white_texture;
    int32_t black_texture;
    int32_t blue_noise_texture;
    int32_t tlas_rid;
    int32_t shadow_type;
    int32_t sampler;          /* LUZ_SAMPLER_*; occupies SceneBlock.pad[0]        */
    int32_t pad[2];
} luz_scene;

typedef struct luz_blas luz_blas;
typedef struct luz_tlas luz_tlas;
typedef struct luz_ctx luz_ctx;
typedef struct luz_frame luz_frame;

/* VkAccelerationStructureInstanceKHR as filled by vkw::CmdBuildTLAS
 * (source/Graphics/VulkanWrapper.cpp:1111-1126): 3x4 row-major object-to-world
 * transform (rows = the first three rows of modelMat), custom index = modelRID,
 * mask 0xFF, triangle facing cull disabled (every traversal here is two-sided). Rays
 * use cull mask 0xFF (light.frag:100,126), so an instance whose mask has none of
 * the low eight bits set is invisible to the G-buffer, shadow and AO rays (shadow
 * maps, a raster pass in the reference, draw every instance). */
typedef struct luz_instance {
    const luz_blas* blas;
    float transform[3][4];
    uint32_t custom_index;
    uint32_t mask;
} luz_instance;

/* BLASDesc (source/Graphics/VulkanWrapper.h:206-213) with host-side buffers. */
typedef struct luz_blas_desc {
    const void* vertices;       /* positions as float[3] at offset 0 of each vertex */
    uint32_t vertex_count;
    uint32_t vertex_stride;     /* bytes; 48 for luz_vertex                          */
    const uint32_t* indices;
    uint32_t index_count;       /* multiple of 3                                     */
} luz_blas_desc;

/* G-buffer / frame planes (formats of DeferredRenderer::CreateImages,
 * source/Graphics/DeferredRenderer.cpp:175-248). */
enum {
    LUZ_PLANE_ALBEDO = 0,       /* RGBA8 UNORM, 4 B/px                               */
    LUZ_PLANE_NORMAL = 1,       /* RGBA32F, 16 B/px                                  */
    LUZ_PLANE_MATERIAL = 2,     /* RGBA8 UNORM (rough, metal, occl, 1)               */
    LUZ_PLANE_EMISSION = 3,     /* RGBA8 UNORM                                       */
    LUZ_PLANE_DEPTH = 4,        /* F32, NDC z in [0,1]                               */
    LUZ_PLANE_LIGHT = 5,        /* RGBA32F light-pass output                         */
    LUZ_PLANE_SHADOW_BITS = 6,  /* u32 bit planes: [slot][ceil(W*H/32)], hit = 1     */
    LUZ_PLANE_AO_BITS = 7,      /* u32 bit planes: [sample][ceil(W*H/32)], miss = 1  */
    LUZ_PLANE_AO = 8,           /* F32 per-pixel AO value (mean of misses)            */
    LUZ_PLANE_AO_DENOISED = 9,  /* F32 per-pixel denoised AO                          */
    LUZ_PLANE_PRIMARY_HIT = 10, /* u32x2 per pixel: (instance custom index, prim id), ~0 = miss */
    LUZ_PLANE_FEATURES = 11,    /* 8 x bf16 per pixel: denoiser input channels           */
    LUZ_PLANE_LIN_DEPTH = 12,   /* F32 distance to the camera, 0 for background          */
    LUZ_PLANE_TAA = 13,         /* RGBA32F temporal anti-aliasing output (= next history)  */
    LUZ_PLANE_COMPOSE = 14,     /* BGRA8 UNORM composed, tone-mapped output (bytes B,G,R,A) */
    LUZ_PLANE_SIGNAL = 15,      /* RGBA32F denoiser input: shadowed direct light S r, g, b, AO */
    LUZ_PLANE_UNSHADOWED = 16,  /* RGBA32F unshadowed direct light U r, g, b, lit fraction     */
    LUZ_PLANE_DENOISED = 17,    /* RGBA32F denoiser output: shadow ratio R r, g, b, AO         */
    LUZ_PLANE_COUNT = 18
};

/* ------------------------------------------------------------------ context
 * luz_ctx_create makes `device` current on the calling thread; another thread that
 * drives the context makes the same device current first (cudaSetDevice), as the
 * entry points launch on the calling thread's current device. The contexts of a
 * process share one device: creating one on another device while a context lives
 * returns LUZ_ERR_INVALID. The one-time setup the kernels need on the device
 * (shared-memory limits, constant tables) is done again after the process's last
 * context was destroyed, so a device reset between contexts is picked up. */
luz_status luz_ctx_create(int device, luz_ctx** out);
void luz_ctx_destroy(luz_ctx* ctx);
const char* luz_last_error(const luz_ctx* ctx);
/* Waits for the context's stream; LUZ_ERR_DEVICE when a kernel has raised the device
 * status word since it was last read (luz_ctx_device_status reads and clears it). */
luz_status luz_ctx_synchronize(luz_ctx* ctx);
/* Reads and clears the device status word (LUZ_DEV_* bits). */
luz_status luz_ctx_device_status(luz_ctx* ctx, uint32_t* bits);
/* Number of kernels this context has launched so far. */
uint64_t luz_ctx_launch_count(const luz_ctx* ctx);
/* Debug knob, off by default (no counterpart in the reference): the traversal steps a
 * shadow / AO ray may take before the visibility kernel ends it (counted as not
 * occluded, AO: a miss) and raises LUZ_DEV_TRAVERSAL_CAP; 0 restores the library's cap
 * (2^22 steps). For testing that a cap which runs out ends the kernel with a status
 * instead of a hang. */
luz_status luz_ctx_set_debug_step_cap(luz_ctx* ctx, uint32_t steps);
/* Uses `stream` (a cudaStream_t) for all later work; NULL = the context's own. */
luz_status luz_ctx_set_stream(luz_ctx* ctx, void* stream);
/* Uploads the substitute blue-noise texture (RGBA8, size*size texels). */
luz_status luz_ctx_set_blue_noise(luz_ctx* ctx, const uint8_t* rgba8, uint32_t size);

/* Launch shape of the persistent visibility kernel (no counterpart in the reference,
 * whose traversal is the driver's): 4-wide TLAS nodes (128 B each) staged in shared
 * memory per CTA (0..1024), idle lanes that trigger a warp's refill (1..32), traversal steps between
 * refill checks (1..1024), CTAs per SM (1..16). All zero restores the defaults. */
typedef struct luz_vis_tuning {
    uint32_t smem_nodes;
    uint32_t refill;
    uint32_t steps;
    uint32_t ctas_per_sm;
} luz_vis_tuning;
luz_status luz_ctx_set_vis_tuning(luz_ctx* ctx, const luz_vis_tuning* tuning);
luz_status luz_ctx_get_vis_tuning(const luz_ctx* ctx, luz_vis_tuning* tuning);

/* Measurement hooks (no counterpart in the reference, which times passes with GPU
 * timestamp queries, source/Core/main.cpp:236-308). luz_ctx_last_blas_build_ms: the
 * device time of the last luz_blas_build[_batch] of this context from the end of its
 * host->device copies to its last kernel (CUDA events on the context's stream).
 * luz_ctx_probe_l2_read: the L2 read bandwidth in GB/s, from `reps` passes of 16-B
 * L2-only loads over a `bytes` buffer (allocated and freed by the call; keep it below
 * the L2 size, e.g. 48 MiB) on every SM. */
luz_status luz_ctx_last_blas_build_ms(luz_ctx* ctx, float* device_ms);
luz_status luz_ctx_probe_l2_read(luz_ctx* ctx, uint64_t bytes, uint32_t reps, float* gbs);
/* Per-kernel device time: with profiling on, every launch of the kernels below is
 * bracketed by a pair of CUDA events on the context's stream (not while the stream is
 * being captured into a graph). luz_ctx_profile(ctx, 1) clears earlier records and
 * starts, (ctx, 0) stops; luz_ctx_profile_read waits for the stream and returns the
 * summed milliseconds and the launch count of one kernel since the start. */
enum {
    LUZ_KERNEL_TLAS_BUILD = 0,  /* fused single-CTA TLAS build                      */
    LUZ_KERNEL_GBUFFER = 1,     /* primary closest-hit G-buffer                      */
    LUZ_KERNEL_RAYGEN = 2,      /* shadow / AO ray generation                        */
    LUZ_KERNEL_TRAVERSAL = 3,   /* persistent shadow / AO any-hit traversal          */
    LUZ_KERNEL_LIGHT_PASS = 4,  /* deferred light pass (every mode)                  */
    LUZ_KERNEL_FEATURES = 5,    /* denoiser features                                 */
    LUZ_KERNEL_DENOISE = 6,     /* denoiser network + filter                         */
    LUZ_KERNEL_TAA = 7,
    LUZ_KERNEL_DENOISE_TRAIN = 8, /* denoiser forward + backward + weight gradients   */
    LUZ_KERNEL_BATCH_FRAME = 9  /* a batch frame in one persistent launch            */
};
luz_status luz_ctx_profile(luz_ctx* ctx, int32_t on);
luz_status luz_ctx_profile_read(luz_ctx* ctx, int32_t kernel, float* total_ms, uint32_t* launches);

/* ------------------------------------------------------------------ BLAS
 * Replaces vkw::CreateBLAS + vkw::CmdBuildBLAS (source/Graphics/VulkanWrapper.h:236,
 * :229; VulkanWrapper.cpp:743-836, 1089-1104) as called by GPUScene::AddMesh
 * (source/Graphics/GPUScene.cpp:108-138). The reference builds one BLAS per
 * synchronous submit; the batched form builds all of them in one device pipeline. */
luz_status luz_blas_build(luz_ctx* ctx, const luz_blas_desc* desc, luz_blas** out);
luz_status luz_blas_build_batch(luz_ctx* ctx, uint32_t count, const luz_blas_desc* descs,
                                luz_blas** out);
void luz_blas_destroy(luz_blas* blas);
uint32_t luz_blas_primitive_count(const luz_blas* blas);

/* luz_blas_build_noalloc — builds one BLAS and allocates nothing. This entry point
 * has no counterpart in the reference renderer.
 *
 * For callers that cannot allocate device memory while they build: a renderer that
 * takes all of its device memory from one up-front budget, code that must not pay
 * the implicit synchronisation of cudaMalloc/cudaFree inside a frame, or a host that
 * owns every device allocation through its own pool. The caller passes device
 * buffers: vertices (luz_vertex, 48-B stride) and u32 indices as input; as output
 * nodes (max(n-1,1) x 64 B), triangles (n x 48 B), sorted Morton codes and sorted
 * primitive order (n x 4 B each), n = index_count / 3. The result is byte-identical
 * to luz_blas_build's (same layouts as luz_blas_download): the binary LBVH only.
 * It is not a luz_blas: the 4-wide nodes that the visibility and G-buffer traversals
 * walk are not built, and no entry point takes these buffers as a TLAS instance.
 *
 * Every temporary lives in one file-scope device array of LUZ_NOALLOC_SCRATCH_BYTES
 * (about 10.3 MiB), which every GPU that loads the library holds until the process
 * exits. n above LUZ_NOALLOC_MAX_TRIANGLES returns LUZ_ERR_LIMIT before any GPU
 * work. No cudaMalloc, cudaFree or allocating library routine is called.
 *
 * `stream` is a cudaStream_t (NULL = the legacy default stream); the call waits for
 * its own work on that stream before it returns. Every call outside a stream capture
 * looks up the array's device address (cudaGetSymbolAddress) with the current device
 * current, so a context torn down and created again after an earlier call is served
 * at the array's new address; a call inside a capture reuses the address of the last
 * call outside one, so make the first call on a device before any stream capture
 * (LUZ_ERR_INVALID otherwise). All calls share the one array and it
 * keeps the last call's contents (each call resets what it reads before writing):
 * calls that overlap on the GPU, from several host threads or streams, race.
 * Returns LUZ_ERR_INVALID for bad arguments or an index outside the vertex buffer
 * (checked on the device, the bad index is never dereferenced), LUZ_ERR_DEVICE if a
 * kernel raised its status word, LUZ_ERR_CUDA if a CUDA call failed. After
 * LUZ_ERR_INVALID from the index check, LUZ_ERR_DEVICE or LUZ_ERR_CUDA the output
 * buffers hold undefined contents (the build ran with the bad indices replaced by 0).
 * n = 0 writes one empty root node (inverted boxes) and nothing else. */
#define LUZ_NOALLOC_MAX_TRIANGLES (1u << 17)
#define LUZ_NOALLOC_SCRATCH_BYTES 10756608u
luz_status luz_blas_build_noalloc(const luz_vertex* d_vertices, uint32_t vertex_count,
                                  const uint32_t* d_indices, uint32_t index_count,
                                  void* d_nodes, void* d_tris, uint32_t* d_morton,
                                  uint32_t* d_order, void* stream);
/* Copies the built BLAS to host memory: nodes (64 B each, count = max(n-1,1)),
 * triangles (48 B each, sorted leaf order), the sorted Morton keys (u32) and the
 * sorted primitive order (u32). Any pointer may be NULL. For parity tests. The root
 * node's third child word (float 14) holds the bounding sphere's squared radius about
 * the root box centre (the largest squared distance of a triangle vertex from it, as
 * float bits); the TLAS build clips each instance box with the transformed sphere. */
luz_status luz_blas_download(luz_ctx* ctx, const luz_blas* blas, void* nodes, void* tris,
                             uint32_t* morton_sorted, uint32_t* order);
/* Copies the 4-wide traversal nodes (128 B each: lo.x[4], hi.x[4], lo.y[4], hi.y[4],
 * lo.z[4], hi.z[4], child[4] as int bits, 16 B zero) to host memory: the even-depth
 * collapse of the binary tree, numbered by rank among the even-depth binary nodes in
 * index order. The buffer holds max(n-1,1) entries; the first K are the nodes, K =
 * the number of even-depth binary nodes. For parity tests. */
luz_status luz_blas_download_wide(luz_ctx* ctx, const luz_blas* blas, void* nodes4);

/* Device bytes held by a BLAS / TLAS, by part: binary nodes (the parity-checked tree;
 * a TLAS build reads each BLAS root's box and bounding sphere from it), 4-wide nodes
 * (every traversal), triangles / instance records, other (sort keys,
 * order, shading copies of the vertex and index buffers; for a TLAS also the shading
 * and input records, near lists, leaf indices and build scratch).
 * The counterpart of the reference's vkGetAccelerationStructureBuildSizesKHR query
 * (source/Graphics/VulkanWrapper.cpp:692-698, 809-812). */
typedef struct luz_memory {
    uint64_t nodes;
    uint64_t wide_nodes;
    uint64_t leaves;
    uint64_t other;
} luz_memory;
luz_status luz_blas_memory(const luz_blas* blas, luz_memory* out);

/* ------------------------------------------------------------------ TLAS
 * Replaces vkw::CreateTLAS(maxInstances) and vkw::CmdBuildTLAS(tlas, instances)
 * (source/Graphics/VulkanWrapper.h:235,:243; VulkanWrapper.cpp:657-741, 1106-1139),
 * rebuilt every frame by GPUScene::UpdateResourcesGPU (GPUScene.cpp:348-366). */
luz_status luz_tlas_create(luz_ctx* ctx, uint32_t max_instances, luz_tlas** out);
luz_status luz_tlas_build(luz_ctx* ctx, luz_tlas* tlas, const luz_instance* instances,
                          uint32_t count);
void luz_tlas_destroy(luz_tlas* tlas);
/* Copies the TLAS nodes (64 B each, breadth-first order) and the sorted instance
 * order (u32) to host memory. For parity tests. */
luz_status luz_tlas_download(luz_ctx* ctx, const luz_tlas* tlas, void* nodes,
                             uint32_t* morton_sorted, uint32_t* order, uint32_t* node_count);
/* The TLAS's 4-wide nodes (layout and numbering as luz_blas_download_wide; the
 * buffer holds max(count,2)-1 entries). */
luz_status luz_tlas_download_wide(luz_ctx* ctx, const luz_tlas* tlas, void* nodes4);
luz_status luz_tlas_memory(const luz_tlas* tlas, luz_memory* out);

/* ------------------------------------------------------------------ frame
 * A luz_frame owns the per-resolution images of DeferredRenderer::CreateImages
 * (source/Graphics/DeferredRenderer.cpp:175-248) plus the visibility planes and the
 * device copies of SceneBlock/ModelBlock/lights (GPUScene.cpp:348-353). At most
 * 65535 pixels wide or high and 2^27 pixels in all (LUZ_ERR_LIMIT beyond). */
luz_status luz_frame_create(luz_ctx* ctx, uint32_t width, uint32_t height, luz_frame** out);
void luz_frame_destroy(luz_frame* frame);
/* Host→device copy of the scene constants, lights and model blocks; mirrors the two
 * CmdCopy calls of GPUScene::UpdateResourcesGPU (GPUScene.cpp:352-353). */
luz_status luz_frame_upload(luz_ctx* ctx, luz_frame* frame, const luz_scene* scene,
                            const luz_light* lights, uint32_t light_count,
                            const luz_model* models, uint32_t model_count);
/* Textures of the frame's ModelBlocks (RGBA8 UNORM, rows top to bottom, 4 B per
 * texel): map fields >= 0 index this list. Replaces earlier textures. Mirrors the
 * RGBA8_unorm images GPUScene::AddTexture creates (GPUScene.cpp:140-156) with the
 * reference's sampler: linear filtering, repeat addressing, one mip level
 * (VulkanWrapper.cpp:500, 2429-2454). count 0 clears. */
typedef struct luz_texture_desc {
    const uint8_t* rgba8;     /* host memory, width * height * 4 bytes */
    uint32_t width, height;
} luz_texture_desc;
luz_status luz_frame_set_textures(luz_ctx* ctx, luz_frame* frame, const luz_texture_desc* textures,
                                  uint32_t count);
/* Shadow maps (scene shadow type LUZ_SHADOW_MAP; light.frag:147-165). Per light the
 * LightBlock tail that the reference fills in GPUScene::UpdateResources
 * (GPUScene.cpp:266-303): point lights have six cube faces (+x, -x, +y, -y, +z, -z)
 * storing distance / z_far, other lights one orthographic map fitted to the camera
 * frustum storing NDC depth. luz_scene_shadow_lights (luz_scene.h) computes them. */
typedef struct luz_shadow_light {
    float view_proj[6][16];   /* column-major; only [0] for non-point lights */
    float z_far;              /* LightNode::shadowMapFar */
    uint32_t faces;           /* 6 point, 1 other, 0 = no map (shadowMap == -1) */
    float position[3];
    uint32_t pad;
} luz_shadow_light;
/* Rasterises every instance of the TLAS into each light's shadow map
 * (DeferredRenderer::ShadowMapPass, DeferredRenderer.cpp:268-292, with the shadowMap
 * vertex/geometry/fragment shaders): resolution^2 texels per face, depth test LESS from
 * a clear of 1.0, front faces culled, counter-clockwise front. The light pass then
 * reads them when the uploaded scene's shadow_type is LUZ_SHADOW_MAP. */
luz_status luz_frame_render_shadow_maps(luz_ctx* ctx, luz_frame* frame, const luz_tlas* tlas,
                                        const luz_shadow_light* lights, uint32_t light_count,
                                        uint32_t resolution);
/* Copies light `light`'s shadow map (faces * resolution^2 floats) to host memory. */
luz_status luz_frame_read_shadow_map(luz_ctx* ctx, luz_frame* frame, uint32_t light, float* dst, size_t bytes);
/* Primary-ray G-buffer: the raster opaque pass (source/Shaders/opaque.vert:21-31,
 * opaque.frag:21-58; main.cpp:242-258) as closest-hit rays through pixel centres.
 * Texture maps are sampled at the hit's interpolated texcoord; a model with a colour
 * map is alpha-tested per hit (opaque.frag's discard below 0.5), so the ray goes on
 * to the surface behind. Each 8x8 tile traces only the TLAS leaves its corner-ray
 * cone keeps (lists built per call from the TLAS's last build); the planes are those
 * of a full traversal bit for bit. Also records each pixel's hit instance for the
 * visibility pass's short-ray starts. */
luz_status luz_gbuffer_primary(luz_ctx* ctx, luz_frame* frame, const luz_tlas* tlas);
/* Shadow (light.frag:86-109,137-146) and AO (light.frag:111-135) any-hit rays of
 * every lit pixel; writes the visibility bit planes (shadow: 1 = occluded, AO: 1 =
 * miss). Rays start below the TLAS root where that cannot change a bit: an AO ray
 * that stays near its primary-hit instance at that instance's leaf (per-call near
 * lists), a shadow ray at the leaves its 32-ray group's capsule reaches (per-call
 * beam lists). By default a shadow sample keeps bit 0 without a ray when the light pass's
 * term of its light cannot depend on the shadow factor (light.frag:209-226 adds
 * ((kD * albedo / pi + spec) * radiance) * max(dot(N, L), 0) with radiance =
 * ((color * intensity) * attenuation) * (1 - shadow)): (a) max(dot(N, L), 0) is 0 or
 * NaN (the light is behind the surface), or (b) every channel of (color * intensity)
 * * attenuation is +-0 (outside a spot light's cone, a black light). The light pass
 * output is then the one of tracing every ray, but the exported bit planes are not
 * light.frag's per-ray results for those samples; luz_frame_set_shadow_cull(frame, 0)
 * traces every sample as light.frag does. */
luz_status luz_trace_visibility(luz_ctx* ctx, luz_frame* frame, const luz_tlas* tlas,
                                int32_t frame_index);
/* enable != 0 (the default): leave out the shadow rays of conditions (a) and (b) above;
 * 0: trace every shadow sample, so that LUZ_PLANE_SHADOW_BITS holds light.frag's
 * per-ray hit results. */
luz_status luz_frame_set_shadow_cull(luz_frame* frame, int32_t enable);
/* The same trace with per-ray work counters (a separate kernel build, for
 * roofline accounting): out[0] rays traversed, out[1] TLAS node visits, out[2] BLAS
 * node visits, out[3] triangle tests, out[4] instance leaves reached (entered or
 * rejected by the bounding-sphere test). Rays with nothing to
 * trace are not counted: a shadow ray left out by the cull above, a ray with a
 * non-finite origin or direction or tMin > tMax (AO: recorded as a miss). */
luz_status luz_trace_visibility_stats(luz_ctx* ctx, luz_frame* frame, const luz_tlas* tlas,
                                      int32_t frame_index, uint64_t out[5]);
/* Per-pixel AO value (mean of the miss bits) into LUZ_PLANE_AO. */
luz_status luz_ao_resolve(luz_ctx* ctx, luz_frame* frame);
/* Number of lit pixels (length(N) != 0) of the last G-buffer pass. */
luz_status luz_frame_lit_count(luz_ctx* ctx, luz_frame* frame, uint32_t* count);
/* DeferredRenderer::LightPass (source/Graphics/DeferredRenderer.cpp:324-345) running
 * light.frag main (light.frag:171-235) over the G-buffer and visibility planes.
 * LUZ_LIGHT_PASS_PLAIN: shadow factors and AO from the bit planes, as light.frag.
 * LUZ_LIGHT_PASS_DENOISED_AO: AO from LUZ_PLANE_AO_DENOISED, shadows from the bits.
 * LUZ_LIGHT_PASS_DENOISED: the frame from the denoiser's output (run luz_denoise
 * first): ambient * AO + U * R + emission per channel, where U is the unshadowed
 * direct light (LUZ_PLANE_UNSHADOWED), R the filtered shadow ratio and AO the filtered
 * AO (LUZ_PLANE_DENOISED). Unlit pixels keep the background colour that the G-buffer
 * pass's lit-pixel compaction wrote (light.frag:178-181). */
#define LUZ_LIGHT_PASS_PLAIN 0
#define LUZ_LIGHT_PASS_DENOISED_AO 1
#define LUZ_LIGHT_PASS_DENOISED 2
luz_status luz_light_pass(luz_ctx* ctx, luz_frame* frame, int32_t mode);
/* One whole frame: TLAS build, primary G-buffer, visibility, light pass. */
luz_status luz_render_frame(luz_ctx* ctx, luz_frame* frame, luz_tlas* tlas,
                            const luz_instance* instances, uint32_t instance_count,
                            int32_t frame_index);
/* Temporal anti-aliasing of the light image (taa.comp, dispatched by
 * DeferredRenderer::TAAPass, DeferredRenderer.cpp:425-445): reprojects last frame's
 * output by the depth-derived motion (SceneBlock prevViewProj / jitter / prevJitter
 * of the uploaded scene), clips it to the 3x3 neighbourhood and blends with
 * anti-flicker weights. reconstruct != 0: Mitchell-weighted 3x3 source (the scene's
 * taaReconstruct). Writes LUZ_PLANE_TAA, which is also the next call's history (the
 * reference's SwapLightHistory, main.cpp:310). The history starts at zero. */
luz_status luz_taa(luz_ctx* ctx, luz_frame* frame, int32_t reconstruct);
luz_status luz_taa_reset(luz_ctx* ctx, luz_frame* frame);
/* Compose pass (present.frag, DeferredRenderer::ComposePass, DeferredRenderer.cpp:347-369)
 * into LUZ_PLANE_COMPOSE, the reference's BGRA8 compose image, headless: image_type 0
 * = ACES tone-mapped light (source 0: LUZ_PLANE_LIGHT, 1: LUZ_PLANE_TAA), 1 albedo,
 * 2 normal, 3 material, 4 emission, 5 linearised depth, 6 all six in a 3x2 grid. The
 * debug-line overlay is empty. */
luz_status luz_compose(luz_ctx* ctx, luz_frame* frame, int32_t source, int32_t image_type);
/* Luminance histogram of the light (source 0) or TAA (1) image and its average
 * (histogram.comp, histogramAverage.comp with DeferredRenderer.cpp:447-466's constants:
 * 256 bins of log2 luminance over [-10, 2]). The bins are exact counts; the
 * reference's shader zeroes the global bins from every workgroup, which races, and
 * stores the weighted bin sum where its average belongs — here the weighted sum, the
 * weighted log average, the average luminance and the luminance adapted from the
 * previous call over delta_time are all returned. */
typedef struct luz_histogram {
    uint32_t bins[256];
    float weighted_sum;
    float log_average;
    float average_luminance;
    float adapted_luminance;
} luz_histogram;
luz_status luz_luminance_histogram(luz_ctx* ctx, luz_frame* frame, int32_t source, float delta_time,
                                   luz_histogram* out);
/* Size in bytes of one plane of this frame (LUZ_PLANE_*). */
size_t luz_frame_plane_bytes(const luz_frame* frame, int32_t plane);
/* Device→host copy of a plane. */
luz_status luz_frame_read(luz_ctx* ctx, luz_frame* frame, int32_t plane, void* host_dst,
                          size_t bytes);
/* Host→device copy into a plane (e.g. to run the light pass on a given G-buffer). */
luz_status luz_frame_write(luz_ctx* ctx, luz_frame* frame, int32_t plane,
                           const void* host_src, size_t bytes);
/* Device pointer of a plane (for zero-copy interop), NULL on error. */
void* luz_frame_plane_device_ptr(luz_frame* frame, int32_t plane);

/* ------------------------------------------------------------------ batches
 * Many independent scenes of uneven size as one unit (no counterpart in the
 * reference, which renders one scene per frame). A render runs, by default, ONE
 * persistent launch (the frame kernel) over every scene: the per-frame TLAS builds,
 * the clearing of the hit/miss planes, the G-buffer passes with their lit-pixel lists,
 * the shadow/AO traversal of all scenes' rays from one work counter, and the light
 * passes; work items are handed out by tickets and wait only on items handed out
 * before them, each wait bounded (LUZ_DEV_BATCH_QUEUE when one gives up). The meshes'
 * BLASes are built before, once, by luz_blas_build_batch (the reference builds them
 * once at load, GPUScene.cpp:108-138). The frame kernel takes scenes of up to 4096
 * instances and 688 lights; a batch with a larger scene renders staged (every TLAS
 * build, G-buffer and light pass its own launch around one visibility launch over all
 * scenes), which luz_batch_set_fused(ctx, b, 0) also selects. Both forms give the same
 * planes bit for bit. Scene constants and instances are uploaded / packed once at
 * creation (the arrays may be freed after luz_batch_create); luz_batch_capture records
 * a render as one CUDA graph that luz_batch_replay launches; luz_batch_autotune picks
 * the traversal launch shape (ray-batch refill size, steps between refills, CTAs per
 * SM) by timing the batch's own launch. */
typedef struct luz_batch luz_batch;
typedef struct luz_batch_scene {
    const luz_instance* instances;
    uint32_t instance_count;
    const luz_scene* scene;
    const luz_light* lights;
    uint32_t light_count;
    const luz_model* models;
    uint32_t model_count;
    uint32_t width, height;
} luz_batch_scene;
luz_status luz_batch_create(luz_ctx* ctx, uint32_t count, const luz_batch_scene* scenes, luz_batch** out);
void luz_batch_destroy(luz_batch* b);
uint32_t luz_batch_count(const luz_batch* b);
/* The frame of scene i (planes readable with luz_frame_read). */
luz_frame* luz_batch_frame(luz_batch* b, uint32_t i);
luz_status luz_batch_render(luz_ctx* ctx, luz_batch* b, int32_t frame_index);
/* A render with the counting visibility kernel: out[0..4] as luz_trace_visibility_stats. */
luz_status luz_batch_stats(luz_ctx* ctx, luz_batch* b, int32_t frame_index, uint64_t out[5]);
/* Records one render (on the context's explicit stream) into a CUDA graph. */
luz_status luz_batch_capture(luz_ctx* ctx, luz_batch* b, int32_t frame_index);
luz_status luz_batch_replay(luz_ctx* ctx, luz_batch* b);
luz_status luz_batch_autotune(luz_ctx* ctx, luz_batch* b, uint32_t reps, luz_vis_tuning* chosen,
                              float* best_ms);
/* on = 1: renders run the frame kernel (LUZ_ERR_LIMIT when a scene does not fit it);
 * on = 0: staged launches. Drops a captured graph. */
luz_status luz_batch_set_fused(luz_ctx* ctx, luz_batch* b, int32_t on);
/* 1 when the batch renders with the frame kernel. */
int32_t luz_batch_fused(const luz_batch* b);

/* ------------------------------------------------------------------ denoiser
 * Learned kernel-predicting denoiser of the 1-sample shadow and AO terms; no
 * counterpart in the reference, which integrates them with lightSamples shadow rays
 * per light (light.frag:86-109) and aoSamples AO rays (light.frag:111-135) per pixel.
 *
 * Its input is the split of the direct light (luz_denoise_features): per lit pixel the
 * shadowed sum S of light.frag's light loop (r, g, b) with the AO value
 * (LUZ_PLANE_SIGNAL), and the same sum U with every shadow factor 0 (r, g, b) with
 * the unoccluded fraction of all the pixel's shadow samples (LUZ_PLANE_UNSHADOWED). One predicted 7x7 kernel w filters both
 * terms: AO' = sum(w AO) / sum(w), and per channel the ratio estimator
 * R = sum(w S) / sum(w U) (1 where sum(w U) = 0), so that neighbours count by their
 * unshadowed light. The frame is then ambient * AO' + U * R + emission
 * (luz_light_pass with LUZ_LIGHT_PASS_DENOISED): the material and light detail of U
 * stay unfiltered.
 *
 * Per pixel an MLP 72 -> 64 -> 64 -> 64 -> 49 (BF16 tensor cores, FP32 accumulation)
 * reads 8 channels over a 3x3 neighbourhood (noisy AO, unoccluded shadow fraction, normal,
 * relative depth, roughness, albedo luminance) and predicts the softmax weights of the
 * 7x7 kernel. Parameters: LUZ_DENOISER_PARAMS FP32 values, row-major [out][in]
 * weights then biases per layer: W1[64][72] b1[64] W2[64][64] b2[64] W3[64][64]
 * b3[64] W4[49][64] b4[49]. Training loss per pixel: sum over the outputs (R r, g, b
 * and AO') of weight x (y - t)^2, mean over the batch; the weights come with the
 * batch, else they are the shadow weight w (1/3 unless set,
 * luz_denoiser_set_shadow_weight) for the ratio outputs and 1 for AO. */
#define LUZ_DENOISER_PARAMS 16177
typedef struct luz_denoiser luz_denoiser;
/* A batch of images in device memory: features (LUZ_PLANE_FEATURES layout),
 * distances (LUZ_PLANE_LIN_DEPTH), the noisy split (LUZ_PLANE_SIGNAL and
 * LUZ_PLANE_UNSHADOWED layouts: 4 floats per pixel each), for training the target
 * (shadow ratio r, g, b and AO per pixel) and optionally a per-pixel loss weight of
 * each output (4 floats per pixel; NULL = the shadow weight for the ratio outputs, 1
 * for AO); `images` images of width x height stored one after the other. */
typedef struct luz_denoise_batch {
    const void* features;
    const float* lin_depth;
    const float* noisy;
    const float* unshadowed;
    const float* target;
    const float* weight;
    uint32_t width, height, images;
} luz_denoise_batch;
luz_status luz_denoiser_create(luz_ctx* ctx, uint64_t seed, luz_denoiser** out);
void luz_denoiser_destroy(luz_denoiser* d);
/* Loss weight w of each shadow-ratio output in training (the AO output weighs 1). */
luz_status luz_denoiser_set_shadow_weight(luz_ctx* ctx, luz_denoiser* d, float weight);
/* Sets / reads the FP32 parameters (resets the Adam moments). */
luz_status luz_denoiser_set_weights(luz_ctx* ctx, luz_denoiser* d, const float* params);
luz_status luz_denoiser_get_weights(luz_ctx* ctx, luz_denoiser* d, float* params);
/* Computes the network inputs of a traced frame: the split of the direct light
 * (LUZ_PLANE_SIGNAL, LUZ_PLANE_UNSHADOWED), then features, distances and the noisy AO
 * (LUZ_PLANE_AO); background pixels get zeros. */
luz_status luz_denoise_features(luz_ctx* ctx, luz_frame* frame);
/* Inputs + network + filter over the frame's lit pixels (length(N) != 0): writes
 * LUZ_PLANE_DENOISED (R r, g, b and AO') and its AO channel to LUZ_PLANE_AO_DENOISED;
 * background pixels receive 0. */
luz_status luz_denoise(luz_ctx* ctx, luz_denoiser* d, luz_frame* frame);
/* The network + filter over every pixel of a batch into d_out (4 floats per pixel,
 * W x H x images); pixels with lin_depth <= 0 receive 0. Agrees bit for bit with
 * luz_denoise on the same planes. */
luz_status luz_denoise_batch_infer(luz_ctx* ctx, luz_denoiser* d, const luz_denoise_batch* b, float* d_out);
/* The training loss against `target` and its gradient (host array of
 * LUZ_DENOISER_PARAMS, may be NULL); deterministic. */
luz_status luz_denoiser_gradient(luz_ctx* ctx, luz_denoiser* d, const luz_denoise_batch* b, float* grad,
                                 float* loss);
/* One Adam step (beta 0.9/0.999, eps 1e-8) on the batch; loss may be NULL. */
luz_status luz_denoiser_train_step(luz_ctx* ctx, luz_denoiser* d, const luz_denoise_batch* b, float lr,
                                   float* loss);

#ifdef __cplusplus
}
#endif
#endif /* LUZ_GB300_H */
