// lightpass.cu — the deferred light pass: light.frag main (light.frag:171-235) over
// the G-buffer planes and the visibility bit planes. Thread t shades the t-th lit
// pixel of the compacted list the G-buffer pass wrote (world position and normal;
// every lane of a warp runs the same light loop). The pass that compacted that list
// wrote the background colour of the unlit pixels.
#include <cstring>

#include "lightpass.cuh"

namespace luz {

template <int kMode>
__global__ void __launch_bounds__(256) light_pass_kernel(LightParams P) {
    extern __shared__ luz_light s_lights[];
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t lit = *P.lit_count;
    // the background (light.frag:178-181) was written by the lit-list pass
    if (blockIdx.x * blockDim.x >= lit) return;   // no lit pixel in this block
    for (uint32_t i = threadIdx.x; i < P.light_count; i += blockDim.x) s_lights[i] = P.lights[i];
    __syncthreads();
    if (t >= lit) return;
    light_pass_pixel<kMode>(P, s_lights, t);
}

// AO value per pixel (mean of the miss bits; 0 for background pixels).
__global__ void __launch_bounds__(256) ao_resolve_kernel(const float4* normal, const uint32_t* ao_bits,
                                                         uint32_t words, uint32_t samples,
                                                         uint32_t pixels, float* ao) {
    uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= pixels) return;
    float4 nn = normal[pix];
    if (length(V3{nn.x, nn.y, nn.z}) == 0.0f) { ao[pix] = 0.0f; return; }
    if (samples == 0) { ao[pix] = 1.0f; return; }
    uint32_t misses = 0;
    for (uint32_t s = 0; s < samples; ++s) misses += bit_at(ao_bits, s, words, pix);
    ao[pix] = (float)misses / (float)samples;
}


// Inputs of the light pass of frame f.
LightParams make_light_params(luz_ctx* ctx, luz_frame* f) {
    LightParams P;
    P.surf = f->surf;
    P.surf_mat = f->surf_mat;
    P.lit_count = f->lit_count;
    P.albedo = f->albedo;
    P.normal = f->normal;
    P.material = f->material;
    P.emission = f->emission;
    P.shadow_bits = f->shadow_bits;
    P.ao_bits = f->ao_bits;
    P.ao_denoised = f->ao_denoised;
    P.denoised = f->denoised;
    P.signal = f->signal;
    P.unshadowed = f->unshadowed;
    P.lights = f->d_lights;
    P.light_slot = f->d_light_slot;
    P.light_count = f->light_count;
    P.words = f->words;
    P.ao_samples = f->ao_samples;
    P.shadow_type = f->h_scene.shadow_type;
    P.shadow_lights = f->d_shadow_lights;
    P.shadow_count = f->shadow_light_count;
    memcpy(P.cam, f->h_scene.cam_pos, 12);
    memcpy(P.ambient, f->h_scene.ambient_light_color, 12);
    P.ambient_intensity = f->h_scene.ambient_light_intensity;
    P.width = f->width;
    P.height = f->height;
    P.out = f->light;
    P.srgb_lut = ctx->d_srgb_lut;
    return P;
}

luz_status launch_light_pass(luz_ctx* ctx, luz_frame* f, int mode) {
    if (mode < kPlain || mode > kCompose) return set_error(ctx, LUZ_ERR_INVALID, "unknown light pass mode");
    luz_status st = ensure_lit_list(ctx, f);
    if (st != LUZ_OK) return st;
    LightParams P = make_light_params(ctx, f);
    size_t smem = (size_t)f->light_count * sizeof(luz_light);
    void (*kernels[4])(LightParams) = {light_pass_kernel<kPlain>, light_pass_kernel<kDenoisedAo>,
                                       light_pass_kernel<kSplit>, light_pass_kernel<kCompose>};
    static DeviceSetup setup[4];   // per kernel: the shared-memory limit above the default 48 KB
    if (smem > 48 * 1024) {
        st = device_setup(setup[mode], setup_generation(), smem, [&]() -> luz_status {
            LUZ_CUDA(ctx, cudaFuncSetAttribute(kernels[mode], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            return LUZ_OK;
        });
        if (st != LUZ_OK) return st;
    }
    uint32_t blocks = (f->pixels + 255) / 256;
    prof_begin(ctx, LUZ_KERNEL_LIGHT_PASS);
    kernels[mode]<<<blocks, 256, smem, ctx->stream>>>(P);
    prof_end(ctx);
    LUZ_LAUNCHED(ctx, "light_pass_kernel");
    return LUZ_OK;
}

luz_status launch_ao_resolve(luz_ctx* ctx, luz_frame* f) {
    uint32_t blocks = (f->pixels + 255) / 256;
    ao_resolve_kernel<<<blocks, 256, 0, ctx->stream>>>(f->normal, f->ao_bits, f->words,
                                                      f->ao_samples, f->pixels, f->ao);
    LUZ_LAUNCHED(ctx, "ao_resolve_kernel");
    return LUZ_OK;
}

}  // namespace luz
