// denoise.cu — learned kernel-predicting denoiser of the 1-sample shadow and AO terms
// (no counterpart in the reference renderer): per pixel, 72 features (8 channels over
// a 3x3 neighbourhood) → 64 → 64 → 64 (ReLU) → 49 logits → softmax → one 7x7 kernel
// that filters the AO and, as the ratio sum(w S) / sum(w U), the shadowed over the
// unshadowed direct light.
//
// BF16 tcgen05 matrix products with FP32 accumulators in tensor memory, operands in
// shared memory in the K-major no-swizzle core-matrix layout. Inference: a block per
// SM, warpgroups with a 128-pixel tile each (thread = pixel row). Training: one
// persistent kernel runs forward, backward and the weight-gradient products over fixed
// pixel tiles; every block accumulates its weight gradients in tensor memory in a
// fixed tile order, writes one partial, and a second kernel sums the partials in block
// order — the gradient is deterministic. Adam keeps FP32 master weights.
//
// Feature channels per pixel: 0 noisy AO, 1 unoccluded fraction of the shadow
// samples, 2-4 normal, 5 depth relative to the centre pixel
// ((d_q - d_p)/d_p, clamped to [-1,1]), 6 roughness, 7 albedo luminance.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "internal.cuh"

namespace luz {
namespace dn {

constexpr int kParams = 16177;
constexpr int oW1 = 0, ob1 = 4608, oW2 = 4672, ob2 = 8768, oW3 = 8832, ob3 = 12928, oW4 = 12992, ob4 = 16128;
// packed BF16 weights (elements), n-major with padded k strides; the kernels copy them
// into the core-matrix layout
constexpr int sW1 = 88, sW = 72;
constexpr int pW1 = 0;
constexpr int pW2 = pW1 + 64 * sW1;
constexpr int pW3 = pW2 + 64 * sW;
constexpr int pW4 = pW3 + 64 * sW;
constexpr int pW2T = pW4 + 56 * sW;     // transposed copies for the backward pass: [in][out]
constexpr int pW3T = pW2T + 64 * sW;
constexpr int pW4T = pW3T + 64 * sW;
constexpr int pEnd = pW4T + 64 * sW;
constexpr int kBias = 64 + 64 + 64 + 56;   // b1 | b2 | b3 | b4 (padded)

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

// ---------------------------------------------------------------- features
struct FeatParams {
    const uint32_t* albedo;
    const float4* normal;
    const uint32_t* material;
    const float* depth;
    uint32_t width, height;
    float inverse_proj[16], inverse_view[16];
    float cam[3];
    uint4* feat;       // 8 x bf16 per pixel
    float* lin_depth;  // distance to the camera (0 = background)
    float* ao;         // noisy AO value
    float* denoised;   // if set: 0 written here for background pixels (the denoiser skips them)
    float4* denoised4; // if set: the same for the filtered plane
    float4* signal;    // read at lit pixels (written by the split pass), zeroed at background pixels
    float4* unshadowed;
    uint32_t* list;    // if set: lit pixels appended (x | y << 16), row-major within a block
    uint32_t* list_count;
};

__constant__ float c_lin_lut[256];   // pow(i/255, 2.2)

// Channels 0 and 1 come from the split pass: the AO value and the unoccluded
// fraction of all the pixel's shadow samples.
__global__ void __launch_bounds__(256) features_kernel(FeatParams F) {
    __shared__ uint32_t s_warp[8];
    __shared__ uint32_t s_base;
    const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t x = pix % F.width, y = pix / F.width;
    const bool inside = pix < F.width * F.height;
    float4 n = inside ? F.normal[pix] : make_float4(0.f, 0.f, 0.f, 0.f);
    const bool lit = inside && !(length(V3{n.x, n.y, n.z}) == 0.0f);
    if (F.list) {   // block-aggregated append, in pixel order within the block
        const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        const uint32_t mask = __ballot_sync(0xFFFFFFFFu, lit);
        if (lane == 0) s_warp[warp] = __popc(mask);
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t t = 0;
            for (int w = 0; w < 8; ++w) { const uint32_t c = s_warp[w]; s_warp[w] = t; t += c; }
            s_base = t ? atomicAdd(F.list_count, t) : 0u;
        }
        __syncthreads();
        if (lit) F.list[s_base + s_warp[warp] + __popc(mask & ((1u << lane) - 1u))] = x | (y << 16);
    }
    if (!inside) return;
    if (!lit) {
        F.feat[pix] = make_uint4(0, 0, 0, 0);
        F.lin_depth[pix] = 0.0f;
        F.ao[pix] = 0.0f;
        const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
        F.signal[pix] = z4;
        F.unshadowed[pix] = z4;
        if (F.denoised) F.denoised[pix] = 0.0f;
        if (F.denoised4) F.denoised4[pix] = z4;
        return;
    }
    const uint32_t a8 = F.albedo[pix], m8 = F.material[pix];
    const float depth = F.depth[pix];
    const float ao = F.signal[pix].w;
    const float shadow = F.unshadowed[pix].w;   // unoccluded shadow fraction of the split pass
    float lum = 0.2127f * c_lin_lut[a8 & 0xFF] + 0.7152f * c_lin_lut[(a8 >> 8) & 0xFF] +
                0.0722f * c_lin_lut[(a8 >> 16) & 0xFF];
    float rough = (float)(m8 & 0xFF) / 255.0f;
    V3 p = depth_to_world(F.inverse_proj, F.inverse_view, pixel_uv(x, F.width), pixel_uv(y, F.height), depth);
    float d = length(p - V3{F.cam[0], F.cam[1], F.cam[2]});
    uint4 v;
    v.x = pack2(ao, shadow);
    v.y = pack2(n.x, n.y);
    v.z = pack2(n.z, 0.0f);
    v.w = pack2(rough, lum);
    F.feat[pix] = v;
    F.lin_depth[pix] = d;
    F.ao[pix] = ao;
}

// ---------------------------------------------------------------- shared pieces
struct ImageGeom {
    uint32_t width, height, pixels;   // one image
    uint32_t images;
};

// Depth of a neighbour relative to the centre, (d_q - d_p) / d_p clamped to [-1, 1],
// from the centre's reciprocal.
__device__ __forceinline__ float relative_depth(float dq, float dc, float inv_dc) {
    return fminf(fmaxf((dq - dc) * inv_dc, -1.0f), 1.0f);
}

// Filtered shadow ratio of one channel: sum(w S) / sum(w U); 1 where sum(w U) = 0 (no
// neighbour receives direct light in that channel: the pixel's own U is 0 then too).
__device__ __forceinline__ float filtered_ratio(float ws, float wu) {
    return wu > 0.0f ? fminf(fmaxf(ws / wu, 0.0f), 1.0f) : 1.0f;
}

// Tap k of the 7x7 filter around pixel (x, y) of image img (image-clamped); zeros when
// !ok or k >= 49.
__device__ __forceinline__ float4 signal_tap(const float4* __restrict__ sig, const ImageGeom& G, bool ok,
                                             uint32_t img, int x, int y, int k) {
    if (!ok || k >= 49) return make_float4(0.f, 0.f, 0.f, 0.f);
    const int qx = min(max(x + k % 7 - 3, 0), (int)G.width - 1);
    const int qy = min(max(y + k / 7 - 3, 0), (int)G.height - 1);
    return __ldg(sig + img * G.pixels + (uint32_t)qy * G.width + (uint32_t)qx);
}

// ---------------------------------------------------------------- inference
struct InferParams {
    const __nv_bfloat16* wpack;
    const float* bias;
    const uint4* feat;
    const float* lin_depth;
    const float4* sig;       // noisy (shadowed direct light S r, g, b, AO)
    const float4* uns;       // unshadowed direct light U (r, g, b, -)
    ImageGeom G;
    float4* out;             // filtered shadow ratio sum(w S) / sum(w U) (r, g, b) and AO
    float* out_ao;           // if set: its AO channel as well
    // optional pixel list (one image): x | y << 16 per entry, the count in *list_count;
    // only the listed pixels are written
    const uint32_t* list;
    const uint32_t* list_count;
};

// ---------------------------------------------------------------- inference on tcgen05
// The four layers of a 128-pixel tile as tcgen05.mma products (M = 128 pixels, N = 64,
// BF16 operands, FP32 accumulator in tensor memory): the activation tile A [128 x K]
// and the weights B [64 x K] sit in shared memory, K-major in the no-swizzle layout of
// 8-row x 16-byte core matrices ((r / 8) * K/8 + k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2;
// one thread issues the K/16 products of a layer and commits them to an mbarrier, then
// every thread reads its pixel's row of the accumulator (tcgen05.ld, lane = pixel),
// adds the bias, applies ReLU, rounds to BF16 and writes the row back as the next A.
// The last layer's 49 logits go through the softmax and 7x7 filter in registers.
//
// A block holds the weights once and kTcGroups warpgroups, each with its own tile,
// A buffer, 64 accumulator columns, mbarrier and named barrier: while one group waits
// for its products the others gather, or run their epilogues.
constexpr int kTcGroups = 4;                    // warpgroups (tiles in flight) per block
constexpr int kTcThreads = 128 * kTcGroups;
constexpr uint32_t kTcCols = 64;                // accumulator columns of one group (N)
constexpr uint32_t kTcAlloc = 256;              // power of two >= kTcGroups * kTcCols
constexpr int kTcW1 = 0, kTcW2 = kTcW1 + 64 * 80 * 2, kTcW3 = kTcW2 + 64 * 64 * 2, kTcW4 = kTcW3 + 64 * 64 * 2;
constexpr int kTcABytes = 128 * 80 * 2;
constexpr int kTcA = kTcW4 + 64 * 64 * 2, kTcBias = kTcA + kTcGroups * kTcABytes, kTcBar = kTcBias + kBias * 4;
constexpr int kTcSmem = kTcBar + 8 * kTcGroups + 16;
constexpr int kTcBlocksPerSm = 1;
static_assert(kTcBlocksPerSm * kTcAlloc <= 512, "tensor-memory columns per SM");
static_assert(kTcGroups * kTcCols <= kTcAlloc, "groups must fit in the allocation");
static_assert(kTcBlocksPerSm * (kTcSmem + 1024) <= 232448, "blocks per SM must fit in shared memory");
constexpr uint32_t kTcWaitCap = 1u << 20;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ uint32_t core_offset(uint32_t r, uint32_t kb, uint32_t kblocks) {
    return ((r >> 3) * kblocks + kb) * 128u + (r & 7u) * 16u;
}
// Shared-memory matrix descriptor, no swizzle: start, leading (K) and stride (8-row)
// byte offsets, descriptor version 1.
__device__ __forceinline__ uint64_t umma_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}
// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major,
// N = 64, M = 128.
constexpr uint32_t kTcIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((kTcCols >> 3) << 17) | ((128u >> 4) << 24);

// One layer: D[tmem] = A[128 x 16*ksteps] * W^T, issued by the calling thread.
__device__ __forceinline__ void tc_layer(uint32_t tmem, uint32_t a_addr, uint32_t w_addr, int ksteps) {
    const uint32_t kblocks = (uint32_t)ksteps * 2u;
    for (int s = 0; s < ksteps; ++s) {
        const uint64_t da = umma_desc(a_addr + (uint32_t)s * 256u, 128u, kblocks * 128u);
        const uint64_t db = umma_desc(w_addr + (uint32_t)s * 256u, 128u, kblocks * 128u);
        asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                     "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
                     :: "r"(tmem), "l"(da), "l"(db), "r"(kTcIdesc), "r"(s > 0 ? 1u : 0u));
    }
}

// Waits (bounded) for the mbarrier phase; false when the cap ran out.
__device__ __forceinline__ bool tc_wait(uint32_t bar, uint32_t phase) {
    uint32_t done = 0;
    for (uint32_t it = 0; it < kTcWaitCap && !done; ++it)
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}\n" : "=r"(done) : "r"(bar), "r"(phase));
    return done != 0;
}

// 16 accumulator columns of this thread's lane.
__device__ __forceinline__ void tc_load16(uint32_t taddr, float v[16]) {
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

// Barrier of one warpgroup (named barrier 1 + group; 0 is the block's).
__device__ __forceinline__ void group_sync(uint32_t group) {
    asm volatile("bar.sync %0, 128;" :: "r"(group + 1u) : "memory");
}

// Issues a layer from the group's first thread after the group's shared-memory writes
// and accumulator reads, commits it to the group's mbarrier, and every thread waits
// (bounded) for the products. A thread whose wait runs out raises the status and waits
// no more from then on (its results are then meaningless, but every barrier is still
// met and every access stays in bounds); `failed` carries that across layers.
__device__ __forceinline__ void tc_run_layer(uint32_t group, uint32_t tmem, uint32_t a_addr, uint32_t w_addr,
                                             int ksteps, uint32_t bar, uint32_t& phase, bool& failed,
                                             uint32_t* status) {
    asm volatile("fence.proxy.async.shared::cta;");
    asm volatile("tcgen05.fence::before_thread_sync;");
    group_sync(group);
    asm volatile("tcgen05.fence::after_thread_sync;");
    if ((threadIdx.x & 127u) == 0) {
        tc_layer(tmem, a_addr, w_addr, ksteps);
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(bar));
    }
    if (!failed && !tc_wait(bar, phase)) {
        atomicOr(status, (uint32_t)LUZ_DEV_MMA_WAIT);
        failed = true;
    }
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;");
}

// relu(lo + b.x), relu(hi + b.y) rounded to BF16 and packed (lo in the low half): one
// packed FP32 add and one converting ReLU (rounding commutes with the clamp at 0).
__device__ __forceinline__ uint32_t bias_relu_bf16x2(float lo, float hi, float2 b) {
    uint32_t d;
    asm("{\n\t.reg .b64 x, y, z;\n\t.reg .f32 l, h;\n\tmov.b64 x, {%1, %2};\n\tmov.b64 y, {%3, %4};\n\t"
        "add.rn.f32x2 z, x, y;\n\tmov.b64 {l, h}, z;\n\tcvt.rn.relu.bf16x2.f32 %0, h, l;\n\t}\n"
        : "=r"(d) : "f"(lo), "f"(hi), "f"(b.x), "f"(b.y));
    return d;
}

// Bias + ReLU + BF16 of this thread's 64 accumulator columns into row `row` of A (K = 64).
__device__ __forceinline__ void tc_relu_to_a(uint32_t tmem_lane, const float* sbias, unsigned char* a, uint32_t row) {
    const float2* b2 = reinterpret_cast<const float2*>(sbias);
#pragma unroll
    for (int c0 = 0; c0 < 64; c0 += 16) {
        float v[16];
        tc_load16(tmem_lane + (uint32_t)c0, v);
        uint32_t w[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) w[j] = bias_relu_bf16x2(v[2 * j], v[2 * j + 1], b2[c0 / 2 + j]);
        *reinterpret_cast<uint4*>(a + core_offset(row, (uint32_t)c0 / 8u, 8u)) = make_uint4(w[0], w[1], w[2], w[3]);
        *reinterpret_cast<uint4*>(a + core_offset(row, (uint32_t)c0 / 8u + 1u, 8u)) = make_uint4(w[4], w[5], w[6], w[7]);
    }
}

// Packed FP32 pairs (one instruction for both lanes of the pair).
__device__ __forceinline__ float2 add2(float2 a, float2 b) {
    float2 d;
    asm("{\n\t.reg .b64 x, y, z;\n\tmov.b64 x, {%2, %3};\n\tmov.b64 y, {%4, %5};\n\t"
        "add.rn.f32x2 z, x, y;\n\tmov.b64 {%0, %1}, z;\n\t}\n"
        : "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
    float2 d;
    asm("{\n\t.reg .b64 x, y, z, w;\n\tmov.b64 x, {%2, %3};\n\tmov.b64 y, {%4, %5};\n\tmov.b64 z, {%6, %7};\n\t"
        "fma.rn.f32x2 w, x, y, z;\n\tmov.b64 {%0, %1}, w;\n\t}\n"
        : "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return d;
}
__device__ __forceinline__ float exp2_approx(float x) {
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Second pass of the softmax and the 7x7 filter: with w_k = 2^((z_k - m) * log2 e),
// z_k = logit + bias, sums of w_k x the shadowed light S_k (r, g, b) and AO_k (acc),
// of w_k x the unshadowed light U_k (accu, r, g, b) and of w_k (the return value).
// kInterior: every tap of the thread's pixel is inside the image (rows addressed
// directly); otherwise clamped.
template <bool kInterior>
__device__ __forceinline__ float signal_filter(uint32_t tmem_lane, const float2* b4, float b48, float m,
                                               const float4* __restrict__ sig, const float4* __restrict__ uns,
                                               uint32_t base, int x, int y, const ImageGeom& G, float4& acc,
                                               float3& accu) {
    constexpr float kLog2e = 1.4426950408889634f;
    const float2 l2e = make_float2(kLog2e, kLog2e);
    const float nm = -m * kLog2e;
    const float2 nm2 = make_float2(nm, nm);
    uint32_t rows[7];
    int qx[7];
#pragma unroll
    for (int d = 0; d < 7; ++d) {
        if (kInterior) {
            rows[d] = base + (uint32_t)(y + d - 3) * G.width + (uint32_t)(x - 3);
        } else {
            rows[d] = base + (uint32_t)min(max(y + d - 3, 0), (int)G.height - 1) * G.width;
            qx[d] = min(max(x + d - 3, 0), (int)G.width - 1);
        }
    }
    auto at = [&](int k) -> uint32_t { return rows[k / 7] + (uint32_t)(kInterior ? k % 7 : qx[k % 7]); };
    float2 s = make_float2(0.f, 0.f);
    float2 a_xy = make_float2(0.f, 0.f), a_zw = make_float2(0.f, 0.f), u_xy = make_float2(0.f, 0.f);
    float u_z = 0.f;
#pragma unroll
    for (int c0 = 0; c0 < 48; c0 += 16) {
        float v[16];
        tc_load16(tmem_lane + (uint32_t)c0, v);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int k = c0 + 2 * j;
            const float2 t = fma2(add2(make_float2(v[2 * j], v[2 * j + 1]), b4[k / 2]), l2e, nm2);
            const float2 e = make_float2(exp2_approx(t.x), exp2_approx(t.y));
            s = add2(s, e);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const uint32_t q = at(k + h);
                const float4 x4 = __ldg(sig + q), u4 = __ldg(uns + q);
                const float eh = h ? e.y : e.x;
                const float2 e2 = make_float2(eh, eh);
                a_xy = fma2(e2, make_float2(x4.x, x4.y), a_xy);
                a_zw = fma2(e2, make_float2(x4.z, x4.w), a_zw);
                u_xy = fma2(e2, make_float2(u4.x, u4.y), u_xy);
                u_z = fmaf(eh, u4.z, u_z);
            }
        }
    }
    float v[16];
    tc_load16(tmem_lane + 48u, v);
    const float e48 = exp2_approx(fmaf(v[0] + b48, kLog2e, nm));
    const uint32_t q = at(48);
    const float4 x48 = __ldg(sig + q), u48 = __ldg(uns + q);
    acc = make_float4(fmaf(e48, x48.x, a_xy.x), fmaf(e48, x48.y, a_xy.y), fmaf(e48, x48.z, a_zw.x),
                      fmaf(e48, x48.w, a_zw.y));
    accu = make_float3(fmaf(e48, u48.x, u_xy.x), fmaf(e48, u48.y, u_xy.y), fmaf(e48, u48.z, u_z));
    return e48 + s.x + s.y;
}

__global__ void __launch_bounds__(kTcThreads, kTcBlocksPerSm) denoise_infer_tc_kernel(InferParams P, uint32_t* status) {
    extern __shared__ __align__(1024) unsigned char tsm[];
    float* sbias = reinterpret_cast<float*>(tsm + kTcBias);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(tsm + kTcBar + 8 * kTcGroups);
    const uint32_t tid = threadIdx.x, warp = tid >> 5, group = tid >> 7, row = tid & 127u;
    const uint32_t bar = smem_u32(tsm + kTcBar + 8 * group);
    // weights into the core-matrix layout (rows of the packed n-major copies)
    for (uint32_t e = tid; e < 64 * 10; e += kTcThreads) {           // W1: K = 80
        const uint32_t n = e / 10, kb = e % 10;
        *reinterpret_cast<uint4*>(tsm + kTcW1 + core_offset(n, kb, 10)) =
            *reinterpret_cast<const uint4*>(P.wpack + pW1 + n * sW1 + kb * 8);
    }
    for (uint32_t e = tid; e < 64 * 8; e += kTcThreads) {            // W2, W3, W4: K = 64
        const uint32_t n = e / 8, kb = e % 8;
        *reinterpret_cast<uint4*>(tsm + kTcW2 + core_offset(n, kb, 8)) =
            *reinterpret_cast<const uint4*>(P.wpack + pW2 + n * sW + kb * 8);
        *reinterpret_cast<uint4*>(tsm + kTcW3 + core_offset(n, kb, 8)) =
            *reinterpret_cast<const uint4*>(P.wpack + pW3 + n * sW + kb * 8);
        *reinterpret_cast<uint4*>(tsm + kTcW4 + core_offset(n, kb, 8)) =
            n < 56 ? *reinterpret_cast<const uint4*>(P.wpack + pW4 + n * sW + kb * 8) : make_uint4(0, 0, 0, 0);
    }
    for (uint32_t i = tid; i < (uint32_t)kBias; i += kTcThreads) sbias[i] = P.bias[i];
    if (row == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(bar));
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" :: "r"(smem_u32(tslot)),
                     "r"(kTcAlloc));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = *tslot + group * kTcCols;               // this group's columns
    const uint32_t tmem_lane = tmem + (((warp & 3u) * 32u) << 16); // this warp's 32 lanes
    unsigned char* a = tsm + kTcA + group * kTcABytes;
    const uint32_t a_addr = smem_u32(a);
    uint32_t phase = 0;
    bool failed = false;
    const uint32_t total = P.list ? *P.list_count : P.G.pixels * P.G.images;
    const uint32_t tiles = (total + 127) / 128;
    const uint32_t stride = gridDim.x * kTcGroups;
    uint32_t tile = blockIdx.x * kTcGroups + group;
    uint32_t next_xy = (P.list && tile * 128 + row < total) ? P.list[tile * 128 + row] : 0u;
    for (; tile < tiles; tile += stride) {
        // features of pixel `row`: 9 taps of 8 channels (relative depth in channel 5), then 8 zeros
        const uint32_t item = tile * 128 + row;
        const bool has = item < total;
        uint32_t img = 0, gp = 0;
        int x = 0, y = 0;
        if (P.list) {
            x = (int)(next_xy & 0xFFFFu);
            y = (int)(next_xy >> 16);
            gp = (uint32_t)y * P.G.width + (uint32_t)x;
            const uint32_t nitem = item + stride * 128;   // this thread's entry of the next tile
            next_xy = nitem < total ? P.list[nitem] : 0u;
        } else if (has) {
            gp = item;
            img = gp / P.G.pixels;
            const uint32_t local = gp - img * P.G.pixels;
            x = (int)(local % P.G.width);
            y = (int)(local / P.G.width);
        }
        // the centre depth and the 9 taps are loaded without waiting on one another
        // (clamped, always in bounds); background centres get a zero row
        const float dc = has ? P.lin_depth[gp] : 0.0f;
        uint32_t tq[9];
        float td[9];
#pragma unroll
        for (int tap = 0; tap < 9; ++tap) {
            const int qx = min(max(x + tap % 3 - 1, 0), (int)P.G.width - 1);
            const int qy = min(max(y + tap / 3 - 1, 0), (int)P.G.height - 1);
            tq[tap] = img * P.G.pixels + (uint32_t)qy * P.G.width + (uint32_t)qx;
            td[tap] = has ? P.lin_depth[tq[tap]] : 0.0f;
        }
        const bool valid = dc > 0.0f;
        const float inv_dc = valid ? 1.0f / dc : 0.0f;
#pragma unroll
        for (int tap = 0; tap < 9; ++tap) {
            uint4 v = has ? P.feat[tq[tap]] : make_uint4(0, 0, 0, 0);
            const float rel = td[tap] > 0.0f ? relative_depth(td[tap], dc, inv_dc) : 0.0f;
            v.z = (v.z & 0xFFFFu) | (pack2(0.0f, rel) & 0xFFFF0000u);
            if (!valid) v = make_uint4(0, 0, 0, 0);
            *reinterpret_cast<uint4*>(a + core_offset(row, (uint32_t)tap, 10)) = v;
        }
        *reinterpret_cast<uint4*>(a + core_offset(row, 9, 10)) = make_uint4(0, 0, 0, 0);
        tc_run_layer(group, tmem, a_addr, smem_u32(tsm + kTcW1), 5, bar, phase, failed, status);
        tc_relu_to_a(tmem_lane, sbias, a, row);
        tc_run_layer(group, tmem, a_addr, smem_u32(tsm + kTcW2), 4, bar, phase, failed, status);
        tc_relu_to_a(tmem_lane, sbias + 64, a, row);
        tc_run_layer(group, tmem, a_addr, smem_u32(tsm + kTcW3), 4, bar, phase, failed, status);
        tc_relu_to_a(tmem_lane, sbias + 128, a, row);
        tc_run_layer(group, tmem, a_addr, smem_u32(tsm + kTcW4), 4, bar, phase, failed, status);
        // softmax over the 49 logits and the 7x7 filter of the noisy AO
        const float2* b4 = reinterpret_cast<const float2*>(sbias + 192);
        float m = -3.0e38f;
#pragma unroll
        for (int c0 = 0; c0 < 48; c0 += 16) {
            float v[16];
            tc_load16(tmem_lane + (uint32_t)c0, v);
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const float2 z = add2(make_float2(v[2 * j], v[2 * j + 1]), b4[c0 / 2 + j]);
                m = fmaxf(m, fmaxf(z.x, z.y));
            }
        }
        {
            float v[16];
            tc_load16(tmem_lane + 48u, v);
            m = fmaxf(m, v[0] + sbias[192 + 48]);
        }
        const uint32_t base = img * P.G.pixels;
        const bool interior = has && x >= 3 && y >= 3 && x + 3 < (int)P.G.width && y + 3 < (int)P.G.height;
        float4 acc;
        float3 accu;
        const float wsum = __all_sync(0xFFFFFFFFu, interior)
                               ? signal_filter<true>(tmem_lane, b4, sbias[192 + 48], m, P.sig, P.uns, base, x, y,
                                                     P.G, acc, accu)
                               : signal_filter<false>(tmem_lane, b4, sbias[192 + 48], m, P.sig, P.uns, base, x, y,
                                                      P.G, acc, accu);
        if (has) {
            const float4 r = valid ? make_float4(filtered_ratio(acc.x, accu.x), filtered_ratio(acc.y, accu.y),
                                                 filtered_ratio(acc.z, accu.z), acc.w * (1.0f / wsum))
                                   : make_float4(0.f, 0.f, 0.f, 0.f);
            P.out[gp] = r;
            if (P.out_ao) P.out_ao[gp] = r.w;
        }
    }
    if (failed) tc_wait(bar, phase ^ 1u);   // products still in flight before the columns are freed
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(*tslot), "r"(kTcAlloc));
}

// ---------------------------------------------------------------- training
struct TrainParams {
    const __nv_bfloat16* wpack;
    const float* bias;
    const uint4* feat;
    const float* lin_depth;
    const float4* sig;         // noisy (shadowed direct light S r, g, b, AO)
    const float4* uns;         // unshadowed direct light U (r, g, b, -)
    const float4* target;      // many-sample shadow ratio (r, g, b) and AO
    const float4* weight;      // per-pixel loss weight of each output, or null (shadow_weight, AO: 1)
    ImageGeom G;
    float grad_scale;          // 2 / number of pixels (mean squared error)
    float shadow_weight;       // loss weight of each shadow-ratio output (AO: 1)
    float* partial;            // [gridDim.x][kParams]
    float* partial_loss;       // [gridDim.x]
};

// ---------------------------------------------------------------- training on tcgen05
// Forward, backward and the weight gradients of a 128-pixel tile as tcgen05.mma
// products (M = 128, BF16 operands in shared memory, FP32 accumulators in tensor
// memory), one warpgroup per SM, thread p = pixel p of the tile:
//   forward   D = A * W^T for the four layers (A = X, H1, H2, H3; as inference);
//   backward  dH_l = dZ_{l+1} * W_{l+1} (B = the transposed weights W^T, K = outputs);
//   gradients dW_l += dZ_l^T * [H_{l-1} | 1]^T over the tile's pixels (M = outputs,
//             rows 64..127 of A zero; N = 80 with the bias column of ones; K = the 128
//             pixels), accumulated in tensor memory over all tiles of the block.
// Every operand sits in the K-major no-swizzle core-matrix layout of the inference
// kernel; the activations and dZ are written twice by their threads: as a row of the
// next product's A and as a column of the transposed copy (dW's A and B). One
// partial per block in the FP32 parameter layout, summed in block order.
constexpr int kTtW1 = 0;                            // [64 x 80] forward B
constexpr int kTtW2 = kTtW1 + 64 * 80 * 2;          // [64 x 64]
constexpr int kTtW3 = kTtW2 + 64 * 64 * 2;
constexpr int kTtW4 = kTtW3 + 64 * 64 * 2;          // rows >= 49 zero
constexpr int kTtW4T = kTtW4 + 64 * 64 * 2;         // [64 hidden x 64 outputs] backward B
constexpr int kTtW3T = kTtW4T + 64 * 64 * 2;
constexpr int kTtW2T = kTtW3T + 64 * 64 * 2;
constexpr int kTtA = kTtW2T + 64 * 64 * 2;          // [128 x 80] X, then H1, H2, H3
constexpr int kTtXT = kTtA + 128 * 80 * 2;          // [80 x 128] X^T, row 72 ones
constexpr int kTtHT = kTtXT + 80 * 128 * 2;         // 3 x [80 x 128] H^T, row 64 ones
constexpr int kTtDZ = kTtHT + 3 * 80 * 128 * 2;     // [128 x 64] dZ
constexpr int kTtDZT = kTtDZ + 128 * 64 * 2;        // [128 x 128] dZ^T in rows 0..63
constexpr int kTtBias = kTtDZT + 128 * 128 * 2;
constexpr int kTtBar = kTtBias + kBias * 4;
constexpr int kTtSmem = kTtBar + 32;
static_assert(kTtSmem + 1024 <= 232448, "training tile must fit in shared memory");
// tensor-memory columns: forward D, backward dH, dW1..dW4 (80 each)
constexpr uint32_t kTtFwd = 0, kTtDH = 64, kTtDW1 = 128, kTtDW2 = 208, kTtDW3 = 288, kTtDW4 = 368;
constexpr uint32_t kTtAlloc = 512;

__host__ __device__ constexpr uint32_t tc_idesc(uint32_t n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((128u >> 4) << 24);
}

// D[tmem] (+)= A[128 x 16 ksteps] * B[N x 16 ksteps]^T; a / b: shared addresses,
// ka / kb: their core-matrix columns (K / 8).
__device__ __forceinline__ void tc_mma(uint32_t tmem, uint32_t a, uint32_t ka, uint32_t b, uint32_t kb, int ksteps,
                                       uint32_t idesc, bool accumulate) {
    for (int s = 0; s < ksteps; ++s) {
        const uint64_t da = umma_desc(a + (uint32_t)s * 256u, 128u, ka * 128u);
        const uint64_t db = umma_desc(b + (uint32_t)s * 256u, 128u, kb * 128u);
        asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                     "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
                     :: "r"(tmem), "l"(da), "l"(db), "r"(idesc), "r"((s > 0 || accumulate) ? 1u : 0u));
    }
}

// Makes the block's shared-memory writes and tensor-memory reads visible to the
// products that thread 0 issues next.
__device__ __forceinline__ void tt_before_issue() {
    asm volatile("fence.proxy.async.shared::cta;");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
}

// Commits the issued products to the mbarrier and waits for them (bounded; see
// tc_run_layer).
__device__ __forceinline__ void tt_commit_wait(uint32_t bar, uint32_t& phase, bool& failed, uint32_t* status) {
    if (threadIdx.x == 0)
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(bar));
    if (!failed && !tc_wait(bar, phase)) {
        atomicOr(status, (uint32_t)LUZ_DEV_MMA_WAIT);
        failed = true;
    }
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;");
}

// Element (r, k) of a core-matrix tile with kblocks core columns, as a 2-byte offset.
__device__ __forceinline__ uint32_t elem_offset(uint32_t r, uint32_t k, uint32_t kblocks) {
    return core_offset(r, k >> 3, kblocks) + (k & 7u) * 2u;
}

__device__ __forceinline__ void st_bf16(unsigned char* base, uint32_t off, float v) {
    *reinterpret_cast<__nv_bfloat16*>(base + off) = __float2bfloat16(v);
}

// Forward epilogue of layers 1-3: bias + ReLU + BF16 of this thread's 64 accumulator
// columns into row `row` of A (the next layer's input) and column `row` of the
// transposed copy ht; bit j of mask = (h_j > 0).
__device__ __forceinline__ void tt_relu_out(uint32_t tl, const float* sb, unsigned char* a, unsigned char* ht,
                                            uint32_t row, uint64_t& mask) {
    mask = 0;
#pragma unroll
    for (int c0 = 0; c0 < 64; c0 += 16) {
        float v[16];
        tc_load16(tl + (uint32_t)c0, v);
        uint32_t w[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const float lo = fmaxf(v[2 * j] + sb[c0 + 2 * j], 0.0f), hi = fmaxf(v[2 * j + 1] + sb[c0 + 2 * j + 1], 0.0f);
            w[j] = pack2(lo, hi);
            const __nv_bfloat162 q = *reinterpret_cast<const __nv_bfloat162*>(&w[j]);
            *reinterpret_cast<__nv_bfloat16*>(ht + elem_offset((uint32_t)(c0 + 2 * j), row, 16)) = q.x;
            *reinterpret_cast<__nv_bfloat16*>(ht + elem_offset((uint32_t)(c0 + 2 * j + 1), row, 16)) = q.y;
            mask |= (uint64_t)(__bfloat162float(q.x) > 0.0f) << (c0 + 2 * j);
            mask |= (uint64_t)(__bfloat162float(q.y) > 0.0f) << (c0 + 2 * j + 1);
        }
        *reinterpret_cast<uint4*>(a + core_offset(row, (uint32_t)c0 / 8u, 8u)) = make_uint4(w[0], w[1], w[2], w[3]);
        *reinterpret_cast<uint4*>(a + core_offset(row, (uint32_t)c0 / 8u + 1u, 8u)) = make_uint4(w[4], w[5], w[6], w[7]);
    }
}

// Backward epilogue of layers 3-1: dZ = dH * ReLU'(h) of this thread's 64 columns into
// row `row` of dZ (when dz != null) and column `row` of dZ^T.
__device__ __forceinline__ void tt_dz_out(uint32_t tl, uint64_t mask, unsigned char* dz, unsigned char* dzt,
                                          uint32_t row) {
#pragma unroll
    for (int c0 = 0; c0 < 64; c0 += 16) {
        float v[16];
        tc_load16(tl + (uint32_t)c0, v);
        uint32_t w[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const float lo = ((mask >> (c0 + 2 * j)) & 1u) ? v[2 * j] : 0.0f;
            const float hi = ((mask >> (c0 + 2 * j + 1)) & 1u) ? v[2 * j + 1] : 0.0f;
            w[j] = pack2(lo, hi);
            const __nv_bfloat162 q = *reinterpret_cast<const __nv_bfloat162*>(&w[j]);
            *reinterpret_cast<__nv_bfloat16*>(dzt + elem_offset((uint32_t)(c0 + 2 * j), row, 16)) = q.x;
            *reinterpret_cast<__nv_bfloat16*>(dzt + elem_offset((uint32_t)(c0 + 2 * j + 1), row, 16)) = q.y;
        }
        if (dz) {
            *reinterpret_cast<uint4*>(dz + core_offset(row, (uint32_t)c0 / 8u, 8u)) = make_uint4(w[0], w[1], w[2], w[3]);
            *reinterpret_cast<uint4*>(dz + core_offset(row, (uint32_t)c0 / 8u + 1u, 8u)) =
                make_uint4(w[4], w[5], w[6], w[7]);
        }
    }
}

__global__ void __launch_bounds__(128, 1) denoise_train_tc_kernel(TrainParams P, uint32_t* status) {
    extern __shared__ __align__(1024) unsigned char tsm[];
    float* sbias = reinterpret_cast<float*>(tsm + kTtBias);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(tsm + kTtBar + 8);
    const uint32_t tid = threadIdx.x, warp = tid >> 5, row = tid;
    const uint32_t bar = smem_u32(tsm + kTtBar);
    // weights into the core-matrix layout: forward (n-major W) and backward (W^T)
    for (uint32_t e = tid; e < 64 * 10; e += 128) {
        const uint32_t n = e / 10, kb = e % 10;
        *reinterpret_cast<uint4*>(tsm + kTtW1 + core_offset(n, kb, 10)) =
            *reinterpret_cast<const uint4*>(P.wpack + pW1 + n * sW1 + kb * 8);
    }
    for (uint32_t e = tid; e < 64 * 8; e += 128) {
        const uint32_t n = e / 8, kb = e % 8;
        const uint32_t o = core_offset(n, kb, 8);
        *reinterpret_cast<uint4*>(tsm + kTtW2 + o) = *reinterpret_cast<const uint4*>(P.wpack + pW2 + n * sW + kb * 8);
        *reinterpret_cast<uint4*>(tsm + kTtW3 + o) = *reinterpret_cast<const uint4*>(P.wpack + pW3 + n * sW + kb * 8);
        *reinterpret_cast<uint4*>(tsm + kTtW4 + o) =
            n < 56 ? *reinterpret_cast<const uint4*>(P.wpack + pW4 + n * sW + kb * 8) : make_uint4(0, 0, 0, 0);
        *reinterpret_cast<uint4*>(tsm + kTtW4T + o) = *reinterpret_cast<const uint4*>(P.wpack + pW4T + n * sW + kb * 8);
        *reinterpret_cast<uint4*>(tsm + kTtW3T + o) = *reinterpret_cast<const uint4*>(P.wpack + pW3T + n * sW + kb * 8);
        *reinterpret_cast<uint4*>(tsm + kTtW2T + o) = *reinterpret_cast<const uint4*>(P.wpack + pW2T + n * sW + kb * 8);
    }
    for (uint32_t i = tid; i < (uint32_t)kBias; i += 128) sbias[i] = P.bias[i];
    // constant parts: zero dZ^T (rows 64..127 stay zero, rows 49..63 of the last layer
    // too) and the ones / zero rows of the transposed activations
    for (uint32_t i = tid; i < 128 * 128 * 2 / 16; i += 128)
        reinterpret_cast<uint4*>(tsm + kTtDZT)[i] = make_uint4(0, 0, 0, 0);
    for (uint32_t i = tid; i < 128 * 64 * 2 / 16; i += 128)
        reinterpret_cast<uint4*>(tsm + kTtDZ)[i] = make_uint4(0, 0, 0, 0);
    {
        const __nv_bfloat16 one = __float2bfloat16(1.0f), zero = __float2bfloat16(0.0f);
        for (uint32_t k = 72; k < 80; ++k)
            *reinterpret_cast<__nv_bfloat16*>(tsm + kTtXT + elem_offset(k, row, 16)) = k == 72 ? one : zero;
        for (int l = 0; l < 3; ++l)
            for (uint32_t k = 64; k < 80; ++k)
                *reinterpret_cast<__nv_bfloat16*>(tsm + kTtHT + l * 80 * 128 * 2 + elem_offset(k, row, 16)) =
                    k == 64 ? one : zero;
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(bar));
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" :: "r"(smem_u32(tslot)),
                     "r"(kTtAlloc));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = *tslot;
    const uint32_t lane_off = ((warp & 3u) * 32u) << 16;
    unsigned char* a = tsm + kTtA;
    unsigned char* xt = tsm + kTtXT;
    unsigned char* ht[3] = {tsm + kTtHT, tsm + kTtHT + 80 * 128 * 2, tsm + kTtHT + 2 * 80 * 128 * 2};
    unsigned char* dz = tsm + kTtDZ;
    unsigned char* dzt = tsm + kTtDZT;
    const uint32_t a_addr = smem_u32(a), dz_addr = smem_u32(dz), dzt_addr = smem_u32(dzt);
    const uint32_t xt_addr = smem_u32(xt);
    const uint32_t ht_addr[3] = {smem_u32(ht[0]), smem_u32(ht[1]), smem_u32(ht[2])};
    const uint32_t wf[4] = {smem_u32(tsm + kTtW1), smem_u32(tsm + kTtW2), smem_u32(tsm + kTtW3), smem_u32(tsm + kTtW4)};
    const uint32_t wt[3] = {smem_u32(tsm + kTtW2T), smem_u32(tsm + kTtW3T), smem_u32(tsm + kTtW4T)};
    const uint32_t dw_col[4] = {kTtDW1, kTtDW2, kTtDW3, kTtDW4};
    uint32_t phase = 0;
    bool failed = false, accumulated = false;
    float loss = 0.f;
    const uint32_t total = P.G.pixels * P.G.images;
    const uint32_t tiles = (total + 127) / 128;
    for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        // ---- features of pixel `row` (9 taps of 8 channels, relative depth in channel 5)
        const uint32_t gp = tile * 128 + row;
        const bool has = gp < total;
        uint32_t img = 0;
        int x = 0, y = 0;
        if (has) {
            img = gp / P.G.pixels;
            const uint32_t local = gp - img * P.G.pixels;
            x = (int)(local % P.G.width);
            y = (int)(local / P.G.width);
        }
        const float dc = has ? P.lin_depth[gp] : 0.0f;
        const bool valid = dc > 0.0f;
        const float inv_dc = valid ? 1.0f / dc : 0.0f;
#pragma unroll
        for (int tap = 0; tap < 9; ++tap) {
            const int qx = min(max(x + tap % 3 - 1, 0), (int)P.G.width - 1);
            const int qy = min(max(y + tap / 3 - 1, 0), (int)P.G.height - 1);
            const uint32_t q = img * P.G.pixels + (uint32_t)qy * P.G.width + (uint32_t)qx;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (valid) {
                v = P.feat[q];
                const float dq = P.lin_depth[q];
                const float rel = dq > 0.0f ? relative_depth(dq, dc, inv_dc) : 0.0f;
                v.z = (v.z & 0xFFFFu) | (pack2(0.0f, rel) & 0xFFFF0000u);
            }
            *reinterpret_cast<uint4*>(a + core_offset(row, (uint32_t)tap, 10)) = v;
            const uint32_t w4[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                *reinterpret_cast<uint16_t*>(xt + elem_offset((uint32_t)(tap * 8 + 2 * c), row, 16)) =
                    (uint16_t)(w4[c] & 0xFFFFu);
                *reinterpret_cast<uint16_t*>(xt + elem_offset((uint32_t)(tap * 8 + 2 * c + 1), row, 16)) =
                    (uint16_t)(w4[c] >> 16);
            }
        }
        *reinterpret_cast<uint4*>(a + core_offset(row, 9, 10)) = make_uint4(0, 0, 0, 0);
        // ---- forward
        uint64_t mask[3];
        const uint32_t tl = tmem + lane_off;
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            tt_before_issue();
            if (tid == 0) tc_mma(tmem + kTtFwd, a_addr, l == 0 ? 10u : 8u, wf[l], l == 0 ? 10u : 8u, l == 0 ? 5 : 4,
                                 tc_idesc(64), false);
            tt_commit_wait(bar, phase, failed, status);
            if (l < 3) tt_relu_out(tl + kTtFwd, sbias + 64 * l, a, ht[l], row, mask[l]);
        }
        // ---- softmax, filter, loss and dL/dz of the last layer (this thread's pixel)
        const float* b4 = sbias + 192;
        float z[49];
#pragma unroll
        for (int c0 = 0; c0 < 64; c0 += 16) {
            float v[16];
            tc_load16(tl + kTtFwd + (uint32_t)c0, v);
#pragma unroll
            for (int j = 0; j < 16; ++j)
                if (c0 + j < 49) z[c0 + j] = v[j] + b4[c0 + j];
        }
        float m = -3.0e38f;
#pragma unroll
        for (int k = 0; k < 49; ++k) m = fmaxf(m, z[k]);
        float sum = 0.f;
#pragma unroll
        for (int k = 0; k < 49; ++k) {
            z[k] = __expf(z[k] - m);
            sum += z[k];
        }
        const float inv = 1.0f / sum;
        float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
        float3 au = make_float3(0.f, 0.f, 0.f);
#pragma unroll
        for (int k = 0; k < 49; ++k) {
            z[k] *= inv;   // the normalised weight w_k
            const float4 sv = signal_tap(P.sig, P.G, has, img, x, y, k);
            const float4 uv = signal_tap(P.uns, P.G, has, img, x, y, k);
            acc.x += z[k] * sv.x;
            acc.y += z[k] * sv.y;
            acc.z += z[k] * sv.z;
            acc.w += z[k] * sv.w;
            au.x += z[k] * uv.x;
            au.y += z[k] * uv.y;
            au.z += z[k] * uv.z;
        }
        const float4 yv = make_float4(filtered_ratio(acc.x, au.x), filtered_ratio(acc.y, au.y),
                                      filtered_ratio(acc.z, au.z), acc.w);
        const float4 tg = valid ? P.target[gp] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 err = valid ? make_float4(yv.x - tg.x, yv.y - tg.y, yv.z - tg.z, yv.w - tg.w)
                                 : make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 cw = (P.weight && valid) ? P.weight[gp]
                                              : make_float4(P.shadow_weight, P.shadow_weight, P.shadow_weight, 1.0f);
        loss += (cw.w * err.w * err.w + cw.x * err.x * err.x + cw.y * err.y * err.y + cw.z * err.z * err.z) *
                (0.5f * P.grad_scale);
        const float4 dy = make_float4(cw.x * err.x * P.grad_scale, cw.y * err.y * P.grad_scale,
                                      cw.z * err.z * P.grad_scale, cw.w * err.w * P.grad_scale);
        const float3 dq = make_float3(au.x > 0.f ? dy.x / au.x : 0.f, au.y > 0.f ? dy.y / au.y : 0.f,
                                      au.z > 0.f ? dy.z / au.z : 0.f);
        const float3 dr = make_float3(dq.x * yv.x, dq.y * yv.y, dq.z * yv.z);
        float g[49];
        float sdot = 0.f;
#pragma unroll
        for (int k = 0; k < 49; ++k) {
            const float4 sv = signal_tap(P.sig, P.G, has, img, x, y, k);
            const float4 uv = signal_tap(P.uns, P.G, has, img, x, y, k);
            g[k] = dy.w * sv.w + (dq.x * sv.x - dr.x * uv.x) + (dq.y * sv.y - dr.y * uv.y) + (dq.z * sv.z - dr.z * uv.z);
            sdot += z[k] * g[k];
        }
#pragma unroll
        for (int k = 0; k < 64; k += 2) {
            const float lo = k < 49 ? z[k] * (g[k] - sdot) : 0.0f;
            const float hi = k + 1 < 49 ? z[k + 1] * (g[k + 1] - sdot) : 0.0f;
            const uint32_t w = pack2(lo, hi);
            *reinterpret_cast<uint32_t*>(dz + elem_offset(row, (uint32_t)k, 8)) = w;
            const __nv_bfloat162 q = *reinterpret_cast<const __nv_bfloat162*>(&w);
            if (k < 49) *reinterpret_cast<__nv_bfloat16*>(dzt + elem_offset((uint32_t)k, row, 16)) = q.x;
            if (k + 1 < 49) *reinterpret_cast<__nv_bfloat16*>(dzt + elem_offset((uint32_t)k + 1, row, 16)) = q.y;
        }
        // ---- backward: dW_l += dZ_l^T [H_{l-1} | 1]^T and dH_{l-1} = dZ_l W_l, l = 4..2;
        // dW_1 += dZ_1^T [X | 1]^T
#pragma unroll
        for (int l = 3; l >= 0; --l) {
            tt_before_issue();
            if (tid == 0) {
                tc_mma(tmem + dw_col[l], dzt_addr, 16u, l == 0 ? xt_addr : ht_addr[l - 1], 16u, 8, tc_idesc(80),
                       accumulated);
                if (l > 0) tc_mma(tmem + kTtDH, dz_addr, 8u, wt[l - 1], 8u, 4, tc_idesc(64), false);
            }
            tt_commit_wait(bar, phase, failed, status);
            if (l > 0) tt_dz_out(tl + kTtDH, mask[l - 1], l > 1 ? dz : nullptr, dzt, row);
        }
        accumulated = true;
    }
    // ---- this block's partial gradient: lanes 0..63 of the dW columns (rows = outputs)
    float* out = P.partial + (size_t)blockIdx.x * kParams;
    const uint32_t tl = tmem + lane_off;
#pragma unroll
    for (int l = 0; l < 4; ++l) {
        const int nin = l == 0 ? 72 : 64, nout = l == 3 ? 49 : 64;
        const int ow = l == 0 ? oW1 : (l == 1 ? oW2 : (l == 2 ? oW3 : oW4));
        const int ob = l == 0 ? ob1 : (l == 1 ? ob2 : (l == 2 ? ob3 : ob4));
        for (int c0 = 0; c0 < 80; c0 += 16) {
            float v[16];
            tc_load16(tl + dw_col[l] + (uint32_t)c0, v);
            if ((int)row < nout && accumulated) {
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int c = c0 + j;
                    if (c < nin) out[ow + (int)row * nin + c] = v[j];
                    else if (c == nin) out[ob + (int)row] = v[j];
                }
            }
        }
    }
    // loss of the block
    loss += __shfl_xor_sync(0xFFFFFFFFu, loss, 1);
    loss += __shfl_xor_sync(0xFFFFFFFFu, loss, 2);
    loss += __shfl_xor_sync(0xFFFFFFFFu, loss, 4);
    loss += __shfl_xor_sync(0xFFFFFFFFu, loss, 8);
    loss += __shfl_xor_sync(0xFFFFFFFFu, loss, 16);
    __shared__ float s_loss[4];
    if ((tid & 31) == 0) s_loss[warp] = loss;
    if (failed) tc_wait(bar, phase ^ 1u);
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (tid == 0) P.partial_loss[blockIdx.x] = s_loss[0] + s_loss[1] + s_loss[2] + s_loss[3];
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(kTtAlloc));
}

// Sums the per-CTA partials in CTA order (deterministic).
__global__ void reduce_partials_kernel(const float* partial, int ctas, float* grad, const float* partial_loss,
                                       float* loss) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kParams) {
        float s = 0.f;
        for (int c = 0; c < ctas; ++c) s += partial[(size_t)c * kParams + i];
        grad[i] = s;
    }
    if (i == 0) {
        float s = 0.f;
        for (int c = 0; c < ctas; ++c) s += partial_loss[c];
        *loss = s;
    }
}

// Adam on the FP32 master weights.
__global__ void adam_kernel(float* w, float* m, float* v, const float* grad, float lr, float b1, float b2,
                            float eps, float bc1, float bc2) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kParams) return;
    float g = grad[i];
    float mi = b1 * m[i] + (1.f - b1) * g;
    float vi = b2 * v[i] + (1.f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
}

// FP32 master → packed BF16 weights (n-major + transposed copies) and padded biases.
__global__ void pack_kernel(const float* w, __nv_bfloat16* pk, float* bias) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < pEnd) {
        float v = 0.f;
        if (i < pW2) { int n = i / sW1, k = i % sW1; v = k < 72 ? w[oW1 + n * 72 + k] : 0.f; }
        else if (i < pW3) { int j = i - pW2, n = j / sW, k = j % sW; v = k < 64 ? w[oW2 + n * 64 + k] : 0.f; }
        else if (i < pW4) { int j = i - pW3, n = j / sW, k = j % sW; v = k < 64 ? w[oW3 + n * 64 + k] : 0.f; }
        else if (i < pW2T) { int j = i - pW4, n = j / sW, k = j % sW; v = (k < 64 && n < 49) ? w[oW4 + n * 64 + k] : 0.f; }
        else if (i < pW3T) { int j = i - pW2T, n = j / sW, k = j % sW; v = k < 64 ? w[oW2 + k * 64 + n] : 0.f; }
        else if (i < pW4T) { int j = i - pW3T, n = j / sW, k = j % sW; v = k < 64 ? w[oW3 + k * 64 + n] : 0.f; }
        else { int j = i - pW4T, n = j / sW, k = j % sW; v = k < 49 ? w[oW4 + k * 64 + n] : 0.f; }
        pk[i] = __float2bfloat16(v);
    }
    if (i < kBias) {
        float b;
        if (i < 64) b = w[ob1 + i];
        else if (i < 128) b = w[ob2 + i - 64];
        else if (i < 192) b = w[ob3 + i - 128];
        else b = (i - 192) < 49 ? w[ob4 + i - 192] : 0.f;
        bias[i] = b;
    }
}

}  // namespace dn
}  // namespace luz

// ---------------------------------------------------------------- host API
struct luz_denoiser {
    luz_ctx* ctx = nullptr;
    float* w = nullptr;          // FP32 master weights
    float* m = nullptr;
    float* v = nullptr;
    float* grad = nullptr;
    __nv_bfloat16* pack = nullptr;
    float* bias = nullptr;
    float* partial = nullptr;    // [ctas][kParams]
    float* partial_loss = nullptr;
    float* loss = nullptr;
    int ctas = 0;
    uint64_t step = 0;
    float shadow_weight = 1.0f / 3.0f;
};

namespace luz {
luz_status launch_light_pass(luz_ctx* ctx, luz_frame* f, int mode);
namespace dn {

static luz_status upload_lut(luz_ctx* ctx) {
    static DeviceSetup setup;
    return device_setup(setup, setup_generation(), 1, [&]() -> luz_status {
        float lut[256];
        for (int i = 0; i < 256; ++i) lut[i] = (float)std::pow((double)((float)i / 255.0f), 2.2);
        LUZ_CUDA(ctx, cudaMemcpyToSymbol(c_lin_lut, lut, sizeof(lut)));
        return LUZ_OK;
    });
}

static luz_status repack(luz_ctx* ctx, luz_denoiser* d) {
    pack_kernel<<<(pEnd + 255) / 256, 256, 0, ctx->stream>>>(d->w, d->pack, d->bias);
    LUZ_LAUNCHED(ctx, "denoise_pack_kernel");
    return LUZ_OK;
}

static luz_status check_batch(luz_ctx* ctx, const luz_denoise_batch* b) {
    if (!b || !b->features || !b->lin_depth || !b->noisy || !b->unshadowed || b->width == 0 || b->height == 0 ||
        b->images == 0)
        return set_error(ctx, LUZ_ERR_INVALID, "incomplete denoiser batch");
    if ((uint64_t)b->width * b->height * b->images >= (1ull << 31))
        return set_error(ctx, LUZ_ERR_LIMIT, "denoiser batch larger than 2^31 pixels");
    return LUZ_OK;
}

// Dense over the batch's pixels, or over the lit-pixel list of one image when `list`
// is given (the other pixels of `out` are then written by the features pass).
static luz_status run_infer(luz_ctx* ctx, luz_denoiser* d, const luz_denoise_batch* b, float4* out,
                            float* out_ao = nullptr, const uint32_t* list = nullptr,
                            const uint32_t* list_count = nullptr) {
    static DeviceSetup setup;
    luz_status st = device_setup(setup, setup_generation(), kTcSmem, [&]() -> luz_status {
        LUZ_CUDA(ctx, cudaFuncSetAttribute(denoise_infer_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           kTcSmem));
        return LUZ_OK;
    });
    if (st != LUZ_OK) return st;
    InferParams P;
    P.wpack = d->pack;
    P.bias = d->bias;
    P.feat = (const uint4*)b->features;
    P.lin_depth = b->lin_depth;
    P.sig = (const float4*)b->noisy;
    P.uns = (const float4*)b->unshadowed;
    P.G = ImageGeom{b->width, b->height, b->width * b->height, b->images};
    P.out = out;
    P.out_ao = out_ao;
    P.list = list;
    P.list_count = list_count;
    uint32_t tiles = (P.G.pixels * P.G.images + 127) / 128;
    uint32_t grid = std::min<uint32_t>((tiles + kTcGroups - 1) / kTcGroups, (uint32_t)ctx->sm_count * kTcBlocksPerSm);
    prof_begin(ctx, LUZ_KERNEL_DENOISE);
    denoise_infer_tc_kernel<<<grid, kTcThreads, kTcSmem, ctx->stream>>>(P, ctx->d_status);
    prof_end(ctx);
    LUZ_LAUNCHED(ctx, "denoise_infer_tc_kernel");
    return LUZ_OK;
}

static luz_status run_gradient(luz_ctx* ctx, luz_denoiser* d, const luz_denoise_batch* b) {
    if (!b->target) return set_error(ctx, LUZ_ERR_INVALID, "training batch without targets");
    TrainParams P;
    P.wpack = d->pack;
    P.bias = d->bias;
    P.feat = (const uint4*)b->features;
    P.lin_depth = b->lin_depth;
    P.sig = (const float4*)b->noisy;
    P.uns = (const float4*)b->unshadowed;
    P.target = (const float4*)b->target;
    P.weight = (const float4*)b->weight;
    P.G = ImageGeom{b->width, b->height, b->width * b->height, b->images};
    P.grad_scale = 2.0f / (float)((double)P.G.pixels * P.G.images);
    P.shadow_weight = d->shadow_weight;
    P.partial = d->partial;
    P.partial_loss = d->partial_loss;
    LUZ_CUDA(ctx, cudaMemsetAsync(d->partial, 0, (size_t)d->ctas * kParams * 4, ctx->stream));
    static DeviceSetup setup;
    luz_status st = device_setup(setup, setup_generation(), kTtSmem, [&]() -> luz_status {
        LUZ_CUDA(ctx, cudaFuncSetAttribute(denoise_train_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           kTtSmem));
        return LUZ_OK;
    });
    if (st != LUZ_OK) return st;
    prof_begin(ctx, LUZ_KERNEL_DENOISE_TRAIN);
    denoise_train_tc_kernel<<<d->ctas, 128, kTtSmem, ctx->stream>>>(P, ctx->d_status);
    prof_end(ctx);
    LUZ_LAUNCHED(ctx, "denoise_train_tc_kernel");
    reduce_partials_kernel<<<(kParams + 255) / 256, 256, 0, ctx->stream>>>(d->partial, d->ctas, d->grad,
                                                                          d->partial_loss, d->loss);
    LUZ_LAUNCHED(ctx, "denoise_reduce_kernel");
    return LUZ_OK;
}

}  // namespace dn
}  // namespace luz

using namespace luz;
using namespace luz::dn;

extern "C" {

luz_status luz_denoiser_create(luz_ctx* ctx, uint64_t seed, luz_denoiser** out) {
    if (!ctx || !out) return LUZ_ERR_INVALID;
    luz_status s = upload_lut(ctx);
    if (s != LUZ_OK) return s;
    luz_denoiser* d = new luz_denoiser();
    d->ctx = ctx;
    d->ctas = ctx->sm_count;
    cudaError_t e = cudaSuccess;
    auto A = [&](void** p, size_t bytes) { if (e == cudaSuccess) e = cudaMalloc(p, bytes); };
    A((void**)&d->w, kParams * 4);
    A((void**)&d->m, kParams * 4);
    A((void**)&d->v, kParams * 4);
    A((void**)&d->grad, kParams * 4);
    A((void**)&d->pack, (size_t)pEnd * 2);
    A((void**)&d->bias, kBias * 4);
    A((void**)&d->partial, (size_t)d->ctas * kParams * 4);
    A((void**)&d->partial_loss, (size_t)d->ctas * 4);
    A((void**)&d->loss, 4);
    if (e != cudaSuccess) { luz_denoiser_destroy(d); return cuda_error(ctx, e, "cudaMalloc(denoiser)"); }
    // He-uniform initialisation from a SplitMix64 stream.
    std::vector<float> w(kParams, 0.0f);
    uint64_t st = seed * 0x9E3779B97F4A7C15ull + 1;
    auto next = [&]() {
        uint64_t z = (st += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return (float)((z ^ (z >> 31)) >> 40) * (1.0f / 16777216.0f);
    };
    const int offs[4] = {oW1, oW2, oW3, oW4}, fan_in[4] = {72, 64, 64, 64}, fan_out[4] = {64, 64, 64, 49};
    for (int l = 0; l < 4; ++l) {
        float lim = std::sqrt(6.0f / (float)fan_in[l]) * (l == 3 ? 0.1f : 1.0f);
        for (int k = 0; k < fan_in[l] * fan_out[l]; ++k) w[offs[l] + k] = (2.0f * next() - 1.0f) * lim;
    }
    s = luz_denoiser_set_weights(ctx, d, w.data());
    if (s != LUZ_OK) { luz_denoiser_destroy(d); return s; }
    *out = d;
    return LUZ_OK;
}

void luz_denoiser_destroy(luz_denoiser* d) {
    if (!d) return;
    cudaDeviceSynchronize();   // the handle may outlive its context: do not touch it
    void* p[] = {d->w, d->m, d->v, d->grad, d->pack, d->bias, d->partial, d->partial_loss, d->loss};
    for (void* x : p)
        if (x) cudaFree(x);
    delete d;
}

luz_status luz_denoiser_set_weights(luz_ctx* ctx, luz_denoiser* d, const float* params) {
    if (!ctx || !d || !params) return LUZ_ERR_INVALID;
    LUZ_CUDA(ctx, cudaMemcpyAsync(d->w, params, kParams * 4, cudaMemcpyHostToDevice, ctx->stream));
    LUZ_CUDA(ctx, cudaMemsetAsync(d->m, 0, kParams * 4, ctx->stream));
    LUZ_CUDA(ctx, cudaMemsetAsync(d->v, 0, kParams * 4, ctx->stream));
    LUZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    d->step = 0;
    return repack(ctx, d);
}

luz_status luz_denoiser_get_weights(luz_ctx* ctx, luz_denoiser* d, float* params) {
    if (!ctx || !d || !params) return LUZ_ERR_INVALID;
    LUZ_CUDA(ctx, cudaMemcpyAsync(params, d->w, kParams * 4, cudaMemcpyDeviceToHost, ctx->stream));
    LUZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return LUZ_OK;
}

luz_status luz_denoiser_gradient(luz_ctx* ctx, luz_denoiser* d, const luz_denoise_batch* b, float* grad,
                                 float* loss) {
    if (!ctx || !d) return LUZ_ERR_INVALID;
    luz_status s = check_batch(ctx, b);
    if (s == LUZ_OK) s = run_gradient(ctx, d, b);
    if (s != LUZ_OK) return s;
    if (grad) LUZ_CUDA(ctx, cudaMemcpyAsync(grad, d->grad, kParams * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (loss) LUZ_CUDA(ctx, cudaMemcpyAsync(loss, d->loss, 4, cudaMemcpyDeviceToHost, ctx->stream));
    LUZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return LUZ_OK;
}

luz_status luz_denoiser_train_step(luz_ctx* ctx, luz_denoiser* d, const luz_denoise_batch* b, float lr,
                                   float* loss) {
    if (!ctx || !d) return LUZ_ERR_INVALID;
    luz_status s = check_batch(ctx, b);
    if (s == LUZ_OK) s = run_gradient(ctx, d, b);
    if (s != LUZ_OK) return s;
    d->step++;
    const float b1 = 0.9f, b2 = 0.999f;
    float bc1 = 1.0f - (float)std::pow(b1, (double)d->step), bc2 = 1.0f - (float)std::pow(b2, (double)d->step);
    adam_kernel<<<(kParams + 255) / 256, 256, 0, ctx->stream>>>(d->w, d->m, d->v, d->grad, lr, b1, b2, 1e-8f, bc1,
                                                                bc2);
    LUZ_LAUNCHED(ctx, "adam_kernel");
    if ((s = repack(ctx, d)) != LUZ_OK) return s;
    if (loss) {
        LUZ_CUDA(ctx, cudaMemcpyAsync(loss, d->loss, 4, cudaMemcpyDeviceToHost, ctx->stream));
        LUZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return LUZ_OK;
}

luz_status luz_denoise_batch_infer(luz_ctx* ctx, luz_denoiser* d, const luz_denoise_batch* b, float* d_out) {
    if (!ctx || !d || !d_out) return LUZ_ERR_INVALID;
    luz_status s = check_batch(ctx, b);
    if (s != LUZ_OK) return s;
    return run_infer(ctx, d, b, (float4*)d_out);
}

// Network inputs of a traced frame: the split pass (shadowed and unshadowed direct
// light and AO of the lit pixels), then the feature planes. With `for_denoise` the
// features pass also writes 0 to the denoised planes at the background pixels and
// lists the lit pixels for the denoiser.
static luz_status launch_features(luz_ctx* ctx, luz_frame* f, bool for_denoise) {
    luz_status s = upload_lut(ctx);
    if (s == LUZ_OK) s = launch_light_pass(ctx, f, 2);
    if (s != LUZ_OK) return s;
    FeatParams F;
    F.albedo = f->albedo;
    F.normal = f->normal;
    F.material = f->material;
    F.depth = f->depth;
    F.width = f->width;
    F.height = f->height;
    memcpy(F.inverse_proj, f->h_scene.inverse_proj, 64);
    memcpy(F.inverse_view, f->h_scene.inverse_view, 64);
    memcpy(F.cam, f->h_scene.cam_pos, 12);
    F.feat = (uint4*)f->features;
    F.lin_depth = f->lin_depth;
    F.ao = f->ao;
    F.denoised = for_denoise ? f->ao_denoised : nullptr;
    F.denoised4 = for_denoise ? f->denoised : nullptr;
    F.signal = f->signal;
    F.unshadowed = f->unshadowed;
    F.list = for_denoise ? f->dn_list : nullptr;
    F.list_count = f->dn_count;
    if (for_denoise) LUZ_CUDA(ctx, cudaMemsetAsync(f->dn_count, 0, 4, ctx->stream));
    prof_begin(ctx, LUZ_KERNEL_FEATURES);
    features_kernel<<<(f->pixels + 255) / 256, 256, 0, ctx->stream>>>(F);
    prof_end(ctx);
    LUZ_LAUNCHED(ctx, "denoise_features_kernel");
    return LUZ_OK;
}

luz_status luz_denoise_features(luz_ctx* ctx, luz_frame* f) {
    if (!ctx || !f) return LUZ_ERR_INVALID;
    return launch_features(ctx, f, false);
}

luz_status luz_denoise(luz_ctx* ctx, luz_denoiser* d, luz_frame* f) {
    if (!ctx || !d || !f) return LUZ_ERR_INVALID;
    luz_status s = launch_features(ctx, f, true);
    if (s != LUZ_OK) return s;
    luz_denoise_batch b{f->features, f->lin_depth, (const float*)f->signal, (const float*)f->unshadowed, nullptr,
                        nullptr, f->width, f->height, 1};
    return run_infer(ctx, d, &b, f->denoised, f->ao_denoised, f->dn_list, f->dn_count);
}

luz_status luz_denoiser_set_shadow_weight(luz_ctx* ctx, luz_denoiser* d, float weight) {
    if (!ctx || !d || !(weight >= 0.0f) || !(weight <= 1e6f)) return LUZ_ERR_INVALID;
    d->shadow_weight = weight;
    return LUZ_OK;
}

}  // extern "C"
