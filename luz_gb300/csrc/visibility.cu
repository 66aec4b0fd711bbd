// visibility.cu — the persistent wavefront kernel that traces every shadow and AO ray
// of a frame (light.frag:86-135) and writes the hit/miss bit planes.
//
// Work items are (slot, lit pixel) pairs, slot-major, so neighbouring items share a
// light and lie in neighbouring pixels. Each lane holds one ray as an explicit
// traversal state. After every few traversal steps the warp counts its idle lanes
// with a ballot; when enough are idle, one lane takes that many items with a single
// atomic and the idle lanes pick theirs by rank (popc of the lower lanes' ballot
// bits), then generate their rays while the others keep traversing. Lanes are never
// left idle for a whole ray of a slow neighbour.
//
// Traversal: the TLAS top (breadth-first prefix) is staged in shared memory; BLAS
// nodes and triangles come through 16-B vector loads; the stack is warp-interleaved
// in shared memory (entry k of lane l at [k][l]) with a local-memory tail for rare
// deep paths.
#include <algorithm>
#include <cstring>

#include "raygen.cuh"
#include "traverse.cuh"

namespace luz {

struct VisParams {
    const float4* tlas_nodes;
    uint32_t tlas_node_count;
    uint32_t smem_nodes;         // TLAS nodes staged in shared memory
    const DevInstance* instances;
    uint32_t instance_count;
    const float4* surf;
    const uint32_t* lit_count;
    const luz_light* lights;
    const uint32_t* slot_table;
    uint32_t shadow_slots, ao_samples;
    float cam[3];
    float ao_min, ao_max;
    int sampler, frame;
    const uint8_t* blue_noise;
    uint32_t bn_size;
    uint32_t width;
    uint32_t words;
    uint32_t* shadow_bits;
    uint32_t* ao_bits;
    unsigned long long* work_counter;
    uint32_t* status;
    uint32_t refill;             // refill when at least this many lanes are idle
    uint32_t steps;              // traversal steps between refill checks
};

constexpr int kSmemStack = 16;                      // shared-memory stack entries per lane
constexpr int kLocalStack = kStackSize - kSmemStack;
constexpr uint32_t kRayStepCap = 1u << 22;

template <bool kStats>
__global__ void __launch_bounds__(256, 3) visibility_kernel(VisParams P, unsigned long long* stats) {
    extern __shared__ float4 smem[];
    const uint32_t staged = min(P.tlas_node_count, P.smem_nodes);
    for (uint32_t i = threadIdx.x; i < staged * kNodeF4; i += blockDim.x) smem[i] = __ldg(P.tlas_nodes + i);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t* s_stack = reinterpret_cast<uint32_t*>(smem + staged * kNodeF4) + warp * (kSmemStack * 32) + lane;
    int lstack[kLocalStack];
    __syncthreads();

    const uint32_t full = 0xFFFFFFFFu;
    const uint32_t lit = *P.lit_count;
    const unsigned long long total = (unsigned long long)lit * (P.shadow_slots + P.ao_samples);
    const V3 cam = V3{P.cam[0], P.cam[1], P.cam[2]};
    const uint32_t lt_mask = (1u << lane) - 1u;
    uint32_t err = 0;
    TraceCounters cnt{0, 0, 0, 0};
    uint32_t rays = 0;

    // per-lane ray state
    bool active = false, exhausted = false;
    V3 wo{}, wd{}, widir{}, idir{};
    WtRay wt{};
    float tmin = 0.f, tmax = 0.f;
    int node = 0, sp = 0;
    bool in_blas = false;
    const float4* bn = nullptr;
    const float4* bt = nullptr;
    uint32_t out_word = 0, out_bit = 0, budget = 0;
    bool record_hit = false;

    // Items with nothing to trace (empty TLAS, invalid rays) still owe their bit.
    for (;;) {
        uint32_t idle = __ballot_sync(full, !active);
        if (!exhausted && __popc(idle) >= (int)P.refill) {
            int leader = __ffs(idle) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(P.work_counter, (unsigned long long)__popc(idle));
            base = __shfl_sync(full, base, leader);
            if (base + __popc(idle) >= total) exhausted = true;
            if (!active) {
                unsigned long long item = base + __popc(idle & lt_mask);
                if (item < total) {
                    uint32_t slot = (uint32_t)(item / lit);
                    uint32_t j = (uint32_t)(item - (unsigned long long)slot * lit);
                    float4 s0 = __ldg(P.surf + 2 * (size_t)j), s1 = __ldg(P.surf + 2 * (size_t)j + 1);
                    V3 p = V3{s0.x, s0.y, s0.z}, N = V3{s1.x, s1.y, s1.z};
                    uint32_t pix = __float_as_uint(s0.w);
                    uint32_t px = pix % P.width, py = pix / P.width;
                    float rx, ry;
                    if (slot < P.shadow_slots) {
                        uint32_t e = __ldg(P.slot_table + slot);
                        uint32_t li = e & 0xFFFFu, si = e >> 16;
                        sample_rg(P.blue_noise, P.bn_size, P.sampler, px, py, (int)si, P.frame, li + 1, &rx, &ry);
                        shadow_ray(P.lights[li], p, N, cam, rx, ry, wo, wd, tmax);
                        tmin = 0.001f;
                        out_word = slot * P.words + (pix >> 5);
                        record_hit = true;
                    } else {
                        uint32_t a = slot - P.shadow_slots;
                        sample_rg(P.blue_noise, P.bn_size, P.sampler, px, py, (int)a, P.frame, 0u, &rx, &ry);
                        ao_ray(p, N, cam, rx, ry, wo, wd);
                        tmin = P.ao_min;
                        tmax = P.ao_max;
                        out_word = (P.shadow_slots + a) * P.words + (pix >> 5);
                        record_hit = false;
                    }
                    out_bit = 1u << (pix & 31);
                    if (kStats) ++rays;
                    bool ok = P.instance_count > 0 && finite3(wo) && finite3(wd) && (tmin <= tmax) &&
                              !(wd.x == 0.0f && wd.y == 0.0f && wd.z == 0.0f);
                    if (ok) {
                        widir = safe_inv(wd);
                        idir = widir;
                        wt.o = wo;
                        node = 0;
                        sp = 0;
                        in_blas = false;
                        budget = 0;
                        active = true;
                    } else if (!record_hit) {
                        // no ray: a miss (AO counts misses; shadow records nothing)
                        uint32_t* w = out_word < P.shadow_slots * P.words ? P.shadow_bits + out_word
                                                                          : P.ao_bits + (out_word - P.shadow_slots * P.words);
                        atomicOr(w, out_bit);
                    }
                }
            }
        }
        if (exhausted && __ballot_sync(full, active) == 0) break;
        for (uint32_t s = 0; s < P.steps && active; ++s) {
            bool finished = false, hit = false;
            if (++budget > kRayStepCap) { err |= LUZ_DEV_TRAVERSAL_CAP; finished = true; }
            else if (node >= 0) {
                if (kStats) { if (in_blas) cnt.blas_nodes++; else cnt.tlas_nodes++; }
                const float4* np = in_blas ? bn : ((uint32_t)node < staged ? smem : P.tlas_nodes);
                np += (size_t)node * kNodeF4;
                float4 n0 = np[0], n1 = np[1], n2 = np[2], n3 = np[3];
                const V3 o = in_blas ? wt.o : wo;
                int c0 = __float_as_int(n3.x), c1 = __float_as_int(n3.y);
                float t0, t1;
                bool h0 = c0 != kEmptyChild && slab(n0.x, n0.y, n0.z, n0.w, n2.x, n2.y, o, idir, tmin, tmax, t0);
                bool h1 = c1 != kEmptyChild && slab(n1.x, n1.y, n1.z, n1.w, n2.z, n2.w, o, idir, tmin, tmax, t1);
                if (h0 && h1) {
                    int nearc = t1 < t0 ? c1 : c0, farc = t1 < t0 ? c0 : c1;
                    if (sp < kSmemStack) s_stack[sp * 32] = (uint32_t)farc;
                    else if (sp < kStackSize) lstack[sp - kSmemStack] = farc;
                    else { err |= LUZ_DEV_STACK_OVERFLOW; finished = true; }
                    ++sp;
                    node = nearc;
                    if (!finished) continue;
                } else if (h0 || h1) {
                    node = h0 ? c0 : c1;
                    continue;
                }
            } else if (!in_blas) {
                if (kStats) cnt.instances++;
                const DevInstance* I = P.instances + (~node);
                const float4* wp = reinterpret_cast<const float4*>(I->w2o);
                uint4 meta = __ldg(reinterpret_cast<const uint4*>(&I->custom_index));
                if ((meta.y & 0xFFu) != 0 && meta.w > 0) {
                    float4 r0 = __ldg(wp), r1 = __ldg(wp + 1), r2 = __ldg(wp + 2);
                    float m[12] = {r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w, r2.x, r2.y, r2.z, r2.w};
                    V3 od = xform_dir(m, wd);
                    wt = wt_setup(xform_point(m, wo), od);
                    idir = safe_inv(od);
                    bn = I->nodes;
                    bt = I->tris;
                    if (sp < kSmemStack) s_stack[sp * 32] = (uint32_t)kStackMarker;
                    else if (sp < kStackSize) lstack[sp - kSmemStack] = kStackMarker;
                    else { err |= LUZ_DEV_STACK_OVERFLOW; finished = true; }
                    ++sp;
                    in_blas = true;
                    node = 0;
                    if (!finished) continue;
                }
            } else {
                if (kStats) cnt.tris++;
                const float4* tp = bt + (size_t)(~node) * kTriF4;
                float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
                float t, U, V, W, det;
                if (wt_test(wt, V3{a.x, a.y, a.z}, V3{b.x, b.y, b.z}, V3{c.x, c.y, c.z}, t, U, V, W, det) &&
                    t >= tmin && t <= tmax) {
                    finished = true;
                    hit = true;
                }
            }
            // pop (at most one TLAS marker lies between two nodes)
            while (!finished) {
                if (sp == 0) { finished = true; break; }
                --sp;
                int v = sp < kSmemStack ? (int)s_stack[sp * 32] : lstack[sp - kSmemStack];
                if (v == kStackMarker) {
                    in_blas = false;
                    idir = widir;
                    continue;
                }
                node = v;
                break;
            }
            if (finished) {
                if (hit == record_hit) {
                    uint32_t* w = out_word < P.shadow_slots * P.words ? P.shadow_bits + out_word
                                                                      : P.ao_bits + (out_word - P.shadow_slots * P.words);
                    atomicOr(w, out_bit);
                }
                active = false;
            }
        }
    }
    if (err) atomicOr(P.status, err);
    if (kStats) {
        atomicAdd(stats + 0, (unsigned long long)rays);
        atomicAdd(stats + 1, (unsigned long long)cnt.tlas_nodes);
        atomicAdd(stats + 2, (unsigned long long)cnt.blas_nodes);
        atomicAdd(stats + 3, (unsigned long long)cnt.tris);
        atomicAdd(stats + 4, (unsigned long long)cnt.instances);
    }
}

// ---------------------------------------------------------------- host launchers
// Defaults: the best shape of a sweep on the 1080p two-level scene (smem nodes
// {0,256,512,1024} x refill {1,4,8,16} x steps {4,8,16,32} x CTAs/SM {2,3,4}).
static const VisTuning g_tuning{256, 16, 32, 3, 1};

luz_status launch_visibility(luz_ctx* ctx, luz_frame* f, const luz_tlas* t, int frame_index,
                             unsigned long long* d_stats) {
    uint32_t S = f->shadow_slots + f->ao_samples;
    cudaStream_t st = ctx->stream;
    if (f->shadow_slots)
        LUZ_CUDA(ctx, cudaMemsetAsync(f->shadow_bits, 0, (size_t)f->shadow_slots * f->words * 4, st));
    if (f->ao_samples)
        LUZ_CUDA(ctx, cudaMemsetAsync(f->ao_bits, 0, (size_t)f->ao_samples * f->words * 4, st));
    if (S == 0) return LUZ_OK;
    LUZ_CUDA(ctx, cudaMemsetAsync(f->work_counter, 0, 8, st));
    const VisTuning& tu = ctx->vis_tuning.set ? ctx->vis_tuning : g_tuning;
    VisParams P;
    P.tlas_nodes = t->nodes;
    P.tlas_node_count = t->count ? t->node_count : 0;
    P.smem_nodes = tu.smem_nodes;
    P.instances = t->instances;
    P.instance_count = t->count;
    P.surf = f->surf;
    P.lit_count = f->lit_count;
    P.lights = f->d_lights;
    P.slot_table = f->d_slot_table;
    P.shadow_slots = f->shadow_slots;
    P.ao_samples = f->ao_samples;
    memcpy(P.cam, f->h_scene.cam_pos, 12);
    P.ao_min = f->h_scene.ao_min;
    P.ao_max = f->h_scene.ao_max;
    P.sampler = f->h_scene.sampler;
    P.frame = frame_index;
    P.blue_noise = ctx->d_blue_noise;
    P.bn_size = ctx->blue_noise_size;
    P.width = f->width;
    P.words = f->words;
    P.shadow_bits = f->shadow_bits;
    // The AO planes follow the shadow planes in one index space (out_word); the
    // kernel splits it back.
    P.ao_bits = f->ao_bits;
    P.work_counter = f->work_counter;
    P.status = ctx->d_status;
    P.refill = tu.refill;
    P.steps = tu.steps;
    uint32_t staged = std::min<uint32_t>(P.tlas_node_count, tu.smem_nodes);
    size_t smem = (size_t)staged * 64 + (size_t)256 * kSmemStack * 4;
    static size_t attr_bytes = 0;
    if (smem > attr_bytes) {
        LUZ_CUDA(ctx, cudaFuncSetAttribute(visibility_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        LUZ_CUDA(ctx, cudaFuncSetAttribute(visibility_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr_bytes = smem;
    }
    uint32_t grid = (uint32_t)ctx->sm_count * tu.ctas_per_sm;
    if (d_stats) {
        LUZ_CUDA(ctx, cudaMemsetAsync(d_stats, 0, 5 * sizeof(unsigned long long), st));
        visibility_kernel<true><<<grid, 256, smem, st>>>(P, d_stats);
        LUZ_LAUNCHED(ctx, "visibility_kernel<stats>");
    } else {
        visibility_kernel<false><<<grid, 256, smem, st>>>(P, nullptr);
        LUZ_LAUNCHED(ctx, "visibility_kernel");
    }
    return LUZ_OK;
}

}  // namespace luz

extern "C" luz_status luz_ctx_set_vis_tuning(luz_ctx* ctx, const luz_vis_tuning* t) {
    using namespace luz;
    if (!ctx || !t) return LUZ_ERR_INVALID;
    if (t->smem_nodes == 0 && t->refill == 0 && t->steps == 0 && t->ctas_per_sm == 0) {
        ctx->vis_tuning = VisTuning{0, 0, 0, 0, 0};
        return LUZ_OK;
    }
    if (t->smem_nodes > 2048 || t->refill < 1 || t->refill > 32 || t->steps < 1 || t->steps > 1024 ||
        t->ctas_per_sm < 1 || t->ctas_per_sm > 16)
        return set_error(ctx, LUZ_ERR_INVALID, "visibility tuning outside its documented ranges");
    ctx->vis_tuning = VisTuning{t->smem_nodes, t->refill, t->steps, t->ctas_per_sm, 1};
    return LUZ_OK;
}

extern "C" luz_status luz_ctx_get_vis_tuning(const luz_ctx* ctx, luz_vis_tuning* t) {
    using namespace luz;
    if (!ctx || !t) return LUZ_ERR_INVALID;
    const VisTuning& tu = ctx->vis_tuning.set ? ctx->vis_tuning : g_tuning;
    *t = luz_vis_tuning{tu.smem_nodes, tu.refill, tu.steps, tu.ctas_per_sm};
    return LUZ_OK;
}

namespace luz {

luz_status frame_lit_count(luz_ctx* ctx, luz_frame* f, uint32_t* count) {
    LUZ_CUDA(ctx, cudaMemcpyAsync(&f->h_lit_count, f->lit_count, 4, cudaMemcpyDeviceToHost, ctx->stream));
    LUZ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *count = f->h_lit_count;
    return LUZ_OK;
}

}  // namespace luz
