// vis_trace.cuh — the any-hit traversal of shadow and AO rays shared by the
// visibility kernels (visibility.cu) and the batched frame kernel (batch.cu): per-lane
// ray state (hot part in registers, cold part in shared memory), ray generation from a
// (slot, lit pixel) item, and the bounded traversal steps over the 4-wide two-level
// BVH.
#pragma once
#include "raygen.cuh"
#include "traverse.cuh"
#include "visibility.cuh"

namespace luz {

// Minimum resident CTAs per SM the visibility kernels are compiled for (register cap).
#ifndef LUZ_VIS_MIN_BLOCKS
#define LUZ_VIS_MIN_BLOCKS 4
#endif

constexpr int kVisThreads = 256;
constexpr int kSmemStack = 16;                      // shared-memory stack entries per lane
constexpr int kLocalStack = kStackSize - kSmemStack;
constexpr uint32_t kRayStepCap = 1u << 22;

// Ray state that traversal touches only when it enters or leaves a BLAS, tests a
// triangle or finishes lives in shared memory, one 32-bit field per row of
// kVisThreads entries (conflict-free): world origin and direction, the output word
// and bit, the origin and direction in the current BLAS's object space (the
// watertight shear is derived from them per triangle test: most entered BLASes see
// no triangle test), and the world-space box-test state restored when the ray leaves
// a BLAS.
enum ColdField : int {
    kWoX, kWoY, kWoZ, kWdX, kWdY, kWdZ,
    kOutLo, kOutHi, kOutBits,     // bit | record_hit << 5
    kOdX, kOdY, kOdZ,             // direction in the current BLAS's object space
    kBtLo, kBtHi,                 // triangles of the current BLAS
    kOoX, kOoY, kOoZ,             // origin in the current BLAS's object space
    kWiX, kWiY, kWiZ,             // world inverse direction and origin offsets, restored on
    kWnX, kWnY, kWnZ,             // the way out of a BLAS
    kWfX, kWfY, kWfZ,
    kColdFields
};
constexpr size_t kColdBytes = (size_t)kColdFields * kVisThreads * 4;
constexpr size_t kStackBytes = (size_t)kVisThreads * kSmemStack * 4;

// Hot per-lane state (registers).
struct LaneRay {
    V3 on, of, idir;     // origin offsets (set_origin) and inverse direction in the current space
    float tmin, tmax;
    int node, sp;
    int signs;           // bit a set: the direction's component a is negative
    bool in_blas;
    const float4* nb;    // 4-wide nodes of the current space (the TLAS, or the entered BLAS)
    const float4* tlas;          // batched kernel: the lane's scene
    const DevInstance* insts;
    uint32_t budget;
};

struct Cold {
    float* f;            // this lane's column: field k at f[k * kVisThreads]
    __device__ __forceinline__ float& operator[](int k) const { return f[k * kVisThreads]; }
    __device__ __forceinline__ V3 wo() const { return V3{(*this)[kWoX], (*this)[kWoY], (*this)[kWoZ]}; }
    __device__ __forceinline__ V3 wd() const { return V3{(*this)[kWdX], (*this)[kWdY], (*this)[kWdZ]}; }
    __device__ __forceinline__ V3 oo() const { return V3{(*this)[kOoX], (*this)[kOoY], (*this)[kOoZ]}; }
    __device__ __forceinline__ V3 od() const { return V3{(*this)[kOdX], (*this)[kOdY], (*this)[kOdZ]}; }
};

// Near-plane rows of a 4-wide node for a ray with inverse direction id: the lower
// plane where the component is non-negative, else the upper one (the far plane is
// the other row, index ^ 1); see slab_ordered in traverse.cuh.
__device__ __forceinline__ void near_planes(LaneRay& r) { r.signs = dir_signs(r.idir); }

// The slab test of traverse.cuh (ordered planes, entry shrink kSlabShrink) on the
// lane's ray, which needs tmin >= 0: shadow rays start at 0.001 and
// luz_frame_upload rejects a negative aoMin (a ray query's tMin must not be
// negative). Plane distances as one FMA each, t = p * idir - o * idir. The product o * idir
// is rounded once per ray, so each axis carries the bound E = |o * idir| * 2^-21 of
// that rounding (and of its own), folded into two per-ray offsets: near planes use
// on = o * idir + E (a lower bound of the distance), far planes of = o * idir - E
// (an upper bound). The remaining errors are relative (the rounding of idir and of
// the FMA) and lie inside the entry shrink. Overflowed offsets only widen the box.
__device__ __forceinline__ void set_origin(LaneRay& r, V3 o) {
    V3 oid = V3{o.x * r.idir.x, o.y * r.idir.y, o.z * r.idir.z};
    V3 e = V3{fabsf(oid.x) * 0x1p-21f, fabsf(oid.y) * 0x1p-21f, fabsf(oid.z) * 0x1p-21f};
    r.on = V3{oid.x + e.x, oid.y + e.y, oid.z + e.z};
    r.of = V3{oid.x - e.x, oid.y - e.y, oid.z - e.z};
}
__device__ __forceinline__ bool slab_ordered(float nx, float fx, float ny, float fy, float nz, float fz,
                                             const LaneRay& r, float& tnear) {
    const V3& id = r.idir;
    float tn = fmaxf(fmaxf(__fmaf_rn(nx, id.x, -r.on.x), __fmaf_rn(ny, id.y, -r.on.y)),
                     fmaxf(__fmaf_rn(nz, id.z, -r.on.z), r.tmin));
    float tf = fminf(fminf(__fmaf_rn(fx, id.x, -r.of.x), __fmaf_rn(fy, id.y, -r.of.y)),
                     fminf(__fmaf_rn(fz, id.z, -r.of.z), r.tmax));
    tnear = tn;
    return tn * kSlabShrink <= tf;
}

// The ray of item (slot, j) of scene S (light.frag:86-135): world origin and
// direction, t range, output word and whether a hit (shadow) or a miss (AO) is
// recorded. Returns false when there is nothing to trace; the miss (AO) has then
// already been recorded.
template <bool kCoherent = false>
__device__ __forceinline__ bool gen_ray(const SceneVis& S, const VisCommon& C, uint32_t slot, uint32_t j, V3& wo,
                                        V3& wd, float& tmin, float& tmax, uint32_t*& out, bool& record_hit,
                                        uint32_t& pix) {
    // kCoherent: the list was written earlier in the same launch (the batch frame
    // kernel), so it is read through L2 rather than the non-coherent read-only path.
    const float4* sp = S.surf + 2 * (size_t)j;
    float4 s0 = kCoherent ? __ldcg(sp) : __ldg(sp), s1 = kCoherent ? __ldcg(sp + 1) : __ldg(sp + 1);
    V3 p = V3{s0.x, s0.y, s0.z}, N = V3{s1.x, s1.y, s1.z};
    pix = __float_as_uint(s0.w);
    const uint32_t pxy = __float_as_uint(s1.w);   // x | y << 16 of the lit pixel
    const uint32_t px = pxy & 0xFFFFu, py = pxy >> 16;
    V3 cam = V3{S.cam[0], S.cam[1], S.cam[2]};
    float rx, ry;
    if (slot < S.shadow_slots) {
        uint32_t e = __ldg(S.slot_table + slot);
        uint32_t li = e & 0xFFFFu, si = e >> 16;
        out = S.shadow_bits + (size_t)slot * S.words + (pix >> 5);
        record_hit = true;
        const V3 L = light_vector(S.lights[li], p);
        // When the light pass's term of this light cannot depend on its shadow factor
        // (zero weight max(dot(N, L), 0) or zero unshadowed radiance, computed as the
        // light pass computes them), the ray is not traced and its bit stays 0.
        if (S.cull && shadow_has_no_effect(S.lights[li], p, N, L)) return false;
        sample_rg(C.blue_noise, C.bn_size, S.sampler, px, py, (int)si, S.frame, li + 1, &rx, &ry);
        shadow_ray(S.lights[li], p, N, cam, rx, ry, L, wo, wd, tmax);
        tmin = 0.001f;
    } else {
        uint32_t a = slot - S.shadow_slots;
        sample_rg(C.blue_noise, C.bn_size, S.sampler, px, py, (int)a, S.frame, 0u, &rx, &ry);
        ao_ray(p, N, cam, rx, ry, wo, wd);
        tmin = S.ao_min;
        tmax = S.ao_max;
        out = S.ao_bits + (size_t)a * S.words + (pix >> 5);
        record_hit = false;
    }
    bool ok = S.instance_count > 0 && finite3(wo) && finite3(wd) && (tmin <= tmax) &&
              !(wd.x == 0.0f && wd.y == 0.0f && wd.z == 0.0f);
    if (!ok && !record_hit) atomicOr(out, 1u << (pix & 31));   // no ray: a miss
    return ok;
}

// Starts a lane on a generated ray: cold state in shared memory, hot state in
// registers, traversal at the TLAS root.
__device__ __forceinline__ void start_ray(LaneRay& r, const Cold& c, const SceneVis& S, V3 wo, V3 wd, float tmin,
                                          float tmax, const uint32_t* out, bool record_hit, uint32_t pix) {
    unsigned long long oa = reinterpret_cast<unsigned long long>(out);
    c[kWoX] = wo.x; c[kWoY] = wo.y; c[kWoZ] = wo.z;
    c[kWdX] = wd.x; c[kWdY] = wd.y; c[kWdZ] = wd.z;
    c[kOutLo] = __uint_as_float((uint32_t)oa);
    c[kOutHi] = __uint_as_float((uint32_t)(oa >> 32));
    c[kOutBits] = __uint_as_float((pix & 31u) | (record_hit ? 32u : 0u));
    r.tmin = tmin;
    r.tmax = tmax;
    r.idir = safe_inv(wd);
    set_origin(r, wo);
    near_planes(r);
    c[kWiX] = r.idir.x; c[kWiY] = r.idir.y; c[kWiZ] = r.idir.z;
    c[kWnX] = r.on.x; c[kWnY] = r.on.y; c[kWnZ] = r.on.z;
    c[kWfX] = r.of.x; c[kWfY] = r.of.y; c[kWfZ] = r.of.z;
    r.node = 0;
    r.sp = 0;
    r.in_blas = false;
    r.budget = 0;
    r.tlas = S.tlas_nodes;
    r.nb = S.tlas_nodes;
    r.insts = S.instances;
}

// Generates and starts the ray of item (slot, j) (the batched kernel).
template <bool kCoherent = false>
__device__ __forceinline__ bool setup_ray(LaneRay& r, const Cold& c, const SceneVis& S, const VisCommon& C,
                                          uint32_t slot, uint32_t j) {
    V3 wo, wd;
    float tmin, tmax;
    uint32_t* out;
    bool record_hit;
    uint32_t pix;
    if (!gen_ray<kCoherent>(S, C, slot, j, wo, wd, tmin, tmax, out, record_hit, pix)) return false;
    start_ray(r, c, S, wo, wd, tmin, tmax, out, record_hit, pix);
    return true;
}

__device__ __forceinline__ void finish_ray(const Cold& c, bool& active, bool hit) {
    uint32_t bits = __float_as_uint(c[kOutBits]);
    if (hit == ((bits & 32u) != 0)) {
        uint32_t* out = reinterpret_cast<uint32_t*>((unsigned long long)__float_as_uint(c[kOutLo]) |
                                                    ((unsigned long long)__float_as_uint(c[kOutHi]) << 32));
        atomicOr(out, 1u << (bits & 31u));
    }
    active = false;
}

// 4-wide node loads: read-only global memory (__ldg) unless the TLAS top may come
// from shared memory (kStaged), where the pointer is generic.
template <bool kStaged>
__device__ __forceinline__ float4 node_load(const float4* p) {
    if (kStaged) return *p;
    return __ldg(p);
}

// Up to `steps` traversal steps of one lane's ray; clears `active` when it ends.
// tlas / insts: the scene's TLAS nodes and instances (kernel parameters in the
// single-scene kernel, the lane's own scene in the batched one). The step cap of a
// ray (kRayStepCap unless a debug cap is set) is charged `steps` per call, so a ray
// ends after at most step_cap + steps; a ray that reaches it ends unoccluded (shadow)
// or as a miss (AO) and raises LUZ_DEV_TRAVERSAL_CAP.
template <bool kStats, bool kStaged>
__device__ __forceinline__ void run_steps(LaneRay& r, const Cold& c, bool& active, const float4* smem_tlas,
                                          uint32_t staged, const float4* tlas, const DevInstance* insts,
                                          uint32_t* s_stack, int* lstack, uint32_t steps, uint32_t step_cap,
                                          uint32_t& err, TraceCounters& cnt) {
    if (active && (r.budget += steps) > step_cap) {
        err |= LUZ_DEV_TRAVERSAL_CAP;
        finish_ray(c, active, false);
    }
    for (uint32_t s = 0; s < steps && active; ++s) {
        bool finished = false, hit = false;
        if (r.node >= 0) {
            // 4-wide node: test the four child boxes, continue with the nearest hit
            // child and push the other hits. Empty slots hold inverted boxes, which
            // no ray overlaps.
            if (kStats) { if (r.in_blas) cnt.blas_nodes++; else cnt.tlas_nodes++; }
            const float4* np = kStaged ? (r.in_blas ? r.nb : ((uint32_t)r.node < staged ? smem_tlas : tlas)) : r.nb;
            np += (size_t)r.node * kNode4F4;
            const int sx = r.signs & 1, sy = (r.signs >> 1) & 1, sz = r.signs >> 2;
            const float4 nx = node_load<kStaged>(np + sx), fx = node_load<kStaged>(np + (sx ^ 1)),
                         ny = node_load<kStaged>(np + 2 + sy), fy = node_load<kStaged>(np + 3 - sy),
                         nz = node_load<kStaged>(np + 4 + sz), fz = node_load<kStaged>(np + 5 - sz),
                         cf = node_load<kStaged>(np + 6);
            const int ch[4] = {__float_as_int(cf.x), __float_as_int(cf.y), __float_as_int(cf.z),
                               __float_as_int(cf.w)};
            float tn[4];
            bool h[4];
            h[0] = slab_ordered(nx.x, fx.x, ny.x, fy.x, nz.x, fz.x, r, tn[0]);
            h[1] = slab_ordered(nx.y, fx.y, ny.y, fy.y, nz.y, fz.y, r, tn[1]);
            h[2] = slab_ordered(nx.z, fx.z, ny.z, fy.z, nz.z, fz.z, r, tn[2]);
            h[3] = slab_ordered(nx.w, fx.w, ny.w, fy.w, nz.w, fz.w, r, tn[3]);
            // Nearest hit child by constant-index selects (a dynamic ch[best] would
            // put ch[] in local memory).
            int best = -1, bc = 0;
            float tb = 0.f;
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (h[k] && (best < 0 || tn[k] < tb)) { best = k; tb = tn[k]; bc = ch[k]; }
            if (best >= 0) {
                // The other hits go on the stack, farthest index first; when they all
                // fit in the shared-memory part the pushes are predicated stores.
                const int n = (int)h[0] + (int)h[1] + (int)h[2] + (int)h[3] - 1;
                if (r.sp + n <= kSmemStack) {
#pragma unroll
                    for (int k = 3; k >= 0; --k)
                        if (h[k] && k != best) { s_stack[r.sp * 32] = (uint32_t)ch[k]; ++r.sp; }
                } else {
#pragma unroll
                    for (int k = 3; k >= 0; --k) {
                        if (!h[k] || k == best) continue;
                        if (r.sp < kSmemStack) s_stack[r.sp * 32] = (uint32_t)ch[k];
                        else if (r.sp < kStackSize) lstack[r.sp - kSmemStack] = ch[k];
                        else { err |= LUZ_DEV_STACK_OVERFLOW; finished = true; }
                        ++r.sp;
                    }
                }
                r.node = bc;
                if (!finished) continue;
            }
        } else if (!r.in_blas) {
            // Instance leaf: entered unless its mask or BLAS is empty or the ray
            // segment provably misses the BLAS's bounding sphere.
            if (kStats) cnt.instances++;
            const DevInstance* I = insts + (~r.node);
            const float4* wp = reinterpret_cast<const float4*>(I->w2o);
            uint4 meta = __ldg(reinterpret_cast<const uint4*>(&I->custom_index));
            float4 q0 = __ldg(wp), q1 = __ldg(wp + 1), q2 = __ldg(wp + 2), sph = __ldg(&I->sphere);
            float m[12] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w, q2.x, q2.y, q2.z, q2.w};
            const V3 od = xform_dir(m, c.wd()), oo = xform_point(m, c.wo());
            if ((meta.y & 0xFFu) != 0 && meta.w > 0 && !sphere_misses(oo, od, r.tmin, r.tmax, sph)) {
                c[kOdX] = od.x;
                c[kOdY] = od.y;
                c[kOdZ] = od.z;
                c[kOoX] = oo.x;
                c[kOoY] = oo.y;
                c[kOoZ] = oo.z;
                r.idir = safe_inv(od);
                set_origin(r, oo);
                near_planes(r);
                const ulonglong2 pt = __ldg(reinterpret_cast<const ulonglong2*>(&I->nodes4));
                r.nb = reinterpret_cast<const float4*>(pt.x);
                c[kBtLo] = __uint_as_float((uint32_t)pt.y);
                c[kBtHi] = __uint_as_float((uint32_t)(pt.y >> 32));
                if (r.sp < kSmemStack) s_stack[r.sp * 32] = (uint32_t)kStackMarker;
                else if (r.sp < kStackSize) lstack[r.sp - kSmemStack] = kStackMarker;
                else { err |= LUZ_DEV_STACK_OVERFLOW; finished = true; }
                ++r.sp;
                r.in_blas = true;
                r.node = 0;
                if (!finished) continue;
            }
        } else {
            if (kStats) cnt.tris++;
            const float4* bt = reinterpret_cast<const float4*>((unsigned long long)__float_as_uint(c[kBtLo]) |
                                                               ((unsigned long long)__float_as_uint(c[kBtHi]) << 32));
            const float4* tp = bt + (size_t)(~r.node) * kTriF4;
            float4 a = __ldg(tp), b = __ldg(tp + 1), cc = __ldg(tp + 2);
            const WtRay wt = wt_setup(c.oo(), c.od());
            float t, U, V, W, det;
            if (wt_test(wt, V3{a.x, a.y, a.z}, V3{b.x, b.y, b.z}, V3{cc.x, cc.y, cc.z}, t, U, V, W, det) &&
                t >= r.tmin && t <= r.tmax) {
                finished = true;
                hit = true;
            }
        }
        // pop (at most one TLAS marker lies between two nodes)
        while (!finished) {
            if (r.sp == 0) { finished = true; break; }
            --r.sp;
            int v = r.sp < kSmemStack ? (int)s_stack[r.sp * 32] : lstack[r.sp - kSmemStack];
            if (v == kStackMarker) {
                r.in_blas = false;
                r.nb = tlas;
                r.idir = V3{c[kWiX], c[kWiY], c[kWiZ]};
                r.on = V3{c[kWnX], c[kWnY], c[kWnZ]};
                r.of = V3{c[kWfX], c[kWfY], c[kWfZ]};
                near_planes(r);
                continue;
            }
            r.node = v;
            break;
        }
        if (finished) finish_ray(c, active, hit);
    }
}

__device__ __forceinline__ void flush_stats(unsigned long long* stats, uint32_t rays, const TraceCounters& cnt) {
    atomicAdd(stats + 0, (unsigned long long)rays);
    atomicAdd(stats + 1, (unsigned long long)cnt.tlas_nodes);
    atomicAdd(stats + 2, (unsigned long long)cnt.blas_nodes);
    atomicAdd(stats + 3, (unsigned long long)cnt.tris);
    atomicAdd(stats + 4, (unsigned long long)cnt.instances);
}

}  // namespace luz
