// traverse.cuh — two-level BVH traversal on the SMs (no RT cores are used: the
// reference's rayQueryProceedEXT loop, light.frag:99-106,125-132, becomes this).
//
// * Rays are tested against triangles with the watertight test of S. Woop,
//   C. Benthin and I. Wald, "Watertight Ray/Triangle Intersection", JCGT 2(1),
//   2013. Its edge functions are recomputed in FP64 only when an FP32 value is
//   exactly zero. Triangles are two-sided (instances carry
//   TRIANGLE_FACING_CULL_DISABLE, source/Graphics/VulkanWrapper.cpp:1119).
// * Any-hit (gl_RayFlagsTerminateOnFirstHitEXT) returns the OR over all triangles
//   with t in [tmin, tmax]; closest-hit keeps the smallest t, ties broken by
//   (instance input index, primitive), so both results are independent of the
//   traversal order.
// * Box tests are conservative: leaf boxes are padded and the slab interval is
//   widened by a relative 2^-16, so no box that holds an accepted hit is culled.
// * Traversal runs over the 4-wide nodes (the even-depth collapse of the binary
//   LBVH): the nearest hit child is visited next, the other hits are pushed
//   farthest first.
#pragma once
#include "internal.cuh"

namespace luz {

constexpr uint32_t kTraversalCap = 1u << 24;

__device__ __forceinline__ float comp(V3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

struct WtRay {
    V3 o;
    int kx, ky, kz;
    float sx, sy, sz;
};

__device__ __forceinline__ WtRay wt_setup(V3 o, V3 d) {
    WtRay r;
    r.o = o;
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    int kz = ax >= ay ? (ax >= az ? 0 : 2) : (ay >= az ? 1 : 2);
    int kx = kz == 2 ? 0 : kz + 1;
    int ky = kx == 2 ? 0 : kx + 1;
    float dz = comp(d, kz);
    if (dz < 0.0f) { int t = kx; kx = ky; ky = t; }
    r.kx = kx; r.ky = ky; r.kz = kz;
    r.sx = comp(d, kx) / dz;
    r.sy = comp(d, ky) / dz;
    r.sz = 1.0f / dz;
    return r;
}

// Returns true with t, (u,v,w) barycentric numerators and det when the ray crosses
// the triangle (before the [tmin,tmax] check).
__device__ __forceinline__ bool wt_test(const WtRay& r, V3 v0, V3 v1, V3 v2, float& t, float& U,
                                        float& V, float& W, float& det) {
    V3 A = v0 - r.o, B = v1 - r.o, C = v2 - r.o;
    float akx = comp(A, r.kx), aky = comp(A, r.ky), akz = comp(A, r.kz);
    float bkx = comp(B, r.kx), bky = comp(B, r.ky), bkz = comp(B, r.kz);
    float ckx = comp(C, r.kx), cky = comp(C, r.ky), ckz = comp(C, r.kz);
    float Ax = akx - r.sx * akz, Ay = aky - r.sy * akz;
    float Bx = bkx - r.sx * bkz, By = bky - r.sy * bkz;
    float Cx = ckx - r.sx * ckz, Cy = cky - r.sy * ckz;
    U = Cx * By - Cy * Bx;
    V = Ax * Cy - Ay * Cx;
    W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        double CxBy = (double)Cx * (double)By, CyBx = (double)Cy * (double)Bx;
        U = (float)(CxBy - CyBx);
        double AxCy = (double)Ax * (double)Cy, AyCx = (double)Ay * (double)Cx;
        V = (float)(AxCy - AyCx);
        double BxAy = (double)Bx * (double)Ay, ByAx = (double)By * (double)Ax;
        W = (float)(BxAy - ByAx);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    det = U + V + W;
    if (det == 0.0f) return false;
    float Az = r.sz * akz, Bz = r.sz * bkz, Cz = r.sz * ckz;
    float T = U * Az + V * Bz + W * Cz;
    t = T / det;
    return true;
}

__device__ __forceinline__ V3 safe_inv(V3 d) {
    const float tiny = 1e-20f;
    float x = fabsf(d.x) > tiny ? d.x : copysignf(tiny, d.x);
    float y = fabsf(d.y) > tiny ? d.y : copysignf(tiny, d.y);
    float z = fabsf(d.z) > tiny ? d.z : copysignf(tiny, d.z);
    return V3{1.0f / x, 1.0f / y, 1.0f / z};
}

// Conservative slab test of one box with near / far planes already picked by the
// ray's direction signs (rounding is monotonic, so near <= far for every
// non-inverted box). Entry distances are >= tmin >= 0, so scaling the entry down by
// 2^-16 relative widens the interval past the rounding of the plane distances; an
// inverted (empty) slot gives tn = +inf, tf = -inf and fails.
constexpr float kSlabShrink = 1.0f - 0x1p-16f;
__device__ __forceinline__ bool slab_ordered(float nx, float fx, float ny, float fy, float nz, float fz, V3 o,
                                             V3 id, float tmin, float tmax, float& tnear) {
    float tn = fmaxf(fmaxf((nx - o.x) * id.x, (ny - o.y) * id.y), fmaxf((nz - o.z) * id.z, tmin));
    float tf = fminf(fminf((fx - o.x) * id.x, (fy - o.y) * id.y), fminf((fz - o.z) * id.z, tmax));
    tnear = tn;
    return tn * kSlabShrink <= tf;
}
// True when the segment o + t d, t in [tmin, tmax], provably passes outside the
// sphere s = (centre, radius) of a BLAS, so that no triangle of it can be hit: the
// instance is then not entered. Conservative: the segment point at the clamped
// projection parameter t* (rounded: any segment point bounds the distance from
// above, and the error of t* moves it by at most a few ulps of |c - o|) is compared
// against the radius grown by 2^-16 x (|c - o|_1 + radius), which covers the
// rounding of that distance, of the stored radius and of the watertight test's
// hit point (within a few ulps of |vertex - o| of the triangle). A NaN anywhere
// keeps the instance, as does a |d|^2 outside [2^-100, 2^100] (where the fast
// division could be off).
__device__ __forceinline__ bool sphere_misses(V3 o, V3 d, float tmin, float tmax, float4 s) {
    const float wx = s.x - o.x, wy = s.y - o.y, wz = s.z - o.z;
    const float dd = __fmaf_rn(d.x, d.x, __fmaf_rn(d.y, d.y, d.z * d.z));
    if (!(dd > 0x1p-100f && dd < 0x1p100f)) return false;
    float t = __fdividef(__fmaf_rn(wx, d.x, __fmaf_rn(wy, d.y, wz * d.z)), dd);
    t = fminf(fmaxf(t, tmin), tmax);
    const float qx = __fmaf_rn(t, d.x, -wx), qy = __fmaf_rn(t, d.y, -wy), qz = __fmaf_rn(t, d.z, -wz);
    const float q2 = __fmaf_rn(qx, qx, __fmaf_rn(qy, qy, qz * qz));
    const float r = __fmaf_rn(0x1p-16f, fabsf(wx) + fabsf(wy) + fabsf(wz) + s.w, s.w);
    return q2 > r * r;
}

__device__ __forceinline__ int dir_signs(V3 idir) {
    return (idir.x < 0.0f ? 1 : 0) | (idir.y < 0.0f ? 2 : 0) | (idir.z < 0.0f ? 4 : 0);
}

struct TlasView {
    const float4* __restrict__ nodes;    // global 4-wide nodes
    const DevInstance* __restrict__ instances;
    uint32_t count;
};

struct ClosestHit {
    float t;
    uint32_t inst_input;   // instance input index
    uint32_t prim;
    uint32_t custom;
    float b0, b1, b2;      // barycentric weights of v0, v1, v2
};

// Work counters of one ray (kStats builds only).
struct TraceCounters {
    uint32_t tlas_nodes, blas_nodes, tris, instances;
};

// Accepts every closest-hit candidate.
struct AcceptAll {
    __device__ __forceinline__ bool operator()(uint32_t, uint32_t, uint32_t, float, float, float) const { return true; }
};

// kClosest = false: any-hit, returns at the first accepted triangle.
// skip: closest-hit skips instances whose custom index is flagged 1 in `skip`; for a
// flag of 2 every candidate hit is offered to `accept(instance input, custom index,
// primitive, b0, b1, b2)` first, and a rejected hit leaves the ray going (an
// alpha test).
// start / nstart: when nstart >= 0 the ray visits only the TLAS leaves start[0..nstart)
// (in that order), in place of the TLAS from its root: a superset of the instances
// whose boxes the ray can reach gives the full traversal's result.
template <bool kClosest, bool kStats = false, typename Accept = AcceptAll>
__device__ __forceinline__ bool trace_ray(const TlasView& T, V3 wo, V3 wd, float tmin, float tmax,
                                          uint32_t ray_mask, const uint8_t* __restrict__ skip,
                                          uint32_t skip_count, ClosestHit* hit, uint32_t& err,
                                          TraceCounters* cnt = nullptr, const Accept& accept = Accept(),
                                          const uint32_t* start = nullptr, int nstart = -1) {
    if (T.count == 0 || nstart == 0) return false;
    if (!finite3(wo) || !finite3(wd) || !(tmin <= tmax)) return false;
    if (wd.x == 0.0f && wd.y == 0.0f && wd.z == 0.0f) return false;
    const V3 widir = safe_inv(wd);
    V3 o = wo, idir = widir;
    int signs = dir_signs(idir);
    const float tmin_box = fmaxf(tmin, 0.0f);   // the entry shrink wants tn >= 0; callers pass tmin >= 0
    WtRay wt{};
    int stack[kStackSize];
    int sp = 0;
    int node = 0;
    if (nstart > 0) {   // nstart <= kStackSize: the caller's lists are short
        node = ~(int)start[0];
        for (int k = nstart - 1; k >= 1; --k) stack[sp++] = ~(int)start[k];
    }
    bool in_blas = false;
    const float4* __restrict__ nodes = T.nodes;
    const float4* __restrict__ tris = nullptr;
    uint32_t inst_input = 0, inst_custom = 0;
    bool inst_tested = false;
    bool found = false;
    unsigned long long best_key = ~0ull;
    for (uint32_t iter = 0;; ++iter) {
        if (iter > kTraversalCap) { err |= LUZ_DEV_TRAVERSAL_CAP; return false; }
        bool pop = true;
        if (node >= 0) {
            if (kStats) { if (in_blas) cnt->blas_nodes++; else cnt->tlas_nodes++; }
            const float4* np = nodes + (size_t)node * kNode4F4;
            const int sx = signs & 1, sy = (signs >> 1) & 1, sz = signs >> 2;
            const float4 nx = __ldg(np + sx), fx = __ldg(np + (sx ^ 1)), ny = __ldg(np + 2 + sy),
                         fy = __ldg(np + 3 - sy), nz = __ldg(np + 4 + sz), fz = __ldg(np + 5 - sz), cf = __ldg(np + 6);
            int ch[4] = {__float_as_int(cf.x), __float_as_int(cf.y), __float_as_int(cf.z), __float_as_int(cf.w)};
            float tn[4];
            bool h[4];
            h[0] = slab_ordered(nx.x, fx.x, ny.x, fy.x, nz.x, fz.x, o, idir, tmin_box, tmax, tn[0]);
            h[1] = slab_ordered(nx.y, fx.y, ny.y, fy.y, nz.y, fz.y, o, idir, tmin_box, tmax, tn[1]);
            h[2] = slab_ordered(nx.z, fx.z, ny.z, fy.z, nz.z, fz.z, o, idir, tmin_box, tmax, tn[2]);
            h[3] = slab_ordered(nx.w, fx.w, ny.w, fy.w, nz.w, fz.w, o, idir, tmin_box, tmax, tn[3]);
            // Misses sort last; a network of five compare-exchanges orders the hits by
            // entry distance (constant indices keep everything in registers).
            const float inf = __int_as_float(0x7f800000);
#pragma unroll
            for (int k = 0; k < 4; ++k) if (!h[k]) tn[k] = inf;
#define LUZ_CX(a, b)                                                              \
            if (tn[b] < tn[a]) {                                                  \
                float tt = tn[a]; tn[a] = tn[b]; tn[b] = tt;                      \
                int tc = ch[a]; ch[a] = ch[b]; ch[b] = tc;                        \
                bool th = h[a]; h[a] = h[b]; h[b] = th;                           \
            }
            LUZ_CX(0, 1) LUZ_CX(2, 3) LUZ_CX(0, 2) LUZ_CX(1, 3) LUZ_CX(1, 2)
#undef LUZ_CX
            if (h[0]) {
#pragma unroll
                for (int k = 3; k >= 1; --k) {
                    if (!h[k]) continue;
                    if (sp >= kStackSize) { err |= LUZ_DEV_STACK_OVERFLOW; return false; }
                    stack[sp++] = ch[k];
                }
                node = ch[0];
                pop = false;
            }
        } else if (!in_blas) {
            if (kStats) cnt->instances++;
            const DevInstance* I = T.instances + (~node);
            const float4* wp = reinterpret_cast<const float4*>(I->w2o);
            float4 r0 = __ldg(wp), r1 = __ldg(wp + 1), r2 = __ldg(wp + 2), sph = __ldg(&I->sphere);
            const float4* pnodes = I->nodes4;
            const float4* ptris = I->tris;
            uint4 meta = __ldg(reinterpret_cast<const uint4*>(&I->custom_index));
            // meta = (custom_index, mask, input_index, blas_prims)
            bool take = (meta.y & ray_mask) != 0 && meta.w > 0;
            bool tested = false;
            if (kClosest && take && skip && meta.x < skip_count) {
                take = skip[meta.x] != 1;
                tested = skip[meta.x] == 2;
            }
            // Skipped too when the segment provably misses the BLAS's bounding sphere.
            const float m[12] = {r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w, r2.x, r2.y, r2.z, r2.w};
            const V3 oo = xform_point(m, wo), od = xform_dir(m, wd);
            if (take && !sphere_misses(oo, od, tmin, tmax, sph)) {
                if (sp >= kStackSize) { err |= LUZ_DEV_STACK_OVERFLOW; return false; }
                stack[sp++] = kStackMarker;
                o = oo;
                idir = safe_inv(od);
                signs = dir_signs(idir);
                wt = wt_setup(oo, od);
                in_blas = true;
                nodes = pnodes;
                tris = ptris;
                inst_input = meta.z;
                inst_custom = meta.x;
                inst_tested = tested;
                node = 0;
                pop = false;
            }
        } else {
            if (kStats) cnt->tris++;
            const float4* tp = tris + (size_t)(~node) * kTriF4;
            float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
            float t, U, V, W, det;
            if (wt_test(wt, V3{a.x, a.y, a.z}, V3{b.x, b.y, b.z}, V3{c.x, c.y, c.z}, t, U, V, W, det) &&
                t >= tmin && t <= tmax) {
                if (!kClosest) return true;
                uint32_t prim = (uint32_t)__float_as_int(a.w);
                unsigned long long key = ((unsigned long long)inst_input << 32) | prim;
                if ((!found || t < tmax || key < best_key) &&
                    (!inst_tested || accept(inst_input, inst_custom, prim, U / det, V / det, W / det))) {
                    found = true;
                    tmax = t;
                    best_key = key;
                    hit->t = t;
                    hit->inst_input = inst_input;
                    hit->prim = prim;
                    hit->custom = inst_custom;
                    hit->b0 = U / det;
                    hit->b1 = V / det;
                    hit->b2 = W / det;
                }
            }
        }
        if (pop) {
            for (;;) {
                if (sp == 0) return found;
                node = stack[--sp];
                if (node == kStackMarker) {
                    in_blas = false;
                    nodes = T.nodes;
                    o = wo;
                    idir = widir;
                    signs = dir_signs(idir);
                    continue;
                }
                break;
            }
        }
    }
}

}  // namespace luz
