// visibility.cu — the persistent wavefront kernel that traces every shadow and AO ray
// of a frame (light.frag:86-135) and writes the hit/miss bit planes; and its batched
// form, one launch over the rays of many scenes.
//
// Work items are (slot, lit pixel) pairs, slot-major, so neighbouring items share a
// light and lie in neighbouring pixels. Each lane holds one ray as an explicit
// traversal state. After every few traversal steps the warp counts its idle lanes
// with a ballot; when enough are idle, one lane takes that many items with a single
// atomic and the idle lanes pick theirs by rank (popc of the lower lanes' ballot
// bits), then generate their rays while the others keep traversing.
//
// Traversal runs over 4-wide nodes (the even-depth collapse of the binary LBVH):
// one step tests four child boxes, with the near and far planes picked per ray by
// the direction's signs. Nodes and triangles come through 16-B vector loads (the
// TLAS top can also be staged in shared memory); the stack is warp-interleaved in
// shared memory (entry k of lane l at [k][l]) with a local-memory tail for rare deep
// paths. Only the state a node step needs stays in registers; the rest of a ray
// (world origin and direction, output bit, watertight shear) sits in shared memory,
// which keeps the kernel at 64 registers and 4 CTAs per SM without spills.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "vis_trace.cuh"

namespace luz {

// ---------------------------------------------------------------- near lists
// A ray whose whole segment stays within `reach` of its own instance's box can only
// hit instances whose boxes come within `reach` of that box: for such a ray the
// traversal starts at its own TLAS leaf with the leaves of those of them whose boxes
// its segment overlaps on its stack, in place of the TLAS root. Short rays (AO rays of
// radius aoMax) then skip the TLAS levels above their own instance. Per instance
// (input order) the record holds (leaf, count, near[0..1]), (near[2..5]), (box lo,
// near[6]), (box hi, near[7]), near[] as input indices; count = ~0 when there are more
// than kNearMax such instances or the box is empty or not finite. The result is that
// of the full traversal: a hit at q on instance j needs box_j within
// |q - o| + dist(o, box_i) of box_i and the segment to overlap box_j, and entering an
// instance whose leaf box the full traversal would cull finds no hit either (boxes
// are conservative).
constexpr uint32_t kNearMax = 8;
// Shadow-ray beams: groups of kBeamGroup consecutive items (lanes of a warp in ray
// generation), lists of up to kBeamMax TLAS leaves.
#ifndef LUZ_BEAM_SHIFT
#define LUZ_BEAM_SHIFT 5
#endif
constexpr uint32_t kBeamShift = LUZ_BEAM_SHIFT;
constexpr uint32_t kBeamGroup = 1u << kBeamShift;
constexpr uint32_t kBeamMax = 31;             // list room: count + 31 leaves (128 B per group)
constexpr uint32_t kBeamWords = kBeamMax + 1;
// Leaves a list may hold before its group falls back to the TLAS root: 15 up to 2048
// instances, 31 above. The traversal kernel is built for each cap (its start loop
// reads that many): on the 1080p two-level frame the longer lists cost 0.5 % of the
// traversal and 3 % of the list kernel, on the 4096-instance scene they take the TLAS
// visits per traversed ray from 3.1 to 0.9.
constexpr uint32_t kBeamCapSmall = 15, kBeamCapLarge = 31;
inline uint32_t beam_cap(uint32_t instances) { return instances > 2048 ? kBeamCapLarge : kBeamCapSmall; }
#ifndef LUZ_NEAR_REACH
#define LUZ_NEAR_REACH 1.5f
#endif
constexpr uint32_t kNearFlag = 0x80000000u;   // rays_b.w: the ray starts at its near list
constexpr uint32_t kNearLeafBits = 24;        // rays_c: own leaf | overlapped near[] bits << 24
constexpr uint32_t kNearMaxInstances = 16384; // pairs tested per call: 2.7e8 at most

__device__ __forceinline__ bool box_ok(float4 lo, float4 hi) {
    return lo.x <= hi.x && lo.y <= hi.y && lo.z <= hi.z;   // false for empty or NaN boxes
}
__device__ __forceinline__ float box_mag(float4 lo, float4 hi) {
    return fmaxf(fmaxf(fmaxf(fabsf(lo.x), fabsf(lo.y)), fmaxf(fabsf(lo.z), fabsf(hi.x))),
                 fmaxf(fabsf(hi.y), fabsf(hi.z)));
}

// One block per instance i: the instances (other than i, with valid boxes) whose box
// distance to box_i is at most reach, grown by 2^-10 relative and 2^-18 of the boxes'
// coordinate magnitude (the rounding of the distances here and in near_start), in
// index order.
__global__ void __launch_bounds__(256) near_list_kernel(const float4* __restrict__ inst_box,
                                                        const uint32_t* __restrict__ leaf_of, uint32_t n,
                                                        float reach, uint4* __restrict__ near) {
    __shared__ uint32_t s_warp[8];
    __shared__ uint32_t s_list[kNearMax];
    const uint32_t i = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const float4 lo = inst_box[2 * i], hi = inst_box[2 * i + 1];
    const bool valid = box_ok(lo, hi);
    const float mi = box_mag(lo, hi);
    uint32_t total = 0;
    for (uint32_t base = 0; valid && base < n; base += blockDim.x) {
        const uint32_t j = base + tid;
        bool nb = false;
        if (j < n && j != i) {
            const float4 lj = inst_box[2 * j], hj = inst_box[2 * j + 1];
            if (box_ok(lj, hj)) {
                const float dx = fmaxf(fmaxf(lj.x - hi.x, lo.x - hj.x), 0.0f);
                const float dy = fmaxf(fmaxf(lj.y - hi.y, lo.y - hj.y), 0.0f);
                const float dz = fmaxf(fmaxf(lj.z - hi.z, lo.z - hj.z), 0.0f);
                const float d2 = dx * dx + dy * dy + dz * dz;
                const float lim = reach * (1.0f + 0x1p-10f) + 0x1p-18f * (mi + box_mag(lj, hj));
                nb = d2 <= lim * lim;
            }
        }
        const uint32_t bal = __ballot_sync(0xFFFFFFFFu, nb);
        if (lane == 0) s_warp[warp] = __popc(bal);
        __syncthreads();
        uint32_t off = total, sum = 0;
        for (uint32_t w = 0; w < blockDim.x / 32; ++w) {
            if (w < warp) off += s_warp[w];
            sum += s_warp[w];
        }
        const uint32_t pos = off + __popc(bal & ((1u << lane) - 1u));
        if (nb && pos < kNearMax) s_list[pos] = j;
        total += sum;
        __syncthreads();
    }
    if (tid == 0) {
        const uint32_t cnt = valid && total <= kNearMax ? total : 0xFFFFFFFFu;
        uint32_t l[kNearMax];
#pragma unroll
        for (uint32_t k = 0; k < kNearMax; ++k) l[k] = k < cnt ? s_list[k] : 0u;
        near[4 * i] = make_uint4(leaf_of[i], cnt, l[0], l[1]);
        near[4 * i + 1] = make_uint4(l[2], l[3], l[4], l[5]);
        near[4 * i + 2] = make_uint4(__float_as_uint(lo.x), __float_as_uint(lo.y), __float_as_uint(lo.z), l[6]);
        near[4 * i + 3] = make_uint4(__float_as_uint(hi.x), __float_as_uint(hi.y), __float_as_uint(hi.z), l[7]);
    }
}

// Whether the segment o + t d, t in [tmin, tmax], may overlap the box: the slab
// interval with the near / far distances widened by 2^-12 relative (their rounding;
// the inverse direction is that of safe_inv, finite).
__device__ __forceinline__ bool segment_overlaps(V3 o, V3 id, float tmin, float tmax, float4 lo, float4 hi) {
    const float x0 = (lo.x - o.x) * id.x, x1 = (hi.x - o.x) * id.x;
    const float y0 = (lo.y - o.y) * id.y, y1 = (hi.y - o.y) * id.y;
    const float z0 = (lo.z - o.z) * id.z, z1 = (hi.z - o.z) * id.z;
    const float tn = fmaxf(fmaxf(fminf(x0, x1), fminf(y0, y1)), fmaxf(fminf(z0, z1), tmin));
    const float tf = fminf(fminf(fmaxf(x0, x1), fmaxf(y0, y1)), fminf(fmaxf(z0, z1), tmax));
    return tn * (1.0f - 0x1p-12f) <= tf + fabsf(tf) * 0x1p-12f;
}

// The start of a ray of pixel pix at its near list, or ~0: the own instance's TLAS
// leaf | the bits of the near instances whose boxes the segment may overlap << 24.
// The segment's length plus the origin's distance to the box of the pixel's
// primary-hit instance, grown by 2^-10 relative and 2^-18 of the coordinates'
// magnitude, must stay within S.near_reach.
__device__ __forceinline__ uint32_t near_start(const SceneVis& S, V3 o, V3 d, float tmin, float tmax, uint32_t pix) {
    const float len = tmax * sqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
    if (!(len <= S.near_reach)) return ~0u;
    const uint32_t inst = __ldg(S.hit_instance + pix);
    if (inst >= S.instance_count) return ~0u;
    const uint4* rec = S.near + 4 * (size_t)inst;
    const uint4 u0 = __ldg(rec);
    if (u0.y > kNearMax) return ~0u;
    const uint4 u2 = __ldg(rec + 2), u3 = __ldg(rec + 3);
    const float4 lo = make_float4(__uint_as_float(u2.x), __uint_as_float(u2.y), __uint_as_float(u2.z), 0.f),
                 hi = make_float4(__uint_as_float(u3.x), __uint_as_float(u3.y), __uint_as_float(u3.z), 0.f);
    if (!box_ok(lo, hi)) return ~0u;
    const float ex = fmaxf(fmaxf(lo.x - o.x, o.x - hi.x), 0.0f);
    const float ey = fmaxf(fmaxf(lo.y - o.y, o.y - hi.y), 0.0f);
    const float ez = fmaxf(fmaxf(lo.z - o.z, o.z - hi.z), 0.0f);
    const float m = fmaxf(box_mag(lo, hi), fmaxf(fmaxf(fabsf(o.x), fabsf(o.y)), fabsf(o.z)));
    const float r = (sqrtf(ex * ex + ey * ey + ez * ez) + len) * (1.0f + 0x1p-10f) + 0x1p-18f * m;
    if (!(r <= S.near_reach)) return ~0u;
    uint32_t bits = 0;
    if (u0.y > 0) {
        const uint4 u1 = __ldg(rec + 1);
        const uint32_t l[kNearMax] = {u0.z, u0.w, u1.x, u1.y, u1.z, u1.w, u2.w, u3.w};
        const V3 id = safe_inv(d);
#pragma unroll
        for (uint32_t k = 0; k < kNearMax; ++k) {
            if (k >= u0.y) break;
            const uint4* nr = S.near + 4 * (size_t)l[k];
            const uint4 a = __ldg(nr + 2), b = __ldg(nr + 3);
            const float4 nlo = make_float4(__uint_as_float(a.x), __uint_as_float(a.y), __uint_as_float(a.z), 0.f),
                         nhi = make_float4(__uint_as_float(b.x), __uint_as_float(b.y), __uint_as_float(b.z), 0.f);
            if (segment_overlaps(o, id, tmin, tmax, nlo, nhi)) bits |= 1u << k;
        }
    }
    return u0.x | (bits << kNearLeafBits);
}

// Ray generation pass of one chunk: items [k0, k0 + chunk) of the frame's
// (slot, lit pixel) list, slot-major, one record per item in structure-of-arrays
// form: rays_a = (origin, tMax), rays_b = (direction, pixel). An item with no ray
// gets tMax = -inf (its AO miss is recorded here) and no rays_b entry. Separated from traversal so the
// long arithmetic of light.frag's sampling runs on full warps, not on the few idle
// lanes of a traversing warp. Also resets the traversal's work counter.
__global__ void __launch_bounds__(256, 5) raygen_kernel(SceneVis S, VisCommon C, unsigned long long k0,
                                                     unsigned long long chunk, float4* __restrict__ rays_a,
                                                     float4* __restrict__ rays_b, uint32_t* __restrict__ rays_c,
                                                     float4* __restrict__ beams) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *C.work_counter = 0ull;
    const uint32_t lit = *S.lit_count;
    const unsigned long long total = (unsigned long long)lit * (S.shadow_slots + S.ao_samples);
    if (k0 >= total) return;
    const unsigned long long end = min(total, k0 + chunk);
    const uint32_t stride = gridDim.x * blockDim.x, lane = threadIdx.x & 31;
    const unsigned long long shadow_items = (unsigned long long)lit * S.shadow_slots;
    const float ninf = __int_as_float(0xff800000);
    // (slot, j) of the thread's first item by one division, then stepped by the stride.
    // The loop runs while any lane of the warp has an item (the beam reductions below
    // take the whole warp): a warp's 32 items are consecutive and 32-aligned.
    unsigned long long item = k0 + blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t slot = (uint32_t)(item / lit), j = (uint32_t)(item - (unsigned long long)slot * lit);
    const uint32_t step_slot = stride / lit, step_j = stride - step_slot * lit;
    for (; item - lane < end; item += stride) {
        const bool live = item < end;
        V3 wo{0.f, 0.f, 0.f}, wd{0.f, 0.f, 0.f};
        float tmin = 0.f, tmax = 0.f;
        uint32_t* out;
        bool record_hit = false;
        uint32_t pix;
        const bool ok = live && gen_ray(S, C, slot, j, wo, wd, tmin, tmax, out, record_hit, pix);
        if (live) rays_a[item - k0] = make_float4(wo.x, wo.y, wo.z, ok ? tmax : ninf);
        if (ok) {   // read only for rays
            uint32_t tag = pix;
            if (S.near_reach > 0.0f && !record_hit) {   // AO rays (shadow rays have their beams)
                const uint32_t start = near_start(S, wo, wd, tmin, tmax, pix);
                if (start != ~0u) {
                    tag |= kNearFlag;
                    rays_c[item - k0] = start;
                }
            }
            rays_b[item - k0] = make_float4(wd.x, wd.y, wd.z, __uint_as_float(tag));
        }
        if (beams && item - lane < shadow_items) {
            // Beam of a group of kBeamGroup items (lanes): balls around the origins and
            // around the end points of its traced shadow rays, centred on the first such ray.
            const bool sh = ok && record_hit;
            const uint32_t first = lane & ~(kBeamGroup - 1u);
            const uint32_t m = (__ballot_sync(0xFFFFFFFFu, sh) >> first) & (0xFFFFFFFFu >> (32 - kBeamGroup));
            const unsigned long long g = (item - k0) >> kBeamShift;
            if (m == 0u) {
                if (lane == first) beams[2 * g] = make_float4(0.f, 0.f, 0.f, -1.0f);   // no traced shadow ray
            }
            {
                const int src = (int)first + (m ? __ffs(m) - 1 : 0);
                const V3 e = V3{wo.x + wd.x * tmax, wo.y + wd.y * tmax, wo.z + wd.z * tmax};
                const V3 co = V3{__shfl_sync(0xFFFFFFFFu, wo.x, src), __shfl_sync(0xFFFFFFFFu, wo.y, src),
                                 __shfl_sync(0xFFFFFFFFu, wo.z, src)};
                const V3 ce = V3{__shfl_sync(0xFFFFFFFFu, e.x, src), __shfl_sync(0xFFFFFFFFu, e.y, src),
                                 __shfl_sync(0xFFFFFFFFu, e.z, src)};
                float ro = sh ? length(wo - co) : 0.0f, re = sh ? length(e - ce) : 0.0f;
                uint32_t bad = sh && !(finite3(e) && ro <= 3.0e38f && re <= 3.0e38f) ? 1u : 0u;
#pragma unroll
                for (int o = kBeamGroup / 2; o >= 1; o >>= 1) {
                    ro = fmaxf(ro, __shfl_xor_sync(0xFFFFFFFFu, ro, o));
                    re = fmaxf(re, __shfl_xor_sync(0xFFFFFFFFu, re, o));
                    bad |= __shfl_xor_sync(0xFFFFFFFFu, bad, o);
                }
                if (lane == first && m != 0u) {   // r_o = +inf: an end point not finite
                    beams[2 * g] = make_float4(co.x, co.y, co.z, bad ? __int_as_float(0x7f800000) : ro);
                    beams[2 * g + 1] = make_float4(ce.x, ce.y, ce.z, re);
                }
            }
        }
        slot += step_slot;
        j += step_j;
        if (j >= lit) { j -= lit; ++slot; }
    }
}

// ---------------------------------------------------------------- beam lists
// The traced shadow rays of a group of kBeamGroup consecutive items (one light sample,
// neighbouring lit pixels in tile order) start in a ball B_o around their origins and
// end in a ball B_e around their end points, so each lies in the convex hull of the
// two balls, itself inside the capsule of radius max(r_o, r_e) around the segment
// between the centres. A leaf whose box, grown by that radius, the segment misses
// cannot be hit by any ray of the group: the group's rays traverse only the leaves the
// capsule reaches (nearest first), or the TLAS from its root when there are more than
// S.beam_cap of them. The radius is grown by 2^-10 relative and 2^-16 of the centres'
// magnitude, above the rounding of the centres, radii, end points and hit points.
constexpr uint32_t kBeamAll = 0xFFFFFFFFu;    // count: traverse from the TLAS root
constexpr int kBeamStack = 48;                 // overflow: the list falls back to the TLAS root

__global__ void __launch_bounds__(256) beam_list_kernel(SceneVis S, unsigned long long k0, unsigned long long chunk,
                                                        const float4* __restrict__ beams, uint32_t* __restrict__ lists) {
    const uint32_t lit = *S.lit_count;
    const unsigned long long shadow_items = (unsigned long long)lit * S.shadow_slots;
    if (k0 >= shadow_items) return;
    const unsigned long long n = min(chunk, shadow_items - k0);
    const unsigned long long g = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= (n + kBeamGroup - 1) / kBeamGroup) return;
    uint32_t* list = lists + kBeamWords * g;
    const float4 bo = beams[2 * g], be = beams[2 * g + 1];
    if (bo.w < 0.0f) return;   // no traced shadow ray in the group: the list is never read
    const V3 o = V3{bo.x, bo.y, bo.z}, d = V3{be.x - bo.x, be.y - bo.y, be.z - bo.z};
    const float r0 = fmaxf(bo.w, be.w);
    const float mag = ((fabsf(bo.x) + fabsf(bo.y)) + (fabsf(bo.z) + fabsf(be.x))) + (fabsf(be.y) + fabsf(be.z));
    const float r = r0 * (1.0f + 0x1p-10f) + 0x1p-16f * (mag + r0);
    if (!(r <= 3.0e38f) || !finite3(o) || !finite3(d)) {
        list[0] = kBeamAll;
        return;
    }
    const V3 id = safe_inv(d);
    uint32_t out[kBeamMax];
    uint32_t cnt = 0;
    int stack[kBeamStack];
    int sp = 0, node = 0;
    bool done = false;
    for (uint32_t iter = 0; iter < kTraversalCap; ++iter) {
        const float4* np = S.tlas_nodes + (size_t)node * kNode4F4;
        const float4 lx = __ldg(np), hx = __ldg(np + 1), ly = __ldg(np + 2), hy = __ldg(np + 3), lz = __ldg(np + 4),
                     hz = __ldg(np + 5), cf = __ldg(np + 6);
        const float L[3][4] = {{lx.x, lx.y, lx.z, lx.w}, {ly.x, ly.y, ly.z, ly.w}, {lz.x, lz.y, lz.z, lz.w}};
        const float H[3][4] = {{hx.x, hx.y, hx.z, hx.w}, {hy.x, hy.y, hy.z, hy.w}, {hz.x, hz.y, hz.z, hz.w}};
        const int ch[4] = {__float_as_int(cf.x), __float_as_int(cf.y), __float_as_int(cf.z), __float_as_int(cf.w)};
        float tk[4];
        bool hk[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float ax0 = (L[0][k] - r - o.x) * id.x, ax1 = (H[0][k] + r - o.x) * id.x;
            const float ay0 = (L[1][k] - r - o.y) * id.y, ay1 = (H[1][k] + r - o.y) * id.y;
            const float az0 = (L[2][k] - r - o.z) * id.z, az1 = (H[2][k] + r - o.z) * id.z;
            const float tn = fmaxf(fmaxf(fminf(ax0, ax1), fminf(ay0, ay1)), fmaxf(fminf(az0, az1), 0.0f));
            const float tf = fminf(fminf(fmaxf(ax0, ax1), fmaxf(ay0, ay1)), fminf(fmaxf(az0, az1), 1.0f));
            hk[k] = ch[k] != kEmptyChild && tn <= tf + fabsf(tf) * 0x1p-12f;
            tk[k] = tn;
        }
        // Hit children by entry distance (misses last): leaves appended nearest first,
        // internal nodes pushed farthest first (the nearest is visited next).
        int ck[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            ck[k] = hk[k] ? ch[k] : kEmptyChild;
            if (!hk[k]) tk[k] = __int_as_float(0x7f800000);
        }
#define LUZ_BX(a, b)                                                                          \
        if (tk[b] < tk[a]) {                                                                  \
            const float t_ = tk[a]; tk[a] = tk[b]; tk[b] = t_;                               \
            const int c_ = ck[a]; ck[a] = ck[b]; ck[b] = c_;                                  \
        }
        LUZ_BX(0, 1) LUZ_BX(2, 3) LUZ_BX(0, 2) LUZ_BX(1, 3) LUZ_BX(1, 2)
#undef LUZ_BX
        bool overflow = false;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            if (ck[q] < 0 && ck[q] != kEmptyChild) {
                if (cnt < kBeamMax) out[cnt] = (uint32_t)~ck[q];
                ++cnt;
            }
        }
#pragma unroll
        for (int q = 3; q >= 0; --q) {
            if (ck[q] >= 0) {
                if (sp < kBeamStack) stack[sp++] = ck[q];
                else overflow = true;
            }
        }
        if (overflow || cnt > S.beam_cap) {
            list[0] = kBeamAll;
            return;
        }
        if (sp == 0) {
            done = true;
            break;
        }
        node = stack[--sp];
    }
    if (!done) {   // the step cap ran out
        list[0] = kBeamAll;
        return;
    }
    list[0] = cnt;
    for (uint32_t k = 0; k < cnt; ++k) list[1 + k] = out[k];
}

// The slab test of a TLAS leaf's box for the lane's (world-space) ray, as a 4-wide
// node applies it to the slot holding that leaf.
__device__ __forceinline__ bool leaf_overlaps(const LaneRay& r, const float4* __restrict__ leaf_box, uint32_t leaf) {
    const float4 lo = __ldg(leaf_box + 2 * (size_t)leaf), hi = __ldg(leaf_box + 2 * (size_t)leaf + 1);
    const bool sx = r.signs & 1, sy = (r.signs >> 1) & 1, sz = (r.signs >> 2) & 1;
    float tn;
    return slab_ordered(sx ? hi.x : lo.x, sx ? lo.x : hi.x, sy ? hi.y : lo.y, sy ? lo.y : hi.y, sz ? hi.z : lo.z,
                        sz ? lo.z : hi.z, r, tn);
}

// Traversal of one chunk of generated rays (one scene; the TLAS top may be staged
// in shared memory). Shared memory: staged TLAS nodes, then the stacks, then the
// cold ray state.
template <bool kStats, bool kStaged, uint32_t kCap>
__global__ void __launch_bounds__(kVisThreads, LUZ_VIS_MIN_BLOCKS)
visibility_kernel(SceneVis S, VisCommon C, unsigned long long k0, unsigned long long chunk,
                  const float4* __restrict__ rays_a, const float4* __restrict__ rays_b,
                  const uint32_t* __restrict__ rays_c, unsigned long long* stats) {
    extern __shared__ float4 smem[];
    const uint32_t staged = min(S.tlas_node_count, C.smem_nodes);
    for (uint32_t i = threadIdx.x; i < staged * kNode4F4; i += blockDim.x) smem[i] = __ldg(S.tlas_nodes + i);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t* stack_base = reinterpret_cast<uint32_t*>(smem + staged * kNode4F4);
    uint32_t* s_stack = stack_base + warp * (kSmemStack * 32) + lane;
    const Cold c{reinterpret_cast<float*>(stack_base + kVisThreads * kSmemStack) + threadIdx.x};
    int lstack[kLocalStack];
    __syncthreads();
    const uint32_t full = 0xFFFFFFFFu, lt_mask = (1u << lane) - 1u;
    const uint32_t lit = *S.lit_count;
    const unsigned long long total = (unsigned long long)lit * (S.shadow_slots + S.ao_samples);
    const unsigned long long n = total > k0 ? min(chunk, total - k0) : 0ull;   // items of this chunk
    uint32_t err = 0, rays = 0;
    TraceCounters cnt{0, 0, 0, 0};
    LaneRay r{};
    bool active = false, exhausted = false;
    for (;;) {
        uint32_t idle = __ballot_sync(full, !active);
        if (!exhausted && __popc(idle) >= (int)C.refill) {
            int leader = __ffs(idle) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(C.work_counter, (unsigned long long)__popc(idle));
            base = __shfl_sync(full, base, leader);
            if (base + __popc(idle) >= n) exhausted = true;
            // Slot of the warp's first item, by one division in the leader; the
            // lanes step from it (their items follow in rank order).
            uint32_t slot0 = 0, j0 = 0;
            if (lane == leader && base < n) {
                const unsigned long long g = k0 + base;
                slot0 = (uint32_t)(g / lit);
                j0 = (uint32_t)(g - (unsigned long long)slot0 * lit);
            }
            slot0 = __shfl_sync(full, slot0, leader);
            j0 = __shfl_sync(full, j0, leader);
            if (!active) {
                const uint32_t rank = __popc(idle & lt_mask);
                const unsigned long long local = base + rank;
                if (local < n) {
                    uint32_t slot = slot0, j = j0 + rank;
                    while (j >= lit) { j -= lit; ++slot; }
                    const float4 a = __ldg(rays_a + local);
                    const bool record_hit = slot < S.shadow_slots;
                    const float tmin = record_hit ? 0.001f : S.ao_min;
                    if (tmin <= a.w) {
                        const float4 b = __ldg(rays_b + local);
                        if (kStats) ++rays;
                        const uint32_t tag = __float_as_uint(b.w), pix = tag & ~kNearFlag;
                        uint32_t* out = record_hit ? S.shadow_bits + (size_t)slot * S.words + (pix >> 5)
                                                   : S.ao_bits + (size_t)(slot - S.shadow_slots) * S.words + (pix >> 5);
                        start_ray(r, c, S, V3{a.x, a.y, a.z}, V3{b.x, b.y, b.z}, tmin, a.w, out, record_hit, pix);
                        bool go = true;
                        if (record_hit && S.beam_lists) {
                            // A shadow ray starts at its group's beam list unless that ran over.
                            const uint4* bl = reinterpret_cast<const uint4*>(S.beam_lists + kBeamWords * (local >> kBeamShift));
                            const uint4 u0 = __ldg(bl);
                            if (u0.x != kBeamAll) {
                                // The list's leaves whose boxes this ray's slab test keeps
                                // (the test the TLAS node holding the leaf would apply),
                                // the nearest first: it starts at the nearest, the others
                                // stacked; with none it ends unoccluded.
                                int sp = 0, cur = 0;
#pragma unroll
                                for (int q = (int)(kCap + 1) / 4 - 1; q >= 0; --q) {
                                    if (4u * (uint32_t)q > u0.x) continue;
                                    const uint4 u = q == 0 ? u0 : __ldg(bl + q);
                                    const uint32_t l[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
                                    for (int k = 3; k >= 0; --k) {
                                        const uint32_t w = 4u * (uint32_t)q + (uint32_t)k;
                                        if (w >= 1 && w <= u0.x && leaf_overlaps(r, S.leaf_box, l[k])) {
                                            if (cur) {   // past the shared part (kCap 31): local
                                                if (kCap < kSmemStack || sp < kSmemStack) s_stack[sp * 32] = (uint32_t)cur;
                                                else lstack[sp - kSmemStack] = cur;
                                                ++sp;
                                            }
                                            cur = ~(int)l[k];
                                        }
                                    }
                                }
                                go = cur != 0;
                                r.node = cur;
                                r.sp = sp;
                            }
                        }
                        if (tag & kNearFlag) {
                            // Start at the own instance's leaf, the overlapped near
                            // instances' leaves stacked.
                            const uint32_t start = __ldg(rays_c + local), leaf = start & ((1u << kNearLeafBits) - 1u);
                            r.node = ~(int)leaf;
                            if (start >> kNearLeafBits) {
                                const uint4* rec = S.near + 4 * (size_t)__ldg(S.order + leaf);
                                const uint4 u0 = __ldg(rec), u1 = __ldg(rec + 1);
                                const uint32_t l[kNearMax] = {u0.z, u0.w, u1.x, u1.y, u1.z, u1.w,
                                                              __ldg(rec + 2).w, __ldg(rec + 3).w};
                                int sp = 0;
#pragma unroll
                                for (uint32_t k = 0; k < kNearMax; ++k)
                                    if ((start >> (kNearLeafBits + k)) & 1u) s_stack[(sp++) * 32] = ~__ldg(S.leaf_of + l[k]);
                                r.sp = sp;
                            }
                        }
                        active = go;
                    }
                }
            }
        }
        if (exhausted && __ballot_sync(full, active) == 0) break;
        run_steps<kStats, kStaged>(r, c, active, smem, staged, S.tlas_nodes, S.instances, s_stack, lstack, C.steps,
                                   C.step_cap, err,
                                   cnt);
    }
    if (err) atomicOr(C.status, err);
    if (kStats) flush_stats(stats, rays, cnt);
}

// Many scenes in one launch: item g belongs to the scene s with
// offsets[s] <= g < offsets[s+1]; each lane carries its scene's TLAS and outputs.
template <bool kStats>
__global__ void __launch_bounds__(kVisThreads, LUZ_VIS_MIN_BLOCKS)
visibility_batch_kernel(const SceneVis* __restrict__ scenes, uint32_t n, const unsigned long long* __restrict__ offsets,
                        VisCommon C, unsigned long long* stats) {
    extern __shared__ float4 smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t* stack_base = reinterpret_cast<uint32_t*>(smem);
    uint32_t* s_stack = stack_base + warp * (kSmemStack * 32) + lane;
    const Cold c{reinterpret_cast<float*>(stack_base + kVisThreads * kSmemStack) + threadIdx.x};
    int lstack[kLocalStack];
    const uint32_t full = 0xFFFFFFFFu, lt_mask = (1u << lane) - 1u;
    const unsigned long long total = offsets[n];
    uint32_t err = 0, rays = 0;
    TraceCounters cnt{0, 0, 0, 0};
    LaneRay r{};
    bool active = false, exhausted = false;
    for (;;) {
        uint32_t idle = __ballot_sync(full, !active);
        if (!exhausted && __popc(idle) >= (int)C.refill) {
            int leader = __ffs(idle) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(C.work_counter, (unsigned long long)__popc(idle));
            base = __shfl_sync(full, base, leader);
            if (base + __popc(idle) >= total) exhausted = true;
            if (!active) {
                unsigned long long item = base + __popc(idle & lt_mask);
                if (item < total) {
                    uint32_t lo = 0, hi = n - 1;
                    while (lo < hi) {
                        uint32_t mid = (lo + hi + 1) >> 1;
                        if (offsets[mid] <= item) lo = mid; else hi = mid - 1;
                    }
                    const SceneVis& S = scenes[lo];
                    uint32_t lit = *S.lit_count;
                    unsigned long long local = item - offsets[lo];
                    uint32_t slot = (uint32_t)(local / lit);
                    uint32_t j = (uint32_t)(local - (unsigned long long)slot * lit);
                    active = setup_ray(r, c, S, C, slot, j);
                    if (kStats && active) ++rays;
                }
            }
        }
        if (exhausted && __ballot_sync(full, active) == 0) break;
        run_steps<kStats, false>(r, c, active, nullptr, 0u, r.tlas, r.insts, s_stack, lstack, C.steps, C.step_cap, err,
                                 cnt);
    }
    if (err) atomicOr(C.status, err);
    if (kStats) flush_stats(stats, rays, cnt);
}

// offsets[s] = rays of scenes 0..s-1 (lit pixels x samples), read after the
// G-buffer passes have counted the lit pixels.
__global__ void batch_offsets_kernel(const SceneVis* scenes, uint32_t n, unsigned long long* offsets) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    unsigned long long acc = 0;
    for (uint32_t s = 0; s < n; ++s) {
        offsets[s] = acc;
        acc += (unsigned long long)(*scenes[s].lit_count) * (scenes[s].shadow_slots + scenes[s].ao_samples);
    }
    offsets[n] = acc;
}

// ---------------------------------------------------------------- host side
// Defaults: the best shape of a sweep on the 1080p two-level scene (smem nodes
// {0,128} x refill {2,4,8,16,24} x steps {8,16,32} x CTAs/SM {3,4}, kernel compiled
// for 4 CTAs/SM; steps 16 until the near and beam lists made the rays shorter, then
// refill {16,24,32} x steps {8,16,24}: 8 steps, 2.28 vs 2.33 ms). Staging the TLAS top
// in shared memory did not pay: L1 holds it.
static const VisTuning g_tuning{0, 24, 8, 4, 1};

const VisTuning& vis_tuning(const luz_ctx* ctx) { return ctx->vis_tuning.set ? ctx->vis_tuning : g_tuning; }

SceneVis make_scene_vis(const luz_frame* f, const luz_tlas* t, int frame_index) {
    SceneVis S;
    // 4-wide nodes; node_count (the binary count) bounds the 4-wide count and the
    // size of the nodes4 buffer, so staging that many stays inside it.
    S.tlas_nodes = t->nodes4;
    S.tlas_node_count = t->count ? t->node_count : 0;
    S.instance_count = t->count;
    S.instances = t->instances;
    S.surf = f->surf;
    S.lit_count = f->lit_count;
    S.lights = f->d_lights;
    S.slot_table = f->d_slot_table;
    S.shadow_slots = f->shadow_slots;
    S.ao_samples = f->ao_samples;
    memcpy(S.cam, f->h_scene.cam_pos, 12);
    S.ao_min = f->h_scene.ao_min;
    S.ao_max = f->h_scene.ao_max;
    S.sampler = f->h_scene.sampler;
    S.frame = frame_index;
    S.width = f->width;
    S.words = f->words;
    S.shadow_bits = f->shadow_bits;
    S.ao_bits = f->ao_bits;
    S.cull = f->shadow_cull ? 1 : 0;
    S.near = t->near;
    S.order = t->order;
    S.leaf_of = t->leaf_of;
    S.hit_instance = f->hit_instance;
    S.near_reach = 0.0f;
    S.beam_lists = nullptr;
    S.leaf_box = nullptr;
    S.beam_cap = 0;
    return S;
}

VisCommon make_vis_common(luz_ctx* ctx, unsigned long long* work_counter) {
    const VisTuning& tu = vis_tuning(ctx);
    VisCommon C;
    C.blue_noise = ctx->d_blue_noise;
    C.bn_size = ctx->blue_noise_size;
    C.work_counter = work_counter;
    C.status = ctx->d_status;
    C.refill = tu.refill;
    C.steps = tu.steps;
    C.smem_nodes = tu.smem_nodes;
    C.step_cap = ctx->debug_step_cap ? ctx->debug_step_cap : kRayStepCap;
    return C;
}

luz_status clear_visibility(luz_ctx* ctx, luz_frame* f) {
    cudaStream_t st = ctx->stream;
    if (f->shadow_slots)
        LUZ_CUDA(ctx, cudaMemsetAsync(f->shadow_bits, 0, (size_t)f->shadow_slots * f->words * 4, st));
    if (f->ao_samples)
        LUZ_CUDA(ctx, cudaMemsetAsync(f->ao_bits, 0, (size_t)f->ao_samples * f->words * 4, st));
    return LUZ_OK;
}


// The traversal of one chunk, built for the scene's beam-list cap.
template <bool kStats, uint32_t kCap>
static void launch_traversal(bool staged, uint32_t grid, size_t smem, cudaStream_t st, const SceneVis& S,
                             const VisCommon& C, unsigned long long k0, unsigned long long chunk, const luz_frame* f,
                             unsigned long long* d_stats) {
    if (staged)
        visibility_kernel<kStats, true, kCap><<<grid, 256, smem, st>>>(S, C, k0, chunk, f->rays_a, f->rays_b,
                                                                       f->rays_c, d_stats);
    else
        visibility_kernel<kStats, false, kCap><<<grid, 256, smem, st>>>(S, C, k0, chunk, f->rays_a, f->rays_b,
                                                                        f->rays_c, d_stats);
}

luz_status launch_visibility(luz_ctx* ctx, luz_frame* f, const luz_tlas* t, int frame_index,
                             unsigned long long* d_stats) {
    luz_status s = clear_visibility(ctx, f);
    if (s != LUZ_OK) return s;
    if ((s = ensure_lit_list(ctx, f)) != LUZ_OK) return s;
    if (f->shadow_slots + f->ao_samples == 0) return LUZ_OK;
    cudaStream_t st = ctx->stream;
    SceneVis S = make_scene_vis(f, t, frame_index);
    VisCommon C = make_vis_common(ctx, f->work_counter);
    const VisTuning& tu = vis_tuning(ctx);
    uint32_t staged = std::min<uint32_t>(S.tlas_node_count, tu.smem_nodes);
    size_t smem = (size_t)staged * kNode4F4 * 16 + kStackBytes + kColdBytes;
    static DeviceSetup setup;   // the traversal kernels' shared-memory limit
    s = device_setup(setup, setup_generation(), smem, [&]() -> luz_status {
        const void* fns[8] = {(const void*)visibility_kernel<false, false, kBeamCapSmall>,
                              (const void*)visibility_kernel<true, false, kBeamCapSmall>,
                              (const void*)visibility_kernel<false, true, kBeamCapSmall>,
                              (const void*)visibility_kernel<true, true, kBeamCapSmall>,
                              (const void*)visibility_kernel<false, false, kBeamCapLarge>,
                              (const void*)visibility_kernel<true, false, kBeamCapLarge>,
                              (const void*)visibility_kernel<false, true, kBeamCapLarge>,
                              (const void*)visibility_kernel<true, true, kBeamCapLarge>};
        for (const void* fn : fns)
            LUZ_CUDA(ctx, cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        return LUZ_OK;
    });
    if (s != LUZ_OK) return s;
    uint32_t grid = (uint32_t)ctx->sm_count * tu.ctas_per_sm;
    if (d_stats) LUZ_CUDA(ctx, cudaMemsetAsync(d_stats, 0, 5 * sizeof(unsigned long long), st));
    // Chunks of at most rays_cap items over the largest possible ray count (every
    // pixel lit); a chunk past the frame's actual count returns at once on the device.
    const unsigned long long max_items = (unsigned long long)f->pixels * (f->shadow_slots + f->ao_samples);
    const uint32_t need = (uint32_t)std::min<unsigned long long>(max_items, kRayChunk);
    if (need > f->rays_cap) {   // first trace of this frame shape: allocate the ray records
        LUZ_CUDA(ctx, cudaStreamSynchronize(st));
        cudaFree(f->rays_a);
        cudaFree(f->rays_b);
        cudaFree(f->rays_c);
        cudaFree(f->beams);
        cudaFree(f->beam_lists);
        f->rays_a = f->rays_b = nullptr;
        f->rays_c = f->beam_lists = nullptr;
        f->beams = nullptr;
        f->rays_cap = 0;
        const size_t groups = ((size_t)need + kBeamGroup - 1) / kBeamGroup;
        LUZ_CUDA(ctx, cudaMalloc(&f->rays_a, (size_t)need * sizeof(float4)));
        LUZ_CUDA(ctx, cudaMalloc(&f->rays_b, (size_t)need * sizeof(float4)));
        LUZ_CUDA(ctx, cudaMalloc(&f->rays_c, (size_t)need * sizeof(uint32_t)));
        LUZ_CUDA(ctx, cudaMalloc(&f->beams, groups * 2 * sizeof(float4)));
        LUZ_CUDA(ctx, cudaMalloc(&f->beam_lists, groups * kBeamWords * sizeof(uint32_t)));
        f->rays_cap = need;
    }
    const unsigned long long chunk = std::min<unsigned long long>(max_items, f->rays_cap);
    // Near lists of this TLAS for the AO rays that stay within LUZ_NEAR_REACH AO radii
    // of their own instance's box. The list kernel tests every pair of instances, so
    // larger TLASes (above kNearMaxInstances) start their AO rays at the root.
    const float reach = LUZ_NEAR_REACH * f->h_scene.ao_max;
    if (t->count > 0 && t->count <= kNearMaxInstances && reach > 0.0f && std::isfinite(reach)) {
        near_list_kernel<<<t->count, 256, 0, st>>>(tlas_instance_boxes(t), t->leaf_of, t->count, reach, t->near);
        LUZ_LAUNCHED(ctx, "near_list_kernel");
        S.near_reach = reach;
    }
    const bool beam = t->count > 0 && f->shadow_slots > 0;
    if (beam) {
        S.beam_lists = f->beam_lists;
        S.leaf_box = tlas_leaf_boxes(t);
    }
    S.beam_cap = beam_cap(t->count);
    if (ctx->raygen_blocks == 0) {   // resident 256-thread blocks per SM: the grid is one wave
        int blocks = 0;
        LUZ_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, raygen_kernel, 256, 0));
        ctx->raygen_blocks = std::max(blocks, 1);
    }
    const int raygen_blocks = ctx->raygen_blocks;
    for (unsigned long long k0 = 0; k0 < max_items; k0 += chunk) {
        prof_begin(ctx, LUZ_KERNEL_RAYGEN);
        raygen_kernel<<<(uint32_t)(ctx->sm_count * raygen_blocks), 256, 0, st>>>(S, C, k0, chunk, f->rays_a,
                                                                                  f->rays_b, f->rays_c,
                                                                                  beam ? f->beams : nullptr);
        LUZ_LAUNCHED(ctx, "raygen_kernel");
        if (beam) {   // timed with ray generation
            const unsigned long long groups = (chunk + kBeamGroup - 1) / kBeamGroup;
            beam_list_kernel<<<(uint32_t)((groups + 255) / 256), 256, 0, st>>>(S, k0, chunk, f->beams, f->beam_lists);
            LUZ_LAUNCHED(ctx, "beam_list_kernel");
        }
        prof_end(ctx);
        if (d_stats) {
            if (S.beam_cap == kBeamCapLarge)
                launch_traversal<true, kBeamCapLarge>(staged, grid, smem, st, S, C, k0, chunk, f, d_stats);
            else
                launch_traversal<true, kBeamCapSmall>(staged, grid, smem, st, S, C, k0, chunk, f, d_stats);
            LUZ_LAUNCHED(ctx, "visibility_kernel<stats>");
        } else {
            prof_begin(ctx, LUZ_KERNEL_TRAVERSAL);
            if (S.beam_cap == kBeamCapLarge)
                launch_traversal<false, kBeamCapLarge>(staged, grid, smem, st, S, C, k0, chunk, f, nullptr);
            else
                launch_traversal<false, kBeamCapSmall>(staged, grid, smem, st, S, C, k0, chunk, f, nullptr);
            prof_end(ctx);
            LUZ_LAUNCHED(ctx, "visibility_kernel");
        }
    }
    return LUZ_OK;
}

luz_status launch_visibility_batch(luz_ctx* ctx, const SceneVis* d_scenes, uint32_t n,
                                   unsigned long long* d_offsets, unsigned long long* work_counter,
                                   unsigned long long* d_stats) {
    cudaStream_t st = ctx->stream;
    batch_offsets_kernel<<<1, 32, 0, st>>>(d_scenes, n, d_offsets);
    LUZ_LAUNCHED(ctx, "batch_offsets_kernel");
    LUZ_CUDA(ctx, cudaMemsetAsync(work_counter, 0, 8, st));
    VisCommon C = make_vis_common(ctx, work_counter);
    const VisTuning& tu = vis_tuning(ctx);
    size_t smem = kStackBytes + kColdBytes;
    uint32_t grid = (uint32_t)ctx->sm_count * tu.ctas_per_sm;
    if (d_stats) {
        LUZ_CUDA(ctx, cudaMemsetAsync(d_stats, 0, 5 * sizeof(unsigned long long), st));
        visibility_batch_kernel<true><<<grid, 256, smem, st>>>(d_scenes, n, d_offsets, C, d_stats);
        LUZ_LAUNCHED(ctx, "visibility_batch_kernel<stats>");
    } else {
        visibility_batch_kernel<false><<<grid, 256, smem, st>>>(d_scenes, n, d_offsets, C, nullptr);
        LUZ_LAUNCHED(ctx, "visibility_batch_kernel");
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
    if (t->smem_nodes > 1024 || t->refill < 1 || t->refill > 32 || t->steps < 1 || t->steps > 1024 ||
        t->ctas_per_sm < 1 || t->ctas_per_sm > 16)
        return set_error(ctx, LUZ_ERR_INVALID, "visibility tuning outside its documented ranges");
    ctx->vis_tuning = VisTuning{t->smem_nodes, t->refill, t->steps, t->ctas_per_sm, 1};
    return LUZ_OK;
}

extern "C" luz_status luz_ctx_get_vis_tuning(const luz_ctx* ctx, luz_vis_tuning* t) {
    using namespace luz;
    if (!ctx || !t) return LUZ_ERR_INVALID;
    const VisTuning& tu = vis_tuning(ctx);
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
