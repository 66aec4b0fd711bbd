// lbvh_device.cuh — device functions of the LBVH builds shared by the build kernels
// (lbvh.cu) and the batched frame kernel (batch.cu): ordered-float bounds, the Karras
// hierarchy node, the bottom-up refit, the 4-wide collapse, the TLAS instance boxes and
// leaves, the breadth-first relayout, and the whole TLAS build by one block.
#pragma once
#include "internal.cuh"
#include "lbvh_kernels.cuh"

namespace luz {

__device__ __forceinline__ uint32_t float_to_ordered(float f) {
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__device__ __forceinline__ float ordered_to_float(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

__device__ __forceinline__ void decode_bounds(const uint32_t* b, V3& cmin, V3& ext) {
    cmin = V3{ordered_to_float(b[0]), ordered_to_float(b[1]), ordered_to_float(b[2])};
    V3 cmax = V3{ordered_to_float(b[3]), ordered_to_float(b[4]), ordered_to_float(b[5])};
    ext = cmax - cmin;
}

__device__ __forceinline__ int kdelta(const unsigned long long* keys, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    uint32_t ki = (uint32_t)keys[i] & 0x3FFFFFFFu, kj = (uint32_t)keys[j] & 0x3FFFFFFFu;
    if (ki != kj) return __clz(ki ^ kj);
    return 32 + __clz((uint32_t)i ^ (uint32_t)j);
}

__device__ __forceinline__ void write_inverted_slot(float4* node, int slot) {
    const float inf = __int_as_float(0x7f800000);
    if (slot == 0) {
        node[0] = make_float4(inf, -inf, inf, -inf);
        node[2].x = inf; node[2].y = -inf;
    } else {
        node[1] = make_float4(inf, -inf, inf, -inf);
        node[2].z = inf; node[2].w = -inf;
    }
}

// seg_node_off: first internal node of each segment (global); sorted keys per segment
// start at seg_prim_off. node_parent / leaf_parent: (local parent << 1) | side.
// Internal node i of segment sd.
__device__ __forceinline__ void karras_node(const SegDesc& sd, int i, const unsigned long long* keys,
                                            uint32_t* node_parent, uint32_t* leaf_parent, uint32_t* dev_status) {
    int n = (int)sd.prim_count;
    float4* node = sd.nodes + (size_t)i * kNodeF4;
    if (n <= 1) {
        // Single node: child0 = leaf 0 (if any), child1 = empty.
        write_inverted_slot(node, 0);
        write_inverted_slot(node, 1);
        int c0 = n == 1 ? ~0 : kEmptyChild;
        node[3] = make_float4(__int_as_float(c0), __int_as_float(kEmptyChild), 0.f, 0.f);
        if (n == 1) leaf_parent[sd.prim_off] = 0u;
        node_parent[sd.node_off] = 0xFFFFFFFFu;
        if (sd.node_range) sd.node_range[0] = make_uint2(0u, 0u);
        return;
    }
    const unsigned long long* k = keys + sd.prim_off;
    int d = (kdelta(k, n, i, i + 1) - kdelta(k, n, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = kdelta(k, n, i, i - d);
    int lmax = 2;
    int guard = 0;
    while (kdelta(k, n, i, i + lmax * d) > dmin) {
        lmax <<= 1;
        if (++guard > 40) { atomicOr(dev_status, (uint32_t)LUZ_DEV_KARRAS_RANGE); return; }
    }
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (kdelta(k, n, i, i + (l + t) * d) > dmin) l += t;
    int j = i + l * d;
    int dnode = kdelta(k, n, i, j);
    int split = 0, step = l;
    do {
        step = (step + 1) >> 1;
        if (kdelta(k, n, i, i + (split + step) * d) > dnode) split += step;
    } while (step > 1);
    int gamma = i + split * d + min(d, 0);
    int lo = min(i, j), hi = max(i, j);
    if (sd.node_range) sd.node_range[i] = make_uint2((uint32_t)lo, (uint32_t)hi);
    int c0, c1;
    if (lo == gamma) { c0 = ~gamma; leaf_parent[sd.prim_off + gamma] = ((uint32_t)i << 1) | 0u; }
    else { c0 = gamma; node_parent[sd.node_off + gamma] = ((uint32_t)i << 1) | 0u; }
    if (hi == gamma + 1) { c1 = ~(gamma + 1); leaf_parent[sd.prim_off + gamma + 1] = ((uint32_t)i << 1) | 1u; }
    else { c1 = gamma + 1; node_parent[sd.node_off + gamma + 1] = ((uint32_t)i << 1) | 1u; }
    node[3] = make_float4(__int_as_float(c0), __int_as_float(c1), 0.f, 0.f);
}

__device__ __forceinline__ void write_slot(float4* node, int slot, float4 lo, float4 hi) {
    if (slot == 0) {
        node[0] = make_float4(lo.x, hi.x, lo.y, hi.y);
        node[2].x = lo.z; node[2].y = hi.z;
    } else {
        node[1] = make_float4(lo.x, hi.x, lo.y, hi.y);
        node[2].z = lo.z; node[2].w = hi.z;
    }
}

// Leaf g (global index) of segment sd: writes its box into its parent and climbs
// while it is the second child to arrive. kBlock: every leaf of the tree is handled
// by one CTA, so block-scope fences order the node writes.
__device__ __forceinline__ uint32_t atomic_add_acq_rel_gpu(uint32_t* p, uint32_t v) {
    uint32_t old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

template <bool kBlock>
__device__ __forceinline__ void refit_leaf(const SegDesc& sd, uint32_t g, const float4* leaf_box,
                                           const uint32_t* node_parent, const uint32_t* leaf_parent,
                                           uint32_t* flags) {
    float4 lo = leaf_box[2 * g], hi = leaf_box[2 * g + 1];
    uint32_t p = leaf_parent[g];
    const uint32_t node_count = sd.prim_count > 1 ? sd.prim_count - 1 : 1;
    // Depth is bounded by the node count; the loop always ends at the root.
    for (uint32_t guard = 0; guard <= sd.prim_count + 1; ++guard) {
        uint32_t local = p >> 1;
        if (p == 0xFFFFFFFFu || local >= node_count) return;
        float4* node = sd.nodes + (size_t)local * kNodeF4;
        write_slot(node, p & 1, lo, hi);
        uint32_t old;
        if (kBlock) {
            __threadfence_block();
            old = atomicAdd(flags + sd.node_off + local, 1u);
            if (old == 0) return;
            __threadfence_block();
        } else {
            // One acquire-release atomic instead of two device-wide fences: its release
            // half publishes this child's slot, its acquire half (for the second
            // arrival) makes the first child's slot visible to the L2 loads below.
            old = atomic_add_acq_rel_gpu(flags + sd.node_off + local, 1u);
            if (old == 0) return;
        }
        float4 n0 = __ldcg(node + 0), n1 = __ldcg(node + 1), n2 = __ldcg(node + 2);
        lo = make_float4(fmin_(n0.x, n1.x), fmin_(n0.z, n1.z), fmin_(n2.x, n2.z), 0.f);
        hi = make_float4(fmax_(n0.y, n1.y), fmax_(n0.w, n1.w), fmax_(n2.y, n2.w), 0.f);
        p = node_parent[sd.node_off + local];
        if (p == 0xFFFFFFFFu) return;
    }
}

// Centre of a BLAS's root box (the union of the root node's two slots).
__device__ __forceinline__ V3 root_centre(float4 n0, float4 n1, float4 n2) {
    V3 lo = V3{fmin_(n0.x, n1.x), fmin_(n0.z, n1.z), fmin_(n2.x, n2.z)};
    V3 hi = V3{fmax_(n0.y, n1.y), fmax_(n0.w, n1.w), fmax_(n2.y, n2.w)};
    return V3{(lo.x + hi.x) * 0.5f + 0.0f, (lo.y + hi.y) * 0.5f + 0.0f, (lo.z + hi.z) * 0.5f + 0.0f};
}

struct Slot4 {
    float lx[4], hx[4], ly[4], hy[4], lz[4], hz[4];
    int ch[4];
    int k;
};

__device__ __forceinline__ void slot4_put(Slot4& s, const float4* n2, int side, int child) {
    float4 a = n2[side], z = n2[2];
    s.lx[s.k] = a.x; s.hx[s.k] = a.y; s.ly[s.k] = a.z; s.hy[s.k] = a.w;
    s.lz[s.k] = side ? z.z : z.x;
    s.hz[s.k] = side ? z.w : z.y;
    s.ch[s.k] = child;
    ++s.k;
}

__device__ __forceinline__ void slot4_store(Slot4& s, float4* out) {
    const float inf = __int_as_float(0x7f800000);
    for (; s.k < 4; ++s.k) {
        s.lx[s.k] = s.ly[s.k] = s.lz[s.k] = inf;
        s.hx[s.k] = s.hy[s.k] = s.hz[s.k] = -inf;
        s.ch[s.k] = kEmptyChild;
    }
    out[0] = make_float4(s.lx[0], s.lx[1], s.lx[2], s.lx[3]);
    out[1] = make_float4(s.hx[0], s.hx[1], s.hx[2], s.hx[3]);
    out[2] = make_float4(s.ly[0], s.ly[1], s.ly[2], s.ly[3]);
    out[3] = make_float4(s.hy[0], s.hy[1], s.hy[2], s.hy[3]);
    out[4] = make_float4(s.lz[0], s.lz[1], s.lz[2], s.lz[3]);
    out[5] = make_float4(s.hz[0], s.hz[1], s.hz[2], s.hz[3]);
    out[6] = make_float4(__int_as_float(s.ch[0]), __int_as_float(s.ch[1]), __int_as_float(s.ch[2]),
                         __int_as_float(s.ch[3]));
    out[7] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// TLAS: the binary tree is in breadth-first order with level table
// levels = {L, start_0, ..., start_L}; the 4-wide nodes are the even levels, in order.
__device__ __forceinline__ void tlas_bvh4_block(const float4* nodes, uint32_t m, const uint32_t* levels,
                                                float4* nodes4) {
    __shared__ uint32_t s_start[66], s_even[66];
    __shared__ uint32_t s_levels;
    if (threadIdx.x == 0) {
        uint32_t L = min(levels[0], 64u);
        s_levels = L;
        uint32_t acc = 0;
        for (uint32_t l = 0; l <= L; ++l) s_start[l] = levels[1 + l];
        for (uint32_t l = 0; l < L; ++l) {
            s_even[l] = acc;
            if ((l & 1u) == 0) acc += s_start[l + 1] - s_start[l];
        }
    }
    __syncthreads();
    const uint32_t L = s_levels;
    for (uint32_t b = threadIdx.x; b < m; b += blockDim.x) {
        uint32_t l = 0;
        while (l + 1 < L && s_start[l + 1] <= b) ++l;
        if (l & 1u) continue;
        const float4* n2 = nodes + (size_t)b * kNodeF4;
        float4 n3 = n2[3];
        int c[2] = {__float_as_int(n3.x), __float_as_int(n3.y)};
        Slot4 s4;
        s4.k = 0;
        for (int side = 0; side < 2; ++side) {
            if (c[side] < 0) {
                slot4_put(s4, n2, side, c[side]);
                continue;
            }
            const float4* mm = nodes + (size_t)c[side] * kNodeF4;
            float4 m3 = mm[3];
            int g[2] = {__float_as_int(m3.x), __float_as_int(m3.y)};
            for (int s2 = 0; s2 < 2; ++s2) {
                int ref = g[s2];
                if (ref >= 0 && l + 2 < L) ref = (int)(s_even[l + 2] + ((uint32_t)ref - s_start[l + 2]));
                slot4_put(s4, mm, s2, ref);
            }
        }
        slot4_store(s4, nodes4 + (size_t)(s_even[l] + (b - s_start[l])) * kNode4F4);
    }
}

// Instance i: shading record, padded world box; returns false when the box centre
// is not finite (no contribution to the Morton bounds).
__device__ __forceinline__ bool tlas_instance_one(const DevInstanceInput* in, uint32_t i, float4* inst_box,
                                                  DevShadeInstance* shade, V3& c) {
    const DevInstanceInput ii = in[i];
    float w2o[12];
    affine_inverse(ii.o2w, w2o);
    DevShadeInstance sh;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) sh.normal_mat[r * 3 + c] = w2o[c * 4 + r];
    sh.pad0 = 0.f;
    sh.vertices = ii.vertices;
    sh.indices = ii.indices;
    shade[i] = sh;
    const float inf = __int_as_float(0x7f800000);
    V3 wlo = V3{inf, inf, inf}, whi = V3{-inf, -inf, -inf};
    if (ii.blas_prims > 0) {
        float4 n0 = ii.nodes[0], n1 = ii.nodes[1], n2 = ii.nodes[2];
        V3 lo = V3{fmin_(n0.x, n1.x), fmin_(n0.z, n1.z), fmin_(n2.x, n2.z)};
        V3 hi = V3{fmax_(n0.y, n1.y), fmax_(n0.w, n1.w), fmax_(n2.y, n2.w)};
        for (int c = 0; c < 8; ++c) {
            V3 p = V3{(c & 1) ? hi.x : lo.x, (c & 2) ? hi.y : lo.y, (c & 4) ? hi.z : lo.z};
            V3 w = xform_point(ii.o2w, p);
            wlo = V3{fmin_(wlo.x, w.x), fmin_(wlo.y, w.y), fmin_(wlo.z, w.z)};
            whi = V3{fmax_(whi.x, w.x), fmax_(whi.y, w.y), fmax_(whi.z, w.z)};
        }
        // Clip with the axis box of the transformed bounding sphere: an ellipsoid
        // c' + M u (|u| <= r) reaches r * |row_a(M)| from its centre along world axis a.
        uint32_t r2 = __float_as_uint(ii.nodes[3].z);
        if (r2 < 0x7F800000u) {
            V3 c = root_centre(n0, n1, n2);
            V3 cw = xform_point(ii.o2w, c);
            float r = sqrtf(__uint_as_float(r2));
            const float* m = ii.o2w;
            float ex = r * sqrtf(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
            float ey = r * sqrtf(m[4] * m[4] + m[5] * m[5] + m[6] * m[6]);
            float ez = r * sqrtf(m[8] * m[8] + m[9] * m[9] + m[10] * m[10]);
            wlo = V3{fmax_(wlo.x, cw.x - ex), fmax_(wlo.y, cw.y - ey), fmax_(wlo.z, cw.z - ez)};
            whi = V3{fmin_(whi.x, cw.x + ex), fmin_(whi.y, cw.y + ey), fmin_(whi.z, cw.z + ez)};
        }
        float px = box_pad(wlo.x, whi.x), py = box_pad(wlo.y, whi.y), pz = box_pad(wlo.z, whi.z);
        wlo = V3{wlo.x - px, wlo.y - py, wlo.z - pz};
        whi = V3{whi.x + px, whi.y + py, whi.z + pz};
    }
    inst_box[2 * i] = make_float4(wlo.x, wlo.y, wlo.z, 0.f);
    inst_box[2 * i + 1] = make_float4(whi.x, whi.y, whi.z, 0.f);
    c = V3{(wlo.x + whi.x) * 0.5f + 0.0f, (wlo.y + whi.y) * 0.5f + 0.0f, (wlo.z + whi.z) * 0.5f + 0.0f};
    return finite3(c);
}

// Leaf j of the sorted order: instance record, leaf box, sorted Morton key and order.
__device__ __forceinline__ void tlas_emit_one(const DevInstanceInput* in, const float4* inst_box, uint32_t j,
                                              unsigned long long key, uint32_t i, DevInstance* inst_out,
                                              float4* leaf_box, uint32_t* morton_out, uint32_t* order_out,
                                              uint32_t* leaf_of_out) {
    morton_out[j] = (uint32_t)key & 0x3FFFFFFFu;
    order_out[j] = i;
    leaf_of_out[i] = j;
    const DevInstanceInput ii = in[i];
    DevInstance d;
    affine_inverse(ii.o2w, d.w2o);
    d.sphere = make_float4(0.f, 0.f, 0.f, __int_as_float(0x7f800000));
    if (ii.blas_prims > 0) {
        const float4 n0 = ii.nodes[0], n1 = ii.nodes[1], n2 = ii.nodes[2];
        const V3 c = root_centre(n0, n1, n2);
        const uint32_t r2 = __float_as_uint(ii.nodes[3].z);
        if (r2 < 0x7F800000u) d.sphere = make_float4(c.x, c.y, c.z, sqrtf(__uint_as_float(r2)));
    }
    d.nodes4 = ii.nodes4;
    d.tris = ii.tris;
    d.custom_index = ii.custom_index;
    d.mask = ii.mask;
    d.input_index = i;
    d.blas_prims = ii.blas_prims;
    inst_out[j] = d;
    leaf_box[2 * j] = inst_box[2 * i];
    leaf_box[2 * j + 1] = inst_box[2 * i + 1];
}

// Breadth-first relayout of one tree by one block (any multiple of 32 threads up to
// 1024). Children of a level keep their parents' order, left before right.
__device__ __forceinline__ void bfs_relayout_block(const float4* src, float4* dst, uint32_t m, uint32_t* queue,
                                                   uint32_t* newidx, uint32_t* levels) {
    __shared__ uint32_t s_warp[32];
    __shared__ uint32_t s_carry;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t nt = blockDim.x, nwarps = nt >> 5;
    if (tid == 0) { queue[0] = 0; newidx[0] = 0; s_carry = 0; }
    __syncthreads();
    uint32_t head = 0, tail = 1, level = 0;
    while (head < tail && tail <= m) {
        uint32_t level_end = tail;
        // level table {L, start_0, ..., start_L} (depth is far below 64 for a TLAS)
        if (tid == 0 && level < 64) levels[1 + level] = head;
        ++level;
        for (uint32_t base = head; base < level_end; base += nt) {
            uint32_t q = base + tid;
            int c0 = 0, c1 = 0;
            uint32_t cnt = 0;
            if (q < level_end) {
                uint32_t old = queue[q];
                float4 n3 = src[(size_t)old * kNodeF4 + 3];
                c0 = __float_as_int(n3.x);
                c1 = __float_as_int(n3.y);
                cnt = (c0 >= 0) + (c1 >= 0);
            }
            // block exclusive scan of cnt
            uint32_t x = cnt;
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
                if (lane >= o) x += y;
            }
            if (lane == 31) s_warp[warp] = x;
            __syncthreads();
            uint32_t wpre = 0, total = 0;
            for (int w = 0; w < (int)nwarps; ++w) {
                uint32_t t = s_warp[w];
                if (w < warp) wpre += t;
                total += t;
            }
            uint32_t pos = tail + s_carry + wpre + x - cnt;
            if (q < level_end) {
                // A tree has exactly m nodes: positions and child indices stay below m.
                if (c0 >= 0) {
                    if (pos < m && (uint32_t)c0 < m) { queue[pos] = (uint32_t)c0; newidx[c0] = pos; }
                    ++pos;
                }
                if (c1 >= 0 && pos < m && (uint32_t)c1 < m) { queue[pos] = (uint32_t)c1; newidx[c1] = pos; }
            }
            __syncthreads();
            if (tid == 0) s_carry += total;
            __syncthreads();
        }
        head = level_end;
        tail = level_end + s_carry;
        __syncthreads();
        if (tid == 0) s_carry = 0;
        __syncthreads();
    }
    if (tid == 0) {
        uint32_t L = level < 64 ? level : 64;
        levels[0] = L;
        levels[1 + L] = tail;
    }
    for (uint32_t old = tid; old < m; old += nt) {
        const float4* s = src + (size_t)old * kNodeF4;
        float4* d = dst + (size_t)newidx[old] * kNodeF4;
        float4 n3 = s[3];
        int c0 = __float_as_int(n3.x), c1 = __float_as_int(n3.y);
        if (c0 >= 0) c0 = (int)newidx[c0];
        if (c1 >= 0) c1 = (int)newidx[c1];
        d[0] = s[0];
        d[1] = s[1];
        d[2] = s[2];
        d[3] = make_float4(__int_as_float(c0), __int_as_float(c1), 0.f, 0.f);
    }
}

// Everything one TLAS build reads and writes (the instance inputs, the TLAS's own
// scratch and its outputs).
struct TlasBuildArgs {
    const DevInstanceInput* in;
    uint32_t n;
    float4* inst_box;
    DevShadeInstance* shade;
    unsigned long long* keys;
    uint32_t* vals;
    float4* karras_nodes;
    uint32_t* node_parent;
    uint32_t* leaf_parent;
    uint32_t* flags;
    DevInstance* inst_out;
    float4* leaf_box;
    uint32_t* morton_out;
    uint32_t* order_out;
    uint32_t* leaf_of_out;      // instance input index -> its leaf
    float4* nodes_out;
    uint32_t* queue;
    uint32_t* newidx;
    uint32_t* levels;
    float4* nodes4;
};

// The whole TLAS build by one block for up to kFusedTlasMax instances (the per-frame
// rebuild of GPUScene::UpdateResourcesGPU is otherwise a chain of ten small launches):
// instance boxes and Morton bounds, Morton keys sorted with their index in shared
// memory (bitonic network; the (key, index) order is the stable order the radix sort
// gives), Karras hierarchy, leaves, refit, breadth-first relayout and 4-wide collapse,
// separated by block barriers. Same results as the multi-kernel path, bit for bit, at
// any block size (a multiple of 32 up to 1024). s_keys: kFusedTlasMax entries of shared
// memory, s_bounds: 6 words of shared memory. Every thread of the block calls it.
// Args: TlasBuildArgs by value where A is a kernel parameter (no local copy of the
// parameter block), const TlasBuildArgs& where it sits in device memory.
constexpr uint32_t kFusedTlasMax = 4096;
template <typename Args>
__device__ __forceinline__ void tlas_build_block(Args A, unsigned long long* s_keys, uint32_t* s_bounds,
                                                 uint32_t* dev_status) {
    const uint32_t tid = threadIdx.x, nt = blockDim.x;
    const uint32_t n = A.n;
    const uint32_t m = max(n, 2u) - 1;
    if (tid < 6) s_bounds[tid] = tid < 3 ? 0xFFFFFFFFu : 0u;
    for (uint32_t q = tid; q < m; q += nt) { A.node_parent[q] = 0xFFFFFFFFu; A.flags[q] = 0u; }
    for (uint32_t g = tid; g < n; g += nt) A.leaf_parent[g] = 0xFFFFFFFFu;
    __syncthreads();
    for (uint32_t i = tid; i < n; i += nt) {
        V3 c;
        if (!tlas_instance_one(A.in, i, A.inst_box, A.shade, c)) continue;
        atomicMin(s_bounds + 0, float_to_ordered(c.x));
        atomicMin(s_bounds + 1, float_to_ordered(c.y));
        atomicMin(s_bounds + 2, float_to_ordered(c.z));
        atomicMax(s_bounds + 3, float_to_ordered(c.x));
        atomicMax(s_bounds + 4, float_to_ordered(c.y));
        atomicMax(s_bounds + 5, float_to_ordered(c.z));
    }
    __syncthreads();
    uint32_t P = 1;
    while (P < n) P <<= 1;
    {
        V3 cmin, ext;
        decode_bounds(s_bounds, cmin, ext);
        for (uint32_t i = tid; i < P; i += nt) {
            if (i < n) {
                const float4 l = A.inst_box[2 * i], h = A.inst_box[2 * i + 1];
                const unsigned long long key = morton30(V3{l.x, l.y, l.z}, V3{h.x, h.y, h.z}, cmin, ext);
                s_keys[i] = (key << 32) | i;
            } else {
                s_keys[i] = ~0ull;
            }
        }
    }
    __syncthreads();
    for (uint32_t k = 2; k <= P; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t i = tid; i < P; i += nt) {
                const uint32_t ixj = i ^ j;
                if (ixj > i) {
                    const unsigned long long a = s_keys[i], b = s_keys[ixj];
                    if ((a > b) == ((i & k) == 0)) { s_keys[i] = b; s_keys[ixj] = a; }
                }
            }
            __syncthreads();
        }
    }
    for (uint32_t j = tid; j < n; j += nt) {
        A.keys[j] = s_keys[j] >> 32;
        A.vals[j] = (uint32_t)s_keys[j];
    }
    __syncthreads();
    SegDesc sd{};
    sd.prim_count = n;
    sd.nodes = A.karras_nodes;
    for (uint32_t q = tid; q < m; q += nt) karras_node(sd, (int)q, A.keys, A.node_parent, A.leaf_parent, dev_status);
    __syncthreads();
    for (uint32_t j = tid; j < n; j += nt)
        tlas_emit_one(A.in, A.inst_box, j, A.keys[j], A.vals[j], A.inst_out, A.leaf_box, A.morton_out, A.order_out,
                      A.leaf_of_out);
    __syncthreads();
    for (uint32_t g = tid; g < n; g += nt) refit_leaf<true>(sd, g, A.leaf_box, A.node_parent, A.leaf_parent, A.flags);
    __syncthreads();
    bfs_relayout_block(A.karras_nodes, A.nodes_out, m, A.queue, A.newidx, A.levels);
    __syncthreads();
    tlas_bvh4_block(A.nodes_out, m, A.levels, A.nodes4);
}

}  // namespace luz
