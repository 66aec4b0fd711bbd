// lbvh.cu — device-built two-level LBVH: BLAS over triangles (batched over many
// meshes as sort segments) and TLAS over instances.
//
// Pipeline (each step a kernel on the context stream):
//   bounds   : centroid bounds per segment (order-preserving uint atomics, exact)
//   morton   : 64-bit key = segment << 30 | morton30(centroid), value = primitive
//   sort     : LSD radix sort, 8-bit digits, one upsweep histogram kernel for all
//              passes + one "onesweep" kernel per pass (tile-local warp multi-split
//              ranking, decoupled look-back across tiles). Stable.
//   karras   : T. Karras, "Maximizing Parallelism in the Construction of BVHs,
//              Octrees, and k-d Trees", HPG 2012 — one thread per internal node,
//              duplicate codes split by index (delta = 32 + clz(i ^ j)).
//   emit     : gather triangles / instances into leaf order, padded leaf boxes
//   refit    : bottom-up, second arrival at a node (atomic flag) merges its children
//   bfs      : (TLAS) breadth-first relayout so that the top of the tree is a prefix
//              of the node array, staged into shared memory by the traversal.
// Replaces the driver builds behind vkw::CmdBuildBLAS / vkw::CmdBuildTLAS
// (source/Graphics/VulkanWrapper.cpp:1089-1139).
#include <algorithm>
#include <cstring>
#include <vector>

#include "internal.cuh"
#include "lbvh_device.cuh"

namespace luz {

// ---------------------------------------------------------------- helpers

__device__ __forceinline__ int find_seg(const uint32_t* offs, int nseg, uint32_t g) {
    int lo = 0, hi = nseg - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (offs[mid] <= g) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ V3 load_pos(const luz_vertex* v, uint32_t i) {
    const float* p = v[i].position;
    return V3{p[0], p[1], p[2]};
}

__device__ __forceinline__ void tri_box(V3 a, V3 b, V3 c, V3& lo, V3& hi) {
    lo = V3{fmin_(fmin_(a.x, b.x), c.x), fmin_(fmin_(a.y, b.y), c.y), fmin_(fmin_(a.z, b.z), c.z)};
    hi = V3{fmax_(fmax_(a.x, b.x), c.x), fmax_(fmax_(a.y, b.y), c.y), fmax_(fmax_(a.z, b.z), c.z)};
}

// Leaf padding of a triangle box (relative 2^-20 of the coordinate magnitude).
__device__ __forceinline__ float leaf_pad(float lo, float hi) {
    return fmax_(fabsf(lo), fabsf(hi)) * 0x1p-20f + 0x1p-100f;
}

// ---------------------------------------------------------------- bounds + morton
// seg_bounds: 6 ordered uints per segment (min xyz, max xyz); init min=~0, max=0.
// A block walks kBoundsIters rows of 256 consecutive primitives. Per row, a warp whose
// lanes all belong to one segment reduces its ordered centroid keys (redux.sync) and
// lane 0 merges them into a running min/max of that segment, which goes to the global
// words (six atomics) only when the segment changes or the block's range ends; a warp
// that straddles a segment boundary issues per-lane atomics. Min and max do not
// depend on the order, so the result is the one of any reduction order.
__global__ void __launch_bounds__(256) blas_bounds_kernel(const SegDesc* segs, const uint32_t* seg_prim_off,
                                                          int nseg, uint32_t total, uint32_t* seg_bounds) {
    const uint32_t full = 0xFFFFFFFFu;
    const bool leader = (threadIdx.x & 31) == 0;
    int acc_s = -1;
    uint32_t acc[6] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u, 0u};
    auto flush = [&]() {
        if (acc_s < 0) return;
        uint32_t* b = seg_bounds + 6 * acc_s;
        for (int a = 0; a < 3; ++a) if (acc[a] != 0xFFFFFFFFu) atomicMin(b + a, acc[a]);
        for (int a = 3; a < 6; ++a) if (acc[a] != 0u) atomicMax(b + a, acc[a]);
    };
    const uint32_t base = blockIdx.x * (blockDim.x * kBoundsIters);
    for (int it = 0; it < kBoundsIters; ++it) {
        const uint32_t row = base + (uint32_t)it * blockDim.x;
        if (row >= total) break;   // uniform across the block
        const uint32_t g = row + threadIdx.x;
        const bool in = g < total;
        const int s = in ? find_seg(seg_prim_off, nseg, g) : -1;
        uint32_t k[6] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u, 0u};
        if (in) {
            const SegDesc sd = segs[s];
            const uint32_t p = g - sd.prim_off;
            const uint32_t i0 = sd.indices[3 * p], i1 = sd.indices[3 * p + 1], i2 = sd.indices[3 * p + 2];
            V3 lo, hi;
            tri_box(load_pos(sd.vertices, i0), load_pos(sd.vertices, i1), load_pos(sd.vertices, i2), lo, hi);
            V3 c = V3{(lo.x + hi.x) * 0.5f + 0.0f, (lo.y + hi.y) * 0.5f + 0.0f, (lo.z + hi.z) * 0.5f + 0.0f};
            if (finite3(c)) {
                k[0] = k[3] = float_to_ordered(c.x);
                k[1] = k[4] = float_to_ordered(c.y);
                k[2] = k[5] = float_to_ordered(c.z);
            }
        }
        const int s0 = __shfl_sync(full, s, 0);
        if (__all_sync(full, s == s0 || s < 0)) {
            uint32_t r[6];
            for (int a = 0; a < 3; ++a) r[a] = __reduce_min_sync(full, k[a]);
            for (int a = 3; a < 6; ++a) r[a] = __reduce_max_sync(full, k[a]);
            if (leader && s0 >= 0) {
                if (s0 != acc_s) {
                    flush();
                    acc_s = s0;
                    for (int a = 0; a < 3; ++a) { acc[a] = 0xFFFFFFFFu; acc[a + 3] = 0u; }
                }
                for (int a = 0; a < 3; ++a) acc[a] = min(acc[a], r[a]);
                for (int a = 3; a < 6; ++a) acc[a] = max(acc[a], r[a]);
            }
        } else if (s >= 0 && k[0] != 0xFFFFFFFFu) {
            uint32_t* b = seg_bounds + 6 * s;
            for (int a = 0; a < 3; ++a) atomicMin(b + a, k[a]);
            for (int a = 3; a < 6; ++a) atomicMax(b + a, k[a]);
        }
    }
    if (leader) flush();
}


__global__ void blas_morton_kernel(const SegDesc* segs, const uint32_t* seg_prim_off, int nseg,
                                   uint32_t total, const uint32_t* seg_bounds,
                                   unsigned long long* keys, uint32_t* vals) {
    uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= total) return;
    int s = find_seg(seg_prim_off, nseg, g);
    const SegDesc sd = segs[s];
    uint32_t p = g - sd.prim_off;
    uint32_t i0 = sd.indices[3 * p], i1 = sd.indices[3 * p + 1], i2 = sd.indices[3 * p + 2];
    V3 lo, hi;
    tri_box(load_pos(sd.vertices, i0), load_pos(sd.vertices, i1), load_pos(sd.vertices, i2), lo, hi);
    V3 cmin, ext;
    decode_bounds(seg_bounds + 6 * s, cmin, ext);
    uint32_t m = morton30(lo, hi, cmin, ext);
    keys[g] = ((unsigned long long)s << 30) | m;
    vals[g] = g;
}

// ---------------------------------------------------------------- onesweep radix sort
__global__ void sort_histogram_kernel(const unsigned long long* keys, uint32_t n, int passes,
                                      uint32_t* hist) {
    __shared__ uint32_t s_hist[kMaxPasses][kRadix];
    for (int i = threadIdx.x; i < kMaxPasses * kRadix; i += blockDim.x) (&s_hist[0][0])[i] = 0;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        unsigned long long k = keys[i];
        for (int p = 0; p < passes; ++p) atomicAdd(&s_hist[p][(k >> (8 * p)) & 0xFF], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * kRadix; i += blockDim.x) {
        uint32_t v = (&s_hist[0][0])[i];
        if (v) atomicAdd(hist + i, v);
    }
}

// Block-wide exclusive scan of one value per thread (blockDim.x == 256).
__device__ __forceinline__ uint32_t block_excl_scan_256(uint32_t v, uint32_t* s_tmp /*8*/,
                                                        uint32_t* total) {
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_tmp[warp] = x;
    __syncthreads();
    uint32_t wsum = 0, all = 0;
    for (int w = 0; w < 8; ++w) {
        uint32_t t = s_tmp[w];
        if (w < warp) wsum += t;
        all += t;
    }
    __syncthreads();
    if (total) *total = all;
    return wsum + x - v;
}

__global__ void sort_scan_kernel(const uint32_t* hist, uint32_t* offsets) {
    __shared__ uint32_t s_tmp[8];
    int p = blockIdx.x;
    uint32_t v = hist[p * kRadix + threadIdx.x];
    offsets[p * kRadix + threadIdx.x] = block_excl_scan_256(v, s_tmp, nullptr);
}

__device__ __forceinline__ uint32_t ld_volatile_u32(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.volatile.global.u32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ void st_volatile_u32(uint32_t* p, uint32_t v) {
    asm volatile("st.volatile.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__global__ void __launch_bounds__(kSortThreads)
onesweep_pass_kernel(const unsigned long long* __restrict__ kin, const uint32_t* __restrict__ vin,
                     unsigned long long* __restrict__ kout, uint32_t* __restrict__ vout, uint32_t n,
                     int shift, const uint32_t* __restrict__ pass_offsets, uint32_t* tile_status,
                     uint32_t* tile_counter, uint32_t* dev_status) {
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_warp_hist[kSortWarps][kRadix];
    __shared__ uint32_t s_digit_excl[kRadix];
    __shared__ uint32_t s_global_base[kRadix];
    __shared__ uint32_t s_tmp[8];
    __shared__ unsigned long long s_keys[kSortTile];
    __shared__ uint32_t s_vals[kSortTile];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_tile = atomicAdd(tile_counter, 1u);
    for (int i = tid; i < kSortWarps * kRadix; i += kSortThreads) (&s_warp_hist[0][0])[i] = 0;
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t base = tile * kSortTile;

    unsigned long long key[kSortItems];
    uint32_t val[kSortItems], dig[kSortItems], rank[kSortItems];
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        uint32_t idx = base + warp * (32 * kSortItems) + k * 32 + lane;
        bool valid = idx < n;
        key[k] = valid ? kin[idx] : 0ull;
        val[k] = valid ? vin[idx] : 0u;
        dig[k] = valid ? (uint32_t)((key[k] >> shift) & 0xFF) : 256u;
    }
    const uint32_t lt_mask = (1u << lane) - 1u;
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        uint32_t d = dig[k];
        uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
        uint32_t before = peers & lt_mask;
        uint32_t cnt = (d < 256) ? s_warp_hist[warp][d] : 0u;
        rank[k] = cnt + __popc(before);
        __syncwarp();
        if (d < 256 && before == 0) s_warp_hist[warp][d] = cnt + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // Digit `tid`: exclusive scan across warps and tile total.
    uint32_t tile_count = 0;
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) {
        uint32_t c = s_warp_hist[w][tid];
        s_warp_hist[w][tid] = tile_count;
        tile_count += c;
    }
    // Decoupled look-back for digit `tid`.
    uint32_t* my_status = tile_status + (size_t)tile * kRadix + tid;
    uint32_t global_base;
    if (tile == 0) {
        global_base = pass_offsets[tid];
        st_volatile_u32(my_status, kFlagPrefix | (global_base + tile_count));
    } else {
        st_volatile_u32(my_status, kFlagAggregate | tile_count);
        uint32_t excl = 0;
        int j = (int)tile - 1;
        uint32_t spins = 0;
        while (j >= 0) {
            uint32_t s = ld_volatile_u32(tile_status + (size_t)j * kRadix + tid);
            uint32_t flag = s & ~kValueMask;
            if (flag == 0) {
                if (++spins > kLookbackSpinLimit) {
                    atomicOr(dev_status, (uint32_t)LUZ_DEV_SORT_LOOKBACK_TIMEOUT);
                    break;
                }
                continue;
            }
            excl += s & kValueMask;
            if (flag == kFlagPrefix) break;
            --j;
        }
        global_base = excl;
        st_volatile_u32(my_status, kFlagPrefix | (excl + tile_count));
    }
    s_global_base[tid] = global_base;
    s_digit_excl[tid] = block_excl_scan_256(tile_count, s_tmp, nullptr);
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        uint32_t d = dig[k];
        if (d < 256) {
            uint32_t pos = s_digit_excl[d] + s_warp_hist[warp][d] + rank[k];
            s_keys[pos] = key[k];
            s_vals[pos] = val[k];
        }
    }
    __syncthreads();
    uint32_t tile_n = min((uint32_t)kSortTile, n - base);
    for (uint32_t i = tid; i < tile_n; i += kSortThreads) {
        unsigned long long k = s_keys[i];
        uint32_t d = (uint32_t)((k >> shift) & 0xFF);
        uint32_t out = s_global_base[d] + (i - s_digit_excl[d]);
        if (out < n) {   // always true unless a look-back timed out (status word raised)
            kout[out] = k;
            vout[out] = s_vals[i];
        }
    }
}

// ---------------------------------------------------------------- Karras hierarchy



__global__ void karras_kernel(const SegDesc* segs, const uint32_t* seg_node_off, int nseg,
                              uint32_t total_nodes, const unsigned long long* keys,
                              uint32_t* node_parent, uint32_t* leaf_parent, uint32_t* dev_status) {
    uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= total_nodes) return;
    int s = find_seg(seg_node_off, nseg, q);
    const SegDesc sd = segs[s];
    karras_node(sd, (int)(q - sd.node_off), keys, node_parent, leaf_parent, dev_status);
}

// ---------------------------------------------------------------- leaves + refit
// BLAS: gather triangles into leaf order; padded leaf boxes; sorted morton/order into
// the segment's own arrays.
__global__ void blas_emit_kernel(const SegDesc* segs, const uint32_t* seg_prim_off, int nseg,
                                 uint32_t total, const unsigned long long* keys,
                                 const uint32_t* vals, float4* leaf_box) {
    uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= total) return;
    int s = find_seg(seg_prim_off, nseg, g);
    const SegDesc sd = segs[s];
    uint32_t j = g - sd.prim_off;
    uint32_t prim = vals[g] - sd.prim_off;
    sd.morton[j] = (uint32_t)keys[g] & 0x3FFFFFFFu;
    sd.order[j] = prim;
    uint32_t i0 = sd.indices[3 * prim], i1 = sd.indices[3 * prim + 1], i2 = sd.indices[3 * prim + 2];
    V3 a = load_pos(sd.vertices, i0), b = load_pos(sd.vertices, i1), c = load_pos(sd.vertices, i2);
    float4* t = sd.tris + (size_t)j * kTriF4;
    t[0] = make_float4(a.x, a.y, a.z, __int_as_float((int)prim));
    t[1] = make_float4(b.x, b.y, b.z, 0.f);
    t[2] = make_float4(c.x, c.y, c.z, 0.f);
    V3 lo, hi;
    tri_box(a, b, c, lo, hi);
    float px = leaf_pad(lo.x, hi.x), py = leaf_pad(lo.y, hi.y), pz = leaf_pad(lo.z, hi.z);
    leaf_box[2 * g] = make_float4(lo.x - px, lo.y - py, lo.z - pz, 0.f);
    leaf_box[2 * g + 1] = make_float4(hi.x + px, hi.y + py, hi.z + pz, 0.f);
}



__global__ void refit_kernel(const SegDesc* segs, const uint32_t* seg_prim_off, int nseg,
                             uint32_t total, const float4* leaf_box, const uint32_t* node_parent,
                             const uint32_t* leaf_parent, uint32_t* flags) {
    uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= total) return;
    int s = find_seg(seg_prim_off, nseg, g);
    refit_leaf<false>(segs[s], g, leaf_box, node_parent, leaf_parent, flags);
}

// The refit with the nodes of a block's own leaves in shared memory. Block b takes the
// kRefitLeaves consecutive leaves [b0, b0 + kRefitLeaves) of the sorted order. An
// internal node whose leaf range (kept by the hierarchy pass) lies inside them has both
// children inside as well, so its two child boxes, its arrival count, its parent and
// its range live in shared memory at index (first leaf of its segment + node index -
// b0): the node index lies in its own leaf range. The climbs through these nodes touch
// shared memory only, and the block writes their slots to device memory at the end,
// one node per thread. The first node whose range leaves the block (and so every node above
// it) goes through refit_leaf's device-memory protocol. Same slots as refit_kernel, bit
// for bit: every box is a min / max union.
__global__ void __launch_bounds__(kRefitLeaves)
refit_local_kernel(const SegDesc* segs, const uint32_t* seg_prim_off, int nseg, uint32_t total,
                   const float4* leaf_box, const uint32_t* node_parent, const uint32_t* leaf_parent,
                   uint32_t* flags) {
    __shared__ float s_box[kRefitLeaves][2][6];   // per local node: child slot 0 / 1 (lo xyz, hi xyz)
    __shared__ uint32_t s_flag[kRefitLeaves];
    __shared__ uint32_t s_parent[kRefitLeaves];   // parent and leaf range of node (g - prim_off)
    __shared__ uint2 s_range[kRefitLeaves];
    const uint32_t b0 = blockIdx.x * kRefitLeaves, g = b0 + threadIdx.x;
    s_flag[threadIdx.x] = 0u;
    int s = 0;
    SegDesc sd{};
    if (g < total) {
        s = find_seg(seg_prim_off, nseg, g);
        sd = segs[s];
        // the node with the index of this leaf position (every leaf position of a segment
        // but its last has one): loaded once, coalesced, for the climbs of the block
        const uint32_t q = g - sd.prim_off;
        if (q + 1 < sd.prim_count) {
            s_parent[threadIdx.x] = node_parent[sd.node_off + q];
            s_range[threadIdx.x] = sd.node_range[q];
        }
    }
    __syncthreads();
    if (g < total) {
        float4 lo = leaf_box[2 * g], hi = leaf_box[2 * g + 1];
        uint32_t p = leaf_parent[g];
        const uint32_t node_count = sd.prim_count > 1 ? sd.prim_count - 1 : 1;
        bool global = sd.prim_count <= 1;   // a one-primitive segment's node has one child (one arrival)
        for (uint32_t guard = 0; guard <= sd.prim_count + 1; ++guard) {
            const uint32_t local = p >> 1;
            if (p == 0xFFFFFFFFu || local >= node_count) break;
            // the node index lies in its own leaf range: a node whose index is outside the
            // block's positions spans other blocks' leaves (and so does every node above it)
            const uint32_t k = sd.prim_off + local - b0;
            if (!global) {
                if (k >= (uint32_t)kRefitLeaves) {
                    global = true;
                } else {
                    const uint2 range = s_range[k];
                    global = sd.prim_off + range.x < b0 || sd.prim_off + range.y >= b0 + kRefitLeaves;
                }
            }
            if (global) {
                float4* node = sd.nodes + (size_t)local * kNodeF4;
                write_slot(node, p & 1, lo, hi);
                if (atomic_add_acq_rel_gpu(flags + sd.node_off + local, 1u) == 0) break;
                const float4 n0 = __ldcg(node + 0), n1 = __ldcg(node + 1), n2 = __ldcg(node + 2);
                lo = make_float4(fmin_(n0.x, n1.x), fmin_(n0.z, n1.z), fmin_(n2.x, n2.z), 0.f);
                hi = make_float4(fmax_(n0.y, n1.y), fmax_(n0.w, n1.w), fmax_(n2.y, n2.w), 0.f);
                p = node_parent[sd.node_off + local];
                continue;
            }
            // local: shared memory only; the block writes these nodes' slots at the end
            float* slot = s_box[k][p & 1];
            slot[0] = lo.x; slot[1] = lo.y; slot[2] = lo.z;
            slot[3] = hi.x; slot[4] = hi.y; slot[5] = hi.z;
            __threadfence_block();
            if (atomicAdd(s_flag + k, 1u) == 0) break;
            __threadfence_block();
            const float* c0 = s_box[k][0];
            const float* c1 = s_box[k][1];
            lo = make_float4(fmin_(c0[0], c1[0]), fmin_(c0[1], c1[1]), fmin_(c0[2], c1[2]), 0.f);
            hi = make_float4(fmax_(c0[3], c1[3]), fmax_(c0[4], c1[4]), fmax_(c0[5], c1[5]), 0.f);
            p = s_parent[k];
        }
    }
    __syncthreads();
    // the slots of every node completed in shared memory (both arrivals), one node per
    // thread at the node of this thread's leaf position
    if (g < total && s_flag[threadIdx.x] == 2u) {
        const float* c0 = s_box[threadIdx.x][0];
        const float* c1 = s_box[threadIdx.x][1];
        float4* node = sd.nodes + (size_t)(g - sd.prim_off) * kNodeF4;
        node[0] = make_float4(c0[0], c0[3], c0[1], c0[4]);
        node[1] = make_float4(c1[0], c1[3], c1[1], c1[4]);
        node[2] = make_float4(c0[2], c0[5], c1[2], c1[5]);
    }
}

// ---------------------------------------------------------------- bounding sphere

// Bounding sphere of every BLAS about its root box centre: the largest squared
// distance of a triangle vertex from the centre, kept as float bits in the root
// node's spare word n3.z (zero after karras_kernel; positive floats order like their
// bits, so atomicMax on the bits is a float max). Runs after the refit. The TLAS
// build intersects each instance's transformed root box with the transformed sphere.
__global__ void blas_radius_kernel(const SegDesc* segs, const uint32_t* seg_prim_off, int nseg,
                                   uint32_t total) {
    uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    bool in = g < total;
    int s = in ? find_seg(seg_prim_off, nseg, g) : -1;
    uint32_t r2 = 0u;
    float4* root = nullptr;
    if (in) {
        const SegDesc sd = segs[s];
        root = sd.nodes;
        V3 c = root_centre(__ldcg(root + 0), __ldcg(root + 1), __ldcg(root + 2));
        const float4* t = sd.tris + (size_t)(g - sd.prim_off) * kTriF4;
        for (int k = 0; k < 3; ++k) {
            float4 v = t[k];
            float dx = v.x - c.x, dy = v.y - c.y, dz = v.z - c.z;
            float d2 = dx * dx + dy * dy + dz * dz;
            r2 = max(r2, __float_as_uint(d2));
        }
    }
    const uint32_t full = 0xFFFFFFFFu;
    int s0 = __shfl_sync(full, s, 0);
    bool uniform = __all_sync(full, s == s0 || s < 0);
    if (uniform) {
        uint32_t r = __reduce_max_sync(full, r2);
        float4* root0 = (float4*)__shfl_sync(full, (unsigned long long)root, 0);
        if ((threadIdx.x & 31) == 0 && s0 >= 0) atomicMax((uint32_t*)&root0[3].z, r);
    } else if (s >= 0) {
        atomicMax((uint32_t*)&root[3].z, r2);
    }
}

// ---------------------------------------------------------------- 4-wide collapse
// Every binary node at even depth becomes a 4-wide node whose slots are its
// grandchildren (or its children, where a child is a leaf). Numbering: the rank of
// the node among its segment's even-depth nodes in binary-node order (root first).

// flags[q] = 1 when internal node q lies at even depth in its segment's tree.
__global__ void even_depth_kernel(const SegDesc* segs, const uint32_t* seg_node_off, int nseg, uint32_t total_nodes,
                                  const uint32_t* node_parent, uint32_t* flags) {
    uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= total_nodes) return;
    int s = find_seg(seg_node_off, nseg, q);
    const uint32_t off = segs[s].node_off;
    uint32_t d = 0, p = node_parent[q];
    for (uint32_t guard = 0; p != 0xFFFFFFFFu && guard < 4096; ++guard) {
        ++d;
        p = node_parent[off + (p >> 1)];
    }
    flags[q] = (d & 1u) == 0u;
}

// Chunked exclusive scan of u32 (chunks of 1024 = 256 threads x 4).
__global__ void __launch_bounds__(256) chunk_sum_kernel(const uint32_t* in, uint32_t n, uint32_t* sums) {
    __shared__ uint32_t s_tmp[8];
    uint32_t base = blockIdx.x * 1024 + threadIdx.x * 4, c = 0;
    for (int k = 0; k < 4; ++k) c += base + k < n ? in[base + k] : 0u;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xFFFFFFFFu, c, o);
    if ((threadIdx.x & 31) == 0) s_tmp[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < 8; ++w) t += s_tmp[w];
        sums[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(1024) chunk_scan_kernel(uint32_t* sums, uint32_t chunks) {
    __shared__ uint32_t s_warp[32];
    __shared__ uint32_t s_carry;
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    for (uint32_t base = 0; base < chunks; base += 1024) {
        uint32_t i = base + threadIdx.x;
        uint32_t v = i < chunks ? sums[i] : 0u, x = v;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) s_warp[warp] = x;
        __syncthreads();
        uint32_t pre = 0, all = 0;
        for (int w = 0; w < 32; ++w) {
            if (w < warp) pre += s_warp[w];
            all += s_warp[w];
        }
        uint32_t carry = s_carry;
        if (i < chunks) sums[i] = carry + pre + x - v;
        __syncthreads();
        if (threadIdx.x == 0) s_carry = carry + all;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256) chunk_apply_kernel(const uint32_t* in, uint32_t n, const uint32_t* offs,
                                                          uint32_t* out) {
    __shared__ uint32_t s_tmp[8];
    uint32_t base = blockIdx.x * 1024 + threadIdx.x * 4;
    uint32_t v[4], c = 0;
    for (int k = 0; k < 4; ++k) { v[k] = base + k < n ? in[base + k] : 0u; c += v[k]; }
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = c;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_tmp[warp] = x;
    __syncthreads();
    uint32_t pre = 0;
    for (int w = 0; w < warp; ++w) pre += s_tmp[w];
    uint32_t run = offs[blockIdx.x] + pre + x - c;
    for (int k = 0; k < 4; ++k) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
}




// idx4[q]: exclusive prefix of the even-depth flags over all segments' nodes.
__global__ void bvh4_emit_kernel(const SegDesc* segs, const uint32_t* seg_node_off, int nseg, uint32_t total_nodes,
                                 const uint32_t* flags, const uint32_t* idx4) {
    uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= total_nodes || !flags[q]) return;
    int s = find_seg(seg_node_off, nseg, q);
    const SegDesc sd = segs[s];
    if (!sd.nodes4) return;
    const uint32_t base4 = idx4[sd.node_off];
    const float4* n2 = sd.nodes + (size_t)(q - sd.node_off) * kNodeF4;
    float4 n3 = n2[3];
    int c[2] = {__float_as_int(n3.x), __float_as_int(n3.y)};
    Slot4 s4;
    s4.k = 0;
    for (int side = 0; side < 2; ++side) {
        if (c[side] < 0) {
            slot4_put(s4, n2, side, c[side]);
            continue;
        }
        const float4* m = sd.nodes + (size_t)c[side] * kNodeF4;
        float4 m3 = m[3];
        int g[2] = {__float_as_int(m3.x), __float_as_int(m3.y)};
        for (int s2 = 0; s2 < 2; ++s2)
            slot4_put(s4, m, s2, g[s2] < 0 ? g[s2] : (int)(idx4[sd.node_off + g[s2]] - base4));
    }
    slot4_store(s4, sd.nodes4 + (size_t)(idx4[q] - base4) * kNode4F4);
}


__global__ void __launch_bounds__(1024) tlas_bvh4_kernel(const float4* nodes, uint32_t m, const uint32_t* levels,
                                                         float4* nodes4) {
    tlas_bvh4_block(nodes, m, levels, nodes4);
}

// ---------------------------------------------------------------- TLAS

__global__ void tlas_instance_kernel(const DevInstanceInput* in, uint32_t n, float4* inst_box,
                                     DevShadeInstance* shade, uint32_t* seg_bounds) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    V3 c;
    if (!tlas_instance_one(in, i, inst_box, shade, c)) return;
    atomicMin(seg_bounds + 0, float_to_ordered(c.x));
    atomicMin(seg_bounds + 1, float_to_ordered(c.y));
    atomicMin(seg_bounds + 2, float_to_ordered(c.z));
    atomicMax(seg_bounds + 3, float_to_ordered(c.x));
    atomicMax(seg_bounds + 4, float_to_ordered(c.y));
    atomicMax(seg_bounds + 5, float_to_ordered(c.z));
}

__global__ void tlas_setup_kernel(uint32_t* bounds, SegDesc* seg, SegDesc value, uint32_t* zero) {
    if (threadIdx.x < 6) bounds[threadIdx.x] = threadIdx.x < 3 ? 0xFFFFFFFFu : 0u;
    if (threadIdx.x == 0) {
        *seg = value;
        *zero = 0;
    }
}

__global__ void tlas_morton_kernel(const float4* inst_box, uint32_t n, const uint32_t* seg_bounds,
                                   unsigned long long* keys, uint32_t* vals) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 l = inst_box[2 * i], h = inst_box[2 * i + 1];
    V3 cmin, ext;
    decode_bounds(seg_bounds, cmin, ext);
    keys[i] = morton30(V3{l.x, l.y, l.z}, V3{h.x, h.y, h.z}, cmin, ext);
    vals[i] = i;
}


__global__ void tlas_emit_kernel(const DevInstanceInput* in, const float4* inst_box, uint32_t n,
                                 const unsigned long long* keys, const uint32_t* vals,
                                 DevInstance* inst_out, float4* leaf_box, uint32_t* morton_out,
                                 uint32_t* order_out, uint32_t* leaf_of_out) {
    uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    tlas_emit_one(in, inst_box, j, keys[j], vals[j], inst_out, leaf_box, morton_out, order_out, leaf_of_out);
}



__global__ void __launch_bounds__(1024)
bfs_relayout_kernel(const float4* src, float4* dst, uint32_t m, uint32_t* queue,
                    uint32_t* newidx, uint32_t* levels) {
    bfs_relayout_block(src, dst, m, queue, newidx, levels);
}

// The TLAS build of tlas_build_block as one CTA of 1024 threads.
__global__ void __launch_bounds__(1024) tlas_fused_kernel(TlasBuildArgs A, uint32_t* dev_status) {
    __shared__ unsigned long long s_keys[kFusedTlasMax];
    __shared__ uint32_t s_bounds[6];
    tlas_build_block<TlasBuildArgs>(A, s_keys, s_bounds, dev_status);
}

// ---------------------------------------------------------------- host drivers
static inline uint32_t cdiv(uint64_t a, uint64_t b) { return (uint32_t)((a + b - 1) / b); }

static int passes_for(int nseg) {
    int bits = 30;
    int sb = 0;
    while ((1 << sb) < nseg) ++sb;
    return (bits + sb + 7) / 8;
}

struct SortBuffers {
    unsigned long long* keys[2];
    uint32_t* vals[2];
    uint32_t* hist;       // passes * 256
    uint32_t* offsets;    // passes * 256
    uint32_t* tile_status;  // passes * tiles * 256
    uint32_t* tile_counter; // passes
    uint32_t tiles;
};

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Bytes of scratch for a sort of n keys with `passes` passes.
static size_t sort_scratch_bytes(uint32_t n, int passes) {
    uint32_t tiles = std::max(1u, cdiv(n, kSortTile));
    return 2 * align256((size_t)n * 8) + 2 * align256((size_t)n * 4) +
           2 * align256((size_t)passes * 256 * 4) +
           align256((size_t)passes * tiles * 256 * 4) + align256((size_t)passes * 4);
}

static char* carve_sort(char* p, uint32_t n, int passes, SortBuffers& sb) {
    sb.tiles = std::max(1u, cdiv(n, kSortTile));
    sb.keys[0] = (unsigned long long*)p; p += align256((size_t)n * 8);
    sb.keys[1] = (unsigned long long*)p; p += align256((size_t)n * 8);
    sb.vals[0] = (uint32_t*)p; p += align256((size_t)n * 4);
    sb.vals[1] = (uint32_t*)p; p += align256((size_t)n * 4);
    sb.hist = (uint32_t*)p; p += align256((size_t)passes * 256 * 4);
    sb.offsets = (uint32_t*)p; p += align256((size_t)passes * 256 * 4);
    sb.tile_status = (uint32_t*)p; p += align256((size_t)passes * sb.tiles * 256 * 4);
    sb.tile_counter = (uint32_t*)p; p += align256((size_t)passes * 4);
    return p;
}

// Sorts sb.keys[0]/vals[0]; returns the index (0/1) of the buffer holding the result.
static luz_status run_sort(luz_ctx* ctx, SortBuffers& sb, uint32_t n, int passes, int& result) {
    cudaStream_t st = ctx->stream;
    LUZ_CUDA(ctx, cudaMemsetAsync(sb.hist, 0, (size_t)passes * 256 * 4, st));
    LUZ_CUDA(ctx, cudaMemsetAsync(sb.tile_status, 0, (size_t)passes * sb.tiles * 256 * 4, st));
    LUZ_CUDA(ctx, cudaMemsetAsync(sb.tile_counter, 0, (size_t)passes * 4, st));
    uint32_t hblocks = std::min<uint32_t>(std::max(1u, cdiv(n, 256 * 16)), (uint32_t)ctx->sm_count * 4);
    sort_histogram_kernel<<<hblocks, 256, 0, st>>>(sb.keys[0], n, passes, sb.hist);
    LUZ_LAUNCHED(ctx, "sort_histogram_kernel");
    sort_scan_kernel<<<passes, 256, 0, st>>>(sb.hist, sb.offsets);
    LUZ_LAUNCHED(ctx, "sort_scan_kernel");
    int cur = 0;
    for (int p = 0; p < passes; ++p) {
        onesweep_pass_kernel<<<sb.tiles, kSortThreads, 0, st>>>(
            sb.keys[cur], sb.vals[cur], sb.keys[cur ^ 1], sb.vals[cur ^ 1], n, 8 * p,
            sb.offsets + p * 256, sb.tile_status + (size_t)p * sb.tiles * 256, sb.tile_counter + p,
            ctx->d_status);
        LUZ_LAUNCHED(ctx, "onesweep_pass_kernel");
        cur ^= 1;
    }
    result = cur;
    return LUZ_OK;
}

luz_status build_blas_batch(luz_ctx* ctx, uint32_t count, const luz_blas_desc* descs,
                            luz_blas** out) {
    // Validate on the host (indices in range, sizes) before any device work.
    std::vector<SegDesc> segs(count);
    std::vector<uint32_t> prim_off(count), node_off(count);
    uint64_t total_prims = 0, total_nodes = 0, total_verts = 0;
    for (uint32_t s = 0; s < count; ++s) {
        const luz_blas_desc& d = descs[s];
        if (d.index_count % 3 != 0)
            return set_error(ctx, LUZ_ERR_INVALID, "index_count is not a multiple of 3");
        if (d.vertex_stride < 12 || (d.vertex_count > 0 && !d.vertices) ||
            (d.index_count > 0 && !d.indices))
            return set_error(ctx, LUZ_ERR_INVALID, "bad vertex/index buffer description");
        for (uint32_t k = 0; k < d.index_count; ++k)
            if (d.indices[k] >= d.vertex_count)
                return set_error(ctx, LUZ_ERR_INVALID, "index out of range of the vertex buffer");
        uint32_t n = d.index_count / 3;
        prim_off[s] = (uint32_t)total_prims;
        node_off[s] = (uint32_t)total_nodes;
        total_prims += n;
        total_nodes += std::max(n, 2u) - 1;
        total_verts += d.vertex_count;
    }
    if (total_prims >= (1ull << 30) - 1)
        return set_error(ctx, LUZ_ERR_LIMIT, "more than 2^30 triangles in one batch");
    cudaStream_t st = ctx->stream;
    // Persistent arena: per BLAS nodes | 4-wide nodes | tris | morton | order | vertices | indices.
    std::vector<size_t> off_nodes(count), off_tris(count), off_mort(count), off_ord(count),
        off_vtx(count), off_idx(count), off_nodes4(count);
    size_t arena_bytes = 0;
    for (uint32_t s = 0; s < count; ++s) {
        uint32_t n = descs[s].index_count / 3;
        uint32_t m = std::max(n, 2u) - 1;
        off_nodes[s] = arena_bytes; arena_bytes += align256((size_t)m * 64);
        off_nodes4[s] = arena_bytes; arena_bytes += align256((size_t)m * 128);
        off_tris[s] = arena_bytes; arena_bytes += align256((size_t)std::max(n, 1u) * 48);
        off_mort[s] = arena_bytes; arena_bytes += align256((size_t)std::max(n, 1u) * 4);
        off_ord[s] = arena_bytes; arena_bytes += align256((size_t)std::max(n, 1u) * 4);
        off_vtx[s] = arena_bytes; arena_bytes += align256((size_t)std::max(descs[s].vertex_count, 1u) * sizeof(luz_vertex));
        off_idx[s] = arena_bytes; arena_bytes += align256((size_t)std::max(descs[s].index_count, 3u) * 4);
    }
    Arena* arena = new Arena();
    cudaError_t e = cudaMalloc(&arena->base, arena_bytes);
    if (e != cudaSuccess) { delete arena; return cuda_error(ctx, e, "cudaMalloc(BLAS arena)"); }
    char* ab = (char*)arena->base;
    // Upload vertices (repacked to 48-B luz_vertex when the stride differs) and indices.
    for (uint32_t s = 0; s < count; ++s) {
        const luz_blas_desc& d = descs[s];
        luz_vertex* dv = (luz_vertex*)(ab + off_vtx[s]);
        if (d.vertex_stride == sizeof(luz_vertex)) {
            if (d.vertex_count)
                LUZ_CUDA(ctx, cudaMemcpyAsync(dv, d.vertices, (size_t)d.vertex_count * 48,
                                              cudaMemcpyHostToDevice, st));
        } else {
            std::vector<luz_vertex> tmp(d.vertex_count);
            for (uint32_t v = 0; v < d.vertex_count; ++v) {
                memset(&tmp[v], 0, sizeof(luz_vertex));
                memcpy(tmp[v].position, (const char*)d.vertices + (size_t)v * d.vertex_stride, 12);
                if (d.vertex_stride >= 24)
                    memcpy(tmp[v].normal, (const char*)d.vertices + (size_t)v * d.vertex_stride + 12, 12);
            }
            if (d.vertex_count)
                LUZ_CUDA(ctx, cudaMemcpy(dv, tmp.data(), (size_t)d.vertex_count * 48,
                                         cudaMemcpyHostToDevice));
        }
        if (d.index_count)
            LUZ_CUDA(ctx, cudaMemcpyAsync(ab + off_idx[s], d.indices, (size_t)d.index_count * 4,
                                          cudaMemcpyHostToDevice, st));
        SegDesc& sd = segs[s];
        sd.prim_off = prim_off[s];
        sd.prim_count = d.index_count / 3;
        sd.node_off = node_off[s];
        sd.pad = 0;
        sd.vertices = dv;
        sd.indices = (const uint32_t*)(ab + off_idx[s]);
        sd.nodes = (float4*)(ab + off_nodes[s]);
        sd.tris = (float4*)(ab + off_tris[s]);
        sd.nodes4 = (float4*)(ab + off_nodes4[s]);
        sd.morton = (uint32_t*)(ab + off_mort[s]);
        sd.order = (uint32_t*)(ab + off_ord[s]);
    }
    // Scratch: segs | prim_off | node_off | bounds | sort | leaf boxes | parents | flags |
    // 4-wide collapse indices | leaf ranges.
    uint32_t N = (uint32_t)total_prims, M = (uint32_t)total_nodes;
    int passes = passes_for((int)count);
    size_t need = align256(count * sizeof(SegDesc)) + 2 * align256(count * 4) +
                  align256(count * 24) + sort_scratch_bytes(std::max(N, 1u), passes) +
                  align256((size_t)std::max(N, 1u) * 32) + align256((size_t)M * 4) +
                  align256((size_t)std::max(N, 1u) * 4) + align256((size_t)M * 4) +
                  2 * align256((size_t)M * 4) +
                  align256((size_t)(M / 1024 + 1) * 4) + align256((size_t)M * 8);
    luz_status stt = ensure_scratch(ctx, need);
    if (stt != LUZ_OK) { cudaFree(arena->base); delete arena; return stt; }
    char* p = (char*)ctx->d_scratch;
    SegDesc* d_segs = (SegDesc*)p; p += align256(count * sizeof(SegDesc));
    uint32_t* d_prim_off = (uint32_t*)p; p += align256(count * 4);
    uint32_t* d_node_off = (uint32_t*)p; p += align256(count * 4);
    uint32_t* d_bounds = (uint32_t*)p; p += align256(count * 24);
    SortBuffers sb;
    p = carve_sort(p, std::max(N, 1u), passes, sb);
    float4* d_leaf_box = (float4*)p; p += align256((size_t)std::max(N, 1u) * 32);
    uint32_t* d_node_parent = (uint32_t*)p; p += align256((size_t)M * 4);
    uint32_t* d_leaf_parent = (uint32_t*)p; p += align256((size_t)std::max(N, 1u) * 4);
    uint32_t* d_flags = (uint32_t*)p; p += align256((size_t)M * 4);
    uint32_t* d_even = (uint32_t*)p; p += align256((size_t)M * 4);
    uint32_t* d_idx4 = (uint32_t*)p; p += align256((size_t)M * 4);
    uint32_t* d_sums = (uint32_t*)p; p += align256((size_t)(M / 1024 + 1) * 4);
    uint2* d_range = (uint2*)p; p += align256((size_t)M * 8);
    for (uint32_t s = 0; s < count; ++s) segs[s].node_range = d_range + node_off[s];

    LUZ_CUDA(ctx, cudaMemcpyAsync(d_segs, segs.data(), count * sizeof(SegDesc), cudaMemcpyHostToDevice, st));
    LUZ_CUDA(ctx, cudaMemcpyAsync(d_prim_off, prim_off.data(), count * 4, cudaMemcpyHostToDevice, st));
    LUZ_CUDA(ctx, cudaMemcpyAsync(d_node_off, node_off.data(), count * 4, cudaMemcpyHostToDevice, st));
    std::vector<uint32_t> binit(count * 6);
    for (uint32_t s = 0; s < count; ++s)
        for (int k = 0; k < 6; ++k) binit[s * 6 + k] = k < 3 ? 0xFFFFFFFFu : 0u;
    LUZ_CUDA(ctx, cudaMemcpyAsync(d_bounds, binit.data(), count * 24, cudaMemcpyHostToDevice, st));
    LUZ_CUDA(ctx, cudaEventRecord(ctx->build_ev[0], st));   // device pipeline starts here
    LUZ_CUDA(ctx, cudaMemsetAsync(d_node_parent, 0xFF, (size_t)M * 4, st));
    LUZ_CUDA(ctx, cudaMemsetAsync(d_leaf_parent, 0xFF, (size_t)std::max(N, 1u) * 4, st));
    LUZ_CUDA(ctx, cudaMemsetAsync(d_flags, 0, (size_t)M * 4, st));
    if (N > 0) {
        blas_bounds_kernel<<<cdiv(N, 256 * kBoundsIters), 256, 0, st>>>(d_segs, d_prim_off, count, N, d_bounds);
        LUZ_LAUNCHED(ctx, "blas_bounds_kernel");
        blas_morton_kernel<<<cdiv(N, 256), 256, 0, st>>>(d_segs, d_prim_off, count, N, d_bounds,
                                                         sb.keys[0], sb.vals[0]);
        LUZ_LAUNCHED(ctx, "blas_morton_kernel");
    }
    int res = 0;
    if (N > 0) {
        stt = run_sort(ctx, sb, N, passes, res);
        if (stt != LUZ_OK) { cudaFree(arena->base); delete arena; return stt; }
    }
    // Every segment has at least one node; segments with 0 or 1 primitive get their
    // single node (empty / one leaf) here without reading keys.
    karras_kernel<<<cdiv(M, 256), 256, 0, st>>>(d_segs, d_node_off, count, M, sb.keys[res],
                                                d_node_parent, d_leaf_parent, ctx->d_status);
    LUZ_LAUNCHED(ctx, "karras_kernel");
    if (N > 0) {
        blas_emit_kernel<<<cdiv(N, 256), 256, 0, st>>>(d_segs, d_prim_off, count, N, sb.keys[res],
                                                       sb.vals[res], d_leaf_box);
        LUZ_LAUNCHED(ctx, "blas_emit_kernel");
        refit_local_kernel<<<cdiv(N, kRefitLeaves), kRefitLeaves, 0, st>>>(d_segs, d_prim_off, count, N,
                                                                           d_leaf_box, d_node_parent, d_leaf_parent,
                                                                           d_flags);
        LUZ_LAUNCHED(ctx, "refit_local_kernel");
        blas_radius_kernel<<<cdiv(N, 256), 256, 0, st>>>(d_segs, d_prim_off, count, N);
        LUZ_LAUNCHED(ctx, "blas_radius_kernel");
    }
    // 4-wide collapse of every segment's tree (the traversal structure of the
    // shadow/AO rays; the binary tree stays the parity-checked structure).
    {
        uint32_t chunks = cdiv(M, 1024);
        even_depth_kernel<<<cdiv(M, 256), 256, 0, st>>>(d_segs, d_node_off, count, M, d_node_parent, d_even);
        LUZ_LAUNCHED(ctx, "even_depth_kernel");
        chunk_sum_kernel<<<chunks, 256, 0, st>>>(d_even, M, d_sums);
        LUZ_LAUNCHED(ctx, "chunk_sum_kernel");
        chunk_scan_kernel<<<1, 1024, 0, st>>>(d_sums, chunks);
        LUZ_LAUNCHED(ctx, "chunk_scan_kernel");
        chunk_apply_kernel<<<chunks, 256, 0, st>>>(d_even, M, d_sums, d_idx4);
        LUZ_LAUNCHED(ctx, "chunk_apply_kernel");
        bvh4_emit_kernel<<<cdiv(M, 256), 256, 0, st>>>(d_segs, d_node_off, count, M, d_even, d_idx4);
        LUZ_LAUNCHED(ctx, "bvh4_emit_kernel");
    }
    LUZ_CUDA(ctx, cudaEventRecord(ctx->build_ev[1], st));
    ctx->build_timed = true;
    LUZ_CUDA(ctx, cudaStreamSynchronize(st));
    uint32_t bits = 0;
    LUZ_CUDA(ctx, cudaMemcpy(&bits, ctx->d_status, 4, cudaMemcpyDeviceToHost));
    if (bits) {
        cudaFree(arena->base);
        delete arena;
        return set_error(ctx, LUZ_ERR_DEVICE, "BLAS build kernel raised the device status word");
    }
    for (uint32_t s = 0; s < count; ++s) {
        luz_blas* b = new luz_blas();
        b->ctx = ctx;
        b->arena = arena;
        arena->refs++;
        b->nodes = segs[s].nodes;
        b->nodes4 = segs[s].nodes4;
        b->memory.nodes = off_nodes4[s] - off_nodes[s];
        b->memory.wide_nodes = off_tris[s] - off_nodes4[s];
        b->memory.leaves = off_mort[s] - off_tris[s];
        b->memory.other = (s + 1 < count ? off_nodes[s + 1] : arena_bytes) - off_mort[s];
        b->tris = segs[s].tris;
        b->morton = (uint32_t*)(ab + off_mort[s]);
        b->order = (uint32_t*)(ab + off_ord[s]);
        b->vertices = (luz_vertex*)(ab + off_vtx[s]);
        b->indices = (uint32_t*)(ab + off_idx[s]);
        b->prims = segs[s].prim_count;
        b->vertex_count = descs[s].vertex_count;
        out[s] = b;
    }
    return LUZ_OK;
}

// TLAS scratch layout (allocated once per luz_tlas for max_instances).
static size_t tlas_tmp_bytes(uint32_t cap) {
    uint32_t m = std::max(cap, 2u) - 1;
    return align256((size_t)cap * 32) + align256(24) + sort_scratch_bytes(std::max(cap, 1u), 4) +
           align256((size_t)cap * 32) + align256((size_t)m * 4) + align256((size_t)cap * 4) +
           align256((size_t)m * 4) + align256((size_t)m * 64) + 2 * align256((size_t)m * 4) +
           align256(sizeof(SegDesc)) + 2 * align256(4);
}

luz_status launch_tlas_build(luz_ctx* ctx, luz_tlas* t);

luz_status tlas_alloc(luz_ctx* ctx, luz_tlas* t) {
    uint32_t cap = std::max(t->max_instances, 1u);
    uint32_t m = std::max(cap, 2u) - 1;
    LUZ_CUDA(ctx, cudaMalloc(&t->nodes, (size_t)m * 64));
    LUZ_CUDA(ctx, cudaMalloc(&t->nodes4, (size_t)m * 128));
    LUZ_CUDA(ctx, cudaMalloc(&t->levels, 66 * 4));
    LUZ_CUDA(ctx, cudaMalloc(&t->instances, (size_t)cap * sizeof(DevInstance)));
    LUZ_CUDA(ctx, cudaMalloc(&t->shade, (size_t)cap * sizeof(DevShadeInstance)));
    LUZ_CUDA(ctx, cudaMalloc(&t->d_input, (size_t)cap * sizeof(DevInstanceInput)));
    LUZ_CUDA(ctx, cudaMallocHost(&t->h_input, (size_t)cap * sizeof(DevInstanceInput)));
    LUZ_CUDA(ctx, cudaMalloc(&t->morton, (size_t)cap * 4));
    LUZ_CUDA(ctx, cudaMalloc(&t->order, (size_t)cap * 4));
    LUZ_CUDA(ctx, cudaMalloc(&t->near, (size_t)cap * 4 * sizeof(uint4)));
    LUZ_CUDA(ctx, cudaMalloc(&t->leaf_of, (size_t)cap * 4));
    t->tmp_bytes = tlas_tmp_bytes(cap);
    LUZ_CUDA(ctx, cudaMalloc(&t->tmp, t->tmp_bytes));
    return LUZ_OK;
}

// Host part of a TLAS build: validates the instances and packs them into the pinned
// staging buffer (the buffer must not be in use by an earlier build's copy).
luz_status pack_tlas_input(luz_ctx* ctx, luz_tlas* t, const luz_instance* inst, uint32_t n) {
    if (n > t->max_instances)
        return set_error(ctx, LUZ_ERR_LIMIT, "instance count exceeds the TLAS max_instances");
    for (uint32_t i = 0; i < n; ++i) {
        const luz_blas* b = inst[i].blas;
        if (!b) return set_error(ctx, LUZ_ERR_INVALID, "instance without a BLAS");
        DevInstanceInput& d = t->h_input[i];
        memcpy(d.o2w, inst[i].transform, 48);
        d.nodes = b->nodes;
        d.tris = b->tris;
        d.vertices = b->vertices;
        d.indices = b->indices;
        d.custom_index = inst[i].custom_index;
        d.mask = inst[i].mask;
        d.blas_prims = b->prims;
        d.pad = 0;
        d.nodes4 = b->nodes4;
    }
    t->count = n;
    t->node_count = std::max(n, 2u) - 1;
    return LUZ_OK;
}

luz_status build_tlas(luz_ctx* ctx, luz_tlas* t, const luz_instance* inst, uint32_t n) {
    luz_status s = pack_tlas_input(ctx, t, inst, n);
    if (s != LUZ_OK) return s;
    return launch_tlas_build(ctx, t);
}

// The TLAS's scratch buffer (t->tmp) carved for a build of up to max_instances.
struct TlasScratch {
    TlasBuildArgs a;
    uint32_t* bounds;
    SortBuffers sb;
    SegDesc* d_seg;
    uint32_t* d_zero;
};

static TlasScratch carve_tlas(luz_tlas* t) {
    TlasScratch s;
    uint32_t cap = std::max(t->max_instances, 1u);
    uint32_t mcap = std::max(cap, 2u) - 1;
    char* p = (char*)t->tmp;
    TlasBuildArgs& a = s.a;
    a.in = t->d_input;
    a.n = t->count;
    a.shade = t->shade;
    a.inst_box = (float4*)p; p += align256((size_t)cap * 32);
    s.bounds = (uint32_t*)p; p += align256(24);
    p = carve_sort(p, cap, 4, s.sb);
    a.keys = s.sb.keys[0];
    a.vals = s.sb.vals[0];
    a.leaf_box = (float4*)p; p += align256((size_t)cap * 32);
    a.node_parent = (uint32_t*)p; p += align256((size_t)mcap * 4);
    a.leaf_parent = (uint32_t*)p; p += align256((size_t)cap * 4);
    a.flags = (uint32_t*)p; p += align256((size_t)mcap * 4);
    a.karras_nodes = (float4*)p; p += align256((size_t)mcap * 64);
    a.queue = (uint32_t*)p; p += align256((size_t)mcap * 4);
    a.newidx = (uint32_t*)p; p += align256((size_t)mcap * 4);
    s.d_seg = (SegDesc*)p; p += align256(sizeof(SegDesc));
    s.d_zero = (uint32_t*)p; p += align256(4);
    a.inst_out = t->instances;
    a.morton_out = t->morton;
    a.order_out = t->order;
    a.leaf_of_out = t->leaf_of;
    a.nodes_out = t->nodes;
    a.levels = t->levels;
    a.nodes4 = t->nodes4;
    return s;
}

TlasBuildArgs tlas_build_args(luz_tlas* t) { return carve_tlas(t).a; }
const float4* tlas_instance_boxes(const luz_tlas* t) { return carve_tlas(const_cast<luz_tlas*>(t)).a.inst_box; }
const float4* tlas_leaf_boxes(const luz_tlas* t) { return carve_tlas(const_cast<luz_tlas*>(t)).a.leaf_box; }

// Device part of a TLAS build from the packed staging buffer: one host-to-device copy
// from pinned memory and the LBVH kernels; no host synchronisation (graph-capturable).
luz_status launch_tlas_build(luz_ctx* ctx, luz_tlas* t) {
    cudaStream_t st = ctx->stream;
    const uint32_t n = t->count;
    if (n == 0) return LUZ_OK;
    LUZ_CUDA(ctx, cudaMemcpyAsync(t->d_input, t->h_input, (size_t)n * sizeof(DevInstanceInput),
                                  cudaMemcpyHostToDevice, st));
    const uint32_t m = std::max(n, 2u) - 1;
    TlasScratch ts = carve_tlas(t);
    const TlasBuildArgs& A = ts.a;
    float4* inst_box = A.inst_box;
    uint32_t* bounds = ts.bounds;
    SortBuffers& sb = ts.sb;
    float4* leaf_box = A.leaf_box;
    uint32_t* node_parent = A.node_parent;
    uint32_t* leaf_parent = A.leaf_parent;
    uint32_t* flags = A.flags;
    float4* karras_nodes = A.karras_nodes;
    uint32_t* queue = A.queue;
    uint32_t* newidx = A.newidx;
    SegDesc* d_seg = ts.d_seg;
    uint32_t* d_zero = ts.d_zero;

    if (n <= kFusedTlasMax) {
        prof_begin(ctx, LUZ_KERNEL_TLAS_BUILD);
        tlas_fused_kernel<<<1, 1024, 0, st>>>(A, ctx->d_status);
        prof_end(ctx);
        LUZ_LAUNCHED(ctx, "tlas_fused_kernel");
        return LUZ_OK;
    }
    SegDesc sd{};
    sd.prim_off = 0;
    sd.prim_count = n;
    sd.node_off = 0;
    sd.nodes = karras_nodes;
    // Bounds initialiser, segment descriptor and zero offset are written by a kernel from
    // its parameters: a copy from host memory would, inside a CUDA graph, re-read a
    // host address that no longer holds them.
    tlas_setup_kernel<<<1, 32, 0, st>>>(bounds, d_seg, sd, d_zero);
    LUZ_LAUNCHED(ctx, "tlas_setup_kernel");
    LUZ_CUDA(ctx, cudaMemsetAsync(node_parent, 0xFF, (size_t)m * 4, st));
    LUZ_CUDA(ctx, cudaMemsetAsync(leaf_parent, 0xFF, (size_t)n * 4, st));
    LUZ_CUDA(ctx, cudaMemsetAsync(flags, 0, (size_t)m * 4, st));

    tlas_instance_kernel<<<cdiv(n, 128), 128, 0, st>>>(t->d_input, n, inst_box, t->shade, bounds);
    LUZ_LAUNCHED(ctx, "tlas_instance_kernel");
    tlas_morton_kernel<<<cdiv(n, 128), 128, 0, st>>>(inst_box, n, bounds, sb.keys[0], sb.vals[0]);
    LUZ_LAUNCHED(ctx, "tlas_morton_kernel");
    int res = 0;
    luz_status s = run_sort(ctx, sb, n, 4, res);
    if (s != LUZ_OK) return s;
    karras_kernel<<<cdiv(m, 128), 128, 0, st>>>(d_seg, d_zero, 1, m, sb.keys[res], node_parent,
                                                leaf_parent, ctx->d_status);
    LUZ_LAUNCHED(ctx, "karras_kernel");
    tlas_emit_kernel<<<cdiv(n, 128), 128, 0, st>>>(t->d_input, inst_box, n, sb.keys[res],
                                                   sb.vals[res], t->instances, leaf_box,
                                                   t->morton, t->order, t->leaf_of);
    LUZ_LAUNCHED(ctx, "tlas_emit_kernel");
    refit_kernel<<<cdiv(n, 128), 128, 0, st>>>(d_seg, d_zero, 1, n, leaf_box, node_parent,
                                               leaf_parent, flags);
    LUZ_LAUNCHED(ctx, "refit_kernel");
    bfs_relayout_kernel<<<1, 1024, 0, st>>>(karras_nodes, t->nodes, m, queue, newidx, t->levels);
    LUZ_LAUNCHED(ctx, "bfs_relayout_kernel");
    tlas_bvh4_kernel<<<1, 1024, 0, st>>>(t->nodes, m, t->levels, t->nodes4);
    LUZ_LAUNCHED(ctx, "tlas_bvh4_kernel");
    return LUZ_OK;
}

}  // namespace luz
