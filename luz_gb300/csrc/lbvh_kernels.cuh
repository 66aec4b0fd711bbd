// lbvh_kernels.cuh — declarations of the LBVH build kernels (defined in lbvh.cu) and
// the segment descriptor they share, so that other translation units can launch the
// same kernels.
#pragma once
#include "internal.cuh"

namespace luz {

// One mesh of a batched BLAS build: a contiguous run of primitives in the sort.
struct SegDesc {
    uint32_t prim_off;     // first primitive (global)
    uint32_t prim_count;
    uint32_t node_off;     // first internal node (global), max(n-1,1) nodes
    uint32_t pad;
    const luz_vertex* vertices;  // device copy, 48-B stride (BLAS only)
    const uint32_t* indices;
    float4* nodes;         // output nodes of this segment
    float4* tris;          // output triangles of this segment
    float4* nodes4;        // output 4-wide nodes (NULL: not built)
    uint2* node_range;     // leaf range [lo, hi] of each internal node (NULL: not kept)
    uint32_t* morton;      // BLAS: output sorted 30-bit Morton codes of this segment
    uint32_t* order;       // BLAS: output primitive index of each leaf
};

// Onesweep radix sort geometry.
constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;   // 2048 keys
constexpr int kRadix = 256;
constexpr int kMaxPasses = 6;
constexpr uint32_t kFlagAggregate = 1u << 30;
constexpr uint32_t kFlagPrefix = 2u << 30;
constexpr uint32_t kValueMask = (1u << 30) - 1;
constexpr uint32_t kLookbackSpinLimit = 1u << 22;

// Rows of 256 primitives one block of blas_bounds_kernel reduces (launch 256 threads
// and ceil(total / (256 * kBoundsIters)) blocks).
constexpr int kBoundsIters = 16;
__global__ void __launch_bounds__(256) blas_bounds_kernel(const SegDesc* segs, const uint32_t* seg_prim_off,
                                                          int nseg, uint32_t total, uint32_t* seg_bounds);
__global__ void blas_morton_kernel(const SegDesc* segs, const uint32_t* seg_prim_off, int nseg,
                                   uint32_t total, const uint32_t* seg_bounds,
                                   unsigned long long* keys, uint32_t* vals);
__global__ void sort_histogram_kernel(const unsigned long long* keys, uint32_t n, int passes,
                                      uint32_t* hist);
__global__ void sort_scan_kernel(const uint32_t* hist, uint32_t* offsets);
__global__ void onesweep_pass_kernel(const unsigned long long* __restrict__ kin,
                                     const uint32_t* __restrict__ vin,
                                     unsigned long long* __restrict__ kout,
                                     uint32_t* __restrict__ vout, uint32_t n, int shift,
                                     const uint32_t* __restrict__ pass_offsets,
                                     uint32_t* tile_status, uint32_t* tile_counter,
                                     uint32_t* dev_status);
__global__ void karras_kernel(const SegDesc* segs, const uint32_t* seg_node_off, int nseg,
                              uint32_t total_nodes, const unsigned long long* keys,
                              uint32_t* node_parent, uint32_t* leaf_parent, uint32_t* dev_status);
__global__ void blas_emit_kernel(const SegDesc* segs, const uint32_t* seg_prim_off, int nseg,
                                 uint32_t total, const unsigned long long* keys,
                                 const uint32_t* vals, float4* leaf_box);
__global__ void refit_kernel(const SegDesc* segs, const uint32_t* seg_prim_off, int nseg,
                             uint32_t total, const float4* leaf_box, const uint32_t* node_parent,
                             const uint32_t* leaf_parent, uint32_t* flags);
// Leaves per block of refit_local_kernel (one thread each).
constexpr int kRefitLeaves = 512;
__global__ void __launch_bounds__(kRefitLeaves)
refit_local_kernel(const SegDesc* segs, const uint32_t* seg_prim_off, int nseg, uint32_t total,
                   const float4* leaf_box, const uint32_t* node_parent, const uint32_t* leaf_parent,
                   uint32_t* flags);
__global__ void blas_radius_kernel(const SegDesc* segs, const uint32_t* seg_prim_off, int nseg,
                                   uint32_t total);

}  // namespace luz
