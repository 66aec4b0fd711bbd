// blas_noalloc.cu — luz_blas_build_noalloc: one BLAS built without allocating memory.
//
// Some callers cannot allocate device memory when they build an acceleration
// structure: a renderer whose device memory comes from one up-front budget, code
// that runs where an allocation's implicit synchronisation would break a frame-time
// guarantee, or a host that owns every device allocation through its own pool. This
// entry point serves them: the caller passes its own device buffers for the inputs
// and outputs, and every temporary of the build (sort keys and values, tile state,
// leaf boxes, parent links, refit flags) lives in one file-scope device array of
// fixed size. Nothing here calls cudaMalloc, cudaFree or an allocating library
// routine.
//
// The kernels are the ones of the batched build (lbvh.cu), run over one segment, so
// the result is byte-identical to luz_blas_build's.
#include <algorithm>
#include <mutex>

#include "lbvh_kernels.cuh"

namespace luz {
namespace {

constexpr uint32_t kMaxTris = LUZ_NOALLOC_MAX_TRIANGLES;
constexpr uint32_t kMaxNodes = kMaxTris;                 // max(n-1, 1) <= n for n >= 1
constexpr uint32_t kTiles = (kMaxTris + kSortTile - 1) / kSortTile;
constexpr int kPasses = 4;                               // 30-bit Morton keys, one segment

constexpr size_t al(size_t x) { return (x + 255) & ~(size_t)255; }

// Scratch layout (byte offsets into the static array).
constexpr size_t kOffHeader = 0;                                   // status | seg | offsets | bounds
constexpr size_t kOffIndices = al(kOffHeader + 256);
constexpr size_t kOffKeys0 = al(kOffIndices + (size_t)3 * 4 * kMaxTris);
constexpr size_t kOffKeys1 = al(kOffKeys0 + (size_t)8 * kMaxTris);
constexpr size_t kOffVals0 = al(kOffKeys1 + (size_t)8 * kMaxTris);
constexpr size_t kOffVals1 = al(kOffVals0 + (size_t)4 * kMaxTris);
constexpr size_t kOffHist = al(kOffVals1 + (size_t)4 * kMaxTris);
constexpr size_t kOffOffsets = al(kOffHist + (size_t)kPasses * kRadix * 4);
constexpr size_t kOffTileStatus = al(kOffOffsets + (size_t)kPasses * kRadix * 4);
constexpr size_t kOffTileCounter = al(kOffTileStatus + (size_t)kPasses * kTiles * kRadix * 4);
constexpr size_t kOffLeafBox = al(kOffTileCounter + (size_t)kPasses * 4);
constexpr size_t kOffNodeParent = al(kOffLeafBox + (size_t)32 * kMaxTris);
constexpr size_t kOffLeafParent = al(kOffNodeParent + (size_t)4 * kMaxNodes);
constexpr size_t kOffFlags = al(kOffLeafParent + (size_t)4 * kMaxTris);
constexpr size_t kScratchBytes = al(kOffFlags + (size_t)4 * kMaxNodes);
static_assert(kScratchBytes == LUZ_NOALLOC_SCRATCH_BYTES, "scratch size in luz.h is out of date");

// Header words at kOffHeader.
struct Header {
    uint32_t status;        // LUZ_DEV_* bits of this build
    uint32_t zero;          // prim_off = node_off = 0 of the single segment
    uint32_t bounds[6];     // ordered-uint centroid bounds
    uint32_t pad[8];
    SegDesc seg;
};
static_assert(sizeof(Header) <= 256, "header region");

// Every GPU that loads this library holds this array until the process exits.
__device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
void* g_scratch_ptr[kMaxDevices] = {};

// Writes the segment descriptor and resets the header from kernel parameters, so no
// host memory is copied.
__global__ void noalloc_setup_kernel(Header* h, SegDesc seg) {
    if (threadIdx.x == 0) {
        h->status = 0;
        h->zero = 0;
        for (int k = 0; k < 6; ++k) h->bounds[k] = k < 3 ? 0xFFFFFFFFu : 0u;
        h->seg = seg;
    }
}

// Copies the caller's indices into scratch; an index outside the vertex buffer is
// replaced by 0 and reported, so no later kernel reads outside the caller's buffer.
__global__ void noalloc_indices_kernel(const uint32_t* __restrict__ in, uint32_t count,
                                       uint32_t vertex_count, uint32_t* __restrict__ out,
                                       uint32_t* status) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    uint32_t v = in[i];
    if (v >= vertex_count) {
        atomicOr(status, (uint32_t)LUZ_DEV_BAD_INDEX);
        v = 0;
    }
    out[i] = v;
}

inline uint32_t cdiv(uint32_t a, uint32_t b) { return (a + b - 1) / b; }

}  // namespace
}  // namespace luz

using namespace luz;

#define NOALLOC_CUDA(call)                                               \
    do {                                                                 \
        if ((call) != cudaSuccess) return LUZ_ERR_CUDA;                  \
    } while (0)
#define NOALLOC_LAUNCHED()                                               \
    do {                                                                 \
        if (cudaGetLastError() != cudaSuccess) return LUZ_ERR_CUDA;      \
    } while (0)

extern "C" luz_status luz_blas_build_noalloc(const luz_vertex* d_vertices, uint32_t vertex_count,
                                             const uint32_t* d_indices, uint32_t index_count,
                                             void* d_nodes, void* d_tris, uint32_t* d_morton,
                                             uint32_t* d_order, void* stream) {
    if (index_count % 3 != 0) return LUZ_ERR_INVALID;
    const uint32_t n = index_count / 3;
    if (n > kMaxTris) return LUZ_ERR_LIMIT;
    if (!d_nodes || (n > 0 && (!d_vertices || !d_indices || !d_tris || !d_morton || !d_order ||
                               vertex_count == 0)))
        return LUZ_ERR_INVALID;
    int dev = 0;
    NOALLOC_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return LUZ_ERR_LIMIT;
    cudaStream_t st = (cudaStream_t)stream;
    // The address of g_scratch as the device sees it (the symbol itself is only a
    // host-side stand-in), looked up with this device current. Outside a stream
    // capture it is looked up on every call, so a context that was torn down and
    // created again (cudaDeviceReset) gets the array's new address; inside a capture
    // the address of the last call outside one is used.
    cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
    NOALLOC_CUDA(cudaStreamIsCapturing(st, &capture));
    unsigned char* base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_mutex);
        if (capture == cudaStreamCaptureStatusNone) {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p) return LUZ_ERR_CUDA;
            g_scratch_ptr[dev] = p;
        } else if (!g_scratch_ptr[dev]) {
            return LUZ_ERR_INVALID;   // first call on this device inside a capture
        }
        base = (unsigned char*)g_scratch_ptr[dev];
    }
    Header* h = (Header*)(base + kOffHeader);
    uint32_t* status = &h->status;
    uint32_t* zero = &h->zero;
    uint32_t* bounds = h->bounds;
    SegDesc* d_seg = &h->seg;
    uint32_t* idx = (uint32_t*)(base + kOffIndices);
    unsigned long long* keys[2] = {(unsigned long long*)(base + kOffKeys0), (unsigned long long*)(base + kOffKeys1)};
    uint32_t* vals[2] = {(uint32_t*)(base + kOffVals0), (uint32_t*)(base + kOffVals1)};
    uint32_t* hist = (uint32_t*)(base + kOffHist);
    uint32_t* offsets = (uint32_t*)(base + kOffOffsets);
    uint32_t* tile_status = (uint32_t*)(base + kOffTileStatus);
    uint32_t* tile_counter = (uint32_t*)(base + kOffTileCounter);
    float4* leaf_box = (float4*)(base + kOffLeafBox);
    uint32_t* node_parent = (uint32_t*)(base + kOffNodeParent);
    uint32_t* leaf_parent = (uint32_t*)(base + kOffLeafParent);
    uint32_t* flags = (uint32_t*)(base + kOffFlags);

    SegDesc seg{};
    seg.prim_off = 0;
    seg.prim_count = n;
    seg.node_off = 0;
    seg.vertices = d_vertices;
    seg.indices = idx;
    seg.nodes = (float4*)d_nodes;
    seg.tris = (float4*)d_tris;
    seg.morton = d_morton;
    seg.order = d_order;
    const uint32_t m = n > 1 ? n - 1 : 1;
    const uint32_t tiles = n > 0 ? cdiv(n, kSortTile) : 1;

    // The array keeps the previous call's contents: reset everything read before written.
    noalloc_setup_kernel<<<1, 32, 0, st>>>(h, seg);
    NOALLOC_LAUNCHED();
    NOALLOC_CUDA(cudaMemsetAsync(node_parent, 0xFF, (size_t)m * 4, st));
    NOALLOC_CUDA(cudaMemsetAsync(leaf_parent, 0xFF, (size_t)(n ? n : 1) * 4, st));
    NOALLOC_CUDA(cudaMemsetAsync(flags, 0, (size_t)m * 4, st));
    if (n > 0) {
        noalloc_indices_kernel<<<cdiv(index_count, 256), 256, 0, st>>>(d_indices, index_count, vertex_count,
                                                                        idx, status);
        NOALLOC_LAUNCHED();
        blas_bounds_kernel<<<cdiv(n, 256 * kBoundsIters), 256, 0, st>>>(d_seg, zero, 1, n, bounds);
        NOALLOC_LAUNCHED();
        blas_morton_kernel<<<cdiv(n, 256), 256, 0, st>>>(d_seg, zero, 1, n, bounds, keys[0], vals[0]);
        NOALLOC_LAUNCHED();
        NOALLOC_CUDA(cudaMemsetAsync(hist, 0, (size_t)kPasses * kRadix * 4, st));
        NOALLOC_CUDA(cudaMemsetAsync(tile_status, 0, (size_t)kPasses * tiles * kRadix * 4, st));
        NOALLOC_CUDA(cudaMemsetAsync(tile_counter, 0, (size_t)kPasses * 4, st));
        sort_histogram_kernel<<<std::max(1u, std::min(cdiv(n, 4096), 256u)), 256, 0, st>>>(keys[0], n, kPasses, hist);
        NOALLOC_LAUNCHED();
        sort_scan_kernel<<<kPasses, 256, 0, st>>>(hist, offsets);
        NOALLOC_LAUNCHED();
        for (int p = 0; p < kPasses; ++p) {
            int cur = p & 1;
            onesweep_pass_kernel<<<tiles, kSortThreads, 0, st>>>(
                keys[cur], vals[cur], keys[cur ^ 1], vals[cur ^ 1], n, 8 * p, offsets + p * kRadix,
                tile_status + (size_t)p * tiles * kRadix, tile_counter + p, status);
            NOALLOC_LAUNCHED();
        }
    }
    // kPasses is even: the sorted keys are back in keys[0].
    karras_kernel<<<cdiv(m, 256), 256, 0, st>>>(d_seg, zero, 1, m, keys[0], node_parent, leaf_parent, status);
    NOALLOC_LAUNCHED();
    if (n > 0) {
        blas_emit_kernel<<<cdiv(n, 256), 256, 0, st>>>(d_seg, zero, 1, n, keys[0], vals[0], leaf_box);
        NOALLOC_LAUNCHED();
        refit_kernel<<<cdiv(n, 256), 256, 0, st>>>(d_seg, zero, 1, n, leaf_box, node_parent, leaf_parent, flags);
        NOALLOC_LAUNCHED();
        blas_radius_kernel<<<cdiv(n, 256), 256, 0, st>>>(d_seg, zero, 1, n);
        NOALLOC_LAUNCHED();
    }
    // Synchronous, like the reference's per-mesh build (GPUScene.cpp:132-137): read
    // this build's status word into host memory.
    uint32_t bits = 0;
    NOALLOC_CUDA(cudaMemcpyAsync(&bits, status, 4, cudaMemcpyDeviceToHost, st));
    NOALLOC_CUDA(cudaStreamSynchronize(st));
    if (bits & LUZ_DEV_BAD_INDEX) return LUZ_ERR_INVALID;
    if (bits) return LUZ_ERR_DEVICE;
    return LUZ_OK;
}
