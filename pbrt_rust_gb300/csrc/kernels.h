// kernels.h - host-callable launchers of the device kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

#include "../../include/pbrt_gpu.h"
#include "trace.cuh"
#include "trace4.cuh"

namespace pbrt {

// Per-device launch-shape caches, safe to fill from several host threads at
// once: every entry is one atomic word that holds a complete, valid value
// (>= 1) or 0 = not yet known, so a reader never sees half of a pair.
constexpr int kShapeCacheDevices = 64;
using ShapeCache = std::atomic<int>[kShapeCacheDevices];

// SM count of the current device.
inline int device_sms() {
    static ShapeCache cache;  // static storage: zero-initialised
    int dev = 0;
    cudaGetDevice(&dev);
    int v = (dev >= 0 && dev < kShapeCacheDevices) ? cache[dev].load(std::memory_order_relaxed) : 0;
    if (v == 0) {
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v < 1) v = 1;
        if (dev >= 0 && dev < kShapeCacheDevices) cache[dev].store(v, std::memory_order_relaxed);
    }
    return v;
}

// Resident blocks per SM of `kernel` on the current device, cached in the
// caller's `cache` (one per kernel and launch configuration).
template <class Kernel>
inline int resident_blocks(ShapeCache& cache, Kernel kernel, int block, size_t smem) {
    int dev = 0;
    cudaGetDevice(&dev);
    int v = (dev >= 0 && dev < kShapeCacheDevices) ? cache[dev].load(std::memory_order_relaxed) : 0;
    if (v == 0) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, kernel, block, smem) != cudaSuccess || v < 1) v = 1;
        if (dev >= 0 && dev < kShapeCacheDevices) cache[dev].store(v, std::memory_order_relaxed);
    }
    return v;
}

// Largest traversal stack the kernels carry for a tree of this depth, or
// 0 if the tree is too deep for any compiled variant.
int trace_stack_for_depth(uint32_t depth);

// Closest hit into `hits` (occluded == nullptr) or any hit into `occluded`.
// All pointers are device pointers; d_status receives a PbrtStatus > 0 on a
// device-side failure.
// `wide` (may be null) selects the 4-wide layout with the given stack bound.
// `kernel` >= 0 overrides the process-wide choice (PBRT_TRACE_*).  With
// `order` (a permutation of [0, n)) the kernels take ray order[j] as their
// j-th ray; hits still land at each ray's own index.  `work` is the 4-wide
// persistent kernel's chunk counter (see trace_chunk).  `replay` (closest
// hit: required; a device word, zero at launch) flags that some ray's walk
// accepted a NaN distance; a replay kernel queued after the traversal then
// rewrites those rays' hits by the exact walk (see Traversal in trace.cuh).
// `in.ready` (streamed input; needs `work` and trace_streams()): the rays
// arrive in pieces of 2^in.shift rays while the walk runs, in.ready[k] (zero
// at launch) turning non-zero once piece k has landed; a piece that has not
// landed within in.wait_ms ends the walk with PBRT_ERR_TIMEOUT in d_status.
// `host_hits` (closest hits; needs `work` and trace_streams()): pinned host
// memory mapped into the device's address space that receives the hits,
// chunk by chunk as they complete; `hits` is then the device staging array.
// Streamed input of a walk: piece flags (null: the rays are all there),
// rays per piece (2^shift) and how long a warp waits for a piece.
struct StreamIn {
    const uint32_t* ready = nullptr;
    uint32_t shift = 0;
    uint32_t wait_ms = 0;
};
cudaError_t launch_trace(const DevBVH& bvh, uint32_t depth, const PbrtRay* rays, uint32_t n, PbrtHit* hits,
                         uint8_t* occluded, int* d_status, cudaStream_t stream, const DevBVH4* wide = nullptr,
                         uint32_t wide_bound = 0, int kernel = -1, const uint32_t* order = nullptr,
                         uint32_t* work = nullptr, uint32_t* replay = nullptr, StreamIn in = {},
                         PbrtHit* host_hits = nullptr);
// Whether the configured traversal of this tree can take streamed input
// (the 4-wide persistent walk with its shared counter, rays in order).
bool trace_streams(const DevBVH& bvh, const DevBVH4* wide, uint32_t wide_bound, uint32_t n);
// Process-wide traversal configuration (PBRT_TRACE_* and the environment
// variables of pbrt_gpu.h); set returns 0 on success, 1 for invalid fields.
int set_trace_config(const PbrtTraceConfig& cfg);
void get_trace_config(PbrtTraceConfig* cfg);
// Batches of at least this many rays are reordered when the configuration
// asks for it (smaller ones gain nothing from it).
constexpr uint32_t kReorderMinRays = 1u << 15;
bool trace_reorder();
// Rays a warp of the 4-wide persistent kernel takes from a shared counter at
// a time (0: fixed per-warp ranges).  The counter (`work` of launch_trace,
// 4 bytes, zero at launch) is the caller's.
unsigned trace_chunk();

// Coherence ordering of a ray batch (reorder.cu).  `scale` maps an origin
// inside the world bounds to [0, 8) x [0, 4) x [0, 4).
struct ReorderBounds {
    float lo[3];
    float scale[3];
};
size_t ray_order_scratch_bytes(uint32_t n);
// Fills the permutation at the start of `scratch` (ray_order_scratch_bytes(n)
// bytes, 256-byte aligned) and returns it in *order; stream-ordered.
cudaError_t build_ray_order(const PbrtRay* rays, uint32_t n, const ReorderBounds& bounds, void* scratch,
                            uint32_t** order, cudaStream_t stream);
// The sampler's ChaCha block code on its own (render.cu): blocks ctr ..
// ctr + n_blocks - 1 with `rounds` rounds (8, 12 or 20) and stream id sid,
// single-block or paired routine; and words [first, first + n) of the
// stream with key `key` through the seekable reader, one seek per `seg`
// words.  d_out: device memory, 16 words per block / n words.
cudaError_t launch_chacha_blocks(const uint32_t key[8], uint64_t ctr, uint64_t sid, uint32_t rounds, bool paired,
                                 uint32_t n_blocks, uint32_t* d_out, cudaStream_t s);
cudaError_t launch_rng_words(const uint32_t key[8], uint64_t first, uint32_t n, uint32_t seg, uint32_t* d_out,
                             cudaStream_t s);
// Kernel used for the coherent camera and shadow rays of a render.
int render_trace_kernel();
// 64 or 256 when a compiled 4-wide variant covers this stack bound, else 0.
int wide_stack_variant(uint32_t bound);

}  // namespace pbrt
