// kernels.h - host-callable launchers of the device kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/pbrt_gpu.h"
#include "trace.cuh"
#include "trace4.cuh"

namespace pbrt {

// Largest traversal stack the kernels carry for a tree of this depth, or
// 0 if the tree is too deep for any compiled variant.
int trace_stack_for_depth(uint32_t depth);

// Closest hit into `hits` (occluded == nullptr) or any hit into `occluded`.
// All pointers are device pointers; d_status receives a PbrtStatus > 0 on a
// device-side failure.
// `wide` (may be null) selects the 4-wide layout with the given stack bound.
// `kernel` >= 0 overrides the process-wide choice (PBRT_TRACE_*).
cudaError_t launch_trace(const DevBVH& bvh, uint32_t depth, const PbrtRay* rays, uint32_t n, PbrtHit* hits,
                         uint8_t* occluded, int* d_status, cudaStream_t stream, const DevBVH4* wide = nullptr,
                         uint32_t wide_bound = 0, int kernel = -1);
// Process-wide traversal kernel choice (PBRT_TRACE_*); 0 on success.
int set_trace_config(int kernel, unsigned refill, unsigned min_blocks, int render_kernel);
void get_trace_config(int* kernel, unsigned* refill, unsigned* min_blocks, int* render_kernel);
// Kernel used for the coherent camera and shadow rays of a render.
int render_trace_kernel();
// 64 or 256 when a compiled 4-wide variant covers this stack bound, else 0.
int wide_stack_variant(uint32_t bound);

}  // namespace pbrt
