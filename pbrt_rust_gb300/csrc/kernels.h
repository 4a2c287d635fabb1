// kernels.h - host-callable launchers of the device kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/pbrt_gpu.h"
#include "trace.cuh"

namespace pbrt {

// Largest traversal stack the kernels carry for a tree of this depth, or
// 0 if the tree is too deep for any compiled variant.
int trace_stack_for_depth(uint32_t depth);

// Closest hit into `hits` (occluded == nullptr) or any hit into `occluded`.
// All pointers are device pointers; d_status receives a PbrtStatus > 0 on a
// device-side failure.
cudaError_t launch_trace(const DevBVH& bvh, uint32_t depth, const PbrtRay* rays, uint32_t n, PbrtHit* hits,
                         uint8_t* occluded, int* d_status, cudaStream_t stream);

}  // namespace pbrt
