// trace.cu - batched closest-hit / any-hit kernels over PbrtRay arrays.
#include <cuda_runtime.h>

#include "../../include/pbrt_gpu.h"
#include "kernels.h"
#include "trace.cuh"

namespace pbrt {

// One thread per ray.  Rays are two float4 loads (32 B, coalesced); a
// closest hit is one 16-byte store, an any-hit answer one byte.
template <int STACK, bool ANY>
__global__ void __launch_bounds__(128) k_trace(DevBVH bvh, const float4* __restrict__ rays, uint32_t n,
                                               float4* __restrict__ hits, uint8_t* __restrict__ occ,
                                               int* __restrict__ status) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 a = __ldg(rays + 2 * (size_t)i), b = __ldg(rays + 2 * (size_t)i + 1);
    DRay r = make_dray(a, b);
    TraceResult res;
    int st = 0;
    bool found = traverse<STACK, ANY>(bvh, r, &res, &st);
    if (st) atomicMax(status, st);
    if (ANY)
        occ[i] = found ? 1 : 0;
    else
        hits[i] = make_float4(__int_as_float(res.prim), res.t, res.b1, res.b2);
}

int trace_stack_for_depth(uint32_t depth) {
    if (depth <= 64) return 64;
    if (depth <= 256) return 256;
    return 0;
}

cudaError_t launch_trace(const DevBVH& bvh, uint32_t depth, const PbrtRay* rays, uint32_t n, PbrtHit* hits,
                         uint8_t* occluded, int* d_status, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    const int block = 128;
    const unsigned grid = (unsigned)((n + block - 1) / block);
    const float4* r4 = reinterpret_cast<const float4*>(rays);
    float4* h4 = reinterpret_cast<float4*>(hits);
    int stack = trace_stack_for_depth(depth);
    bool any = occluded != nullptr;
    if (stack == 64) {
        if (any)
            k_trace<64, true><<<grid, block, 0, stream>>>(bvh, r4, n, nullptr, occluded, d_status);
        else
            k_trace<64, false><<<grid, block, 0, stream>>>(bvh, r4, n, h4, nullptr, d_status);
    } else if (stack == 256) {
        if (any)
            k_trace<256, true><<<grid, block, 0, stream>>>(bvh, r4, n, nullptr, occluded, d_status);
        else
            k_trace<256, false><<<grid, block, 0, stream>>>(bvh, r4, n, h4, nullptr, d_status);
    } else {
        return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace pbrt
