// reorder.cu - coherence ordering of a ray batch before traversal.
//
// Incoherent rays (random origins, random directions) put unrelated rays in
// one warp: the lanes walk different parts of the BVH and most of them sit
// idle at every divergent branch.  Before a batch is traced, its rays are
// binned by a 16-bit key - the direction's cube-map face and an 8x8 cell on
// that face, then a 7-bit Morton code of the origin inside the BVH's world
// bounds - with a counting sort (histogram, scan, scatter).  The trace
// kernels then take rays in bin order through the resulting permutation and
// write each hit back at the ray's own index, so the output is the same
// array in the same order; only which rays share a warp changes.  Every
// ray's traversal is unchanged, so results are bit-identical.  Order inside
// a bin depends on atomic arrival and is not deterministic; nothing in the
// output depends on it.
#include <cuda_runtime.h>

#include <cstdint>

#include "kernels.h"

namespace pbrt {

namespace {

constexpr uint32_t kBins = 1u << 16;

__device__ __forceinline__ uint32_t clampi(int v, int lo, int hi) { return (uint32_t)min(max(v, lo), hi); }

// Spreads the low 3 bits of v to positions 0, 3, 6.
__device__ __forceinline__ uint32_t spread3(uint32_t v) {
    return (v & 1u) | ((v & 2u) << 2) | ((v & 4u) << 4);
}

__device__ __forceinline__ uint32_t ray_key(float4 a, float4 b, const ReorderBounds& B) {
    const float dx = b.x, dy = b.y, dz = b.z;
    const float ax = fabsf(dx), ay = fabsf(dy), az = fabsf(dz);
    uint32_t face;
    float m, u, v;
    if (ax >= ay && ax >= az) {
        face = dx < 0.0f ? 1u : 0u;
        m = ax, u = dy, v = dz;
    } else if (ay >= az) {
        face = dy < 0.0f ? 3u : 2u;
        m = ay, u = dz, v = dx;
    } else {
        face = dz < 0.0f ? 5u : 4u;
        m = az, u = dx, v = dy;
    }
    // (u/m, v/m) in [-1, 1] -> 8 cells each; NaN (zero or NaN direction)
    // converts to 0 and the clamp keeps every index in range
    const float inv = m > 0.0f ? 4.0f / m : 0.0f;
    const uint32_t cu = clampi(__float2int_rd(u * inv + 4.0f), 0, 7);
    const uint32_t cv = clampi(__float2int_rd(v * inv + 4.0f), 0, 7);
    // origin cell: 3 bits of x, 2 of y, 2 of z, interleaved x y z x y z x
    const uint32_t ox = clampi(__float2int_rd((a.x - B.lo[0]) * B.scale[0]), 0, 7);
    const uint32_t oy = clampi(__float2int_rd((a.y - B.lo[1]) * B.scale[1]), 0, 3);
    const uint32_t oz = clampi(__float2int_rd((a.z - B.lo[2]) * B.scale[2]), 0, 3);
    const uint32_t morton = (spread3(ox) | (spread3(oy) << 1) | (spread3(oz) << 2)) & 0x7fu;
    return (face << 13) | (cu << 10) | (cv << 7) | morton;
}

__global__ void __launch_bounds__(256) k_ray_keys(const float4* __restrict__ rays, uint32_t n, ReorderBounds B,
                                                  uint16_t* __restrict__ keys, uint32_t* __restrict__ bins) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t k = ray_key(__ldg(rays + 2 * (size_t)i), __ldg(rays + 2 * (size_t)i + 1), B);
    keys[i] = (uint16_t)k;
    atomicAdd(bins + k, 1u);
}

// Exclusive prefix sum of the kBins counters, in place; one block of 1024
// threads, 64 consecutive bins per thread.
__global__ void __launch_bounds__(1024) k_bins_scan(uint32_t* __restrict__ bins) {
    constexpr uint32_t per = kBins / 1024;
    __shared__ uint32_t warp_sums[32];
    const uint32_t t = threadIdx.x, lane = t & 31u, w = t >> 5;
    uint32_t* mine = bins + t * per;
    uint32_t sum = 0;
    for (uint32_t j = 0; j < per; ++j) sum += mine[j];
    // inclusive scan of the per-thread sums across the warp, then the block
    uint32_t x = sum;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) warp_sums[w] = x;
    __syncthreads();
    if (w == 0) {
        uint32_t s = warp_sums[lane];
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= (uint32_t)o) s += y;
        }
        warp_sums[lane] = s;
    }
    __syncthreads();
    uint32_t run = x - sum + (w ? warp_sums[w - 1] : 0u);
    for (uint32_t j = 0; j < per; ++j) {
        uint32_t c = mine[j];
        mine[j] = run;
        run += c;
    }
}

__global__ void __launch_bounds__(256) k_ray_scatter(const uint16_t* __restrict__ keys, uint32_t n,
                                                     uint32_t* __restrict__ offsets, uint32_t* __restrict__ order) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    order[atomicAdd(offsets + keys[i], 1u)] = i;
}

}  // namespace

size_t ray_order_scratch_bytes(uint32_t n) {
    // order (4 B/ray), keys (2 B/ray, padded to 256 B), bins
    return (size_t)n * 4 + (((size_t)n * 2 + 255) & ~(size_t)255) + (size_t)kBins * 4;
}

cudaError_t build_ray_order(const PbrtRay* rays, uint32_t n, const ReorderBounds& B, void* scratch,
                            uint32_t** order_out, cudaStream_t s) {
    unsigned char* p = static_cast<unsigned char*>(scratch);
    uint32_t* order = reinterpret_cast<uint32_t*>(p);
    uint16_t* keys = reinterpret_cast<uint16_t*>(p + (size_t)n * 4);
    uint32_t* bins = reinterpret_cast<uint32_t*>(p + (size_t)n * 4 + (((size_t)n * 2 + 255) & ~(size_t)255));
    cudaError_t e = cudaMemsetAsync(bins, 0, (size_t)kBins * 4, s);
    if (e != cudaSuccess) return e;
    const unsigned grid = (n + 255) / 256;
    const float4* r4 = reinterpret_cast<const float4*>(rays);
    k_ray_keys<<<grid, 256, 0, s>>>(r4, n, B, keys, bins);
    k_bins_scan<<<1, 1024, 0, s>>>(bins);
    k_ray_scatter<<<grid, 256, 0, s>>>(keys, n, bins, order);
    *order_out = order;
    return cudaGetLastError();
}

}  // namespace pbrt
