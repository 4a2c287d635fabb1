// batch.cu - the non-traversal stages of the batched wavefront and the
// launch sequence of one batch.
//
//   generate : every sampler pixel of every render job
//   extend   : batch_trace.cu (camera rays and query rays)
//   shade    : every camera sample; shadow rays of all jobs go to one queue
//              tagged with their job
//   shadow   : batch_trace.cu (the queue)
//   combine  : every camera sample
//   film     : every film pixel of every render job
// The non-traversal stages are grid-stride loops over the concatenated items
// with a grid fixed by the device, so the launch sequence does not depend on
// the batch's contents and can be captured once as a CUDA graph.  Each item
// runs the single-render step of wavefront.cuh with its job's parameters.
#include <cuda_runtime.h>

#include "batch.h"
#include "kernels.h"
#include "wavefront.cuh"

namespace pbrt {

cudaError_t launch_batch_trace(const BatchArgs& A, const BatchTuning& T, bool shadow, bool mixed, bool inst,
                               uint32_t cover_pair, uint32_t cover_wide, int sms, cudaStream_t s);
cudaError_t launch_batch_replay(const BatchArgs& A, const BatchTuning& T, int sms, cudaStream_t s);

namespace {

struct Cursor {
    uint32_t j;
    uint64_t lo, hi;
};

__device__ __forceinline__ uint32_t locate(const uint64_t* __restrict__ off, uint32_t n, uint64_t g, Cursor& c) {
    if (g >= c.lo && g < c.hi) return c.j;
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (__ldg(off + mid) <= g)
            lo = mid;
        else
            hi = mid;
    }
    c.j = lo;
    c.lo = __ldg(off + lo);
    c.hi = __ldg(off + lo + 1);
    return lo;
}

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) kb_generate(BatchArgs A) {
    __shared__ uint32_t words[32 * BLOCK];  // the threads' ChaCha block pairs
    const uint64_t total = A.hdr->pix;
    const uint32_t nj = A.hdr->n_jobs;
    Cursor c{0, 1, 0};
    for (uint64_t g = (uint64_t)blockIdx.x * BLOCK + threadIdx.x; g < total; g += (uint64_t)gridDim.x * BLOCK) {
        const uint32_t j = locate(A.off_pix, nj, g, c);
        generate_pixel(A.jobs[j].P, (uint32_t)(g - c.lo), words + threadIdx.x, (uint32_t)BLOCK);
    }
}

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) kb_shade(BatchArgs A) {
    const uint64_t total = A.hdr->samples;
    const uint32_t nj = A.hdr->n_jobs;
    const ShadowSink Q{A.q_rays, A.q_slot, A.q_job, A.counters + kCtrShadowCount};
    Cursor c{0, 1, 0};
    // the block-uniform loop keeps whole warps together for shade_sample's
    // warp-aggregated queue append
    for (uint64_t base = (uint64_t)blockIdx.x * BLOCK; base < total; base += (uint64_t)gridDim.x * BLOCK) {
        const uint64_t g = base + threadIdx.x;
        const bool live = g < total;
        const uint32_t j = live ? locate(A.off_smp, nj, g, c) : 0u;
        shade_sample(A.jobs[j].P, live ? g - c.lo : 0u, live, Q, j);
    }
}

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) kb_combine(BatchArgs A) {
    const uint64_t total = A.hdr->samples;
    const uint32_t nj = A.hdr->n_jobs;
    Cursor c{0, 1, 0};
    for (uint64_t g = (uint64_t)blockIdx.x * BLOCK + threadIdx.x; g < total; g += (uint64_t)gridDim.x * BLOCK) {
        const uint32_t j = locate(A.off_smp, nj, g, c);
        combine_sample(A.jobs[j].P, g - c.lo);
    }
}

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) kb_film(BatchArgs A) {
    const uint64_t total = A.hdr->film;
    const uint32_t nj = A.hdr->n_jobs;
    Cursor c{0, 1, 0};
    for (uint64_t g = (uint64_t)blockIdx.x * BLOCK + threadIdx.x; g < total; g += (uint64_t)gridDim.x * BLOCK) {
        const uint32_t j = locate(A.off_film, nj, g, c);
        film_pixel(A.jobs[j].P, (uint32_t)(g - c.lo));
    }
}

}  // namespace

cudaError_t launch_batch_stages(const BatchArgs& A, const BatchTuning& T, bool mixed, bool inst, uint32_t cover_pair,
                                uint32_t cover_wide, int sms, size_t counter_bytes, cudaStream_t s, int* launches) {
    *launches = 0;
    cudaError_t e = cudaMemsetAsync(A.counters, 0, counter_bytes, s);
    if (e != cudaSuccess) return e;
    // grid-stride stages: 8 blocks of 128 (4 of 256) threads per SM
    const int grid = sms * (T.block == 256 ? 4 : 8);
    auto stage = [&](auto kernel) -> cudaError_t {
        kernel<<<grid, T.block, 0, s>>>(A);
        ++*launches;
        return cudaGetLastError();
    };
    const bool b256 = T.block == 256;
    if ((e = b256 ? stage(kb_generate<256>) : stage(kb_generate<128>)) != cudaSuccess) return e;
    if ((e = launch_batch_trace(A, T, false, mixed, inst, cover_pair, cover_wide, sms, s)) != cudaSuccess) return e;
    ++*launches;
    if ((e = launch_batch_replay(A, T, sms, s)) != cudaSuccess) return e;
    ++*launches;
    if ((e = b256 ? stage(kb_shade<256>) : stage(kb_shade<128>)) != cudaSuccess) return e;
    if ((e = launch_batch_trace(A, T, true, false, inst, cover_pair, cover_wide, sms, s)) != cudaSuccess) return e;
    ++*launches;
    if ((e = b256 ? stage(kb_combine<256>) : stage(kb_combine<128>)) != cudaSuccess) return e;
    if ((e = b256 ? stage(kb_film<256>) : stage(kb_film<128>)) != cudaSuccess) return e;
    return cudaSuccess;
}

}  // namespace pbrt
