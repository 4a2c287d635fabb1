// render.cu - the SamplerRenderer wavefront on the device.
//
//   generate : one thread per sampler pixel - stratified samples, light
//              sample arrays and camera rays (sampler/stratified.rs:60-127,
//              camera/mod.rs:168-271), reading the pixel's slice of its
//              task's ChaCha12 stream
//   extend   : closest hit of every camera ray (trace.cuh)
//   shade    : dg, emitted radiance, per-light sample_l, BSDF and the
//              unoccluded contribution; shadow rays go to a compacted queue
//              (integrator/whitted.rs:30-65, light/point.rs:28-35)
//   shadow   : any hit of every queued shadow ray
//   combine  : L = Le + sum over lights of the unoccluded contributions, in
//              light order
//   film     : every film pixel gathers the samples that land on it, from
//              its own task only, in the task's sample order
//              (camera/film.rs:192-249, 175-186, 316-354)
// The library is compiled with --fmad=false and IEEE div/sqrt, so each
// step repeats the reference's f32 operations.
#include <cuda_runtime.h>

#include "kernels.h"
#include "wavefront.cuh"

namespace pbrt {

__global__ void __launch_bounds__(128) k_generate(RenderParams P) {
    __shared__ uint32_t words[32 * 128];  // the threads' ChaCha block pairs
    uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= P.n_pixels) return;
    generate_pixel(P, pix, words + threadIdx.x, 128u);
}

__global__ void __launch_bounds__(128) k_shade(RenderParams P) {
    const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const ShadowSink Q{P.shadow_rays, P.shadow_slot, nullptr, &P.counters[0]};
    shade_sample(P, s, s < P.n_samples, Q, 0u);
}

// ---------------------------------------------------------------- shadow ---
template <int STACK, bool INST = false>
__global__ void __launch_bounds__(128) k_shadow(RenderParams P) {
    uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= *(volatile uint32_t*)&P.counters[0]) return;
    const float4* r4 = reinterpret_cast<const float4*>(P.shadow_rays);
    DRay r = make_dray(r4[2 * (size_t)q], r4[2 * (size_t)q + 1]);
    TraceResult res;
    int st = 0;
    bool occ = traverse<STACK, true, INST>(P.bvh, r, &res, &st);
    if (st) atomicMax((int*)&P.counters[2], st);
    P.occluded[P.shadow_slot[q]] = occ ? 1 : 0;
}

// k_shadow with warps of shadow rays that share their direction signs
// walked together (traverse_packet); the same answers.
template <int STACK>
__global__ void __launch_bounds__(128) k_shadow_packet(RenderParams P) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = q < *(volatile uint32_t*)&P.counters[0];  // every lane stays for the warp's votes
    const float4* r4 = reinterpret_cast<const float4*>(P.shadow_rays);
    DRay r = make_dray(active ? r4[2 * (size_t)q] : make_float4(0, 0, 0, 0),
                       active ? r4[2 * (size_t)q + 1] : make_float4(0, 0, 1, 0));
    TraceResult res;
    int st = 0;
    bool occ = false;
    if (warp_signs_uniform(r, active))
        occ = traverse_packet<STACK, true>(P.bvh, r, active, &res, &st);
    else if (active)
        occ = traverse<STACK, true>(P.bvh, r, &res, &st);
    if (!active) return;
    if (st) atomicMax((int*)&P.counters[2], st);
    P.occluded[P.shadow_slot[q]] = occ ? 1 : 0;
}

template <int SMAX, int OVF, bool INST = false>
__global__ void __launch_bounds__(128) k_shadow4(RenderParams P) {
    extern __shared__ uint2 smem_stack[];
    uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= *(volatile uint32_t*)&P.counters[0]) return;
    const float4* r4 = reinterpret_cast<const float4*>(P.shadow_rays);
    DRay r = make_dray(r4[2 * (size_t)q], r4[2 * (size_t)q + 1]);
    Traversal4<SMAX, OVF, INST> T;
    T.bind(smem_stack, threadIdx.x, blockDim.x);
    if (T.start(P.bvh4, r))
        while (T.template step<true>(P.bvh4, r)) {
        }
    if (T.overflow) atomicMax((int*)&P.counters[2], 6);
    P.occluded[P.shadow_slot[q]] = T.found ? 1 : 0;
}

// --------------------------------------------------------------- combine ---
__global__ void __launch_bounds__(256) k_combine(RenderParams P) {
    const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= P.n_samples) return;
    combine_sample(P, s);
}

// ------------------------------------------------------------------ film ---
__global__ void __launch_bounds__(128) k_film(RenderParams P) {
    const int32_t fw = P.fx1 - P.fx0, fh = P.fy1 - P.fy0;
    const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (uint32_t)(fw * fh)) return;
    film_pixel(P, idx);
}

// ------------------------------------------------------ sampler stream ---
// The sampler's ChaCha code, run on its own so that it can be compared with
// other implementations: thread i computes block ctr0 + i (PAIR: blocks
// ctr0 + 2i and ctr0 + 2i + 1 with the paired routine), 16 words a block.
struct Key8 {
    uint32_t k[8];
};
template <int DR, bool PAIR>
__global__ void __launch_bounds__(128) k_chacha_blocks(Key8 key, uint64_t ctr0, uint64_t sid, uint32_t n_blocks,
                                                       uint32_t* out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (PAIR) {
        if (2ull * i + 1 >= n_blocks) return;
        chacha12_block2<DR>(key.k, ctr0 + 2ull * i, out + 32ull * i, 1u, sid);
    } else {
        if (i >= n_blocks) return;
        chacha12_block<DR>(key.k, ctr0 + i, out + 16ull * i, 1u, sid);
    }
}

// Words [first, first + n) of one task's stream as generate_pixel reads
// them: thread t seeks to word first + t * seg and reads its segment of seg
// words (the last one shorter) with the WordStream reader.
__global__ void __launch_bounds__(128) k_rng_words(Key8 key, uint64_t first, uint32_t n, uint32_t seg,
                                                   uint32_t* out) {
    __shared__ uint32_t words[32 * 128];
    const uint64_t lo = (uint64_t)(blockIdx.x * blockDim.x + threadIdx.x) * seg;
    if (lo >= n) return;
    const uint64_t hi = lo + seg < n ? lo + seg : n;
    WordStream rng;
    rng.seek(key.k, first + lo, first + hi, words + threadIdx.x, 128u);
    for (uint64_t w = lo; w < hi; ++w) out[w] = rng.next_u32();
}

// ------------------------------------------------------------ launchers ---
static inline unsigned blocks_for(uint64_t n, int b) { return (unsigned)((n + b - 1) / b); }

cudaError_t launch_chacha_blocks(const uint32_t key[8], uint64_t ctr, uint64_t sid, uint32_t rounds, bool paired,
                                 uint32_t n_blocks, uint32_t* d_out, cudaStream_t s) {
    Key8 k;
    for (int i = 0; i < 8; ++i) k.k[i] = key[i];
    const unsigned grid = blocks_for(paired ? (n_blocks + 1) / 2 : n_blocks, 128);
    if (!grid) return cudaSuccess;
    if (rounds == 8)
        paired ? k_chacha_blocks<4, true><<<grid, 128, 0, s>>>(k, ctr, sid, n_blocks, d_out)
               : k_chacha_blocks<4, false><<<grid, 128, 0, s>>>(k, ctr, sid, n_blocks, d_out);
    else if (rounds == 12)
        paired ? k_chacha_blocks<6, true><<<grid, 128, 0, s>>>(k, ctr, sid, n_blocks, d_out)
               : k_chacha_blocks<6, false><<<grid, 128, 0, s>>>(k, ctr, sid, n_blocks, d_out);
    else if (rounds == 20)
        paired ? k_chacha_blocks<10, true><<<grid, 128, 0, s>>>(k, ctr, sid, n_blocks, d_out)
               : k_chacha_blocks<10, false><<<grid, 128, 0, s>>>(k, ctr, sid, n_blocks, d_out);
    else
        return cudaErrorInvalidValue;
    return cudaGetLastError();
}

cudaError_t launch_rng_words(const uint32_t key[8], uint64_t first, uint32_t n, uint32_t seg, uint32_t* d_out,
                             cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    if (seg == 0) return cudaErrorInvalidValue;
    Key8 k;
    for (int i = 0; i < 8; ++i) k.k[i] = key[i];
    k_rng_words<<<blocks_for(((uint64_t)n + seg - 1) / seg, 128), 128, 0, s>>>(k, first, n, seg, d_out);
    return cudaGetLastError();
}

cudaError_t launch_render(const RenderParams& P, cudaStream_t s) {
    cudaError_t e;
    if (P.n_pixels) {
        k_generate<<<blocks_for(P.n_pixels, 128), 128, 0, s>>>(P);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    if (P.n_samples) {
        // camera rays of neighbouring pixels are coherent: one thread per
        // ray keeps them together in a warp
        const int rk = render_trace_kernel();
        e = launch_trace(P.bvh, P.depth, P.rays, (uint32_t)P.n_samples, reinterpret_cast<PbrtHit*>(P.hits), nullptr,
                         (int*)&P.counters[2], s, P.has_wide ? &P.bvh4 : nullptr, P.wide_bound, rk, nullptr, nullptr,
                         &P.counters[3]);
        if (e != cudaSuccess) return e;
        k_shade<<<blocks_for(P.n_samples, 128), 128, 0, s>>>(P);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        uint64_t max_shadow = P.n_samples * P.n_lights;
        if (max_shadow) {
            const size_t smem = 16 * sizeof(uint2) * 128;
            // scenes with instances: the 4-wide walk with instances when a
            // variant covers its stack bound, else the binary one
            const bool inst = P.bvh.insts != nullptr;
            const int iv = (inst && P.has_wide) ? wide_stack_variant(P.wide_bound) : 0;
            const bool wide_rk = rk == PBRT_TRACE_WIDE || rk == PBRT_TRACE_WIDE_PERSISTENT || rk == PBRT_TRACE_WIDE_SPECULATIVE;
            int wv = (P.has_wide && wide_rk && !inst) ? wide_stack_variant(P.wide_bound) : 0;
            if (iv == 64)
                k_shadow4<16, 48, true><<<blocks_for(max_shadow, 128), 128, smem, s>>>(P);
            else if (iv == 256)
                k_shadow4<16, 240, true><<<blocks_for(max_shadow, 128), 128, smem, s>>>(P);
            else if (inst && trace_stack_for_depth(P.depth) == 64)
                k_shadow<64, true><<<blocks_for(max_shadow, 128), 128, 0, s>>>(P);
            else if (inst)
                k_shadow<256, true><<<blocks_for(max_shadow, 128), 128, 0, s>>>(P);
            else if (rk == PBRT_TRACE_PAIR_PACKET && trace_stack_for_depth(P.depth) == 64)
                k_shadow_packet<64><<<blocks_for(max_shadow, 128), 128, 0, s>>>(P);
            else if (rk == PBRT_TRACE_PAIR_PACKET)
                k_shadow_packet<256><<<blocks_for(max_shadow, 128), 128, 0, s>>>(P);
            else if (wv == 64)
                k_shadow4<16, 48><<<blocks_for(max_shadow, 128), 128, smem, s>>>(P);
            else if (wv == 256)
                k_shadow4<16, 240><<<blocks_for(max_shadow, 128), 128, smem, s>>>(P);
            else if (trace_stack_for_depth(P.depth) == 64)
                k_shadow<64><<<blocks_for(max_shadow, 128), 128, 0, s>>>(P);
            else
                k_shadow<256><<<blocks_for(max_shadow, 128), 128, 0, s>>>(P);
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
        }
        k_combine<<<blocks_for(P.n_samples, 256), 256, 0, s>>>(P);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    uint64_t npx = (uint64_t)(P.fx1 - P.fx0) * (uint64_t)(P.fy1 - P.fy0);
    if (npx) {
        k_film<<<blocks_for(npx, 128), 128, 0, s>>>(P);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace pbrt
