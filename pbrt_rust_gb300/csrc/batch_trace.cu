// batch_trace.cu - the traversal stages of the batched wavefront.
//
// extend: closest hit (renders, closest-hit queries) or any hit (any-hit
//         queries) of every ray of every job
// shadow: any hit of every queued shadow ray of every render job
// Both are persistent kernels: a grid of resident warps takes `chunk` rays
// at a time from a device work counter and refills a warp's idle lanes once
// `refill` of them are idle, each lane finding its ray's job (and so its
// scene's BVH and its output) by a binary search over the job offsets.
// Each ray's traversal is the single-scene kernels' (trace.cuh,
// trace4.cuh), so results are the same bit for bit.
#include <cuda_runtime.h>

#include "batch.h"
#include "kernels.h"
#include "trace.cuh"
#include "trace4.cuh"

namespace pbrt {

namespace {

constexpr unsigned kFull = 0xffffffffu;

struct Cursor {
    uint32_t j;
    uint64_t lo, hi;
};

// Job of item g: the j with off[j] <= g < off[j + 1] (empty jobs have
// off[j] == off[j + 1] and are never returned); the last answer is reused
// while g stays inside it.
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

// The chunked work source of one warp; every member call is warp-uniform.
struct WorkSource {
    uint64_t next = 0, end = 0;
    bool more = true;

    __device__ __forceinline__ void fetch(uint32_t* counter, uint32_t chunk, uint64_t n, unsigned lane) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(counter, chunk);
        base = __shfl_sync(kFull, base, 0);
        if ((uint64_t)base < n) {
            next = base;
            end = (uint64_t)base + chunk < n ? (uint64_t)base + chunk : n;
        } else {
            more = false;
        }
    }
};

// Which hit the extend stage looks for: closest for every ray, any for
// every ray, or each job's own choice.
enum { kClosest = 0, kAny = 1, kPerJob = 2 };

template <bool WIDE, int S1, int S2>
struct Walker;  // traversal state over one layout

template <int SMAX, int OVF>
struct Walker<true, SMAX, OVF> {
    Traversal4<SMAX, OVF> T;
    DevBVH4 bv;
    __device__ __forceinline__ void bind(uint2* smem) { T.bind(smem, threadIdx.x, blockDim.x); }
    __device__ __forceinline__ bool start(const RenderParams& P, const DRay& r) {
        bv = P.bvh4;
        return T.start(bv, r);
    }
    template <int MODE>
    __device__ __forceinline__ bool step(const DRay& r, bool any) {
        if (MODE == kClosest) return T.template step<false>(bv, r);
        if (MODE == kAny) return T.template step<true>(bv, r);
        return any ? T.template step<true>(bv, r) : T.template step<false>(bv, r);
    }
    __device__ __forceinline__ int failure() const { return T.overflow ? 6 : 0; }
    __device__ __forceinline__ bool found() const { return T.found; }
    __device__ __forceinline__ bool nan_hit() const { return T.nan_hit; }
    __device__ __forceinline__ const TraceResult& res() const { return T.res; }
};

// INST = 1: the tree may hold instances (Traversal with INST).
template <int STACK, int INST>
struct Walker<false, STACK, INST> {
    Traversal<STACK, INST != 0> T;
    DevBVH bv;
    int st = 0;
    __device__ __forceinline__ void bind(uint2*) {}
    __device__ __forceinline__ bool start(const RenderParams& P, const DRay& r) {
        bv = P.bvh;
        return T.start(bv, r);
    }
    template <int MODE>
    __device__ __forceinline__ bool step(const DRay& r, bool any) {
        if (MODE == kClosest) return T.template step<false>(bv, r, &st);
        if (MODE == kAny) return T.template step<true>(bv, r, &st);
        return any ? T.template step<true>(bv, r, &st) : T.template step<false>(bv, r, &st);
    }
    __device__ __forceinline__ int failure() const { return st; }
    __device__ __forceinline__ bool found() const { return T.found; }
    __device__ __forceinline__ bool nan_hit() const { return T.nan_hit; }
    __device__ __forceinline__ const TraceResult& res() const { return T.res; }
};

// SHADOW = false: extend over the job rays; true: the shadow queue (any
// hit, MODE = kAny).
template <int BLOCK, bool SHADOW, bool WIDE, int S1, int S2, int MODE>
__global__ void __launch_bounds__(BLOCK) kb_trace(BatchArgs A) {
    extern __shared__ uint2 smem_stack[];
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t nj = A.hdr->n_jobs;
    const uint64_t n = SHADOW ? (uint64_t) * (volatile uint32_t*)(A.counters + kCtrShadowCount) : A.hdr->rays;
    uint32_t* counter = A.counters + (SHADOW ? kCtrShadowWork : kCtrExtendWork);
    const uint32_t refill = SHADOW ? A.refill_shadow : A.refill;
    WorkSource W;
    Cursor c{0, 1, 0};
    Walker<WIDE, S1, S2> K;
    K.bind(smem_stack);
    DRay r;
    bool busy = false, any = MODE == kAny;
    uint32_t job = 0;
    uint64_t item = 0;  // extend: index inside the job; shadow: queue entry
    auto finish = [&]() {
        const JobRec& J = A.jobs[job];
        if (const int f = K.failure()) atomicMax((int*)(J.P.counters + 2), f);
        if (SHADOW) {
            J.P.occluded[__ldg(A.q_slot + item)] = K.found() ? 1 : 0;
        } else if (any) {
            J.occ[item] = K.found() ? 1 : 0;
        } else if (K.nan_hit()) {  // rewritten by the replay stage
            J.hits[item] = make_float4(__int_as_float(kReplayMark), 0.0f, 0.0f, 0.0f);
            A.counters[kCtrReplay] = 1u;
        } else {
            const TraceResult& R = K.res();
            J.hits[item] = make_float4(__int_as_float(R.prim), R.t, R.b1, R.b2);
        }
        busy = false;
    };
    for (;;) {
        const unsigned idle = __ballot_sync(kFull, !busy);
        const unsigned nidle = __popc(idle);
        if (W.more && W.next >= W.end && nidle >= refill) W.fetch(counter, A.chunk, n, lane);
        const bool tail = !W.more && W.next + nidle >= W.end;
        if (W.next < W.end && nidle >= (tail ? 1u : refill)) {
            if (!busy) {
                const uint64_t my = W.next + __popc(idle & ((1u << lane) - 1u));
                if (my < W.end) {
                    const float4* src;
                    if (SHADOW) {
                        job = __ldg(A.q_job + my);
                        item = my;
                        src = reinterpret_cast<const float4*>(A.q_rays) + 2 * my;
                    } else {
                        job = locate(A.off_ray, nj, my, c);
                        item = my - c.lo;
                        if (MODE == kPerJob) any = A.jobs[job].any != 0;
                        src = A.jobs[job].rays + 2 * item;
                    }
                    r = make_dray(__ldg(src), __ldg(src + 1));
                    busy = true;
                    if (!K.start(A.jobs[job].P, r)) finish();
                }
            }
            W.next += nidle;
        }
        if (!__any_sync(kFull, busy)) {
            if (W.next >= W.end && !W.more) break;
            continue;
        }
        if (busy && !K.template step<MODE>(r, any)) finish();
    }
}

// kb_trace with refill = 32, where a warp takes new rays only once all of
// its lanes are done: each lane walks its ray to the end in the
// single-scene kernels' loop, with no warp vote per traversal step and only
// the fields of the job's tree the walk reads held in registers.  The same
// rays go to the same warps in the same groups, each walked in the same
// order, so the results equal kb_trace's (measured on GB300, the
// 1024x1024x16 heightfield frame as one job: extend 3.47 -> 2.3 ms, shadow
// 3.28 -> 2.3 ms, as with the single-render kernels).
template <int BLOCK, bool SHADOW, bool WIDE, int S1, int S2, int MODE>
__global__ void __launch_bounds__(BLOCK) kb_trace_flat(BatchArgs A) {
    extern __shared__ uint2 smem_stack[];
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t nj = A.hdr->n_jobs;
    const uint64_t n = SHADOW ? (uint64_t) * (volatile uint32_t*)(A.counters + kCtrShadowCount) : A.hdr->rays;
    uint32_t* counter = A.counters + (SHADOW ? kCtrShadowWork : kCtrExtendWork);
    const uint32_t chunk = A.chunk;
    Cursor c{0, 1, 0};
    for (;;) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(counter, chunk);
        base = __shfl_sync(kFull, base, 0);
        if ((uint64_t)base >= n) break;
        const uint64_t end = (uint64_t)base + chunk < n ? (uint64_t)base + chunk : n;
        for (uint64_t my = (uint64_t)base + lane; my < end; my += 32u) {
            uint32_t job;
            uint64_t item;  // extend: index inside the job; shadow: queue entry
            const float4* src;
            if (SHADOW) {
                job = __ldg(A.q_job + my);
                item = my;
                src = reinterpret_cast<const float4*>(A.q_rays) + 2 * my;
            } else {
                job = locate(A.off_ray, nj, my, c);
                item = my - c.lo;
                src = A.jobs[job].rays + 2 * item;
            }
            const JobRec& J = A.jobs[job];
            const bool any = MODE == kAny || (MODE == kPerJob && J.any != 0);
            const DRay r = make_dray(__ldg(src), __ldg(src + 1));
            TraceResult res;
            int fail = 0;
            bool nan = false, found;
            if (WIDE) {
                Traversal4<S1, S2> T;
                T.bind(smem_stack, threadIdx.x, blockDim.x);
                // by reference: the walk reads the tree's arrays from the job
                // table (L1) instead of holding them in registers (80 -> 72,
                // one more block per SM); the per-job mode keeps its copy
                // (it spills without it)
                const DevBVH4 bv_copy = MODE == kPerJob ? J.P.bvh4 : DevBVH4{};
                const DevBVH4& bv = MODE == kPerJob ? bv_copy : J.P.bvh4;
                if (T.start(bv, r)) {
                    if (any) {
                        while (T.template step<true>(bv, r)) {
                        }
                    } else {
                        while (T.template step<false>(bv, r)) {
                        }
                    }
                }
                found = T.found;
                nan = T.nan_hit;
                res = T.res;
                fail = T.overflow ? 6 : 0;
            } else {
                const DevBVH& bv = J.P.bvh;  // from the job table, as above
                found = any ? traverse<S1, true, S2 != 0>(bv, r, &res, &fail)
                            : traverse<S1, false, S2 != 0>(bv, r, &res, &fail, &nan);
            }
            if (fail) atomicMax((int*)(J.P.counters + 2), fail);
            if (SHADOW) {
                J.P.occluded[__ldg(A.q_slot + item)] = found ? 1 : 0;
            } else if (any) {
                J.occ[item] = found ? 1 : 0;
            } else if (nan) {  // rewritten by the replay stage
                J.hits[item] = make_float4(__int_as_float(kReplayMark), 0.0f, 0.0f, 0.0f);
                A.counters[kCtrReplay] = 1u;
            } else {
                J.hits[item] = make_float4(__int_as_float(res.prim), res.t, res.b1, res.b2);
            }
        }
    }
}

// kb_trace over the 4-wide layout, shaped as the single-scene persistent
// walk (k_trace4_persistent): a lane keeps only its ray, its job and its
// item, finds the job by a fresh binary search when it takes a ray, and
// reads the job's tree from the job table at each step instead of holding
// a copy, so the kernel fits the registers of 7 blocks of 128 per SM.
// Idle lanes take new rays once `refill` of them are idle.  Each ray's walk
// is the same as in the other stage kernels, so are the results.
template <int BLOCK, bool SHADOW, int S1, int S2, int MODE>
__global__ void __launch_bounds__(BLOCK, 896 / BLOCK) kb_trace4_refill(BatchArgs A) {
    extern __shared__ uint2 smem_stack[];
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t nj = A.hdr->n_jobs;
    const uint32_t n =
        SHADOW ? *(volatile uint32_t*)(A.counters + kCtrShadowCount) : (uint32_t)A.hdr->rays;  // < 2^32 (launch)
    uint32_t* counter = A.counters + (SHADOW ? kCtrShadowWork : kCtrExtendWork);
    const uint32_t refill = SHADOW ? A.refill_shadow : A.refill;
    constexpr uint32_t kNone = 0xffffffffu;
    uint32_t next = 0, end = 0;
    bool more = true;
    uint32_t job = kNone, item = 0;
    bool any = MODE == kAny;
    DRay r;
    Traversal4<S1, S2> T;
    T.bind(smem_stack, threadIdx.x, blockDim.x);
    auto finish = [&]() {
        const JobRec& J = A.jobs[job];
        if (T.overflow) atomicMax((int*)(J.P.counters + 2), 6);
        if (SHADOW) {
            J.P.occluded[__ldg(A.q_slot + item)] = T.found ? 1 : 0;
        } else if (any) {
            J.occ[item] = T.found ? 1 : 0;
        } else if (T.nan_hit) {  // rewritten by the replay stage
            J.hits[item] = make_float4(__int_as_float(kReplayMark), 0.0f, 0.0f, 0.0f);
            A.counters[kCtrReplay] = 1u;
        } else {
            J.hits[item] = make_float4(__int_as_float(T.res.prim), T.res.t, T.res.b1, T.res.b2);
        }
        job = kNone;
    };
    for (;;) {
        const unsigned idle = __ballot_sync(kFull, job == kNone);
        const unsigned nidle = __popc(idle);
        if (more && next >= end && nidle >= refill) {  // warp-uniform
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(counter, A.chunk);
            base = __shfl_sync(kFull, base, 0);
            if (base < n) {
                next = base;
                end = n - base > A.chunk ? base + A.chunk : n;
            } else {
                more = false;
            }
        }
        const bool tail = !more && next + nidle >= end;
        if (next < end && nidle >= (tail ? 1u : refill)) {
            if (job == kNone) {
                const uint32_t my = next + (uint32_t)__popc(idle & ((1u << lane) - 1u));
                if (my < end) {
                    const float4* src;
                    if (SHADOW) {
                        job = __ldg(A.q_job + my);
                        item = my;
                        src = reinterpret_cast<const float4*>(A.q_rays) + 2 * (size_t)my;
                    } else {
                        Cursor c{0, 1, 0};
                        job = locate(A.off_ray, nj, my, c);
                        item = (uint32_t)(my - c.lo);
                        if (MODE == kPerJob) any = A.jobs[job].any != 0;
                        src = A.jobs[job].rays + 2 * (size_t)item;
                    }
                    r = make_dray(__ldg(src), __ldg(src + 1));
                    if (!T.start(A.jobs[job].P.bvh4, r)) finish();
                }
            }
            next += nidle;
        }
        if (!__any_sync(kFull, job != kNone)) {
            if (next >= end && !more) break;
            continue;
        }
        if (job != kNone) {
            const DevBVH4& bv = A.jobs[job].P.bvh4;
            bool going;
            if (MODE == kClosest)
                going = T.template step<false>(bv, r);
            else if (MODE == kAny)
                going = T.template step<true>(bv, r);
            else
                going = any ? T.template step<true>(bv, r) : T.template step<false>(bv, r);
            if (!going) finish();
        }
    }
}

// The exact replay of the closest hits the extend stage marked (see
// Traversal in trace.cuh): the binary walk with instances allowed; returns
// at once when nothing was marked.
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) kb_replay(BatchArgs A) {
    if (*(const volatile uint32_t*)(A.counters + kCtrReplay) == 0u) return;
    const uint64_t n = A.hdr->rays;
    const uint32_t nj = A.hdr->n_jobs;
    Cursor c{0, 1, 0};
    for (uint64_t g = (uint64_t)blockIdx.x * BLOCK + threadIdx.x; g < n; g += (uint64_t)gridDim.x * BLOCK) {
        const uint32_t j = locate(A.off_ray, nj, g, c);
        const JobRec& J = A.jobs[j];
        if (J.any) continue;
        const uint64_t item = g - c.lo;
        if (__float_as_int(J.hits[item].x) != kReplayMark) continue;
        const DRay r = make_dray(__ldg(J.rays + 2 * item), __ldg(J.rays + 2 * item + 1));
        TraceResult res;
        int st = 0;
        traverse<256, false, true, true>(J.P.bvh, r, &res, &st);
        if (st) atomicMax((int*)(J.P.counters + 2), st);
        J.hits[item] = make_float4(__int_as_float(res.prim), res.t, res.b1, res.b2);
    }
}

// FLAT: kb_trace_flat (the stage's refill is 32), else kb_trace.
template <int BLOCK, bool SHADOW, bool WIDE, int S1, int S2, int MODE, bool FLAT>
cudaError_t go(const BatchArgs& A, int sms, cudaStream_t s) {
    static ShapeCache bps_cache;
    const size_t smem = WIDE ? (size_t)S1 * sizeof(uint2) * BLOCK : 0;
    auto pick_kernel = [] {
        if constexpr (FLAT)
            return kb_trace_flat<BLOCK, SHADOW, WIDE, S1, S2, MODE>;
        else if constexpr (WIDE)
            return kb_trace4_refill<BLOCK, SHADOW, S1, S2, MODE>;
        else
            return kb_trace<BLOCK, SHADOW, WIDE, S1, S2, MODE>;
    };
    auto kernel = pick_kernel();
    const int bps = resident_blocks(bps_cache, kernel, BLOCK, smem);
    kernel<<<(unsigned)(sms * bps), BLOCK, smem, s>>>(A);
    return cudaGetLastError();
}

template <int BLOCK, bool SHADOW, int MODE, bool FLAT>
cudaError_t pick_layout(const BatchArgs& A, const BatchTuning& T, bool wide, bool inst, uint32_t cover, int sms,
                        cudaStream_t s) {
    if (inst) return go<BLOCK, SHADOW, false, 256, 1, MODE, FLAT>(A, sms, s);
    if (wide) {
        if (T.smax == 8)
            return cover <= 64 ? go<BLOCK, SHADOW, true, 8, 56, MODE, FLAT>(A, sms, s)
                               : go<BLOCK, SHADOW, true, 8, 248, MODE, FLAT>(A, sms, s);
        return cover <= 64 ? go<BLOCK, SHADOW, true, 16, 48, MODE, FLAT>(A, sms, s)
                           : go<BLOCK, SHADOW, true, 16, 240, MODE, FLAT>(A, sms, s);
    }
    return cover <= 64 ? go<BLOCK, SHADOW, false, 64, 0, MODE, FLAT>(A, sms, s)
                       : go<BLOCK, SHADOW, false, 256, 0, MODE, FLAT>(A, sms, s);
}

template <int BLOCK, bool SHADOW, int MODE>
cudaError_t pick(const BatchArgs& A, const BatchTuning& T, bool wide, bool inst, uint32_t cover, int sms,
                 cudaStream_t s) {
    const uint32_t refill = SHADOW ? T.refill_shadow : T.refill;
    return refill >= 32 ? pick_layout<BLOCK, SHADOW, MODE, true>(A, T, wide, inst, cover, sms, s)
                        : pick_layout<BLOCK, SHADOW, MODE, false>(A, T, wide, inst, cover, sms, s);
}

template <int BLOCK>
cudaError_t pick_block(const BatchArgs& A, const BatchTuning& T, bool shadow, bool mixed, bool wide, bool inst,
                       uint32_t cover, int sms, cudaStream_t s) {
    if (shadow) return pick<BLOCK, true, kAny>(A, T, wide, inst, cover, sms, s);
    return mixed ? pick<BLOCK, false, kPerJob>(A, T, wide, inst, cover, sms, s)
                 : pick<BLOCK, false, kClosest>(A, T, wide, inst, cover, sms, s);
}

}  // namespace

cudaError_t launch_batch_replay(const BatchArgs& A, const BatchTuning& T, int sms, cudaStream_t s) {
    if (T.block == 256)
        kb_replay<256><<<(unsigned)(sms * 2), 256, 0, s>>>(A);
    else
        kb_replay<128><<<(unsigned)(sms * 4), 128, 0, s>>>(A);
    return cudaGetLastError();
}

cudaError_t launch_batch_trace(const BatchArgs& A, const BatchTuning& T, bool shadow, bool mixed, bool inst,
                               uint32_t cover_pair, uint32_t cover_wide, int sms, cudaStream_t s) {
    const bool wide = !inst && (shadow ? T.shadow_wide : T.extend_wide);
    const uint32_t cover = wide ? cover_wide : cover_pair;
    if (cover > 256) return cudaErrorInvalidValue;
    if (T.block == 256) return pick_block<256>(A, T, shadow, mixed, wide, inst, cover, sms, s);
    return pick_block<128>(A, T, shadow, mixed, wide, inst, cover, sms, s);
}

}  // namespace pbrt
