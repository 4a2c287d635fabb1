// trace.cu - batched closest-hit / any-hit kernels over PbrtRay arrays.
#include <cuda_runtime.h>

#include <cstdlib>
#include <cstring>
#include <type_traits>

#include "../../include/pbrt_gpu.h"
#include "kernels.h"
#include "trace.cuh"
#include "trace4.cuh"

namespace pbrt {

// One thread per ray.  Rays are two float4 loads (32 B, coalesced); a
// closest hit is one 16-byte store, an any-hit answer one byte.
template <int STACK, bool ANY>
__global__ void __launch_bounds__(128) k_trace(const __grid_constant__ DevBVH bvh, const float4* __restrict__ rays,
                                               uint32_t n,
                                               const uint32_t* __restrict__ order, float4* __restrict__ hits,
                                               uint8_t* __restrict__ occ, int* __restrict__ status,
                                               uint32_t* __restrict__ replay) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (order) i = __ldg(order + i);
    float4 a = __ldg(rays + 2 * (size_t)i), b = __ldg(rays + 2 * (size_t)i + 1);
    DRay r = make_dray(a, b);
    TraceResult res;
    int st = 0;
    bool nan_hit = false;
    bool found = traverse<STACK, ANY>(bvh, r, &res, &st, &nan_hit);
    if (st) atomicMax(status, st);
    if (ANY) {
        occ[i] = found ? 1 : 0;
    } else if (nan_hit) {
        hits[i] = make_float4(__int_as_float(kReplayMark), 0.0f, 0.0f, 0.0f);
        *replay = 1u;
    } else {
        hits[i] = make_float4(__int_as_float(res.prim), res.t, res.b1, res.b2);
    }
}

// One thread per ray; a warp whose rays share their direction signs walks
// them together (traverse_packet), any other warp walks each lane's ray on
// its own (traverse).  Results equal k_trace's bit for bit.
template <int STACK, bool ANY>
__global__ void __launch_bounds__(128) k_trace_packet(const __grid_constant__ DevBVH bvh,
                                                      const float4* __restrict__ rays, uint32_t n,
                                                      const uint32_t* __restrict__ order, float4* __restrict__ hits,
                                                      uint8_t* __restrict__ occ, int* __restrict__ status,
                                                      uint32_t* __restrict__ replay) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = i < n;  // every lane stays for the warp's votes
    if (active && order) i = __ldg(order + i);
    DRay r = make_dray(active ? __ldg(rays + 2 * (size_t)i) : make_float4(0, 0, 0, 0),
                       active ? __ldg(rays + 2 * (size_t)i + 1) : make_float4(0, 0, 1, 0));
    TraceResult res;
    int st = 0;
    bool nan_hit = false, found = false;
    if (warp_signs_uniform(r, active))
        found = traverse_packet<STACK, ANY>(bvh, r, active, &res, &st, &nan_hit);
    else if (active)
        found = traverse<STACK, ANY>(bvh, r, &res, &st, &nan_hit);
    if (!active) return;
    if (st) atomicMax(status, st);
    if (ANY) {
        occ[i] = found ? 1 : 0;
    } else if (nan_hit) {
        hits[i] = make_float4(__int_as_float(kReplayMark), 0.0f, 0.0f, 0.0f);
        *replay = 1u;
    } else {
        hits[i] = make_float4(__int_as_float(res.prim), res.t, res.b1, res.b2);
    }
}

// Persistent warps: the grid holds exactly the resident warps; each warp
// owns a contiguous range of rays and, whenever at least REFILL of its
// lanes are idle, hands them the next rays of its range.  Rays of very
// different lengths then share warps without leaving lanes idle until the
// longest one finishes.  Each ray's own traversal is unchanged, so results
// are identical to k_trace.
template <int STACK, bool ANY, bool INST = false>
__global__ void __launch_bounds__(128) k_trace_persistent(const __grid_constant__ DevBVH bvh,
                                                          const float4* __restrict__ rays, uint32_t n,
                                                          const uint32_t* __restrict__ order, float4* __restrict__ hits,
                                                          uint8_t* __restrict__ occ, int* __restrict__ status,
                                                          uint32_t per_warp, uint32_t refill,
                                                          uint32_t* __restrict__ replay) {
    const unsigned lane = threadIdx.x & 31u;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint64_t next = warp * per_warp;
    const uint64_t end = (next + per_warp < (uint64_t)n) ? next + per_warp : (uint64_t)n;
    const uint32_t kNone = 0xffffffffu;
    uint32_t ray = kNone;
    int st = 0;
    DRay r;
    Traversal<STACK, INST> T;
    T.found = false;
    auto finish = [&]() {
        if (ANY) {
            occ[ray] = T.found ? 1 : 0;
        } else {
            if (T.nan_hit) {
                hits[ray] = make_float4(__int_as_float(kReplayMark), 0.0f, 0.0f, 0.0f);
                *replay = 1u;
            } else {
                hits[ray] = make_float4(__int_as_float(T.res.prim), T.res.t, T.res.b1, T.res.b2);
            }
        }
        ray = kNone;
    };
    for (;;) {
        unsigned idle = __ballot_sync(0xffffffffu, ray == kNone);
        unsigned nidle = __popc(idle);
        if (next < end && nidle >= (next + nidle >= end ? 1u : refill)) {
            if (ray == kNone) {
                uint64_t my = next + __popc(idle & ((1u << lane) - 1u));
                if (my < end) {
                    ray = order ? __ldg(order + my) : (uint32_t)my;
                    r = make_dray(__ldg(rays + 2 * (size_t)ray), __ldg(rays + 2 * (size_t)ray + 1));
                    if (!T.start(bvh, r)) finish();
                }
            }
            next += nidle;
        }
        bool busy = ray != kNone;
        if (!__any_sync(0xffffffffu, busy)) {
            if (next >= end) break;
            continue;
        }
        if (busy && !T.template step<ANY>(bvh, r, &st)) finish();
    }
    if (st) atomicMax(status, st);
}

// 4-wide traversal, one thread per ray.
template <int SMAX, int OVF, bool ANY>
__global__ void __launch_bounds__(128) k_trace4(const __grid_constant__ DevBVH4 bvh, const float4* __restrict__ rays,
                                                uint32_t n,
                                                const uint32_t* __restrict__ order, float4* __restrict__ hits,
                                                uint8_t* __restrict__ occ, int* __restrict__ status,
                                                uint32_t* __restrict__ replay) {
    extern __shared__ uint2 smem_stack[];
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (order) i = __ldg(order + i);
    DRay r = make_dray(__ldg(rays + 2 * (size_t)i), __ldg(rays + 2 * (size_t)i + 1));
    Traversal4<SMAX, OVF> T;
    T.bind(smem_stack, threadIdx.x, blockDim.x);
    if (T.start(bvh, r))
        while (T.template step<ANY>(bvh, r)) {
        }
    if (T.overflow) atomicMax(status, 6);
    if (ANY) {
        occ[i] = T.found ? 1 : 0;
    } else {
        if (T.nan_hit) {
            hits[i] = make_float4(__int_as_float(kReplayMark), 0.0f, 0.0f, 0.0f);
            *replay = 1u;
        } else {
            hits[i] = make_float4(__int_as_float(T.res.prim), T.res.t, T.res.b1, T.res.b2);
        }
    }
}

// A ray is read once: its lines go to L2 only, leaving L1 to the tree.
__device__ __forceinline__ float4 ld_stream(const float4* p) {
    float4 v;
    asm volatile("ld.global.nc.L1::no_allocate.v4.f32 {%0,%1,%2,%3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "l"(p));
    return v;
}

// Streamed input: the rays arrive in pieces of 2^piece_shift rays while the
// traversal already runs, and ready[k] turns non-zero once piece k has
// landed (the copy stream writes it with a 4-byte copy queued behind the
// piece's own copy).  %globaltimer is the GPU's nanosecond clock.
__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
// A flag that has not come within `wait_ms` means the copies did not run
// beside the walk (or at all), and the warp gives up instead of hanging (at
// once when another warp already gave up: *status holds the timeout).
__device__ __noinline__ bool wait_piece(const uint32_t* ready, uint32_t k, uint32_t wait_ms, const int* status) {
    if (ld_acquire_u32(ready + k)) return true;
    const uint64_t t0 = global_ns(), limit = (uint64_t)wait_ms * 1000000ull;
    for (;;) {
        __nanosleep(256);
        if (ld_acquire_u32(ready + k)) return true;
        if (global_ns() - t0 > limit ||
            ld_acquire_u32(reinterpret_cast<const uint32_t*>(status)) == (uint32_t)PBRT_ERR_TIMEOUT)
            return false;
    }
}

// 4-wide traversal with persistent warps refilling idle lanes (see
// k_trace_persistent).  Without `work`, warp w owns rays
// [w * per_warp, (w + 1) * per_warp); with it, warps take chunks of
// per_warp rays from the shared counter *work (zero at launch) whenever
// their chunk is used up, so warps that drew short rays take more of them
// and no warp is left with a long tail.  With `ready` (streamed input; only
// with `work`, which hands out chunks in ray order) a warp that takes a
// chunk first waits for the piece holding its last ray, and reads rays
// through L2 (they are written while the kernel runs); a wait that runs out
// sets PBRT_ERR_TIMEOUT and the warp drops its chunk.
//
// HOSTOUT (closest hits, with `work`): `hits` is a device staging array and
// `host_hits` the caller's pinned host memory mapped into the device's
// address space.  Scattered 16-byte stores across NVLink-C2C run at a fifth
// of its bandwidth (measured on GB300: 37 against 191 GB/s for 1 KiB runs),
// so each warp counts its chunks' finished rays in a ring of 4 slots in
// shared memory and copies a chunk's hits from the staging array to the
// host in coalesced rows once its last ray is done; a warp takes a new
// chunk only when a slot is free (always the case once all its lanes are
// idle).  The copies spread over the walk, sharing the link with the
// streamed input.
constexpr uint32_t kRingWords = 10 + 32;  // HOSTOUT: per warp, see k_trace4_persistent
// HOSTOUT's copy of finished chunks (ring[9]: one bit per slot) from the
// staging array to the host, one row of the warp's lanes at a time; out of
// line, so that the walk keeps its registers.
static __device__ __noinline__ void write_out_chunks(uint32_t* ring, const float4* hits, float4* host_hits, uint32_t n,
                                                     uint32_t per_warp) {
    const unsigned lane = threadIdx.x & 31u;
    uint32_t dm = ring[9];
    __syncwarp();
    if (lane == 0) ring[9] = 0u;
    while (dm) {
        const uint32_t j = (uint32_t)(__ffs(dm) - 1);
        dm &= dm - 1u;
        const uint32_t base = ring[4 + j];
        const uint32_t cnt = min(per_warp, n - base);
        for (uint32_t k = lane; k < cnt; k += 32u) host_hits[base + k] = __ldcg(hits + base + k);
    }
}
template <int SMAX, int OVF, bool ANY, int MINB, bool INST = false, bool HOSTOUT = false>
__global__ void __launch_bounds__(128, MINB)
    k_trace4_persistent(const __grid_constant__ DevBVH4 bvh, const float4* __restrict__ rays, uint32_t n,
                        const uint32_t* __restrict__ order,
                        float4* __restrict__ hits, uint8_t* __restrict__ occ, int* __restrict__ status,
                        uint32_t per_warp, uint32_t refill, uint32_t* __restrict__ work,
                        uint32_t* __restrict__ replay, const StreamIn in, float4* __restrict__ host_hits) {
    static_assert(!(HOSTOUT && ANY), "host write-out is for closest hits");
    extern __shared__ uint2 smem_stack[];
    const unsigned lane = threadIdx.x & 31u;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    // ray positions (32 bits suffice for the counter mode, n <= 0xF0000000)
    using Pos = typename std::conditional<HOSTOUT, uint32_t, uint64_t>::type;
    Pos next = work ? 0 : (Pos)(warp * per_warp);
    Pos end = work ? 0 : (Pos)((warp * per_warp + per_warp < (uint64_t)n) ? warp * per_warp + per_warp : (uint64_t)n);
    bool more = work != nullptr;  // the shared counter may still hold rays
    const uint32_t kNone = 0xffffffffu;
    uint32_t ray = kNone;
    bool overflow = false;
    DRay r;
    Traversal4<SMAX, OVF, INST> T;
    T.bind(smem_stack, threadIdx.x, blockDim.x);
    // HOSTOUT: this warp's ring in shared memory: rays left in slot j at
    // ring[j], the slot's first ray at ring[4 + j], the slot of the chunk
    // being handed out at ring[8], the slots whose last ray finished (a bit
    // each) at ring[9], then each lane's slot at ring[10 + lane].  Nothing of
    // it lives in registers, which the walk needs.
    auto ring_of = [&]() -> uint32_t* {
        uint32_t tid;  // read afresh at each use: the address is not kept in a register across the walk
        asm volatile("mov.u32 %0, %%tid.x;" : "=r"(tid));
        return reinterpret_cast<uint32_t*>(smem_stack + SMAX * blockDim.x) + (tid >> 5) * kRingWords;
    };
    if constexpr (HOSTOUT) {
        if (lane < 10) ring_of()[lane] = 0u;
        __syncwarp();
    }
    auto put = [&](float4 h) {
        // written once and not read here: streaming, except the staged hits
        // that the write-out reads back
        if constexpr (HOSTOUT)
            hits[ray] = h;
        else
            __stcs(hits + ray, h);
        if constexpr (HOSTOUT) {
            uint32_t* ring = ring_of();
            const uint32_t j = ring[10 + lane];
            if (atomicSub(ring + j, 1u) == 1u) atomicOr(ring + 9, 1u << j);
        }
    };
    // HOSTOUT: the chunks whose last ray finished go out to the host.  Done
    // when the warp takes its next chunk (which needs a slot) and at the
    // end, not at every step of the walk.
    auto write_out = [&]() {
        if constexpr (HOSTOUT) {
            __syncwarp();  // the chunks' staged hits and the ring are visible to every lane
            uint32_t* ring = ring_of();
            if (ring[9]) write_out_chunks(ring, hits, host_hits, n, per_warp);
        }
    };
    for (;;) {
        unsigned idle = __ballot_sync(0xffffffffu, ray == kNone);
        unsigned nidle = __popc(idle);
        if (more && next >= end && nidle >= refill) {  // warp-uniform
            int fs = 0;  // HOSTOUT: a free slot for the next chunk, -1 when none is
            if constexpr (HOSTOUT) {
                write_out();  // frees the slots of finished chunks
                __syncwarp();
                const uint32_t* ring = ring_of();
                fs = -1;
                for (int j = 3; j >= 0; --j)
                    if (ring[j] == 0u) fs = j;
            }
            if (fs >= 0) {
                uint32_t base = 0;
                if (lane == 0) base = atomicAdd(work, per_warp);
                base = __shfl_sync(0xffffffffu, base, 0);
                if (base < n) {
                    next = base;
                    end = (Pos)((uint64_t)base + per_warp < (uint64_t)n ? (uint64_t)base + per_warp : (uint64_t)n);
                    if (in.ready) {  // streamed input: the chunk's rays must have landed
                        int ok = 1;
                        if (lane == 0)
                            ok = wait_piece(in.ready, (uint32_t)((end - 1) >> in.shift), in.wait_ms, status) ? 1 : 0;
                        if (!__shfl_sync(0xffffffffu, ok, 0)) {
                            if (lane == 0) atomicMax(status, PBRT_ERR_TIMEOUT);
                            next = end;
                            more = false;
                        }
                    }
                    if constexpr (HOSTOUT) {
                        if (next < end) {
                            if (lane == 0) {
                                uint32_t* ring = ring_of();
                                ring[fs] = (uint32_t)(end - next);
                                ring[4 + fs] = base;
                                ring[8] = (uint32_t)fs;
                            }
                            __syncwarp();
                        }
                    }
                } else {
                    more = false;
                }
            }
        }
        const bool tail = !more && next + nidle >= end;
        if (next < end && nidle >= (tail ? 1u : refill)) {
            if (ray == kNone) {
                const Pos my = next + __popc(idle & ((1u << lane) - 1u));
                if (my < end) {
                    ray = order ? __ldg(order + my) : (uint32_t)my;
                    if constexpr (HOSTOUT) {
                        uint32_t* ring = ring_of();
                        ring[10 + lane] = ring[8];
                    }
                    const float4* rp = rays + 2 * (size_t)ray;
                    r = in.ready ? make_dray(__ldcg(rp), __ldcg(rp + 1)) : make_dray(ld_stream(rp), ld_stream(rp + 1));
                    bool live = T.start(bvh, r);
                    if (!live) {
                        if (ANY)
                            occ[ray] = 0;
                        else
                            put(make_float4(__int_as_float(-1), 0.0f, 0.0f, 0.0f));
                        ray = kNone;
                    }
                }
            }
            next += nidle;
        }
        bool busy = ray != kNone;
        if (!__any_sync(0xffffffffu, busy)) {
            if (next >= end && !more) break;
            continue;
        }
        if (busy && !T.template step<ANY>(bvh, r)) {
            overflow |= T.overflow;
            if (ANY) {
                occ[ray] = T.found ? 1 : 0;
            } else {
                if (T.nan_hit) {
                    put(make_float4(__int_as_float(kReplayMark), 0.0f, 0.0f, 0.0f));
                    *replay = 1u;
                } else {
                    put(make_float4(__int_as_float(T.res.prim), T.res.t, T.res.b1, T.res.b2));
                }
            }
            ray = kNone;
        }
    }
    write_out();
    if (overflow) atomicMax(status, 6);
}

// 4-wide persistent traversal with postponed leaves.  A lane that reaches a
// leaf keeps it aside and carries on down its stack; the warp tests the kept
// leaves together once enough lanes are stuck behind a second leaf (or have
// nothing else left), so the leaf code runs with many lanes instead of one
// or two.  A kept leaf is always tested before the lane's next leaf, so
// primitives are still tested in the reference's depth-first order; the
// nodes a lane visits while a leaf is kept are tested against a maxt that
// the kept leaf may still shrink, so some nodes the reference culls are
// visited too - their primitives are all farther than the closest hit - and
// the result, ties included, is the reference's.  Work comes from the
// shared counter (chunks of per_warp rays) or from fixed per-warp ranges.
template <int SMAX, int OVF, bool ANY>
__global__ void __launch_bounds__(128)
    k_trace4_spec(DevBVH4 bvh, const float4* __restrict__ rays, uint32_t n, const uint32_t* __restrict__ order,
                  float4* __restrict__ hits, uint8_t* __restrict__ occ, int* __restrict__ status, uint32_t per_warp,
                  uint32_t refill, uint32_t* __restrict__ work) {
    extern __shared__ uint2 smem_stack[];
    const unsigned lane = threadIdx.x & 31u;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint64_t next = work ? 0 : warp * per_warp;
    uint64_t end = work ? 0 : ((next + per_warp < (uint64_t)n) ? next + per_warp : (uint64_t)n);
    bool more = work != nullptr;
    const uint32_t kNone = 0xffffffffu;
    uint32_t ray = kNone;
    uint32_t kept = kNone;  // postponed leaf
    bool live = false;      // `T.cur` holds the next node or leaf
    bool overflow = false;
    DRay r;
    Traversal4<SMAX, OVF> T;
    T.bind(smem_stack, threadIdx.x, blockDim.x);
    auto finish = [&]() {
        overflow |= T.overflow;
        if (ANY)
            occ[ray] = T.found ? 1 : 0;
        else
            hits[ray] = make_float4(__int_as_float(T.res.prim), T.res.t, T.res.b1, T.res.b2);
        ray = kNone;
        kept = kNone;
        live = false;
    };
    for (;;) {
        const unsigned idle = __ballot_sync(0xffffffffu, ray == kNone);
        const unsigned nidle = __popc(idle);
        if (more && next >= end && nidle >= refill) {  // warp-uniform
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(work, per_warp);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base < n) {
                next = base;
                end = (uint64_t)base + per_warp < (uint64_t)n ? (uint64_t)base + per_warp : (uint64_t)n;
            } else {
                more = false;
            }
        }
        const bool tail = !more && next + nidle >= end;
        if (next < end && nidle >= (tail ? 1u : refill)) {
            if (ray == kNone) {
                const uint64_t my = next + __popc(idle & ((1u << lane) - 1u));
                if (my < end) {
                    ray = order ? __ldg(order + my) : (uint32_t)my;
                    r = make_dray(__ldg(rays + 2 * (size_t)ray), __ldg(rays + 2 * (size_t)ray + 1));
                    live = T.start(bvh, r);
                    if (!live) finish();
                }
            }
            next += nidle;
        }
        const bool busy = ray != kNone;
        if (!__any_sync(0xffffffffu, busy)) {
            if (next >= end && !more) break;
            continue;
        }
        const bool at_leaf = busy && live && (T.cur & kNode4Leaf);
        const bool blocked = busy && kept != kNone && (at_leaf || !live);
        const unsigned nbusy = __popc(__ballot_sync(0xffffffffu, busy));
        const unsigned nblocked = __popc(__ballot_sync(0xffffffffu, blocked));
        const unsigned nkept = __popc(__ballot_sync(0xffffffffu, busy && kept != kNone));
        if (nblocked && (4 * nblocked >= nbusy || nkept == nbusy)) {
            // leaf round: every kept leaf is tested now
            if (busy && kept != kNone) {
                const bool stop = T.template leaf<ANY>(bvh, r, kept) == 1;
                kept = kNone;
                if (stop || T.overflow) finish();
            }
        } else if (busy && live && !blocked) {  // a blocked lane waits for the leaf round
            if (at_leaf) {  // keep it, go on with the next stack entry
                kept = T.cur;
                live = T.pop();
            } else {
                live = T.template node<ANY>(bvh, r);
                if (T.overflow) finish();
            }
        }
        if (ray != kNone && !live && kept == kNone) finish();
    }
    if (overflow) atomicMax(status, 6);
}

enum {
    kVariantPairPlain = 0,
    kVariantPairPersistent = 1,
    kVariantWidePlain = 2,
    kVariantWidePersistent = 3,
    kVariantWideSpeculative = 4,
    kVariantPairPacket = 5
};
static int g_kernel_variant = -1;
static unsigned g_refill = 4;
static unsigned g_min_blocks = 0;
static int g_render_kernel = kVariantPairPlain;
static unsigned g_reorder = 0;
static unsigned g_chunk = 64;

static int variant_from_name(const char* v, int dflt) {
    if (!strcmp(v, "plain")) return kVariantPairPlain;
    if (!strcmp(v, "pt")) return kVariantPairPersistent;
    if (!strcmp(v, "w4")) return kVariantWidePlain;
    if (!strcmp(v, "w4pt")) return kVariantWidePersistent;
    if (!strcmp(v, "w4spec")) return kVariantWideSpeculative;
    if (!strcmp(v, "packet")) return kVariantPairPacket;
    return dflt;
}

static void read_variant() {
    if (g_kernel_variant >= 0) return;
    g_kernel_variant = kVariantWidePersistent;
    if (const char* v = getenv("PBRT_TRACE_KERNEL")) g_kernel_variant = variant_from_name(v, g_kernel_variant);
    if (const char* r = getenv("PBRT_TRACE_REFILL")) {
        int x = atoi(r);
        if (x >= 1 && x <= 32) g_refill = (unsigned)x;
    }
    if (const char* m = getenv("PBRT_TRACE_MINB")) {
        int x = atoi(m);
        if (x == 0 || x == 7 || x == 8 || x == 9) g_min_blocks = (unsigned)x;
    }
    if (const char* v = getenv("PBRT_TRACE_CHUNK")) {
        int x = atoi(v);
        if (x == 0 || (x >= 32 && x <= 4096 && x % 32 == 0)) g_chunk = (unsigned)x;
    }
    if (const char* v = getenv("PBRT_TRACE_REORDER")) {
        if (!strcmp(v, "0") || !strcmp(v, "1")) g_reorder = (unsigned)(v[0] - '0');
    }
    if (const char* v = getenv("PBRT_RENDER_KERNEL")) {
        int k = variant_from_name(v, g_render_kernel);
        if (k >= kVariantPairPlain && k <= kVariantPairPacket) g_render_kernel = k;
    }
}

// Rewrites the closest hits marked kReplayMark by the EXACT walk (see
// Traversal in trace.cuh); returns at once when no ray of the launch was
// marked, so a launch without NaN-distance hits pays one empty kernel.
// `host_hits` (may be null): a second copy of the hits that the rewritten
// ones also go to (the host memory of a write-out walk).
template <int SMAX, int OVF, bool INST>
__global__ void __launch_bounds__(128) k_replay4(const __grid_constant__ DevBVH4 bvh, const float4* __restrict__ rays,
                                                 uint32_t n, float4* __restrict__ hits,
                                                 const uint32_t* __restrict__ replay, int* __restrict__ status,
                                                 float4* __restrict__ host_hits) {
    extern __shared__ uint2 smem_stack[];
    if (*(const volatile uint32_t*)replay == 0u) return;
    Traversal4<SMAX, OVF, INST, true, true> T;
    T.bind(smem_stack, threadIdx.x, blockDim.x);
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        if (__float_as_int(hits[i].x) != kReplayMark) continue;
        DRay r = make_dray(__ldg(rays + 2 * i), __ldg(rays + 2 * i + 1));
        if (T.start(bvh, r)) {
            while (T.template step<false>(bvh, r)) {
            }
        }
        if (T.overflow) atomicMax(status, 6);
        hits[i] = make_float4(__int_as_float(T.res.prim), T.res.t, T.res.b1, T.res.b2);
        if (host_hits) host_hits[i] = hits[i];
    }
}

template <int STACK, bool INST>
__global__ void __launch_bounds__(128) k_replay2(const __grid_constant__ DevBVH bvh, const float4* __restrict__ rays,
                                                 uint32_t n, float4* __restrict__ hits,
                                                 const uint32_t* __restrict__ replay, int* __restrict__ status) {
    if (*(const volatile uint32_t*)replay == 0u) return;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        if (__float_as_int(hits[i].x) != kReplayMark) continue;
        DRay r = make_dray(__ldg(rays + 2 * i), __ldg(rays + 2 * i + 1));
        TraceResult res;
        int st = 0;
        traverse<STACK, false, INST, true>(bvh, r, &res, &st);
        if (st) atomicMax(status, st);
        hits[i] = make_float4(__int_as_float(res.prim), res.t, res.b1, res.b2);
    }
}

// `host_hits` (closest hits, with `work`): the HOSTOUT walk, `h4` its
// staging array.
template <int SMAX, int OVF, bool ANY, int MINB, bool INST = false, bool HOSTOUT = false>
static cudaError_t launch_wide_persistent(const DevBVH4& bvh, const float4* r4, uint32_t n, const uint32_t* order,
                                          float4* h4, uint8_t* occ, int* d_status, cudaStream_t stream,
                                          uint32_t* work, uint32_t* replay, StreamIn in = {},
                                          float4* host_hits = nullptr) {
    const int block = 128;
    // HOSTOUT: each warp's ring after the stacks
    const size_t smem = (size_t)SMAX * sizeof(uint2) * block + (HOSTOUT ? (block / 32) * kRingWords * sizeof(uint32_t) : 0);
    static ShapeCache bps_cache;
    const int sms = device_sms();
    const int bps = resident_blocks(bps_cache, k_trace4_persistent<SMAX, OVF, ANY, MINB, INST, HOSTOUT>, block, smem);
    uint64_t warps = (uint64_t)sms * bps * (block / 32);
    uint32_t per_warp = (uint32_t)((n + warps - 1) / warps);
    if (per_warp < 32) per_warp = 32;
    if (work && g_chunk && n <= 0xF0000000u) {  // the counter cannot wrap past n
        // every resident warp, each taking g_chunk rays at a time; no more
        // warps than chunks
        uint64_t chunks = (n + g_chunk - 1) / g_chunk;
        uint64_t w = chunks < warps ? chunks : warps;
        unsigned grid = (unsigned)((w + (block / 32) - 1) / (block / 32));
        k_trace4_persistent<SMAX, OVF, ANY, MINB, INST, HOSTOUT><<<grid, block, smem, stream>>>(
            bvh, r4, n, order, h4, occ, d_status, g_chunk, g_refill, work, replay, in, host_hits);
        return cudaGetLastError();
    }
    // fixed per-warp ranges would read rays out of order and have no chunks
    // to write out: no streamed input, no write-out
    if (in.ready || HOSTOUT) return cudaErrorInvalidValue;
    uint64_t need_warps = (n + per_warp - 1) / per_warp;
    unsigned grid = (unsigned)((need_warps + (block / 32) - 1) / (block / 32));
    k_trace4_persistent<SMAX, OVF, ANY, MINB, INST, HOSTOUT><<<grid, block, smem, stream>>>(
        bvh, r4, n, order, h4, occ, d_status, per_warp, g_refill, nullptr, replay, StreamIn{}, nullptr);
    return cudaGetLastError();
}

template <int SMAX, int OVF, bool ANY>
static cudaError_t launch_wide_spec(const DevBVH4& bvh, const float4* r4, uint32_t n, const uint32_t* order,
                                    float4* h4, uint8_t* occ, int* d_status, cudaStream_t stream, uint32_t* work) {
    const int block = 128;
    const size_t smem = (size_t)SMAX * sizeof(uint2) * block;
    static ShapeCache bps_cache;
    const int sms = device_sms();
    const int bps = resident_blocks(bps_cache, k_trace4_spec<SMAX, OVF, ANY>, block, smem);
    const uint64_t warps = (uint64_t)sms * bps * (block / 32);
    if (work && g_chunk && n <= 0xF0000000u) {
        const uint64_t chunks = (n + g_chunk - 1) / g_chunk;
        const uint64_t w = chunks < warps ? chunks : warps;
        const unsigned grid = (unsigned)((w + (block / 32) - 1) / (block / 32));
        k_trace4_spec<SMAX, OVF, ANY><<<grid, block, smem, stream>>>(bvh, r4, n, order, h4, occ, d_status, g_chunk,
                                                                   g_refill, work);
        return cudaGetLastError();
    }
    uint32_t per_warp = (uint32_t)((n + warps - 1) / warps);
    if (per_warp < 32) per_warp = 32;
    const uint64_t need_warps = (n + per_warp - 1) / per_warp;
    const unsigned grid = (unsigned)((need_warps + (block / 32) - 1) / (block / 32));
    k_trace4_spec<SMAX, OVF, ANY><<<grid, block, smem, stream>>>(bvh, r4, n, order, h4, occ, d_status, per_warp,
                                                               g_refill, nullptr);
    return cudaGetLastError();
}

template <int SMAX, int OVF, bool ANY>
static cudaError_t launch_wide(const DevBVH4& bvh, const float4* r4, uint32_t n, const uint32_t* order, float4* h4,
                               uint8_t* occ, int* d_status, cudaStream_t stream, bool persistent, uint32_t* work,
                               uint32_t* replay) {
    const int block = 128;
    const size_t smem = (size_t)SMAX * sizeof(uint2) * block;
    if (!persistent) {
        unsigned grid = (unsigned)((n + block - 1) / block);
        k_trace4<SMAX, OVF, ANY><<<grid, block, smem, stream>>>(bvh, r4, n, order, h4, occ, d_status, replay);
        return cudaGetLastError();
    }
    if (g_min_blocks == 7)
        return launch_wide_persistent<SMAX, OVF, ANY, 7>(bvh, r4, n, order, h4, occ, d_status, stream, work,
                                                         replay);
    if (g_min_blocks == 8)
        return launch_wide_persistent<SMAX, OVF, ANY, 8>(bvh, r4, n, order, h4, occ, d_status, stream, work,
                                                         replay);
    if (g_min_blocks == 9)
        return launch_wide_persistent<SMAX, OVF, ANY, 9>(bvh, r4, n, order, h4, occ, d_status, stream, work,
                                                         replay);
    return launch_wide_persistent<SMAX, OVF, ANY, 0>(bvh, r4, n, order, h4, occ, d_status, stream, work,
                                                         replay);
}

int set_trace_config(const PbrtTraceConfig& c) {
    if (c.kernel < kVariantPairPlain || c.kernel > kVariantPairPacket || c.refill < 1 || c.refill > 32) return 1;
    if (!(c.min_blocks == 0 || c.min_blocks == 7 || c.min_blocks == 8 || c.min_blocks == 9)) return 1;
    if (c.render_kernel < kVariantPairPlain || c.render_kernel > kVariantPairPacket) return 1;
    if (c.reorder > 1) return 1;
    if (!(c.chunk == 0 || (c.chunk >= 32 && c.chunk <= 4096 && c.chunk % 32 == 0))) return 1;
    read_variant();
    g_kernel_variant = c.kernel;
    g_refill = c.refill;
    g_min_blocks = c.min_blocks;
    g_render_kernel = c.render_kernel;
    g_reorder = c.reorder;
    g_chunk = c.chunk;
    return 0;
}
void get_trace_config(PbrtTraceConfig* c) {
    read_variant();
    c->kernel = g_kernel_variant;
    c->refill = g_refill;
    c->min_blocks = g_min_blocks;
    c->render_kernel = g_render_kernel;
    c->reorder = g_reorder;
    c->chunk = g_chunk;
}
unsigned trace_chunk() {
    read_variant();
    return g_chunk;
}
bool trace_reorder() {
    read_variant();
    return g_reorder != 0;
}
int render_trace_kernel() {
    read_variant();
    return g_render_kernel;
}

int wide_stack_variant(uint32_t bound) {
    if (bound <= 64) return 64;
    if (bound <= 256) return 256;
    return 0;
}

template <int STACK, bool ANY, bool INST = false>
static cudaError_t launch_persistent(const DevBVH& bvh, const float4* r4, uint32_t n, const uint32_t* order,
                                     float4* h4, uint8_t* occ, int* d_status, cudaStream_t stream,
                                     uint32_t* replay) {
    static ShapeCache bps_cache;  // one per instantiation
    const int block = 128;
    const int sms = device_sms();
    const int bps = resident_blocks(bps_cache, k_trace_persistent<STACK, ANY, INST>, block, 0);
    uint64_t warps = (uint64_t)sms * bps * (block / 32);
    uint32_t per_warp = (uint32_t)((n + warps - 1) / warps);
    if (per_warp < 32) per_warp = 32;
    uint64_t need_warps = (n + per_warp - 1) / per_warp;
    unsigned grid = (unsigned)((need_warps + (block / 32) - 1) / (block / 32));
    k_trace_persistent<STACK, ANY, INST><<<grid, block, 0, stream>>>(bvh, r4, n, order, h4, occ, d_status, per_warp,
                                                                     g_refill, replay);
    return cudaGetLastError();
}

int trace_stack_for_depth(uint32_t depth) {
    if (depth <= 64) return 64;
    if (depth <= 256) return 256;
    return 0;
}

static cudaError_t launch_main(const DevBVH& bvh, uint32_t depth, const PbrtRay* rays, uint32_t n, PbrtHit* hits,
                               uint8_t* occluded, int* d_status, cudaStream_t stream, const DevBVH4* wide,
                               uint32_t wide_bound, int kernel, const uint32_t* order, uint32_t* work,
                               uint32_t* replay) {
    if (bvh.insts) {
        // a scene with instances: the persistent walk with nested instance
        // traversal (4-wide when a variant covers the stack bound),
        // whatever the configured kernel
        const float4* r4 = reinterpret_cast<const float4*>(rays);
        float4* h4 = reinterpret_cast<float4*>(hits);
        const int stack = trace_stack_for_depth(depth);
        const bool any = occluded != nullptr;
        const int v = wide ? wide_stack_variant(wide_bound) : 0;
        if (v == 64)
            return any ? launch_wide_persistent<16, 48, true, 0, true>(*wide, r4, n, order, nullptr, occluded, d_status,
                                                                       stream, work, replay)
                       : launch_wide_persistent<16, 48, false, 0, true>(*wide, r4, n, order, h4, nullptr, d_status,
                                                                        stream, work, replay);
        if (v == 256)
            return any ? launch_wide_persistent<16, 240, true, 0, true>(*wide, r4, n, order, nullptr, occluded,
                                                                        d_status, stream, work, replay)
                       : launch_wide_persistent<16, 240, false, 0, true>(*wide, r4, n, order, h4, nullptr, d_status,
                                                                         stream, work, replay);
        if (stack == 64)
            return any ? launch_persistent<64, true, true>(bvh, r4, n, order, nullptr, occluded, d_status, stream, replay)
                       : launch_persistent<64, false, true>(bvh, r4, n, order, h4, nullptr, d_status, stream, replay);
        if (stack == 256)
            return any ? launch_persistent<256, true, true>(bvh, r4, n, order, nullptr, occluded, d_status, stream, replay)
                       : launch_persistent<256, false, true>(bvh, r4, n, order, h4, nullptr, d_status, stream, replay);
        return cudaErrorInvalidValue;
    }
    const int variant = kernel >= 0 ? kernel : g_kernel_variant;
    if (wide && variant == kVariantWideSpeculative) {
        const float4* r4 = reinterpret_cast<const float4*>(rays);
        float4* h4 = reinterpret_cast<float4*>(hits);
        const bool any = occluded != nullptr;
        const int v = wide_stack_variant(wide_bound);
        if (v == 64)
            return any ? launch_wide_spec<16, 48, true>(*wide, r4, n, order, nullptr, occluded, d_status, stream, work)
                       : launch_wide_spec<16, 48, false>(*wide, r4, n, order, h4, nullptr, d_status, stream, work);
        if (v == 256)
            return any ? launch_wide_spec<16, 240, true>(*wide, r4, n, order, nullptr, occluded, d_status, stream, work)
                       : launch_wide_spec<16, 240, false>(*wide, r4, n, order, h4, nullptr, d_status, stream, work);
    }
    if (wide && (variant == kVariantWidePlain || variant == kVariantWidePersistent)) {
        const float4* r4 = reinterpret_cast<const float4*>(rays);
        float4* h4 = reinterpret_cast<float4*>(hits);
        const bool any = occluded != nullptr, pt = variant == kVariantWidePersistent;
        int v = wide_stack_variant(wide_bound);
        if (v == 64)
            return any ? launch_wide<16, 48, true>(*wide, r4, n, order, nullptr, occluded, d_status, stream, pt, work, replay)
                       : launch_wide<16, 48, false>(*wide, r4, n, order, h4, nullptr, d_status, stream, pt, work, replay);
        if (v == 256)
            return any ? launch_wide<16, 240, true>(*wide, r4, n, order, nullptr, occluded, d_status, stream, pt, work, replay)
                       : launch_wide<16, 240, false>(*wide, r4, n, order, h4, nullptr, d_status, stream, pt, work, replay);
    }
    const int block = 128;
    const unsigned grid = (unsigned)((n + block - 1) / block);
    const float4* r4 = reinterpret_cast<const float4*>(rays);
    float4* h4 = reinterpret_cast<float4*>(hits);
    int stack = trace_stack_for_depth(depth);
    bool any = occluded != nullptr;
    if (variant == kVariantPairPersistent) {
        if (stack == 64)
            return any ? launch_persistent<64, true>(bvh, r4, n, order, nullptr, occluded, d_status, stream, replay)
                       : launch_persistent<64, false>(bvh, r4, n, order, h4, nullptr, d_status, stream, replay);
        if (stack == 256)
            return any ? launch_persistent<256, true>(bvh, r4, n, order, nullptr, occluded, d_status, stream, replay)
                       : launch_persistent<256, false>(bvh, r4, n, order, h4, nullptr, d_status, stream, replay);
        return cudaErrorInvalidValue;
    }
    if (variant == kVariantPairPacket) {
        if (stack == 64) {
            if (any)
                k_trace_packet<64, true><<<grid, block, 0, stream>>>(bvh, r4, n, order, nullptr, occluded, d_status,
                                                                     replay);
            else
                k_trace_packet<64, false><<<grid, block, 0, stream>>>(bvh, r4, n, order, h4, nullptr, d_status, replay);
        } else if (stack == 256) {
            if (any)
                k_trace_packet<256, true><<<grid, block, 0, stream>>>(bvh, r4, n, order, nullptr, occluded, d_status,
                                                                      replay);
            else
                k_trace_packet<256, false><<<grid, block, 0, stream>>>(bvh, r4, n, order, h4, nullptr, d_status,
                                                                       replay);
        } else {
            return cudaErrorInvalidValue;
        }
        return cudaGetLastError();
    }
    if (stack == 64) {
        if (any)
            k_trace<64, true><<<grid, block, 0, stream>>>(bvh, r4, n, order, nullptr, occluded, d_status, replay);
        else
            k_trace<64, false><<<grid, block, 0, stream>>>(bvh, r4, n, order, h4, nullptr, d_status, replay);
    } else if (stack == 256) {
        if (any)
            k_trace<256, true><<<grid, block, 0, stream>>>(bvh, r4, n, order, nullptr, occluded, d_status, replay);
        else
            k_trace<256, false><<<grid, block, 0, stream>>>(bvh, r4, n, order, h4, nullptr, d_status, replay);
    } else {
        return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

bool trace_streams(const DevBVH& bvh, const DevBVH4* wide, uint32_t wide_bound, uint32_t n) {
    read_variant();
    if (!wide || !wide_stack_variant(wide_bound) || !g_chunk || g_reorder || n > 0xF0000000u) return false;
    // scenes with instances always take the 4-wide persistent walk
    return bvh.insts != nullptr || (g_kernel_variant == kVariantWidePersistent && g_min_blocks == 0);
}

// The launch of a streamed-input or write-out call: the 4-wide persistent
// walk with its shared counter (the only kernel that takes rays in order).
static cudaError_t launch_streamed(const DevBVH& bvh, const PbrtRay* rays, uint32_t n, PbrtHit* hits,
                                   uint8_t* occ, int* d_status, cudaStream_t stream, const DevBVH4* wide,
                                   uint32_t wide_bound, uint32_t* work, uint32_t* replay, StreamIn in,
                                   PbrtHit* host_hits) {
    if (!work || !trace_streams(bvh, wide, wide_bound, n) || (host_hits && occ)) return cudaErrorInvalidValue;
    const float4* r4 = reinterpret_cast<const float4*>(rays);
    float4* h4 = reinterpret_cast<float4*>(hits);
    const bool any = occ != nullptr, inst = bvh.insts != nullptr;
    if (host_hits) {
        float4* hh = reinterpret_cast<float4*>(host_hits);
        if (wide_stack_variant(wide_bound) == 64)
            return inst ? launch_wide_persistent<16, 48, false, 0, true, true>(*wide, r4, n, nullptr, h4, nullptr,
                                                                              d_status, stream, work, replay, in,
                                                                              hh)
                        : launch_wide_persistent<16, 48, false, 0, false, true>(*wide, r4, n, nullptr, h4, nullptr,
                                                                               d_status, stream, work, replay, in,
                                                                               hh);
        return inst ? launch_wide_persistent<16, 240, false, 0, true, true>(*wide, r4, n, nullptr, h4, nullptr,
                                                                           d_status, stream, work, replay, in,
                                                                           hh)
                    : launch_wide_persistent<16, 240, false, 0, false, true>(*wide, r4, n, nullptr, h4, nullptr,
                                                                            d_status, stream, work, replay, in,
                                                                            hh);
    }
    if (wide_stack_variant(wide_bound) == 64) {
        if (inst)
            return any ? launch_wide_persistent<16, 48, true, 0, true>(*wide, r4, n, nullptr, nullptr, occ, d_status,
                                                                       stream, work, replay, in)
                       : launch_wide_persistent<16, 48, false, 0, true>(*wide, r4, n, nullptr, h4, nullptr, d_status,
                                                                        stream, work, replay, in);
        return any ? launch_wide_persistent<16, 48, true, 0>(*wide, r4, n, nullptr, nullptr, occ, d_status, stream,
                                                             work, replay, in)
                   : launch_wide_persistent<16, 48, false, 0>(*wide, r4, n, nullptr, h4, nullptr, d_status, stream,
                                                              work, replay, in);
    }
    if (inst)
        return any ? launch_wide_persistent<16, 240, true, 0, true>(*wide, r4, n, nullptr, nullptr, occ, d_status,
                                                                    stream, work, replay, in)
                   : launch_wide_persistent<16, 240, false, 0, true>(*wide, r4, n, nullptr, h4, nullptr, d_status,
                                                                     stream, work, replay, in);
    return any ? launch_wide_persistent<16, 240, true, 0>(*wide, r4, n, nullptr, nullptr, occ, d_status, stream,
                                                          work, replay, in)
               : launch_wide_persistent<16, 240, false, 0>(*wide, r4, n, nullptr, h4, nullptr, d_status, stream, work,
                                                           replay, in);
}

cudaError_t launch_trace(const DevBVH& bvh, uint32_t depth, const PbrtRay* rays, uint32_t n, PbrtHit* hits,
                         uint8_t* occluded, int* d_status, cudaStream_t stream, const DevBVH4* wide,
                         uint32_t wide_bound, int kernel, const uint32_t* order, uint32_t* work, uint32_t* replay,
                         StreamIn in, PbrtHit* host_hits) {
    if (n == 0) return cudaSuccess;
    if (!occluded && !replay) return cudaErrorInvalidValue;
    read_variant();
    if ((in.ready || host_hits) && order) return cudaErrorInvalidValue;
    cudaError_t e = in.ready || host_hits
                        ? launch_streamed(bvh, rays, n, hits, occluded, d_status, stream, wide, wide_bound, work,
                                          replay, in, host_hits)
                        : launch_main(bvh, depth, rays, n, hits, occluded, d_status, stream, wide, wide_bound, kernel,
                                      order, work, replay);
    if (e != cudaSuccess || occluded) return e;
    // the replay pass of closest hits (one empty launch unless a ray was marked)
    const unsigned grid = (unsigned)(device_sms() * 4);
    const float4* r4 = reinterpret_cast<const float4*>(rays);
    float4* h4 = reinterpret_cast<float4*>(hits);
    const bool inst = bvh.insts != nullptr;
    const int v = wide ? wide_stack_variant(wide_bound) : 0;
    const size_t smem = 16 * sizeof(uint2) * 128;
    float4* hh = reinterpret_cast<float4*>(host_hits);
    if (v == 64)
        inst ? k_replay4<16, 48, true><<<grid, 128, smem, stream>>>(*wide, r4, n, h4, replay, d_status, hh)
             : k_replay4<16, 48, false><<<grid, 128, smem, stream>>>(*wide, r4, n, h4, replay, d_status, hh);
    else if (v == 256)
        inst ? k_replay4<16, 240, true><<<grid, 128, smem, stream>>>(*wide, r4, n, h4, replay, d_status, hh)
             : k_replay4<16, 240, false><<<grid, 128, smem, stream>>>(*wide, r4, n, h4, replay, d_status, hh);
    else if (trace_stack_for_depth(depth) == 64)
        inst ? k_replay2<64, true><<<grid, 128, 0, stream>>>(bvh, r4, n, h4, replay, d_status)
             : k_replay2<64, false><<<grid, 128, 0, stream>>>(bvh, r4, n, h4, replay, d_status);
    else
        inst ? k_replay2<256, true><<<grid, 128, 0, stream>>>(bvh, r4, n, h4, replay, d_status)
             : k_replay2<256, false><<<grid, 128, 0, stream>>>(bvh, r4, n, h4, replay, d_status);
    return cudaGetLastError();
}

}  // namespace pbrt
