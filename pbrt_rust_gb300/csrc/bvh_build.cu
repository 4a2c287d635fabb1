// bvh_build.cu - BVHAccelerator::new's tree built on the device.
//
// The same tree as the host restatement (host_scene.cpp build_tree, itself
// the reference's recursive_build, src/primitive/aggregates/bvh.rs:86-258):
// the same nodes, bounds, split axes and primitive order, bit for bit.  The
// recursion becomes two phases over one array of primitive indices, every
// node owning a contiguous range of it:
//
//   A. ranges above kSmall (32) primitives, one tree level per round: every range
//      of the level is cut into chunks; chunk kernels reduce its bounds and
//      centroid bounds, fill the twelve SAH buckets (or test the middle
//      split) and count the left side, one thread per range picks the split,
//      and a stable scatter writes the two sides in their original order
//      (Iterator::partition keeps order, bvh.rs:89, 174).  The host reads the
//      few per-range decisions back and lays out the next level.
//   B. ranges of at most kSmall primitives: one thread runs the whole
//      subtree with the host algorithm (including partition_by for the
//      equal-counts split of ranges of up to four, utils/mod.rs:112-169),
//      writing its nodes in pre-order.
//
// Bounds are combined with a min/max that ignores NaN and orders -0 below
// +0, in any order; f32 bucket indices and SAH costs repeat the host's
// operations (--fmad=false).  The host then numbers all nodes in the
// reference's depth-first order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pbrt_gpu.h"
#include "host_scene.h"

namespace pbrt {

namespace {

#ifndef PBRT_BUILD_SMALL
#define PBRT_BUILD_SMALL 32
#endif
// ranges of at most this many primitives go to phase B (one thread each:
// small ranges keep that serial work short and the thread count high)
constexpr uint32_t kSmall = PBRT_BUILD_SMALL;
constexpr uint32_t kChunk = 2048; // phase A chunk
constexpr int kNB = 12;           // SAH buckets (bvh.rs:188)

// ---- order-independent min / max ------------------------------------------
// Floats as ints whose signed order is the float order with -0 < +0.
__host__ __device__ inline int32_t ord(float f) {
    int32_t i;
    memcpy(&i, &f, 4);
    return i >= 0 ? i : (int32_t)(i ^ 0x7fffffff);
}
__host__ __device__ inline float unord(int32_t i) {
    int32_t b = i >= 0 ? i : (int32_t)(i ^ 0x7fffffff);
    float f;
    memcpy(&f, &b, 4);
    return f;
}
__device__ inline float dmin(float a, float b) {  // std::fmin, -0 below +0
    if (a != a) return b;
    if (b != b) return a;
    return ord(a) <= ord(b) ? a : b;
}
__device__ inline float dmax(float a, float b) {
    if (a != a) return b;
    if (b != b) return a;
    return ord(a) >= ord(b) ? a : b;
}

struct DBox {
    float lx, ly, lz, hx, hy, hz;
};
__device__ inline DBox dbox_empty() { return DBox{FLT_MAX, FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX, -FLT_MAX}; }
__device__ inline DBox dunion(const DBox& a, const DBox& b) {
    return DBox{dmin(a.lx, b.lx), dmin(a.ly, b.ly), dmin(a.lz, b.lz),
                dmax(a.hx, b.hx), dmax(a.hy, b.hy), dmax(a.hz, b.hz)};
}
__device__ inline float darea(const DBox& b) {  // bbox.rs:73-78
    float dx = fmaxf(b.hx - b.lx, 0.0f), dy = fmaxf(b.hy - b.ly, 0.0f), dz = fmaxf(b.hz - b.lz, 0.0f);
    return 2.0f * (dx * dy + dx * dz + dy * dz);
}
__device__ inline int dmax_extent(const DBox& b) {  // bbox.rs:87-96
    float dx = b.hx - b.lx, dy = b.hy - b.ly, dz = b.hz - b.lz;
    if (dx > dy && dx > dz) return 0;
    if (dy > dz) return 1;
    return 2;
}
__device__ inline size_t to_usize(float f) {  // Rust `as usize`: saturating, NaN -> 0
    if (!(f > 0.0f)) return 0;
    if (f >= 18446744073709551615.0f) return (size_t)-1;
    return (size_t)f;
}
__device__ inline int bucket_of(float key, float cmin, float dist) {  // bvh.rs:118-131
    size_t b = to_usize((float)kNB * ((key - cmin) / dist));
    // key lies in [cmin, cmin + dist], so b <= kNB; the clamp only guards
    return b >= (size_t)kNB ? kNB - 1 : (int)b;
}

struct Prims {
    const float4* lo;   // bounds
    const float4* hi;
    const float* cen[3];  // centroids by axis
};
__device__ inline DBox pbox(const Prims& P, uint32_t p) {
    float4 a = __ldg(P.lo + p), b = __ldg(P.hi + p);
    return DBox{a.x, a.y, a.z, b.x, b.y, b.z};
}

// ---- phase A ---------------------------------------------------------------
struct Chunk {
    uint32_t seg, lo, hi, pad;
};
// Per range: [0..5] bounds, [6..11] centroid bounds (ord ints, min fields
// stored as is, max fields too), then 12 buckets of count + 6 bounds.
constexpr int kAccWords = 12 + kNB * 7;

struct SegDecision {   // filled by k_decide / k_choose
    float cmin, dist, pmid;
    int32_t dim;
    int32_t action;    // 0 leaf, 1 split by bucket <= best, 2 split by key < pmid
    int32_t best;
    float lo[3], hi[3];  // range bounds
};

__global__ void k_acc_init(int32_t* acc, uint32_t nseg) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nseg * kAccWords) return;
    const uint32_t w = i % kAccWords;
    int f;  // min fields start at +FLT_MAX, max fields at -FLT_MAX, counts at 0
    if (w < 12) {
        f = (w % 6) < 3 ? ord(FLT_MAX) : ord(-FLT_MAX);
    } else {
        const uint32_t k = (w - 12) % 7;
        f = k == 0 ? 0 : (k <= 3 ? ord(FLT_MAX) : ord(-FLT_MAX));
    }
    acc[i] = f;
}

__device__ inline void warp_min_to(int32_t v, int32_t* dst) {
    for (int o = 16; o; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) atomicMin(dst, v);
}
__device__ inline void warp_max_to(int32_t v, int32_t* dst) {
    for (int o = 16; o; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) atomicMax(dst, v);
}

// Bounds and centroid bounds of each range (NaN-free inputs: the int order
// then is the float order of dmin / dmax).
__global__ void __launch_bounds__(256) k_a_bounds(Prims P, const uint32_t* __restrict__ idx,
                                                  const Chunk* __restrict__ chunks, int32_t* acc) {
    const Chunk c = chunks[blockIdx.x];
    int32_t m[12];
    for (int k = 0; k < 12; ++k) m[k] = (k % 6) < 3 ? ord(FLT_MAX) : ord(-FLT_MAX);
    for (uint32_t i = c.lo + threadIdx.x; i < c.hi; i += blockDim.x) {
        const uint32_t p = __ldg(idx + i);
        const DBox b = pbox(P, p);
        const float cx = __ldg(P.cen[0] + p), cy = __ldg(P.cen[1] + p), cz = __ldg(P.cen[2] + p);
        m[0] = min(m[0], ord(b.lx)), m[1] = min(m[1], ord(b.ly)), m[2] = min(m[2], ord(b.lz));
        m[3] = max(m[3], ord(b.hx)), m[4] = max(m[4], ord(b.hy)), m[5] = max(m[5], ord(b.hz));
        m[6] = min(m[6], ord(cx)), m[7] = min(m[7], ord(cy)), m[8] = min(m[8], ord(cz));
        m[9] = max(m[9], ord(cx)), m[10] = max(m[10], ord(cy)), m[11] = max(m[11], ord(cz));
    }
    int32_t* a = acc + (size_t)c.seg * kAccWords;
    for (int k = 0; k < 12; ++k) {
        if ((k % 6) < 3)
            warp_min_to(m[k], a + k);
        else
            warp_max_to(m[k], a + k);
    }
}

// One thread per range: split axis and centroid extent (bvh.rs:208-217).
__global__ void k_a_decide(const int32_t* __restrict__ acc, SegDecision* dec, const uint32_t* __restrict__ counts,
                           uint32_t nseg, int split) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nseg) return;
    const int32_t* a = acc + (size_t)s * kAccWords;
    DBox cb{unord(a[6]), unord(a[7]), unord(a[8]), unord(a[9]), unord(a[10]), unord(a[11])};
    SegDecision d;
    for (int k = 0; k < 3; ++k) {
        d.lo[k] = unord(a[k]);
        d.hi[k] = unord(a[3 + k]);
    }
    d.dim = dmax_extent(cb);
    const float cmin = d.dim == 0 ? cb.lx : (d.dim == 1 ? cb.ly : cb.lz);
    const float cmax = d.dim == 0 ? cb.hx : (d.dim == 1 ? cb.hy : cb.hz);
    d.cmin = cmin;
    d.dist = cmax - cmin;
    d.pmid = 0.5f * (cmin + cmax);
    d.best = 0;
    if (counts[s] <= 1 || cmin == cmax)
        d.action = 0;
    else
        d.action = split == PBRT_SPLIT_MIDDLE ? 2 : 1;
    dec[s] = d;
}

// SAH buckets of each range.
__global__ void __launch_bounds__(256) k_a_buckets(Prims P, const uint32_t* __restrict__ idx,
                                                   const Chunk* __restrict__ chunks,
                                                   const SegDecision* __restrict__ dec, int32_t* acc) {
    __shared__ int32_t sb[kNB * 7];
    const Chunk c = chunks[blockIdx.x];
    const SegDecision d = dec[c.seg];
    if (d.action != 1) return;
    for (int i = threadIdx.x; i < kNB * 7; i += blockDim.x) {
        const int k = i % 7;
        sb[i] = k == 0 ? 0 : (k <= 3 ? ord(FLT_MAX) : ord(-FLT_MAX));
    }
    __syncthreads();
    const float* key = d.dim == 0 ? P.cen[0] : (d.dim == 1 ? P.cen[1] : P.cen[2]);
    for (uint32_t i = c.lo + threadIdx.x; i < c.hi; i += blockDim.x) {
        const uint32_t p = __ldg(idx + i);
        const int b = bucket_of(__ldg(key + p), d.cmin, d.dist);
        const DBox bx = pbox(P, p);
        int32_t* q = sb + b * 7;
        atomicAdd(q, 1);
        atomicMin(q + 1, ord(bx.lx)), atomicMin(q + 2, ord(bx.ly)), atomicMin(q + 3, ord(bx.lz));
        atomicMax(q + 4, ord(bx.hx)), atomicMax(q + 5, ord(bx.hy)), atomicMax(q + 6, ord(bx.hz));
    }
    __syncthreads();
    int32_t* a = acc + (size_t)c.seg * kAccWords + 12;
    for (int i = threadIdx.x; i < kNB * 7; i += blockDim.x) {
        const int k = i % 7;
        if (k == 0)
            atomicAdd(a + i, sb[i]);
        else if (k <= 3)
            atomicMin(a + i, sb[i]);
        else
            atomicMax(a + i, sb[i]);
    }
}

// One thread per range: the SAH costs in the host's order and the leaf test
// (bvh.rs:133-185).
__global__ void k_a_choose(const int32_t* __restrict__ acc, SegDecision* dec, const uint32_t* __restrict__ counts,
                           uint32_t nseg, uint32_t mp) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nseg) return;
    SegDecision d = dec[s];
    if (d.action != 1) return;
    const int32_t* a = acc + (size_t)s * kAccWords + 12;
    size_t bc[kNB];
    DBox bb[kNB];
    for (int i = 0; i < kNB; ++i) {
        const int32_t* q = a + i * 7;
        bc[i] = (size_t)q[0];
        bb[i] = DBox{unord(q[1]), unord(q[2]), unord(q[3]), unord(q[4]), unord(q[5]), unord(q[6])};
    }
    DBox total{d.lo[0], d.lo[1], d.lo[2], d.hi[0], d.hi[1], d.hi[2]};
    const float tsa = darea(total);
    int best = 0;
    float best_cost = FLT_MAX;
    for (int sp = 0; sp + 1 < kNB; ++sp) {
        size_t c0 = 0, c1 = 0;
        DBox b0 = dbox_empty(), b1 = dbox_empty();
        for (int j = 0; j <= sp; ++j) {
            c0 += bc[j];
            b0 = dunion(b0, bb[j]);
        }
        for (int j = sp + 1; j < kNB; ++j) {
            c1 += bc[j];
            b1 = dunion(b1, bb[j]);
        }
        const float cost = 0.125f * ((float)c0 * darea(b0) + (float)c1 * darea(b1)) / tsa;
        if (cost < best_cost) {
            best_cost = cost;
            best = sp;
        }
    }
    const size_t cnt = counts[s];
    if (!(mp < cnt || to_usize(best_cost) < cnt)) d.action = 0;  // a leaf of cnt primitives
    d.best = best;
    dec[s] = d;
}

__device__ inline bool goes_left(const Prims& P, const SegDecision& d, uint32_t p) {
    const float* key = d.dim == 0 ? P.cen[0] : (d.dim == 1 ? P.cen[1] : P.cen[2]);
    const float k = __ldg(key + p);
    if (d.action == 2) return k < d.pmid;
    return bucket_of(k, d.cmin, d.dist) <= d.best;
}

// Left-side count of every chunk.
__global__ void __launch_bounds__(256) k_a_count(Prims P, const uint32_t* __restrict__ idx,
                                                 const Chunk* __restrict__ chunks,
                                                 const SegDecision* __restrict__ dec, uint32_t* left) {
    const Chunk c = chunks[blockIdx.x];
    const SegDecision d = dec[c.seg];
    uint32_t n = 0;
    if (d.action != 0)
        for (uint32_t i = c.lo + threadIdx.x; i < c.hi; i += blockDim.x) n += goes_left(P, d, __ldg(idx + i));
    for (int o = 16; o; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
    __shared__ uint32_t ws[8];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = n;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += ws[w];
        left[blockIdx.x] = t;
    }
}

// Stable two-way scatter of every chunk: left side to base_left + rank,
// right side to base_right + rank, in index order.  base_* per chunk come
// from the host.
__global__ void __launch_bounds__(256) k_a_scatter(Prims P, const uint32_t* __restrict__ idx, uint32_t* out,
                                                   const Chunk* __restrict__ chunks,
                                                   const SegDecision* __restrict__ dec,
                                                   const uint2* __restrict__ base) {
    __shared__ uint32_t ws[8];
    __shared__ uint32_t carry;  // left elements of the chunk before this round
    const Chunk c = chunks[blockIdx.x];
    const SegDecision d = dec[c.seg];
    const uint2 b = base[blockIdx.x];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const unsigned lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (uint32_t i0 = c.lo; i0 < c.hi; i0 += blockDim.x) {
        const uint32_t i = i0 + threadIdx.x;
        const bool live = i < c.hi;
        const uint32_t p = live ? idx[i] : 0u;
        const bool left = live && (d.action == 0 || goes_left(P, d, p));  // leaves keep their order
        const unsigned m = __ballot_sync(0xffffffffu, left);
        if (lane == 0) ws[w] = __popc(m);
        __syncthreads();
        uint32_t before = 0, total = 0;
        for (unsigned k = 0; k < nw; ++k) {
            if (k < w) before += ws[k];
            total += ws[k];
        }
        // left elements before this one in the chunk, and right ones
        const uint32_t rank_l = carry + before + __popc(m & ((1u << lane) - 1u));
        const uint32_t rank_r = (i - c.lo) - rank_l;
        if (live) out[left ? b.x + rank_l : b.y + rank_r] = p;
        __syncthreads();
        if (threadIdx.x == 0) carry += total;
        __syncthreads();
    }
}

__global__ void k_copy_ranges(const uint32_t* __restrict__ src, uint32_t* dst, const Chunk* __restrict__ chunks) {
    const Chunk c = chunks[blockIdx.x];
    for (uint32_t i = c.lo + threadIdx.x; i < c.hi; i += blockDim.x) dst[i] = src[i];
}

// ---- phase B ---------------------------------------------------------------
struct Job {
    uint32_t lo, hi;   // primitive range
    uint32_t node0;    // first node slot in the pool
    uint32_t pad;
};
struct PoolNode {      // a = leaf ? first prim : second child (pool index); b = leaf ? kLeaf | count : axis
    float lo[3];
    uint32_t a;
    float hi[3];
    uint32_t b;
};
constexpr uint32_t kLeaf = 0x80000000u;
struct Task {
    uint32_t lo, hi;
    int32_t parent;
    uint32_t depth;
};
struct JobOut {
    uint32_t nodes, depth, err, pad;
};

// utils/mod.rs:112-169 (as host_scene.cpp partition_by_key)
__device__ void partition_by_key(uint32_t* v, uint32_t n, const float* key) {
    while (true) {
        if (n < 3) {
            if (n == 2 && key[v[1]] < key[v[0]]) {
                uint32_t t = v[0];
                v[0] = v[1];
                v[1] = t;
            }
            return;
        }
        float a = key[v[0]], b = key[v[n / 2]], c = key[v[n - 1]];
        float pivot = (a < b && b < c) ? b : ((b < a && a < c) ? a : c);
        uint32_t ls = 0, np = 0;
        for (uint32_t i = 0; i < n; ++i) {
            float k = key[v[i]];
            if (k < pivot) {
                uint32_t t = v[ls + np];
                v[ls + np] = v[i];
                v[i] = t;
                t = v[ls + np];
                v[ls + np] = v[ls];
                v[ls] = t;
                ++ls;
            } else if (k == pivot) {
                uint32_t t = v[ls + np];
                v[ls + np] = v[i];
                v[i] = t;
                ++np;
            }
        }
        uint32_t pi = ls > 1 ? ls : 1;
        if (pi + np <= n / 2) {
            v += pi;
            n -= pi;
        } else if (pi >= n / 2) {
            n = pi;
        } else {
            return;
        }
    }
}

// One thread per job: build_tree on [lo, hi) (host_scene.cpp), nodes in
// pre-order at pool[node0 ...]; `stack` and `tmp` are scratch at the same
// offsets as the range.
__global__ void __launch_bounds__(128) k_b_build(Prims P, uint32_t* idx, uint32_t* tmp, Task* stack,
                                                 const Job* __restrict__ jobs, uint32_t njobs, PoolNode* pool,
                                                 JobOut* outs, uint32_t mp, int split) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= njobs) return;
    const Job J = jobs[j];
    Task* st = stack + J.lo;
    uint32_t sp = 0, nn = 0, maxd = 0, err = 0;
    st[sp++] = Task{J.lo, J.hi, -1, 1};
    while (sp > 0) {
        const Task t = st[--sp];
        const uint32_t k = nn++;
        if (t.parent >= 0) pool[J.node0 + t.parent].a = k;
        maxd = max(maxd, t.depth);
        const uint32_t cnt = t.hi - t.lo;
        DBox bbox = dbox_empty();
        for (uint32_t i = t.lo; i < t.hi; ++i) bbox = dunion(bbox, pbox(P, idx[i]));
        uint32_t mid = 0;
        bool split_it = false;
        int dim = 0;
        if (cnt > 1) {
            DBox cb = dbox_empty();
            for (uint32_t i = t.lo; i < t.hi; ++i) {
                const uint32_t p = idx[i];
                const float cx = __ldg(P.cen[0] + p), cy = __ldg(P.cen[1] + p), cz = __ldg(P.cen[2] + p);
                cb = dunion(cb, DBox{cx, cy, cz, cx, cy, cz});
            }
            dim = dmax_extent(cb);
            const float cmin = dim == 0 ? cb.lx : (dim == 1 ? cb.ly : cb.lz);
            const float cmax = dim == 0 ? cb.hx : (dim == 1 ? cb.hy : cb.hz);
            const float* key = P.cen[dim];
            if (cmin != cmax) {
                auto stable_split = [&](auto pred) {
                    uint32_t w = t.lo, r = t.lo;
                    for (uint32_t i = t.lo; i < t.hi; ++i) {
                        const uint32_t p = idx[i];
                        if (pred(p))
                            idx[w++] = p;
                        else
                            tmp[r++] = p;
                    }
                    mid = w;
                    for (uint32_t i = t.lo; i < r; ++i) idx[w++] = tmp[i];
                    split_it = true;
                };
                if (split == PBRT_SPLIT_MIDDLE) {
                    const float p_mid = 0.5f * (cmin + cmax);
                    stable_split([&](uint32_t p) { return key[p] < p_mid; });
                } else if (split == PBRT_SPLIT_EQUAL || cnt <= 4) {
                    partition_by_key(idx + t.lo, cnt, key);
                    mid = t.lo + cnt / 2;
                    split_it = true;
                } else {
                    const float dist = cmax - cmin;
                    size_t bc[kNB];
                    DBox bb[kNB];
                    for (int i = 0; i < kNB; ++i) {
                        bc[i] = 0;
                        bb[i] = dbox_empty();
                    }
                    for (uint32_t i = t.lo; i < t.hi; ++i) {
                        const uint32_t p = idx[i];
                        const int b = bucket_of(key[p], cmin, dist);
                        bc[b] += 1;
                        bb[b] = dunion(bb[b], pbox(P, p));
                    }
                    const float tsa = darea(bbox);
                    int best = 0;
                    float best_cost = FLT_MAX;
                    for (int s = 0; s + 1 < kNB; ++s) {
                        size_t c0 = 0, c1 = 0;
                        DBox b0 = dbox_empty(), b1 = dbox_empty();
                        for (int q = 0; q <= s; ++q) {
                            c0 += bc[q];
                            b0 = dunion(b0, bb[q]);
                        }
                        for (int q = s + 1; q < kNB; ++q) {
                            c1 += bc[q];
                            b1 = dunion(b1, bb[q]);
                        }
                        const float cost = 0.125f * ((float)c0 * darea(b0) + (float)c1 * darea(b1)) / tsa;
                        if (cost < best_cost) {
                            best_cost = cost;
                            best = s;
                        }
                    }
                    if (mp < cnt || to_usize(best_cost) < cnt)
                        stable_split([&](uint32_t p) { return bucket_of(key[p], cmin, dist) <= best; });
                }
            }
        }
        PoolNode& N = pool[J.node0 + k];
        N.lo[0] = bbox.lx, N.lo[1] = bbox.ly, N.lo[2] = bbox.lz;
        N.hi[0] = bbox.hx, N.hi[1] = bbox.hy, N.hi[2] = bbox.hz;
        if (split_it) {
            if (mid == t.lo || mid == t.hi) err = 1;
            N.a = 0;
            N.b = (uint32_t)dim;
            st[sp++] = Task{mid, t.hi, (int32_t)k, t.depth + 1};
            st[sp++] = Task{t.lo, mid, -1, t.depth + 1};
            if (err) break;
        } else {
            N.a = t.lo;
            N.b = kLeaf | cnt;
        }
    }
    // inner bounds are the union of the two children (bvh.rs:247)
    for (uint32_t k = nn; k-- > 0;) {
        PoolNode& N = pool[J.node0 + k];
        if (N.b & kLeaf) continue;
        const PoolNode& L = pool[J.node0 + k + 1];
        const PoolNode& R = pool[J.node0 + N.a];
        for (int c = 0; c < 3; ++c) {
            N.lo[c] = dmin(L.lo[c], R.lo[c]);
            N.hi[c] = dmax(L.hi[c], R.hi[c]);
        }
    }
    outs[j] = JobOut{nn, maxd, err, 0};
}

// ---- host ------------------------------------------------------------------
struct Buf {  // a device allocation owned by the build
    void* p = nullptr;
    Buf() = default;
    Buf(const Buf&) = delete;
    Buf& operator=(const Buf&) = delete;
    ~Buf() { reset(); }
    void reset() {
        if (p) cudaFree(p);
        p = nullptr;
    }
    template <class T>
    T* as() {
        return static_cast<T*>(p);
    }
};

#define CK(x)                                                          \
    do {                                                               \
        cudaError_t e_ = (x);                                          \
        if (e_ != cudaSuccess) {                                       \
            *err = std::string("device BVH build: ") + cudaGetErrorString(e_); \
            return PBRT_ERR_CUDA;                                      \
        }                                                              \
    } while (0)

// Host tree of phase A: nodes with children or a phase-B job.
struct ANode {
    bool leaf = false, small = false;  // small: the subtree is job `job`
    uint32_t lo = 0, cnt = 0, dim = 0, depth = 1;
    int32_t left = -1, right = -1, job = -1;
    Box box{};
};

}  // namespace

int device_build_tree(HostBVH& H, uint32_t mp, int split, std::string* err) {
    const size_t n = H.prims.size();
    H.nodes.clear();
    H.ordered.resize(n);
    H.depth = 0;
    if (n == 0) return PBRT_OK;
    if (n >= (1u << 31)) {
        *err = "device BVH build: more than 2^31 primitives";
        return PBRT_ERR_UNSUPPORTED;
    }
    std::vector<Box> bounds;
    std::vector<float> cx, cy, cz;
    prim_bounds(H, &bounds, &cx, &cy, &cz);
    std::vector<float4> lo(n), hi(n);
    for (size_t i = 0; i < n; ++i) {
        lo[i] = make_float4(bounds[i].lo.x, bounds[i].lo.y, bounds[i].lo.z, 0.0f);
        hi[i] = make_float4(bounds[i].hi.x, bounds[i].hi.y, bounds[i].hi.z, 0.0f);
    }
    Buf d_lo, d_hi, d_c[3], d_idx, d_tmp, d_stack, d_pool;
    CK(cudaMalloc(&d_lo.p, n * sizeof(float4)));
    CK(cudaMalloc(&d_hi.p, n * sizeof(float4)));
    for (int k = 0; k < 3; ++k) CK(cudaMalloc(&d_c[k].p, n * sizeof(float)));
    CK(cudaMalloc(&d_idx.p, n * 4));
    CK(cudaMalloc(&d_tmp.p, n * 4));
    CK(cudaMemcpy(d_lo.p, lo.data(), n * sizeof(float4), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_hi.p, hi.data(), n * sizeof(float4), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_c[0].p, cx.data(), n * 4, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_c[1].p, cy.data(), n * 4, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_c[2].p, cz.data(), n * 4, cudaMemcpyHostToDevice));
    {
        std::vector<uint32_t> iota(n);
        for (size_t i = 0; i < n; ++i) iota[i] = (uint32_t)i;
        CK(cudaMemcpy(d_idx.p, iota.data(), n * 4, cudaMemcpyHostToDevice));
    }
    Prims P;
    P.lo = d_lo.as<float4>();
    P.hi = d_hi.as<float4>();
    for (int k = 0; k < 3; ++k) P.cen[k] = d_c[k].as<float>();

    // ---- phase A: one level per round
    std::vector<ANode> A;
    A.push_back(ANode{});
    A[0].lo = 0;
    A[0].cnt = (uint32_t)n;
    std::vector<uint32_t> level;  // phase-A nodes of this level
    std::vector<Job> jobs;
    auto to_small = [&](uint32_t a) {
        A[a].small = true;
        A[a].job = (int32_t)jobs.size();
        jobs.push_back(Job{A[a].lo, A[a].lo + A[a].cnt, 0, 0});
    };
    if (n <= kSmall)
        to_small(0);
    else
        level.push_back(0);
    Buf d_acc, d_dec, d_cnt, d_chunks, d_left, d_base;
    while (!level.empty()) {
        const uint32_t S = (uint32_t)level.size();
        std::vector<Chunk> chunks;
        std::vector<uint32_t> counts(S);
        for (uint32_t s = 0; s < S; ++s) {
            const ANode& a = A[level[s]];
            counts[s] = a.cnt;
            for (uint32_t o = 0; o < a.cnt; o += kChunk)
                chunks.push_back(Chunk{s, a.lo + o, a.lo + std::min(a.cnt, o + kChunk), 0});
        }
        const uint32_t NC = (uint32_t)chunks.size();
        // per-level buffers (freed by the next assignment)
        for (Buf* b : {&d_acc, &d_dec, &d_cnt, &d_chunks, &d_left, &d_base}) b->reset();
        CK(cudaMalloc(&d_acc.p, (size_t)S * kAccWords * 4));
        CK(cudaMalloc(&d_dec.p, (size_t)S * sizeof(SegDecision)));
        CK(cudaMalloc(&d_cnt.p, (size_t)S * 4));
        CK(cudaMalloc(&d_chunks.p, (size_t)NC * sizeof(Chunk)));
        CK(cudaMalloc(&d_left.p, (size_t)NC * 4));
        CK(cudaMalloc(&d_base.p, (size_t)NC * sizeof(uint2)));
        CK(cudaMemcpy(d_cnt.p, counts.data(), (size_t)S * 4, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(d_chunks.p, chunks.data(), (size_t)NC * sizeof(Chunk), cudaMemcpyHostToDevice));
        const uint32_t acc_words = S * kAccWords;
        k_acc_init<<<(acc_words + 255) / 256, 256>>>(d_acc.as<int32_t>(), S);
        k_a_bounds<<<NC, 256>>>(P, d_idx.as<uint32_t>(), d_chunks.as<Chunk>(), d_acc.as<int32_t>());
        k_a_decide<<<(S + 127) / 128, 128>>>(d_acc.as<int32_t>(), d_dec.as<SegDecision>(), d_cnt.as<uint32_t>(), S,
                                             split);
        if (split == PBRT_SPLIT_SAH) {
            k_a_buckets<<<NC, 256>>>(P, d_idx.as<uint32_t>(), d_chunks.as<Chunk>(), d_dec.as<SegDecision>(),
                                     d_acc.as<int32_t>());
            k_a_choose<<<(S + 127) / 128, 128>>>(d_acc.as<int32_t>(), d_dec.as<SegDecision>(), d_cnt.as<uint32_t>(),
                                                 S, mp);
        }
        k_a_count<<<NC, 256>>>(P, d_idx.as<uint32_t>(), d_chunks.as<Chunk>(), d_dec.as<SegDecision>(),
                               d_left.as<uint32_t>());
        CK(cudaGetLastError());
        std::vector<SegDecision> dec(S);
        std::vector<uint32_t> left(NC);
        CK(cudaMemcpy(dec.data(), d_dec.p, (size_t)S * sizeof(SegDecision), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(left.data(), d_left.p, (size_t)NC * 4, cudaMemcpyDeviceToHost));
        // per-range left totals, then each chunk's destinations
        std::vector<uint32_t> total_left(S, 0);
        for (uint32_t c = 0; c < NC; ++c) total_left[chunks[c].seg] += left[c];
        std::vector<uint2> base(NC);
        std::vector<uint32_t> run_l(S, 0), run_r(S, 0);
        for (uint32_t c = 0; c < NC; ++c) {
            const uint32_t s = chunks[c].seg;
            const ANode& a = A[level[s]];
            const bool split_it = dec[s].action != 0;
            const uint32_t mid = split_it ? a.lo + total_left[s] : a.lo + a.cnt;
            base[c] = make_uint2(a.lo + run_l[s], mid + run_r[s]);
            const uint32_t nc = chunks[c].hi - chunks[c].lo;
            const uint32_t nl = split_it ? left[c] : nc;
            run_l[s] += nl;
            run_r[s] += nc - nl;
        }
        CK(cudaMemcpy(d_base.p, base.data(), (size_t)NC * sizeof(uint2), cudaMemcpyHostToDevice));
        k_a_scatter<<<NC, 256>>>(P, d_idx.as<uint32_t>(), d_tmp.as<uint32_t>(), d_chunks.as<Chunk>(),
                                 d_dec.as<SegDecision>(), d_base.as<uint2>());
        k_copy_ranges<<<NC, 256>>>(d_tmp.as<uint32_t>(), d_idx.as<uint32_t>(), d_chunks.as<Chunk>());
        CK(cudaGetLastError());
        std::vector<uint32_t> next;
        for (uint32_t s = 0; s < S; ++s) {
            const uint32_t ai = level[s];
            const SegDecision& d = dec[s];
            A[ai].box = Box{v3(d.lo[0], d.lo[1], d.lo[2]), v3(d.hi[0], d.hi[1], d.hi[2])};
            if (d.action == 0) {
                A[ai].leaf = true;
                continue;
            }
            const uint32_t lo_ = A[ai].lo, cnt = A[ai].cnt, nl = total_left[s];
            if (nl == 0 || nl == cnt) {
                *err = "BVH build: empty partition (the reference asserts at bvh.rs:237-238)";
                return PBRT_ERR_BUILD;
            }
            A[ai].dim = (uint32_t)d.dim;
            const uint32_t depth = A[ai].depth + 1;
            for (int side = 0; side < 2; ++side) {
                ANode c;
                c.lo = side == 0 ? lo_ : lo_ + nl;
                c.cnt = side == 0 ? nl : cnt - nl;
                c.depth = depth;
                const uint32_t ci = (uint32_t)A.size();
                A.push_back(c);
                (side == 0 ? A[ai].left : A[ai].right) = (int32_t)ci;
                if (c.cnt <= kSmall)
                    to_small(ci);
                else
                    next.push_back(ci);
            }
        }
        level.swap(next);
    }

    // ---- phase B: every small range, one thread each
    const uint32_t NJ = (uint32_t)jobs.size();
    uint64_t pool_nodes = 0;
    for (Job& j : jobs) {
        j.node0 = (uint32_t)pool_nodes;
        pool_nodes += 2ull * (j.hi - j.lo) - 1;
    }
    Buf d_jobs, d_outs;
    CK(cudaMalloc(&d_stack.p, n * sizeof(Task)));
    CK(cudaMalloc(&d_pool.p, pool_nodes * sizeof(PoolNode)));
    CK(cudaMalloc(&d_jobs.p, (size_t)NJ * sizeof(Job)));
    CK(cudaMalloc(&d_outs.p, (size_t)NJ * sizeof(JobOut)));
    CK(cudaMemcpy(d_jobs.p, jobs.data(), (size_t)NJ * sizeof(Job), cudaMemcpyHostToDevice));
    k_b_build<<<(NJ + 127) / 128, 128>>>(P, d_idx.as<uint32_t>(), d_tmp.as<uint32_t>(), d_stack.as<Task>(),
                                         d_jobs.as<Job>(), NJ, d_pool.as<PoolNode>(), d_outs.as<JobOut>(), mp, split);
    CK(cudaGetLastError());
    std::vector<JobOut> outs(NJ);
    std::vector<PoolNode> pool(pool_nodes);
    CK(cudaMemcpy(outs.data(), d_outs.p, (size_t)NJ * sizeof(JobOut), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(pool.data(), d_pool.p, pool_nodes * sizeof(PoolNode), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(H.ordered.data(), d_idx.p, n * 4, cudaMemcpyDeviceToHost));
    for (const JobOut& o : outs)
        if (o.err) {
            *err = "BVH build: empty partition (the reference asserts at bvh.rs:237-238)";
            return PBRT_ERR_BUILD;
        }

    // ---- number every node in the reference's depth-first order
    // subtree sizes of phase-A nodes, children first
    std::vector<uint64_t> size(A.size(), 0);
    std::vector<Box> abox(A.size());
    for (size_t i = A.size(); i-- > 0;) {
        const ANode& a = A[i];
        if (a.small) {
            size[i] = outs[a.job].nodes;
            const PoolNode& r = pool[jobs[a.job].node0];
            abox[i] = Box{v3(r.lo[0], r.lo[1], r.lo[2]), v3(r.hi[0], r.hi[1], r.hi[2])};
        } else if (a.leaf) {
            size[i] = 1;
            abox[i] = a.box;
        } else {
            size[i] = 1 + size[a.left] + size[a.right];
            abox[i] = box_union(abox[a.left], abox[a.right]);  // bvh.rs:247
        }
    }
    H.nodes.resize(size[0]);
    struct Item {
        uint32_t a;
        uint64_t at;
    };
    std::vector<Item> todo{{0, 0}};
    while (!todo.empty()) {
        const Item it = todo.back();
        todo.pop_back();
        const ANode& a = A[it.a];
        if (a.small) {
            const Job& J = jobs[a.job];
            const JobOut& o = outs[a.job];
            for (uint32_t k = 0; k < o.nodes; ++k) {
                const PoolNode& p = pool[J.node0 + k];
                FlatNode& f = H.nodes[it.at + k];
                f.box = Box{v3(p.lo[0], p.lo[1], p.lo[2]), v3(p.hi[0], p.hi[1], p.hi[2])};
                f.leaf = (p.b & kLeaf) != 0;
                f.offset = f.leaf ? p.a : (uint32_t)(it.at + p.a);
                f.count = f.leaf ? (p.b & ~kLeaf) : p.b;
            }
            H.depth = std::max(H.depth, a.depth + o.depth - 1);
            continue;
        }
        FlatNode& f = H.nodes[it.at];
        f.box = abox[it.a];
        H.depth = std::max(H.depth, a.depth);
        if (a.leaf) {
            f.leaf = true;
            f.offset = a.lo;
            f.count = a.cnt;
            continue;
        }
        f.leaf = false;
        f.count = a.dim;
        const uint64_t right_at = it.at + 1 + size[a.left];
        f.offset = (uint32_t)right_at;
        todo.push_back(Item{(uint32_t)a.right, right_at});
        todo.push_back(Item{(uint32_t)a.left, it.at + 1});
    }
    return PBRT_OK;
}

}  // namespace pbrt
