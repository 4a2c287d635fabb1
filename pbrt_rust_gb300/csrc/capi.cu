// capi.cu - the C ABI declared in include/pbrt_gpu.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/pbrt_gpu.h"
#include "capi_internal.h"
#include "host_scene.h"
#include "kernels.h"

using namespace pbrt;

namespace pbrt {

static thread_local std::string g_last_error;

int set_error(int status, const std::string& msg) {
    g_last_error = msg;
    return status;
}

int cuda_status(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return PBRT_OK;
    int st = (e == cudaErrorMemoryAllocation) ? PBRT_ERR_OUT_OF_MEMORY
             : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) ? PBRT_ERR_NO_DEVICE
                                                                              : PBRT_ERR_CUDA;
    return set_error(st, std::string(what) + ": " + cudaGetErrorString(e));
}

int DeviceBuf::reserve(size_t bytes) {
    if (cap >= bytes) return PBRT_OK;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t want = bytes < 256 ? 256 : bytes;
    int st = cuda_status(cudaMalloc(&p, want), "cudaMalloc");
    if (st) return st;
    cap = want;
    return PBRT_OK;
}
void DeviceBuf::release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
}

bool cuda_device_present() {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return n > 0;
}

bool is_device_pointer(const void* ptr) {
    if (!ptr) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

DeviceGuard::DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) {
        cudaGetLastError();
        prev = -1;
    }
    if (prev != dev) cudaSetDevice(dev);
}
DeviceGuard::~DeviceGuard() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
}

template <class T>
static int upload(T** dst, const std::vector<T>& src) {
    *dst = nullptr;
    if (src.empty()) return PBRT_OK;
    int st = cuda_status(cudaMalloc((void**)dst, src.size() * sizeof(T)), "cudaMalloc");
    if (st) return st;
    return cuda_status(cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice), "cudaMemcpy");
}

int bvh_upload(PbrtBVH* b) {
    std::lock_guard<std::mutex> lk(b->upload_mu);
    if (b->uploaded) return PBRT_OK;
    int st;
    if ((st = cuda_status(cudaGetDevice(&b->device), "cudaGetDevice"))) return st;
    if ((st = upload(&b->d_pairs, b->host.pairs))) return st;
    if ((st = upload(&b->d_prims, b->host.recs))) return st;
    if ((st = upload(&b->d_spheres, b->host.spheres))) return st;
    if ((st = upload(&b->d_nodes4, b->host.nodes4))) return st;
    if ((st = cuda_status(cudaMalloc(&b->d_status, sizeof(int)), "cudaMalloc"))) return st;
    if ((st = cuda_status(cudaMemset(b->d_status, 0, sizeof(int)), "cudaMemset"))) return st;
    // instance definitions: 4-wide layout, walked by instance_test
    std::vector<DevBVH4> defs;
    for (const HostBVH& I : b->host.insts) {
        Node4* nodes = nullptr;
        PrimRec* prims = nullptr;
        SphereRec* spheres = nullptr;
        st = upload(&nodes, I.nodes4);
        if (nodes) b->d_inst_bufs.push_back(nodes);
        if (!st) st = upload(&prims, I.recs);
        if (prims) b->d_inst_bufs.push_back(prims);
        if (!st) st = upload(&spheres, I.spheres);
        if (spheres) b->d_inst_bufs.push_back(spheres);
        if (st) return st;
        DevBVH4 d{};
        d.nodes = nodes;
        d.prims = prims;
        d.spheres = spheres;
        d.root = I.root4;
        d.empty = I.nodes.empty() ? 1u : 0u;
        d.insts = nullptr;
        defs.push_back(d);
    }
    b->inst_dev = defs;
    if ((st = upload(&b->d_insts, defs))) return st;
    b->dev.insts = b->d_insts;
    b->dev4.insts = b->d_insts;
    b->dev.pairs = b->d_pairs;
    b->dev.prims = b->d_prims;
    b->dev.spheres = b->d_spheres;
    b->dev.root = b->host.root;
    b->dev.has_spheres = b->host.has_spheres ? 1u : 0u;
    b->dev.n_prims = (uint32_t)b->host.recs.size();
    b->dev.empty = b->host.nodes.empty() ? 1u : 0u;
    b->dev4.nodes = b->d_nodes4;
    b->dev4.prims = b->d_prims;
    b->dev4.spheres = b->d_spheres;
    b->dev4.root = b->host.root4;
    b->dev4.empty = b->dev.empty;
    b->uploaded = true;
    return PBRT_OK;
}

// The 4-wide layout when a compiled variant covers its stack bound.
const DevBVH4* wide_of(const PbrtBVH* b) {
    return wide_stack_variant(b->host.stack4_bound) ? &b->dev4 : nullptr;
}

// Stream-ordered scratch for per-call temporaries (the ray permutation):
// one pool per device owned by the library, which keeps freed memory for the
// next call instead of returning it to the driver at every synchronisation.
static std::mutex g_pool_mu;
static cudaMemPool_t g_pools[16];

static int scratch_pool(int dev, cudaMemPool_t* out) {
    if (dev < 0 || dev >= 16) return set_error(PBRT_ERR_UNSUPPORTED, "device index above 15");
    std::lock_guard<std::mutex> lk(g_pool_mu);
    if (!g_pools[dev]) {
        cudaMemPoolProps props;
        std::memset(&props, 0, sizeof(props));
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t pool;
        int st = cuda_status(cudaMemPoolCreate(&pool, &props), "cudaMemPoolCreate");
        if (st) return st;
        uint64_t keep = ~0ull;
        if ((st = cuda_status(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep),
                              "cudaMemPoolSetAttribute"))) {
            cudaMemPoolDestroy(pool);
            return st;
        }
        g_pools[dev] = pool;
    }
    *out = g_pools[dev];
    return PBRT_OK;
}

// Traces device-resident rays, first binning a large batch by direction and
// origin when the configuration asks for it (reorder.cu); the permutation
// lives in stream-ordered scratch released on the same stream.
static int launch_batch(PbrtBVH* b, const PbrtRay* d_rays, uint32_t n, PbrtHit* d_hits, uint8_t* d_occ,
                        cudaStream_t s, StreamIn in = {}, PbrtHit* host_hits = nullptr) {
    const uint32_t* order = nullptr;
    uint32_t* work = nullptr;
    void* scratch = nullptr;
    int st;
    const bool reorder = !in.ready && !host_hits && trace_reorder() && n >= kReorderMinRays && !b->host.nodes.empty();
    const bool chunked = in.ready || host_hits || trace_chunk() != 0;
    // [256 B: chunk counter, replay flag][permutation scratch]
    cudaMemPool_t pool = nullptr;
    if ((st = scratch_pool(b->device, &pool))) return st;
    const size_t bytes = 256 + (reorder ? ray_order_scratch_bytes(n) : 0);
    if ((st = cuda_status(cudaMallocFromPoolAsync(&scratch, bytes, pool, s), "cudaMallocFromPoolAsync"))) return st;
    work = static_cast<uint32_t*>(scratch);
    uint32_t* replay = work + 1;
    if ((st = cuda_status(cudaMemsetAsync(work, 0, 2 * sizeof(uint32_t), s), "cudaMemsetAsync"))) {
        cudaFreeAsync(scratch, s);
        return st;
    }
    if (!chunked) work = nullptr;
    if (reorder) {
        const Box& wb = b->host.nodes[0].box;
        ReorderBounds B;
        const float lo[3] = {wb.lo.x, wb.lo.y, wb.lo.z}, hi[3] = {wb.hi.x, wb.hi.y, wb.hi.z};
        const float cells[3] = {8.0f, 4.0f, 4.0f};
        for (int k = 0; k < 3; ++k) {
            float ext = hi[k] - lo[k];
            B.lo[k] = std::isfinite(lo[k]) ? lo[k] : 0.0f;
            B.scale[k] = (ext > 0.0f && std::isfinite(ext)) ? cells[k] / ext : 0.0f;
        }
        uint32_t* ord = nullptr;
        if ((st = cuda_status(build_ray_order(d_rays, n, B, static_cast<unsigned char*>(scratch) + 256, &ord, s),
                              "ray reorder"))) {
            cudaFreeAsync(scratch, s);
            return st;
        }
        order = ord;
    }
    st = cuda_status(launch_trace(b->dev, b->host.depth, d_rays, n, d_hits, d_occ, b->d_status, s, wide_of(b),
                                  b->host.stack4_bound, -1, order, work, replay, in, host_hits),
                     "trace launch");
    cudaFreeAsync(scratch, s);
    return st;
}

// Pinned host memory is mapped into the device's address space (on GB300
// it is the Grace memory behind NVLink-C2C).  With PBRT_HOST_MAPPED=1 (read
// at every call) the traversal reads the rays and writes the results there
// directly, with no staging copies; by default pinned buffers take the
// streamed form (trace_streamed) and other host buffers the copy pipeline
// below.  Measured with 2^22 heightfield rays in pinned buffers on GB300
// boxes: in place 1.57-1.99 ms per call depending on the box (its scattered
// 16-byte stores run at 37 GB/s across the link on some boxes), the copy
// pipeline 1.68-1.76 ms, the streamed form 1.48 ms.  Identical results.
static bool host_mapped_enabled() {
    const char* v = getenv("PBRT_HOST_MAPPED");
    return v && v[0] == '1';
}
// The device address of a pinned, mapped host allocation, else nullptr.
static void* mapped_host_pointer(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// Other host-buffer calls of at least 2 * kPipeChunkMin rays run in
// pipe_chunks() chunks (PBRT_PIPE_CHUNKS: 1 = one piece, at most
// kPipeChunks; default 4) whose copies overlap the other chunks' traversal;
// consecutive chunks trace on two streams so that one kernel's tail overlaps
// the next one's start.  Measured on GB300 with 2^22 heightfield rays and
// pinned buffers: 2.32 ms in one piece; 1.84 / 1.76 / 1.77 ms in 3 / 4 / 6
// chunks (one compute stream: 1.82 / 1.87 / 2.04 ms).
constexpr uint32_t kPipeChunkMin = 1u << 18;
constexpr uint32_t kPipeChunks = 8;
constexpr uint32_t kStreamPieces = 16;  // streamed input (trace_streamed): pieces per call at most
static uint32_t pipe_chunks() {
    static const uint32_t k = [] {
        const char* v = getenv("PBRT_PIPE_CHUNKS");
        const int x = v ? atoi(v) : 4;
        return (uint32_t)(x < 1 ? 1 : (x > (int)kPipeChunks ? (int)kPipeChunks : x));
    }();
    return k;
}

// The handle's device-side status after a finished call (cleared when set).
static int device_status(PbrtBVH* b) {
    int dev_status = 0, st;
    if ((st = cuda_status(cudaMemcpy(&dev_status, b->d_status, sizeof(int), cudaMemcpyDeviceToHost), "status")))
        return st;
    if (dev_status) {
        cudaMemset(b->d_status, 0, sizeof(int));
        return set_error(dev_status, dev_status == PBRT_ERR_TIMEOUT ? "streamed rays did not arrive in time"
                                                                     : "device-side traversal failure");
    }
    return PBRT_OK;
}

// The handle's copy streams and events (created on first use; the caller
// holds stage_mu).
static int pipe_streams(PbrtBVH* b) {
    if (b->pipe_in) return PBRT_OK;
    int st;
    if ((st = cuda_status(cudaStreamCreateWithFlags(&b->pipe_in, cudaStreamNonBlocking), "cudaStreamCreate")) ||
        (st = cuda_status(cudaStreamCreateWithFlags(&b->pipe_out, cudaStreamNonBlocking), "cudaStreamCreate")) ||
        (st = cuda_status(cudaStreamCreateWithFlags(&b->pipe_k, cudaStreamNonBlocking), "cudaStreamCreate")))
        return st;
    for (cudaEvent_t& e : b->pipe_ev)
        if ((st = cuda_status(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate"))) return st;
    if ((st = cuda_status(cudaMalloc(&b->d_ready, kStreamPieces * sizeof(uint32_t)), "cudaMalloc")) ||
        (st = cuda_status(cudaHostAlloc(&b->h_one, sizeof(uint32_t), cudaHostAllocDefault), "cudaHostAlloc")))
        return st;
    *b->h_one = 1u;
    return PBRT_OK;
}

// Streamed host input.  Rays in pinned host memory, results in device
// memory or (closest hits) in pinned host memory mapped into the device's
// address space: the rays go in pieces of 2^shift rays (at most
// kStreamPieces, at least 2^kStreamShiftMin rays each) on the copy stream,
// each piece's copy followed by a 4-byte copy that sets the piece's flag,
// and the traversal is launched behind them on the caller's stream without
// waiting for them.  The kernel's warps take rays in order and wait
// (bounded) for the piece they need, so the traversal starts after the
// first piece instead of after every copy, and one launch replaces the
// copy pipeline's per-chunk launches.  Closest hits for host memory are
// staged on the device and written out by the walk itself, each chunk of
// rays in coalesced rows once its last ray is done (HOSTOUT in trace.cu);
// any-hit answers for host memory go through the staging buffer and one
// copy of n bytes.  PBRT_STREAM_IN=0 (read at every call) takes the copy
// pipeline instead.  Measured on GB300 with 2^22 heightfield rays (the walk
// alone: 1.30 ms): closest hits 1.48 ms per call (pipeline 1.68 ms), any hit
// 1.22 ms (1.40 ms); with device outputs 1.39 ms.  Over the pipeline's
// per-piece launches it saves the tails each launch leaves (a 2^22-ray pass
// in four launches spent 1.50 ms in kernels against 1.30 ms in one).
constexpr uint32_t kStreamShiftMin = 16;
static bool stream_in_enabled() {
    const char* v = getenv("PBRT_STREAM_IN");
    return !(v && v[0] == '0');
}
// The caller holds stage_mu.  `hits`: the closest hits' destination, device
// memory (`out_dev`) or mapped pinned host memory; `occ`: the any-hit
// destination, device memory (`out_dev`) or any host memory.
static int trace_streamed(PbrtBVH* b, const PbrtRay* rays, uint32_t n, PbrtHit* hits, uint8_t* occ, bool out_dev,
                          cudaStream_t s) {
    int st;
    if ((st = pipe_streams(b)) || (st = b->stage_in.reserve((size_t)n * sizeof(PbrtRay)))) return st;
    uint8_t* d_occ = occ;
    PbrtHit* d_hits = hits;
    PbrtHit* host_hits = nullptr;
    if (!out_dev) {
        if ((st = b->stage_out.reserve(hits ? (size_t)n * sizeof(PbrtHit) : (size_t)n))) return st;
        if (hits) {
            host_hits = hits;
            d_hits = static_cast<PbrtHit*>(b->stage_out.p);
        } else {
            d_occ = static_cast<uint8_t*>(b->stage_out.p);
        }
    }
    uint32_t shift = kStreamShiftMin;
    while (((uint64_t)kStreamPieces << shift) < n) ++shift;
    const uint32_t pieces = (uint32_t)(((uint64_t)n + (1ull << shift) - 1) >> shift);
    PbrtRay* d_rays = static_cast<PbrtRay*>(b->stage_in.p);
    // the flags are cleared before the copy stream may set them
    if ((st = cuda_status(cudaMemsetAsync(b->d_ready, 0, kStreamPieces * sizeof(uint32_t), s), "cudaMemsetAsync")) ||
        (st = cuda_status(cudaEventRecord(b->pipe_ev[0], s), "cudaEventRecord")) ||
        (st = cuda_status(cudaStreamWaitEvent(b->pipe_in, b->pipe_ev[0], 0), "cudaStreamWaitEvent")))
        return st;
    // A warp waits for a piece at most 50 ms + 2 ns per ray of the call
    // (the copies move a ray in 0.15 ns); a walk that runs out (the copies
    // did not run beside it) is redone below over the rays then staged.
    const uint32_t wait_ms = 50u + (uint32_t)((2ull * n) / 1000000ull);
    // The copies are queued before the launch (32 calls, a few microseconds
    // of host time, while the first piece is already moving), so a walk that
    // a profiler runs only after earlier work finds every piece landed.
    // PBRT_TEST_HOLD_STREAM_COPIES=1 (tests) queues them only after the walk
    // has given up instead, which exercises the redo.
    const char* hold_env = getenv("PBRT_TEST_HOLD_STREAM_COPIES");
    const bool hold = hold_env && hold_env[0] == '1';
    const uint32_t pre = hold ? 0u : pieces;
    int copy_st = PBRT_OK;
    auto enqueue = [&](uint32_t k) {
        const uint64_t lo = (uint64_t)k << shift;
        const uint64_t cnt = std::min<uint64_t>((uint64_t)n - lo, 1ull << shift);
        copy_st = cuda_status(cudaMemcpyAsync(d_rays + lo, rays + lo, cnt * sizeof(PbrtRay), cudaMemcpyHostToDevice,
                                              b->pipe_in),
                              "cudaMemcpyAsync H2D");
        if (!copy_st)
            copy_st = cuda_status(cudaMemcpyAsync(b->d_ready + k, b->h_one, sizeof(uint32_t), cudaMemcpyHostToDevice,
                                                  b->pipe_in),
                                  "cudaMemcpyAsync H2D");
    };
    for (uint32_t k = 0; k < pre && !copy_st; ++k) enqueue(k);
    const int launch_st =
        copy_st ? PBRT_OK : launch_batch(b, d_rays, n, d_hits, d_occ, s, StreamIn{b->d_ready, shift, wait_ms}, host_hits);
    if (hold) cudaStreamSynchronize(s);
    // the held copies are queued whatever the launch did: a walk that did
    // start waits for them
    for (uint32_t k = pre; k < pieces && !copy_st; ++k) enqueue(k);
    auto copy_back = [&]() {  // any-hit answers staged for host memory
        return occ && d_occ != occ
                   ? cuda_status(cudaMemcpyAsync(occ, d_occ, n, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync D2H")
                   : PBRT_OK;
    };
    if (!launch_st && !copy_st) copy_st = copy_back();
    // a walk whose pieces never come ends by itself (PBRT_ERR_TIMEOUT)
    const int sync_st = cuda_status(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    const int sync_in = cuda_status(cudaStreamSynchronize(b->pipe_in), "cudaStreamSynchronize");
    if (launch_st || copy_st) {
        const int first = launch_st ? launch_st : copy_st;
        device_status(b);  // clears a timeout the failed copies caused
        return first;
    }
    if (sync_st || sync_in) return sync_st ? sync_st : sync_in;
    int dev_status = 0;
    if ((st = cuda_status(cudaMemcpy(&dev_status, b->d_status, sizeof(int), cudaMemcpyDeviceToHost), "status")))
        return st;
    if (dev_status == PBRT_ERR_TIMEOUT) {
        // the walk gave up on pieces that had not landed; every copy has
        // finished now, so the staged rays are traced again in full
        cudaMemset(b->d_status, 0, sizeof(int));
        if ((st = launch_batch(b, d_rays, n, d_hits, d_occ, s, StreamIn{}, host_hits)) || (st = copy_back()) ||
            (st = cuda_status(cudaStreamSynchronize(s), "cudaStreamSynchronize")))
            return st;
        return device_status(b);
    }
    if (dev_status) {
        cudaMemset(b->d_status, 0, sizeof(int));
        return set_error(dev_status, "device-side traversal failure");
    }
    return PBRT_OK;
}

// Runs closest/any hit for host or device buffers.
static int trace_call(const PbrtBVH* cb, const PbrtRay* rays, uint32_t n, PbrtHit* hits, uint8_t* occ,
                      void* stream_v) {
    PbrtBVH* b = const_cast<PbrtBVH*>(cb);
    if (!b) return set_error(PBRT_ERR_INVALID_ARGUMENT, "bvh is NULL");
    if (n == 0) return PBRT_OK;
    if (!rays || (!hits && !occ)) return set_error(PBRT_ERR_INVALID_ARGUMENT, "rays/output is NULL");
    int st;
    if (!b->uploaded && (st = bvh_upload(b))) return st;
    DeviceGuard g(b->device);
    cudaStream_t s = (cudaStream_t)stream_v;
    void* out = hits ? (void*)hits : (void*)occ;
    size_t out_bytes = hits ? (size_t)n * sizeof(PbrtHit) : (size_t)n;
    bool dr = is_device_pointer(rays), dout = is_device_pointer(out);
    if (dr && dout) return launch_batch(b, rays, n, hits, occ, s);
    if (dr && hits && stream_in_enabled() && !host_mapped_enabled() && n >= (2u << kStreamShiftMin) &&
        trace_streams(b->dev, wide_of(b), b->host.stack4_bound, n)) {
        // device rays, closest hits for mapped pinned host memory: the walk
        // writes them out chunk by chunk from a staging array
        if (PbrtHit* mh = static_cast<PbrtHit*>(mapped_host_pointer(hits))) {
            std::lock_guard<std::mutex> lk(b->stage_mu);
            if ((st = b->stage_out.reserve((size_t)n * sizeof(PbrtHit))) ||
                (st = launch_batch(b, rays, n, static_cast<PbrtHit*>(b->stage_out.p), nullptr, s, StreamIn{}, mh)) ||
                (st = cuda_status(cudaStreamSynchronize(s), "cudaStreamSynchronize")))
                return st;
            return device_status(b);
        }
    }
    if (host_mapped_enabled()) {
        const void* mr = dr ? (const void*)rays : mapped_host_pointer(rays);
        void* mo = dout ? out : mapped_host_pointer(out);
        if (mr && mo) {
            if ((st = launch_batch(b, static_cast<const PbrtRay*>(mr), n, hits ? static_cast<PbrtHit*>(mo) : nullptr,
                                   hits ? nullptr : static_cast<uint8_t*>(mo), s)))
                return st;
            return cuda_status(cudaStreamSynchronize(s), "cudaStreamSynchronize");
        }
    }
    std::lock_guard<std::mutex> lk(b->stage_mu);
    if (!dr && n >= (2u << kStreamShiftMin) && stream_in_enabled() && mapped_host_pointer(rays) &&
        trace_streams(b->dev, wide_of(b), b->host.stack4_bound, n)) {
        PbrtHit* d_hits = hits && !dout ? static_cast<PbrtHit*>(mapped_host_pointer(hits)) : hits;
        if (!hits || d_hits) {
            return trace_streamed(b, rays, n, d_hits, occ, dout, s);
        }
    }
    const PbrtRay* d_rays = rays;
    if (!dr) {
        if ((st = b->stage_in.reserve((size_t)n * sizeof(PbrtRay)))) return st;
        d_rays = (const PbrtRay*)b->stage_in.p;
    }
    void* d_out = out;
    if (!dout) {
        if ((st = b->stage_out.reserve(out_bytes))) return st;
        d_out = b->stage_out.p;
    }
    const size_t out_unit = hits ? sizeof(PbrtHit) : 1;
    if (n >= 2 * kPipeChunkMin && pipe_chunks() > 1) {
        // Pipelined: chunk c's copy in (stream pipe_in), traversal (the
        // caller's stream for even c, pipe_k for odd c) and copy out
        // (pipe_out) overlap with the other chunks' - the copies hide
        // behind the kernels.
        if ((st = pipe_streams(b))) return st;
        // the first and last chunks are half the others: the copy before
        // the first traversal and the one after the last are what no
        // kernel hides
        const uint32_t chunks = std::min<uint32_t>(pipe_chunks(), n / kPipeChunkMin);
        const uint64_t weight = chunks > 2 ? 2ull * (chunks - 1) : chunks;
        auto bound = [&](uint32_t c) -> uint32_t {  // first ray of chunk c
            if (c == 0) return 0;
            if (c >= chunks) return n;
            const uint64_t w = chunks > 2 ? 1ull + 2ull * (c - 1) : c;
            return (uint32_t)((uint64_t)n * w / weight);
        };
        cudaEvent_t* ev = b->pipe_ev;
        if ((st = cuda_status(cudaEventRecord(ev[0], s), "cudaEventRecord")) ||
            (st = cuda_status(cudaStreamWaitEvent(b->pipe_in, ev[0], 0), "cudaStreamWaitEvent")))
            return st;
        for (uint32_t c = 0; c < chunks; ++c) {
            const uint32_t lo = bound(c), cnt = bound(c + 1) - lo;
            if (cnt == 0) continue;
            cudaEvent_t in_done = ev[1 + 2 * c], traced = ev[2 + 2 * c];
            if (!dr) {
                if ((st = cuda_status(cudaMemcpyAsync((PbrtRay*)b->stage_in.p + lo, rays + lo, (size_t)cnt * sizeof(PbrtRay),
                                                      cudaMemcpyHostToDevice, b->pipe_in),
                                      "cudaMemcpyAsync H2D")))
                    return st;
            }
            cudaStream_t ks = (c & 1) ? b->pipe_k : s;  // alternate compute streams: kernel tails overlap
            if ((st = cuda_status(cudaEventRecord(in_done, b->pipe_in), "cudaEventRecord")) ||
                (st = cuda_status(cudaStreamWaitEvent(ks, in_done, 0), "cudaStreamWaitEvent")))
                return st;
            uint8_t* o = static_cast<uint8_t*>(d_out) + (size_t)lo * out_unit;
            if ((st = launch_batch(b, d_rays + lo, cnt, hits ? (PbrtHit*)o : nullptr, hits ? nullptr : o, ks)))
                return st;
            if ((st = cuda_status(cudaEventRecord(traced, ks), "cudaEventRecord")) ||
                (st = cuda_status(cudaStreamWaitEvent(b->pipe_out, traced, 0), "cudaStreamWaitEvent")))
                return st;
            if (!dout && (st = cuda_status(cudaMemcpyAsync(static_cast<uint8_t*>(out) + (size_t)lo * out_unit, o,
                                                          (size_t)cnt * out_unit, cudaMemcpyDeviceToHost, b->pipe_out),
                                          "cudaMemcpyAsync D2H")))
                return st;
        }
        if ((st = cuda_status(cudaStreamSynchronize(b->pipe_out), "cudaStreamSynchronize")) ||
            (st = cuda_status(cudaStreamSynchronize(b->pipe_k), "cudaStreamSynchronize")) ||
            (st = cuda_status(cudaStreamSynchronize(s), "cudaStreamSynchronize")))
            return st;
    } else {
        if (!dr && (st = cuda_status(cudaMemcpyAsync(b->stage_in.p, rays, (size_t)n * sizeof(PbrtRay),
                                                     cudaMemcpyHostToDevice, s),
                                     "cudaMemcpyAsync H2D")))
            return st;
        if ((st = launch_batch(b, d_rays, n, hits ? (PbrtHit*)d_out : nullptr, hits ? nullptr : (uint8_t*)d_out, s)))
            return st;
        if (!dout && (st = cuda_status(cudaMemcpyAsync(out, d_out, out_bytes, cudaMemcpyDeviceToHost, s),
                                       "cudaMemcpyAsync D2H")))
            return st;
        if ((st = cuda_status(cudaStreamSynchronize(s), "cudaStreamSynchronize"))) return st;
    }
    return device_status(b);
}

}  // namespace pbrt

PbrtBVH::~PbrtBVH() {
    for (cudaEvent_t e : pipe_ev)
        if (e) cudaEventDestroy(e);
    if (pipe_in) cudaStreamDestroy(pipe_in);
    if (pipe_out) cudaStreamDestroy(pipe_out);
    if (pipe_k) cudaStreamDestroy(pipe_k);
    if (d_ready) cudaFree(d_ready);
    if (h_one) cudaFreeHost(h_one);
    for (void* p : d_inst_bufs) cudaFree(p);
    if (d_insts) cudaFree(d_insts);
    if (d_pairs) cudaFree(d_pairs);
    if (d_prims) cudaFree(d_prims);
    if (d_spheres) cudaFree(d_spheres);
    if (d_nodes4) cudaFree(d_nodes4);
    if (d_status) cudaFree(d_status);
    stage_in.release();
    stage_out.release();
}

extern "C" {

int pbrtgpu_abi_version(void) { return PBRT_GPU_ABI_VERSION; }

const char* pbrtgpu_status_str(int s) {
    switch (s) {
        case PBRT_OK: return "ok";
        case PBRT_ERR_INVALID_ARGUMENT: return "invalid argument";
        case PBRT_ERR_CUDA: return "CUDA error";
        case PBRT_ERR_OUT_OF_MEMORY: return "out of device memory";
        case PBRT_ERR_UNSUPPORTED: return "unsupported";
        case PBRT_ERR_BUILD: return "BVH build failed";
        case PBRT_ERR_STACK_OVERFLOW: return "traversal stack overflow";
        case PBRT_ERR_BUDGET: return "device-memory budget exceeded";
        case PBRT_ERR_TIMEOUT: return "device wait timed out";
        case PBRT_ERR_NAN: return "NaN radiance";
        case PBRT_ERR_NO_DEVICE: return "no CUDA device";
        case PBRT_ERR_CANCELLED: return "cancelled";
        default: return "unknown status";
    }
}

const char* pbrtgpu_last_error(void) { return pbrt::g_last_error.c_str(); }

int pbrtgpu_bvh_create(const PbrtShapeDesc* shapes, uint32_t n_shapes, uint32_t max_prims, const char* split_method,
                       PbrtBVH** out) {
    return pbrtgpu_bvh_create_ex(shapes, n_shapes, max_prims, split_method, 0, out);
}

static int bvh_create(const PbrtShapeDesc* shapes, uint32_t n_shapes, const PbrtInstanceDesc* defs, uint32_t n_defs,
                      uint32_t max_prims, const char* split_method, uint32_t flags, PbrtBVH** out) {
    if (!out || (!shapes && n_shapes) || (!defs && n_defs)) return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = nullptr;
    for (uint32_t k = 0; k < n_defs; ++k)
        if (!defs[k].shapes && defs[k].n_shapes) return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (flags & ~(uint32_t)PBRT_BUILD_ON_DEVICE) return set_error(PBRT_ERR_INVALID_ARGUMENT, "unknown build flags");
    const bool on_device = (flags & PBRT_BUILD_ON_DEVICE) != 0;
    if (on_device && !cuda_device_present()) return set_error(PBRT_ERR_NO_DEVICE, "no CUDA device for the build");
    PbrtBVH* b = new PbrtBVH();
    std::string err;
    int st = build_host_bvh(shapes, n_shapes, max_prims, split_method, &b->host, &err, on_device, defs, n_defs);
    if (st) {
        delete b;
        return set_error(st, err);
    }
    if (trace_stack_for_depth(b->host.depth) == 0) {
        std::string msg = "BVH depth " + std::to_string(b->host.depth) + " exceeds the deepest traversal stack (256)";
        delete b;
        return set_error(PBRT_ERR_STACK_OVERFLOW, msg);
    }
    // Resident from creation when a device is present, so allocation
    // failures surface here and the first query pays no upload.
    if (cuda_device_present() && (st = bvh_upload(b))) {
        delete b;
        return st;
    }
    *out = b;
    return PBRT_OK;
}

int pbrtgpu_bvh_create_ex(const PbrtShapeDesc* shapes, uint32_t n_shapes, uint32_t max_prims,
                          const char* split_method, uint32_t flags, PbrtBVH** out) {
    return bvh_create(shapes, n_shapes, nullptr, 0, max_prims, split_method, flags, out);
}

int pbrtgpu_bvh_create_desc(const PbrtSceneDesc* d, PbrtBVH** out) {
    if (!d) return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
    const char* names[3] = {"sah", "middle", "equal"};
    const char* sm = (d->split_method >= 0 && d->split_method < 3) ? names[d->split_method] : "sah";
    return bvh_create(d->shapes, d->n_shapes, d->instances, d->n_instances, d->max_prims_in_node, sm, d->build_flags,
                      out);
}

void pbrtgpu_bvh_destroy(PbrtBVH* b) {
    if (!b) return;
    DeviceGuard g(b->device);
    delete b;
}

int pbrtgpu_bvh_world_bound(const PbrtBVH* b, float lo[3], float hi[3]) {
    if (!b || !lo || !hi) return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
    Box bx = b->host.nodes.empty() ? box_empty() : b->host.nodes[0].box;  // bvh.rs:365-373
    lo[0] = bx.lo.x;
    lo[1] = bx.lo.y;
    lo[2] = bx.lo.z;
    hi[0] = bx.hi.x;
    hi[1] = bx.hi.y;
    hi[2] = bx.hi.z;
    return PBRT_OK;
}

int pbrtgpu_bvh_num_primitives(const PbrtBVH* b, uint32_t* n) {
    if (!b || !n) return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
    *n = (uint32_t)b->host.prims.size();
    return PBRT_OK;
}
int pbrtgpu_bvh_device_bytes(const PbrtBVH* b, uint64_t* bytes) {
    if (!b || !bytes) return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
    const HostBVH& H = b->host;
    uint64_t n = H.pairs.size() * sizeof(NodePair) + H.recs.size() * sizeof(PrimRec) +
                 H.spheres.size() * sizeof(SphereRec) + H.nodes4.size() * sizeof(Node4) + sizeof(int);
    for (const HostBVH& I : H.insts)
        n += I.nodes4.size() * sizeof(Node4) + I.recs.size() * sizeof(PrimRec) + I.spheres.size() * sizeof(SphereRec);
    n += H.insts.size() * sizeof(DevBVH4);
    *bytes = n;
    return PBRT_OK;
}
int pbrtgpu_bvh_num_nodes(const PbrtBVH* b, uint32_t* n) {
    if (!b || !n) return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
    *n = (uint32_t)b->host.nodes.size();
    return PBRT_OK;
}
int pbrtgpu_bvh_depth(const PbrtBVH* b, uint32_t* d) {
    if (!b || !d) return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
    *d = b->host.depth;
    return PBRT_OK;
}
int pbrtgpu_bvh_get_nodes(const PbrtBVH* b, PbrtPackedNode* out, uint32_t cap) {
    if (!b || (!out && !b->host.nodes.empty())) return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (cap < b->host.nodes.size()) return set_error(PBRT_ERR_INVALID_ARGUMENT, "capacity too small");
    for (size_t i = 0; i < b->host.nodes.size(); ++i) {
        const FlatNode& n = b->host.nodes[i];
        PbrtPackedNode& o = out[i];
        o.lo[0] = n.box.lo.x;
        o.lo[1] = n.box.lo.y;
        o.lo[2] = n.box.lo.z;
        o.hi[0] = n.box.hi.x;
        o.hi[1] = n.box.hi.y;
        o.hi[2] = n.box.hi.z;
        o.is_leaf = n.leaf ? 1 : 0;
        o.offset = n.offset;
        o.count = n.count;
    }
    return PBRT_OK;
}
int pbrtgpu_bvh_get_primitive_order(const PbrtBVH* b, uint32_t* out, uint32_t cap) {
    if (!b || (!out && !b->host.ordered.empty())) return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (cap < b->host.ordered.size()) return set_error(PBRT_ERR_INVALID_ARGUMENT, "capacity too small");
    if (!b->host.ordered.empty()) std::memcpy(out, b->host.ordered.data(), b->host.ordered.size() * sizeof(uint32_t));
    return PBRT_OK;
}

int pbrtgpu_set_trace_config(const PbrtTraceConfig* cfg) {
    if (!cfg || set_trace_config(*cfg))
        return set_error(PBRT_ERR_INVALID_ARGUMENT,
                         "trace config: kernel 0..4, refill 1..32, min_blocks 0/7/8/9, render_kernel 0..4, "
                         "reorder 0/1");
    return PBRT_OK;
}

int pbrtgpu_get_trace_config(PbrtTraceConfig* cfg) {
    if (!cfg) return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
    get_trace_config(cfg);
    return PBRT_OK;
}

int pbrtgpu_intersect(const PbrtBVH* b, const PbrtRay* rays, uint32_t n, PbrtHit* hits, void* stream) {
    if (!hits && n) return set_error(PBRT_ERR_INVALID_ARGUMENT, "hits is NULL");
    return trace_call(b, rays, n, hits, nullptr, stream);
}

int pbrtgpu_intersect_p(const PbrtBVH* b, const PbrtRay* rays, uint32_t n, uint8_t* occluded, void* stream) {
    if (!occluded && n) return set_error(PBRT_ERR_INVALID_ARGUMENT, "occluded is NULL");
    return trace_call(b, rays, n, nullptr, occluded, stream);
}

int pbrtgpu_intersect_streamed(const PbrtBVH* cb, const PbrtRay* rays, uint32_t n, PbrtHit* hits, uint8_t* occluded,
                               const uint32_t* ready, uint32_t piece_shift, void* stream) {
    using namespace pbrt;
    PbrtBVH* b = const_cast<PbrtBVH*>(cb);
    if (!b) return set_error(PBRT_ERR_INVALID_ARGUMENT, "bvh is NULL");
    if (n == 0) return PBRT_OK;
    if (!rays || !ready || (!hits) == (!occluded))
        return set_error(PBRT_ERR_INVALID_ARGUMENT, "rays/ready NULL or not exactly one of hits/occluded");
    if (piece_shift < 5 || piece_shift > 31) return set_error(PBRT_ERR_INVALID_ARGUMENT, "piece_shift not in [5, 31]");
    void* out = hits ? (void*)hits : (void*)occluded;
    if (!is_device_pointer(rays) || !is_device_pointer(out) || !is_device_pointer(ready))
        return set_error(PBRT_ERR_INVALID_ARGUMENT, "rays, results and flags must be device memory");
    int st;
    if (!b->uploaded && (st = bvh_upload(b))) return st;
    DeviceGuard g(b->device);
    if (!trace_streams(b->dev, wide_of(b), b->host.stack4_bound, n))
        return set_error(PBRT_ERR_UNSUPPORTED, "streamed rays need the 4-wide persistent walk with a work counter");
    cudaStream_t s = (cudaStream_t)stream;
    if ((st = launch_batch(b, rays, n, hits, occluded, s, StreamIn{ready, piece_shift, 2000}))) return st;
    if ((st = cuda_status(cudaStreamSynchronize(s), "cudaStreamSynchronize"))) return st;
    return device_status(b);
}

}  // extern "C"
