// capi_batch.cu - the batched multi-scene wavefront of the C ABI
// (pbrtgpu_batch_*), its CUDA graph and its autotuner.
//
// Memory: everything a batch uses is allocated once, at creation, from its
// limits - one device arena (wavefront buffers of all jobs, the shadow
// queue, counters, the job/offset/task upload block and the staging of host
// inputs and outputs) and one pinned host block (the host side of the upload
// block and the counter read-back).  Adding a job only assigns it slices of
// those buffers, so a full batch is refused up front instead of failing on
// the device.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/pbrt_gpu.h"
#include "batch.h"
#include "capi_internal.h"
#include "kernels.h"

using namespace pbrt;

namespace {

constexpr size_t kAlign = 256;
size_t up(size_t x) { return (x + kAlign - 1) & ~(kAlign - 1); }

// Byte layout of the device arena and of the upload block inside it.
struct Layout {
    size_t rays, hits, img, pixbox, le, L;          // per sample (pixbox: per pixel, pixels <= samples)
    size_t lsamp, contrib, occ, qrays, qslot, qjob;  // per light sample
    size_t counters;
    size_t upload, o_pix, o_ray, o_smp, o_film, o_jobs, o_tables, o_tasks, upload_bytes;
    size_t st_rays, st_hits, st_occ, st_rgb;
    size_t total;
    size_t pinned;  // upload block + counters

    explicit Layout(const PbrtBatchLimits& L0) {
        const uint64_t S = L0.max_samples, SL = L0.max_light_samples, J = L0.max_jobs, Q = L0.max_query_rays;
        size_t o = 0;
        auto take = [&](size_t bytes) {
            size_t at = o;
            o += up(bytes ? bytes : 1);
            return at;
        };
        rays = take(S * sizeof(PbrtRay));
        hits = take(S * 16);
        img = take(S * 8);
        pixbox = take(S * 16);
        le = take(S * 16);
        L = take(S * 16);
        lsamp = take(SL * 12);
        contrib = take(SL * 16);
        occ = take(SL);
        qrays = take(SL * sizeof(PbrtRay));
        qslot = take(SL * 4);
        qjob = take(SL * 4);
        counters = take((J + 1) * kCtrWords * 4);
        // upload block: [hdr | 4 offset arrays | jobs | filter tables | tasks]
        o_pix = up(sizeof(BatchHdr));
        o_ray = o_pix + up((J + 1) * 8);
        o_smp = o_ray + up((J + 1) * 8);
        o_film = o_smp + up((J + 1) * 8);
        o_jobs = o_film + up((J + 1) * 8);
        o_tables = o_jobs + up(J * sizeof(JobRec));
        o_tasks = o_tables + up(J * 256 * sizeof(float));
        upload_bytes = o_tasks + up((size_t)L0.max_tasks * sizeof(TaskRec));
        upload = take(upload_bytes);
        st_rays = take(Q * sizeof(PbrtRay));
        st_hits = take(Q * 16);
        st_occ = take(Q);
        st_rgb = take(L0.max_film_pixels * 12);
        total = o;
        pinned = upload_bytes + up((J + 1) * kCtrWords * 4);
    }
};

int check_limits(const PbrtBatchLimits* L) {
    if (!L) return set_error(PBRT_ERR_INVALID_ARGUMENT, "limits are NULL");
    if (L->max_jobs == 0 || L->max_jobs > (1u << 20))
        return set_error(PBRT_ERR_INVALID_ARGUMENT, "max_jobs must be in [1, 2^20]");
    const uint64_t lim = 1ull << 31;  // work counters are 32-bit
    if (L->max_samples >= lim || L->max_light_samples >= lim || L->max_film_pixels >= lim ||
        L->max_query_rays >= lim)
        return set_error(PBRT_ERR_INVALID_ARGUMENT, "sample, light-sample, film and ray limits must be below 2^31");
    return PBRT_OK;
}

struct Copy {
    void* dst;
    const void* src;
    size_t bytes;
};

}  // namespace

struct PbrtBatch {
    PbrtBatchLimits lim{};
    Layout lay;
    int device = 0, sms = 0;
    unsigned char* d = nullptr;  // device arena
    unsigned char* h = nullptr;  // pinned: upload block, then counters
    cudaStream_t cap_stream = nullptr;
    cudaEvent_t done = nullptr, t0 = nullptr, t1 = nullptr;
    std::mutex mu;

    // current jobs
    uint32_t n_jobs = 0;
    uint64_t n_pix = 0, n_ray = 0, n_smp = 0, n_lsmp = 0, n_film = 0, n_tasks = 0, n_stage = 0;
    uint32_t cover_pair = 64, cover_wide = 64;
    bool all_wide = true, mixed = false, inst = false;
    std::vector<Copy> h2d, d2h;  // staged host inputs / outputs of the jobs
    bool in_flight = false;

    // 4-wide walks where every job has the layout; camera and query rays
    // walked to the end per lane, shadow rays refilled once 8 lanes are idle
    // (serving mix of 32 soups: 5280 against 5100 requests/s with 32 / 32)
    BatchTuning tune{1, 1, 128, 16, 64, 32, 8};
    bool use_graph = true;
    cudaGraphExec_t graph = nullptr;
    BatchTuning graph_tune{};
    bool graph_mixed = false;
    bool graph_inst = false;
    uint32_t graph_cover_pair = 0, graph_cover_wide = 0;
    int graph_kernels = 0;
    int last_kernels = 0;
    bool last_graph = false;

    explicit PbrtBatch(const PbrtBatchLimits& L) : lim(L), lay(L) {}
    ~PbrtBatch() {
        if (graph) cudaGraphExecDestroy(graph);
        if (done) cudaEventDestroy(done);
        if (t0) cudaEventDestroy(t0);
        if (t1) cudaEventDestroy(t1);
        if (cap_stream) cudaStreamDestroy(cap_stream);
        if (d) cudaFree(d);
        if (h) cudaFreeHost(h);
    }

    BatchHdr* hdr() { return reinterpret_cast<BatchHdr*>(h); }
    uint64_t* off(size_t o) { return reinterpret_cast<uint64_t*>(h + o); }
    JobRec* jobs() { return reinterpret_cast<JobRec*>(h + lay.o_jobs); }
    TaskRec* tasks() { return reinterpret_cast<TaskRec*>(h + lay.o_tasks); }
    uint32_t* counters_h() { return reinterpret_cast<uint32_t*>(h + lay.upload_bytes); }
    template <class T>
    T* dev(size_t o) {
        return reinterpret_cast<T*>(d + o);
    }

    BatchArgs args() {
        BatchArgs A;
        std::memset(&A, 0, sizeof(A));
        unsigned char* u = d + lay.upload;
        A.hdr = reinterpret_cast<const BatchHdr*>(u);
        A.jobs = reinterpret_cast<const JobRec*>(u + lay.o_jobs);
        A.off_pix = reinterpret_cast<const uint64_t*>(u + lay.o_pix);
        A.off_ray = reinterpret_cast<const uint64_t*>(u + lay.o_ray);
        A.off_smp = reinterpret_cast<const uint64_t*>(u + lay.o_smp);
        A.off_film = reinterpret_cast<const uint64_t*>(u + lay.o_film);
        A.q_rays = dev<PbrtRay>(lay.qrays);
        A.q_slot = dev<uint32_t>(lay.qslot);
        A.q_job = dev<uint32_t>(lay.qjob);
        A.counters = dev<uint32_t>(lay.counters);
        A.chunk = tune.chunk;
        A.refill = tune.refill;
        A.refill_shadow = tune.refill_shadow;
        return A;
    }

    void clear() {
        n_jobs = 0;
        n_pix = n_ray = n_smp = n_lsmp = n_film = n_tasks = n_stage = 0;
        cover_pair = cover_wide = 64;
        all_wide = true;
        mixed = false;
        inst = false;
        h2d.clear();
        d2h.clear();
        uint64_t* offs[4] = {off(lay.o_pix), off(lay.o_ray), off(lay.o_smp), off(lay.o_film)};
        for (uint64_t* o : offs) o[0] = 0;
    }

    // Appends job j's offsets (n_* already advanced).
    void close_job() {
        off(lay.o_pix)[n_jobs + 1] = n_pix;
        off(lay.o_ray)[n_jobs + 1] = n_ray;
        off(lay.o_smp)[n_jobs + 1] = n_smp;
        off(lay.o_film)[n_jobs + 1] = n_film;
        ++n_jobs;
    }

    size_t counter_bytes() const { return (size_t)(n_jobs + 1) * kCtrWords * 4; }
};

namespace {

int enqueue_stages(PbrtBatch* b, cudaStream_t s) {
    BatchArgs A = b->args();
    const bool key_match = b->graph && !std::memcmp(&b->graph_tune, &b->tune, sizeof(BatchTuning)) &&
                           b->graph_mixed == b->mixed && b->graph_inst == b->inst &&
                           b->graph_cover_pair == b->cover_pair &&
                           b->graph_cover_wide == b->cover_wide;
    // the graph zeroes every job slot's counters, so it serves any job count
    const size_t cbytes = (size_t)(b->lim.max_jobs + 1) * kCtrWords * 4;
    if (b->use_graph && key_match) {
        b->last_graph = true;
        b->last_kernels = b->graph_kernels;
        return cuda_status(cudaGraphLaunch(b->graph, s), "cudaGraphLaunch");
    }
    int n = 0;
    int st = cuda_status(launch_batch_stages(A, b->tune, b->mixed, b->inst, b->cover_pair, b->cover_wide, b->sms, cbytes, s, &n),
                         "batch stages");
    if (st) return st;
    b->last_graph = false;
    b->last_kernels = n;
    if (b->use_graph) {
        // capture the same sequence for the next launches with this key (the
        // direct launch above has fixed every kernel's occupancy first)
        if (b->graph) cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
        cudaGraph_t g = nullptr;
        if ((st = cuda_status(cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeThreadLocal),
                              "cudaStreamBeginCapture")))
            return st;
        int m = 0;
        cudaError_t e =
            launch_batch_stages(A, b->tune, b->mixed, b->inst, b->cover_pair, b->cover_wide, b->sms, cbytes,
                                b->cap_stream, &m);
        cudaError_t e2 = cudaStreamEndCapture(b->cap_stream, &g);
        if (e == cudaSuccess) e = e2;
        if (e == cudaSuccess) e = cudaGraphInstantiate(&b->graph, g, 0);
        if (g) cudaGraphDestroy(g);
        if ((st = cuda_status(e, "batch graph capture"))) {
            b->graph = nullptr;
            return st;
        }
        b->graph_tune = b->tune;
        b->graph_mixed = b->mixed;
        b->graph_inst = b->inst;
        b->graph_cover_pair = b->cover_pair;
        b->graph_cover_wide = b->cover_wide;
        b->graph_kernels = m;
    }
    return PBRT_OK;
}

// Uploads the jobs, runs the stages and queues the output copies; records
// b->done.  With `timed`, events t0/t1 bracket the stages.
int launch_locked(PbrtBatch* b, cudaStream_t s, bool timed) {
    if (b->in_flight) return set_error(PBRT_ERR_INVALID_ARGUMENT, "the previous launch has not been waited for");
    DeviceGuard g(b->device);
    BatchHdr* H = b->hdr();
    H->n_jobs = b->n_jobs;
    H->pix = b->n_pix;
    H->rays = b->n_ray;
    H->samples = b->n_smp;
    H->film = b->n_film;
    int st;
    unsigned char* du = b->d + b->lay.upload;
    if ((st = cuda_status(cudaMemcpyAsync(du, b->h, b->lay.o_tables + (size_t)b->n_jobs * 256 * sizeof(float),
                                          cudaMemcpyHostToDevice, s),
                          "batch jobs H2D")))
        return st;
    if (b->n_tasks &&
        (st = cuda_status(cudaMemcpyAsync(du + b->lay.o_tasks, b->h + b->lay.o_tasks, b->n_tasks * sizeof(TaskRec),
                                          cudaMemcpyHostToDevice, s),
                          "batch tasks H2D")))
        return st;
    for (const Copy& c : b->h2d)
        if ((st = cuda_status(cudaMemcpyAsync(c.dst, c.src, c.bytes, cudaMemcpyHostToDevice, s), "query rays H2D")))
            return st;
    if (timed) cudaEventRecord(b->t0, s);
    if (b->n_jobs && (st = enqueue_stages(b, s))) return st;
    if (timed) cudaEventRecord(b->t1, s);
    for (const Copy& c : b->d2h)
        if ((st = cuda_status(cudaMemcpyAsync(c.dst, c.src, c.bytes, cudaMemcpyDeviceToHost, s), "outputs D2H")))
            return st;
    if ((st = cuda_status(cudaMemcpyAsync(b->counters_h(), b->d + b->lay.counters, b->counter_bytes(),
                                          cudaMemcpyDeviceToHost, s),
                          "counters D2H")) ||
        (st = cuda_status(cudaEventRecord(b->done, s), "cudaEventRecord")))
        return st;
    b->in_flight = true;
    return PBRT_OK;
}

// Waits for the launch and collects per-job status; keeps the jobs.
int wait_locked(PbrtBatch* b, int32_t* job_status) {
    if (!b->in_flight) return set_error(PBRT_ERR_INVALID_ARGUMENT, "nothing launched");
    DeviceGuard g(b->device);
    int st = cuda_status(cudaEventSynchronize(b->done), "cudaEventSynchronize");
    b->in_flight = false;
    if (st) return st;
    const uint32_t* C = b->counters_h();
    int first = PBRT_OK;
    std::string msg;
    for (uint32_t j = 0; j < b->n_jobs; ++j) {
        const uint32_t* c = C + (size_t)(j + 1) * kCtrWords;
        int js = PBRT_OK;
        if (c[2]) {
            js = (int)c[2];
            if (!first) msg = "job " + std::to_string(j) + ": device-side traversal failure";
        } else if (c[1]) {
            js = PBRT_ERR_NAN;
            if (!first)
                msg = "job " + std::to_string(j) + ": " + std::to_string(c[1]) +
                      " radiance samples were NaN (sampler_renderer.rs:105)";
        }
        if (job_status) job_status[j] = js;
        if (js && !first) first = js;
    }
    return first ? set_error(first, msg) : PBRT_OK;
}

}  // namespace

extern "C" {

int pbrtgpu_batch_bytes(const PbrtBatchLimits* limits, uint64_t* device_bytes, uint64_t* pinned_bytes) {
    int st = check_limits(limits);
    if (st) return st;
    Layout L(*limits);
    if (device_bytes) *device_bytes = L.total;
    if (pinned_bytes) *pinned_bytes = L.pinned;
    return PBRT_OK;
}

int pbrtgpu_batch_create(const PbrtBatchLimits* limits, PbrtBatch** out) {
    if (!out) return set_error(PBRT_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    int st = check_limits(limits);
    if (st) return st;
    if (!cuda_device_present()) return set_error(PBRT_ERR_NO_DEVICE, "no CUDA device");
    PbrtBatch* b = new PbrtBatch(*limits);
    auto fail = [&](int s) {
        delete b;
        return s;
    };
    if ((st = cuda_status(cudaGetDevice(&b->device), "cudaGetDevice")) ||
        (st = cuda_status(cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device), "SM count")) ||
        (st = cuda_status(cudaMalloc(&b->d, b->lay.total), "cudaMalloc (batch arena)")) ||
        (st = cuda_status(cudaMallocHost(&b->h, b->lay.pinned), "cudaMallocHost (batch staging)")) ||
        (st = cuda_status(cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking), "cudaStreamCreate")) ||
        (st = cuda_status(cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming), "cudaEventCreate")) ||
        (st = cuda_status(cudaEventCreate(&b->t0), "cudaEventCreate")) ||
        (st = cuda_status(cudaEventCreate(&b->t1), "cudaEventCreate")))
        return fail(st);
    std::memset(b->h, 0, b->lay.pinned);
    b->clear();
    *out = b;
    return PBRT_OK;
}

void pbrtgpu_batch_destroy(PbrtBatch* b) {
    if (!b) return;
    {
        std::lock_guard<std::mutex> lk(b->mu);
        if (b->in_flight) cudaEventSynchronize(b->done);
    }
    delete b;
}

int pbrtgpu_batch_add_render(PbrtBatch* b, const PbrtScene* cS, const PbrtCameraDesc* cam,
                             const PbrtSamplerDesc* smp, float* rgb_out, uint32_t* job) {
    if (!b || !cS || !cam || !smp || !rgb_out) return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
    std::lock_guard<std::mutex> lk(b->mu);
    if (b->in_flight) return set_error(PBRT_ERR_INVALID_ARGUMENT, "the batch is running: wait for it first");
    PbrtScene* S = const_cast<PbrtScene*>(cS);
    if (S->bvh->device != b->device && S->uploaded)
        return set_error(PBRT_ERR_INVALID_ARGUMENT, "the scene lives on another device than the batch");
    RenderParams P;
    std::vector<TaskRec> tasks;
    int st = prepare_render(S, cam, smp, 0, smp->num_tasks, &P, &tasks);
    if (st) return st;
    const uint64_t nl = P.n_lights, SL = P.n_samples * nl;
    const uint64_t npx = (uint64_t)(P.fx1 - P.fx0) * (uint64_t)(P.fy1 - P.fy0);
    const PbrtBatchLimits& L = b->lim;
    if (b->n_jobs + 1 > L.max_jobs || b->n_smp + P.n_samples > L.max_samples ||
        b->n_lsmp + SL > L.max_light_samples || b->n_film + npx > L.max_film_pixels ||
        b->n_tasks + tasks.size() > L.max_tasks)
        return set_error(PBRT_ERR_BUDGET, "the render does not fit the batch's remaining jobs, samples, light "
                                          "samples, film pixels or tasks");
    if (b->n_ray + P.n_samples >= (1ull << 31))  // the traversal stages count rays in 32 bits
        return set_error(PBRT_ERR_BUDGET, "the batch's rays would reach 2^31");
    const uint32_t cp = (uint32_t)trace_stack_for_depth(P.depth);
    if (cp == 0) return set_error(PBRT_ERR_UNSUPPORTED, "BVH deeper than the batch kernels' stacks");
    const bool inst = P.bvh.insts != nullptr;  // batches walk instanced jobs over the binary layout
    const uint32_t cw = (P.has_wide && !inst) ? (uint32_t)wide_stack_variant(P.wide_bound) : 0u;
    const uint32_t j = b->n_jobs;
    const Layout& Y = b->lay;
    float* table = reinterpret_cast<float*>(b->h + Y.o_tables) + (size_t)j * 256;
    filter_table(*cam, table);  // kind checked by prepare_render
    P.filter_table = reinterpret_cast<const float*>(b->d + Y.upload + Y.o_tables) + (size_t)j * 256;
    P.tasks = reinterpret_cast<const TaskRec*>(b->d + Y.upload + Y.o_tasks) + b->n_tasks;
    P.n_tasks = smp->num_tasks;
    P.rays = b->dev<PbrtRay>(Y.rays) + b->n_smp;
    P.hits = b->dev<float4>(Y.hits) + b->n_smp;
    P.img = b->dev<float2>(Y.img) + b->n_smp;
    P.pixbox = b->dev<float4>(Y.pixbox) + b->n_pix;
    P.le = b->dev<float4>(Y.le) + b->n_smp;
    P.L = b->dev<float4>(Y.L) + b->n_smp;
    P.lsamp = b->dev<float>(Y.lsamp) + 3 * b->n_lsmp;
    P.contrib = b->dev<float4>(Y.contrib) + b->n_lsmp;
    P.occluded = b->dev<uint8_t>(Y.occ) + b->n_lsmp;
    P.shadow_rays = nullptr;
    P.shadow_slot = nullptr;
    P.counters = b->dev<uint32_t>(Y.counters) + (size_t)(j + 1) * kCtrWords;
    const bool dev_out = is_device_pointer(rgb_out);
    P.rgb = dev_out ? rgb_out : b->dev<float>(Y.st_rgb) + 3 * b->n_film;
    if (!dev_out) b->d2h.push_back(Copy{rgb_out, P.rgb, (size_t)npx * 12});

    JobRec& J = b->jobs()[j];
    std::memset(&J, 0, sizeof(J));
    J.P = P;
    J.rays = reinterpret_cast<const float4*>(P.rays);
    J.hits = P.hits;
    J.kind = kJobRender;
    J.wide = cw ? 1u : 0u;
    std::memcpy(b->tasks() + b->n_tasks, tasks.data(), tasks.size() * sizeof(TaskRec));
    b->n_tasks += tasks.size();
    b->n_pix += P.n_pixels;
    b->n_ray += P.n_samples;
    b->n_smp += P.n_samples;
    b->n_lsmp += SL;
    b->n_film += npx;
    b->cover_pair = std::max(b->cover_pair, cp);
    b->inst = b->inst || inst;
    if (cw)
        b->cover_wide = std::max(b->cover_wide, cw);
    else
        b->all_wide = false;
    b->close_job();
    if (job) *job = j;
    return PBRT_OK;
}

int pbrtgpu_batch_add_query(PbrtBatch* b, const PbrtBVH* cb, const PbrtRay* rays, uint32_t n, PbrtHit* hits,
                            uint8_t* occluded, uint32_t* job) {
    if (!b || !cb) return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n && (!rays || (!hits && !occluded))) return set_error(PBRT_ERR_INVALID_ARGUMENT, "rays/output is NULL");
    std::lock_guard<std::mutex> lk(b->mu);
    if (b->in_flight) return set_error(PBRT_ERR_INVALID_ARGUMENT, "the batch is running: wait for it first");
    PbrtBVH* B = const_cast<PbrtBVH*>(cb);
    int st;
    if (!B->uploaded && (st = bvh_upload(B))) return st;
    if (B->device != b->device) return set_error(PBRT_ERR_INVALID_ARGUMENT, "the BVH lives on another device");
    const bool dr = n ? is_device_pointer(rays) : true;
    void* out = hits ? (void*)hits : (void*)occluded;
    const bool dout = n ? is_device_pointer(out) : true;
    const bool staged = !dr || !dout;
    const PbrtBatchLimits& L = b->lim;
    if (b->n_jobs + 1 > L.max_jobs || (staged && b->n_stage + n > L.max_query_rays))
        return set_error(PBRT_ERR_BUDGET, "the query does not fit the batch's remaining jobs or staged rays");
    // the traversal stages count the batch's rays in 32 bits (their work
    // counters, the refilling walk's ray positions)
    if (b->n_ray + n >= (1ull << 31))
        return set_error(PBRT_ERR_BUDGET, "the batch's rays would reach 2^31");
    const uint32_t cp = (uint32_t)trace_stack_for_depth(B->host.depth);
    if (cp == 0) return set_error(PBRT_ERR_UNSUPPORTED, "BVH deeper than the batch kernels' stacks");
    const bool inst = B->dev.insts != nullptr;  // batches walk instanced jobs over the binary layout
    const DevBVH4* w = inst ? nullptr : wide_of(B);
    const uint32_t cw = w ? (uint32_t)wide_stack_variant(B->host.stack4_bound) : 0u;
    const uint32_t j = b->n_jobs;
    const Layout& Y = b->lay;
    JobRec& J = b->jobs()[j];
    std::memset(&J, 0, sizeof(J));
    J.P.bvh = B->dev;
    J.P.depth = B->host.depth;
    J.P.bvh4 = B->dev4;
    J.P.wide_bound = B->host.stack4_bound;
    J.P.has_wide = w ? 1u : 0u;
    J.P.counters = b->dev<uint32_t>(Y.counters) + (size_t)(j + 1) * kCtrWords;
    J.kind = kJobQuery;
    J.any = hits ? 0u : 1u;
    J.wide = cw ? 1u : 0u;
    if (dr) {
        J.rays = reinterpret_cast<const float4*>(rays);
    } else {
        PbrtRay* dst = b->dev<PbrtRay>(Y.st_rays) + b->n_stage;
        b->h2d.push_back(Copy{dst, rays, (size_t)n * sizeof(PbrtRay)});
        J.rays = reinterpret_cast<const float4*>(dst);
    }
    if (hits) {
        J.hits = dout ? reinterpret_cast<float4*>(hits) : b->dev<float4>(Y.st_hits) + b->n_stage;
        if (!dout) b->d2h.push_back(Copy{hits, J.hits, (size_t)n * 16});
    } else {
        J.occ = dout ? occluded : b->dev<uint8_t>(Y.st_occ) + b->n_stage;
        if (!dout) b->d2h.push_back(Copy{occluded, J.occ, (size_t)n});
        b->mixed = true;
    }
    if (staged) b->n_stage += n;
    b->n_ray += n;
    b->cover_pair = std::max(b->cover_pair, cp);
    b->inst = b->inst || inst;
    if (cw)
        b->cover_wide = std::max(b->cover_wide, cw);
    else
        b->all_wide = false;
    b->close_job();
    if (job) *job = j;
    return PBRT_OK;
}

int pbrtgpu_batch_launch(PbrtBatch* b, void* stream) {
    if (!b) return set_error(PBRT_ERR_INVALID_ARGUMENT, "batch is NULL");
    std::lock_guard<std::mutex> lk(b->mu);
    // a 4-wide tuning needs every job's 4-wide layout
    BatchTuning keep = b->tune;
    if (!b->all_wide) b->tune.extend_wide = b->tune.shadow_wide = 0;
    int st = launch_locked(b, (cudaStream_t)stream, false);
    b->tune = keep;
    return st;
}

int pbrtgpu_batch_poll(PbrtBatch* b, int32_t* done) {
    if (!b || !done) return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
    std::lock_guard<std::mutex> lk(b->mu);
    if (!b->in_flight) {
        *done = 1;
        return PBRT_OK;
    }
    cudaError_t e = cudaEventQuery(b->done);
    if (e == cudaErrorNotReady) {
        *done = 0;
        return PBRT_OK;
    }
    *done = 1;
    return cuda_status(e, "cudaEventQuery");
}

int pbrtgpu_batch_wait(PbrtBatch* b, int32_t* job_status) {
    if (!b) return set_error(PBRT_ERR_INVALID_ARGUMENT, "batch is NULL");
    std::lock_guard<std::mutex> lk(b->mu);
    int st = b->in_flight ? wait_locked(b, job_status) : PBRT_OK;  // never launched: just empty it
    b->clear();
    return st;
}

int pbrtgpu_batch_set_tuning(PbrtBatch* b, const PbrtBatchTuning* t) {
    if (!b || !t) return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
    auto kern_ok = [](int32_t k) { return k == PBRT_TRACE_PAIR || k == PBRT_TRACE_WIDE; };
    if (!kern_ok(t->extend_kernel) || !kern_ok(t->shadow_kernel) || (t->block != 128 && t->block != 256) ||
        (t->stack != 8 && t->stack != 16) || t->chunk < 32 || t->chunk > 4096 || t->chunk % 32 ||
        t->refill < 1 || t->refill > 32 || t->refill_shadow < 1 || t->refill_shadow > 32 || t->use_graph > 1)
        return set_error(PBRT_ERR_INVALID_ARGUMENT,
                         "batch tuning: kernels pair/wide, block 128/256, stack 8/16, chunk 32..4096 (multiple of "
                         "32), refills 1..32, use_graph 0/1");
    std::lock_guard<std::mutex> lk(b->mu);
    b->tune.extend_wide = t->extend_kernel == PBRT_TRACE_WIDE;
    b->tune.shadow_wide = t->shadow_kernel == PBRT_TRACE_WIDE;
    b->tune.block = (int)t->block;
    b->tune.smax = (int)t->stack;
    b->tune.chunk = t->chunk;
    b->tune.refill = t->refill;
    b->tune.refill_shadow = t->refill_shadow;
    b->use_graph = t->use_graph != 0;
    return PBRT_OK;
}

int pbrtgpu_batch_get_tuning(const PbrtBatch* cb, PbrtBatchTuning* t) {
    if (!cb || !t) return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
    PbrtBatch* b = const_cast<PbrtBatch*>(cb);
    std::lock_guard<std::mutex> lk(b->mu);
    t->extend_kernel = b->tune.extend_wide ? PBRT_TRACE_WIDE : PBRT_TRACE_PAIR;
    t->shadow_kernel = b->tune.shadow_wide ? PBRT_TRACE_WIDE : PBRT_TRACE_PAIR;
    t->block = (uint32_t)b->tune.block;
    t->stack = (uint32_t)b->tune.smax;
    t->chunk = b->tune.chunk;
    t->refill = b->tune.refill;
    t->refill_shadow = b->tune.refill_shadow;
    t->use_graph = b->use_graph ? 1u : 0u;
    return PBRT_OK;
}

int pbrtgpu_batch_stats(const PbrtBatch* cb, PbrtBatchStats* s) {
    if (!cb || !s) return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
    PbrtBatch* b = const_cast<PbrtBatch*>(cb);
    std::lock_guard<std::mutex> lk(b->mu);
    std::memset(s, 0, sizeof(*s));
    s->jobs = b->n_jobs;
    s->kernels = (uint32_t)b->last_kernels;
    s->samples = b->n_smp;
    s->light_samples = b->n_lsmp;
    s->film_pixels = b->n_film;
    s->query_rays = b->n_ray - b->n_smp;
    s->graph = b->last_graph ? 1u : 0u;
    return PBRT_OK;
}

int pbrtgpu_batch_autotune(PbrtBatch* b, void* stream, uint32_t repeats, PbrtBatchTuning* best, float* best_ms) {
    if (!b) return set_error(PBRT_ERR_INVALID_ARGUMENT, "batch is NULL");
    if (repeats == 0) repeats = 3;
    std::lock_guard<std::mutex> lk(b->mu);
    if (b->in_flight) return set_error(PBRT_ERR_INVALID_ARGUMENT, "the batch is running: wait for it first");
    if (b->n_jobs == 0) return set_error(PBRT_ERR_INVALID_ARGUMENT, "the batch has no jobs to tune on");
    cudaStream_t s = (cudaStream_t)stream;
    // time of one configuration: the fastest of `repeats` launches (stages only)
    auto trial = [&](const BatchTuning& T, bool graph, float* ms) -> int {
        b->tune = T;
        b->use_graph = graph;
        float m = 1e30f;
        for (uint32_t r = 0; r <= repeats; ++r) {  // the first launch (and graph capture) is not timed
            int st = launch_locked(b, s, true);
            if (!st) st = wait_locked(b, nullptr);
            if (st) return st;
            float x = 0.0f;
            if ((st = cuda_status(cudaEventElapsedTime(&x, b->t0, b->t1), "cudaEventElapsedTime"))) return st;
            if (r > 0) m = std::min(m, x);
        }
        *ms = m;
        return PBRT_OK;
    };
    BatchTuning cur = b->tune;
    bool graph = b->use_graph;
    if (!b->all_wide) cur.extend_wide = cur.shadow_wide = 0;
    float cur_ms;
    int st = trial(cur, graph, &cur_ms);
    if (st) return st;
    // coordinate descent, one pass in this order
    std::vector<std::vector<int>> space = {
        b->all_wide ? std::vector<int>{0, 1} : std::vector<int>{0},  // extend_wide
        b->all_wide ? std::vector<int>{0, 1} : std::vector<int>{0},  // shadow_wide
        {128, 256},                                                   // block
        {8, 16},                                                      // smax
        {32, 64, 128, 256},                                           // chunk
        {4, 8, 16, 32},                                               // refill
        {4, 8, 16, 32},                                               // refill_shadow
        {0, 1},                                                       // graph
    };
    for (size_t d = 0; d < space.size(); ++d) {
        if (d == 3 && !cur.extend_wide && !cur.shadow_wide) continue;  // stack only matters for 4-wide
        for (int v : space[d]) {
            BatchTuning T = cur;
            bool gr = graph;
            switch (d) {
                case 0: if (T.extend_wide == v) continue; T.extend_wide = v; break;
                case 1: if (T.shadow_wide == v) continue; T.shadow_wide = v; break;
                case 2: if (T.block == v) continue; T.block = v; break;
                case 3: if (T.smax == v) continue; T.smax = v; break;
                case 4: if ((int)T.chunk == v) continue; T.chunk = (uint32_t)v; break;
                case 5: if ((int)T.refill == v) continue; T.refill = (uint32_t)v; break;
                case 6: if ((int)T.refill_shadow == v) continue; T.refill_shadow = (uint32_t)v; break;
                default: if ((int)gr == v) continue; gr = v != 0; break;
            }
            float ms;
            if ((st = trial(T, gr, &ms))) return st;
            if (ms < cur_ms) {
                cur = T;
                graph = gr;
                cur_ms = ms;
            }
        }
    }
    b->tune = cur;
    b->use_graph = graph;
    if (best) {
        best->extend_kernel = cur.extend_wide ? PBRT_TRACE_WIDE : PBRT_TRACE_PAIR;
        best->shadow_kernel = cur.shadow_wide ? PBRT_TRACE_WIDE : PBRT_TRACE_PAIR;
        best->block = (uint32_t)cur.block;
        best->stack = (uint32_t)cur.smax;
        best->chunk = cur.chunk;
        best->refill = cur.refill;
        best->refill_shadow = cur.refill_shadow;
        best->use_graph = graph ? 1u : 0u;
    }
    if (best_ms) *best_ms = cur_ms;
    return PBRT_OK;
}

}  // extern "C"
