// server.cu - the serving loop (host code only) of the C ABI (pbrtgpu_server_*): resident
// scenes, continuous batching over the batch engine, latency statistics.
//
// One worker thread owns the batch slots.  Each turn it
//   1. retires every slot whose launch has finished (pbrtgpu_batch_poll),
//      stamping its requests with their completion time and status;
//   2. fills each free slot with the waiting requests, oldest first, until
//      one does not fit the slot's limits (the others wait for the next
//      slot), and launches it on the slot's stream;
//   3. sleeps until a submission arrives or, while batches are in flight,
//      for a short poll interval.
// So a request is admitted as soon as a slot is free, whatever else is on
// the device, and launches of different slots overlap.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/pbrt_gpu.h"
#include "capi_internal.h"

using namespace pbrt;

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    uint64_t ticket = 0;
    bool render = true;
    const PbrtScene* scene = nullptr;
    PbrtCameraDesc cam{};
    PbrtSamplerDesc smp{};
    float* rgb = nullptr;
    const PbrtBVH* bvh = nullptr;
    const PbrtRay* rays = nullptr;
    uint32_t n = 0;
    PbrtHit* hits = nullptr;
    uint8_t* occ = nullptr;
    Clock::time_point t_submit, t_done;
    bool done = false;
    int32_t status = PBRT_OK;
};

struct Slot {
    PbrtBatch* batch = nullptr;
    cudaStream_t stream = nullptr;
    std::vector<Request*> reqs;
    bool busy = false;
};

}  // namespace

struct PbrtServer {
    PbrtServerConfig cfg{};
    int device = 0;
    std::vector<Slot> slots;
    std::deque<Request*> pending;
    std::unordered_map<uint64_t, Request*> live;  // submitted, not yet waited for
    uint64_t next_ticket = 1;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::thread worker;
    bool stop = false;
    // device-memory pool (cfg.pool_bytes > 0): the slots' arenas and the
    // resident handles (scene or BVH -> bytes charged; a scene's BVH is
    // resident with it)
    uint64_t slot_bytes = 0, resident_bytes = 0;
    std::unordered_map<const void*, uint64_t> resident;
    std::unordered_map<const PbrtBVH*, uint32_t> resident_bvh;  // -> handles that make it resident
    // statistics
    uint64_t submitted = 0, completed = 0, failed = 0, batches = 0, batched_requests = 0;
    uint64_t deferred = 0, refused = 0;
    std::vector<double> latency_ms;
    bool have_first = false;
    Clock::time_point first_submit, last_done;

    void run();
    void retire(Slot& s);
    bool fill(Slot& s);
};

void PbrtServer::retire(Slot& s) {
    std::vector<int32_t> st(s.reqs.size(), PBRT_OK);
    pbrtgpu_batch_wait(s.batch, st.data());
    const Clock::time_point now = Clock::now();
    std::lock_guard<std::mutex> lk(mu);
    for (size_t i = 0; i < s.reqs.size(); ++i) {
        Request* r = s.reqs[i];
        r->status = st[i];
        r->t_done = now;
        r->done = true;
        ++completed;
        if (st[i]) ++failed;
        latency_ms.push_back(std::chrono::duration<double, std::milli>(now - r->t_submit).count());
    }
    last_done = now;
    s.reqs.clear();
    s.busy = false;
    cv_done.notify_all();
}

// Moves waiting requests into the slot's batch; true if it launched.
bool PbrtServer::fill(Slot& s) {
    std::vector<Request*> take;
    for (;;) {
        Request* r;
        {
            std::lock_guard<std::mutex> lk(mu);
            if (pending.empty()) break;
            r = pending.front();
            pending.pop_front();
        }
        // the job set-up (task windows, uploads on first use) runs without
        // the lock, so submissions are not held up
        uint32_t job;
        int st = r->render ? pbrtgpu_batch_add_render(s.batch, r->scene, &r->cam, &r->smp, r->rgb, &job)
                           : pbrtgpu_batch_add_query(s.batch, r->bvh, r->rays, r->n, r->hits, r->occ, &job);
        if (st == PBRT_ERR_BUDGET && !take.empty()) {  // full: it waits for the next slot, still first in line
            std::lock_guard<std::mutex> lk(mu);
            pending.push_front(r);
            ++deferred;
            break;
        }
        if (st) {  // it can never run (invalid, or larger than a whole slot)
            std::lock_guard<std::mutex> lk(mu);
            r->status = st;
            r->t_done = Clock::now();
            r->done = true;
            ++completed;
            ++failed;
            ++refused;
            cv_done.notify_all();
            continue;
        }
        take.push_back(r);
    }
    if (take.empty()) return false;
    s.reqs = std::move(take);
    int st = pbrtgpu_batch_launch(s.batch, (void*)s.stream);
    if (st) {  // nothing ran: fail the requests
        pbrtgpu_batch_wait(s.batch, nullptr);
        std::lock_guard<std::mutex> lk(mu);
        for (Request* r : s.reqs) {
            r->status = st;
            r->t_done = Clock::now();
            r->done = true;
            ++completed;
            ++failed;
        }
        s.reqs.clear();
        cv_done.notify_all();
        return false;
    }
    s.busy = true;
    std::lock_guard<std::mutex> lk(mu);
    ++batches;
    batched_requests += s.reqs.size();
    return true;
}

void PbrtServer::run() {
    cudaSetDevice(device);
    for (;;) {
        bool any_busy = false;
        for (Slot& s : slots) {
            if (!s.busy) continue;
            int32_t done = 0;
            pbrtgpu_batch_poll(s.batch, &done);
            if (done)
                retire(s);
            else
                any_busy = true;
        }
        for (Slot& s : slots)
            if (!s.busy && fill(s)) any_busy = true;
        std::unique_lock<std::mutex> lk(mu);
        if (stop && pending.empty() && !any_busy) {
            bool idle = true;
            for (Slot& s : slots) idle = idle && !s.busy;
            if (idle) return;
        }
        if (any_busy) {
            // batches in flight: poll again soon, or at once on a submission
            cv_work.wait_for(lk, std::chrono::microseconds(50));
        } else if (pending.empty()) {
            cv_work.wait_for(lk, std::chrono::milliseconds(20), [&] { return stop || !pending.empty(); });
        }
    }
}

namespace {

int submit(PbrtServer* S, Request* r, uint64_t* ticket) {
    {
        std::lock_guard<std::mutex> lk(S->mu);
        if (S->stop) {
            delete r;
            return set_error(PBRT_ERR_INVALID_ARGUMENT, "the server is shutting down");
        }
        r->ticket = S->next_ticket++;
        r->t_submit = Clock::now();
        if (!S->have_first) {
            S->first_submit = r->t_submit;
            S->have_first = true;
        }
        ++S->submitted;
        S->live[r->ticket] = r;
        S->pending.push_back(r);
    }
    S->cv_work.notify_one();
    if (ticket) *ticket = r->ticket;
    return PBRT_OK;
}

}  // namespace

extern "C" {

int pbrtgpu_server_create(const PbrtServerConfig* cfg, PbrtServer** out) {
    if (!cfg || !out) return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = nullptr;
    if (cfg->slots < 1 || cfg->slots > 8) return set_error(PBRT_ERR_INVALID_ARGUMENT, "slots must be in [1, 8]");
    uint64_t per_slot = 0;
    if (int st0 = pbrtgpu_batch_bytes(&cfg->limits, &per_slot, nullptr)) return st0;
    if (cfg->pool_bytes && per_slot * cfg->slots > cfg->pool_bytes)
        return set_error(PBRT_ERR_BUDGET, "the slots' arenas (" + std::to_string(per_slot * cfg->slots) +
                                              " bytes) exceed the pool of " + std::to_string(cfg->pool_bytes));
    PbrtServer* S = new PbrtServer();
    S->cfg = *cfg;
    S->slot_bytes = per_slot * cfg->slots;
    int st = cuda_status(cudaGetDevice(&S->device), "cudaGetDevice");
    for (uint32_t i = 0; !st && i < cfg->slots; ++i) {
        Slot s;
        st = pbrtgpu_batch_create(&cfg->limits, &s.batch);
        if (!st && cfg->use_tuning) st = pbrtgpu_batch_set_tuning(s.batch, &cfg->tuning);
        if (!st) st = cuda_status(cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking), "cudaStreamCreate");
        if (s.batch || s.stream) S->slots.push_back(s);
    }
    if (st) {
        for (Slot& s : S->slots) {
            if (s.batch) pbrtgpu_batch_destroy(s.batch);
            if (s.stream) cudaStreamDestroy(s.stream);
        }
        delete S;
        return st;
    }
    S->worker = std::thread([S] { S->run(); });
    *out = S;
    return PBRT_OK;
}

void pbrtgpu_server_destroy(PbrtServer* S) {
    if (!S) return;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
    }
    S->cv_work.notify_all();
    if (S->worker.joinable()) S->worker.join();
    for (Slot& s : S->slots) {
        pbrtgpu_batch_destroy(s.batch);
        cudaStreamDestroy(s.stream);
    }
    for (auto& kv : S->live) delete kv.second;
    delete S;
}

namespace {

// A submission naming a handle outside the pool is refused (pool mode only).
int check_resident(PbrtServer* S, const void* handle, bool is_bvh) {
    if (!S->cfg.pool_bytes) return PBRT_OK;
    std::lock_guard<std::mutex> lk(S->mu);
    const bool ok = is_bvh ? S->resident_bvh.count(static_cast<const PbrtBVH*>(handle)) != 0
                           : S->resident.count(handle) != 0;
    if (ok) return PBRT_OK;
    ++S->refused;
    return set_error(PBRT_ERR_BUDGET, is_bvh ? "the BVH is not resident in the server's pool (pbrtgpu_server_admit)"
                                             : "the scene is not resident in the server's pool (pbrtgpu_server_admit)");
}

}  // namespace

int pbrtgpu_server_admit(PbrtServer* S, const PbrtScene* scene, const PbrtBVH* bvh) {
    if (!S || (!scene == !bvh)) return set_error(PBRT_ERR_INVALID_ARGUMENT, "exactly one of scene and bvh");
    const void* h = scene ? (const void*)scene : (const void*)bvh;
    const PbrtBVH* b = scene ? scene->bvh : bvh;
    uint64_t bytes = 0;
    int st = scene ? pbrtgpu_scene_device_bytes(scene, &bytes) : pbrtgpu_bvh_device_bytes(bvh, &bytes);
    if (st) return st;
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->resident.count(h)) return PBRT_OK;
    const uint64_t pool = S->cfg.pool_bytes;
    if (pool && S->slot_bytes + S->resident_bytes + bytes > pool)
        return set_error(PBRT_ERR_BUDGET, "admitting " + std::to_string(bytes) + " bytes would exceed the pool (" +
                                              std::to_string(S->slot_bytes + S->resident_bytes) + " of " +
                                              std::to_string(pool) + " bytes in use)");
    S->resident[h] = bytes;
    S->resident_bytes += bytes;
    ++S->resident_bvh[b];
    return PBRT_OK;
}

int pbrtgpu_server_release(PbrtServer* S, const PbrtScene* scene, const PbrtBVH* bvh) {
    if (!S || (!scene == !bvh)) return set_error(PBRT_ERR_INVALID_ARGUMENT, "exactly one of scene and bvh");
    const void* h = scene ? (const void*)scene : (const void*)bvh;
    const PbrtBVH* b = scene ? scene->bvh : bvh;
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->resident.find(h);
    if (it == S->resident.end()) return set_error(PBRT_ERR_INVALID_ARGUMENT, "not resident");
    S->resident_bytes -= it->second;
    S->resident.erase(it);
    auto jt = S->resident_bvh.find(b);
    if (jt != S->resident_bvh.end() && --jt->second == 0) S->resident_bvh.erase(jt);
    return PBRT_OK;
}

int pbrtgpu_server_submit_render(PbrtServer* S, const PbrtScene* scene, const PbrtCameraDesc* cam,
                                 const PbrtSamplerDesc* smp, float* rgb_out, uint64_t* ticket) {
    if (!S || !scene || !cam || !smp || !rgb_out) return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (int st = check_resident(S, scene, false)) return st;
    const PbrtBatchLimits& L = S->cfg.limits;
    const uint64_t spp = (uint64_t)smp->x_samples * smp->y_samples;
    const int64_t w = (int64_t)smp->x_end - smp->x_start, h = (int64_t)smp->y_end - smp->y_start;
    if (w > 0 && h > 0 && ((uint64_t)(w * h) * spp > L.max_samples || smp->num_tasks > L.max_tasks)) {
        std::lock_guard<std::mutex> lk(S->mu);
        ++S->refused;
        return set_error(PBRT_ERR_BUDGET, "the render needs more samples or tasks than a whole batch slot holds");
    }
    Request* r = new Request();
    r->render = true;
    r->scene = scene;
    r->cam = *cam;
    r->smp = *smp;
    r->rgb = rgb_out;
    return submit(S, r, ticket);
}

int pbrtgpu_server_submit_query(PbrtServer* S, const PbrtBVH* bvh, const PbrtRay* rays, uint32_t n, PbrtHit* hits,
                                uint8_t* occluded, uint64_t* ticket) {
    if (!S || !bvh) return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n && (!rays || (!hits && !occluded))) return set_error(PBRT_ERR_INVALID_ARGUMENT, "rays/output is NULL");
    if (int st = check_resident(S, bvh, true)) return st;
    Request* r = new Request();
    r->render = false;
    r->bvh = bvh;
    r->rays = rays;
    r->n = n;
    r->hits = hits;
    r->occ = hits ? nullptr : occluded;
    return submit(S, r, ticket);
}

int pbrtgpu_server_wait(PbrtServer* S, uint64_t ticket, double timeout_s, int32_t* status) {
    if (!S) return set_error(PBRT_ERR_INVALID_ARGUMENT, "server is NULL");
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->live.find(ticket);
    if (it == S->live.end()) return set_error(PBRT_ERR_INVALID_ARGUMENT, "unknown ticket");
    Request* r = it->second;
    auto ready = [&] { return r->done; };
    if (timeout_s < 0) {
        S->cv_done.wait(lk, ready);
    } else if (!S->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), ready)) {
        return set_error(PBRT_ERR_CANCELLED, "the request has not completed within the timeout");
    }
    if (status) *status = r->status;
    S->live.erase(it);
    delete r;
    return PBRT_OK;
}

int pbrtgpu_server_drain(PbrtServer* S) {
    if (!S) return set_error(PBRT_ERR_INVALID_ARGUMENT, "server is NULL");
    std::unique_lock<std::mutex> lk(S->mu);
    S->cv_done.wait(lk, [&] { return S->completed == S->submitted; });
    return PBRT_OK;
}

int pbrtgpu_server_stats(PbrtServer* S, PbrtServerStats* out) {
    if (!S || !out) return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
    std::lock_guard<std::mutex> lk(S->mu);
    std::memset(out, 0, sizeof(*out));
    out->submitted = S->submitted;
    out->completed = S->completed;
    out->failed = S->failed;
    out->batches = S->batches;
    out->mean_batch_requests = S->batches ? (double)S->batched_requests / (double)S->batches : 0.0;
    out->pool_bytes = S->cfg.pool_bytes;
    out->slot_bytes = S->slot_bytes;
    out->resident_bytes = S->resident_bytes;
    out->resident_count = S->resident.size();
    out->deferred = S->deferred;
    out->refused = S->refused;
    std::vector<double> v = S->latency_ms;
    if (!v.empty()) {
        std::sort(v.begin(), v.end());
        auto pct = [&](double q) {
            size_t i = (size_t)std::min<double>((double)(v.size() - 1), q * (double)(v.size() - 1) + 0.5);
            return v[i];
        };
        double sum = 0.0;
        for (double x : v) sum += x;
        out->p50_ms = pct(0.50);
        out->p99_ms = pct(0.99);
        out->mean_ms = sum / (double)v.size();
        out->max_ms = v.back();
        if (S->have_first) {
            out->span_s = std::chrono::duration<double>(S->last_done - S->first_submit).count();
            if (out->span_s > 0) out->requests_per_s = (double)v.size() / out->span_s;
        }
    }
    return PBRT_OK;
}

int pbrtgpu_server_reset_stats(PbrtServer* S) {
    if (!S) return set_error(PBRT_ERR_INVALID_ARGUMENT, "server is NULL");
    std::lock_guard<std::mutex> lk(S->mu);
    S->latency_ms.clear();
    S->submitted -= S->completed;
    S->completed = 0;
    S->failed = 0;
    S->batches = 0;
    S->batched_requests = 0;
    S->deferred = 0;
    S->refused = 0;
    S->have_first = false;
    return PBRT_OK;
}

}  // extern "C"
