// capi_noalloc.cu - pbrtgpu_render_noalloc: a render entry point that
// allocates nothing.
//
// pbrtgpu_render keeps grow-only scratch buffers per scene and allocates
// them with cudaMalloc on first use or when a larger frame arrives.  Some
// callers cannot allow that at render time: a serving process that
// reserves its device memory up front and admits work against that fixed
// budget, or an interactive frame loop that cannot afford the device-wide
// synchronisation a cudaMalloc/cudaFree may imply.  This entry point runs
// the same wavefront kernels with all of its scratch (rays, hits, sample
// data, the shadow-ray queue, counters, the task and filter tables and,
// for host outputs, the staging of the image) carved out of one fixed
// array of device memory that exists for the life of the process.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/pbrt_gpu.h"
#include "capi_internal.h"
#include "host_scene.h"
#include "kernels.h"
#include "render_types.h"

using namespace pbrt;

namespace pbrt {

cudaError_t launch_render(const RenderParams& P, cudaStream_t s);

// The scratch: 64 MiB on every GPU where this file's device code is
// loaded, held until the process exits.
constexpr size_t kNoAllocScratchBytes = (size_t)64 << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kNoAllocMaxDevices = 64;
constexpr uint32_t kNoAllocMaxTasks = 256;
static std::mutex g_noalloc_mu;

// The scratch's device address on one device, and the id of the CUDA
// context it was looked up in: a context made after cudaDeviceReset has a
// new id and its own copy of the array, so the address is looked up again.
struct NoAllocSlot {
    unsigned long long ctx_id = 0;
    unsigned char* base = nullptr;
};
static NoAllocSlot g_noalloc_slot[kNoAllocMaxDevices];

// cuCtxGetCurrent + cuCtxGetId through the runtime's driver entry points
// (no link against libcuda): the id of the calling thread's current context,
// unique for the life of the process; 0 when it cannot be read.
static unsigned long long current_context_id() {
    using GetCurrent = CUresult (*)(CUcontext*);
    using GetId = CUresult (*)(CUcontext, unsigned long long*);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<GetCurrent>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<GetId>(f);
    });
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS)
        return 0;
    return id;
}

// Device address of the scratch on `dev`, which must be the current device.
// In host code the array's name is only a host-side stand-in, never a
// device address, so the address comes from cudaGetSymbolAddress, looked
// up once per device (and context); the lookup loads the array's module,
// i.e. reserves the 64 MiB on that device.  Leaves the thread's error text
// alone; returns the CUDA error.
static cudaError_t noalloc_scratch(int dev, unsigned char** out) {
    if (dev < 0 || dev >= kNoAllocMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    NoAllocSlot& slot = g_noalloc_slot[dev];
    const unsigned long long ctx = current_context_id();
    if (!slot.base || ctx != slot.ctx_id) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        slot.base = static_cast<unsigned char*>(p);
        slot.ctx_id = ctx;
    }
    *out = slot.base;
    return cudaSuccess;
}

int noalloc_prepare(int dev) {
    unsigned char* base = nullptr;
    return noalloc_scratch(dev, &base) == cudaSuccess ? PBRT_OK : PBRT_ERR_CUDA;
}

// Carves 256-byte aligned pieces; with base == nullptr it only measures.
struct Carve {
    unsigned char* base;
    size_t off;
    void* take(size_t bytes) {
        size_t o = (off + 255) & ~(size_t)255;
        off = o + bytes;
        return base ? base + o : nullptr;
    }
};

}  // namespace pbrt

extern "C" int pbrtgpu_render_noalloc(const PbrtScene* cS, const PbrtCameraDesc* cam, const PbrtSamplerDesc* smp,
                                      float* rgb_out, void* stream_v) {
    PbrtScene* S = const_cast<PbrtScene*>(cS);
    if (!S || !cam || !smp || !rgb_out) return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (smp->num_tasks == 0 || smp->num_tasks > kNoAllocMaxTasks)
        return set_error(PBRT_ERR_INVALID_ARGUMENT, "num_tasks must be in [1, 256] for pbrtgpu_render_noalloc");
    if (smp->x_end <= smp->x_start || smp->y_end <= smp->y_start)
        return set_error(PBRT_ERR_INVALID_ARGUMENT, "empty sampler window");
    const uint32_t spp = smp->x_samples * smp->y_samples;
    if (spp == 0 || spp > 64) return set_error(PBRT_ERR_UNSUPPORTED, "samples per pixel must be in [1, 64]");
    if (cam->x_res == 0 || cam->y_res == 0) return set_error(PBRT_ERR_INVALID_ARGUMENT, "empty film");
    if (!(cam->filter_x_width > 0.0f) || !(cam->filter_y_width > 0.0f) || cam->filter_x_width > 16.0f ||
        cam->filter_y_width > 16.0f)
        return set_error(PBRT_ERR_INVALID_ARGUMENT, "filter width must be in (0, 16]");
    if (!S->uploaded)
        return set_error(PBRT_ERR_INVALID_ARGUMENT,
                         "the scene has no device copy; pbrtgpu_scene_create makes one when a CUDA device is present");
    DeviceGuard g(S->bvh->device);
    std::lock_guard<std::mutex> lk(S->mu);
    unsigned char* base = nullptr;
    int st;
    if (S->bvh->device < 0 || S->bvh->device >= kNoAllocMaxDevices)
        return set_error(PBRT_ERR_UNSUPPORTED, "device index out of range");
    if ((st = cuda_status(noalloc_scratch(S->bvh->device, &base), "cudaGetSymbolAddress"))) return st;
    cudaStream_t s = (cudaStream_t)stream_v;
    const uint32_t nl = (uint32_t)S->lights.size();
    uint32_t n_pixels;
    uint64_t n_samples;
    if ((st = sampler_counts(smp, spp, nl, &n_pixels, &n_samples))) return st;

    RenderParams P;
    std::memset(&P, 0, sizeof(P));
    camera_matrices(*cam, P.r2c, P.c2w);
    P.lens_radius = cam->lens_radius;
    P.focal_distance = cam->focal_distance;
    P.sx0 = smp->x_start;
    P.sx1 = smp->x_end;
    P.sy0 = smp->y_start;
    P.sy1 = smp->y_end;
    P.xs = smp->x_samples;
    P.ys = smp->y_samples;
    P.spp = spp;
    P.jitter = smp->jitter ? 1u : 0u;
    P.sopen = smp->shutter_open;
    P.sclose = smp->shutter_close;
    P.words_per_pixel = (P.jitter ? 5u * spp : 0u) + 4u * spp + 9u * nl * spp;
    P.n_pixels = n_pixels;
    P.n_samples = n_samples;
    int32_t fe[4];
    film_extent(cam->x_res, cam->y_res, cam->crop_window, fe);
    P.fx0 = fe[0];
    P.fx1 = fe[1];
    P.fy0 = fe[2];
    P.fy1 = fe[3];
    P.filter_xw = cam->filter_x_width;
    P.filter_yw = cam->filter_y_width;
    P.filter_inv_xw = 1.0f / cam->filter_x_width;
    P.filter_inv_yw = 1.0f / cam->filter_y_width;
    gather_offsets(cam->filter_x_width, P.sx0, P.sx1, &P.gx0, &P.gx1);
    gather_offsets(cam->filter_y_width, P.sy0, P.sy1, &P.gy0, &P.gy1);

    // task table and filter table on the host stack (no heap use)
    TaskRec tasks[kNoAllocMaxTasks];
    const float aspect = (float)cam->x_res / (float)cam->y_res;
    const float* crop = cam->crop_window;
    for (uint32_t t = 0; t < smp->num_tasks; ++t) {
        TaskRec& T = tasks[t];
        std::memset(&T, 0, sizeof(T));
        int32_t w[4];
        sub_window(*smp, t, w);
        chacha_key(t, T.key);
        if (w[0] == w[1] || w[2] == w[3]) continue;
        T.wx0 = w[0];
        T.wx1 = w[1];
        T.wy0 = w[2];
        T.wy1 = w[3];
        float cw[4];
        crop_window(t, smp->num_tasks, aspect, cw);
        float dx = crop[1] - crop[0], dy = crop[3] - crop[2];
        float sub[4] = {crop[0] + cw[0] * dx, crop[0] + cw[1] * dx, crop[2] + cw[2] * dy, crop[2] + cw[3] * dy};
        int32_t te[4];
        film_extent(cam->x_res, cam->y_res, sub, te);
        T.fx0 = std::max(te[0], P.fx0);
        T.fx1 = std::min(te[1], P.fx1);
        T.fy0 = std::max(te[2], P.fy0);
        T.fy1 = std::min(te[3], P.fy1);
    }
    float table[256];
    if (filter_table(*cam, table)) return set_error(PBRT_ERR_INVALID_ARGUMENT, "unknown filter kind");

    const uint64_t S_ = P.n_samples, SL = P.n_samples * (uint64_t)nl;
    const uint64_t npx = (uint64_t)(P.fx1 - P.fx0) * (uint64_t)(P.fy1 - P.fy0);
    const bool dev_out = is_device_pointer(rgb_out);
    void *p_rays, *p_hits, *p_img, *p_pixbox, *p_lsamp, *p_contrib, *p_le, *p_L, *p_srays, *p_sslot, *p_occ, *p_cnt, *p_tasks,
        *p_table, *p_rgb = nullptr;
    auto layout = [&](Carve& c) {
        p_rays = c.take(S_ * sizeof(PbrtRay));
        p_hits = c.take(S_ * 16);
        p_img = c.take(S_ * 8);
        p_pixbox = c.take((uint64_t)P.n_pixels * 16);
        p_lsamp = c.take(S_ * 3 * nl * 4 + 4);
        p_contrib = c.take(SL * 16 + 16);
        p_le = c.take(S_ * 16);
        p_L = c.take(S_ * 16);
        p_srays = c.take(SL * sizeof(PbrtRay) + 32);
        p_sslot = c.take(SL * 4 + 4);
        p_occ = c.take(SL + 1);
        p_cnt = c.take(64);
        p_tasks = c.take(smp->num_tasks * sizeof(TaskRec));
        p_table = c.take(sizeof(table));
        if (!dev_out) p_rgb = c.take(npx * 3 * 4);
    };
    Carve probe{nullptr, 0};
    layout(probe);
    if (probe.off > kNoAllocScratchBytes)
        return set_error(PBRT_ERR_BUDGET, "this frame needs " + std::to_string(probe.off) +
                                              " bytes of scratch; pbrtgpu_render_noalloc has " +
                                              std::to_string(kNoAllocScratchBytes) +
                                              " (render it with pbrtgpu_render, or fewer samples or pixels)");
    Carve real{base, 0};
    layout(real);

    // The scratch keeps the previous call's contents: the counters must
    // start at zero; every other buffer is written before it is read.
    if ((st = cuda_status(cudaMemsetAsync(p_cnt, 0, 64, s), "counters")) ||
        (st = cuda_status(cudaMemcpyAsync(p_tasks, tasks, smp->num_tasks * sizeof(TaskRec), cudaMemcpyHostToDevice, s),
                          "tasks H2D")) ||
        (st = cuda_status(cudaMemcpyAsync(p_table, table, sizeof(table), cudaMemcpyHostToDevice, s), "table H2D")))
        return st;
    P.filter_table = (const float*)p_table;
    P.tasks = (const TaskRec*)p_tasks;
    P.n_tasks = smp->num_tasks;
    scene_params(S, &P);
    P.rays = (PbrtRay*)p_rays;
    P.hits = (float4*)p_hits;
    P.img = (float2*)p_img;
    P.pixbox = (float4*)p_pixbox;
    P.lsamp = (float*)p_lsamp;
    P.contrib = (float4*)p_contrib;
    P.le = (float4*)p_le;
    P.L = (float4*)p_L;
    P.shadow_rays = (PbrtRay*)p_srays;
    P.shadow_slot = (uint32_t*)p_sslot;
    P.counters = (uint32_t*)p_cnt;
    P.occluded = (uint8_t*)p_occ;
    P.rgb = dev_out ? rgb_out : (float*)p_rgb;
    if ((st = cuda_status(launch_render(P, s), "render launch"))) return st;
    if (!dev_out &&
        (st = cuda_status(cudaMemcpyAsync(rgb_out, p_rgb, npx * 3 * 4, cudaMemcpyDeviceToHost, s), "rgb D2H")))
        return st;
    uint32_t cnt[4] = {0, 0, 0, 0};
    if ((st = cuda_status(cudaMemcpyAsync(cnt, p_cnt, sizeof(cnt), cudaMemcpyDeviceToHost, s), "counters")))
        return st;
    if ((st = cuda_status(cudaStreamSynchronize(s), "cudaStreamSynchronize"))) return st;
    if (cnt[2]) return set_error((int)cnt[2], "device-side traversal failure");
    if (cnt[1])
        return set_error(PBRT_ERR_NAN, std::to_string(cnt[1]) + " radiance samples were NaN (sampler_renderer.rs:105)");
    return PBRT_OK;
}
