// capi_internal.h - handle types and helpers shared by the C ABI files.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/pbrt_gpu.h"
#include "host_scene.h"
#include "trace.cuh"
#include "trace4.cuh"
#include "render_types.h"

namespace pbrt {

int set_error(int status, const std::string& msg);
int cuda_status(cudaError_t e, const char* what);
bool is_device_pointer(const void* p);
bool cuda_device_present();

// Grow-only device allocation reused across calls.
struct DeviceBuf {
    void* p = nullptr;
    size_t cap = 0;
    int reserve(size_t bytes);
    void release();
};

// Makes `dev` current for the scope and restores the caller's device.
struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev);
    ~DeviceGuard();
};

}  // namespace pbrt

struct PbrtBVH {
    pbrt::HostBVH host;
    int device = 0;
    pbrt::NodePair* d_pairs = nullptr;
    pbrt::PrimRec* d_prims = nullptr;
    pbrt::SphereRec* d_spheres = nullptr;
    pbrt::Node4* d_nodes4 = nullptr;
    pbrt::DevBVH4* d_insts = nullptr;    // per instance definition
    std::vector<void*> d_inst_bufs;      // the definitions' device arrays
    std::vector<pbrt::DevBVH4> inst_dev;  // host copy of d_insts
    int* d_status = nullptr;
    pbrt::DevBVH dev{};
    pbrt::DevBVH4 dev4{};
    std::mutex stage_mu;
    std::mutex upload_mu;
    std::atomic<bool> uploaded{false};  // device copy made by the first call that needs it
    pbrt::DeviceBuf stage_in, stage_out;
    cudaStream_t pipe_in = nullptr, pipe_out = nullptr, pipe_k = nullptr;  // pipelined host-buffer calls
    cudaEvent_t pipe_ev[17] = {};                        // entry + 2 per chunk (8 chunks)
    uint32_t* d_ready = nullptr;  // streamed input: a flag per piece
    uint32_t* h_one = nullptr;    // pinned host word holding 1, copied into a flag
    ~PbrtBVH();
};

namespace pbrt {
int bvh_upload(PbrtBVH* b);
const DevBVH4* wide_of(const PbrtBVH* b);
}

struct PbrtScene {
    PbrtBVH* bvh = nullptr;
    std::vector<pbrt::ShadePrim> shade;
    std::vector<float4> materials;
    std::vector<pbrt::LightRec> lights;
    std::vector<pbrt::AreaTri> area_tris;
    std::vector<float> area_cdf;
    std::vector<std::vector<pbrt::ShadePrim>> inst_shade;  // per instance definition
    std::vector<uint4> inst_map;                           // RenderParams::inst_map
    std::vector<void*> d_inst_bufs;
    uint4* d_inst_map = nullptr;
    pbrt::InstShade* d_inst_defs = nullptr;
    pbrt::ShadePrim* d_shade = nullptr;
    float4* d_materials = nullptr;
    pbrt::LightRec* d_lights = nullptr;
    pbrt::AreaTri* d_area_tris = nullptr;
    float* d_area_cdf = nullptr;
    std::atomic<bool> uploaded{false};
    std::mutex mu;  // serialises renders: they share the scratch buffers below
    pbrt::DeviceBuf rays, hits, img, pixbox, lsamp, contrib, le, L, srays, sslot, occ, counters, tasks, table, rgb;
    ~PbrtScene() {
        if (bvh) delete bvh;
        for (void* p : {(void*)d_shade, (void*)d_materials, (void*)d_lights, (void*)d_area_tris, (void*)d_area_cdf,
                        (void*)d_inst_map, (void*)d_inst_defs})
            if (p) cudaFree(p);
        for (void* p : d_inst_bufs) cudaFree(p);
        for (pbrt::DeviceBuf* b : {&rays, &hits, &img, &pixbox, &lsamp, &contrib, &le, &L, &srays, &sslot, &occ, &counters,
                                   &tasks, &table, &rgb})
            b->release();
    }
};

namespace pbrt {
// Validates a render's descriptors, uploads the scene on first use and fills
// every field of *out except the filter table, the task array and the
// per-render buffers (capi_render.cu).
int prepare_render(PbrtScene* S, const PbrtCameraDesc* cam, const PbrtSamplerDesc* smp, uint32_t task_lo,
                   uint32_t task_hi, RenderParams* out, std::vector<TaskRec>* tasks);
// The scene's fields of RenderParams (BVH layouts, shading tables, lights,
// instances); the scene is uploaded (capi_render.cu).
void scene_params(const PbrtScene* S, RenderParams* P);
// Render set-up helpers (capi_render.cu), the reference's f32 arithmetic.
int32_t f2i32(float f);
size_t f2usize(float f);
void crop_window(size_t num, size_t count, float aspect, float out[4]);
void gather_offsets(float filter_width, int32_t sampler_start, int32_t sampler_end, int32_t* lo, int32_t* hi);
void sub_window(const PbrtSamplerDesc& s, size_t num, int32_t out[4]);
void film_extent(uint32_t xres, uint32_t yres, const float crop[4], int32_t ext[4]);
void chacha_key(uint64_t state, uint32_t key[8]);
// Pixels and samples of the sampler's window, refused with
// PBRT_ERR_INVALID_ARGUMENT when the window is empty, a side exceeds
// INT32_MAX, or the pixels or (samples x lights) exceed the 32-bit ray and
// shadow-queue indices (capi_render.cu).
int sampler_counts(const PbrtSamplerDesc* smp, uint32_t spp, uint32_t n_lights, uint32_t* n_pixels,
                   uint64_t* n_samples);
// Resolves the no-allocation render's scratch on `dev` (the current device),
// which loads its 64 MiB array there; called when a scene is uploaded so the
// array is in place before any render (capi_noalloc.cu).
int noalloc_prepare(int dev);
}
