// capi_internal.h - handle types and helpers shared by the C ABI files.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>
#include <string>

#include "../../include/pbrt_gpu.h"
#include "host_scene.h"
#include "trace.cuh"
#include "trace4.cuh"

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
    int* d_status = nullptr;
    pbrt::DevBVH dev{};
    pbrt::DevBVH4 dev4{};
    std::mutex stage_mu;
    std::mutex upload_mu;
    std::atomic<bool> uploaded{false};  // device copy made by the first call that needs it
    pbrt::DeviceBuf stage_in, stage_out;
    ~PbrtBVH();
};

namespace pbrt {
int bvh_upload(PbrtBVH* b);
const DevBVH4* wide_of(const PbrtBVH* b);
}
