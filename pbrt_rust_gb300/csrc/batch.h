// batch.h - records of the batched multi-scene wavefront (host + device).
//
// A batch holds up to max_jobs jobs: renders (a scene, camera and sampler,
// exactly what pbrtgpu_render takes) and ray queries (closest or any hit of
// a ray array against one BVH).  Every stage of the wavefront is one launch
// over the items of all jobs at once - sampler pixels, rays, samples,
// shadow rays, film pixels - laid end to end in job order; an item finds its
// job by a binary search over the stage's prefix offsets.  The traversal
// stages are persistent kernels fed by a device work counter, so the grid of
// every launch is fixed by the device, not by the batch, and one captured
// CUDA graph replays any batch that fits the buffers.
#pragma once
#include <stdint.h>

#include "render_types.h"

namespace pbrt {

enum { kJobRender = 0, kJobQuery = 1 };

struct JobRec {
    RenderParams P;        // renders: everything; queries: the BVH fields only
    const float4* rays;    // extend input (renders: P.rays)
    float4* hits;          // closest-hit output (renders: P.hits), or nullptr
    uint8_t* occ;          // any-hit output, or nullptr
    uint32_t kind;
    uint32_t any;          // query: any hit
    uint32_t wide;         // trace this job over its 4-wide layout
    uint32_t pad;
};

// Counts of the current batch, written by the host before each launch.
struct BatchHdr {
    uint32_t n_jobs;
    uint32_t pad;
    uint64_t pix, rays, samples, film;  // totals of the prefix offsets below
};

// Device buffer counters (uint32 each).
enum {
    kCtrShadowCount = 0,  // shadow rays queued by shade
    kCtrExtendWork = 1,   // work counter of the extend kernel
    kCtrShadowWork = 2,   // work counter of the shadow kernel
    kCtrReplay = 3,       // some closest hit needs the exact replay (Traversal in trace.cuh)
    kCtrWords = 8         // counters per slot; slot 0 = batch, slot j+1 = job j
};

// Fixed device addresses of one batch: kernel arguments of every stage.
struct BatchArgs {
    const BatchHdr* hdr;
    const JobRec* jobs;
    const uint64_t* off_pix;    // n_jobs + 1 prefix offsets: sampler pixels
    const uint64_t* off_ray;    //   extend rays (render samples + query rays)
    const uint64_t* off_smp;    //   render samples (shade, combine)
    const uint64_t* off_film;   //   film pixels
    PbrtRay* q_rays;            // shadow queue (all jobs)
    uint32_t* q_slot;           //   (sample, light) slot inside the job
    uint32_t* q_job;            //   job of the entry
    uint32_t* counters;         // kCtrWords * (max_jobs + 1)
    uint32_t chunk;             // rays a warp takes from a work counter at a time
    uint32_t refill;            // extend: refill a warp when this many lanes are idle
    uint32_t refill_shadow;     // shadow: same
    uint32_t pad;
};

// Stage launch choices (the autotuner's search space).
struct BatchTuning {
    int extend_wide;    // 4-wide layout for extend (else binary pairs)
    int shadow_wide;    // 4-wide layout for shadow rays
    int block;          // 128 or 256 threads per block
    int smax;           // 4-wide kernels: shared-memory stack entries (8 or 16)
    uint32_t chunk;
    uint32_t refill;
    uint32_t refill_shadow;
};

// Enqueues every stage of the batch on `s`, starting with zeroing the
// counter_bytes of A.counters.  mixed: some query job wants any hit (the
// extend kernel then decides per job).  inst: some job's scene has
// instances (the binary layout with nested instance traversal is used).
// cover_pair / cover_wide: the stack size the jobs need (64 or 256
// entries).  *launches gets the number of
// kernels launched.  A traversal failure of job j goes to
// jobs[j].P.counters[2] (PbrtStatus, max over its rays).
cudaError_t launch_batch_stages(const BatchArgs& A, const BatchTuning& T, bool mixed, bool inst, uint32_t cover_pair,
                                uint32_t cover_wide, int sms, size_t counter_bytes, cudaStream_t s, int* launches);

}  // namespace pbrt
