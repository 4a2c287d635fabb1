// render_types.h - records of the render wavefront (host + device).
#pragma once
#include <stdint.h>

#include "../../include/pbrt_gpu.h"
#include "layout.h"
#include "trace.cuh"
#include "trace4.cuh"

namespace pbrt {

// One SamplerRenderer task (src/sampler_renderer.rs:61-144): its sampler
// sub-window (sampler/base.rs:29-48), its sub-film pixel extent
// (camera/film.rs:124-147) and the ChaCha key of RNG::new(task).
struct alignas(16) TaskRec {
    int32_t wx0, wx1, wy0, wy1;
    int32_t fx0, fx1, fy0, fy1;
    uint32_t key[8];
};
static_assert(sizeof(TaskRec) == 64, "task record is 64 bytes");

// Shading data of one refined primitive (indexed by its refined index):
//   a = (p1.xyz, material index bits)
//   b = (p2.xyz, area light index + 1 bits, 0 = not an emitter)
//   c = (p3.xyz, flags bits: bit0 flip normal, bit1 sphere, bits 2.. sphere index)
struct alignas(16) ShadePrim {
    float a[4], b[4], c[4];
};
constexpr uint32_t kShadeFlip = 1u;
constexpr uint32_t kShadeSphere = 2u;

// Shading tables of one instance definition.
struct InstShade {
    const ShadePrim* shade;
    const SphereRec* spheres;
};

enum { kLightPoint = 0, kLightArea = 1 };

struct alignas(16) LightRec {
    uint32_t kind;
    uint32_t tri_first;  // area: first triangle in area_tris
    uint32_t tri_count;
    float area;          // area: total emitting area
    float pos[4];        // point: position; area: pos[3] bits = offset of the CDF in area_cdf
    float spec[4];       // point: intensity; area: emitted radiance
};

// An emitting triangle, vertices in refined order; p1[3] = flip flag.
struct alignas(16) AreaTri {
    float p1[4], p2[4], p3[4];
};

struct RenderParams {
    // camera (camera/mod.rs:168-271)
    float r2c[16];
    float c2w[16];
    float lens_radius, focal_distance;
    // sampler (sampler/stratified.rs:60-127)
    int32_t sx0, sx1, sy0, sy1;
    uint32_t xs, ys, spp, jitter;
    float sopen, sclose;
    uint32_t words_per_pixel;
    uint32_t n_pixels;   // sampler-window pixels
    uint64_t n_samples;
    // film (camera/film.rs)
    int32_t fx0, fx1, fy0, fy1;  // main film pixel extent
    float filter_xw, filter_yw, filter_inv_xw, filter_inv_yw;
    // film pixel p gathers the samples of source pixels p + [g*0, g*1]
    // (gather_offsets in capi_render.cu)
    int32_t gx0, gx1, gy0, gy1;
    const float* filter_table;   // 16 x 16
    // tasks
    const TaskRec* tasks;
    uint32_t n_tasks;
    // scene
    DevBVH bvh;
    uint32_t depth;
    DevBVH4 bvh4;
    uint32_t wide_bound;  // 4-wide stack bound; wide layout used when has_wide
    uint32_t has_wide;
    const ShadePrim* shade;
    const SphereRec* spheres;
    const float4* materials;     // two per material: (kd.rgb clamped >= 0, Oren-Nayar A), (B, oren flag bits, 0, 0)
    const LightRec* lights;
    uint32_t n_lights;
    const AreaTri* area_tris;
    const float* area_cdf;
    // instances (TransformedPrimitive): per instance primitive in id order
    // (first hit id, refined index, definition size, analytic record), and
    // per definition its shading tables; n_inst = 0 without instances
    uint32_t n_inst;
    const uint4* inst_map;
    const InstShade* inst_defs;
    // buffers
    PbrtRay* rays;
    float4* hits;
    float2* img;
    float4* pixbox;     // per sampler pixel: (min x, min y, max x, max y) of its sample positions
    float* lsamp;       // 3 * n_lights floats per sample: components then positions
    float4* contrib;    // per (sample, light): rgb, w = 1 if a shadow ray decides it
    float4* le;         // per sample emitted radiance
    float4* L;          // per sample radiance
    PbrtRay* shadow_rays;
    uint32_t* shadow_slot;
    uint32_t* counters;  // [0] shadow rays, [1] NaN samples, [2] status, [3] replay flag (zero at launch)
    uint8_t* occluded;   // per (sample, light)
    float* rgb;          // film output
};

}  // namespace pbrt
