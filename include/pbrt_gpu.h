/*
 * pbrt_gpu.h - C ABI of the GB300 (sm_103a) implementation of pbrt_rust's
 * data-parallel hot path: BVH traversal with triangle/sphere tests
 * (closest hit and any hit), camera-ray generation from the stratified
 * sampler, and the direct-lighting Li with shadow rays.
 *
 * Every entry point is plain C: pointers, sizes and an int status
 * (0 == PBRT_OK).  No exception and no C++ or torch type crosses it.
 * Handles are opaque.  A handle may be used from several host threads as
 * long as every thread passes its own CUDA stream.
 *
 * Citations are to the reference crate (Mokosha/pbrt_rust), path:line.
 */
#ifndef PBRT_GPU_H
#define PBRT_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PBRT_GPU_ABI_VERSION 2

/* Status codes.  The reference signals failures with panic!/assert!
 * (e.g. src/primitive/aggregates/bvh.rs:237-238); here they come back as
 * codes and pbrtgpu_last_error() gives the detail. */
typedef enum PbrtStatus {
    PBRT_OK = 0,
    PBRT_ERR_INVALID_ARGUMENT = 1,
    PBRT_ERR_CUDA = 2,
    PBRT_ERR_OUT_OF_MEMORY = 3,
    PBRT_ERR_UNSUPPORTED = 4,
    PBRT_ERR_BUILD = 5,          /* a BVH build invariant failed (bvh.rs:237-238) */
    PBRT_ERR_STACK_OVERFLOW = 6, /* traversal stack too small for the tree depth */
    PBRT_ERR_BUDGET = 7,         /* admission refused: device-memory budget */
    PBRT_ERR_TIMEOUT = 8,        /* a bounded device-side wait ran out */
    PBRT_ERR_NAN = 9,            /* a radiance sample was NaN (sampler_renderer.rs:105) */
    PBRT_ERR_NO_DEVICE = 10,
    PBRT_ERR_CANCELLED = 11
} PbrtStatus;

/* Ray: 32 bytes.  Mirrors src/ray.rs:8-15 (o, d, mint, maxt); time and
 * depth are not needed by traversal. */
typedef struct PbrtRay {
    float ox, oy, oz, tmin;
    float dx, dy, dz, tmax;
} PbrtRay;

/* Closest hit: 16 bytes.  prim = index of the primitive in the fully
 * refined input list (every mesh expands to its triangles in index order,
 * src/shape/mesh.rs:325-335 + src/primitive/mod.rs:47-63), -1 on a miss.
 * For triangles b1/b2 are the barycentrics of src/shape/mesh.rs:41-72;
 * for spheres both are 0.  With instances (PBRT_SHAPE_INSTANCE) each
 * instance takes as many indices as its definition has refined
 * primitives, so prim = the instance's first index + the hit primitive's
 * refined index inside the definition: the indices the same scene would
 * give with every instance copied out. */
typedef struct PbrtHit {
    int32_t prim;
    float t;
    float b1;
    float b2;
} PbrtHit;

/* The reference Transform {m, m_inv} (src/transform/transform.rs:14-19),
 * row-major 4x4 matrices. */
typedef struct PbrtTransform {
    float m[16];
    float m_inv[16];
} PbrtTransform;

enum {
    PBRT_SHAPE_TRIANGLE_MESH = 0,
    PBRT_SHAPE_SPHERE = 1,
    PBRT_SHAPE_DISK = 2,
    PBRT_SHAPE_CYLINDER = 3,
    PBRT_SHAPE_INSTANCE = 4 /* TransformedPrimitive (src/primitive/transformed.rs:14-59) */
};
enum { PBRT_SPLIT_SAH = 0, PBRT_SPLIT_MIDDLE = 1, PBRT_SPLIT_EQUAL = 2 };

/* One input primitive.  Mirrors Shape::triangle_mesh and Shape::sphere
 * (src/shape/mod.rs:170-190) wrapped by Primitive::geometric
 * (src/primitive/mod.rs:87-99).  world_to_object is taken as the
 * inverse of object_to_world, i.e. Transform{m_inv, m}. */
typedef struct PbrtShapeDesc {
    int32_t kind;                 /* PBRT_SHAPE_* */
    int32_t reverse_orientation;
    PbrtTransform object_to_world;
    /* triangle mesh (object space; transformed to world at creation,
     * src/shape/mesh.rs:299-314) */
    const float* points;          /* 3 * n_points floats */
    uint32_t n_points;
    const uint32_t* indices;      /* n_indices, a multiple of 3 */
    uint32_t n_indices;
    /* sphere (src/shape/sphere.rs:28-44): radius, z0, z1, phi_max_deg;
     * cylinder (src/shape/cylinder.rs:26-36): radius, z0, z1, phi_max_deg;
     * disk (src/shape/disk.rs:24-34): height, radius, inner_radius,
     * phi_max_deg */
    float radius, z0, z1, phi_max_deg;
    float height, inner_radius;
    /* instance: index into PbrtSceneDesc.instances; object_to_world places
     * the definition in the world (its inverse is the world-to-primitive
     * transform of TransformedPrimitive) */
    int32_t instance;
    /* render-only */
    int32_t material;             /* index into PbrtSceneDesc.materials */
    int32_t area_light;           /* index into PbrtSceneDesc.lights or -1 */
} PbrtShapeDesc;

/* Matte material (src/material/matte.rs:30-51) with constant textures:
 * Lambertian (src/bsdf/lambertian.rs) or Oren-Nayar (src/bsdf/orennayar.rs). */
typedef struct PbrtMaterialDesc {
    float kd[3];
    float sigma;                  /* degrees, clamped to [0, 90]: 0 = Lambertian, else Oren-Nayar */
} PbrtMaterialDesc;

enum { PBRT_LIGHT_POINT = 0, PBRT_LIGHT_DIFFUSE_AREA = 1 };

/* Point light (src/light/point.rs:16-35) or a diffuse area light over the
 * triangles of one mesh shape (src/area_light.rs is a stub in the
 * reference; this follows pbrt-v2's DiffuseAreaLight). */
typedef struct PbrtLightDesc {
    int32_t kind;                 /* PBRT_LIGHT_* */
    PbrtTransform light_to_world; /* point: position = light_to_world(0,0,0) */
    float spectrum[3];            /* point: intensity; area: emitted radiance */
    int32_t shape;                /* area: index of the emitting mesh shape */
} PbrtLightDesc;

/* One object definition (ObjectBegin ... ObjectEnd): its shapes in
 * instance space, materials indexing the scene's table.  Definitions hold
 * no instances and no area lights.  Every PBRT_SHAPE_INSTANCE shape of the
 * scene is one primitive of the scene's BVH whose own BVH over the
 * definition is shared by all its instances. */
typedef struct PbrtInstanceDesc {
    const PbrtShapeDesc* shapes;
    uint32_t n_shapes;
} PbrtInstanceDesc;

typedef struct PbrtSceneDesc {
    const PbrtShapeDesc* shapes;
    uint32_t n_shapes;
    const PbrtMaterialDesc* materials;
    uint32_t n_materials;
    const PbrtLightDesc* lights;
    uint32_t n_lights;
    uint32_t max_prims_in_node;   /* BVHAccelerator::new mp (bvh.rs:335) */
    int32_t split_method;         /* PBRT_SPLIT_* */
    uint32_t build_flags;         /* PBRT_BUILD_* */
    const PbrtInstanceDesc* instances;
    uint32_t n_instances;
} PbrtSceneDesc;

/* Build flags.  PBRT_BUILD_ON_DEVICE: the BVH tree (bvh.rs:86-258) is built
 * by CUDA kernels instead of on the host; same nodes and primitive order
 * (bit for bit where the host's fmin/fmax order -0 below +0, as on Arm; on
 * x86 hosts the sign of a zero bound may differ).  The equal-counts split
 * method stays on the host. */
enum { PBRT_BUILD_ON_DEVICE = 1 };

/* Perspective camera (src/camera/mod.rs:105-135) with an image film
 * (src/camera/film.rs:77-122) and a box filter (src/filter.rs:45-50). */
typedef struct PbrtCameraDesc {
    PbrtTransform camera_to_world; /* static: AnimatedTransform of equal ends */
    float fov_deg;
    float screen_window[4];
    float lens_radius, focal_distance;
    float shutter_open, shutter_close;
    uint32_t x_res, y_res;
    float crop_window[4];
    float filter_x_width, filter_y_width;
    /* Filter of the film (src/filter.rs:44-85): PBRT_FILTER_*, with
     * p0 = alpha (gaussian), B (mitchell) or tau (lanczos) and
     * p1 = C (mitchell). */
    int32_t filter_kind;
    float filter_p0, filter_p1;
} PbrtCameraDesc;

enum {
    PBRT_FILTER_BOX = 0,      /* Filter::mean */
    PBRT_FILTER_TRIANGLE = 1,
    PBRT_FILTER_GAUSSIAN = 2,
    PBRT_FILTER_MITCHELL = 3,
    PBRT_FILTER_LANCZOS = 4
};

/* Stratified sampler (src/sampler/stratified.rs:23-37) and the task count
 * of SamplerRenderer (src/sampler_renderer.rs:39-44), given explicitly so
 * the random streams do not depend on the host's core count. */
typedef struct PbrtSamplerDesc {
    int32_t x_start, x_end, y_start, y_end;
    uint32_t x_samples, y_samples;
    int32_t jitter;
    float shutter_open, shutter_close;
    uint32_t num_tasks;
} PbrtSamplerDesc;

/* One node of the reference's linearised BVH (PackedBVHNode,
 * src/primitive/aggregates/bvh.rs:260-326), exported for inspection. */
typedef struct PbrtPackedNode {
    float lo[3];
    float hi[3];
    int32_t is_leaf;
    uint32_t offset;     /* leaf: prim_offset; inner: second_child_offset */
    uint32_t count;      /* leaf: num_prims; inner: split axis */
} PbrtPackedNode;

typedef struct PbrtBVH PbrtBVH;
typedef struct PbrtScene PbrtScene;

/* ---- library ---------------------------------------------------------- */

int pbrtgpu_abi_version(void);
const char* pbrtgpu_status_str(int status);
/* Detail of the last failing call on this host thread ("" if none). */
const char* pbrtgpu_last_error(void);

/* ---- aggregate: the GpuBVHAccel drop-in ------------------------------- */

/* Replaces BVHAccelerator::new(p, mp, sm)
 * (src/primitive/aggregates/bvh.rs:334-363) and Aggregate::bvh
 * (src/primitive/aggregates/mod.rs:27-29).  The primitives are fully
 * refined, the SAH/middle/equal tree is built on the host with the
 * reference's arithmetic and flattened.
 * An unknown split_method falls back to "sah" with a warning, as
 * bvh.rs:341-349 does.  When a CUDA device is present the device copy is
 * made here, on the current device; otherwise the first call that needs
 * it makes it. */
int pbrtgpu_bvh_create(const PbrtShapeDesc* shapes, uint32_t n_shapes,
                       uint32_t max_prims_in_node, const char* split_method,
                       PbrtBVH** out);
/* pbrtgpu_bvh_create with PBRT_BUILD_* flags (no counterpart in the
 * reference). */
int pbrtgpu_bvh_create_ex(const PbrtShapeDesc* shapes, uint32_t n_shapes, uint32_t max_prims,
                          const char* split_method, uint32_t flags, PbrtBVH** out);
/* The aggregate of a scene description's shapes, instances included
 * (BVHAccelerator::new over primitives some of which are
 * TransformedPrimitive, src/primitive/transformed.rs:14-73); uses
 * max_prims_in_node, split_method, build_flags and the instance
 * definitions, ignores materials and lights. */
int pbrtgpu_bvh_create_desc(const PbrtSceneDesc* desc, PbrtBVH** out);
void pbrtgpu_bvh_destroy(PbrtBVH* bvh);

/* Replaces HasBounds::world_bound for BVHAccelerator (bvh.rs:365-373). */
int pbrtgpu_bvh_world_bound(const PbrtBVH* bvh, float lo[3], float hi[3]);
int pbrtgpu_bvh_num_primitives(const PbrtBVH* bvh, uint32_t* n);
/* Device memory the aggregate keeps resident (node layouts, primitive and
 * analytic records, instance definitions); no counterpart in the
 * reference. */
int pbrtgpu_bvh_device_bytes(const PbrtBVH* bvh, uint64_t* bytes);
int pbrtgpu_bvh_num_nodes(const PbrtBVH* bvh, uint32_t* n);
int pbrtgpu_bvh_depth(const PbrtBVH* bvh, uint32_t* depth);
/* The reference-order linearised nodes (bvh.rs:319-325). */
int pbrtgpu_bvh_get_nodes(const PbrtBVH* bvh, PbrtPackedNode* out,
                          uint32_t capacity);
/* ordered_prims of bvh.rs:356: out[i] = input index of the i-th primitive. */
int pbrtgpu_bvh_get_primitive_order(const PbrtBVH* bvh, uint32_t* out,
                                    uint32_t capacity);

/* Replaces Intersectable::intersect for the BVH (bvh.rs:375-422) over a
 * batch of rays: closest hit per ray.  rays/hits may be device pointers
 * or host pointers (pinned or pageable).  Host buffers take one of three
 * forms, all with the same results:
 *  - streamed (default for rays in pinned memory, 2^17 rays or more, the
 *    default traversal kernel): the traversal on `stream` starts at once
 *    and the rays follow in pieces on the handle's copy stream, each warp
 *    waiting for the piece it takes (see pbrtgpu_intersect_streamed; a
 *    walk whose pieces do not come within 50 ms + 2 ns per ray, e.g. under
 *    a profiler that serialises work, is redone over the staged rays);
 *    closest hits go straight to device memory or are written to pinned
 *    host memory by the walk, any-hit answers to host memory through one
 *    copy.  PBRT_STREAM_IN=0 turns it off;
 *  - in place (PBRT_HOST_MAPPED=1, pinned buffers): the traversal reads and
 *    writes the mapped host memory;
 *  - pipelined (every other host buffer): copies in and out and the
 *    traversal in PBRT_PIPE_CHUNKS (default 4) pieces on the handle's own
 *    streams, for 2^19 rays or more, each piece's copies overlapping the
 *    others' traversal.
 * The call returns after the work is queued for device buffers and after
 * completion for host buffers.  `stream` is a cudaStream_t (NULL = legacy
 * default stream). */
int pbrtgpu_intersect(const PbrtBVH* bvh, const PbrtRay* rays, uint32_t n,
                      PbrtHit* hits, void* stream);

/* Replaces Intersectable::intersect_p (src/intersection.rs:61-66) for the
 * BVH: occluded[i] = 1 if any primitive is hit within [tmin, tmax]. */
int pbrtgpu_intersect_p(const PbrtBVH* bvh, const PbrtRay* rays, uint32_t n,
                        uint8_t* occluded, void* stream);

/* Closest hits (hits non-NULL) or any-hit answers (occluded non-NULL),
 * device buffers only, for rays that arrive while the walk runs: piece k,
 * rays [k << piece_shift, (k + 1) << piece_shift), may be read once
 * ready[k] != 0 (ready: device memory, one uint32 per piece).  Set each
 * flag with a copy queued behind its piece's copy on another stream
 * (cudaMemcpyAsync of a non-zero word), never from a kernel: the walk may
 * hold every SM until the flags are set.  piece_shift in [5, 31].  Needs the 4-wide persistent walk
 * with its work counter (the default configuration; PBRT_ERR_UNSUPPORTED
 * otherwise).  Returns after the walk; a piece whose flag is not set within
 * 2 s ends the call with PBRT_ERR_TIMEOUT and its rays get no result.  The
 * streamed form of pbrtgpu_intersect is this call with the library setting
 * the flags behind its own copies.  No counterpart in the reference. */
int pbrtgpu_intersect_streamed(const PbrtBVH* bvh, const PbrtRay* rays,
                               uint32_t n, PbrtHit* hits, uint8_t* occluded,
                               const uint32_t* ready, uint32_t piece_shift,
                               void* stream);

/* Traversal kernel choice (process-wide), set by the autotuner.  Every
 * kernel visits the reference's tree in the reference's order, so results
 * do not depend on the choice.  The first value is also read from the
 * environment (PBRT_TRACE_KERNEL = plain | pt | w4 | w4pt | w4spec | packet,
 * PBRT_TRACE_REFILL = 1..32, PBRT_TRACE_MINB = 0 | 8 | 9,
 * PBRT_RENDER_KERNEL = plain | w4 | packet, PBRT_TRACE_REORDER = 0 | 1,
 * PBRT_TRACE_CHUNK = 0 | 32..4096) when no call has set it. */
enum {
    PBRT_TRACE_PAIR = 0,            /* binary pairs, one thread per ray */
    PBRT_TRACE_PAIR_PERSISTENT = 1, /* binary pairs, persistent warps */
    PBRT_TRACE_WIDE = 2,            /* 4-wide nodes, one thread per ray */
    PBRT_TRACE_WIDE_PERSISTENT = 3, /* 4-wide nodes, persistent warps */
    PBRT_TRACE_WIDE_SPECULATIVE = 4, /* 4-wide nodes, persistent warps, leaves tested in warp-wide rounds */
    PBRT_TRACE_PAIR_PACKET = 5       /* binary pairs, one thread per ray; a warp whose rays share their
                                        direction signs walks them together, node by node, each lane
                                        testing what its own walk tests (coherent rays) */
};
typedef struct PbrtTraceConfig {
    int32_t kernel;         /* PBRT_TRACE_*: pbrtgpu_intersect / intersect_p batches */
    uint32_t refill;        /* persistent kernels: refill a warp when this many lanes idle */
    uint32_t min_blocks;    /* 4-wide persistent kernel: 0, or 7 / 8 / 9 resident 128-thread
                               blocks per SM requested (fewer registers per thread) */
    int32_t render_kernel;  /* PBRT_TRACE_*: camera rays inside pbrtgpu_render; shadow
                               rays take the 4-wide kernel with a 4-wide choice, else
                               the binary one */
    uint32_t reorder;       /* 1: pbrtgpu_intersect / intersect_p batches of 32768 rays
                               or more are binned by direction and origin before
                               traversal (same results, more coherent warps) */
    uint32_t chunk;         /* 4-wide persistent kernel: 0 = each warp owns a fixed
                               range of the batch; 32..4096 (a multiple of 32) = warps
                               take this many rays at a time from a shared counter */
} PbrtTraceConfig;
int pbrtgpu_set_trace_config(const PbrtTraceConfig* cfg);
int pbrtgpu_get_trace_config(PbrtTraceConfig* cfg);

/* ---- renderer: the GpuSamplerRenderer drop-in ------------------------- */

/* Builds the aggregate plus the device copies of materials and lights
 * (Scene::new_with, src/scene.rs:31-39); device residency as for
 * pbrtgpu_bvh_create. */
int pbrtgpu_scene_create(const PbrtSceneDesc* desc, PbrtScene** out);
void pbrtgpu_scene_destroy(PbrtScene* scene);
/* Device bytes a scene holds: its BVH's (pbrtgpu_bvh_device_bytes) plus its
 * shading tables, lights and instance records; per-render scratch not
 * included. */
int pbrtgpu_scene_device_bytes(const PbrtScene* scene, uint64_t* bytes);
/* The scene's aggregate, usable with pbrtgpu_intersect*. */
int pbrtgpu_scene_bvh(const PbrtScene* scene, const PbrtBVH** out);

/* Replaces Renderer::render for SamplerRenderer
 * (src/sampler_renderer.rs:147-182, run_task :61-144, li :184-206) as a
 * wavefront: generate -> extend -> shade -> shadow -> accumulate.
 * rgb_out receives the film's pixel extent (film.rs:301-309) as linear
 * float RGB, 3 floats per pixel, row-major; host or device pointer. */
int pbrtgpu_render(const PbrtScene* scene, const PbrtCameraDesc* camera,
                   const PbrtSamplerDesc* sampler, float* rgb_out,
                   void* stream);

/* Renders only tasks [task_lo, task_hi) of the sampler's task split
 * (sampler_renderer.rs:39-75): pixels owned by other tasks come out +0, and
 * every other pixel equals pbrtgpu_render's, so the sum of the images of
 * disjoint task ranges covering [0, num_tasks) is pbrtgpu_render's image bit
 * for bit.  One range per device or process shards a frame with no exchange
 * but that sum.  No counterpart in the reference: SamplerRenderer::render
 * (sampler_renderer.rs:146-176) runs all tasks of a frame in one process.
 * PBRT_ERR_INVALID_ARGUMENT unless task_lo <= task_hi <= num_tasks. */
int pbrtgpu_render_tasks(const PbrtScene* scene, const PbrtCameraDesc* camera, const PbrtSamplerDesc* sampler,
                         uint32_t task_lo, uint32_t task_hi, float* rgb_out, void* stream);

/* pbrtgpu_render without any device allocation.  This entry point has no
 * counterpart in the reference.  It is for callers that cannot allocate
 * device memory while rendering: a serving process that reserves its
 * memory up front and admits work against that fixed budget, or a frame
 * loop that cannot afford the device-wide synchronisation cudaMalloc and
 * cudaFree may cause.  Its scratch is one static array of 64 MiB of device
 * memory, present on every GPU where the library's code is loaded until the
 * process exits; a frame needing more (about 220 bytes per sample with two
 * lights, e.g. 256x256 at 4 spp) is refused with PBRT_ERR_BUDGET, and
 * num_tasks is limited to 256; windows beyond 2^32 - 1 pixels or
 * samples x lights are refused with PBRT_ERR_INVALID_ARGUMENT.  The scene
 * must have its device copy (pbrtgpu_scene_create makes it when a device is
 * present).  Set-up happens when a scene is uploaded to a device: the
 * scratch's device address is looked up there, which also places the
 * 64 MiB array on that device; should that fail, the first call on the
 * device does it, so make that first call before any stream capture.  The
 * address is looked up again after the device's context has been reset.
 * Under CUDA's lazy module loading the render kernels' code is loaded by
 * their first launch, as for any kernel: a caller that budgets device
 * memory strictly makes one call (or one pbrtgpu_render) before its
 * budgeted phase.  All calls share the one scratch array, which keeps the
 * previous call's contents: calls that overlap on the GPU (other streams,
 * other threads) race and must be serialised by the caller.  Results equal
 * pbrtgpu_render's bit for bit. */
int pbrtgpu_render_noalloc(const PbrtScene* scene, const PbrtCameraDesc* camera,
                           const PbrtSamplerDesc* sampler, float* rgb_out,
                           void* stream);

/* ---- batched multi-scene wavefront -----------------------------------
 * No counterpart in the reference: SamplerRenderer::render
 * (sampler_renderer.rs:146-176) renders one scene per call and
 * BVHAccelerator::intersect (bvh.rs:375-422) answers one ray per call.  A
 * batch collects many render jobs (what pbrtgpu_render takes) and ray-query
 * jobs (what pbrtgpu_intersect / intersect_p take) over any number of
 * scenes and runs them together: each stage of the wavefront is one launch
 * over the items of every job, the traversal stages are persistent kernels
 * fed by a device work counter, and the launch sequence is replayed as one
 * CUDA graph.  Every job's output equals what the single-job entry point
 * gives for it (bit for bit).
 *
 * Life cycle: create (all device and pinned memory is allocated here, sized
 * by the limits; pbrtgpu_batch_bytes tells the device bytes up front) ->
 * add jobs -> launch (asynchronous on the stream) -> wait (copies host
 * outputs, reports per-job status, empties the batch) -> add ... A job that
 * would exceed a limit is refused with PBRT_ERR_BUDGET and the batch stays
 * as it was.  Scenes, BVHs and output buffers must stay valid until wait
 * returns.  One batch is used by one host thread at a time. */
typedef struct PbrtBatchLimits {
    uint32_t max_jobs;          /* render + query jobs per launch */
    uint32_t max_tasks;         /* render tasks over all render jobs */
    uint64_t max_samples;       /* camera samples over all render jobs */
    uint64_t max_light_samples; /* camera samples x lights over all render jobs */
    uint64_t max_film_pixels;   /* film pixels over all render jobs */
    uint64_t max_query_rays;    /* rays of query jobs with host buffers */
} PbrtBatchLimits;

/* Launch choices of a batch (the autotuner's search space).  A new batch
 * starts with 4-wide extend and shadow walks (binary where a job's tree has
 * no 4-wide layout), 128 threads, 16 stack entries, chunk 64, refill 32
 * (extend) / 8 (shadow), graphs on. */
typedef struct PbrtBatchTuning {
    int32_t extend_kernel;  /* PBRT_TRACE_PAIR or PBRT_TRACE_WIDE: camera and query rays */
    int32_t shadow_kernel;  /* PBRT_TRACE_PAIR or PBRT_TRACE_WIDE: shadow rays */
    uint32_t block;         /* threads per block: 128 or 256 */
    uint32_t stack;         /* 4-wide kernels: shared-memory stack entries per ray, 8 or 16 */
    uint32_t chunk;         /* rays a warp takes from the work counter at a time: 32..4096, multiple of 32 */
    uint32_t refill;        /* extend: refill a warp when this many lanes are idle, 1..32;
                               32: each lane walks its ray to the end, no per-step vote */
    uint32_t refill_shadow; /* shadow: same, 1..32 */
    uint32_t use_graph;     /* 1: replay the stage sequence as one CUDA graph */
} PbrtBatchTuning;

typedef struct PbrtBatchStats {
    uint32_t jobs;
    uint32_t kernels;       /* kernels of the last launch */
    uint64_t samples, light_samples, film_pixels, query_rays;
    uint32_t graph;         /* the last launch replayed a graph */
    uint32_t pad;
} PbrtBatchStats;

typedef struct PbrtBatch PbrtBatch;

int pbrtgpu_batch_bytes(const PbrtBatchLimits* limits, uint64_t* device_bytes, uint64_t* pinned_bytes);
int pbrtgpu_batch_create(const PbrtBatchLimits* limits, PbrtBatch** out);
void pbrtgpu_batch_destroy(PbrtBatch* batch);
/* Adds a render; rgb_out as for pbrtgpu_render.  *job (may be NULL) gets its index. */
int pbrtgpu_batch_add_render(PbrtBatch* batch, const PbrtScene* scene, const PbrtCameraDesc* camera,
                             const PbrtSamplerDesc* sampler, float* rgb_out, uint32_t* job);
/* Adds a ray query: closest hits into `hits`, or (hits NULL) any hit into
 * `occluded`; host or device buffers. */
int pbrtgpu_batch_add_query(PbrtBatch* batch, const PbrtBVH* bvh, const PbrtRay* rays, uint32_t n,
                            PbrtHit* hits, uint8_t* occluded, uint32_t* job);
int pbrtgpu_batch_launch(PbrtBatch* batch, void* stream);
/* 1 in *done once the last launch has finished (does not wait). */
int pbrtgpu_batch_poll(PbrtBatch* batch, int32_t* done);
/* Waits for the last launch, finishes host outputs, writes each job's status
 * to job_status[job] (may be NULL) and empties the batch; returns the first
 * failing job's status.  Without a launch since the jobs were added it only
 * empties the batch. */
int pbrtgpu_batch_wait(PbrtBatch* batch, int32_t* job_status);
int pbrtgpu_batch_set_tuning(PbrtBatch* batch, const PbrtBatchTuning* tuning);
int pbrtgpu_batch_get_tuning(const PbrtBatch* batch, PbrtBatchTuning* tuning);
int pbrtgpu_batch_stats(const PbrtBatch* batch, PbrtBatchStats* stats);
/* Times the jobs now in the batch under each candidate tuning (coordinate
 * descent over kernel, block, stack, chunk, refill and graph choices,
 * `repeats` launches each, CUDA events on `stream`), keeps the fastest and
 * returns it with its time.  The jobs stay in the batch; their outputs are
 * written by every trial (with the same values). */
int pbrtgpu_batch_autotune(PbrtBatch* batch, void* stream, uint32_t repeats, PbrtBatchTuning* best,
                           float* best_ms);

/* ---- serving loop ----------------------------------------------------
 * No counterpart in the reference (a one-shot renderer).  A server keeps
 * scenes resident (the caller's PbrtScene / PbrtBVH handles), accepts render
 * and ray-query requests from any host thread, and runs them with
 * continuous batching: a worker thread packs the requests waiting in arrival
 * order into the first free batch slot - as many as fit the slot's device
 * memory limits - and launches it at once, so requests that arrive while
 * other batches run on the device are admitted as slots free up, and up to
 * `slots` batches are in flight together (each on its own stream).  A
 * request larger than a slot's limits is refused at submission with
 * PBRT_ERR_BUDGET.  Each result equals what the single-request entry point
 * gives (bit for bit), alone or in any mix.
 *
 * Device-memory pool: with pool_bytes > 0 the server holds its resident
 * scenes and its slots' arenas to that budget.  The slots are charged at
 * creation (PBRT_ERR_BUDGET if they alone exceed it); a scene or BVH
 * becomes resident by pbrtgpu_server_admit, charged its device bytes, and
 * is refused with PBRT_ERR_BUDGET when it would not fit; requests name
 * resident scenes (a render) or resident BVHs, a scene's own BVH included
 * (a query), others are refused at submission.  pool_bytes = 0: no pool
 * accounting and any scene may be named. */
typedef struct PbrtServerConfig {
    uint32_t slots;          /* batches in flight at once, 1..8 */
    uint32_t use_tuning;     /* 1: apply `tuning` to every slot */
    PbrtBatchLimits limits;  /* device memory of each slot (pbrtgpu_batch_bytes) */
    PbrtBatchTuning tuning;
    uint64_t pool_bytes;     /* device budget of resident scenes + slot arenas; 0 = none */
} PbrtServerConfig;

typedef struct PbrtServerStats {
    uint64_t submitted, completed, failed, batches;
    double mean_batch_requests;
    double p50_ms, p99_ms, mean_ms, max_ms;  /* submission to result, completed requests */
    double span_s;                           /* first submission to last result */
    double requests_per_s;                   /* completed / span_s */
    /* pool: budget, bytes of the slot arenas and of the resident scenes and
     * BVHs (and how many), requests that found the free slot full and
     * waited for the next one, requests refused (not resident, larger than
     * a slot, invalid) */
    uint64_t pool_bytes, slot_bytes, resident_bytes, resident_count;
    uint64_t deferred, refused;
} PbrtServerStats;

typedef struct PbrtServer PbrtServer;

int pbrtgpu_server_create(const PbrtServerConfig* config, PbrtServer** out);
/* Makes a scene (and with it its BVH) or a bare BVH resident in the
 * server's pool: exactly one of scene / bvh is non-NULL.  Charged its
 * device bytes (pbrtgpu_scene_device_bytes / pbrtgpu_bvh_device_bytes);
 * PBRT_ERR_BUDGET if the pool cannot hold it.  Admitting a resident handle
 * again changes nothing.  pbrtgpu_server_release takes it out of the pool
 * (its requests must have completed). */
int pbrtgpu_server_admit(PbrtServer* server, const PbrtScene* scene, const PbrtBVH* bvh);
int pbrtgpu_server_release(PbrtServer* server, const PbrtScene* scene, const PbrtBVH* bvh);
/* Finishes every submitted request, then frees the server. */
void pbrtgpu_server_destroy(PbrtServer* server);
/* The camera and sampler descriptions are copied; the scene, rgb_out and
 * (for queries) the rays and outputs must stay valid until the request has
 * completed.  *ticket identifies the request. */
int pbrtgpu_server_submit_render(PbrtServer* server, const PbrtScene* scene, const PbrtCameraDesc* camera,
                                 const PbrtSamplerDesc* sampler, float* rgb_out, uint64_t* ticket);
int pbrtgpu_server_submit_query(PbrtServer* server, const PbrtBVH* bvh, const PbrtRay* rays, uint32_t n,
                                PbrtHit* hits, uint8_t* occluded, uint64_t* ticket);
/* Waits until the request has completed (timeout_s < 0: no limit) and
 * forgets it; *status gets its PbrtStatus.  PBRT_ERR_CANCELLED if the
 * timeout passed first (the request stays queued), PBRT_ERR_INVALID_ARGUMENT
 * for an unknown ticket. */
int pbrtgpu_server_wait(PbrtServer* server, uint64_t ticket, double timeout_s, int32_t* status);
/* Waits until every submitted request has completed. */
int pbrtgpu_server_drain(PbrtServer* server);
int pbrtgpu_server_stats(PbrtServer* server, PbrtServerStats* stats);
/* Forgets the latency record (completed requests stay waitable). */
int pbrtgpu_server_reset_stats(PbrtServer* server);

/* The sampler's random stream on the device (RNG, src/rng.rs:4-33: rand
 * 0.8.5 StdRng = rand_chacha 0.3.1 ChaCha12, seeded by rand_core 0.6.4
 * seed_from_u64), exposed so that it can be checked against other
 * implementations.  pbrtgpu_chacha_blocks: keystream blocks counter ..
 * counter + n_blocks - 1 of the ChaCha state (the four constants, key[8],
 * the 64-bit block counter in words 12-13, the 64-bit stream id in words
 * 14-15) after `rounds` rounds (8, 12 or 20), by the device routine the
 * sampler uses (paired = 1: the two-block routine, n_blocks even); 16
 * words per block into host memory `out`.  StdRng is rounds = 12,
 * stream_id = 0.  pbrtgpu_rng_words: words [first_word, first_word +
 * n_words) of RNG::new(seed)'s u32 stream (rng.rs:11-13) as the render
 * kernels read them, each run of `segment` words from its own seek.  Both
 * synchronous; at most 2^20 blocks / 2^24 words per call. */
int pbrtgpu_chacha_blocks(const uint32_t key[8], uint64_t counter, uint64_t stream_id, uint32_t rounds,
                          uint32_t paired, uint32_t n_blocks, uint32_t* out);
int pbrtgpu_rng_words(uint64_t seed, uint64_t first_word, uint32_t n_words, uint32_t segment, uint32_t* out);

/* The film's 16 x 16 filter table (film.rs:89-97: the filter evaluated at
 * ((i + 0.5) / 16) of its width), row-major by y; the table every render
 * entry point uses for this camera. */
int pbrtgpu_filter_table(const PbrtCameraDesc* camera, float table[256]);

/* Film output (Film::write_image, src/camera/film.rs:316-354, and
 * write_img, film.rs:15-33).  rgb: host memory, width * height RGB triples
 * of linear float as the render entry points return them.  The format
 * follows the file extension: .png / .ppm get 8-bit channels
 * (255 * p^(1/2.2) + 0.5, clamped to [0, 255] and truncated, as write_img
 * computes them), .pfm and .exr (OpenEXR, scanline, uncompressed, 32-bit
 * float B/G/R channels) the linear floats.  pbrtgpu_image_bytes gives those
 * 8-bit values without writing a file. */
int pbrtgpu_write_image(const float* rgb, uint32_t width, uint32_t height, const char* path);
int pbrtgpu_image_bytes(const float* rgb, uint32_t width, uint32_t height, uint8_t* out);

/* Pixel extent (x0, x1, y0, y1) of the film a camera describes
 * (Film::get_pixel_extent, src/camera/film.rs:301-309). */
int pbrtgpu_film_pixel_extent(const PbrtCameraDesc* camera, int32_t ext[4]);

#ifdef __cplusplus
}
#endif

#endif /* PBRT_GPU_H */
