/*
 * oracle.h - TEST INFRASTRUCTURE, not product code.
 *
 * A plain C++ restatement of the reference CPU path of pbrt_rust
 * (Mokosha/pbrt_rust) for BVH build/traversal, triangle and sphere tests,
 * the stratified sampler and its RNG, the perspective camera, the
 * direct-lighting light loop and the film.  Each function in oracle.cpp
 * cites the reference file:line it follows.  It is compiled with
 * -O2 -ffp-contract=off -fno-fast-math so that every f32 operation is the
 * same IEEE operation, in the same order, as rustc emits (rustc never
 * contracts to FMA).
 *
 * Only the tests, the smoke check and the benchmark's CPU-baseline leg
 * load this library; it is the checker, never part of the product path.
 *
 * Parity: the BVH, shape, slab, quadratic, partition, crop-window,
 * sub-window, strata, projection, look_at, film-extent and filter parts
 * are pinned by the reference's own unit tests (ported into tests/).
 * The RNG stream (rand 0.8.5 StdRng = rand_chacha 0.3.1 ChaCha12 seeded
 * through rand_core 0.6.4 seed_from_u64) is restated from the published
 * algorithms; no reference test pins its values, so sample streams are
 * "parity unpinned" against the Rust crate beyond the two shuffle
 * properties src/rng.rs:49-87 checks.
 */
#ifndef PBRT_ORACLE_H
#define PBRT_ORACLE_H

#include "../include/pbrt_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct OracleBVH OracleBVH;

int oracle_bvh_create(const PbrtShapeDesc* shapes, uint32_t n_shapes,
                      uint32_t max_prims_in_node, const char* split_method,
                      OracleBVH** out);
/* The aggregate of a scene description's shapes and instance definitions
 * (TransformedPrimitive, src/primitive/transformed.rs:14-73). */
int oracle_bvh_create_desc(const PbrtSceneDesc* desc, OracleBVH** out);
void oracle_bvh_destroy(OracleBVH* bvh);
int oracle_bvh_num_nodes(const OracleBVH* bvh, uint32_t* n);
int oracle_bvh_num_primitives(const OracleBVH* bvh, uint32_t* n);
int oracle_bvh_depth(const OracleBVH* bvh, uint32_t* depth);
int oracle_bvh_get_nodes(const OracleBVH* bvh, PbrtPackedNode* out, uint32_t cap);
int oracle_bvh_get_primitive_order(const OracleBVH* bvh, uint32_t* out, uint32_t cap);
int oracle_bvh_world_bound(const OracleBVH* bvh, float lo[3], float hi[3]);
/* Triangle i of the refined list: 9 floats (p1, p2, p3) in the order the
 * intersection test uses them (reversed index order, mesh.rs:325-335). */
int oracle_bvh_triangle(const OracleBVH* bvh, uint32_t prim, float out[9]);

/* counters (may be NULL): [0] nodes tested, [1] triangle tests,
 * [2] sphere tests, summed over all rays. */
int oracle_intersect(const OracleBVH* bvh, const PbrtRay* rays, uint32_t n,
                     PbrtHit* hits, uint64_t* counters, int nthreads);
int oracle_intersect_p(const OracleBVH* bvh, const PbrtRay* rays, uint32_t n,
                       uint8_t* occluded, uint64_t* counters, int nthreads);
/* The any-hit answer with the traversal stopped at the first accepted
 * primitive (reference order otherwise): the work an early-exit any-hit
 * walk does, counted as above.  The answers equal oracle_intersect_p's. */
int oracle_count_first_hit(const OracleBVH* bvh, const PbrtRay* rays, uint32_t n,
                           uint8_t* occluded, uint64_t* counters, int nthreads);

/* Full render of SamplerRenderer::render with the restated direct-light
 * integrator.  rgb: pixel extent * 3 floats.  task_lo/task_hi select a
 * range of tasks (0, num_tasks for all); pixels of other tasks stay 0.
 * stats (may be NULL, else 8 words): [0] camera rays, [1] shadow rays,
 * [2] / [3] / [4] nodes, triangles and analytic shapes tested by the camera
 * rays' traversals, [5] / [6] / [7] the same for the shadow rays'. */
int oracle_render(const PbrtSceneDesc* scene, const PbrtCameraDesc* camera,
                  const PbrtSamplerDesc* sampler, float* rgb, int nthreads,
                  uint32_t task_lo, uint32_t task_hi, uint64_t* stats);

/* The same render over a scene built once (BVH and shading tables), so
 * that repeated renders time the renderer alone. */
typedef struct OracleScene OracleScene;
int oracle_scene_create(const PbrtSceneDesc* scene, OracleScene** out);
void oracle_scene_destroy(OracleScene* scene);
int oracle_scene_render(const OracleScene* scene, const PbrtCameraDesc* camera,
                        const PbrtSamplerDesc* sampler, float* rgb, int nthreads,
                        uint32_t task_lo, uint32_t task_hi, uint64_t* stats);

/* Per-sample dump of one task, in the task's order: for each pixel of the
 * task's sub-window, for each of its samples, `stride` floats:
 * image_x, image_y, lens_u, lens_v, time, then the integrator arrays
 * (for each light: 1 float component sample, then for each light two
 * floats position sample), then ray o.xyz, d.xyz, then L.rgb.
 * Returns the number of samples written in *n_out. */
int oracle_task_samples(const PbrtSceneDesc* scene, const PbrtCameraDesc* camera,
                        const PbrtSamplerDesc* sampler, uint32_t task,
                        float* out, uint64_t capacity_floats, uint32_t* n_out,
                        uint32_t* stride);

/* ---- known-answer helpers ---------------------------------------------- */
int oracle_quadratic(float a, float b, float c, float* t0, float* t1);
void oracle_partition_by_f32(float* v, uint32_t n);
void oracle_partition_by_i64(int64_t* v, uint32_t n);
void oracle_crop_window(uint32_t num, uint32_t count, float aspect, float out[4]);
void oracle_sub_window(int32_t xs, int32_t xe, int32_t ys, int32_t ye,
                       uint32_t num, uint32_t count, int32_t out[4]);
int oracle_bbox_intersect(const float lo[3], const float hi[3], const PbrtRay* ray,
                          float out[2]);
void oracle_bbox_metrics(const float lo[3], const float hi[3], float* area,
                         int32_t* max_extent);
/* Triangle p1,p2,p3 (9 floats) test: returns 1 and (t, b1, b2) on a hit. */
int oracle_triangle_intersect(const float tri[9], const PbrtRay* ray, float out[3]);
/* Sphere (o2w transform, radius, z0, z1, phimax degrees):
 * mode 0 = intersect_p; mode 1 = intersect with dg.
 * out (mode 1): t, eps, p.xyz, nn.xyz, u, v, dpdu.xyz, dpdv.xyz (16 floats). */
/* Disk (kind PBRT_SHAPE_DISK: a = height, b = radius, c = inner radius) or
 * cylinder (PBRT_SHAPE_CYLINDER: a = radius, b = z0, c = z1) against a ray;
 * out as oracle_sphere_intersect. */
int oracle_quadric_intersect(int kind, const PbrtTransform* o2w, float a, float b, float c, float phimax,
                             const PbrtRay* ray, int mode, float out[16]);
int oracle_sphere_intersect(const PbrtTransform* o2w, float radius, float z0, float z1,
                            float phimax, const PbrtRay* ray, int mode, float out[16]);
int oracle_matrix_invert(const float m[16], float out[16]);
void oracle_look_at(const float pos[3], const float look[3], const float up[3],
                    PbrtTransform* out);
/* Projection::new (camera/projective.rs:48-72) for a given camera-to-screen
 * transform: out[0] camera_to_screen, [1] raster_to_screen,
 * [2] screen_to_raster, [3] raster_to_camera. */
void oracle_projection(uint32_t xres, uint32_t yres, const PbrtTransform* proj,
                       const float screen[4], PbrtTransform out[4]);
/* Perspective camera transform of Camera::perspective (camera/mod.rs:105-135). */
void oracle_perspective(float fov_deg, PbrtTransform* out);
void oracle_transform_point(const PbrtTransform* t, const float p[3], float out[3]);
void oracle_transform_vector(const PbrtTransform* t, const float v[3], float out[3]);
void oracle_film_extents(uint32_t xres, uint32_t yres, const float crop[4],
                         float xw, float yw, int32_t sample_ext[4], int32_t pixel_ext[4]);
/* Box filter table value and the other filters of src/filter.rs:87-124
 * (kind: 0 box, 1 triangle, 2 gaussian(alpha=p0), 3 mitchell(b=p0,c=p1),
 * 4 lanczos(tau=p0)). */
float oracle_filter_eval(int kind, float xw, float yw, float p0, float p1,
                         float x, float y);

/* RNG (src/rng.rs:11-33): the u32 word stream of RNG::new(seed) from
 * word `first`, and sequences of draws. */
void oracle_rng_words(uint64_t seed, uint64_t first, uint32_t n, uint32_t* out);
/* Blocks counter .. counter + n_blocks - 1 of the ChaCha keystream with
 * `rounds` rounds (even), the key, the 64-bit block counter in state words
 * 12-13 and the 64-bit stream id in words 14-15: 16 words per block.
 * StdRng's blocks are rounds = 12, stream = 0. */
void oracle_chacha_blocks(const uint32_t key[8], uint64_t counter, uint64_t stream, uint32_t rounds,
                          uint32_t n_blocks, uint32_t* out);
/* The ChaCha key of RNG::new(seed) (seed_from_u64's expansion). */
void oracle_rng_key(uint64_t seed, uint32_t key[8]);
void oracle_rng_floats(uint64_t seed, uint32_t n, float* out);
void oracle_rng_uints(uint64_t seed, uint32_t n, uint64_t* out);
void oracle_rng_shuffle_i64(uint64_t seed, int64_t* v, uint32_t n, uint32_t dims,
                            uint32_t skip_draws);
void oracle_rng_permutation(uint64_t seed, uint64_t* v, uint32_t n);
/* stratified_sample_1d/2d (montecarlo.rs:106-128) on one RNG, in sequence:
 * calls[k] = {kind(1|2), nx, ny, jitter}; out gets every call's samples. */
void oracle_stratified(uint64_t seed, const int32_t* calls, uint32_t n_calls, float* out);
void oracle_latin_hypercube(uint64_t seed, uint32_t num, uint32_t dim, float* out);

#ifdef __cplusplus
}
#endif

#endif
