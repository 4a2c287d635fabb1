// wavefront.cuh - the per-item steps of the SamplerRenderer wavefront,
// shared by the single-render kernels (render.cu) and the batched
// multi-scene kernels (batch.cu), so both run the same f32 operations:
//
//   generate_pixel : stratified samples, light sample arrays and camera
//                    rays of one sampler pixel (sampler/stratified.rs:60-127,
//                    camera/mod.rs:168-271), reading the pixel's slice of
//                    its task's ChaCha12 stream
//   shade_sample   : dg, emitted radiance, per-light sample_l, BSDF and the
//                    unoccluded contribution of one camera sample; shadow
//                    rays go to a compacted queue (integrator/whitted.rs:30-65,
//                    light/point.rs:28-35)
//   combine_sample : L = Le + the unoccluded contributions in light order
//   film_pixel     : one film pixel gathers the samples that land on it, from
//                    its own task only, in the task's sample order
//                    (camera/film.rs:192-249, 175-186, 316-354)
// Every translation unit including it is compiled with --fmad=false and IEEE
// div/sqrt.
#pragma once
#include <cuda_runtime.h>

#include <cfloat>

#include "chacha.cuh"
#include "render_types.h"
#include "trace.cuh"

namespace pbrt {

constexpr int kMaxSpp = 64;

__device__ __forceinline__ int32_t dev_f2i32(float f) {  // Rust `as i32`: saturating, NaN -> 0
    if (f != f) return 0;
    if (f >= 2147483647.0f) return 2147483647;
    if (f <= -2147483648.0f) return (-2147483647 - 1);
    return (int32_t)f;
}

// ------------------------------------------------------------- generate ---
// montecarlo.rs:115-128
__device__ __forceinline__ void stratified_2d(float* s, uint32_t nx, uint32_t ny, WordStream& rng, bool jitter) {
    float dx = 1.0f / (float)nx, dy = 1.0f / (float)ny;
    for (uint32_t y = 0; y < ny; ++y)
        for (uint32_t x = 0; x < nx; ++x) {
            float jx = jitter ? rng.random_float() : 0.5f;
            float jy = jitter ? rng.random_float() : 0.5f;
            uint32_t off = 2 * (y * nx + x);
            s[off] = ((float)x + jx) * dx;
            s[off + 1] = ((float)y + jy) * dy;
        }
}
// montecarlo.rs:106-113
__device__ __forceinline__ void stratified_1d(float* s, uint32_t n, WordStream& rng, bool jitter) {
    float inv = 1.0f / (float)n;
    for (uint32_t i = 0; i < n; ++i) {
        float d = jitter ? rng.random_float() : 0.5f;
        s[i] = ((float)i + d) * inv;
    }
}
// rng.rs:23-33
__device__ __forceinline__ void shuffle(float* v, uint32_t count, uint32_t dims, WordStream& rng) {
    for (uint32_t i = 0; i < count; ++i) {
        uint32_t other = i + (uint32_t)(rng.random_uint() % (uint64_t)(count - i));
        for (uint32_t j = 0; j < dims; ++j) {
            float t = v[dims * i + j];
            v[dims * i + j] = v[dims * other + j];
            v[dims * other + j] = t;
        }
    }
}

// r2c / c2w: the camera's raster-to-camera and camera-to-world matrices
// (a copy in registers, or the parameters themselves).
__device__ __forceinline__ void camera_ray(const RenderParams& P, const float* r2c, const float* c2w, float ix,
                                           float iy, float lu, float lv, PbrtRay* out) {
    float pc[3];
    xf_point(r2c, ix, iy, 0.0f, pc);
    float len = sqrtf(pc[0] * pc[0] + pc[1] * pc[1] + pc[2] * pc[2]);
    float rl = 1.0f / len;
    float o[3] = {0.0f, 0.0f, 0.0f};
    float d[3] = {pc[0] * rl, pc[1] * rl, pc[2] * rl};
    if (P.lens_radius > 0.0f) {  // projective.rs:79-96 (concentric_sample_disk is the identity there)
        float u = lu * P.lens_radius, v = lv * P.lens_radius;
        float ft = P.focal_distance / d[2];
        float pf[3] = {o[0] + d[0] * ft, o[1] + d[1] * ft, o[2] + d[2] * ft};
        o[0] = u;
        o[1] = v;
        o[2] = 0.0f;
        float w[3] = {pf[0] - o[0], pf[1] - o[1], pf[2] - o[2]};
        float wl = 1.0f / sqrtf(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
        d[0] = w[0] * wl;
        d[1] = w[1] * wl;
        d[2] = w[2] * wl;
    }
    float wo[3], wd[3];
    xf_point(c2w, o[0], o[1], o[2], wo);
    xf_vector(c2w, d[0], d[1], d[2], wd);
    out->ox = wo[0];
    out->oy = wo[1];
    out->oz = wo[2];
    out->tmin = 0.0f;
    out->dx = wd[0];
    out->dy = wd[1];
    out->dz = wd[2];
    out->tmax = FLT_MAX;  // ray.rs:36
}

// One ray as a single 256-bit store: the lanes of a warp write rays that lie
// 32 x spp bytes apart, and one request per ray fills its 32-byte sector
// where two 16-byte stores would each write half of it (measured on GB300:
// k_generate 1.33 -> 0.49 ms for 1024^2 x 16 samples).  `p` is 32-byte
// aligned: every ray buffer the wavefront writes starts on a 256-byte
// boundary and holds 32-byte rays.
__device__ __forceinline__ void st_ray(PbrtRay* p, const PbrtRay& r) {
    asm volatile("st.global.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(p), "f"(r.ox), "f"(r.oy),
                 "f"(r.oz), "f"(r.tmin), "f"(r.dx), "f"(r.dy), "f"(r.dz), "f"(r.tmax)
                 : "memory");
}

// The image positions of one pixel's samples, written in order: two
// consecutive samples whose pair is 16-byte aligned go out as one store.
struct PosWriter {
    float2* img;  // the pixel's first sample
    uint32_t n;   // samples in the pixel
    uint32_t odd; // 1 when img is 8 mod 16: sample 0 completes the previous pixel's pair
    float2 held;
    __device__ __forceinline__ PosWriter(float2* p, uint32_t count)
        : img(p), n(count), odd((uint32_t)(reinterpret_cast<uintptr_t>(p) >> 3) & 1u), held(make_float2(0, 0)) {}
    __device__ __forceinline__ void put(uint32_t k, float2 v) {
        if (((k + odd) & 1u) != 0u) {  // second of an aligned pair
            if (k > 0)
                *reinterpret_cast<float4*>(img + k - 1) = make_float4(held.x, held.y, v.x, v.y);
            else
                img[k] = v;
        } else if (k + 1 == n) {
            img[k] = v;
        } else {
            held = v;
        }
    }
};

// One sampler pixel (k_generate's item).  `rng_col`: this thread's column
// of 32 words in shared memory (word k at rng_col[k * stride]).
__device__ __forceinline__ void generate_pixel(const RenderParams& P, uint32_t pix, uint32_t* rng_col,
                                               uint32_t stride) {
    int32_t sw = P.sx1 - P.sx0;
    int32_t x = P.sx0 + (int32_t)(pix % (uint32_t)sw);
    int32_t y = P.sy0 + (int32_t)(pix / (uint32_t)sw);
    uint32_t t = 0;
    for (; t < P.n_tasks; ++t) {
        const TaskRec& T = P.tasks[t];
        if (x >= T.wx0 && x < T.wx1 && y >= T.wy0 && y < T.wy1) break;
    }
    const uint32_t spp = P.spp, nl = P.n_lights;
    const uint64_t s0 = (uint64_t)pix * spp;
    if (t == P.n_tasks) {  // not covered by any task (another shard's task, or no tiling)
        PosWriter pos(P.img + s0, spp);
        for (uint32_t i = 0; i < spp; ++i) {
            pos.put(i, make_float2(-1.0e30f, -1.0e30f));
            const PbrtRay r = {0, 0, 0, 1.0f, 0, 0, 1.0f, 0.0f};
            st_ray(P.rays + s0 + i, r);
        }
        P.pixbox[pix] = make_float4(-1.0e30f, -1.0e30f, -1.0e30f, -1.0e30f);
        return;
    }
    const TaskRec& T = P.tasks[t];
    uint64_t j = (uint64_t)(y - T.wy0) * (uint64_t)(T.wx1 - T.wx0) + (uint64_t)(x - T.wx0);
    WordStream rng;
    rng.seek(T.key, j * P.words_per_pixel, (j + 1) * P.words_per_pixel, rng_col, stride);
    const bool jit = P.jitter != 0;
    if (!(P.lens_radius > 0.0f)) {
        // Pinhole camera: the ray depends on the image position alone, so
        // the lens and time samples and their two shuffles (which permute
        // only those arrays) are never read - their words are skipped
        // instead of drawn, and each stratum's camera ray is made as soon
        // as its image position is known (image samples are not shuffled).
        // Same stream positions, same values as the general path below.
        // the matrices go to registers once per pixel (in a batch P lives in
        // global memory, where every use would be a load)
        float r2c[16], c2w[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            r2c[k] = P.r2c[k];
            c2w[k] = P.c2w[k];
        }
        const float dx = 1.0f / (float)P.xs, dy = 1.0f / (float)P.ys;
        float4 bb = make_float4(FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX);
        PosWriter pos(P.img + s0, spp);
        for (uint32_t yy = 0; yy < P.ys; ++yy)
            for (uint32_t xx = 0; xx < P.xs; ++xx) {
                const float jx = jit ? rng.random_float() : 0.5f;
                const float jy = jit ? rng.random_float() : 0.5f;
                const float ix = (((float)xx + jx) * dx) + (float)x;
                const float iy = (((float)yy + jy) * dy) + (float)y;
                const uint32_t k = yy * P.xs + xx;
                pos.put(k, make_float2(ix, iy));
                bb = make_float4(fminf(bb.x, ix), fminf(bb.y, iy), fmaxf(bb.z, ix), fmaxf(bb.w, iy));
                PbrtRay r;
                camera_ray(P, r2c, c2w, ix, iy, 0.0f, 0.0f, &r);
                st_ray(P.rays + s0 + k, r);
            }
        P.pixbox[pix] = bb;
        // lens (2 spp) and time (spp) strata when jittered, then one u64 per
        // element of each shuffle (2 x 2 spp words)
        rng.skip((jit ? 3u * spp : 0u) + 4u * spp);
        for (uint32_t i = 0; i < spp; ++i) {
            float* ls = P.lsamp + (s0 + i) * (3 * nl);
            for (uint32_t l = 0; l < nl; ++l) {
                ls[l] = (0.0f + rng.random_float()) * 1.0f;
                rng.skip(2);
            }
            for (uint32_t l = 0; l < nl; ++l) {
                float u0 = (0.0f + rng.random_float()) * 1.0f;
                float u1 = (0.0f + rng.random_float()) * 1.0f;
                rng.skip(4);
                ls[nl + 2 * l] = u0;
                ls[nl + 2 * l + 1] = u1;
            }
        }
        return;
    }
    float image[2 * kMaxSpp], lens[2 * kMaxSpp], time[kMaxSpp];
    stratified_2d(image, P.xs, P.ys, rng, jit);
    stratified_2d(lens, P.xs, P.ys, rng, jit);
    stratified_1d(time, spp, rng, jit);
    float4 bb = make_float4(FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX);
    for (uint32_t i = 0; i < spp; ++i) {
        image[2 * i] += (float)x;
        image[2 * i + 1] += (float)y;
        bb = make_float4(fminf(bb.x, image[2 * i]), fminf(bb.y, image[2 * i + 1]), fmaxf(bb.z, image[2 * i]),
                         fmaxf(bb.w, image[2 * i + 1]));
    }
    P.pixbox[pix] = bb;
    shuffle(lens, spp, 2, rng);
    shuffle(time, spp, 1, rng);
    PosWriter pos(P.img + s0, spp);
    for (uint32_t i = 0; i < spp; ++i) {
        const uint64_t s = s0 + i;
        pos.put(i, make_float2(image[2 * i], image[2 * i + 1]));
        // integrator arrays: one 1-D and one 2-D sample per light, each a
        // latin_hypercube of one sample (montecarlo.rs:88-104): the floats,
        // then one swap draw per dimension (always with itself).
        float* ls = P.lsamp + s * (3 * nl);
        for (uint32_t l = 0; l < nl; ++l) {
            ls[l] = (0.0f + rng.random_float()) * 1.0f;
            rng.random_uint();
        }
        for (uint32_t l = 0; l < nl; ++l) {
            float u0 = (0.0f + rng.random_float()) * 1.0f;
            float u1 = (0.0f + rng.random_float()) * 1.0f;
            rng.random_uint();
            rng.random_uint();
            ls[nl + 2 * l] = u0;
            ls[nl + 2 * l + 1] = u1;
        }
        PbrtRay r;
        camera_ray(P, P.r2c, P.c2w, image[2 * i], image[2 * i + 1], lens[2 * i], lens[2 * i + 1], &r);
        st_ray(P.rays + s, r);
    }
}

// ----------------------------------------------------------------- shade ---
struct V {
    float x, y, z;
};
__device__ __forceinline__ V mkv(float x, float y, float z) { return V{x, y, z}; }
__device__ __forceinline__ V vsub(V a, V b) { return mkv(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V vadd(V a, V b) { return mkv(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V vmul(V a, float f) { return mkv(a.x * f, a.y * f, a.z * f); }
__device__ __forceinline__ float vdot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V vcross(V a, V b) {
    return mkv((a.y * b.z) - (a.z * b.y), (a.z * b.x) - (a.x * b.z), (a.x * b.y) - (a.y * b.x));
}
__device__ __forceinline__ float vlen(V a) { return sqrtf(a.x * a.x + a.y * a.y + a.z * a.z); }
__device__ __forceinline__ V vnorm(V a) {  // geometry/normal.rs:181-186
    float r = 1.0f / vlen(a);
    return vmul(a, r);
}
__device__ __forceinline__ V ld3(const float* p) { return mkv(p[0], p[1], p[2]); }

// visibility_tester.rs:16-24
__device__ __forceinline__ void segment(V p1, float eps1, V p2, float eps2, PbrtRay* r) {
    float dist = vlen(vsub(p1, p2));
    float rd = 1.0f / dist;
    V d = vmul(vsub(p2, p1), rd);
    r->ox = p1.x;
    r->oy = p1.y;
    r->oz = p1.z;
    r->tmin = eps1;
    r->dx = d.x;
    r->dy = d.y;
    r->dz = d.z;
    r->tmax = (1.0f - eps2) * dist;
}

// Hit point, geometric normal and dp/du (world space) of refined primitive
// `sp` (its analytic record in `spheres`) for the ray (ro, rd) at t: the
// dg.p / dg.nn / dg.dpdu that the shape's intersect builds.
__device__ __forceinline__ void surface_point(const ShadePrim& sp, const SphereRec* spheres, V ro, V rd, float t,
                                              V* p_out, V* nn_out, V* dpdu_out) {
    const uint32_t flags = __float_as_uint(sp.c[3]);
    V nn = mkv(0, 0, 1);
    if ((flags & kShadeSphere) && spheres[flags >> 2].kind != kQuadSphere) {
        const SphereRec& S = spheres[flags >> 2];
        float o[3], d[3];
        xf_point(S.w2o, ro.x, ro.y, ro.z, o);
        xf_vector(S.w2o, rd.x, rd.y, rd.z, d);
        const V ph = mkv(o[0] + d[0] * t, o[1] + d[1] * t, o[2] + d[2] * t);
        float pw[3];
        xf_point(S.o2w, ph.x, ph.y, ph.z, pw);
        *p_out = ld3(pw);
        if (S.kind == kQuadDisk) {
            // disk.rs:106-129: the normal is the transformed +-z (by the
            // side of the object-space ray origin), neither normalised
            // nor flipped
            const float nz = o[2] > 0.0f ? 1.0f : -1.0f;  // transform.rs:220-227 (inverse transpose)
            nn = mkv(S.w2o[0] * 0.0f + S.w2o[4] * 0.0f + S.w2o[8] * nz,
                     S.w2o[1] * 0.0f + S.w2o[5] * 0.0f + S.w2o[9] * nz,
                     S.w2o[2] * 0.0f + S.w2o[6] * 0.0f + S.w2o[10] * nz);
            const float k = S.phi_max / (2.0f * 3.14159265358979323846f);  // disk.rs:114-116
            const V dpdu = vmul(mkv(-S.phi_max * ph.y, S.phi_max * ph.x, 0.0f), k);
            float du[3];
            xf_vector(S.o2w, dpdu.x, dpdu.y, dpdu.z, du);
            *dpdu_out = ld3(du);
        } else {
            // cylinder.rs:143-164 + helpers.rs:17-43 + diff_geom.rs:52-79
            V dpdu = mkv(S.phi_max * -ph.y, S.phi_max * ph.x, 0.0f);
            V dpdv = mkv(0.0f, 0.0f, S.z_max - S.z_min);
            float du[3], dv[3];
            xf_vector(S.o2w, dpdu.x, dpdu.y, dpdu.z, du);
            xf_vector(S.o2w, dpdv.x, dpdv.y, dpdv.z, dv);
            nn = vnorm(vcross(ld3(du), ld3(dv)));
            if (S.flip) nn = vmul(nn, -1.0f);
            *dpdu_out = ld3(du);
        }
    } else if (flags & kShadeSphere) {
        // sphere.rs:135-176 + shape/helpers.rs:17-43 + diff_geom.rs:52-79
        const SphereRec& S = spheres[flags >> 2];
        float o[3], d[3];
        xf_point(S.w2o, ro.x, ro.y, ro.z, o);
        xf_vector(S.w2o, rd.x, rd.y, rd.z, d);
        V ph = mkv(o[0] + d[0] * t, o[1] + d[1] * t, o[2] + d[2] * t);
        float zc = ph.z / S.radius;
        zc = zc < -1.0f ? -1.0f : (zc > 1.0f ? 1.0f : zc);
        float theta = acosf(zc);
        float zradius = sqrtf(ph.x * ph.x + ph.y * ph.y);
        float inv_zr = 1.0f / zradius;
        float cos_phi = ph.x * inv_zr, sin_phi = ph.y * inv_zr;
        float dtheta = S.theta_max - S.theta_min;
        V dpdu = mkv(-S.phi_max * ph.y, S.phi_max * ph.x, 0.0f);
        V dpdv = vmul(mkv(ph.z * cos_phi, ph.z * sin_phi, -S.radius * sinf(theta)), dtheta);
        float pw[3], du[3], dv[3];
        xf_point(S.o2w, ph.x, ph.y, ph.z, pw);
        xf_vector(S.o2w, dpdu.x, dpdu.y, dpdu.z, du);
        xf_vector(S.o2w, dpdv.x, dpdv.y, dpdv.z, dv);
        *p_out = ld3(pw);
        nn = vnorm(vcross(ld3(du), ld3(dv)));
        if (S.flip) nn = vmul(nn, -1.0f);
        *dpdu_out = ld3(du);
    } else {
        // mesh.rs:212-264 with the default uvs: du1 = -1, du2 = 0,
        // dv1 = -1, dv2 = -1, determinant 1
        V p1 = ld3(sp.a), p2 = ld3(sp.b), p3 = ld3(sp.c);
        const float du1 = 0.0f - 1.0f, du2 = 1.0f - 1.0f, dv1 = 0.0f - 1.0f, dv2 = 0.0f - 1.0f;
        V dp1 = vsub(p1, p3), dp2 = vsub(p2, p3);
        float inv_det = 1.0f / (du1 * dv2 - dv1 * du2);
        V dpdu = vmul(vsub(vmul(dp1, dv2), vmul(dp2, dv1)), inv_det);
        V dpdv = vmul(vadd(vmul(dp1, -du2), vmul(dp2, du1)), inv_det);
        *p_out = mkv(ro.x + rd.x * t, ro.y + rd.y * t, ro.z + rd.z * t);
        nn = vnorm(vcross(dpdu, dpdv));
        if (flags & kShadeFlip) nn = vmul(nn, -1.0f);
        *dpdu_out = dpdu;
    }
    *nn_out = nn;
}

// OrenNayar::f (orennayar.rs:31-62) without the reflectance: a + b *
// maxcos * sin(alpha) * tan(beta) for local wo, wi (bsdf/utils.rs:5-28).
__device__ __forceinline__ float sin_theta_l(V v) { return sqrtf(fmaxf(0.0f, 1.0f - v.z * v.z)); }
__device__ __forceinline__ float clamp_unit(float x) { return x < -1.0f ? -1.0f : (x > 1.0f ? 1.0f : x); }
__device__ __forceinline__ float oren_nayar_term(float a, float b, V wo, V wi) {
    const float sinthetai = sin_theta_l(wi), sinthetao = sin_theta_l(wo);
    float maxcos = 0.0f;
    if (!(sinthetai < 1e-4f || sinthetao < 1e-4f)) {
        const float cpi = sinthetai == 0.0f ? 1.0f : clamp_unit(wi.x / sinthetai);
        const float spi = sinthetai == 0.0f ? 0.0f : clamp_unit(wi.y / sinthetai);
        const float cpo = sinthetao == 0.0f ? 1.0f : clamp_unit(wo.x / sinthetao);
        const float spo = sinthetao == 0.0f ? 0.0f : clamp_unit(wo.y / sinthetao);
        maxcos = fmaxf(cpi * cpo + spi * spo, 0.0f);
    }
    float sinalpha, tanbeta;
    if (fabsf(wi.z) > fabsf(wo.z)) {
        sinalpha = sinthetao;
        tanbeta = sinthetai / fabsf(wi.z);
    } else {
        sinalpha = sinthetai;
        tanbeta = sinthetao / fabsf(wo.z);
    }
    return a + b * maxcos * sinalpha * tanbeta;
}

// Where shade_sample appends its shadow rays: the ray, the (sample, light)
// slot it decides and, in a batch, the job it belongs to.
struct ShadowSink {
    PbrtRay* rays;
    uint32_t* slot;
    uint32_t* job;  // nullptr for a single render
    uint32_t* count;
};

// One camera sample (k_shade's item); every lane of the warp calls it, with
// live = false past the end.  `job` tags the queued shadow rays in a batch.
// The light loop runs to the warp's largest light count so that the
// warp-aggregated queue append stays convergent when lanes belong to
// different jobs.
__device__ __forceinline__ void shade_sample(const RenderParams& P, uint64_t s, bool live, const ShadowSink& Q,
                                             uint32_t job) {
    const uint32_t nl = live ? P.n_lights : 0u;
    const unsigned lane = threadIdx.x & 31;
    const uint32_t nl_warp = __reduce_max_sync(0xffffffffu, nl);
    float4 h = live ? P.hits[s] : make_float4(__int_as_float(-1), 0, 0, 0);
    int32_t prim = __float_as_int(h.x);
    bool hit = live && prim >= 0;
    V p = mkv(0, 0, 0), nn = mkv(0, 0, 1), wo = mkv(0, 0, 1), dpdu = mkv(1, 0, 0);
    float eps = 0.0f;
    float kd[3] = {0, 0, 0};
    float on_a = 0.0f, on_b = 0.0f;  // Oren-Nayar A, B (oren)
    bool oren = false;
    float le[3] = {0, 0, 0};
    if (hit) {
        const PbrtRay r = P.rays[s];
        float t = h.y;
        V o = mkv(r.ox, r.oy, r.oz), d = mkv(r.dx, r.dy, r.dz);
        const ShadePrim* shade = P.shade;
        const SphereRec* spheres = P.spheres;
        const SphereRec* inst = nullptr;
        uint32_t id = (uint32_t)prim;
        if (P.n_inst) {
            // the last instance whose first id is <= id (ids are in refined order)
            uint32_t lo = 0, hi = P.n_inst;
            while (lo < hi) {
                const uint32_t mid = (lo + hi) >> 1;
                if (P.inst_map[mid].x <= id)
                    lo = mid + 1;
                else
                    hi = mid;
            }
            if (lo > 0) {
                const uint4 e = P.inst_map[lo - 1];
                if (id - e.x < e.z) {
                    // inside the instance: shade the definition's primitive on
                    // the primitive-space ray (transformed.rs:37-38)
                    inst = P.spheres + e.w;
                    const InstShade D = P.inst_defs[inst->instance];
                    shade = D.shade;
                    spheres = D.spheres;
                    id -= e.x;
                    float oi[3], di[3];
                    xf_point(inst->w2o, o.x, o.y, o.z, oi);
                    xf_vector(inst->w2o, d.x, d.y, d.z, di);
                    o = ld3(oi);
                    d = ld3(di);
                } else {
                    id = e.y + 1u + (id - e.x - e.z);  // a primitive after that instance
                }
            }
        }
        const ShadePrim& sp = shade[id];
        surface_point(sp, spheres, o, d, t, &p, &nn, &dpdu);
        if (inst) {
            // transformed.rs:45-49: p and dpdu by primitive-to-world, nn by
            // its normal transform (w2p transposed), normalised
            float pw[3], du[3];
            xf_point(inst->o2w, p.x, p.y, p.z, pw);
            p = ld3(pw);
            xf_vector(inst->o2w, dpdu.x, dpdu.y, dpdu.z, du);
            dpdu = ld3(du);
            const float* m = inst->w2o;
            nn = vnorm(mkv(m[0] * nn.x + m[4] * nn.y + m[8] * nn.z, m[1] * nn.x + m[5] * nn.y + m[9] * nn.z,
                           m[2] * nn.x + m[6] * nn.y + m[10] * nn.z));
        }
        eps = t * 5e-4f;  // mesh.rs:262, sphere.rs:174
        wo = mkv(-r.dx, -r.dy, -r.dz);
        uint32_t al = __float_as_uint(sp.b[3]);
        if (al != 0u) {  // Le of an emitter (pbrt-v2 semantics; intersection.rs:58 is 0)
            const LightRec& L = P.lights[al - 1];
            if (L.kind == kLightArea && vdot(nn, wo) > 0.0f) {
                le[0] = L.spec[0];
                le[1] = L.spec[1];
                le[2] = L.spec[2];
            }
        }
        const uint32_t mi = __float_as_uint(sp.a[3]);
        const float4 m = P.materials[2 * mi], m2 = P.materials[2 * mi + 1];
        kd[0] = m.x;
        kd[1] = m.y;
        kd[2] = m.z;
        on_a = m.w;
        on_b = m2.x;
        oren = __float_as_uint(m2.y) != 0u;
    }
    // BSDF frame of Oren-Nayar (bsdf/mod.rs:70-86): tn = normalize(dpdu),
    // sn = nn x tn, world_to_local(v) = (v.sn, v.tn, v.nn)
    V tn = mkv(0, 0, 0), sn = mkv(0, 0, 0), wo_l = mkv(0, 0, 0);
    if (oren) {
        tn = vnorm(dpdu);
        sn = vcross(nn, tn);
        wo_l = mkv(vdot(wo, sn), vdot(wo, tn), vdot(wo, nn));
    }
    if (live) P.le[s] = make_float4(le[0], le[1], le[2], 0.0f);
    const float invpi = 1.0f / 3.14159265358979323846f;  // lambertian.rs:21
    for (uint32_t l = 0; l < nl_warp; ++l) {
        bool want = false;
        PbrtRay sr;
        float4 c = make_float4(0, 0, 0, 0);
        if (hit && l < nl) {
            const LightRec& L = P.lights[l];
            const float* ls = P.lsamp + s * (3 * nl);
            float Li[3], pdf;
            V wi;
            if (L.kind == kLightPoint) {  // point.rs:28-35 with wi normalised (D6)
                V lp = ld3(L.pos);
                V w = vsub(lp, p);
                float d2 = w.x * w.x + w.y * w.y + w.z * w.z;
                Li[0] = L.spec[0] / d2;
                Li[1] = L.spec[1] / d2;
                Li[2] = L.spec[2] / d2;
                wi = vnorm(w);
                pdf = 1.0f;
                segment(p, eps, lp, 0.0f, &sr);
            } else {  // diffuse area light (D5)
                float comp = ls[l], u0 = ls[nl + 2 * l], u1 = ls[nl + 2 * l + 1];
                uint32_t k = 0, n = L.tri_count;
                const float* cdf = P.area_cdf + __float_as_uint(L.pos[3]);
                while (k + 1 < n && !(comp < cdf[k + 1])) ++k;
                const AreaTri& T = P.area_tris[L.tri_first + k];
                V a = ld3(T.p1), b = ld3(T.p2), cc = ld3(T.p3);
                float su1 = sqrtf(u0);
                float b1 = 1.0f - su1;
                float b2 = u1 * su1;
                V ps = vadd(vadd(vmul(a, b1), vmul(b, b2)), vmul(cc, (1.0f - b1) - b2));
                V ns = vnorm(vcross(vsub(b, a), vsub(cc, a)));
                if (T.p1[3] != 0.0f) ns = vmul(ns, -1.0f);
                wi = vnorm(vsub(ps, p));
                V dd = vsub(p, ps);
                float d2 = dd.x * dd.x + dd.y * dd.y + dd.z * dd.z;
                V mw = mkv(-wi.x, -wi.y, -wi.z);
                float cs = vdot(ns, mw);
                float ac = fabsf(cs);
                pdf = (ac == 0.0f) ? 0.0f : d2 / (ac * L.area);
                bool lit = cs > 0.0f;
                Li[0] = lit ? L.spec[0] : 0.0f;
                Li[1] = lit ? L.spec[1] : 0.0f;
                Li[2] = lit ? L.spec[2] : 0.0f;
                segment(p, eps, ps, 1e-3f, &sr);
            }
            bool black = Li[0] == 0.0f && Li[1] == 0.0f && Li[2] == 0.0f;
            if (!black && pdf != 0.0f) {
                bool refl = vdot(wi, nn) * vdot(wo, nn) > 0.0f;  // bsdf/mod.rs:133-137
                float f[3] = {0, 0, 0};
                if (refl && !oren) {  // Lambertian::f (lambertian.rs:20-23)
                    f[0] = kd[0] * invpi;
                    f[1] = kd[1] * invpi;
                    f[2] = kd[2] * invpi;
                } else if (refl) {  // OrenNayar::f (orennayar.rs:31-62)
                    const float g = oren_nayar_term(on_a, on_b, wo_l, mkv(vdot(wi, sn), vdot(wi, tn), vdot(wi, nn)));
                    f[0] = kd[0] * invpi * g;
                    f[1] = kd[1] * invpi * g;
                    f[2] = kd[2] * invpi * g;
                }
                if (!(f[0] == 0.0f && f[1] == 0.0f && f[2] == 0.0f)) {
                    float ad = fabsf(vdot(wi, nn));
                    c.x = ((f[0] * Li[0]) * ad) / pdf;
                    c.y = ((f[1] * Li[1]) * ad) / pdf;
                    c.z = ((f[2] * Li[2]) * ad) / pdf;
                    c.w = 1.0f;
                    want = true;
                }
            }
        }
        if (live && l < nl) P.contrib[s * nl + l] = c;
        // warp-aggregated append to the shadow-ray queue
        unsigned mask = __ballot_sync(0xffffffffu, want);
        if (mask) {
            uint32_t base = 0;
            int leader = __ffs(mask) - 1;
            if ((int)lane == leader) base = atomicAdd(Q.count, (uint32_t)__popc(mask));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (want) {
                uint32_t q = base + (uint32_t)__popc(mask & ((1u << lane) - 1u));
                st_ray(Q.rays + q, sr);
                Q.slot[q] = (uint32_t)(s * nl + l);
                if (Q.job) Q.job[q] = job;
            }
        }
    }
}

// One sample (k_combine's item).
__device__ __forceinline__ void combine_sample(const RenderParams& P, uint64_t s) {
    float4 e = P.le[s];
    float L0 = e.x, L1 = e.y, L2 = e.z;
    for (uint32_t l = 0; l < P.n_lights; ++l) {
        float4 c = P.contrib[s * P.n_lights + l];
        if (c.w != 0.0f && !P.occluded[s * P.n_lights + l]) {
            L0 = L0 + c.x;
            L1 = L1 + c.y;
            L2 = L2 + c.z;
        }
    }
    if (L0 != L0 || L1 != L1 || L2 != L2) atomicAdd(&P.counters[1], 1u);
    P.L[s] = make_float4(L0, L1, L2, 0.0f);
}

// ------------------------------------------------------------------ film ---
__device__ __forceinline__ void rgb_to_xyz(float r, float g, float b, float* x) {  // spectrum.rs:37-41
    x[0] = 0.412453f * r + 0.357580f * g + 0.180423f * b;
    x[1] = 0.212671f * r + 0.715160f * g + 0.072169f * b;
    x[2] = 0.019334f * r + 0.119193f * g + 0.950227f * b;
}
__device__ __forceinline__ void xyz_to_rgb(const float* x, float* r) {  // spectrum.rs:31-35
    r[0] = 3.240479f * x[0] - 1.37150f * x[1] - 0.498535f * x[2];
    r[1] = -0.969256f * x[0] + 1.875991f * x[1] + 0.041556f * x[2];
    r[2] = 0.055648f * x[0] - 0.204043f * x[1] + 1.057311f * x[2];
}

// One film pixel, idx in [0, film width * height) (k_film's item).
__device__ __forceinline__ void film_pixel(const RenderParams& P, uint32_t idx) {
    const int32_t fw = P.fx1 - P.fx0;
    const int32_t px = P.fx0 + (int32_t)(idx % (uint32_t)fw);
    const int32_t py = P.fy0 + (int32_t)(idx / (uint32_t)fw);
    float xyz[3] = {0.0f, 0.0f, 0.0f};
    float wsum = 0.0f;
    uint32_t t = 0;
    for (; t < P.n_tasks; ++t) {
        const TaskRec& T = P.tasks[t];
        if (px >= T.fx0 && px < T.fx1 && py >= T.fy0 && py < T.fy1) break;
    }
    if (t < P.n_tasks) {
        const TaskRec& T = P.tasks[t];
        const int32_t ylo = max(py + P.gy0, T.wy0), yhi = min(py + P.gy1, T.wy1 - 1);
        const int32_t xlo = max(px + P.gx0, T.wx0), xhi = min(px + P.gx1, T.wx1 - 1);
        const int32_t sw = P.sx1 - P.sx0;
        for (int32_t sy = ylo; sy <= yhi; ++sy)
            for (int32_t sx = xlo; sx <= xhi; ++sx) {
                const uint64_t sp = (uint64_t)(sy - P.sy0) * (uint64_t)sw + (uint64_t)(sx - P.sx0);
                // The landing bounds below are non-decreasing in the sample
                // position, so if the source pixel's extreme samples cannot
                // land on (px, py), none of its samples can.
                const float4 bb = P.pixbox[sp];
                if (dev_f2i32(floorf((bb.z - 0.5f) + P.filter_xw)) < px ||
                    dev_f2i32(ceilf((bb.x - 0.5f) - P.filter_xw)) > px ||
                    dev_f2i32(floorf((bb.w - 0.5f) + P.filter_yw)) < py ||
                    dev_f2i32(ceilf((bb.y - 0.5f) - P.filter_yw)) > py)
                    continue;
                const uint64_t base = sp * P.spp;
                for (uint32_t i = 0; i < P.spp; ++i) {
                    const float2 im = P.img[base + i];
                    // film.rs:198-210 against the task film's extent
                    float dix = im.x - 0.5f, diy = im.y - 0.5f;
                    int32_t x0 = max(T.fx0, dev_f2i32(ceilf(dix - P.filter_xw)));
                    int32_t x1 = min(T.fx1 - 1, dev_f2i32(floorf(dix + P.filter_xw)));
                    int32_t y0 = max(T.fy0, dev_f2i32(ceilf(diy - P.filter_yw)));
                    int32_t y1 = min(T.fy1 - 1, dev_f2i32(floorf(diy + P.filter_yw)));
                    if ((x1 - x0) < 0 || (y1 - y0) < 0) continue;
                    if (px < x0 || px > x1 || py < y0 || py > y1) continue;
                    const float4 Ls = P.L[base + i];
                    float sx3[3];
                    rgb_to_xyz(Ls.x, Ls.y, Ls.z, sx3);
                    float fx = ((float)px - dix) * P.filter_inv_xw * 16.0f;
                    float fy = ((float)py - diy) * P.filter_inv_yw * 16.0f;
                    int ix = min(dev_f2i32(floorf(fabsf(fx))), 15);
                    int iy = min(dev_f2i32(floorf(fabsf(fy))), 15);
                    float w = P.filter_table[iy * 16 + ix];
                    xyz[0] += w * sx3[0];
                    xyz[1] += w * sx3[1];
                    xyz[2] += w * sx3[2];
                    wsum += w;
                }
            }
    }
    // write_image with the intended normalisation (film.rs:316-354, D8)
    float c[3];
    xyz_to_rgb(xyz, c);
    if (wsum != 0.0f) {
        float inv = 1.0f / wsum;
        c[0] = fmaxf(c[0] * inv, 0.0f);
        c[1] = fmaxf(c[1] * inv, 0.0f);
        c[2] = fmaxf(c[2] * inv, 0.0f);
    }
    const float zero[3] = {0.0f, 0.0f, 0.0f};
    float sp[3];
    xyz_to_rgb(zero, sp);
    float* o = P.rgb + 3 * (size_t)idx;
    o[0] = c[0] + sp[0] * 1.0f;
    o[1] = c[1] + sp[1] * 1.0f;
    o[2] = c[2] + sp[2] * 1.0f;
}

}  // namespace pbrt
