// capi_render.cu - scene creation and the render entry point of the C ABI.
//
// Host code here is compiled with -ffp-contract=off: the task windows,
// film extents, area-light CDFs and ChaCha keys are computed with the
// reference's f32 arithmetic.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/pbrt_gpu.h"
#include "capi_internal.h"
#include "host_scene.h"
#include "kernels.h"
#include "render_types.h"

using namespace pbrt;

namespace pbrt {
cudaError_t launch_render(const RenderParams& P, cudaStream_t s);
}

namespace pbrt {

static float clampf(float x, float lo, float hi) {
    if (x < lo) x = lo;
    if (x > hi) x = hi;
    return x;
}

// Rust `f as i32` / `f as usize` (saturating, NaN -> 0)
int32_t f2i32(float f) {
    if (f != f) return 0;
    if (f >= 2147483647.0f) return INT32_MAX;
    if (f <= -2147483648.0f) return INT32_MIN;
    return (int32_t)f;
}
size_t f2usize(float f) {
    if (!(f > 0.0f)) return 0;
    if (f >= 18446744073709551615.0f) return SIZE_MAX;
    return (size_t)f;
}

// src/utils/mod.rs:171-205
void crop_window(size_t num, size_t count, float aspect, float out[4]) {
    auto split = [](size_t cnt, size_t asp, size_t* nx, size_t* ny) {
        size_t x = 1, y = cnt;
        while ((y % 2) == 0 && 2 * asp * x < y) {
            y /= 2;
            x *= 2;
        }
        *nx = x;
        *ny = y;
    };
    size_t nx, ny;
    if (aspect < 1.0f) {
        split(count, f2usize(1.0f / aspect), &nx, &ny);
    } else {
        size_t x, y;
        split(count, f2usize(aspect), &x, &y);
        nx = y;
        ny = x;
    }
    size_t xo = num % nx, yo = num / nx;
    out[0] = (float)xo / (float)nx;
    out[1] = (float)(xo + 1) / (float)nx;
    out[2] = (float)yo / (float)ny;
    out[3] = (float)(yo + 1) / (float)ny;
}

float lerpf(float a, float b, float t) { return a * (1.0f - t) + b * t; }  // utils/mod.rs:15-21

// src/sampler/base.rs:29-48
void sub_window(const PbrtSamplerDesc& s, size_t num, int32_t out[4]) {
    size_t dx = (size_t)(s.x_end - s.x_start), dy = (size_t)(s.y_end - s.y_start);
    float aspect = (float)dx / (float)dy;
    float t[4];
    crop_window(num, s.num_tasks, aspect, t);
    float psx = (float)s.x_start, psy = (float)s.y_start, pex = (float)s.x_end, pey = (float)s.y_end;
    out[0] = f2i32(lerpf(psx, pex, t[0]));
    out[1] = f2i32(lerpf(psx, pex, t[1]));
    out[2] = f2i32(lerpf(psy, pey, t[2]));
    out[3] = f2i32(lerpf(psy, pey, t[3]));
}

// src/camera/film.rs:81-84 -> (x0, x1, y0, y1)
void film_extent(uint32_t xres, uint32_t yres, const float crop[4], int32_t ext[4]) {
    int32_t xs = f2i32(std::ceil((float)xres * crop[0]));
    int32_t xc = std::max(f2i32(std::ceil((float)xres * crop[1])) - xs, 1);
    int32_t ys = f2i32(std::ceil((float)yres * crop[2]));
    int32_t yc = std::max(f2i32(std::ceil((float)yres * crop[3])) - ys, 1);
    ext[0] = xs;
    ext[1] = xs + xc;
    ext[2] = ys;
    ext[3] = ys + yc;
}

// Source pixels whose samples can land on film pixel p, along one axis:
// p + [*lo, *hi].  A sample of source pixel s lies at a position v in
// [s, s + 1], and it lands on p only if ceil(v - 0.5 - w) <= p <=
// floor(v - 0.5 + w) (film.rs:198-210), i.e. v in [p + 0.5 - w, p + 0.5 + w]
// up to the f32 rounding of those sums, which stays below 1/16 for sample
// coordinates under 2^20.  Hence s in [p + ceil(-0.5 - w - 1/16),
// p + floor(0.5 + w + 1/16)]: 3 source pixels per axis for the box filter
// of radius 0.5.  Windows reaching beyond 2^20 take a wider margin.
void gather_offsets(float w, int32_t s0, int32_t s1, int32_t* lo, int32_t* hi) {
    const int32_t big = 1 << 20;
    if (s0 > -big && s1 < big) {
        *lo = (int32_t)std::ceil(-0.5f - w - 0.0625f);
        *hi = (int32_t)std::floor(0.5f + w + 0.0625f);
    } else {
        *lo = -((int32_t)std::ceil(w) + 2);
        *hi = (int32_t)std::ceil(w) + 2;
    }
}

int sampler_counts(const PbrtSamplerDesc* smp, uint32_t spp, uint32_t n_lights, uint32_t* n_pixels,
                   uint64_t* n_samples) {
    // window sides and area in 64 bits: int32 differences and products wrap
    const int64_t w = (int64_t)smp->x_end - (int64_t)smp->x_start;
    const int64_t h = (int64_t)smp->y_end - (int64_t)smp->y_start;
    if (w <= 0 || h <= 0) return set_error(PBRT_ERR_INVALID_ARGUMENT, "empty sampler window");
    const uint64_t area = (uint64_t)w * (uint64_t)h;
    if (w > INT32_MAX || h > INT32_MAX || area > UINT32_MAX)
        return set_error(PBRT_ERR_INVALID_ARGUMENT, "sampler window of " + std::to_string(w) + " x " +
                                                        std::to_string(h) + " pixels exceeds 2^32 - 1 pixels");
    const uint64_t ns = area * spp;
    // rays, and (sample, light) slots of the shadow queue, are indexed in 32 bits
    if (ns * (uint64_t)std::max<uint32_t>(n_lights, 1u) > UINT32_MAX)
        return set_error(PBRT_ERR_INVALID_ARGUMENT, "the frame's " + std::to_string(ns) + " samples x " +
                                                        std::to_string(n_lights) +
                                                        " lights exceed 2^32 - 1 ray and shadow-queue slots");
    *n_pixels = (uint32_t)area;
    *n_samples = ns;
    return PBRT_OK;
}

// rand_core 0.6.4 SeedableRng::seed_from_u64 (the published PCG32 seed
// expansion: multiplier 6364136223846793005, increment
// 11634580027462260723, XSH-RR output, state advanced before output).
void chacha_key(uint64_t state, uint32_t key[8]) {
    for (int i = 0; i < 8; ++i) {
        state = state * 6364136223846793005ULL + 11634580027462260723ULL;
        uint32_t xs = (uint32_t)(((state >> 18) ^ state) >> 27);
        uint32_t rot = (uint32_t)(state >> 59);
        key[i] = (xs >> rot) | (xs << ((32u - rot) & 31u));
    }
}

static int scene_upload(PbrtScene* S) {
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->uploaded) return PBRT_OK;
    int st;
    if (!S->bvh->uploaded && (st = bvh_upload(S->bvh))) return st;
    auto up = [](auto** dst, const auto& v) -> int {
        *dst = nullptr;
        if (v.empty()) return PBRT_OK;
        size_t bytes = v.size() * sizeof(v[0]);
        int s2 = cuda_status(cudaMalloc((void**)dst, bytes), "cudaMalloc");
        if (s2) return s2;
        return cuda_status(cudaMemcpy(*dst, v.data(), bytes, cudaMemcpyHostToDevice), "cudaMemcpy");
    };
    if ((st = up(&S->d_shade, S->shade))) return st;
    if ((st = up(&S->d_materials, S->materials))) return st;
    if ((st = up(&S->d_lights, S->lights))) return st;
    if ((st = up(&S->d_area_tris, S->area_tris))) return st;
    if ((st = up(&S->d_area_cdf, S->area_cdf))) return st;
    if ((st = up(&S->d_inst_map, S->inst_map))) return st;
    std::vector<InstShade> defs;
    for (size_t k = 0; k < S->inst_shade.size(); ++k) {
        ShadePrim* sh = nullptr;
        st = up(&sh, S->inst_shade[k]);
        if (sh) S->d_inst_bufs.push_back(sh);
        if (st) return st;
        defs.push_back(InstShade{sh, S->bvh->inst_dev[k].spheres});
    }
    if ((st = up(&S->d_inst_defs, defs))) return st;
    // the no-allocation render's scratch is set up with the scene, not in
    // that entry point's first call; a failure here is reported by that
    // entry point, which tries again
    {
        DeviceGuard g(S->bvh->device);
        if (noalloc_prepare(S->bvh->device) != PBRT_OK) (void)cudaGetLastError();
    }
    S->uploaded = true;
    return PBRT_OK;
}

static inline float bitsf(uint32_t u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

void scene_params(const PbrtScene* S, RenderParams* P) {
    P->bvh = S->bvh->dev;
    P->depth = S->bvh->host.depth;
    P->bvh4 = S->bvh->dev4;
    P->wide_bound = S->bvh->host.stack4_bound;
    P->has_wide = wide_of(S->bvh) ? 1u : 0u;
    P->shade = S->d_shade;
    P->spheres = S->bvh->d_spheres;
    P->materials = S->d_materials;
    P->lights = S->d_lights;
    P->n_lights = (uint32_t)S->lights.size();
    P->area_tris = S->d_area_tris;
    P->area_cdf = S->d_area_cdf;
    P->n_inst = (uint32_t)S->inst_map.size();
    P->inst_map = S->d_inst_map;
    P->inst_defs = S->d_inst_defs;
}

// Per refined primitive shading records (ShadePrim) of one BVH.
static void shade_records(const HostBVH& H, std::vector<ShadePrim>* out) {
    out->resize(H.prims.size());
    for (size_t i = 0; i < H.prims.size(); ++i) {
        const HostPrim& p = H.prims[i];
        ShadePrim& r = (*out)[i];
        std::memset(&r, 0, sizeof(r));
        r.a[0] = p.p1.x;
        r.a[1] = p.p1.y;
        r.a[2] = p.p1.z;
        r.a[3] = bitsf((uint32_t)p.material);
        r.b[0] = p.p2.x;
        r.b[1] = p.p2.y;
        r.b[2] = p.p2.z;
        r.b[3] = bitsf(p.area_light >= 0 ? (uint32_t)p.area_light + 1u : 0u);
        r.c[0] = p.p3.x;
        r.c[1] = p.p3.y;
        r.c[2] = p.p3.z;
        uint32_t flags = (p.flip ? kShadeFlip : 0u);
        if (p.kind == PBRT_SHAPE_SPHERE) flags |= kShadeSphere | ((uint32_t)p.sphere << 2);
        r.c[3] = bitsf(flags);
    }
}

}  // namespace pbrt

extern "C" {

int pbrtgpu_scene_create(const PbrtSceneDesc* d, PbrtScene** out) {
    if (!d || !out || (!d->shapes && d->n_shapes) || (!d->lights && d->n_lights) ||
        (!d->materials && d->n_materials))
        return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = nullptr;
    if (!d->instances && d->n_instances) return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
    for (uint32_t k = 0; k < d->n_instances; ++k) {
        const PbrtInstanceDesc& D = d->instances[k];
        if (!D.shapes && D.n_shapes) return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
        for (uint32_t i = 0; i < D.n_shapes; ++i)
            if (D.shapes[i].kind != PBRT_SHAPE_INSTANCE &&
                (D.shapes[i].material < 0 || (uint32_t)D.shapes[i].material >= d->n_materials))
                return set_error(PBRT_ERR_INVALID_ARGUMENT, "instance definition " + std::to_string(k) + " shape " +
                                                                std::to_string(i) + ": material index out of range");
    }
    for (uint32_t i = 0; i < d->n_shapes; ++i) {
        const PbrtShapeDesc& sd = d->shapes[i];
        if (sd.kind == PBRT_SHAPE_INSTANCE) {  // its definition's shapes carry the materials
            if (sd.area_light >= 0)
                return set_error(PBRT_ERR_UNSUPPORTED, "shape " + std::to_string(i) + ": area light on an instance");
            continue;
        }
        if (sd.material < 0 || (uint32_t)sd.material >= d->n_materials)
            return set_error(PBRT_ERR_INVALID_ARGUMENT, "shape " + std::to_string(i) + ": material index out of range");
        if (sd.area_light >= 0) {
            if ((uint32_t)sd.area_light >= d->n_lights || d->lights[sd.area_light].kind != PBRT_LIGHT_DIFFUSE_AREA ||
                d->lights[sd.area_light].shape != (int32_t)i)
                return set_error(PBRT_ERR_INVALID_ARGUMENT,
                                 "shape " + std::to_string(i) + ": area light must be a diffuse area light on it");
        }
    }
    const char* names[3] = {"sah", "middle", "equal"};
    const char* sm = (d->split_method >= 0 && d->split_method < 3) ? names[d->split_method] : "sah";
    PbrtScene* S = new PbrtScene();
    S->bvh = new PbrtBVH();
    std::string err;
    if (d->build_flags & ~(uint32_t)PBRT_BUILD_ON_DEVICE) {
        delete S;
        return set_error(PBRT_ERR_INVALID_ARGUMENT, "unknown build flags");
    }
    const bool on_device = (d->build_flags & PBRT_BUILD_ON_DEVICE) != 0;
    if (on_device && !cuda_device_present()) {
        delete S;
        return set_error(PBRT_ERR_NO_DEVICE, "no CUDA device for the build");
    }
    int st = build_host_bvh(d->shapes, d->n_shapes, d->max_prims_in_node, sm, &S->bvh->host, &err, on_device,
                            d->instances, d->n_instances);
    if (st) {
        delete S;
        return set_error(st, err);
    }
    if (trace_stack_for_depth(S->bvh->host.depth) == 0) {
        delete S;
        return set_error(PBRT_ERR_STACK_OVERFLOW, "BVH too deep for the traversal stack");
    }
    const HostBVH& H = S->bvh->host;
    shade_records(H, &S->shade);
    S->inst_shade.resize(H.insts.size());
    for (size_t k = 0; k < H.insts.size(); ++k) shade_records(H.insts[k], &S->inst_shade[k]);
    for (size_t i = 0; i < H.prims.size(); ++i) {
        const HostPrim& p = H.prims[i];
        if (p.sphere < 0 || H.spheres[p.sphere].kind != kQuadInstance) continue;
        const uint32_t n_inner = (uint32_t)H.insts[H.spheres[p.sphere].instance].prims.size();
        S->inst_map.push_back(make_uint4(H.flat_id[i], (uint32_t)i, n_inner, (uint32_t)p.sphere));
    }
    // MatteMaterial::get_bsdf (matte.rs:30-51): Kd clamped to [0, f32::MAX],
    // sigma to [0, 90]; sigma == 0 -> Lambertian, else OrenNayar::new
    // (orennayar.rs:15-28) with A and B computed here in f32
    for (uint32_t i = 0; i < d->n_materials; ++i) {
        const PbrtMaterialDesc& m = d->materials[i];
        const float sig = clampf(m.sigma, 0.0f, 90.0f);
        const float sigma = sig * 3.14159265358979323846f / 180.0f;  // utils/mod.rs:37-39
        const float sigma2 = sigma * sigma;
        const float a = 1.0f - (sigma2 / (2.0f * (sigma + 0.33f)));
        const float b = 0.45f * sigma2 / (sigma2 + 0.09f);
        const bool oren = !(sig == 0.0f);
        S->materials.push_back(make_float4(clampf(m.kd[0], 0.0f, FLT_MAX), clampf(m.kd[1], 0.0f, FLT_MAX),
                                           clampf(m.kd[2], 0.0f, FLT_MAX), a));
        S->materials.push_back(make_float4(b, bitsf(oren ? 1u : 0u), 0.0f, 0.0f));
    }
    for (uint32_t li = 0; li < d->n_lights; ++li) {
        const PbrtLightDesc& L = d->lights[li];
        LightRec r;
        std::memset(&r, 0, sizeof(r));
        r.spec[0] = L.spectrum[0];
        r.spec[1] = L.spectrum[1];
        r.spec[2] = L.spectrum[2];
        if (L.kind == PBRT_LIGHT_POINT) {
            r.kind = kLightPoint;
            Xf l2w = xf_from_desc(L.light_to_world);
            V3 pos = m4_point(l2w.m, v3(0.0f, 0.0f, 0.0f));  // point.rs:79-82
            r.pos[0] = pos.x;
            r.pos[1] = pos.y;
            r.pos[2] = pos.z;
        } else if (L.kind == PBRT_LIGHT_DIFFUSE_AREA) {
            if (L.shape < 0 || (uint32_t)L.shape >= d->n_shapes || d->shapes[L.shape].kind != PBRT_SHAPE_TRIANGLE_MESH) {
                delete S;
                return set_error(PBRT_ERR_INVALID_ARGUMENT, "area light shape must be a triangle mesh");
            }
            r.kind = kLightArea;
            r.tri_first = (uint32_t)S->area_tris.size();
            float acc = 0.0f;
            std::vector<float> cdf{0.0f};
            for (const HostPrim& p : H.prims) {
                if (p.kind != PBRT_SHAPE_TRIANGLE_MESH || p.shape != L.shape) continue;
                AreaTri t;
                t.p1[0] = p.p1.x;
                t.p1[1] = p.p1.y;
                t.p1[2] = p.p1.z;
                t.p1[3] = p.flip ? 1.0f : 0.0f;
                t.p2[0] = p.p2.x;
                t.p2[1] = p.p2.y;
                t.p2[2] = p.p2.z;
                t.p2[3] = 0.0f;
                t.p3[0] = p.p3.x;
                t.p3[1] = p.p3.y;
                t.p3[2] = p.p3.z;
                t.p3[3] = 0.0f;
                S->area_tris.push_back(t);
                acc += 0.5f * len3(cross3(p.p2 - p.p1, p.p3 - p.p1));  // mesh.rs:100-103
                cdf.push_back(acc);
            }
            r.tri_count = (uint32_t)(S->area_tris.size() - r.tri_first);
            if (r.tri_count == 0 || !(acc > 0.0f)) {
                delete S;
                return set_error(PBRT_ERR_INVALID_ARGUMENT, "area light shape has no area");
            }
            r.area = acc;
            // tri_count + 1 CDF entries (area prefix / total area), at the
            // offset stored in pos[3]
            r.pos[3] = bitsf((uint32_t)S->area_cdf.size());
            for (auto& c : cdf) S->area_cdf.push_back(c / acc);
        } else {
            delete S;
            return set_error(PBRT_ERR_UNSUPPORTED, "unsupported light kind");
        }
        S->lights.push_back(r);
    }
    if (cuda_device_present() && (st = scene_upload(S))) {
        delete S;
        return st;
    }
    *out = S;
    return PBRT_OK;
}

void pbrtgpu_scene_destroy(PbrtScene* S) {
    if (!S) return;
    int dev = S->bvh ? S->bvh->device : 0;
    DeviceGuard g(dev);
    delete S;
}

int pbrtgpu_scene_bvh(const PbrtScene* S, const PbrtBVH** out) {
    if (!S || !out) return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = S->bvh;
    return PBRT_OK;
}

int pbrtgpu_filter_table(const PbrtCameraDesc* cam, float table[256]) {
    if (!cam || !table) return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (filter_table(*cam, table)) return set_error(PBRT_ERR_INVALID_ARGUMENT, "unknown filter kind");
    return PBRT_OK;
}

int pbrtgpu_film_pixel_extent(const PbrtCameraDesc* c, int32_t ext[4]) {
    if (!c || !ext) return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
    film_extent(c->x_res, c->y_res, c->crop_window, ext);
    return PBRT_OK;
}

int pbrtgpu_render(const PbrtScene* cS, const PbrtCameraDesc* cam, const PbrtSamplerDesc* smp, float* rgb_out,
                   void* stream_v) {
    if (!smp) return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
    return pbrtgpu_render_tasks(cS, cam, smp, 0, smp->num_tasks, rgb_out, stream_v);
}

}  // extern "C"

namespace pbrt {

// Validates a render's descriptors, uploads the scene on first use and fills
// every field of *out except the filter table, the task array and the
// per-render buffers; *tasks gets the task records (tasks outside
// [task_lo, task_hi) empty).
int prepare_render(PbrtScene* S, const PbrtCameraDesc* cam, const PbrtSamplerDesc* smp, uint32_t task_lo,
                   uint32_t task_hi, RenderParams* out, std::vector<TaskRec>* tasks_out) {
    if (!S || !cam || !smp) return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (smp->num_tasks == 0) return set_error(PBRT_ERR_INVALID_ARGUMENT, "num_tasks must be > 0");
    if (task_lo > task_hi || task_hi > smp->num_tasks)
        return set_error(PBRT_ERR_INVALID_ARGUMENT, "task range must satisfy task_lo <= task_hi <= num_tasks");
    if (smp->x_end <= smp->x_start || smp->y_end <= smp->y_start)
        return set_error(PBRT_ERR_INVALID_ARGUMENT, "empty sampler window");
    const uint32_t spp = smp->x_samples * smp->y_samples;
    if (spp == 0 || spp > 64) return set_error(PBRT_ERR_UNSUPPORTED, "samples per pixel must be in [1, 64]");
    if (cam->x_res == 0 || cam->y_res == 0) return set_error(PBRT_ERR_INVALID_ARGUMENT, "empty film");
    if (!(cam->filter_x_width > 0.0f) || !(cam->filter_y_width > 0.0f) || cam->filter_x_width > 16.0f ||
        cam->filter_y_width > 16.0f)
        return set_error(PBRT_ERR_INVALID_ARGUMENT, "filter width must be in (0, 16]");
    if (cam->filter_kind < PBRT_FILTER_BOX || cam->filter_kind > PBRT_FILTER_LANCZOS)
        return set_error(PBRT_ERR_INVALID_ARGUMENT, "unknown filter kind");
    int st;
    if (!S->uploaded && (st = scene_upload(S))) return st;
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

    // tasks (sampler_renderer.rs:61-75, film.rs:124-147)
    std::vector<TaskRec> tasks(smp->num_tasks);
    const float aspect = (float)cam->x_res / (float)cam->y_res;
    const float* crop = cam->crop_window;
    for (uint32_t t = 0; t < smp->num_tasks; ++t) {
        TaskRec& T = tasks[t];
        std::memset(&T, 0, sizeof(T));
        int32_t w[4];
        sub_window(*smp, t, w);
        chacha_key(t, T.key);
        if (w[0] == w[1] || w[2] == w[3]) continue;  // get_sub_sampler -> None: the task does nothing
        if (t < task_lo || t >= task_hi) continue;   // another shard's task: owns no pixel here
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
        // add_sub_film copies the task film into the main film
        T.fx0 = std::max(te[0], P.fx0);
        T.fx1 = std::min(te[1], P.fx1);
        T.fy0 = std::max(te[2], P.fy0);
        T.fy1 = std::min(te[3], P.fy1);
    }
    scene_params(S, &P);
    *out = P;
    *tasks_out = std::move(tasks);
    return PBRT_OK;
}

}  // namespace pbrt

extern "C" {

int pbrtgpu_scene_device_bytes(const PbrtScene* S, uint64_t* bytes) {
    if (!S || !bytes) return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
    uint64_t n = 0;
    int st = pbrtgpu_bvh_device_bytes(S->bvh, &n);
    if (st) return st;
    n += S->shade.size() * sizeof(ShadePrim) + S->materials.size() * sizeof(float4) +
         S->lights.size() * sizeof(LightRec) + S->area_tris.size() * sizeof(AreaTri) + S->area_cdf.size() * sizeof(float) +
         S->inst_map.size() * sizeof(uint4) + S->inst_shade.size() * sizeof(InstShade);
    for (const auto& v : S->inst_shade) n += v.size() * sizeof(ShadePrim);
    *bytes = n;
    return PBRT_OK;
}

int pbrtgpu_chacha_blocks(const uint32_t key[8], uint64_t counter, uint64_t stream_id, uint32_t rounds,
                          uint32_t paired, uint32_t n_blocks, uint32_t* out) {
    if (!key || (!out && n_blocks)) return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (rounds != 8 && rounds != 12 && rounds != 20)
        return set_error(PBRT_ERR_INVALID_ARGUMENT, "rounds must be 8, 12 or 20");
    if (n_blocks > (1u << 20)) return set_error(PBRT_ERR_INVALID_ARGUMENT, "at most 2^20 blocks per call");
    if (paired && (n_blocks & 1u)) return set_error(PBRT_ERR_INVALID_ARGUMENT, "the paired routine needs an even count");
    if (!n_blocks) return PBRT_OK;
    if (!cuda_device_present()) return set_error(PBRT_ERR_NO_DEVICE, "no CUDA device");
    const size_t bytes = (size_t)n_blocks * 64;
    uint32_t* d = nullptr;
    int st = cuda_status(cudaMalloc((void**)&d, bytes), "cudaMalloc");
    if (!st) st = cuda_status(launch_chacha_blocks(key, counter, stream_id, rounds, paired != 0, n_blocks, d, 0),
                              "chacha launch");
    if (!st) st = cuda_status(cudaMemcpy(out, d, bytes, cudaMemcpyDeviceToHost), "D2H");
    if (d) cudaFree(d);
    return st;
}

int pbrtgpu_rng_words(uint64_t seed, uint64_t first_word, uint32_t n_words, uint32_t segment, uint32_t* out) {
    if (!out && n_words) return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (segment == 0 || segment > 4096) return set_error(PBRT_ERR_INVALID_ARGUMENT, "segment must be in [1, 4096]");
    if (n_words > (1u << 24)) return set_error(PBRT_ERR_INVALID_ARGUMENT, "at most 2^24 words per call");
    if (first_word > UINT64_MAX - n_words - 64)
        return set_error(PBRT_ERR_INVALID_ARGUMENT, "word range past the end of the stream");
    if (!n_words) return PBRT_OK;
    if (!cuda_device_present()) return set_error(PBRT_ERR_NO_DEVICE, "no CUDA device");
    uint32_t key[8];
    chacha_key(seed, key);
    const size_t bytes = (size_t)n_words * 4;
    uint32_t* d = nullptr;
    int st = cuda_status(cudaMalloc((void**)&d, bytes), "cudaMalloc");
    if (!st) st = cuda_status(launch_rng_words(key, first_word, n_words, segment, d, 0), "rng launch");
    if (!st) st = cuda_status(cudaMemcpy(out, d, bytes, cudaMemcpyDeviceToHost), "D2H");
    if (d) cudaFree(d);
    return st;
}

int pbrtgpu_render_tasks(const PbrtScene* cS, const PbrtCameraDesc* cam, const PbrtSamplerDesc* smp,
                         uint32_t task_lo, uint32_t task_hi, float* rgb_out, void* stream_v) {
    PbrtScene* S = const_cast<PbrtScene*>(cS);
    if (!S || !cam || !smp || !rgb_out) return set_error(PBRT_ERR_INVALID_ARGUMENT, "NULL argument");
    RenderParams P;
    std::vector<TaskRec> tasks;
    int st = prepare_render(S, cam, smp, task_lo, task_hi, &P, &tasks);
    if (st) return st;
    DeviceGuard g(S->bvh->device);
    std::lock_guard<std::mutex> lk(S->mu);
    cudaStream_t s = (cudaStream_t)stream_v;
    const uint32_t nl = P.n_lights;
    std::vector<float> table(256);
    filter_table(*cam, table.data());  // kind checked by prepare_render

    const uint64_t S_ = P.n_samples, SL = P.n_samples * (uint64_t)nl;
    const uint64_t npx = (uint64_t)(P.fx1 - P.fx0) * (uint64_t)(P.fy1 - P.fy0);
    if ((st = S->rays.reserve(S_ * sizeof(PbrtRay))) || (st = S->hits.reserve(S_ * 16)) ||
        (st = S->img.reserve(S_ * 8)) || (st = S->pixbox.reserve((uint64_t)P.n_pixels * 16)) ||
        (st = S->lsamp.reserve(S_ * 3 * nl * 4 + 4)) ||
        (st = S->contrib.reserve(SL * 16 + 16)) || (st = S->le.reserve(S_ * 16)) || (st = S->L.reserve(S_ * 16)) ||
        (st = S->srays.reserve(SL * sizeof(PbrtRay) + 32)) || (st = S->sslot.reserve(SL * 4 + 4)) ||
        (st = S->occ.reserve(SL + 1)) || (st = S->counters.reserve(64)) ||
        (st = S->tasks.reserve(tasks.size() * sizeof(TaskRec))) || (st = S->table.reserve(256 * 4)))
        return st;
    bool dev_out = is_device_pointer(rgb_out);
    if (!dev_out && (st = S->rgb.reserve(npx * 3 * 4))) return st;
    if ((st = cuda_status(cudaMemcpyAsync(S->tasks.p, tasks.data(), tasks.size() * sizeof(TaskRec),
                                          cudaMemcpyHostToDevice, s),
                          "tasks H2D")) ||
        (st = cuda_status(cudaMemcpyAsync(S->table.p, table.data(), 256 * 4, cudaMemcpyHostToDevice, s), "table H2D")) ||
        (st = cuda_status(cudaMemsetAsync(S->counters.p, 0, 64, s), "counters")))
        return st;
    P.filter_table = (const float*)S->table.p;
    P.tasks = (const TaskRec*)S->tasks.p;
    P.n_tasks = smp->num_tasks;
    P.rays = (PbrtRay*)S->rays.p;
    P.hits = (float4*)S->hits.p;
    P.img = (float2*)S->img.p;
    P.pixbox = (float4*)S->pixbox.p;
    P.lsamp = (float*)S->lsamp.p;
    P.contrib = (float4*)S->contrib.p;
    P.le = (float4*)S->le.p;
    P.L = (float4*)S->L.p;
    P.shadow_rays = (PbrtRay*)S->srays.p;
    P.shadow_slot = (uint32_t*)S->sslot.p;
    P.counters = (uint32_t*)S->counters.p;
    P.occluded = (uint8_t*)S->occ.p;
    P.rgb = dev_out ? rgb_out : (float*)S->rgb.p;
    if ((st = cuda_status(launch_render(P, s), "render launch"))) return st;
    if (!dev_out &&
        (st = cuda_status(cudaMemcpyAsync(rgb_out, S->rgb.p, npx * 3 * 4, cudaMemcpyDeviceToHost, s), "rgb D2H")))
        return st;
    uint32_t cnt[4] = {0, 0, 0, 0};
    if ((st = cuda_status(cudaMemcpyAsync(cnt, S->counters.p, sizeof(cnt), cudaMemcpyDeviceToHost, s), "counters")))
        return st;
    if ((st = cuda_status(cudaStreamSynchronize(s), "cudaStreamSynchronize"))) return st;
    if (cnt[2]) return set_error((int)cnt[2], "device-side traversal failure");
    if (cnt[1])
        return set_error(PBRT_ERR_NAN, std::to_string(cnt[1]) + " radiance samples were NaN (sampler_renderer.rs:105)");
    return PBRT_OK;
}

}  // extern "C"
