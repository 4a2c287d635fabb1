// trace.cuh - device BVH traversal (closest hit and any hit).
//
// Semantics follow BVHAccelerator::intersect
// (src/primitive/aggregates/bvh.rs:375-422) exactly:
//  * the slab test of src/bbox.rs:185-209 with inv_dir = 1/d per axis,
//    fmaxf/fminf (Rust f32::max/min) and the reference operation order;
//  * the Moller-Trumbore test of src/shape/mesh.rs:41-72 with inclusive
//    [mint, maxt] and maxt shrunk to every accepted hit
//    (src/primitive/geometric.rs:64), so a later primitive at equal t
//    replaces an earlier one;
//  * the sphere test of src/shape/sphere.rs:46-107 in object space;
//  * the reference visiting order: the child that BVHAccelerator pops
//    first (child1 unless dir_is_neg[axis]) is traversed first.
// Instead of testing a node's box when it is popped, both child boxes are
// tested at the parent (one 64-byte pair fetch) and the deferred child is
// pushed with its entry distance t0.  A box test passes iff
// t0 <= min(far planes, maxt); t0 does not depend on maxt and the far part
// was checked at push time, so re-checking t0 <= maxt at pop gives the
// reference's decision.  Hit indices, t and barycentrics are therefore the
// reference's bit for bit (the library is built with --fmad=false and
// IEEE division/sqrt).
#pragma once
#include <stdint.h>

#include "layout.h"

namespace pbrt {

struct DevBVH4;  // trace4.cuh

struct DevBVH {
    const NodePair* pairs;
    const PrimRec* prims;
    const SphereRec* spheres;
    ChildRec root;
    uint32_t has_spheres;
    uint32_t n_prims;
    uint32_t empty;
    const DevBVH4* insts;  // the instance definitions' BVHs (kQuadInstance records index it)
};

struct DRay {
    float ox, oy, oz, tmin;
    float dx, dy, dz, tmax;
    float ix, iy, iz;  // 1/d
    uint32_t neg;      // bit i: inv_dir[i] < 0 (bvh.rs:383); kRayClean
};

// DRay::neg bit: origin and 1/d finite, tmin and tmax not NaN (slab_clean).
constexpr uint32_t kRayClean = 8u;

__device__ __forceinline__ bool finite3(float a, float b, float c) {
    return fabsf(a) <= 3.402823466e38f && fabsf(b) <= 3.402823466e38f && fabsf(c) <= 3.402823466e38f;
}

__device__ __forceinline__ DRay make_dray(float4 a, float4 b) {
    DRay r;
    r.ox = a.x;
    r.oy = a.y;
    r.oz = a.z;
    r.tmin = a.w;
    r.dx = b.x;
    r.dy = b.y;
    r.dz = b.z;
    r.tmax = b.w;
    r.ix = 1.0f / r.dx;
    r.iy = 1.0f / r.dy;
    r.iz = 1.0f / r.dz;
    r.neg = (r.ix < 0.0f ? 1u : 0u) | (r.iy < 0.0f ? 2u : 0u) | (r.iz < 0.0f ? 4u : 0u);
    if (finite3(r.ix, r.iy, r.iz) && finite3(r.ox, r.oy, r.oz) && r.tmin == r.tmin && r.tmax == r.tmax)
        r.neg |= kRayClean;
    return r;
}

// src/bbox.rs:185-209 for one box; returns t0 in *t_enter on a pass.
__device__ __forceinline__ bool slab(float lox, float loy, float loz, float hix, float hiy, float hiz, const DRay& r,
                                     float maxt, float* t_enter) {
    float t0 = r.tmin, t1 = maxt;
    float ta = (lox - r.ox) * r.ix, tb = (hix - r.ox) * r.ix;
    float tn = ta > tb ? tb : ta, tf = ta > tb ? ta : tb;
    t0 = fmaxf(tn, t0);
    t1 = fminf(tf, t1);
    ta = (loy - r.oy) * r.iy;
    tb = (hiy - r.oy) * r.iy;
    tn = ta > tb ? tb : ta;
    tf = ta > tb ? ta : tb;
    t0 = fmaxf(tn, t0);
    t1 = fminf(tf, t1);
    ta = (loz - r.oz) * r.iz;
    tb = (hiz - r.oz) * r.iz;
    tn = ta > tb ? tb : ta;
    tf = ta > tb ? ta : tb;
    t0 = fmaxf(tn, t0);
    t1 = fminf(tf, t1);
    *t_enter = t0;
    return !(t0 > t1);
}

__device__ __forceinline__ float max3f(float a, float b, float c) {
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
__device__ __forceinline__ float min3f(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

// slab() for a kRayClean ray.  Its products (lo - o) * (1/d) can be NaN
// only where a box coordinate is NaN, and a box built from unions and
// transforms of the same points has lo NaN exactly where hi is NaN.  So
// the reference's "swap if tnear > tfar" is min/max, an all-NaN axis drops
// out of min/max as it drops out of the reference's comparisons, and the
// four entry bounds (tmin and the three near planes) and four exit bounds
// combine in any order: the same t0 and the same decision, in fewer
// instructions.
__device__ __forceinline__ bool slab_clean(float lox, float loy, float loz, float hix, float hiy, float hiz,
                                           const DRay& r, float maxt, float* t_enter) {
    const float ax = (lox - r.ox) * r.ix, bx = (hix - r.ox) * r.ix;
    const float ay = (loy - r.oy) * r.iy, by = (hiy - r.oy) * r.iy;
    const float az = (loz - r.oz) * r.iz, bz = (hiz - r.oz) * r.iz;
    const float t0 = max3f(fminf(ax, bx), fminf(ay, by), fmaxf(fminf(az, bz), r.tmin));
    const float t1 = min3f(fmaxf(ax, bx), fmaxf(ay, by), fminf(fmaxf(az, bz), maxt));
    *t_enter = t0;
    return !(t0 > t1);
}

// src/shape/mesh.rs:41-72 with e1, e2 precomputed (same f32 subtraction).
__device__ __forceinline__ bool tri_test(float4 r0, float4 r1, float4 r2, const DRay& r, float maxt, float* t_out,
                                         float* b1_out, float* b2_out) {
    float e1x = r1.x, e1y = r1.y, e1z = r1.z;
    float e2x = r2.x, e2y = r2.y, e2z = r2.z;
    float s1x = (r.dy * e2z) - (r.dz * e2y);
    float s1y = (r.dz * e2x) - (r.dx * e2z);
    float s1z = (r.dx * e2y) - (r.dy * e2x);
    float divisor = s1x * e1x + s1y * e1y + s1z * e1z;
    if (divisor == 0.0f) return false;
    float inv = 1.0f / divisor;
    float sx = r.ox - r0.x, sy = r.oy - r0.y, sz = r.oz - r0.z;
    float b1 = (s1x * sx + s1y * sy + s1z * sz) * inv;
    if (b1 < 0.0f || b1 > 1.0f) return false;
    float s2x = (sy * e1z) - (sz * e1y);
    float s2y = (sz * e1x) - (sx * e1z);
    float s2z = (sx * e1y) - (sy * e1x);
    float b2 = (r.dx * s2x + r.dy * s2y + r.dz * s2z) * inv;
    if (b2 < 0.0f || (b1 + b2) > 1.0f) return false;
    float t = (e2x * s2x + e2y * s2y + e2z * s2z) * inv;
    if (t < r.tmin || t > maxt) return false;
    *t_out = t;
    *b1_out = b1;
    *b2_out = b2;
    return true;
}

// src/transform/transform.rs:195-218 (point with the w != 1 divide; vector)
__device__ __forceinline__ void xf_point(const float* m, float x, float y, float z, float* o) {
    float xt = m[0] * x + m[1] * y + m[2] * z + m[3];
    float yt = m[4] * x + m[5] * y + m[6] * z + m[7];
    float zt = m[8] * x + m[9] * y + m[10] * z + m[11];
    float w = m[12] * x + m[13] * y + m[14] * z + m[15];
    if (w != 1.0f) {
        xt = xt / w;
        yt = yt / w;
        zt = zt / w;
    }
    o[0] = xt;
    o[1] = yt;
    o[2] = zt;
}
__device__ __forceinline__ void xf_vector(const float* m, float x, float y, float z, float* o) {
    o[0] = m[0] * x + m[1] * y + m[2] * z;
    o[1] = m[4] * x + m[5] * y + m[6] * z;
    o[2] = m[8] * x + m[9] * y + m[10] * z;
}

// src/utils/mod.rs:56-92
__device__ __forceinline__ bool quadratic(float a, float b, float c, float* t0, float* t1) {
    float descrim = b * b - 4.0f * a * c;
    if (descrim < 0.0f) return false;
    if (fabsf(descrim) < 1e-6f) {
        if (a == 0.0f) return false;
        float t = -b / (2.0f * a);
        *t0 = t;
        *t1 = t;
        return true;
    }
    float root = sqrtf(descrim);
    float q = b < 0.0f ? -0.5f * (b - root) : -0.5f * (b + root);
    if (a == 0.0f) return false;
    float r0 = q / a, r1 = c / q;
    if (r0 < r1) {
        *t0 = r0;
        *t1 = r1;
    } else {
        *t0 = r1;
        *t1 = r0;
    }
    return true;
}

// src/shape/sphere.rs:46-107 on the object-space ray (o, d).  For full
// spheres the clip test cannot reject (see SphereRec::full) and is
// skipped; partial spheres evaluate it with CUDA's atan2f.
__device__ __forceinline__ bool sphere_obj_test(const SphereRec& s, const float* o, const float* d, float mint,
                                                float maxt, float* t_out) {
    float a = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    float b = 2.0f * (d[0] * o[0] + d[1] * o[1] + d[2] * o[2]);
    float c = (o[0] * o[0] + o[1] * o[1] + o[2] * o[2]) - s.radius * s.radius;
    float t0, t1;
    if (!quadratic(a, b, c, &t0, &t1)) return false;
    if (t0 > maxt || t1 < mint) return false;
    float th = t0;
    if (t0 < mint) {
        th = t1;
        if (th > maxt) return false;
    }
    if (!s.full) {
        auto invalid = [&](float t) {
            float hx = o[0] + d[0] * t, hy = o[1] + d[1] * t, hz = o[2] + d[2] * t;
            if (hx == 0.0f && hy == 0.0f) hx = 1e-5f * s.radius;
            float phi = atan2f(hy, hx);
            if (phi < 0.0f) phi += 2.0f * 3.14159265358979323846f;
            return (hz > -s.radius && hz < s.z_min) || (hz < s.radius && hz > s.z_max) || (phi > s.phi_max);
        };
        if (invalid(th)) {
            if (th == t1) return false;
            if (t1 > maxt) return false;
            th = t1;
            if (invalid(th)) return false;
        }
    }
    *t_out = th;
    return true;
}

__device__ __forceinline__ float phi_of(float x, float y) {  // atan2, moved to [0, 2 pi)
    float a = atan2f(y, x);
    if (a < 0.0f) a += 2.0f * 3.14159265358979323846f;
    return a;
}

// src/shape/disk.rs:36-66 on the object-space ray.
__device__ __forceinline__ bool disk_obj_test(const SphereRec& s, const float* o, const float* d, float mint,
                                              float maxt, float* t_out) {
    if (fabsf(d[2]) < 1e-6f) return false;
    const float t = (s.height - o[2]) / d[2];
    if (t < mint || t > maxt) return false;
    const float px = o[0] + d[0] * t, py = o[1] + d[1] * t;
    const float dist2 = px * px + py * py;
    if (dist2 > (s.radius * s.radius) || dist2 < (s.inner_radius * s.inner_radius)) return false;
    if (!s.full && phi_of(px, py) > s.phi_max) return false;
    *t_out = t;
    return true;
}

// src/shape/cylinder.rs:38-94 on the object-space ray; the z clip always
// applies, the phi clip only to partial cylinders.
__device__ __forceinline__ bool cylinder_obj_test(const SphereRec& s, const float* o, const float* d, float mint,
                                                  float maxt, float* t_out) {
    const float a = d[0] * d[0] + d[1] * d[1];
    const float b = 2.0f * (d[0] * o[0] + d[1] * o[1]);
    const float c = o[0] * o[0] + o[1] * o[1] - s.radius * s.radius;
    float t0, t1;
    if (!quadratic(a, b, c, &t0, &t1)) return false;
    if (t0 > maxt || t1 < mint) return false;
    float th = t0;
    if (t0 < mint) {
        th = t1;
        if (th > maxt) return false;
    }
    auto invalid = [&](float t) {
        float hx = o[0] + d[0] * t, hy = o[1] + d[1] * t, hz = o[2] + d[2] * t;
        if (hz < s.z_min || hz > s.z_max) return true;
        if (s.full) return false;
        if (hx == 0.0f && hy == 0.0f) hx = 1e-5f * s.radius;
        return phi_of(hx, hy) > s.phi_max;
    };
    if (invalid(th)) {
        if (th == t1) return false;
        if (t1 > maxt) return false;
        th = t1;
        if (invalid(th)) return false;
    }
    *t_out = th;
    return true;
}

// Any analytic shape (SphereRec::kind) against the world-space ray.
__device__ __forceinline__ bool sphere_test(const SphereRec* spheres, uint32_t si, const DRay& r, float maxt,
                                            float* t_out) {
    const SphereRec& s = spheres[si];
    float o[3], d[3];
    xf_point(s.w2o, r.ox, r.oy, r.oz, o);
    xf_vector(s.w2o, r.dx, r.dy, r.dz, d);
    if (s.kind == kQuadDisk) return disk_obj_test(s, o, d, r.tmin, maxt, t_out);
    if (s.kind == kQuadCylinder) return cylinder_obj_test(s, o, d, r.tmin, maxt, t_out);
    return sphere_obj_test(s, o, d, r.tmin, maxt, t_out);
}

__device__ __forceinline__ float4 ldg4(const void* p) { return __ldg(reinterpret_cast<const float4*>(p)); }

struct TraceResult {
    int32_t prim;
    float t, b1, b2;
};

// TransformedPrimitive::intersect / intersect_p (transformed.rs:35-59) for
// the instance record `s`: the ray (o, d, tmin, maxt) is taken to primitive
// space by w2p (the record's w2o) and traced through the definition's BVH.
// Returns the definition-local hit (prim = its refined index, -1 on a miss);
// the caller's maxt becomes the hit's t, as ray.set_maxt(r.maxt()) does.
// Kept out of line so that the outer traversal's registers do not grow;
// defined in trace4.cuh (the definitions are walked in the 4-wide layout).
template <bool ANY>
__device__ __noinline__ TraceResult instance_test(const DevBVH4* insts, const SphereRec* s, float ox, float oy,
                                                  float oz, float dx, float dy, float dz, float tmin, float maxt);

// One analytic primitive record: an instance (INST and kQuadInstance) or a
// quadric (sphere_test).  *add gets the definition-local index of an
// instance hit, 0 otherwise; *b1 / *b2 are left alone for quadrics.
template <bool INST, bool ANY>
__device__ __forceinline__ bool analytic_test(const SphereRec* spheres, const DevBVH4* insts, uint32_t si,
                                              const DRay& r, float maxt, float* t, float* b1, float* b2,
                                              uint32_t* add) {
    if (INST && spheres[si].kind == kQuadInstance) {
        TraceResult q = instance_test<ANY>(insts, spheres + si, r.ox, r.oy, r.oz, r.dx, r.dy, r.dz, r.tmin, maxt);
        if (q.prim < 0) return false;
        *t = q.t;
        *b1 = q.b1;
        *b2 = q.b2;
        *add = (uint32_t)q.prim;
        return true;
    }
    return sphere_test(spheres, si, r, maxt, t);
}

// Per-ray traversal state.  start() tests the root box; step() does one
// unit of work (one leaf's primitives, or one inner node's two child
// boxes) and then, if needed, pops the next deferred child; it returns
// false once the ray is finished.  Closest hit (ANY = false) or any hit
// (ANY = true, stopping at the first accepted primitive).  INST: the
// tree may hold instance records; kernels take INST only for scenes that
// have instances, so the others keep the registers of the plain walk.
//
// Replay: child boxes are decided against the maxt of the moment they are
// pushed.  The reference decides them when popped; the two agree because
// maxt only shrinks - except that a primitive test with t = NaN (NaN or
// infinite geometry, overflowing products) is accepted by the reference,
// whose later box tests then ignore maxt.  A closest-hit walk that
// accepted such a hit (nan_hit) is therefore replayed from the root by the
// kernels with EXACT, where children are pushed on their box alone and maxt
// is checked when they are taken, as the reference does.
template <int STACK, bool INST = false, bool EXACT = false>
struct Traversal {
    float maxt;
    uint32_t a, b;
    int sp;
    bool found;
    bool nan_hit;  // a NaN-distance hit was accepted: the result needs an EXACT replay
    TraceResult res;
    // deferred children: (a, b, entry distance bits, unused) - one 16-byte
    // local store and load per entry instead of three
    uint4 st[STACK];

    __device__ __forceinline__ bool start(const DevBVH& bvh, const DRay& r) {
        maxt = r.tmax;
        found = false;
        nan_hit = false;
        sp = 0;
        res.prim = -1;
        res.t = 0.0f;
        res.b1 = 0.0f;
        res.b2 = 0.0f;
        if (bvh.empty) return false;
        float tr;
        const ChildRec& R = bvh.root;
        if (!slab(R.lo_x, R.lo_y, R.lo_z, R.hi_x, R.hi_y, R.hi_z, r, maxt, &tr)) return false;
        a = R.a;
        b = R.b;
        return true;
    }

    // `status` gets PBRT_ERR_STACK_OVERFLOW (6) if the stack would overflow
    // (the host checks the tree depth first, so this only guards).
    template <bool ANY>
    __device__ __forceinline__ bool step(const DevBVH& bvh, const DRay& r, int* status) {
        if (b & kLeafBit) {
            uint32_t cnt = b & kCountMask;
            for (uint32_t i = 0; i < cnt; ++i) {
                const PrimRec* pr = bvh.prims + a + i;
                float4 r0 = ldg4(pr->r0);
                uint32_t id = __float_as_uint(r0.w);
                float t, b1 = 0.0f, b2 = 0.0f;
                uint32_t add = 0;
                bool hit;
                if (id & kSphereBit) {
                    float4 r1 = ldg4(pr->r1);
                    hit = analytic_test<INST, ANY>(bvh.spheres, bvh.insts, __float_as_uint(r1.w), r, maxt, &t, &b1,
                                                   &b2, &add);
                } else {
                    float4 r1 = ldg4(pr->r1), r2 = ldg4(pr->r2);
                    hit = tri_test(r0, r1, r2, r, maxt, &t, &b1, &b2);
                }
                if (hit) {
                    maxt = t;
                    found = true;
                    nan_hit |= !(t == t);
                    res.prim = (int32_t)((id & ~kSphereBit) + add);
                    res.t = t;
                    res.b1 = b1;
                    res.b2 = b2;
                    if (ANY) return false;
                }
            }
        } else {
            const NodePair* np = bvh.pairs + a;
            float4 c0a = ldg4(&np->c[0].lo_x), c0b = ldg4(&np->c[0].hi_x);
            float4 c1a = ldg4(&np->c[1].lo_x), c1b = ldg4(&np->c[1].hi_x);
            float t0, t1;
            bool h0, h1;
            const float lim = EXACT ? __int_as_float(0x7f800000) : maxt;  // replay: box alone
            if (r.neg & kRayClean) {
                h0 = slab_clean(c0a.x, c0a.y, c0a.z, c0b.x, c0b.y, c0b.z, r, lim, &t0);
                h1 = slab_clean(c1a.x, c1a.y, c1a.z, c1b.x, c1b.y, c1b.z, r, lim, &t1);
            } else {
                h0 = slab(c0a.x, c0a.y, c0a.z, c0b.x, c0b.y, c0b.z, r, lim, &t0);
                h1 = slab(c1a.x, c1a.y, c1a.z, c1b.x, c1b.y, c1b.z, r, lim, &t1);
            }
            // Near child: child1 unless dir_is_neg[axis] (bvh.rs:409-415).
            // An any-hit walk may take its children in any order - its
            // answer is whether some primitive whose boxes all pass against
            // the ray's own maxt is hit, whatever the order - so it takes the
            // child whose box it enters first, which meets an occluder near
            // the ray's origin sooner (on shadow rays of the serving scenes
            // the oracle counts ~11 % fewer nodes to the first hit).
            bool swap = (ANY && !EXACT) ? (h1 && (!h0 || t1 < t0)) : ((r.neg >> b) & 1u);
            uint32_t na = swap ? __float_as_uint(c1a.w) : __float_as_uint(c0a.w);
            uint32_t nb = swap ? __float_as_uint(c1b.w) : __float_as_uint(c0b.w);
            uint32_t fa = swap ? __float_as_uint(c0a.w) : __float_as_uint(c1a.w);
            uint32_t fb = swap ? __float_as_uint(c0b.w) : __float_as_uint(c1b.w);
            bool hn = swap ? h1 : h0, hf = swap ? h0 : h1;
            float tf = swap ? t0 : t1;
            if (EXACT) {  // a child taken now must also pass maxt now; a pushed one is checked when popped
                const float tn = swap ? t1 : t0;
                hn = hn && !(tn > maxt);
                if (!hn) hf = hf && !(tf > maxt);
            }
            if (hn) {
                if (hf) {
                    if (sp == STACK) {
                        *status = 6;
                        return false;
                    }
                    st[sp] = make_uint4(fa, fb, __float_as_uint(tf), 0u);
                    ++sp;
                }
                a = na;
                b = nb;
                return true;
            }
            if (hf) {
                a = fa;
                b = fb;
                return true;
            }
        }
        // pop the next deferred child whose box still passes; an any-hit
        // walk ends at its first hit, so its maxt is the one the child was
        // pushed against and the child passes without the check
        while (sp > 0) {
            --sp;
            const uint4 e = st[sp];
            if ((ANY && !EXACT) || !(__uint_as_float(e.z) > maxt)) {
                a = e.x;
                b = e.y;
                return true;
            }
        }
        return false;
    }
};

// Whole traversal of one ray.  `*nan_hit`: the closest hit needs an EXACT
// replay (see Traversal).
template <int STACK, bool ANY, bool INST = false, bool EXACT = false>
__device__ __forceinline__ bool traverse(const DevBVH& bvh, const DRay& r, TraceResult* res, int* status,
                                         bool* nan_hit = nullptr) {
    Traversal<STACK, INST, EXACT> T;
    if (T.start(bvh, r)) {
        while (T.template step<ANY>(bvh, r, status)) {
        }
    }
    *res = T.res;
    if (nan_hit) *nan_hit = T.nan_hit;
    return T.found;
}

// A closest hit whose walk accepted a NaN distance is written with this
// prim value and rewritten by the replay kernels.
constexpr int32_t kReplayMark = -2;

// True when every lane of the warp that has a ray (`active`) shares the
// three direction signs, so that every node orders its children the same
// way for all of them.  Called by all 32 lanes.
__device__ __forceinline__ bool warp_signs_uniform(const DRay& r, bool active) {
    const unsigned s = active ? (r.neg & 7u) : 0u;
    const unsigned any1 = __reduce_or_sync(0xffffffffu, s);
    const unsigned all1 = __reduce_and_sync(0xffffffffu, active ? s : 7u);
    return any1 == all1;
}

// Warp-cooperative walk of coherent rays, for warps whose rays share their
// direction signs (warp_signs_uniform); called by all 32 lanes with the SAME
// tree, `active` false for lanes without a ray.  The warp steps through ONE
// node at a time, carrying the mask of lanes whose walk visits it: at an
// inner node every lane of the mask tests both child boxes, the near child
// (the same for every lane: it depends on the signs only) is taken by the
// lanes whose near box passed and the far child is pushed with the lanes
// whose far box passed; at a leaf every lane of the mask tests its
// primitives.  A popped entry keeps the lanes whose entry distance still
// passes their own maxt (closest hit) or that have not hit yet (any hit).
// Each lane so tests exactly the nodes and primitives of its own walk
// (Traversal::step), in the same order and against the same maxt - the
// nodes of the walk are a subsequence of the warp's depth-first order, and
// nothing between two of them changes the lane's state - so its hit, t,
// barycentrics and NaN flag are the per-lane walk's bit for bit.  Every
// branch below depends only on the tree and on warp votes, so the warp stays
// converged at every vote.  Node and primitive records are read at one
// address by the whole warp.  Trees with instances are not walked here.
// `*status` gets PBRT_ERR_STACK_OVERFLOW (6) if the stack would overflow
// (the stack depth is bounded by the tree depth, as per lane).
template <int STACK, bool ANY>
__device__ __forceinline__ bool traverse_packet(const DevBVH& bvh, const DRay& r, bool active, TraceResult* res,
                                                int* status, bool* nan_hit = nullptr) {
    constexpr unsigned kAll = 0xffffffffu;
    const unsigned me = 1u << (threadIdx.x & 31u);
    float maxt = r.tmax;
    bool found = false, nan = false;
    res->prim = -1;
    res->t = 0.0f;
    res->b1 = 0.0f;
    res->b2 = 0.0f;
    if (bvh.empty) return false;
    float tr;
    const ChildRec& R = bvh.root;
    unsigned mask = __ballot_sync(kAll, active && slab(R.lo_x, R.lo_y, R.lo_z, R.hi_x, R.hi_y, R.hi_z, r, maxt, &tr));
    if (!mask) return false;
    // the signs of the lowest active lane (equal for every lane by the precondition)
    const uint32_t neg = __shfl_sync(kAll, r.neg, __ffs(mask) - 1) & 7u;
    unsigned alive = mask;  // any hit: lanes that have not hit yet
    uint32_t a = R.a, b = R.b;
    uint4 st[STACK];  // (child words, entry distance of this lane, lanes that take it)
    int sp = 0;
    for (;;) {
        const bool in = (mask & me) != 0;
        if (b & kLeafBit) {
            const uint32_t cnt = b & kCountMask;
            bool going = in;
            for (uint32_t i = 0; i < cnt; ++i) {
                const PrimRec* pr = bvh.prims + a + i;
                const float4 r0 = ldg4(pr->r0);
                const uint32_t id = __float_as_uint(r0.w);
                float t, b1 = 0.0f, b2 = 0.0f;
                uint32_t add = 0;
                bool hit = false;
                if (id & kSphereBit) {
                    const float4 r1 = ldg4(pr->r1);
                    if (going)
                        hit = analytic_test<false, ANY>(bvh.spheres, bvh.insts, __float_as_uint(r1.w), r, maxt, &t, &b1,
                                                        &b2, &add);
                } else {
                    const float4 r1 = ldg4(pr->r1), r2 = ldg4(pr->r2);
                    if (going) hit = tri_test(r0, r1, r2, r, maxt, &t, &b1, &b2);
                }
                if (hit) {
                    maxt = t;
                    found = true;
                    nan |= !(t == t);
                    res->prim = (int32_t)((id & ~kSphereBit) + add);
                    res->t = t;
                    res->b1 = b1;
                    res->b2 = b2;
                    if (ANY) going = false;
                }
                if (ANY && !__any_sync(kAll, going)) break;
            }
            if (ANY) alive &= ~__ballot_sync(kAll, found);
        } else {
            const NodePair* np = bvh.pairs + a;
            const float4 c0a = ldg4(&np->c[0].lo_x), c0b = ldg4(&np->c[0].hi_x);
            const float4 c1a = ldg4(&np->c[1].lo_x), c1b = ldg4(&np->c[1].hi_x);
            float t0 = 0.0f, t1 = 0.0f;
            bool h0 = false, h1 = false;
            if (in) {
                if (r.neg & kRayClean) {
                    h0 = slab_clean(c0a.x, c0a.y, c0a.z, c0b.x, c0b.y, c0b.z, r, maxt, &t0);
                    h1 = slab_clean(c1a.x, c1a.y, c1a.z, c1b.x, c1b.y, c1b.z, r, maxt, &t1);
                } else {
                    h0 = slab(c0a.x, c0a.y, c0a.z, c0b.x, c0b.y, c0b.z, r, maxt, &t0);
                    h1 = slab(c1a.x, c1a.y, c1a.z, c1b.x, c1b.y, c1b.z, r, maxt, &t1);
                }
            }
            // near child: child1 unless dir_is_neg[axis] (bvh.rs:409-415), one choice for the warp
            const bool swap = (neg >> b) & 1u;
            const uint32_t na = swap ? __float_as_uint(c1a.w) : __float_as_uint(c0a.w);
            const uint32_t nb = swap ? __float_as_uint(c1b.w) : __float_as_uint(c0b.w);
            const uint32_t fa = swap ? __float_as_uint(c0a.w) : __float_as_uint(c1a.w);
            const uint32_t fb = swap ? __float_as_uint(c0b.w) : __float_as_uint(c1b.w);
            const unsigned mn = __ballot_sync(kAll, swap ? h1 : h0);
            const unsigned mf = __ballot_sync(kAll, swap ? h0 : h1);
            if (mn) {
                if (mf) {
                    if (sp == STACK) {
                        *status = 6;
                        break;
                    }
                    st[sp] = make_uint4(fa, fb, __float_as_uint(swap ? t0 : t1), mf);
                    ++sp;
                }
                a = na;
                b = nb;
                mask = mn;
                continue;
            }
            if (mf) {
                a = fa;
                b = fb;
                mask = mf;
                continue;
            }
        }
        // pop the next deferred child some lane still takes
        bool got = false;
        while (sp > 0) {
            --sp;
            const uint4 e = st[sp];
            const unsigned m = e.w & (ANY ? alive : __ballot_sync(kAll, !(__uint_as_float(e.z) > maxt)));
            if (m) {
                a = e.x;
                b = e.y;
                mask = m;
                got = true;
                break;
            }
        }
        if (!got) break;
    }
    if (nan_hit) *nan_hit = nan;
    return found;
}

}  // namespace pbrt
