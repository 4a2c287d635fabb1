// trace4.cuh - traversal over the 4-wide layout (layout.h: Node4).
//
// Each Node4 holds the four grandchildren of one binary node N of the
// reference tree.  A visit tests the four child boxes against the current
// maxt and orders the hits exactly as BVHAccelerator::intersect
// (src/primitive/aggregates/bvh.rs:390-417) would visit them: N's children
// in dir_is_neg[axis(N)] order, and inside each, that child's children in
// dir_is_neg order of its own axis.  The reference also tests the boxes of
// N's two children; skipping them changes nothing: each is the union of
// its children's boxes, so its planes are among theirs, and because f32
// subtraction and multiplication are monotone the child's slab interval
// always lies inside the parent's - a child that passes implies a parent
// that passes.  The deferred children are pushed with their entry
// distance t0 and re-checked against maxt when popped (see trace.cuh), so
// every box decision, every primitive test and their order are the
// reference's, and results are bit-identical to it, ties included.
//
// The stack lives in shared memory (SMAX 8-byte entries per thread,
// [entry][thread] so a warp's accesses hit distinct banks) with an
// optional local-memory overflow of OVF entries; the host picks a variant
// whose SMAX + OVF covers the tree's bound (HostBVH::stack4_bound).
// INST: the tree may hold instance records (kernels take it only for
// scenes that have instances).
#pragma once
#include <stdint.h>

#include "layout.h"
#include "trace.cuh"

namespace pbrt {

struct DevBVH4 {
    const Node4* nodes;
    const PrimRec* prims;
    const SphereRec* spheres;
    ChildRec root;
    uint32_t empty;
    const DevBVH4* insts;  // the instance definitions' BVHs (kQuadInstance records index it)
};

struct ChildV {
    float lx, ly, lz, hx, hy, hz;
    uint32_t a, b;
};

__device__ __forceinline__ ChildV ld_child(const ChildRec* c) {
    ChildV v;
    float f0, f1, f2, f3, f4, f5, f6, f7;
    asm volatile("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=f"(f0), "=f"(f1), "=f"(f2), "=f"(f3), "=f"(f4), "=f"(f5), "=f"(f6), "=f"(f7)
                 : "l"(c));
    v.lx = f0;
    v.ly = f1;
    v.lz = f2;
    v.a = __float_as_uint(f3);
    v.hx = f4;
    v.hy = f5;
    v.hz = f6;
    v.b = __float_as_uint(f7);
    return v;
}

// The same record through two 128-bit loads.
__device__ __forceinline__ ChildV ld_child_v4(const ChildRec* c) {
    ChildV v;
    const float4 a = __ldg(reinterpret_cast<const float4*>(c)), b = __ldg(reinterpret_cast<const float4*>(c) + 1);
    v.lx = a.x;
    v.ly = a.y;
    v.lz = a.z;
    v.a = __float_as_uint(a.w);
    v.hx = b.x;
    v.hy = b.y;
    v.hz = b.z;
    v.b = __float_as_uint(b.w);
    return v;
}

// Swaps two (child word, hit, entry distance) entries when c.
__device__ __forceinline__ void cswap(bool c, uint32_t& a, uint32_t& b, bool& ha, bool& hb, float& ta, float& tb) {
    const uint32_t x = c ? b : a, y = c ? a : b;
    const bool hx = c ? hb : ha, hy = c ? ha : hb;
    const float tx = c ? tb : ta, ty = c ? ta : tb;
    a = x;
    b = y;
    ha = hx;
    hb = hy;
    ta = tx;
    tb = ty;
}

// Stack word that ends the walk of an instance definition (never a leaf:
// primitive offsets stay below 0x7ffffffe).
constexpr uint32_t kExitInst = 0xfffffffeu;

// LD256: fetch child records with one 256-bit load each (else two 128-bit
// loads; the nested instance walk of the binary kernels lives in an
// out-of-line function, where nvcc 13.0's back end crashes on the 256-bit
// form).
//
// INST: the tree may hold instance records.  An instance is walked in the
// same loop as the scene's tree (TransformedPrimitive::intersect,
// transformed.rs:35-56): when its leaf entry is reached and the
// primitive-space ray w2p(ray) - o as a point, d as a vector, mint and the
// current maxt kept - passes the definition's root box, the walk pushes the
// rest of the leaf and an exit word (both with entry distance -inf, so they
// are always taken) and continues in the definition's tree with that ray;
// popping the exit word restores the world ray and the scene's tree.  The
// definition is thus searched completely, in the reference's order, before
// the leaf's next primitive, and the shared maxt is the reference's
// ray.set_maxt.  Hits inside report the instance's first id + the
// definition-local index.  The stack bound of such a tree includes the
// largest definition's bound + 2 (HostBVH::stack4_bound).
// INST walks' extra state: the arrays of the tree being walked, the world
// ray while inside an instance, and the instance's first id (0 outside).
template <bool INST>
struct InstWalk {
    const Node4* nodes_;
    const PrimRec* prims_;
    const SphereRec* spheres_;
    DRay world_;  // the world ray while inside an instance
    uint32_t base_;
};
template <>
struct InstWalk<false> {};

//
// EXACT: the replay walk (Traversal in trace.cuh): children are pushed on
// their box alone and checked against maxt when taken.
template <int SMAX, int OVF, bool INST = false, bool LD256 = true, bool EXACT = false>
struct Traversal4 : InstWalk<INST> {
    float maxt;
    uint32_t cur;
    int sp;
    bool found;
    bool overflow;
    bool nan_hit;  // a NaN-distance hit was accepted: the result needs an EXACT replay
    TraceResult res;
    uint2* sstack;  // this thread's column: entry k at sstack[k * stride]
    uint32_t stride;
    uint2 ov[OVF > 0 ? OVF : 1];

    __device__ __forceinline__ void bind(uint2* smem, uint32_t tid, uint32_t nthreads) {
        sstack = smem + tid;
        stride = nthreads;
    }

    __device__ __forceinline__ const Node4* node_base(const DevBVH4& bvh) const {
        if constexpr (INST)
            return this->nodes_;
        else
            return bvh.nodes;
    }
    __device__ __forceinline__ const PrimRec* prim_base(const DevBVH4& bvh) const {
        if constexpr (INST)
            return this->prims_;
        else
            return bvh.prims;
    }
    __device__ __forceinline__ const SphereRec* sphere_base(const DevBVH4& bvh) const {
        if constexpr (INST)
            return this->spheres_;
        else
            return bvh.spheres;
    }

    __device__ __forceinline__ bool start(const DevBVH4& bvh, const DRay& r) {
        maxt = r.tmax;
        found = false;
        overflow = false;
        nan_hit = false;
        sp = 0;
        res.prim = -1;
        res.t = 0.0f;
        res.b1 = 0.0f;
        res.b2 = 0.0f;
        if constexpr (INST) {
            this->nodes_ = bvh.nodes;
            this->prims_ = bvh.prims;
            this->spheres_ = bvh.spheres;
            this->base_ = 0;
        }
        if (bvh.empty) return false;
        float tr;
        const ChildRec& R = bvh.root;
        if (!slab(R.lo_x, R.lo_y, R.lo_z, R.hi_x, R.hi_y, R.hi_z, r, maxt, &tr)) return false;
        cur = R.a;
        return true;
    }

    // The host only launches a variant whose SMAX + OVF covers the tree's
    // stack bound; a full stack is still caught and reported, never written.
    __device__ __forceinline__ void push(uint32_t ref, float t0) {
        if (sp >= SMAX + OVF) {
            overflow = true;
            return;
        }
        uint2 e = make_uint2(ref, __float_as_uint(t0));
        if (OVF == 0 || sp < SMAX)
            sstack[(uint32_t)sp * stride] = e;
        else
            ov[sp - SMAX] = e;
        ++sp;
    }

    __device__ __forceinline__ bool pop() {
        while (sp > 0) {
            --sp;
            uint2 e = (OVF == 0 || sp < SMAX) ? sstack[(uint32_t)sp * stride] : ov[sp - SMAX];
            if (!(__uint_as_float(e.y) > maxt)) {
                cur = e.x;
                return true;
            }
        }
        return false;
    }

    // INST: starts the walk of instance record S (first id `first`) if the
    // primitive-space ray hits its definition's root box; `resume` is the
    // leaf word of the rest of the current leaf (0: none).
    template <class R>
    __device__ __forceinline__ bool enter(const DevBVH4& bvh, R& r, const SphereRec* S, uint32_t first,
                                          uint32_t resume) {
        float o[3], d[3];
        xf_point(S->w2o, r.ox, r.oy, r.oz, o);  // transform.rs:230-237
        xf_vector(S->w2o, r.dx, r.dy, r.dz, d);
        // (tmax is not read while walking; it keeps the world ray's for a replay)
        const DRay ri = make_dray(make_float4(o[0], o[1], o[2], r.tmin), make_float4(d[0], d[1], d[2], r.tmax));
        const DevBVH4& D = bvh.insts[S->instance];
        float tr;
        const ChildRec& Rt = D.root;
        if (D.empty || !slab(Rt.lo_x, Rt.lo_y, Rt.lo_z, Rt.hi_x, Rt.hi_y, Rt.hi_z, ri, maxt, &tr)) return false;
        if (resume) push(resume, __int_as_float(0xff800000));  // -inf: always taken
        push(kExitInst, __int_as_float(0xff800000));
        this->world_ = r;
        r = ri;
        this->nodes_ = D.nodes;
        this->prims_ = D.prims;
        this->spheres_ = D.spheres;
        this->base_ = first;
        cur = Rt.a;
        return !overflow;
    }

    // INST: back to the scene's tree and the world ray.
    template <class R>
    __device__ __forceinline__ void leave(const DevBVH4& bvh, R& r) {
        r = this->world_;
        this->nodes_ = bvh.nodes;
        this->prims_ = bvh.prims;
        this->spheres_ = bvh.spheres;
        this->base_ = 0;
    }

    // Tests the primitives of leaf `ref` (a kNode4Leaf child word) in
    // order.  Returns 0 when the leaf is done, 1 when ANY and a primitive
    // was hit, 2 when an instance walk was entered (`cur` set).
    template <bool ANY, class R>
    __device__ __forceinline__ int leaf(const DevBVH4& bvh, R& r, uint32_t ref) {
        uint32_t off = ref & ~kNode4Leaf;
        for (;;) {
            const PrimRec* pr = prim_base(bvh) + off;
            float4 r0 = ldg4(pr->r0);
            float4 r1 = ldg4(pr->r1);
            float4 r2 = ldg4(pr->r2);
            uint32_t id = __float_as_uint(r0.w);
            const bool last = (__float_as_uint(r2.w) & kPrimLastBit) != 0;
            float t, b1 = 0.0f, b2 = 0.0f;
            bool hit;
            if (id & kSphereBit) {
                const uint32_t si = __float_as_uint(r1.w);
                if constexpr (INST) {
                    const SphereRec* S = sphere_base(bvh) + si;
                    if (S->kind == kQuadInstance) {  // only in the scene's tree: definitions hold none
                        if (enter(bvh, r, S, id & ~kSphereBit, last ? 0u : (kNode4Leaf | (off + 1)))) return 2;
                        if (last) return 0;
                        ++off;
                        continue;
                    }
                }
                hit = sphere_test(sphere_base(bvh), si, r, maxt, &t);
            } else {
                hit = tri_test(r0, r1, r2, r, maxt, &t, &b1, &b2);
            }
            if (hit) {
                maxt = t;
                found = true;
                nan_hit |= !(t == t);
                if constexpr (INST)
                    res.prim = (int32_t)(this->base_ + (id & ~kSphereBit));
                else
                    res.prim = (int32_t)(id & ~kSphereBit);
                res.t = t;
                res.b1 = b1;
                res.b2 = b2;
                if (ANY) return 1;
            }
            if (last) return 0;
            ++off;
        }
    }

    // One unit of work; false once the ray is finished.
    template <bool ANY, class R>
    __device__ __forceinline__ bool step(const DevBVH4& bvh, R& r) {
        if constexpr (INST) {
            if (cur == kExitInst) {
                leave(bvh, r);
                return pop();
            }
        }
        if (cur & kNode4Leaf) {
            const int st = leaf<ANY>(bvh, r, cur);
            if (st == 1) return false;
            if (INST && st == 2) return !overflow;
            return pop();
        }
        return node<ANY>(bvh, r);
    }

    // Visits inner node `cur`: tests its children and moves `cur` to the
    // next node or leaf in the reference's order (an any-hit walk: nearest
    // entry first); false once nothing is left.
    template <bool ANY>
    __device__ __forceinline__ bool node(const DevBVH4& bvh, const DRay& r) {
        const Node4* nd = node_base(bvh) + cur;
        ChildV c0, c1, c2, c3;
        if (LD256) {
            c0 = ld_child(&nd->c[0]);
            c1 = ld_child(&nd->c[1]);
            c2 = ld_child(&nd->c[2]);
            c3 = ld_child(&nd->c[3]);
        } else {
            c0 = ld_child_v4(&nd->c[0]);
            c1 = ld_child_v4(&nd->c[1]);
            c2 = ld_child_v4(&nd->c[2]);
            c3 = ld_child_v4(&nd->c[3]);
        }
        float t0, t1, t2, t3;
        bool h0, h1, h2, h3;
        const float lim = EXACT ? __int_as_float(0x7f800000) : maxt;  // replay: box alone
        if (r.neg & kRayClean) {
            h0 = c0.a != kNode4Empty && slab_clean(c0.lx, c0.ly, c0.lz, c0.hx, c0.hy, c0.hz, r, lim, &t0);
            h1 = c1.a != kNode4Empty && slab_clean(c1.lx, c1.ly, c1.lz, c1.hx, c1.hy, c1.hz, r, lim, &t1);
            h2 = c2.a != kNode4Empty && slab_clean(c2.lx, c2.ly, c2.lz, c2.hx, c2.hy, c2.hz, r, lim, &t2);
            h3 = c3.a != kNode4Empty && slab_clean(c3.lx, c3.ly, c3.lz, c3.hx, c3.hy, c3.hz, r, lim, &t3);
        } else {
            h0 = c0.a != kNode4Empty && slab(c0.lx, c0.ly, c0.lz, c0.hx, c0.hy, c0.hz, r, lim, &t0);
            h1 = c1.a != kNode4Empty && slab(c1.lx, c1.ly, c1.lz, c1.hx, c1.hy, c1.hz, r, lim, &t1);
            h2 = c2.a != kNode4Empty && slab(c2.lx, c2.ly, c2.lz, c2.hx, c2.hy, c2.hz, r, lim, &t2);
            h3 = c3.a != kNode4Empty && slab(c3.lx, c3.ly, c3.lz, c3.hx, c3.hy, c3.hz, r, lim, &t3);
        }
        if (!(h0 | h1 | h2 | h3)) return pop();
        const uint32_t meta = c0.b;
        const bool sN = (r.neg >> (meta & 3u)) & 1u;
        const bool sL = (r.neg >> ((meta >> 2) & 3u)) & 1u;
        const bool sR = (r.neg >> ((meta >> 4) & 3u)) & 1u;
        // into visit order (bvh.rs:409-415): each child's pair of children
        // by that child's axis sign, then the two pairs by N's
        uint32_t a0 = c0.a, a1 = c1.a, a2 = c2.a, a3 = c3.a;
        if (ANY && !EXACT) {
            // An any-hit walk's answer does not depend on the order it takes
            // children in (some primitive whose boxes all pass the ray's own
            // maxt is hit, or none is), so it takes them by entry distance:
            // an occluder near the ray's origin is met sooner.  Children that
            // fail sort last; a five-comparator network sorts the four.
            const float inf = __int_as_float(0x7f800000);
            t0 = h0 ? t0 : inf;
            t1 = h1 ? t1 : inf;
            t2 = h2 ? t2 : inf;
            t3 = h3 ? t3 : inf;
            cswap(t0 > t1, a0, a1, h0, h1, t0, t1);
            cswap(t2 > t3, a2, a3, h2, h3, t2, t3);
            cswap(t0 > t2, a0, a2, h0, h2, t0, t2);
            cswap(t1 > t3, a1, a3, h1, h3, t1, t3);
            cswap(t1 > t2, a1, a2, h1, h2, t1, t2);
        } else {
            cswap(sL, a0, a1, h0, h1, t0, t1);
            cswap(sR, a2, a3, h2, h3, t2, t3);
            cswap(sN, a0, a2, h0, h2, t0, t2);
            cswap(sN, a1, a3, h1, h3, t1, t3);
        }
        if (EXACT) {
            // replay: the reference takes the first child whose box passes
            // maxt now, culls the ones before it now, and tests the pushed
            // ones against maxt when it pops them
            bool scan = true;
            if (scan && h0) {
                if (t0 > maxt) h0 = false; else scan = false;
            }
            if (scan && h1) {
                if (t1 > maxt) h1 = false; else scan = false;
            }
            if (scan && h2) {
                if (t2 > maxt) h2 = false; else scan = false;
            }
            if (scan && h3 && t3 > maxt) h3 = false;
            if (!(h0 | h1 | h2 | h3)) return pop();
        }
        const int first = h0 ? 0 : (h1 ? 1 : (h2 ? 2 : 3));
        if (h3 && first < 3) push(a3, t3);
        if (h2 && first < 2) push(a2, t2);
        if (h1 && first < 1) push(a1, t1);
        cur = first == 0 ? a0 : (first == 1 ? a1 : (first == 2 ? a2 : a3));
        return !overflow;
    }
};

// An instance definition's stack bound (HostBVH::stack4_bound) is at most
// kInstStack4 (checked at creation), so the nested stack never overflows.
constexpr int kInstStack4 = 96;

template <bool ANY>
__device__ __noinline__ TraceResult instance_test(const DevBVH4* insts, const SphereRec* s, float ox, float oy,
                                                  float oz, float dx, float dy, float dz, float tmin, float maxt) {
    float o[3], d[3];
    xf_point(s->w2o, ox, oy, oz, o);  // transform.rs:230-237: o as a point, d as a vector
    xf_vector(s->w2o, dx, dy, dz, d);
    DRay ri = make_dray(make_float4(o[0], o[1], o[2], tmin), make_float4(d[0], d[1], d[2], maxt));
    const DevBVH4& B = insts[s->instance];
    Traversal4<0, kInstStack4, false, false> T;  // the whole stack in local memory
    if (T.start(B, ri)) {
        while (T.template step<ANY>(B, ri)) {
        }
    }
    if (ANY || !T.nan_hit) return T.res;
    Traversal4<0, kInstStack4, false, false, true> E;  // replay
    if (E.start(B, ri)) {
        while (E.template step<false>(B, ri)) {
        }
    }
    return E.res;
}

}  // namespace pbrt
