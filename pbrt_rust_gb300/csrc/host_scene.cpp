// host_scene.cpp - primitive refinement, reference BVH build and device
// layout.  Compiled with -ffp-contract=off: every f32 expression follows
// the reference's operation order so the tree, the primitive edges and
// the camera matrices are the reference's bit for bit.
#include "host_scene.h"

#include <algorithm>
#include <cfloat>
#include <cstdio>
#include <cstring>

namespace pbrt {

// ------------------------------------------------------------------ boxes --
Box box_empty() { return Box{v3(FLT_MAX, FLT_MAX, FLT_MAX), v3(-FLT_MAX, -FLT_MAX, -FLT_MAX)}; }
// src/bbox.rs:170-183
Box box_union(const Box& a, const Box& b) {
    return Box{v3(std::fmin(a.lo.x, b.lo.x), std::fmin(a.lo.y, b.lo.y), std::fmin(a.lo.z, b.lo.z)),
               v3(std::fmax(a.hi.x, b.hi.x), std::fmax(a.hi.y, b.hi.y), std::fmax(a.hi.z, b.hi.z))};
}
// src/bbox.rs:155-168
Box box_union(const Box& a, V3 p) {
    return Box{v3(std::fmin(a.lo.x, p.x), std::fmin(a.lo.y, p.y), std::fmin(a.lo.z, p.z)),
               v3(std::fmax(a.hi.x, p.x), std::fmax(a.hi.y, p.y), std::fmax(a.hi.z, p.z))};
}
// src/bbox.rs:73-78
float box_area(const Box& b) {
    float dx = std::fmax(b.hi.x - b.lo.x, 0.0f);
    float dy = std::fmax(b.hi.y - b.lo.y, 0.0f);
    float dz = std::fmax(b.hi.z - b.lo.z, 0.0f);
    return 2.0f * (dx * dy + dx * dz + dy * dz);
}
// src/bbox.rs:87-96
int box_max_extent(const Box& b) {
    V3 d = b.hi - b.lo;
    if (d.x > d.y && d.x > d.z) return 0;
    if (d.y > d.z) return 1;
    return 2;
}

// --------------------------------------------------------------- matrices --
M4 m4_identity() {
    M4 r;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) r.m[i][j] = i == j ? 1.0f : 0.0f;
    return r;
}
// src/transform/matrix4x4.rs:167-182
M4 m4_mul(const M4& a, const M4& b) {
    M4 r;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            r.m[i][j] = a.m[i][0] * b.m[0][j] + a.m[i][1] * b.m[1][j] + a.m[i][2] * b.m[2][j] + a.m[i][3] * b.m[3][j];
    return r;
}
// src/transform/matrix4x4.rs:66-160: scaled partial pivoting where a row
// swap exchanges only columns k..3; the inverse's column c solves A x = e_c.
bool m4_inverse(const M4& a, M4* out) {
    float scale[4];
    for (int i = 0; i < 4; ++i) {
        float s = 0.0f;
        for (int j = 0; j < 4; ++j) s = std::fmax(std::fabs(a.m[i][j]), s);
        scale[i] = s;
    }
    M4 lu = a;
    int piv[4] = {0, 1, 2, 3};
    for (int k = 0; k < 3; ++k) {
        float best = 0.0f;
        int p = k;
        for (int i = k; i < 4; ++i) {
            float c = std::fabs(lu.m[i][k] / scale[i]);
            if (c > best) {
                best = c;
                p = i;
            }
        }
        piv[k] = p;
        if (best == 0.0f) return false;
        if (p != k)
            for (int j = k; j < 4; ++j) std::swap(lu.m[k][j], lu.m[p][j]);
        for (int i = k + 1; i < 4; ++i) {
            float f = lu.m[i][k] / lu.m[k][k];
            lu.m[i][k] = f;
            for (int j = k + 1; j < 4; ++j) lu.m[i][j] = lu.m[i][j] - f * lu.m[k][j];
        }
    }
    if (std::fabs(lu.m[3][3]) < 1.0e-6f) return false;
    M4 inv;
    for (int c = 0; c < 4; ++c) {
        float x[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        x[c] = 1.0f;
        for (int k = 0; k < 3; ++k) {
            if (piv[k] != k) std::swap(x[piv[k]], x[k]);
            for (int i = k + 1; i < 4; ++i) x[i] = x[i] - lu.m[i][k] * x[k];
        }
        x[3] = x[3] / lu.m[3][3];
        for (int i = 2; i >= 0; --i) {
            float acc = 0.0f;
            for (int j = i + 1; j < 4; ++j) acc = acc + lu.m[i][j] * x[j];
            x[i] = (x[i] - acc) / lu.m[i][i];
        }
        for (int r = 0; r < 4; ++r) inv.m[r][c] = x[r];
    }
    *out = inv;
    return true;
}
V3 m4_point(const M4& m, V3 p) {
    float xt = m.m[0][0] * p.x + m.m[0][1] * p.y + m.m[0][2] * p.z + m.m[0][3];
    float yt = m.m[1][0] * p.x + m.m[1][1] * p.y + m.m[1][2] * p.z + m.m[1][3];
    float zt = m.m[2][0] * p.x + m.m[2][1] * p.y + m.m[2][2] * p.z + m.m[2][3];
    float w = m.m[3][0] * p.x + m.m[3][1] * p.y + m.m[3][2] * p.z + m.m[3][3];
    if (w != 1.0f) return v3(xt / w, yt / w, zt / w);
    return v3(xt, yt, zt);
}
V3 m4_vector(const M4& m, V3 v) {
    return v3(m.m[0][0] * v.x + m.m[0][1] * v.y + m.m[0][2] * v.z, m.m[1][0] * v.x + m.m[1][1] * v.y + m.m[1][2] * v.z,
              m.m[2][0] * v.x + m.m[2][1] * v.y + m.m[2][2] * v.z);
}
bool m4_swaps_handedness(const M4& m) {
    float det = m.m[0][0] * (m.m[1][1] * m.m[2][2] - m.m[1][2] * m.m[2][1]) -
                m.m[0][1] * (m.m[1][0] * m.m[2][2] - m.m[1][2] * m.m[2][0]) +
                m.m[0][2] * (m.m[1][0] * m.m[2][1] - m.m[1][1] * m.m[2][0]);
    return 0.0f > det;
}
Xf xf_from_desc(const PbrtTransform& t) {
    Xf x;
    std::memcpy(x.m.m, t.m, sizeof(x.m.m));
    std::memcpy(x.mi.m, t.m_inv, sizeof(x.mi.m));
    return x;
}
Xf xf_mul(const Xf& a, const Xf& b) { return Xf{m4_mul(a.m, b.m), m4_mul(b.mi, a.mi)}; }
Xf xf_inverse(const Xf& a) { return Xf{a.mi, a.m}; }
static Xf xf_scale(float x, float y, float z) {
    Xf t{m4_identity(), m4_identity()};
    t.m.m[0][0] = x;
    t.m.m[1][1] = y;
    t.m.m[2][2] = z;
    t.mi.m[0][0] = 1.0f / x;
    t.mi.m[1][1] = 1.0f / y;
    t.mi.m[2][2] = 1.0f / z;
    return t;
}
static Xf xf_translate(float x, float y, float z) {
    Xf t{m4_identity(), m4_identity()};
    t.m.m[0][3] = x;
    t.m.m[1][3] = y;
    t.m.m[2][3] = z;
    t.mi.m[0][3] = -x;
    t.mi.m[1][3] = -y;
    t.mi.m[2][3] = -z;
    return t;
}

// ------------------------------------------------------------------ shapes --
// transform.rs:248-263 (eight-corner box transform)
static Box xf_box(const M4& m, const Box& b) {
    V3 tx = m4_vector(m, v3(b.hi.x - b.lo.x, 0.0f, 0.0f));
    V3 ty = m4_vector(m, v3(0.0f, b.hi.y - b.lo.y, 0.0f));
    V3 tz = m4_vector(m, v3(0.0f, 0.0f, b.hi.z - b.lo.z));
    V3 tp = m4_point(m, b.lo);
    Box r{tp, tp};
    r = box_union(r, tp + tx);
    r = box_union(r, tp + ty);
    r = box_union(r, tp + tz);
    r = box_union(r, (tp + tx) + ty);
    r = box_union(r, (tp + tx) + tz);
    r = box_union(r, (tp + ty) + tz);
    r = box_union(r, ((tp + tx) + ty) + tz);
    return r;
}

static float clampf(float x, float lo, float hi) {
    if (x < lo) x = lo;
    if (x > hi) x = hi;
    return x;
}

int parse_split_method(const char* s) {
    if (!s || !std::strcmp(s, "sah")) return PBRT_SPLIT_SAH;
    if (!std::strcmp(s, "middle")) return PBRT_SPLIT_MIDDLE;
    if (!std::strcmp(s, "equal")) return PBRT_SPLIT_EQUAL;
    std::fprintf(stderr, "Warning: BVH split method %s unknown. Using \"SAH\"\n", s);  // bvh.rs:345-348
    return PBRT_SPLIT_SAH;
}

// -------------------------------------------------------------- BVH build --
namespace {

// src/utils/mod.rs:112-169 over a slice of primitive indices keyed by a
// centroid coordinate (median-of-three pivot, three-way scan, recursion on
// the side holding the middle).
void partition_by_key(uint32_t* v, size_t n, const float* key) {
    while (true) {
        if (n < 3) {
            if (n == 2 && key[v[1]] < key[v[0]]) std::swap(v[0], v[1]);
            return;
        }
        float a = key[v[0]], b = key[v[n / 2]], c = key[v[n - 1]];
        float pivot = (a < b && b < c) ? b : ((b < a && a < c) ? a : c);
        size_t ls = 0, np = 0;
        for (size_t i = 0; i < n; ++i) {
            float k = key[v[i]];
            if (k < pivot) {
                std::swap(v[ls + np], v[i]);
                std::swap(v[ls + np], v[ls]);
                ++ls;
            } else if (k == pivot) {
                std::swap(v[ls + np], v[i]);
                ++np;
            }
        }
        size_t pi = std::max<size_t>(ls, 1);
        if (pi + np <= n / 2) {
            v += pi;
            n -= pi;
        } else if (pi >= n / 2) {
            n = pi;
        } else {
            return;
        }
    }
}

inline size_t f32_to_usize(float f) {  // Rust `as usize`: saturating, NaN -> 0
    if (!(f > 0.0f)) return 0;
    if (f >= 18446744073709551615.0f) return SIZE_MAX;
    return (size_t)f;
}

struct Task {
    uint32_t lo, hi;
    int32_t parent;  // node whose second-child offset is this node, or -1
    uint32_t depth;
};

}  // namespace

void prim_bounds(const HostBVH& H, std::vector<Box>* bounds, std::vector<float>* cx, std::vector<float>* cy,
                 std::vector<float>* cz) {
    const size_t n = H.prims.size();
    bounds->resize(n);
    cx->resize(n);
    cy->resize(n);
    cz->resize(n);
    for (size_t i = 0; i < n; ++i) {
        const HostPrim& p = H.prims[i];
        Box b;
        if (p.kind == PBRT_SHAPE_TRIANGLE_MESH) {
            b = box_union(box_union(box_union(box_empty(), p.p1), p.p2), p.p3);  // mesh.rs:196-205
        } else {
            const SphereRec& s = H.spheres[p.sphere];
            M4 o2w;
            std::memcpy(o2w.m, s.o2w, sizeof(o2w.m));
            if (s.kind == kQuadInstance) {
                // transformed.rs:62-65: motion_bounds of a static transform =
                // the definition's bound through primitive-to-world
                b = xf_box(o2w, H.insts[s.instance].nodes[0].box);  // definitions are not empty
            } else {
                b = xf_box(o2w, Box{v3(-s.radius, -s.radius, s.z_min), v3(s.radius, s.radius, s.z_max)});
            }
        }
        (*bounds)[i] = b;
        V3 c = (b.lo + b.hi) * 0.5f;  // bvh.rs:77
        (*cx)[i] = c.x;
        (*cy)[i] = c.y;
        (*cz)[i] = c.z;
    }
}

static int build_tree(HostBVH& H, uint32_t mp, int split, std::string* err) {
    const size_t n = H.prims.size();
    H.nodes.clear();
    H.ordered.resize(n);
    if (n == 0) return PBRT_OK;
    std::vector<Box> bounds;
    std::vector<float> cx, cy, cz;
    prim_bounds(H, &bounds, &cx, &cy, &cz);
    for (size_t i = 0; i < n; ++i) H.ordered[i] = (uint32_t)i;
    const float* cent[3] = {cx.data(), cy.data(), cz.data()};
    uint32_t* idx = H.ordered.data();
    H.nodes.reserve(2 * n);
    std::vector<Task> stack;
    stack.push_back(Task{0, (uint32_t)n, -1, 1});
    std::vector<uint32_t> scratch;
    H.depth = 0;
    const size_t NB = 12;
    while (!stack.empty()) {
        Task t = stack.back();
        stack.pop_back();
        uint32_t k = (uint32_t)H.nodes.size();
        if (t.parent >= 0) H.nodes[t.parent].offset = k;
        H.depth = std::max(H.depth, t.depth);
        const size_t cnt = t.hi - t.lo;
        Box bbox = box_empty();
        for (uint32_t i = t.lo; i < t.hi; ++i) bbox = box_union(bbox, bounds[idx[i]]);
        FlatNode node{bbox, true, t.lo, (uint32_t)cnt};
        uint32_t mid = 0;
        bool split_it = false;
        int dim = 0;
        if (cnt > 1) {
            Box cb = box_empty();
            for (uint32_t i = t.lo; i < t.hi; ++i) cb = box_union(cb, v3(cx[idx[i]], cy[idx[i]], cz[idx[i]]));
            dim = box_max_extent(cb);
            float cmin = axis_of(cb.lo, dim), cmax = axis_of(cb.hi, dim);
            const float* key = cent[dim];
            if (cmin != cmax) {
                auto equal_counts = [&]() {  // bvh.rs:92-103
                    partition_by_key(idx + t.lo, cnt, key);
                    mid = t.lo + (uint32_t)(cnt / 2);
                    split_it = true;
                };
                auto stable_split = [&](auto pred) {
                    scratch.clear();
                    uint32_t w = t.lo;
                    for (uint32_t i = t.lo; i < t.hi; ++i) {
                        if (pred(idx[i]))
                            idx[w++] = idx[i];
                        else
                            scratch.push_back(idx[i]);
                    }
                    mid = w;
                    std::copy(scratch.begin(), scratch.end(), idx + w);
                    split_it = true;
                };
                if (split == PBRT_SPLIT_MIDDLE) {  // bvh.rs:86-90
                    float p_mid = 0.5f * (cmin + cmax);
                    stable_split([&](uint32_t p) { return key[p] < p_mid; });
                } else if (split == PBRT_SPLIT_EQUAL) {
                    equal_counts();
                } else if (cnt <= 4) {  // bvh.rs:111-113
                    equal_counts();
                } else {  // bvh.rs:115-185
                    float dist = cmax - cmin;
                    auto bucket = [&](uint32_t p) {
                        float pdist = key[p] - cmin;
                        size_t b = f32_to_usize((float)NB * (pdist / dist));
                        return b == NB ? NB - 1 : b;
                    };
                    size_t bc[12] = {0};
                    Box bb[12];
                    for (size_t i = 0; i < NB; ++i) bb[i] = box_empty();
                    for (uint32_t i = t.lo; i < t.hi; ++i) {
                        size_t b = bucket(idx[i]);
                        bc[b] += 1;
                        bb[b] = box_union(bb[b], bounds[idx[i]]);
                    }
                    float tsa = box_area(bbox);
                    size_t best = 0;
                    float best_cost = FLT_MAX;
                    for (size_t s = 0; s + 1 < NB; ++s) {
                        size_t c0 = 0, c1 = 0;
                        Box b0 = box_empty(), b1 = box_empty();
                        for (size_t j = 0; j <= s; ++j) {
                            c0 += bc[j];
                            b0 = box_union(b0, bb[j]);
                        }
                        for (size_t j = s + 1; j < NB; ++j) {
                            c1 += bc[j];
                            b1 = box_union(b1, bb[j]);
                        }
                        float cost = 0.125f * ((float)c0 * box_area(b0) + (float)c1 * box_area(b1)) / tsa;
                        if (cost < best_cost) {
                            best_cost = cost;
                            best = s;
                        }
                    }
                    if (mp < cnt || f32_to_usize(best_cost) < cnt)
                        stable_split([&](uint32_t p) { return bucket(p) <= best; });
                }
            }
        }
        if (split_it) {
            if (mid == t.lo || mid == t.hi) {
                *err = "BVH build: empty partition (the reference asserts at bvh.rs:237-238)";
                return PBRT_ERR_BUILD;
            }
            node.leaf = false;
            node.offset = 0;
            node.count = (uint32_t)dim;
            H.nodes.push_back(node);
            stack.push_back(Task{mid, t.hi, (int32_t)k, t.depth + 1});
            stack.push_back(Task{t.lo, mid, -1, t.depth + 1});
        } else {
            H.nodes.push_back(node);
        }
    }
    // Inner bounds are the union of the two children (bvh.rs:247).
    for (size_t k = H.nodes.size(); k-- > 0;) {
        FlatNode& nd = H.nodes[k];
        if (!nd.leaf) nd.box = box_union(H.nodes[k + 1].box, H.nodes[nd.offset].box);
    }
    return PBRT_OK;
}

static void fill_device_layout(HostBVH& H) {
    const size_t m = H.nodes.size();
    std::vector<uint32_t> pair_of(m, 0xffffffffu);
    uint32_t np = 0;
    for (size_t k = 0; k < m; ++k)
        if (!H.nodes[k].leaf) pair_of[k] = np++;
    auto rec = [&](size_t k) {
        const FlatNode& nd = H.nodes[k];
        ChildRec c;
        c.lo_x = nd.box.lo.x;
        c.lo_y = nd.box.lo.y;
        c.lo_z = nd.box.lo.z;
        c.hi_x = nd.box.hi.x;
        c.hi_y = nd.box.hi.y;
        c.hi_z = nd.box.hi.z;
        if (nd.leaf) {
            c.a = nd.offset;
            c.b = kLeafBit | nd.count;
        } else {
            c.a = pair_of[k];
            c.b = nd.count;
        }
        return c;
    };
    H.pairs.assign(np, NodePair{});
    for (size_t k = 0; k < m; ++k) {
        const FlatNode& nd = H.nodes[k];
        if (nd.leaf) continue;
        NodePair& p = H.pairs[pair_of[k]];
        p.c[0] = rec(k + 1);
        p.c[1] = rec(nd.offset);
    }
    if (m) H.root = rec(0);
    H.recs.resize(H.ordered.size());
    for (size_t i = 0; i < H.ordered.size(); ++i) {
        const HostPrim& p = H.prims[H.ordered[i]];
        PrimRec& r = H.recs[i];
        std::memset(&r, 0, sizeof(r));
        uint32_t id = H.flat_id.empty() ? H.ordered[i] : H.flat_id[H.ordered[i]];
        if (p.kind == PBRT_SHAPE_TRIANGLE_MESH) {
            V3 e1 = p.p2 - p.p1, e2 = p.p3 - p.p1;  // mesh.rs:45-46
            r.r0[0] = p.p1.x;
            r.r0[1] = p.p1.y;
            r.r0[2] = p.p1.z;
            std::memcpy(&r.r0[3], &id, 4);
            r.r1[0] = e1.x;
            r.r1[1] = e1.y;
            r.r1[2] = e1.z;
            r.r2[0] = e2.x;
            r.r2[1] = e2.y;
            r.r2[2] = e2.z;
        } else {
            uint32_t tagged = id | kSphereBit;
            uint32_t si = (uint32_t)p.sphere;
            std::memcpy(&r.r0[3], &tagged, 4);
            std::memcpy(&r.r1[3], &si, 4);
        }
    }
}

// Collapse the binary tree two levels at a time (see layout.h: Node4) and
// mark the last primitive of every leaf.
static void fill_node4_layout(HostBVH& H) {
    const size_t m = H.nodes.size();
    H.nodes4.clear();
    H.stack4_bound = 0;
    for (size_t k = 0; k < m; ++k) {
        const FlatNode& nd = H.nodes[k];
        if (nd.leaf && nd.count > 0) {
            uint32_t last = nd.offset + nd.count - 1;
            uint32_t flag = kPrimLastBit;
            std::memcpy(&H.recs[last].r2[3], &flag, 4);
        }
    }
    if (m == 0) return;
    auto box_rec = [&](size_t k, ChildRec& c) {
        const FlatNode& nd = H.nodes[k];
        c.lo_x = nd.box.lo.x;
        c.lo_y = nd.box.lo.y;
        c.lo_z = nd.box.lo.z;
        c.hi_x = nd.box.hi.x;
        c.hi_y = nd.box.hi.y;
        c.hi_z = nd.box.hi.z;
    };
    // index of the Node4 rooted at each binary inner node that starts one
    std::vector<uint32_t> n4_of(m, kNode4Empty);
    // pre-order walk: a binary inner node reached as a grandchild (or the
    // root) starts a Node4
    struct Item {
        size_t k;
        uint32_t pushes;  // stack entries the traversal may hold above it
    };
    std::vector<Item> todo{{0, 0}};
    std::vector<size_t> order;
    while (!todo.empty()) {
        Item it = todo.back();
        todo.pop_back();
        const FlatNode& N = H.nodes[it.k];
        if (N.leaf) continue;
        n4_of[it.k] = (uint32_t)order.size();
        order.push_back(it.k);
        size_t L = it.k + 1, R = N.offset;
        size_t kids[4] = {SIZE_MAX, SIZE_MAX, SIZE_MAX, SIZE_MAX};
        if (H.nodes[L].leaf) kids[0] = L; else { kids[0] = L + 1; kids[1] = H.nodes[L].offset; }
        if (H.nodes[R].leaf) kids[2] = R; else { kids[2] = R + 1; kids[3] = H.nodes[R].offset; }
        uint32_t nk = 0;
        for (size_t kk : kids) nk += kk != SIZE_MAX;
        uint32_t here = it.pushes + nk - 1;
        H.stack4_bound = std::max(H.stack4_bound, here);
        for (int s = 3; s >= 0; --s)
            if (kids[s] != SIZE_MAX && !H.nodes[kids[s]].leaf) todo.push_back({kids[s], here});
    }
    H.nodes4.assign(order.size(), Node4{});
    for (size_t i = 0; i < order.size(); ++i) {
        size_t k = order[i];
        const FlatNode& N = H.nodes[k];
        size_t L = k + 1, R = N.offset;
        size_t kids[4] = {SIZE_MAX, SIZE_MAX, SIZE_MAX, SIZE_MAX};
        uint32_t axL = 0, axR = 0;
        if (H.nodes[L].leaf) kids[0] = L; else { kids[0] = L + 1; kids[1] = H.nodes[L].offset; axL = H.nodes[L].count; }
        if (H.nodes[R].leaf) kids[2] = R; else { kids[2] = R + 1; kids[3] = H.nodes[R].offset; axR = H.nodes[R].count; }
        Node4& n4 = H.nodes4[i];
        for (int s = 0; s < 4; ++s) {
            ChildRec& c = n4.c[s];
            if (kids[s] == SIZE_MAX) {
                c.lo_x = c.lo_y = c.lo_z = FLT_MAX;
                c.hi_x = c.hi_y = c.hi_z = -FLT_MAX;
                c.a = kNode4Empty;
            } else {
                box_rec(kids[s], c);
                const FlatNode& G = H.nodes[kids[s]];
                c.a = G.leaf ? (kNode4Leaf | G.offset) : n4_of[kids[s]];
            }
            c.b = 0;
        }
        n4.c[0].b = N.count | (axL << 2) | (axR << 4);
    }
    ChildRec r;
    box_rec(0, r);
    r.a = H.nodes[0].leaf ? (kNode4Leaf | H.nodes[0].offset) : 0u;
    r.b = 0;
    H.root4 = r;
}

int build_host_bvh(const PbrtShapeDesc* shapes, uint32_t n_shapes, uint32_t max_prims, const char* split_method,
                   HostBVH* out, std::string* err, bool on_device, const PbrtInstanceDesc* defs, uint32_t n_defs) {
    HostBVH& H = *out;
    H = HostBVH();
    // the definitions' BVHs, built like the scene's (the instance aggregate
    // of ObjectInstance uses the scene's accelerator, main.rs:735-763)
    H.insts.resize(n_defs);
    for (uint32_t k = 0; k < n_defs; ++k) {
        for (uint32_t i = 0; i < defs[k].n_shapes; ++i)
            if (defs[k].shapes[i].kind == PBRT_SHAPE_INSTANCE || defs[k].shapes[i].area_light >= 0) {
                *err = "instance definitions hold neither instances nor area lights";
                return PBRT_ERR_UNSUPPORTED;
            }
        int st = build_host_bvh(defs[k].shapes, defs[k].n_shapes, max_prims, split_method, &H.insts[k], err,
                                on_device);
        if (st) return st;
        if (H.insts[k].prims.empty()) {
            *err = "instance definition without shapes";
            return PBRT_ERR_INVALID_ARGUMENT;
        }
        if (H.insts[k].stack4_bound > 96) {  // kInstStack4 of the nested walk
            *err = "instance definition BVH too deep for the nested traversal stack (96 entries)";
            return PBRT_ERR_UNSUPPORTED;
        }
    }
    // Full refinement: primitive/mod.rs:47-63, mesh.rs:298-338.
    for (uint32_t si = 0; si < n_shapes; ++si) {
        const PbrtShapeDesc& d = shapes[si];
        Xf o2w = xf_from_desc(d.object_to_world);
        bool flip = (d.reverse_orientation != 0) != m4_swaps_handedness(o2w.m);
        if (d.kind == PBRT_SHAPE_TRIANGLE_MESH) {
            if (d.n_indices % 3 != 0 || (d.n_indices && (!d.indices || !d.points))) {
                *err = "triangle mesh: index count must be a multiple of 3 with points and indices given";
                return PBRT_ERR_INVALID_ARGUMENT;
            }
            std::vector<V3> wp(d.n_points);
            for (uint32_t i = 0; i < d.n_points; ++i)
                wp[i] = m4_point(o2w.m, v3(d.points[3 * i], d.points[3 * i + 1], d.points[3 * i + 2]));
            for (uint32_t k = 0; k < d.n_indices / 3; ++k) {
                uint32_t i0 = d.indices[3 * k], i1 = d.indices[3 * k + 1], i2 = d.indices[3 * k + 2];
                if (i0 >= d.n_points || i1 >= d.n_points || i2 >= d.n_points) {
                    *err = "triangle mesh: vertex index out of range";
                    return PBRT_ERR_INVALID_ARGUMENT;
                }
                HostPrim p{};
                p.kind = PBRT_SHAPE_TRIANGLE_MESH;
                p.shape = (int)si;
                p.material = d.material;
                p.area_light = d.area_light;
                p.p1 = wp[i2];  // refine pops indices: v = (i2, i1, i0)
                p.p2 = wp[i1];
                p.p3 = wp[i0];
                p.flip = flip;
                p.sphere = -1;
                H.prims.push_back(p);
            }
        } else if (d.kind == PBRT_SHAPE_SPHERE) {
            if (!(d.radius > 0.0f)) {
                *err = "sphere: radius must be positive";
                return PBRT_ERR_INVALID_ARGUMENT;
            }
            // sphere.rs:28-44
            SphereRec s{};
            std::memcpy(s.o2w, o2w.m.m, sizeof(s.o2w));
            std::memcpy(s.w2o, o2w.mi.m, sizeof(s.w2o));
            float rad = d.radius;
            s.radius = rad;
            s.z_min = clampf(std::fmin(d.z0, d.z1), -rad, rad);
            s.z_max = clampf(std::fmax(d.z0, d.z1), -rad, rad);
            s.theta_min = std::acos(s.z_min / rad);
            s.theta_max = std::acos(s.z_max / rad);
            s.phi_max = clampf(d.phi_max_deg, 0.0f, 360.0f) * 3.14159265358979323846f / 180.0f;
            // With z_min = -r, z_max = r and phi_max >= 2*pi (f32) the clip
            // test of sphere.rs:88-92 can never reject: atan2 + 2*pi stays
            // <= 2*pi in f32.
            s.full = (s.z_min <= -rad && s.z_max >= rad && s.phi_max >= 2.0f * 3.14159265358979323846f) ? 1u : 0u;
            s.flip = flip ? 1u : 0u;
            s.kind = kQuadSphere;
            HostPrim p{};
            p.kind = PBRT_SHAPE_SPHERE;
            p.shape = (int)si;
            p.material = d.material;
            p.area_light = d.area_light;
            p.flip = flip;
            p.sphere = (int)H.spheres.size();
            H.spheres.push_back(s);
            H.prims.push_back(p);
            H.has_spheres = true;
        } else if (d.kind == PBRT_SHAPE_INSTANCE) {
            if (d.instance < 0 || (uint32_t)d.instance >= n_defs) {
                *err = "instance: definition index out of range";
                return PBRT_ERR_INVALID_ARGUMENT;
            }
            SphereRec s{};
            std::memcpy(s.o2w, o2w.m.m, sizeof(s.o2w));   // primitive to world
            std::memcpy(s.w2o, o2w.mi.m, sizeof(s.w2o));  // world to primitive
            s.kind = kQuadInstance;
            s.instance = (uint32_t)d.instance;
            HostPrim p{};
            p.kind = PBRT_SHAPE_SPHERE;  // one analytic-style primitive
            p.shape = (int)si;
            p.material = d.material;
            p.area_light = -1;
            p.flip = false;
            p.sphere = (int)H.spheres.size();
            H.spheres.push_back(s);
            H.prims.push_back(p);
            H.has_spheres = true;
        } else if (d.kind == PBRT_SHAPE_DISK || d.kind == PBRT_SHAPE_CYLINDER) {
            SphereRec s{};
            std::memcpy(s.o2w, o2w.m.m, sizeof(s.o2w));
            std::memcpy(s.w2o, o2w.mi.m, sizeof(s.w2o));
            s.radius = d.radius;
            s.phi_max = clampf(d.phi_max_deg, 0.0f, 360.0f) * 3.14159265358979323846f / 180.0f;
            if (d.kind == PBRT_SHAPE_DISK) {  // disk.rs:24-34: radii unclamped
                s.kind = kQuadDisk;
                s.height = d.height;
                s.inner_radius = d.inner_radius;
                s.z_min = s.z_max = d.height;
            } else {  // cylinder.rs:26-36
                s.kind = kQuadCylinder;
                s.z_min = std::fmin(d.z0, d.z1);
                s.z_max = std::fmax(d.z0, d.z1);
            }
            // phi = atan2 (+ 2 pi when negative) stays <= 2 pi in f32, so a
            // full turn never rejects on phi
            s.full = s.phi_max >= 2.0f * 3.14159265358979323846f ? 1u : 0u;
            s.flip = flip ? 1u : 0u;
            HostPrim p{};
            p.kind = PBRT_SHAPE_SPHERE;  // refined like a sphere: one analytic primitive
            p.shape = (int)si;
            p.material = d.material;
            p.area_light = d.area_light;
            p.flip = flip;
            p.sphere = (int)H.spheres.size();
            H.spheres.push_back(s);
            H.prims.push_back(p);
            H.has_spheres = true;
        } else {
            *err = "unknown shape kind";
            return PBRT_ERR_INVALID_ARGUMENT;
        }
    }
    bool any_instance = false;
    for (const SphereRec& s : H.spheres) any_instance |= s.kind == kQuadInstance;
    if (any_instance) {
        H.flat_id.resize(H.prims.size());
        uint64_t next = 0;
        for (size_t i = 0; i < H.prims.size(); ++i) {
            H.flat_id[i] = (uint32_t)next;
            const HostPrim& p = H.prims[i];
            const bool inst = p.sphere >= 0 && H.spheres[p.sphere].kind == kQuadInstance;
            next += inst ? H.insts[H.spheres[p.sphere].instance].prims.size() : 1u;
            if (next > 0x7fffffffull) {
                *err = "more than 2^31 - 1 primitives with the instances counted out";
                return PBRT_ERR_UNSUPPORTED;
            }
        }
        H.n_flat = next;
    } else {
        H.n_flat = H.prims.size();
    }
    const int split = parse_split_method(split_method);
    // equal-counts splits of large ranges use the sequential partition_by
    // (utils/mod.rs:112-169), which stays on the host
    int st = (on_device && split != PBRT_SPLIT_EQUAL) ? device_build_tree(H, max_prims, split, err)
                                                      : build_tree(H, max_prims, split, err);
    if (st) return st;
    fill_device_layout(H);
    fill_node4_layout(H);
    if (!H.insts.empty()) {
        // the 4-wide walk enters a definition with two more entries (the
        // rest of the leaf, the exit word) on top of the scene's stack
        uint32_t inner = 0;
        for (const HostBVH& I : H.insts) inner = std::max(inner, I.stack4_bound);
        H.stack4_bound += 2 + inner;
        if (H.recs.size() >= 0x7ffffffeu) {  // leaf words stay clear of the exit word
            *err = "too many primitives for a scene with instances";
            return PBRT_ERR_UNSUPPORTED;
        }
    }
    return PBRT_OK;
}

// -------------------------------------------------------------- camera ----
// Camera::perspective (camera/mod.rs:105-135): persp = scale(1/tan(fov/2))
// * P with n = 1e-2, f = 1000; Projection::new (projective.rs:48-72):
// raster_to_camera = inverse(persp) * inverse(screen_to_raster).
void camera_matrices(const PbrtCameraDesc& cam, float r2c_out[16], float c2w_out[16]) {
    const float znear = 1e-2f, zfar = 1000.0f;
    M4 pm = m4_identity();
    pm.m[2][2] = zfar / (zfar - znear);
    pm.m[2][3] = -(zfar * znear) / (zfar - znear);
    pm.m[3][2] = 1.0f;
    pm.m[3][3] = 0.0f;
    M4 pmi;
    if (!m4_inverse(pm, &pmi)) pmi = m4_identity();
    Xf p{pm, pmi};
    float rad = cam.fov_deg * 3.14159265358979323846f / 180.0f;
    float inv_tan = 1.0f / std::tan(rad / 2.0f);
    Xf persp = xf_mul(xf_scale(inv_tan, inv_tan, 1.0f), p);
    const float* sw = cam.screen_window;
    Xf s2r = xf_mul(xf_mul(xf_scale((float)cam.x_res, (float)cam.y_res, 1.0f),
                           xf_scale(1.0f / (sw[1] - sw[0]), 1.0f / (sw[2] - sw[3]), 1.0f)),
                    xf_translate(-sw[0], -sw[3], 0.0f));
    Xf r2c = xf_mul(xf_inverse(persp), xf_inverse(s2r));
    std::memcpy(r2c_out, r2c.m.m, sizeof(float) * 16);
    std::memcpy(c2w_out, cam.camera_to_world.m, sizeof(float) * 16);
}

}  // namespace pbrt

namespace pbrt {

// ------------------------------------------------------------------ filter ---
namespace {

// utils/mod.rs:207-217
float sinc_1d(float x, float tau) {
    float v = std::fabs(x);
    if (v < 1e-5f) return 1.0f;
    if (v >= 1.0f) return 0.0f;
    v *= 3.14159265358979323846f;
    const float vt = v * tau;
    const float s = std::sin(vt) / vt;
    return s * std::sin(v) / v;
}

// filter.rs:87-124 (Filter::evaluate) for the kinds of PBRT_FILTER_*
float filter_eval(int kind, float xw, float yw, float p0, float p1, float x, float y) {
    const float ixw = 1.0f / xw, iyw = 1.0f / yw;
    switch (kind) {
        case PBRT_FILTER_TRIANGLE: {
            const float dx = (xw - std::fabs(x)) * ixw, dy = (yw - std::fabs(y)) * iyw;
            return std::fmax(dx, 0.0f) * std::fmax(dy, 0.0f);
        }
        case PBRT_FILTER_GAUSSIAN: {  // filter.rs:55-64: exp_x / exp_y fixed at construction
            const float ex = std::exp(-p0 * xw * xw), ey = std::exp(-p0 * yw * yw);
            const float gx = std::fmax(std::exp(-p0 * x * x) - ex, 0.0f);
            const float gy = std::fmax(std::exp(-p0 * y * y) - ey, 0.0f);
            return gx * gy;
        }
        case PBRT_FILTER_MITCHELL: {
            const float b = p0, c = p1;
            auto m = [&](float v) {
                const float t = std::fabs(v * 2.0f);
                float r;
                if (t >= 2.0f)
                    r = 0.0f;
                else if (t > 1.0f)
                    r = (-b - 6.0f * c) * t * t * t + (6.0f * b + 30.0f * c) * t * t + (-12.0f * b - 48.0f * c) * t +
                        (8.0f * b + 24.0f * c);
                else
                    r = (12.0f - 9.0f * b - 6.0f * c) * t * t * t + (-18.0f + 12.0f * b + 6.0f * c) * t * t +
                        (6.0f - 2.0f * b);
                return (1.0f / 6.0f) * r;
            };
            return m(x * ixw) * m(y * iyw);
        }
        case PBRT_FILTER_LANCZOS:
            return sinc_1d(x * ixw, p0) * sinc_1d(y * iyw, p0);
        default:  // PBRT_FILTER_BOX: Filter::mean
            return 1.0f;
    }
}

}  // namespace

int filter_table(const PbrtCameraDesc& cam, float table[256]) {
    if (cam.filter_kind < PBRT_FILTER_BOX || cam.filter_kind > PBRT_FILTER_LANCZOS) return PBRT_ERR_INVALID_ARGUMENT;
    const float xw = cam.filter_x_width, yw = cam.filter_y_width;
    for (int y = 0; y < 16; ++y) {
        const float fy = ((float)y + 0.5f) * yw / 16.0f;
        for (int x = 0; x < 16; ++x) {
            const float fx = ((float)x + 0.5f) * xw / 16.0f;
            table[y * 16 + x] = filter_eval(cam.filter_kind, xw, yw, cam.filter_p0, cam.filter_p1, fx, fy);
        }
    }
    return PBRT_OK;
}

}  // namespace pbrt
