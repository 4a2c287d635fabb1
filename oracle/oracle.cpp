// oracle.cpp - TEST INFRASTRUCTURE: the CPU oracle of the hot path.
//
// A literal C++ restatement of the reference CPU path (Mokosha/pbrt_rust).
// Every function names the reference file:line it follows.  Built with
// -O2 -ffp-contract=off -fno-fast-math: each f32 expression below is
// evaluated left to right exactly as the Rust source writes it, with no
// fused multiply-add, so the results are the reference's bit for bit.
//
// Only tests/, __graft_entry__.smoke() and the benchmark's CPU baseline
// use this library.  Where the reference is stubbed or buggy on the path,
// the decision taken is written beside the code, each with a D-number that
// the device code uses for the same decision.
#include "oracle.h"

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <vector>

namespace {

// ---------------------------------------------------------------- math ----
// src/geometry/vector.rs, point.rs, normal.rs
struct V3 {
    float x, y, z;
};
inline V3 mk(float x, float y, float z) { return V3{x, y, z}; }
inline V3 add(V3 a, V3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 sub(V3 a, V3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 mul(V3 a, float f) { return mk(a.x * f, a.y * f, a.z * f); }
inline V3 neg(V3 a) { return mk(-a.x, -a.y, -a.z); }
// vector.rs:170-172
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// vector.rs:176-181
inline V3 cross(V3 a, V3 b) {
    return mk((a.y * b.z) - (a.z * b.y), (a.z * b.x) - (a.x * b.z), (a.x * b.y) - (a.y * b.x));
}
// vector.rs:41-47
inline float length_sq(V3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
inline float length(V3 a) { return sqrtf(length_sq(a)); }
// vector.rs:116-130: v / f == (1/f) * v
inline V3 vdiv(V3 a, float f) {
    float recip = 1.0f / f;
    return mul(a, recip);
}
// normal.rs:181-186
inline V3 normalize(V3 a) { return vdiv(a, length(a)); }
inline float comp(V3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
inline void set_comp(V3& a, int i, float v) {
    if (i == 0) a.x = v;
    else if (i == 1) a.y = v;
    else a.z = v;
}
// Rust f32::clamp
inline float clampf(float x, float lo, float hi) {
    if (x < lo) x = lo;
    if (x > hi) x = hi;
    return x;
}
// utils/mod.rs:15-21 (Lerp for f32)
inline float lerpf(float a, float b, float t) { return a * (1.0f - t) + b * t; }
const float kPi = 3.14159265358979323846f;
// utils/mod.rs:36-39
inline float as_radians(float d) { return d * kPi / 180.0f; }

struct Ray {
    V3 o, d;
    float mint, maxt;
};
// ray.rs:60
inline V3 point_at(const Ray& r, float t) { return add(r.o, mul(r.d, t)); }

// ---------------------------------------------------------------- bbox ----
// src/bbox.rs
struct BBox {
    V3 pmin, pmax;
};
inline BBox bbox_new() { return BBox{mk(FLT_MAX, FLT_MAX, FLT_MAX), mk(-FLT_MAX, -FLT_MAX, -FLT_MAX)}; }
inline BBox bbox_pt(V3 p) { return BBox{p, p}; }
// bbox.rs:155-168
inline BBox union_pt(const BBox& b, V3 p) {
    return BBox{mk(fminf(b.pmin.x, p.x), fminf(b.pmin.y, p.y), fminf(b.pmin.z, p.z)),
                mk(fmaxf(b.pmax.x, p.x), fmaxf(b.pmax.y, p.y), fmaxf(b.pmax.z, p.z))};
}
// bbox.rs:170-183
inline BBox union_box(const BBox& a, const BBox& b) {
    return BBox{mk(fminf(a.pmin.x, b.pmin.x), fminf(a.pmin.y, b.pmin.y), fminf(a.pmin.z, b.pmin.z)),
                mk(fmaxf(a.pmax.x, b.pmax.x), fmaxf(a.pmax.y, b.pmax.y), fmaxf(a.pmax.z, b.pmax.z))};
}
// bbox.rs:73-78
inline float surface_area(const BBox& b) {
    float dx = fmaxf(b.pmax.x - b.pmin.x, 0.0f);
    float dy = fmaxf(b.pmax.y - b.pmin.y, 0.0f);
    float dz = fmaxf(b.pmax.z - b.pmin.z, 0.0f);
    return 2.0f * (dx * dy + dx * dz + dy * dz);
}
// bbox.rs:87-96
inline int max_extent(const BBox& b) {
    V3 d = sub(b.pmax, b.pmin);
    if (d.x > d.y && d.x > d.z) return 0;
    if (d.y > d.z) return 1;
    return 2;
}
// bbox.rs:185-209 (Intersectable<(f32,f32)> for BBox)
inline bool bbox_intersect(const BBox& b, const Ray& r, float* t0o, float* t1o) {
    float t0 = r.mint, t1 = r.maxt;
    for (int i = 0; i < 3; ++i) {
        float inv = 1.0f / comp(r.d, i);
        float ta = (comp(b.pmin, i) - comp(r.o, i)) * inv;
        float tb = (comp(b.pmax, i) - comp(r.o, i)) * inv;
        if (ta > tb) std::swap(ta, tb);
        t0 = fmaxf(ta, t0);  // t_near.max(t0)
        t1 = fminf(tb, t1);  // t_far.min(t1)
        if (t0 > t1) return false;
    }
    if (t0o) *t0o = t0;
    if (t1o) *t1o = t1;
    return true;
}

// ---------------------------------------------------------- transforms ----
// src/transform/matrix4x4.rs
struct M4 {
    float m[4][4];
};
M4 m4_identity() {
    M4 r;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) r.m[i][j] = (i == j) ? 1.0f : 0.0f;
    return r;
}
// matrix4x4.rs:167-182
M4 m4_mul(const M4& a, const M4& b) {
    M4 r;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            r.m[i][j] = a.m[i][0] * b.m[0][j] + a.m[i][1] * b.m[1][j] + a.m[i][2] * b.m[2][j] +
                        a.m[i][3] * b.m[3][j];
    return r;
}
// matrix4x4.rs:50-56
M4 m4_transpose(const M4& a) {
    M4 r;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) r.m[i][j] = a.m[j][i];
    return r;
}
// matrix4x4.rs:66-117 (Gaussian elimination with scaled partial pivoting,
// swapping only columns k..3 of the pivot rows, as the reference does).
bool m4_lu(const M4& self, M4* lu, int pivot[4]) {
    float s[4];
    for (int i = 0; i < 4; ++i) {
        float acc = 0.0f;
        for (int j = 0; j < 4; ++j) acc = fmaxf(fabsf(self.m[i][j]), acc);
        s[i] = acc;
    }
    M4 r = self;
    for (int i = 0; i < 4; ++i) pivot[i] = i;
    float det = 1.0f;
    for (int k = 0; k < 3; ++k) {
        float c = 0.0f;
        int p = k;
        for (int i = k; i < 4; ++i) {
            float cc = fabsf(r.m[i][k] / s[i]);
            if (cc > c) {
                c = cc;
                p = i;
            }
        }
        pivot[k] = p;
        if (c == 0.0f) return false;
        if (p != k) {
            det = -det;
            for (int j = k; j < 4; ++j) std::swap(r.m[k][j], r.m[p][j]);
        }
        float rkk = r.m[k][k];
        for (int i = k + 1; i < 4; ++i) {
            float mi = r.m[i][k] / r.m[k][k];
            r.m[i][k] = mi;
            for (int j = k + 1; j < 4; ++j) r.m[i][j] = r.m[i][j] - mi * r.m[k][j];
        }
        det = det * rkk;
    }
    (void)det;
    if (fabsf(r.m[3][3]) < 1.0e-6f) return false;
    *lu = r;
    return true;
}
// matrix4x4.rs:119-142
void m4_solve(const M4& lu, const int pivot[4], float b[4]) {
    for (int k = 0; k < 3; ++k) {
        if (pivot[k] != k) std::swap(b[pivot[k]], b[k]);
        for (int i = k + 1; i < 4; ++i) b[i] = b[i] - lu.m[i][k] * b[k];
    }
    b[3] = b[3] / lu.m[3][3];
    for (int i = 2; i >= 0; --i) {
        float sum = 0.0f;
        for (int j = i + 1; j < 4; ++j) sum = sum + lu.m[i][j] * b[j];
        b[i] = (b[i] - sum) / lu.m[i][i];
    }
}
// matrix4x4.rs:147-160
bool m4_invert(const M4& a, M4* out) {
    M4 lu;
    int pivot[4];
    if (!m4_lu(a, &lu, pivot)) return false;
    M4 rows;
    for (int c = 0; c < 4; ++c) {
        float b[4] = {0, 0, 0, 0};
        b[c] = 1.0f;
        m4_solve(lu, pivot, b);
        for (int j = 0; j < 4; ++j) rows.m[c][j] = b[j];
    }
    *out = m4_transpose(rows);
    return true;
}

// src/transform/transform.rs
struct Xf {
    M4 m, mi;
};
Xf xf_identity() { return Xf{m4_identity(), m4_identity()}; }
Xf xf_inverse(const Xf& t) { return Xf{t.mi, t.m}; }
// transform.rs:266-271
Xf xf_mul(const Xf& a, const Xf& b) { return Xf{m4_mul(a.m, b.m), m4_mul(b.mi, a.mi)}; }
// transform.rs:288-293 (From<Matrix4x4>)
Xf xf_from(const M4& m) {
    M4 inv;
    if (!m4_invert(m, &inv)) {
        fprintf(stderr, "oracle: singular matrix\n");
        inv = m4_identity();
    }
    return Xf{m, inv};
}
// transform.rs:39-51
Xf xf_translate(V3 v) {
    Xf t = xf_identity();
    t.m.m[0][3] = v.x;
    t.m.m[1][3] = v.y;
    t.m.m[2][3] = v.z;
    t.mi.m[0][3] = -v.x;
    t.mi.m[1][3] = -v.y;
    t.mi.m[2][3] = -v.z;
    return t;
}
// transform.rs:53-65
Xf xf_scale(float x, float y, float z) {
    Xf t = xf_identity();
    t.m.m[0][0] = x;
    t.m.m[1][1] = y;
    t.m.m[2][2] = z;
    t.mi.m[0][0] = 1.0f / x;
    t.mi.m[1][1] = 1.0f / y;
    t.mi.m[2][2] = 1.0f / z;
    return t;
}
// transform.rs:195-208
V3 xf_point(const M4& m, V3 p) {
    float xt = m.m[0][0] * p.x + m.m[0][1] * p.y + m.m[0][2] * p.z + m.m[0][3];
    float yt = m.m[1][0] * p.x + m.m[1][1] * p.y + m.m[1][2] * p.z + m.m[1][3];
    float zt = m.m[2][0] * p.x + m.m[2][1] * p.y + m.m[2][2] * p.z + m.m[2][3];
    float w = m.m[3][0] * p.x + m.m[3][1] * p.y + m.m[3][2] * p.z + m.m[3][3];
    if (w != 1.0f) return mk(xt / w, yt / w, zt / w);
    return mk(xt, yt, zt);
}
// transform.rs:210-218
V3 xf_vector(const M4& m, V3 v) {
    return mk(m.m[0][0] * v.x + m.m[0][1] * v.y + m.m[0][2] * v.z,
              m.m[1][0] * v.x + m.m[1][1] * v.y + m.m[1][2] * v.z,
              m.m[2][0] * v.x + m.m[2][1] * v.y + m.m[2][2] * v.z);
}
// transform.rs:176-183
bool swaps_handedness(const M4& m) {
    float det = m.m[0][0] * (m.m[1][1] * m.m[2][2] - m.m[1][2] * m.m[2][1]) -
                m.m[0][1] * (m.m[1][0] * m.m[2][2] - m.m[1][2] * m.m[2][0]) +
                m.m[0][2] * (m.m[1][0] * m.m[2][1] - m.m[1][1] * m.m[2][0]);
    return 0.0f > det;
}
// transform.rs:248-263
BBox xf_bbox(const M4& m, const BBox& b) {
    V3 tx = xf_vector(m, mk(b.pmax.x - b.pmin.x, 0.0f, 0.0f));
    V3 ty = xf_vector(m, mk(0.0f, b.pmax.y - b.pmin.y, 0.0f));
    V3 tz = xf_vector(m, mk(0.0f, 0.0f, b.pmax.z - b.pmin.z));
    V3 tp = xf_point(m, b.pmin);
    BBox r = bbox_pt(tp);
    r = union_pt(r, add(tp, tx));
    r = union_pt(r, add(tp, ty));
    r = union_pt(r, add(tp, tz));
    r = union_pt(r, add(add(tp, tx), ty));
    r = union_pt(r, add(add(tp, tx), tz));
    r = union_pt(r, add(add(tp, ty), tz));
    r = union_pt(r, add(add(add(tp, tx), ty), tz));
    return r;
}
// transform.rs:144-174
Xf xf_look_at(V3 pos, V3 look, V3 up) {
    M4 m = m4_identity();
    m.m[0][3] = pos.x;
    m.m[1][3] = pos.y;
    m.m[2][3] = pos.z;
    m.m[3][3] = 1.0f;
    V3 dir = normalize(sub(look, pos));
    V3 left = normalize(cross(normalize(up), dir));
    V3 new_up = cross(dir, left);
    m.m[0][0] = left.x;
    m.m[1][0] = left.y;
    m.m[2][0] = left.z;
    m.m[3][0] = 0.0f;
    m.m[0][1] = new_up.x;
    m.m[1][1] = new_up.y;
    m.m[2][1] = new_up.z;
    m.m[3][1] = 0.0f;
    m.m[0][2] = dir.x;
    m.m[1][2] = dir.y;
    m.m[2][2] = dir.z;
    m.m[3][2] = 0.0f;
    M4 inv;
    if (!m4_invert(m, &inv)) inv = m4_identity();
    return Xf{inv, m};
}
Xf xf_from_desc(const PbrtTransform& t) {
    Xf r;
    memcpy(r.m.m, t.m, sizeof(float) * 16);
    memcpy(r.mi.m, t.m_inv, sizeof(float) * 16);
    return r;
}
void xf_to_desc(const Xf& x, PbrtTransform* t) {
    memcpy(t->m, x.m.m, sizeof(float) * 16);
    memcpy(t->m_inv, x.mi.m, sizeof(float) * 16);
}

// --------------------------------------------------------------- utils ----
// src/utils/mod.rs:56-92
bool quadratic(float a, float b, float c, float* t0, float* t1) {
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
    float q = (b < 0.0f) ? -0.5f * (b - root) : -0.5f * (b + root);
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

// src/utils/mod.rs:112-169 (median-of-three quickselect; recursion on one side)
template <class T, class F>
void partition_by(T* v, size_t nv, F f) {
    if (nv < 3) {
        if (nv == 2 && f(v[1]) < f(v[0])) std::swap(v[0], v[1]);
        return;
    }
    auto fst = f(v[0]);
    auto mid = f(v[nv / 2]);
    auto lst = f(v[nv - 1]);
    auto pivot = (fst < mid && mid < lst) ? mid : ((mid < fst && fst < lst) ? fst : lst);
    size_t last_smaller = 0, num_pivots = 0;
    for (size_t i = 0; i < nv; ++i) {
        auto bv = f(v[i]);
        if (bv < pivot) {
            std::swap(v[last_smaller + num_pivots], v[i]);
            std::swap(v[last_smaller + num_pivots], v[last_smaller]);
            last_smaller += 1;
        } else if (bv == pivot) {
            std::swap(v[last_smaller + num_pivots], v[i]);
            num_pivots += 1;
        }
    }
    size_t pivot_idx = std::max<size_t>(last_smaller, 1);
    if (pivot_idx + num_pivots <= nv / 2)
        partition_by(v + pivot_idx, nv - pivot_idx, f);
    else if (pivot_idx >= nv / 2)
        partition_by(v, pivot_idx, f);
}

// src/utils/mod.rs:171-180
void num_subwindows_2d(size_t count, size_t aspect, size_t* nx, size_t* ny) {
    size_t x = 1, y = count;
    while ((y % 2) == 0 && 2 * aspect * x < y) {
        y /= 2;
        x *= 2;
    }
    *nx = x;
    *ny = y;
}
// Rust `f as usize`: saturating, NaN -> 0
inline size_t f2usize(float f) {
    if (!(f > 0.0f)) return 0;
    if (f >= 18446744073709551615.0f) return SIZE_MAX;
    return (size_t)f;
}
// Rust `f as i32`: saturating, NaN -> 0
inline int32_t f2i32(float f) {
    if (f != f) return 0;
    if (f >= 2147483647.0f) return INT32_MAX;
    if (f <= -2147483648.0f) return INT32_MIN;
    return (int32_t)f;
}
// src/utils/mod.rs:183-205
void crop_window(size_t num, size_t count, float aspect, float out[4]) {
    size_t nx, ny;
    if (aspect < 1.0f) {
        size_t inva = f2usize(1.0f / aspect);
        num_subwindows_2d(count, inva, &nx, &ny);
    } else {
        size_t x, y;
        num_subwindows_2d(count, f2usize(aspect), &x, &y);
        nx = y;
        ny = x;
    }
    size_t xo = num % nx, yo = num / nx;
    out[0] = (float)xo / (float)nx;
    out[1] = (float)(xo + 1) / (float)nx;
    out[2] = (float)yo / (float)ny;
    out[3] = (float)(yo + 1) / (float)ny;
}
// src/sampler/base.rs:29-48
void sub_window(int32_t xs, int32_t xe, int32_t ys, int32_t ye, size_t num, size_t count,
                int32_t out[4]) {
    size_t dx = (size_t)(xe - xs), dy = (size_t)(ye - ys);
    float aspect = (float)dx / (float)dy;
    float t[4];
    crop_window(num, count, aspect, t);
    float psx = (float)xs, psy = (float)ys, pex = (float)xe, pey = (float)ye;
    out[0] = f2i32(lerpf(psx, pex, t[0]));
    out[1] = f2i32(lerpf(psx, pex, t[1]));
    out[2] = f2i32(lerpf(psy, pey, t[2]));
    out[3] = f2i32(lerpf(psy, pey, t[3]));
}

// ---------------------------------------------------------------- RNG ----
// src/rng.rs: RNG = rand::rngs::StdRng (rand 0.8.5) = ChaCha12 (rand_chacha
// 0.3.1) seeded by rand_core 0.6.4 SeedableRng::seed_from_u64.
// Restated from the published algorithms: ChaCha (Bernstein 2008; state
// layout of RFC 8439 with a 64-bit block counter in words 12-13 and a
// zero 64-bit stream id in words 14-15), 12 rounds; the 32-byte key is
// eight PCG32 (O'Neill 2014, XSH-RR) outputs with multiplier
// 6364136223846793005 and increment 11634580027462260723, the state
// advanced before each output.  Output words are the keystream words in
// order; next_u64 takes two consecutive words, low first.
inline uint32_t rotl32(uint32_t v, int c) { return (v << c) | (v >> (32 - c)); }
inline uint32_t rotr32(uint32_t v, uint32_t c) { return (v >> (c & 31)) | (v << ((32 - c) & 31)); }

void seed_key(uint64_t state, uint32_t key[8]) {
    const uint64_t MUL = 6364136223846793005ULL;
    const uint64_t INC = 11634580027462260723ULL;
    for (int i = 0; i < 8; ++i) {
        state = state * MUL + INC;
        uint32_t xorshifted = (uint32_t)(((state >> 18) ^ state) >> 27);
        uint32_t rot = (uint32_t)(state >> 59);
        key[i] = rotr32(xorshifted, rot);
    }
}

#define QR(a, b, c, d)                                   \
    a += b; d ^= a; d = rotl32(d, 16);                   \
    c += d; b ^= c; b = rotl32(b, 12);                   \
    a += b; d ^= a; d = rotl32(d, 8);                    \
    c += d; b ^= c; b = rotl32(b, 7);

// One ChaCha block of `rounds` rounds (an even count: rounds / 2 double
// rounds of four column and four diagonal quarter rounds) over the state
// constants | key | 64-bit block counter | 64-bit stream id, plus the input.
void chacha_block(const uint32_t key[8], uint64_t ctr, uint64_t stream, int rounds, uint32_t out[16]) {
    uint32_t s[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u,
                      key[0], key[1], key[2], key[3], key[4], key[5], key[6], key[7],
                      (uint32_t)ctr, (uint32_t)(ctr >> 32), (uint32_t)stream, (uint32_t)(stream >> 32)};
    uint32_t x[16];
    memcpy(x, s, sizeof(s));
    for (int r = 0; r < rounds / 2; ++r) {
        QR(x[0], x[4], x[8], x[12]);
        QR(x[1], x[5], x[9], x[13]);
        QR(x[2], x[6], x[10], x[14]);
        QR(x[3], x[7], x[11], x[15]);
        QR(x[0], x[5], x[10], x[15]);
        QR(x[1], x[6], x[11], x[12]);
        QR(x[2], x[7], x[8], x[13]);
        QR(x[3], x[4], x[9], x[14]);
    }
    for (int i = 0; i < 16; ++i) out[i] = x[i] + s[i];
}

// StdRng's block: 12 rounds, stream id 0.
void chacha12_block(const uint32_t key[8], uint64_t ctr, uint32_t out[16]) { chacha_block(key, ctr, 0, 12, out); }

struct RNG {
    uint32_t key[8];
    uint64_t block = 0;
    uint32_t buf[16];
    int idx = 16;
    uint64_t words = 0;
    explicit RNG(uint64_t seed) { seed_key(seed, key); }
    uint32_t next_u32() {
        if (idx == 16) {
            chacha12_block(key, block, buf);
            block += 1;
            idx = 0;
        }
        words += 1;
        return buf[idx++];
    }
    uint64_t next_u64() {
        uint64_t lo = next_u32();
        uint64_t hi = next_u32();
        return lo | (hi << 32);
    }
    // rng.rs:15-17: gen::<f32>() = (u32 >> 8) * 2^-24
    float random_float() { return (float)(next_u32() >> 8) * (1.0f / 16777216.0f); }
    // rng.rs:19-21
    uint64_t random_uint() { return next_u64() % 0xFFFFFFFFFFFFFFFFULL; }
    // rng.rs:23-33
    template <class T>
    void shuffle(T* v, size_t len, size_t dims) {
        size_t count = len / dims;
        for (size_t i = 0; i < count; ++i) {
            size_t other = i + (size_t)(random_uint() % (uint64_t)(count - i));
            for (size_t j = 0; j < dims; ++j) std::swap(v[dims * i + j], v[dims * other + j]);
        }
    }
};

// src/montecarlo.rs:88-104
void latin_hypercube(float* samples, size_t num, size_t dim, RNG& rng) {
    float delta = 1.0f / (float)num;
    for (size_t i = 0; i < num; ++i)
        for (size_t j = 0; j < dim; ++j) samples[dim * i + j] = ((float)i + rng.random_float()) * delta;
    for (size_t i = 0; i < dim; ++i)
        for (size_t j = 0; j < num; ++j) {
            size_t other = j + (size_t)(rng.random_uint() % (uint64_t)(num - j));
            std::swap(samples[dim * j + i], samples[dim * other + i]);
        }
}
// src/montecarlo.rs:106-113
void stratified_1d(float* samples, size_t n, RNG& rng, bool jitter) {
    float inv_tot = 1.0f / (float)n;
    for (size_t i = 0; i < n; ++i) {
        float delta = jitter ? rng.random_float() : 0.5f;
        samples[i] = ((float)i + delta) * inv_tot;
    }
}
// src/montecarlo.rs:115-128
void stratified_2d(float* samples, size_t nx, size_t ny, RNG& rng, bool jitter) {
    float dx = 1.0f / (float)nx, dy = 1.0f / (float)ny;
    for (size_t y = 0; y < ny; ++y)
        for (size_t x = 0; x < nx; ++x) {
            float jx = jitter ? rng.random_float() : 0.5f;
            float jy = jitter ? rng.random_float() : 0.5f;
            size_t off = 2 * (y * nx + x);
            samples[off] = ((float)x + jx) * dx;
            samples[off + 1] = ((float)y + jy) * dy;
        }
}

// -------------------------------------------------------------- shapes ----
struct Tri {
    V3 p1, p2, p3;  // mesh.rs:33-39 with v = refined (reversed) order
    bool flip;      // reverse_orientation ^ transform_swaps_handedness
};
// mesh.rs:196-205
BBox tri_bound(const Tri& t) { return union_pt(union_pt(union_pt(bbox_new(), t.p1), t.p2), t.p3); }
// mesh.rs:41-72
bool tri_hit(const Tri& tr, const Ray& r, float* t_out, float* b1_out, float* b2_out) {
    V3 e1 = sub(tr.p2, tr.p1);
    V3 e2 = sub(tr.p3, tr.p1);
    V3 s1 = cross(r.d, e2);
    float divisor = dot(s1, e1);
    if (divisor == 0.0f) return false;
    float inv = 1.0f / divisor;
    V3 s = sub(r.o, tr.p1);
    float b1 = dot(s1, s) * inv;
    if (b1 < 0.0f || b1 > 1.0f) return false;
    V3 s2 = cross(s, e1);
    float b2 = dot(r.d, s2) * inv;
    if (b2 < 0.0f || (b1 + b2) > 1.0f) return false;
    float t = dot(e2, s2) * inv;
    if (t < r.mint || t > r.maxt) return false;
    *t_out = t;
    *b1_out = b1;
    *b2_out = b2;
    return true;
}
// mesh.rs:100-103
float tri_area(const Tri& t) { return 0.5f * length(cross(sub(t.p2, t.p1), sub(t.p3, t.p1))); }
// mesh.rs:212-264 + diff_geom.rs:52-79, default uvs (0,0),(1,0),(1,1)
void tri_dg(const Tri& tr, const Ray& r, float t, V3* p, V3* nn, V3* dpdu_out) {
    const float du1 = 0.0f - 1.0f, du2 = 1.0f - 1.0f, dv1 = 0.0f - 1.0f, dv2 = 0.0f - 1.0f;
    V3 dp1 = sub(tr.p1, tr.p3), dp2 = sub(tr.p2, tr.p3);
    float determinant = du1 * dv2 - dv1 * du2;
    V3 dpdu, dpdv;
    if (determinant == 0.0f) {
        dpdu = mk(0, 0, 0);  // unreachable with the default uvs
        dpdv = mk(0, 0, 0);
    } else {
        float inv_det = 1.0f / determinant;
        dpdu = mul(sub(mul(dp1, dv2), mul(dp2, dv1)), inv_det);
        dpdv = mul(add(mul(dp1, -du2), mul(dp2, du1)), inv_det);
    }
    *p = point_at(r, t);
    V3 n = normalize(cross(dpdu, dpdv));
    if (tr.flip) n = mul(n, -1.0f);
    *nn = n;
    if (dpdu_out) *dpdu_out = dpdu;
}

// Analytic shapes: sphere (sphere.rs:16-25), disk (disk.rs:16-22) and
// cylinder (cylinder.rs:16-23).  A disk keeps its height in z_min = z_max.
enum { QUAD_SPHERE = 0, QUAD_DISK = 1, QUAD_CYLINDER = 2 };
struct Sphere {
    Xf o2w, w2o;
    bool flip;
    float radius, phi_max, z_min, z_max, theta_min, theta_max;
    int kind = QUAD_SPHERE;
    float height = 0.0f, inner_radius = 0.0f;
};
// sphere.rs:28-44
Sphere sphere_new(const Xf& o2w, const Xf& w2o, bool ro, float rad, float z0, float z1, float pm) {
    Sphere s;
    s.o2w = o2w;
    s.w2o = w2o;
    s.flip = ro != swaps_handedness(o2w.m);
    s.radius = rad;
    s.z_min = clampf(fminf(z0, z1), -rad, rad);
    s.z_max = clampf(fmaxf(z0, z1), -rad, rad);
    s.theta_min = acosf(s.z_min / rad);
    s.theta_max = acosf(s.z_max / rad);
    s.phi_max = as_radians(clampf(pm, 0.0f, 360.0f));
    return s;
}
// disk.rs:24-34
Sphere disk_new(const Xf& o2w, const Xf& w2o, bool ro, float ht, float r, float ri, float tmax) {
    Sphere s{};
    s.o2w = o2w;
    s.w2o = w2o;
    s.flip = ro != swaps_handedness(o2w.m);
    s.kind = QUAD_DISK;
    s.height = ht;
    s.radius = r;
    s.inner_radius = ri;
    s.z_min = s.z_max = ht;
    s.phi_max = as_radians(clampf(tmax, 0.0f, 360.0f));
    return s;
}
// cylinder.rs:26-36
Sphere cylinder_new(const Xf& o2w, const Xf& w2o, bool ro, float rad, float z0, float z1, float pm) {
    Sphere s{};
    s.o2w = o2w;
    s.w2o = w2o;
    s.flip = ro != swaps_handedness(o2w.m);
    s.kind = QUAD_CYLINDER;
    s.radius = rad;
    s.z_min = fminf(z0, z1);
    s.z_max = fmaxf(z0, z1);
    s.phi_max = as_radians(clampf(pm, 0.0f, 360.0f));
    return s;
}
// sphere.rs:111-126, disk.rs:68-74, cylinder.rs:96-100
BBox sphere_bound(const Sphere& s) {
    BBox ob{mk(-s.radius, -s.radius, s.z_min), mk(s.radius, s.radius, s.z_max)};
    return xf_bbox(s.o2w.m, ob);
}
// transform.rs:230-237
Ray xf_ray(const M4& m, const Ray& r) {
    Ray o = r;
    o.o = xf_point(m, r.o);
    o.d = xf_vector(m, r.d);
    return o;
}
// sphere.rs:46-107 (ray in object space)
bool sphere_hit_obj(const Sphere& s, const Ray& ray, float* t_out, float* phi_out) {
    float a = length_sq(ray.d);
    float b = 2.0f * dot(ray.d, ray.o);
    float c = length_sq(ray.o) - s.radius * s.radius;
    float t0, t1;
    if (!quadratic(a, b, c, &t0, &t1)) return false;
    if (t0 > ray.maxt || t1 < ray.mint) return false;
    float t_hit = t0;
    if (t0 < ray.mint) {
        t_hit = t1;
        if (t_hit > ray.maxt) return false;
    }
    auto get_hit = [&](float t, V3* hit, float* angle) {
        V3 h = point_at(ray, t);
        if (h.x == 0.0f && h.y == 0.0f) h.x = 1e-5f * s.radius;
        float a2 = atan2f(h.y, h.x);
        if (a2 < 0.0f) a2 += 2.0f * kPi;
        *hit = h;
        *angle = a2;
    };
    auto invalid = [&](V3 h, float phi) {
        return (h.z > -s.radius && h.z < s.z_min) || (h.z < s.radius && h.z > s.z_max) ||
               (phi > s.phi_max);
    };
    V3 h;
    float phi;
    get_hit(t_hit, &h, &phi);
    if (invalid(h, phi)) {
        if (t_hit == t1) return false;
        if (t1 > ray.maxt) return false;
        t_hit = t1;
        get_hit(t_hit, &h, &phi);
        if (invalid(h, phi)) return false;
    }
    *t_out = t_hit;
    *phi_out = phi;
    return true;
}
// disk.rs:36-66 (ray in object space)
bool disk_hit_obj(const Sphere& s, const Ray& ray, float* t_out, float* phi_out) {
    if (fabsf(ray.d.z) < 1e-6f) return false;
    float t_hit = (s.height - ray.o.z) / ray.d.z;
    if (t_hit < ray.mint || t_hit > ray.maxt) return false;
    V3 p = point_at(ray, t_hit);
    float dist2 = p.x * p.x + p.y * p.y;
    if (dist2 > (s.radius * s.radius) || dist2 < (s.inner_radius * s.inner_radius)) return false;
    float phi = atan2f(p.y, p.x);
    if (phi < 0.0f) phi = phi + 2.0f * kPi;
    if (phi > s.phi_max) return false;
    *t_out = t_hit;
    *phi_out = phi;
    return true;
}
// cylinder.rs:38-94 (ray in object space)
bool cylinder_hit_obj(const Sphere& s, const Ray& ray, float* t_out, float* phi_out) {
    float a = ray.d.x * ray.d.x + ray.d.y * ray.d.y;
    float b = 2.0f * (ray.d.x * ray.o.x + ray.d.y * ray.o.y);
    float c = ray.o.x * ray.o.x + ray.o.y * ray.o.y - s.radius * s.radius;
    float t0, t1;
    if (!quadratic(a, b, c, &t0, &t1)) return false;
    if (t0 > ray.maxt || t1 < ray.mint) return false;
    float t_hit = t0;
    if (t0 < ray.mint) {
        t_hit = t1;
        if (t_hit > ray.maxt) return false;
    }
    auto get_hit = [&](float t, V3* hit, float* angle) {
        V3 h = point_at(ray, t);
        if (h.x == 0.0f && h.y == 0.0f) h.x = 1e-5f * s.radius;
        float a2 = atan2f(h.y, h.x);
        if (a2 < 0.0f) a2 = a2 + 2.0f * kPi;
        *hit = h;
        *angle = a2;
    };
    auto invalid = [&](V3 h, float phi) { return h.z < s.z_min || h.z > s.z_max || phi > s.phi_max; };
    V3 h;
    float phi;
    get_hit(t_hit, &h, &phi);
    if (invalid(h, phi)) {
        if (t_hit == t1) return false;
        if (t1 > ray.maxt) return false;
        t_hit = t1;
        get_hit(t_hit, &h, &phi);
        if (invalid(h, phi)) return false;
    }
    *t_out = t_hit;
    *phi_out = phi;
    return true;
}
bool quad_hit_obj(const Sphere& s, const Ray& ray, float* t_out, float* phi_out) {
    if (s.kind == QUAD_DISK) return disk_hit_obj(s, ray, t_out, phi_out);
    if (s.kind == QUAD_CYLINDER) return cylinder_hit_obj(s, ray, t_out, phi_out);
    return sphere_hit_obj(s, ray, t_out, phi_out);
}
// transform.rs:220-227: normals go through the inverse transpose
V3 xf_normal(const M4& m_inv, V3 n) {
    return mk(m_inv.m[0][0] * n.x + m_inv.m[1][0] * n.y + m_inv.m[2][0] * n.z,
              m_inv.m[0][1] * n.x + m_inv.m[1][1] * n.y + m_inv.m[2][1] * n.z,
              m_inv.m[0][2] * n.x + m_inv.m[1][2] * n.y + m_inv.m[2][2] * n.z);
}
// disk.rs:96-131 and cylinder.rs:131-166 (with helpers.rs:17-43): hit point
// and geometric normal.  The disk's normal is the transformed +-z by the side
// of the object-space ray origin, not normalised nor flipped.
void quad_dg(const Sphere& s, const Ray& obj_ray, float t_hit, float phi, V3* p, V3* nn, float* u_out,
             float* v_out, V3* dpdu_o, V3* dpdv_o) {
    V3 ph = point_at(obj_ray, t_hit);
    *p = xf_point(s.o2w.m, ph);
    if (s.kind == QUAD_DISK) {
        float dist = sqrtf(ph.x * ph.x + ph.y * ph.y);
        float u = phi / s.phi_max;
        float v = 1.0f - (dist - s.inner_radius) / (s.radius - s.inner_radius);
        V3 dpdu = mul(mk(-s.phi_max * ph.y, s.phi_max * ph.x, 0.0f), s.phi_max / (2.0f * kPi));
        V3 dpdv = mul(mk(ph.x, ph.y, 0.0f), (s.inner_radius - s.radius) / dist);
        *nn = xf_normal(s.w2o.m, mk(0.0f, 0.0f, obj_ray.o.z > 0.0f ? 1.0f : -1.0f));
        if (u_out) *u_out = u;
        if (v_out) *v_out = v;
        if (dpdu_o) *dpdu_o = xf_vector(s.o2w.m, dpdu);
        if (dpdv_o) *dpdv_o = xf_vector(s.o2w.m, dpdv);
        return;
    }
    float u = phi / s.phi_max;
    float v = (ph.z - s.z_min) / (s.z_max - s.z_min);
    V3 dpdu = mul(mk(-ph.y, ph.x, 0.0f), s.phi_max);
    V3 dpdv = mk(0.0f, 0.0f, s.z_max - s.z_min);
    V3 du = xf_vector(s.o2w.m, dpdu), dv = xf_vector(s.o2w.m, dpdv);
    V3 n = normalize(cross(du, dv));
    if (s.flip) n = mul(n, -1.0f);
    *nn = n;
    if (u_out) *u_out = u;
    if (v_out) *v_out = v;
    if (dpdu_o) *dpdu_o = du;
    if (dpdv_o) *dpdv_o = dv;
}
// sphere.rs:135-176 + shape/helpers.rs:17-43 + diff_geom.rs:52-79
void sphere_dg(const Sphere& s, const Ray& obj_ray, float t_hit, float phi, V3* p, V3* nn, V3* dpdu_w,
               float* u_out, float* v_out, V3* dpdu_o, V3* dpdv_o) {
    V3 ph = point_at(obj_ray, t_hit);
    float u = phi / s.phi_max;
    float theta = acosf(clampf(ph.z / s.radius, -1.0f, 1.0f));
    float v = (theta - s.theta_min) / (s.theta_max - s.theta_min);
    float zradius = sqrtf(ph.x * ph.x + ph.y * ph.y);
    float inv_zradius = 1.0f / zradius;
    float cos_phi = ph.x * inv_zradius;
    float sin_phi = ph.y * inv_zradius;
    V3 dpdu = mk(-s.phi_max * ph.y, s.phi_max * ph.x, 0.0f);
    V3 dpdv = mul(mk(ph.z * cos_phi, ph.z * sin_phi, -s.radius * sinf(theta)), s.theta_max - s.theta_min);
    V3 pw = xf_point(s.o2w.m, ph);
    V3 du = xf_vector(s.o2w.m, dpdu), dv = xf_vector(s.o2w.m, dpdv);
    V3 n = normalize(cross(du, dv));
    if (s.flip) n = mul(n, -1.0f);
    *p = pw;
    *nn = n;
    if (dpdu_w) *dpdu_w = du;
    if (u_out) *u_out = u;
    if (v_out) *v_out = v;
    if (dpdu_o) *dpdu_o = du;
    if (dpdv_o) *dpdv_o = dv;
}

// ----------------------------------------------------------- primitives ---
enum { KIND_TRI = 0, KIND_SPHERE = 1, KIND_INST = 2 };
struct Prim {
    int kind;
    int shape;
    int material;
    int area_light;
    Tri tri;
    int sphere;  // index into spheres
};

// TransformedPrimitive (transformed.rs:14-33) with a static transform:
// w2p = the instance's world-to-primitive matrix, i2w its inverse as given
// (Transform::invert swaps the pair, transform.rs:31-33).
struct Inst {
    M4 i2w, w2i;
    int def;  // index into Refined::defs
};

struct Refined {
    std::vector<Prim> prims;
    std::vector<Sphere> spheres;
    std::vector<Inst> insts;
    std::vector<std::shared_ptr<OracleBVH>> defs;  // instance definitions' aggregates
    std::vector<uint32_t> first_id;  // with instances: the hit id of each refined primitive
    std::string err;
};

Xf desc_o2w(const PbrtShapeDesc& d) { return xf_from_desc(d.object_to_world); }

// Fully refine the input (primitive/mod.rs:47-63, mesh.rs:298-338): a mesh
// becomes its triangles in index order, each with vertices
// (i[3k+2], i[3k+1], i[3k]) of the world-space points.
bool refine_shapes(const PbrtShapeDesc* shapes, uint32_t n, Refined* out) {
    for (uint32_t si = 0; si < n; ++si) {
        const PbrtShapeDesc& d = shapes[si];
        Xf o2w = desc_o2w(d);
        bool flip = (d.reverse_orientation != 0) != swaps_handedness(o2w.m);
        if (d.kind == PBRT_SHAPE_TRIANGLE_MESH) {
            if (d.n_indices % 3 != 0) {
                out->err = "mesh index count is not a multiple of 3";
                return false;
            }
            std::vector<V3> wp(d.n_points);
            for (uint32_t i = 0; i < d.n_points; ++i)
                wp[i] = xf_point(o2w.m, mk(d.points[3 * i], d.points[3 * i + 1], d.points[3 * i + 2]));
            uint32_t nt = d.n_indices / 3;
            for (uint32_t k = 0; k < nt; ++k) {
                uint32_t i0 = d.indices[3 * k], i1 = d.indices[3 * k + 1], i2 = d.indices[3 * k + 2];
                if (i0 >= d.n_points || i1 >= d.n_points || i2 >= d.n_points) {
                    out->err = "mesh index out of range";
                    return false;
                }
                Prim p;
                p.kind = KIND_TRI;
                p.shape = (int)si;
                p.material = d.material;
                p.area_light = d.area_light;
                p.tri = Tri{wp[i2], wp[i1], wp[i0], flip};
                p.sphere = -1;
                out->prims.push_back(p);
            }
        } else if (d.kind == PBRT_SHAPE_SPHERE || d.kind == PBRT_SHAPE_DISK || d.kind == PBRT_SHAPE_CYLINDER) {
            const bool ro = d.reverse_orientation != 0;
            Sphere s = d.kind == PBRT_SHAPE_SPHERE
                           ? sphere_new(o2w, xf_inverse(o2w), ro, d.radius, d.z0, d.z1, d.phi_max_deg)
                       : d.kind == PBRT_SHAPE_DISK
                           ? disk_new(o2w, xf_inverse(o2w), ro, d.height, d.radius, d.inner_radius, d.phi_max_deg)
                           : cylinder_new(o2w, xf_inverse(o2w), ro, d.radius, d.z0, d.z1, d.phi_max_deg);
            Prim p;
            p.kind = KIND_SPHERE;
            p.shape = (int)si;
            p.material = d.material;
            p.area_light = d.area_light;
            p.tri = Tri{};
            p.sphere = (int)out->spheres.size();
            out->spheres.push_back(s);
            out->prims.push_back(p);
        } else if (d.kind == PBRT_SHAPE_INSTANCE) {
            if (d.instance < 0 || (size_t)d.instance >= out->defs.size()) {
                out->err = "instance: definition index out of range";
                return false;
            }
            Prim p;
            p.kind = KIND_INST;
            p.shape = (int)si;
            p.material = -1;
            p.area_light = -1;
            p.tri = Tri{};
            p.sphere = (int)out->insts.size();
            out->insts.push_back(Inst{o2w.m, o2w.mi, d.instance});
            out->prims.push_back(p);
        } else {
            out->err = "unknown shape kind";
            return false;
        }
    }
    return true;
}

BBox def_bound(const OracleBVH* o);
size_t def_size(const OracleBVH* o);

BBox prim_bound(const Refined& R, const Prim& p) {
    if (p.kind == KIND_TRI) return tri_bound(p.tri);
    if (p.kind == KIND_INST) {
        // transformed.rs:62-65 + animated.rs:226-233: the definition's
        // bound through start_transform.inverse() = primitive-to-world
        const Inst& I = R.insts[p.sphere];
        return xf_bbox(I.i2w, def_bound(R.defs[I.def].get()));
    }
    return sphere_bound(R.spheres[p.sphere]);
}

// ----------------------------------------------------------------- BVH ----
// src/primitive/aggregates/bvh.rs
enum SplitMethod { SPLIT_SAH = 0, SPLIT_MIDDLE = 1, SPLIT_EQUAL = 2 };

struct PrimInfo {  // bvh.rs:66-84
    uint32_t prim;
    V3 centroid;
    BBox bounds;
};
struct BuildNode {
    bool leaf;
    BBox bounds;
    uint32_t first, count;
    int c1, c2, axis;
    uint32_t num_nodes;
};
struct Builder {
    std::vector<BuildNode> nodes;
    std::vector<uint32_t> ordered;
    uint32_t mp;
    SplitMethod sm;
    bool failed = false;
    std::string err;
};

const size_t NUM_BUCKETS = 12;

int make_leaf(Builder& B, const BBox& bounds, std::vector<PrimInfo>& prims) {
    BuildNode n{};
    n.leaf = true;
    n.bounds = bounds;
    n.first = (uint32_t)B.ordered.size();
    n.count = (uint32_t)prims.size();
    n.num_nodes = 1;
    for (auto& p : prims) B.ordered.push_back(p.prim);
    B.nodes.push_back(n);
    return (int)B.nodes.size() - 1;
}

// bvh.rs:189-258
int recursive_build(Builder& B, std::vector<PrimInfo> prims) {
    BBox bbox = bbox_new();
    for (auto& p : prims) bbox = union_box(bbox, p.bounds);
    size_t num_prims = prims.size();
    if (num_prims == 1) return make_leaf(B, bbox, prims);
    BBox cb = bbox_new();
    for (auto& p : prims) cb = union_pt(cb, p.centroid);
    int dim = max_extent(cb);
    if (comp(cb.pmin, dim) == comp(cb.pmax, dim)) return make_leaf(B, bbox, prims);

    std::vector<PrimInfo> p1, p2;
    auto equal_counts = [&](std::vector<PrimInfo>& v) {  // bvh.rs:92-103
        partition_by(v.data(), v.size(), [dim](const PrimInfo& p) { return comp(p.centroid, dim); });
        size_t n = v.size();
        for (size_t i = 0; i < n; ++i) (i < n / 2 ? p1 : p2).push_back(v[i]);
    };
    if (B.sm == SPLIT_MIDDLE) {  // bvh.rs:86-90
        float p_mid = 0.5f * (comp(cb.pmin, dim) + comp(cb.pmax, dim));
        for (auto& p : prims) (comp(p.centroid, dim) < p_mid ? p1 : p2).push_back(p);
    } else if (B.sm == SPLIT_EQUAL) {
        equal_counts(prims);
    } else {  // bvh.rs:105-186
        if (num_prims <= 4) {
            equal_counts(prims);
        } else {
            size_t cnt[NUM_BUCKETS];
            BBox bb[NUM_BUCKETS];
            for (size_t i = 0; i < NUM_BUCKETS; ++i) {
                cnt[i] = 0;
                bb[i] = bbox_new();
            }
            auto bucket_for = [&](const PrimInfo& p) {
                float pdist = comp(p.centroid, dim) - comp(cb.pmin, dim);
                float dist = comp(cb.pmax, dim) - comp(cb.pmin, dim);
                size_t b = f2usize((float)NUM_BUCKETS * (pdist / dist));
                return b == NUM_BUCKETS ? NUM_BUCKETS - 1 : b;
            };
            for (auto& p : prims) {
                size_t b = bucket_for(p);
                cnt[b] += 1;
                bb[b] = union_box(bb[b], p.bounds);
            }
            float costs[NUM_BUCKETS - 1];
            for (size_t i = 0; i < NUM_BUCKETS - 1; ++i) {
                size_t c0 = 0, c1 = 0;
                BBox b0 = bbox_new(), b1 = bbox_new();
                for (size_t j = 0; j <= i; ++j) {
                    c0 += cnt[j];
                    b0 = union_box(b0, bb[j]);
                }
                for (size_t j = i + 1; j < NUM_BUCKETS; ++j) {
                    c1 += cnt[j];
                    b1 = union_box(b1, bb[j]);
                }
                float b0sa = (float)c0 * surface_area(b0);
                float b1sa = (float)c1 * surface_area(b1);
                float sc = 0.125f;
                float tsa = surface_area(bbox);
                costs[i] = sc * (b0sa + b1sa) / tsa;
            }
            size_t min_split = 0;
            float min_cost = FLT_MAX;
            for (size_t i = 0; i < NUM_BUCKETS - 1; ++i)
                if (costs[i] < min_cost) {
                    min_split = i;
                    min_cost = costs[i];
                }
            if (B.mp < num_prims || f2usize(min_cost) < num_prims) {
                for (auto& p : prims) (bucket_for(p) <= min_split ? p1 : p2).push_back(p);
            } else {
                return make_leaf(B, bbox, prims);
            }
        }
    }
    if (p1.empty() || p2.empty()) {  // bvh.rs:237-238 assert!
        B.failed = true;
        B.err = "BVH build: empty partition (reference asserts at bvh.rs:237-238)";
        return make_leaf(B, bbox, prims);
    }
    prims.clear();
    prims.shrink_to_fit();
    int left = recursive_build(B, std::move(p1));
    int right = recursive_build(B, std::move(p2));
    BuildNode n{};
    n.leaf = false;
    n.bounds = union_box(B.nodes[left].bounds, B.nodes[right].bounds);
    n.c1 = left;
    n.c2 = right;
    n.axis = dim;
    n.num_nodes = B.nodes[left].num_nodes + B.nodes[right].num_nodes + 1;
    B.nodes.push_back(n);
    return (int)B.nodes.size() - 1;
}

struct Packed {  // PackedBVHNode, bvh.rs:260-272
    BBox bounds;
    bool leaf;
    uint32_t offset;  // leaf prim_offset or inner second_child_offset
    uint32_t count;   // leaf num_prims or inner axis
};

// bvh.rs:282-325 (iterative to bound the host stack; same pre-order)
void linearize(const Builder& B, int root, std::vector<Packed>& out) {
    struct Item {
        int node;
        int parent_slot;  // slot whose offset gets patched, or -1
    };
    std::vector<Item> stack;
    stack.push_back({root, -1});
    while (!stack.empty()) {
        Item it = stack.back();
        stack.pop_back();
        const BuildNode& n = B.nodes[it.node];
        uint32_t slot = (uint32_t)out.size();
        if (it.parent_slot >= 0) out[it.parent_slot].offset = slot;
        Packed p;
        p.bounds = n.bounds;
        p.leaf = n.leaf;
        if (n.leaf) {
            p.offset = n.first;
            p.count = n.count;
            out.push_back(p);
        } else {
            p.offset = 0;
            p.count = (uint32_t)n.axis;
            out.push_back(p);
            stack.push_back({n.c2, (int)slot});  // second child follows child1's subtree
            stack.push_back({n.c1, -1});
        }
    }
}

uint32_t tree_depth(const std::vector<Packed>& nodes) {
    if (nodes.empty()) return 0;
    std::vector<std::pair<uint32_t, uint32_t>> st;
    st.push_back({0, 1});
    uint32_t best = 0;
    while (!st.empty()) {
        auto [n, d] = st.back();
        st.pop_back();
        best = std::max(best, d);
        if (!nodes[n].leaf) {
            st.push_back({n + 1, d + 1});
            st.push_back({nodes[n].offset, d + 1});
        }
    }
    return best;
}

}  // namespace

struct OracleBVH {
    Refined R;
    std::vector<Packed> nodes;
    std::vector<uint32_t> ordered;
    uint32_t depth = 0;
};

namespace {

BBox def_bound(const OracleBVH* o) { return o->nodes[0].bounds; }  // definitions are not empty
size_t def_size(const OracleBVH* o) { return o->R.prims.size(); }

SplitMethod parse_split(const char* sm) {
    if (!sm) return SPLIT_SAH;
    if (!strcmp(sm, "sah")) return SPLIT_SAH;
    if (!strcmp(sm, "middle")) return SPLIT_MIDDLE;
    if (!strcmp(sm, "equal")) return SPLIT_EQUAL;
    fprintf(stderr, "Warning: BVH split method %s unknown. Using \"SAH\"\n", sm);  // bvh.rs:345-348
    return SPLIT_SAH;
}

// bvh.rs:334-363
int build_bvh(OracleBVH* o, uint32_t mp, SplitMethod sm) {
    Builder B;
    B.mp = mp;
    B.sm = sm;
    if (!o->R.prims.empty()) {
        std::vector<PrimInfo> info;
        info.reserve(o->R.prims.size());
        for (uint32_t i = 0; i < o->R.prims.size(); ++i) {
            BBox b = prim_bound(o->R, o->R.prims[i]);
            V3 c = mul(add(b.pmin, b.pmax), 0.5f);  // bvh.rs:77
            info.push_back(PrimInfo{i, c, b});
        }
        int root = recursive_build(B, std::move(info));
        if (B.failed) {
            fprintf(stderr, "oracle: %s\n", B.err.c_str());
            return PBRT_ERR_BUILD;
        }
        linearize(B, root, o->nodes);
    }
    o->ordered = std::move(B.ordered);
    o->depth = tree_depth(o->nodes);
    return PBRT_OK;
}

// The aggregate of shapes with instance definitions: each definition
// refined and built like the scene (the instance aggregate of
// main.rs:745-753 with the scene's accelerator), then the shapes.
int build_aggregate(const PbrtShapeDesc* shapes, uint32_t n, const PbrtInstanceDesc* defs, uint32_t n_defs,
                    uint32_t mp, SplitMethod sm, OracleBVH* o) {
    for (uint32_t k = 0; k < n_defs; ++k) {
        auto d = std::make_shared<OracleBVH>();
        for (uint32_t i = 0; i < defs[k].n_shapes; ++i)
            if (defs[k].shapes[i].kind == PBRT_SHAPE_INSTANCE || defs[k].shapes[i].area_light >= 0) {
                fprintf(stderr, "oracle: instance definitions hold neither instances nor area lights\n");
                return PBRT_ERR_UNSUPPORTED;
            }
        if (!refine_shapes(defs[k].shapes, defs[k].n_shapes, &d->R)) {
            fprintf(stderr, "oracle: %s\n", d->R.err.c_str());
            return PBRT_ERR_INVALID_ARGUMENT;
        }
        if (d->R.prims.empty()) return PBRT_ERR_INVALID_ARGUMENT;
        int st = build_bvh(d.get(), mp, sm);
        if (st) return st;
        o->R.defs.push_back(d);
    }
    if (!refine_shapes(shapes, n, &o->R)) {
        fprintf(stderr, "oracle: %s\n", o->R.err.c_str());
        return PBRT_ERR_INVALID_ARGUMENT;
    }
    if (!o->R.insts.empty()) {
        uint64_t next = 0;
        for (const Prim& p : o->R.prims) {
            o->R.first_id.push_back((uint32_t)next);
            next += p.kind == KIND_INST ? def_size(o->R.defs[o->R.insts[p.sphere].def].get()) : 1u;
        }
        if (next > 0x7fffffffull) return PBRT_ERR_UNSUPPORTED;
    }
    return build_bvh(o, mp, sm);
}

struct Counters {
    uint64_t nodes = 0, tris = 0, spheres = 0;
};

bool bvh_intersect_at(const OracleBVH* o, Ray& ray, PbrtHit* hit, Counters& C, std::vector<uint32_t>& todo,
                      int32_t* inner, bool first_hit = false);

// One primitive's intersect (geometric.rs:62-73): on a hit, shrinks maxt.
// An instance (transformed.rs:35-56) traces the primitive-space ray
// w2p(ray) - o as a point, d as a vector, mint and the current maxt kept -
// through its definition's aggregate and, on a hit, takes its maxt; *inner
// gets the definition-local refined index.
bool prim_intersect(const Refined& R, const Prim& p, Ray& ray, float* t, float* b1, float* b2,
                    Counters& C, int32_t* inner) {
    *inner = 0;
    if (p.kind == KIND_INST) {
        const Inst& I = R.insts[p.sphere];
        Ray r = xf_ray(I.w2i, ray);
        thread_local std::vector<uint32_t> todo2;
        PbrtHit h;
        int32_t unused;
        if (!bvh_intersect_at(R.defs[I.def].get(), r, &h, C, todo2, &unused)) return false;
        *t = h.t;
        *b1 = h.b1;
        *b2 = h.b2;
        *inner = h.prim;
        ray.maxt = r.maxt;
        return true;
    }
    if (p.kind == KIND_TRI) {
        C.tris++;
        if (!tri_hit(p.tri, ray, t, b1, b2)) return false;
    } else {
        C.spheres++;
        const Sphere& s = R.spheres[p.sphere];
        Ray oray = xf_ray(s.w2o.m, ray);
        float phi;
        if (!quad_hit_obj(s, oray, t, &phi)) return false;
        *b1 = 0.0f;
        *b2 = 0.0f;
    }
    ray.maxt = *t;
    return true;
}

// bvh.rs:375-422.  BVH intersect_p is the default intersect().is_some()
// (intersection.rs:61-66), so both use this full closest-hit search.
// *compact gets the hit's refined index in this aggregate (hit->prim is
// its id: with instances, the first id of the instance + the inner index).
// first_hit: stop at the first accepted primitive (the early exit an
// any-hit walk may take, D11: the answer is the same, the work is less);
// used only to count that work.
bool bvh_intersect_at(const OracleBVH* o, Ray& ray, PbrtHit* hit, Counters& C, std::vector<uint32_t>& todo,
                      int32_t* compact, bool first_hit) {
    *compact = -1;
    hit->prim = -1;
    hit->t = 0;
    hit->b1 = 0;
    hit->b2 = 0;
    if (o->nodes.empty()) return false;
    bool dir_is_neg[3];
    {
        V3 inv = mk(1.0f / ray.d.x, 1.0f / ray.d.y, 1.0f / ray.d.z);
        dir_is_neg[0] = inv.x < 0.0f;
        dir_is_neg[1] = inv.y < 0.0f;
        dir_is_neg[2] = inv.z < 0.0f;
    }
    todo.clear();
    todo.push_back(0);
    bool any = false;
    while (!todo.empty()) {
        uint32_t n = todo.back();
        todo.pop_back();
        const Packed& node = o->nodes[n];
        C.nodes++;
        if (!bbox_intersect(node.bounds, ray, nullptr, nullptr)) continue;
        if (node.leaf) {
            for (uint32_t i = 0; i < node.count; ++i) {
                uint32_t pi = o->ordered[node.offset + i];
                float t, b1, b2;
                int32_t inner;
                if (prim_intersect(o->R, o->R.prims[pi], ray, &t, &b1, &b2, C, &inner)) {
                    *compact = (int32_t)pi;
                    hit->prim = (int32_t)((o->R.first_id.empty() ? pi : o->R.first_id[pi]) + (uint32_t)inner);
                    hit->t = t;
                    hit->b1 = b1;
                    hit->b2 = b2;
                    any = true;
                    if (first_hit) return true;
                }
            }
        } else {
            if (dir_is_neg[node.count]) {
                todo.push_back(n + 1);
                todo.push_back(node.offset);
            } else {
                todo.push_back(node.offset);
                todo.push_back(n + 1);
            }
        }
    }
    return any;
}

bool bvh_intersect(const OracleBVH* o, Ray& ray, PbrtHit* hit, Counters& C, std::vector<uint32_t>& todo) {
    int32_t compact;
    return bvh_intersect_at(o, ray, hit, C, todo, &compact);
}

Ray to_ray(const PbrtRay& r) {
    Ray x;
    x.o = mk(r.ox, r.oy, r.oz);
    x.d = mk(r.dx, r.dy, r.dz);
    x.mint = r.tmin;
    x.maxt = r.tmax;
    return x;
}

template <class F>
void parallel_for(uint32_t n, int nthreads, F f) {
    if (nthreads <= 1 || n < 1024) {
        f(0u, n, 0);
        return;
    }
    std::vector<std::thread> th;
    uint32_t chunk = (n + nthreads - 1) / nthreads;
    for (int t = 0; t < nthreads; ++t) {
        uint32_t lo = t * chunk, hi = std::min(n, lo + chunk);
        if (lo >= hi) break;
        th.emplace_back([&, lo, hi, t]() { f(lo, hi, t); });
    }
    for (auto& x : th) x.join();
}

// --------------------------------------------------------------- render ---
// src/filter.rs:87-124
struct Filter {
    int kind;
    float xw, yw, inv_xw, inv_yw, p0, p1, exp_x, exp_y;
};
Filter filter_new(int kind, float xw, float yw, float p0, float p1) {
    Filter f{kind, xw, yw, 1.0f / xw, 1.0f / yw, p0, p1, 0.0f, 0.0f};
    if (kind == 2) {
        f.exp_x = expf(-p0 * xw * xw);
        f.exp_y = expf(-p0 * yw * yw);
    }
    return f;
}
float sinc_1d(float x, float tau) {  // utils/mod.rs:207-217
    float v = fabsf(x);
    if (v < 1e-5f) return 1.0f;
    if (v >= 1.0f) return 0.0f;
    v *= kPi;
    float vtau = v * tau;
    float s = sinf(vtau) / vtau;
    return s * sinf(v) / v;
}
float filter_eval(const Filter& f, float x, float y) {
    switch (f.kind) {
        case 0:
            return 1.0f;
        case 1: {
            float dx = (f.xw - fabsf(x)) * f.inv_xw;
            float dy = (f.yw - fabsf(y)) * f.inv_yw;
            return fmaxf(dx, 0.0f) * fmaxf(dy, 0.0f);
        }
        case 2: {
            auto g = [&](float v, float ex) { return fmaxf(expf(-f.p0 * v * v) - ex, 0.0f); };
            return g(x, f.exp_x) * g(y, f.exp_y);
        }
        case 3: {
            float b = f.p0, c = f.p1;
            auto mitchell = [&](float v) {
                float t = fabsf(v * 2.0f);
                float r;
                if (t >= 2.0f)
                    r = 0.0f;
                else if (t > 1.0f)
                    r = (-b - 6.0f * c) * t * t * t + (6.0f * b + 30.0f * c) * t * t +
                        (-12.0f * b - 48.0f * c) * t + (8.0f * b + 24.0f * c);
                else
                    r = (12.0f - 9.0f * b - 6.0f * c) * t * t * t + (-18.0f + 12.0f * b + 6.0f * c) * t * t +
                        (6.0f - 2.0f * b);
                return (1.0f / 6.0f) * r;
            };
            return mitchell(x * f.inv_xw) * mitchell(y * f.inv_yw);
        }
        default:
            return sinc_1d(x * f.inv_xw, f.p0) * sinc_1d(y * f.inv_yw, f.p0);
    }
}

const int FT_DIM = 16;
struct Pixel {
    float xyz[3] = {0, 0, 0};
    float splat[3] = {0, 0, 0};
    float wsum = 0;
};
// src/camera/film.rs
struct Film {
    uint32_t xres, yres;
    float crop[4];
    Filter filter;
    int32_t x_start, y_start, x_count, y_count;
    float table[FT_DIM * FT_DIM];
    std::vector<Pixel> pixels;
};
// film.rs:77-122
Film film_image(uint32_t xres, uint32_t yres, const Filter& f, const float crop[4], bool alloc = true) {
    Film F;
    F.xres = xres;
    F.yres = yres;
    memcpy(F.crop, crop, sizeof(F.crop));
    F.filter = f;
    F.x_start = f2i32(ceilf((float)xres * crop[0]));
    F.x_count = std::max(f2i32(ceilf((float)xres * crop[1])) - F.x_start, 1);
    F.y_start = f2i32(ceilf((float)yres * crop[2]));
    F.y_count = std::max(f2i32(ceilf((float)yres * crop[3])) - F.y_start, 1);
    for (int y = 0; y < FT_DIM; ++y) {
        float fy = ((float)y + 0.5f) * f.yw / (float)FT_DIM;
        for (int x = 0; x < FT_DIM; ++x) {
            float fx = ((float)x + 0.5f) * f.xw / (float)FT_DIM;
            F.table[y * FT_DIM + x] = filter_eval(f, fx, fy);
        }
    }
    if (alloc) F.pixels.resize((size_t)F.x_count * F.y_count);
    return F;
}
// film.rs:124-147
Film film_sub(const Film& F, size_t num, size_t count) {
    float aspect = (float)F.xres / (float)F.yres;
    float w[4];
    crop_window(num, count, aspect, w);
    float dx = F.crop[1] - F.crop[0], dy = F.crop[3] - F.crop[2];
    float cw[4] = {F.crop[0] + w[0] * dx, F.crop[0] + w[1] * dx, F.crop[2] + w[2] * dy, F.crop[2] + w[3] * dy};
    return film_image(F.xres, F.yres, F.filter, cw);
}
// spectrum.rs:31-41
void xyz_to_rgb(const float x[3], float r[3]) {
    r[0] = 3.240479f * x[0] - 1.37150f * x[1] - 0.498535f * x[2];
    r[1] = -0.969256f * x[0] + 1.875991f * x[1] + 0.041556f * x[2];
    r[2] = 0.055648f * x[0] - 0.204043f * x[1] + 1.057311f * x[2];
}
void rgb_to_xyz(const float r[3], float x[3]) {
    x[0] = 0.412453f * r[0] + 0.357580f * r[1] + 0.180423f * r[2];
    x[1] = 0.212671f * r[0] + 0.715160f * r[1] + 0.072169f * r[2];
    x[2] = 0.019334f * r[0] + 0.119193f * r[1] + 0.950227f * r[2];
}
// film.rs:192-249
void film_add_sample(Film& F, float image_x, float image_y, const float L[3]) {
    float dix = image_x - 0.5f, diy = image_y - 0.5f;
    int32_t x0 = std::max(F.x_start, f2i32(ceilf(dix - F.filter.xw)));
    int32_t x1 = std::min(F.x_start + F.x_count - 1, f2i32(floorf(dix + F.filter.xw)));
    int32_t y0 = std::max(F.y_start, f2i32(ceilf(diy - F.filter.yw)));
    int32_t y1 = std::min(F.y_start + F.y_count - 1, f2i32(floorf(diy + F.filter.yw)));
    if ((x1 - x0) < 0 || (y1 - y0) < 0) return;
    float xyz[3];
    rgb_to_xyz(L, xyz);
    for (int32_t y = y0; y <= y1; ++y) {
        float fy = ((float)y - diy) * F.filter.inv_yw * (float)FT_DIM;
        size_t iy = std::min(f2usize(floorf(fabsf(fy))), (size_t)FT_DIM - 1);
        for (int32_t x = x0; x <= x1; ++x) {
            float fx = ((float)x - dix) * F.filter.inv_xw * (float)FT_DIM;
            size_t ix = std::min(f2usize(floorf(fabsf(fx))), (size_t)FT_DIM - 1);
            float w = F.table[iy * FT_DIM + ix];
            Pixel& p = F.pixels[(size_t)(y - F.y_start) * F.x_count + (size_t)(x - F.x_start)];
            p.xyz[0] += w * xyz[0];
            p.xyz[1] += w * xyz[1];
            p.xyz[2] += w * xyz[2];
            p.wsum += w;
        }
    }
}
// film.rs:149-186
void film_add_sub(Film& F, const Film& S, float* rgb_out_unused) {
    (void)rgb_out_unused;
    for (int32_t y = S.y_start; y < S.y_start + S.y_count; ++y)
        for (int32_t x = S.x_start; x < S.x_start + S.x_count; ++x) {
            if (x < F.x_start || y < F.y_start || x >= F.x_start + F.x_count || y >= F.y_start + F.y_count)
                continue;
            F.pixels[(size_t)(y - F.y_start) * F.x_count + (x - F.x_start)] =
                S.pixels[(size_t)(y - S.y_start) * S.x_count + (x - S.x_start)];
        }
}
// film.rs:316-354 with D8: rgb = max(0, xyz_to_rgb(xyz) / w) + splat term
void film_write(const Film& F, float* rgb, float splat_scale) {
    for (int32_t y = 0; y < F.y_count; ++y)
        for (int32_t x = 0; x < F.x_count; ++x) {
            const Pixel& p = F.pixels[(size_t)y * F.x_count + x];
            float c[3];
            xyz_to_rgb(p.xyz, c);
            if (p.wsum != 0.0f) {
                float inv = 1.0f / p.wsum;
                c[0] = fmaxf(c[0] * inv, 0.0f);
                c[1] = fmaxf(c[1] * inv, 0.0f);
                c[2] = fmaxf(c[2] * inv, 0.0f);
            }
            float s[3];
            xyz_to_rgb(p.splat, s);
            float* o = rgb + 3 * ((size_t)y * F.x_count + x);
            o[0] = c[0] + s[0] * splat_scale;
            o[1] = c[1] + s[1] * splat_scale;
            o[2] = c[2] + s[2] * splat_scale;
        }
}

// Camera::perspective (camera/mod.rs:105-135) + Projection::new
// (camera/projective.rs:48-72)
struct Camera {
    Xf c2w;
    Xf r2c;
    float lens_radius, focal_distance, sopen, sclose;
};
Xf perspective_xf(float fov) {
    float znear = 1e-2f, zfar = 1000.0f;
    M4 pm = m4_identity();
    pm.m[2][2] = zfar / (zfar - znear);
    pm.m[2][3] = -(zfar * znear) / (zfar - znear);
    pm.m[3][2] = 1.0f;
    pm.m[3][3] = 0.0f;
    Xf p = xf_from(pm);
    float inv_tan_ang = 1.0f / tanf(as_radians(fov) / 2.0f);
    return xf_mul(xf_scale(inv_tan_ang, inv_tan_ang, 1.0f), p);
}
void projection(uint32_t xres, uint32_t yres, const Xf& cam_to_screen, const float sw[4], Xf out[4]) {
    Xf s2r = xf_mul(xf_mul(xf_scale((float)xres, (float)yres, 1.0f),
                           xf_scale(1.0f / (sw[1] - sw[0]), 1.0f / (sw[2] - sw[3]), 1.0f)),
                    xf_translate(mk(-sw[0], -sw[3], 0.0f)));
    Xf r2s = xf_inverse(s2r);
    Xf r2c = xf_mul(xf_inverse(cam_to_screen), r2s);
    out[0] = cam_to_screen;
    out[1] = r2s;
    out[2] = s2r;
    out[3] = r2c;
}
Camera camera_new(const PbrtCameraDesc& d) {
    Camera c;
    c.c2w = xf_from_desc(d.camera_to_world);
    Xf out[4];
    projection(d.x_res, d.y_res, perspective_xf(d.fov_deg), d.screen_window, out);
    c.r2c = out[3];
    c.lens_radius = d.lens_radius;
    c.focal_distance = d.focal_distance;
    c.sopen = d.shutter_open;
    c.sclose = d.shutter_close;
    return c;
}
// camera/mod.rs:168-195, 212-271 (main ray; differentials unused, D9),
// projective.rs:79-96 (concentric_sample_disk is the identity stub there)
Ray camera_ray(const Camera& c, float ix, float iy, float lu, float lv) {
    V3 pc = xf_point(c.r2c.m, mk(ix, iy, 0.0f));
    Ray r;
    r.o = mk(0, 0, 0);
    r.d = normalize(pc);
    r.mint = 0.0f;
    r.maxt = FLT_MAX;
    if (c.lens_radius > 0.0f) {
        float u = lu * c.lens_radius, v = lv * c.lens_radius;
        float ft = c.focal_distance / r.d.z;
        V3 pf = point_at(r, ft);
        r.o = mk(u, v, 0.0f);
        r.d = normalize(sub(pf, r.o));
    }
    Ray w = r;
    w.o = xf_point(c.c2w.m, r.o);
    w.d = xf_vector(c.c2w.m, r.d);
    return w;
}

struct AreaLight {
    std::vector<Tri> tris;
    std::vector<float> cdf;  // running area / total, cdf[0] = 0
    float area = 0;
    float L[3];
};
struct Light {
    int kind;
    V3 pos;
    float I[3];
    int area;  // index into area lights
};
// MatteMaterial::get_bsdf (matte.rs:30-51): Kd clamped to [0, f32::MAX],
// sigma to [0, 90]; sigma == 0 -> Lambertian, else OrenNayar::new
// (orennayar.rs:15-28) with its A and B.
struct Matte {
    float kd[3];
    bool oren;
    float a, b;
};
Matte matte_new(const PbrtMaterialDesc& m) {
    Matte r;
    for (int c = 0; c < 3; ++c) r.kd[c] = clampf(m.kd[c], 0.0f, FLT_MAX);
    const float sig = clampf(m.sigma, 0.0f, 90.0f);
    r.oren = !(sig == 0.0f);
    const float sigma = sig * kPi / 180.0f;  // utils/mod.rs:37-39
    const float sigma2 = sigma * sigma;
    r.a = 1.0f - (sigma2 / (2.0f * (sigma + 0.33f)));
    r.b = 0.45f * sigma2 / (sigma2 + 0.09f);
    return r;
}

struct SceneData {
    OracleBVH bvh;
    std::vector<Matte> materials;
    std::vector<Light> lights;
    std::vector<AreaLight> areas;
};

int scene_build(const PbrtSceneDesc* d, SceneData* S) {
    SplitMethod sm = (SplitMethod)d->split_method;
    int st = build_aggregate(d->shapes, d->n_shapes, d->instances, d->n_instances, d->max_prims_in_node, sm, &S->bvh);
    if (st) return st;
    for (uint32_t i = 0; i < d->n_materials; ++i) S->materials.push_back(matte_new(d->materials[i]));
    for (uint32_t i = 0; i < d->n_lights; ++i) {
        const PbrtLightDesc& L = d->lights[i];
        Light l{};
        l.kind = L.kind;
        memcpy(l.I, L.spectrum, sizeof(l.I));
        l.area = -1;
        if (L.kind == PBRT_LIGHT_POINT) {
            l.pos = xf_point(xf_from_desc(L.light_to_world).m, mk(0, 0, 0));  // point.rs:79-82
        } else {
            AreaLight a;
            memcpy(a.L, L.spectrum, sizeof(a.L));
            for (auto& p : S->bvh.R.prims)
                if (p.kind == KIND_TRI && p.shape == L.shape) a.tris.push_back(p.tri);
            a.cdf.push_back(0.0f);
            float acc = 0.0f;
            for (auto& t : a.tris) {
                acc += tri_area(t);
                a.cdf.push_back(acc);
            }
            a.area = acc;
            for (auto& c : a.cdf) c = c / acc;
            l.area = (int)S->areas.size();
            S->areas.push_back(a);
        }
        S->lights.push_back(l);
    }
    return PBRT_OK;
}

// Surface hit record used by shading.
struct SurfHit {
    V3 p, nn, dpdu;
    float eps;
    int prim;
    int material, area_light;
};

// dg.p, dg.nn and dg.dpdu (world space) of refined primitive p (a triangle
// or a quadric of R) hit by ray r at t.
void surface_dg(const Refined& R, const Prim& p, const Ray& r, float t, V3* pos, V3* nn, V3* dpdu) {
    if (p.kind == KIND_TRI) {
        tri_dg(p.tri, r, t, pos, nn, dpdu);
        return;
    }
    const Sphere& s = R.spheres[p.sphere];
    Ray orr = xf_ray(s.w2o.m, r);
    float th, phi;
    quad_hit_obj(s, orr, &th, &phi);  // recompute phi for u (same t)
    if (s.kind == QUAD_SPHERE)
        sphere_dg(s, orr, t, phi, pos, nn, dpdu, nullptr, nullptr, nullptr, nullptr);
    else
        quad_dg(s, orr, t, phi, pos, nn, nullptr, nullptr, dpdu, nullptr);
}

bool scene_intersect(const SceneData& S, const Ray& r_in, SurfHit* sh, Counters& C, std::vector<uint32_t>& todo) {
    Ray r = r_in;
    PbrtHit h;
    int32_t compact;
    if (!bvh_intersect_at(&S.bvh, r, &h, C, todo, &compact)) return false;
    const Refined& R = S.bvh.R;
    const Prim& p = R.prims[compact];
    sh->prim = h.prim;
    sh->eps = h.t * 5e-4f;  // mesh.rs:262, sphere.rs:174
    if (p.kind == KIND_INST) {
        // transformed.rs:37-51: the definition's primitive on the
        // primitive-space ray, then p by primitive-to-world and nn by its
        // normal transform, normalised
        const Inst& I = R.insts[p.sphere];
        const Refined& D = R.defs[I.def]->R;
        const Prim& q = D.prims[(uint32_t)h.prim - R.first_id[compact]];
        V3 pos, nn, dpdu;
        surface_dg(D, q, xf_ray(I.w2i, r_in), h.t, &pos, &nn, &dpdu);
        sh->p = xf_point(I.i2w, pos);
        sh->nn = normalize(xf_normal(I.w2i, nn));
        sh->dpdu = xf_vector(I.i2w, dpdu);
        sh->material = q.material;
        sh->area_light = -1;
    } else {
        surface_dg(R, p, r_in, h.t, &sh->p, &sh->nn, &sh->dpdu);
        sh->material = p.material;
        sh->area_light = p.area_light;
    }
    return true;
}

bool scene_occluded(const SceneData& S, const Ray& r_in, Counters& C, std::vector<uint32_t>& todo) {
    Ray r = r_in;
    PbrtHit h;
    return bvh_intersect(&S.bvh, r, &h, C, todo);
}

// visibility_tester.rs:16-24
Ray segment(V3 p1, float eps1, V3 p2, float eps2) {
    float dist = length(sub(p1, p2));
    V3 dir = vdiv(sub(p2, p1), dist);
    Ray r;
    r.o = p1;
    r.d = dir;
    r.mint = eps1;
    r.maxt = (1.0f - eps2) * dist;
    return r;
}

struct LightSample {
    float comp, u0, u1;
};

// Light::sample_l: point.rs:28-35 with D6 (normalised wi); the diffuse area
// light follows pbrt-v2 (D5): pick a triangle by area with the component
// sample, uniform point b1 = 1 - sqrt(u0), b2 = u1 * sqrt(u0),
// ns = normalize(cross(p2 - p1, p3 - p1)) (flipped with the shape),
// pdf = d^2 / (|ns . -wi| * area), L one-sided, shadow segment eps2 = 1e-3.
bool sample_light(const SceneData& S, const Light& l, V3 p, float eps, const LightSample& ls, float Li[3], V3* wi,
                  float* pdf, Ray* vis) {
    if (l.kind == PBRT_LIGHT_POINT) {
        V3 w = sub(l.pos, p);
        float d2 = length_sq(w);
        Li[0] = l.I[0] / d2;
        Li[1] = l.I[1] / d2;
        Li[2] = l.I[2] / d2;
        *wi = normalize(w);
        *pdf = 1.0f;
        *vis = segment(p, eps, l.pos, 0.0f);
        return true;
    }
    const AreaLight& a = S.areas[l.area];
    size_t n = a.tris.size();
    size_t k = 0;
    while (k + 1 < n && !(ls.comp < a.cdf[k + 1])) ++k;
    const Tri& t = a.tris[k];
    float su1 = sqrtf(ls.u0);
    float b1 = 1.0f - su1;
    float b2 = ls.u1 * su1;
    V3 ps = add(add(mul(t.p1, b1), mul(t.p2, b2)), mul(t.p3, (1.0f - b1) - b2));
    V3 ns = normalize(cross(sub(t.p2, t.p1), sub(t.p3, t.p1)));
    if (t.flip) ns = mul(ns, -1.0f);
    V3 w = normalize(sub(ps, p));
    float d2 = length_sq(sub(p, ps));
    V3 mw = neg(w);
    float c = dot(ns, mw);
    float ac = fabsf(c);
    *wi = w;
    *pdf = (ac == 0.0f) ? 0.0f : d2 / (ac * a.area);
    bool lit = c > 0.0f;
    Li[0] = lit ? a.L[0] : 0.0f;
    Li[1] = lit ? a.L[1] : 0.0f;
    Li[2] = lit ? a.L[2] : 0.0f;
    *vis = segment(p, eps, ps, 1e-3f);
    return true;
}

// OrenNayar::f (orennayar.rs:31-62) without the reflectance: a + b *
// maxcos * sin(alpha) * tan(beta), with bsdf/utils.rs:5-28.
inline float sin_theta_l(V3 v) { return sqrtf(fmaxf(0.0f, 1.0f - v.z * v.z)); }
inline float clamp_unit(float x) { return x < -1.0f ? -1.0f : (x > 1.0f ? 1.0f : x); }
inline float cos_phi_l(V3 v) {
    const float st = sin_theta_l(v);
    return st == 0.0f ? 1.0f : clamp_unit(v.x / st);
}
inline float sin_phi_l(V3 v) {
    const float st = sin_theta_l(v);
    return st == 0.0f ? 0.0f : clamp_unit(v.y / st);
}
float oren_nayar_term(float a, float b, V3 wo, V3 wi) {
    const float sinthetai = sin_theta_l(wi), sinthetao = sin_theta_l(wo);
    float maxcos = 0.0f;
    if (!(sinthetai < 1e-4f || sinthetao < 1e-4f))
        maxcos = fmaxf(cos_phi_l(wi) * cos_phi_l(wo) + sin_phi_l(wi) * sin_phi_l(wo), 0.0f);
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

// WhittedIntegrator::li light loop (integrator/whitted.rs:30-65) as the
// direct-lighting Li (D1), with Lambertian f = Kd/pi when wi, wo lie on the
// same side of ng (bsdf/mod.rs:132-149, D7), no media (D2).
// C counts the camera ray's traversal work, Cs the shadow rays'.
void li_direct(const SceneData& S, const Ray& ray, const float* light_samples, float L[3], Counters& C,
               Counters& Cs, std::vector<uint32_t>& todo, uint64_t* n_shadow) {
    L[0] = L[1] = L[2] = 0.0f;
    SurfHit h;
    if (!scene_intersect(S, ray, &h, C, todo)) return;  // miss: sum of le() is 0
    V3 wo = neg(ray.d);
    // Le at an emitter (pbrt-v2 Intersection::Le; intersection.rs:58 is 0)
    if (h.area_light >= 0 && h.area_light < (int)S.lights.size()) {
        const Light& al = S.lights[h.area_light];
        if (al.kind == PBRT_LIGHT_DIFFUSE_AREA && dot(h.nn, wo) > 0.0f) {
            const AreaLight& a = S.areas[al.area];
            L[0] = a.L[0];
            L[1] = a.L[1];
            L[2] = a.L[2];
        }
    }
    const Matte& m = S.materials[h.material];
    const float* kd = m.kd;
    float invpi = 1.0f / kPi;  // lambertian.rs:21
    // BSDF frame (bsdf/mod.rs:70-86): tn = normalize(dpdu), sn = nn x tn,
    // world_to_local(v) = (v.sn, v.tn, v.nn)
    V3 tn = normalize(h.dpdu), sn = cross(h.nn, tn);
    V3 wo_l = mk(dot(wo, sn), dot(wo, tn), dot(wo, h.nn));
    size_t nl = S.lights.size();
    for (size_t li = 0; li < nl; ++li) {
        LightSample ls{light_samples[li], light_samples[nl + 2 * li], light_samples[nl + 2 * li + 1]};
        float Li[3], pdf;
        V3 wi;
        Ray vis;
        sample_light(S, S.lights[li], h.p, h.eps, ls, Li, &wi, &pdf, &vis);
        bool black = Li[0] == 0.0f && Li[1] == 0.0f && Li[2] == 0.0f;
        if (black || pdf == 0.0f) continue;
        bool refl = dot(wi, h.nn) * dot(wo, h.nn) > 0.0f;
        float f[3] = {0, 0, 0};
        if (refl && !m.oren) {
            f[0] = kd[0] * invpi;
            f[1] = kd[1] * invpi;
            f[2] = kd[2] * invpi;
        } else if (refl) {
            const float g = oren_nayar_term(m.a, m.b, wo_l, mk(dot(wi, sn), dot(wi, tn), dot(wi, h.nn)));
            f[0] = kd[0] * invpi * g;
            f[1] = kd[1] * invpi * g;
            f[2] = kd[2] * invpi * g;
        }
        if (f[0] == 0.0f && f[1] == 0.0f && f[2] == 0.0f) continue;
        if (n_shadow) (*n_shadow)++;
        if (scene_occluded(S, vis, Cs, todo)) continue;
        float ad = fabsf(dot(wi, h.nn));
        for (int c = 0; c < 3; ++c) L[c] = L[c] + ((f[c] * Li[c]) * ad) / pdf;
    }
}

// Number of integrator-array floats per sample: per light one 1-D
// component sample and one 2-D position sample (D17).
size_t integrator_floats(size_t nlights) { return 3 * nlights; }

// StratifiedSampler::get_more_samples (sampler/stratified.rs:60-127) for
// pixel (x, y): fills per-sample camera samples and integrator arrays.
// cs: n*5 floats (image_x, image_y, lens_u, lens_v, time);
// arr: n * 3*nlights floats: 1-D arrays then 2-D arrays.
void pixel_samples(RNG& rng, int32_t x, int32_t y, size_t xs, size_t ys, bool jitter, float sopen, float sclose,
                   size_t nlights, std::vector<float>& buf, float* cs, float* arr) {
    size_t n = xs * ys;
    buf.resize(5 * n);
    float* image = buf.data();
    float* lens = image + 2 * n;
    float* time = lens + 2 * n;
    stratified_2d(image, xs, ys, rng, jitter);
    stratified_2d(lens, xs, ys, rng, jitter);
    stratified_1d(time, n, rng, jitter);
    for (size_t i = 0; i < n; ++i) {
        image[2 * i] += (float)x;
        image[2 * i + 1] += (float)y;
    }
    rng.shuffle(lens, 2 * n, 2);
    rng.shuffle(time, n, 1);
    size_t na = integrator_floats(nlights);
    for (size_t i = 0; i < n; ++i) {
        float t = lerpf(sopen, sclose, time[i]);
        float* c = cs + 5 * i;
        c[0] = image[2 * i];
        c[1] = image[2 * i + 1];
        c[2] = lens[2 * i];
        c[3] = lens[2 * i + 1];
        c[4] = t;
        float* a = arr + na * i;
        for (size_t l = 0; l < nlights; ++l) latin_hypercube(a + l, 1, 1, rng);
        for (size_t l = 0; l < nlights; ++l) latin_hypercube(a + nlights + 2 * l, 1, 2, rng);
    }
}

struct RenderCtx {
    const SceneData* S;
    Camera cam;
    Film film;
    PbrtSamplerDesc sd;
};

// run_task (sampler_renderer.rs:61-144) for one task, with D10 (explicit
// task count), D16 (sampler over the given pixel range) and the intended
// loop bounds (the sampler's own termination, a per-batch radiance list).
void run_task(RenderCtx& R, uint32_t task, std::vector<float>* dump, uint64_t* stats) {
    int32_t w[4];
    sub_window(R.sd.x_start, R.sd.x_end, R.sd.y_start, R.sd.y_end, task, R.sd.num_tasks, w);
    if (w[0] == w[1] || w[2] == w[3]) return;
    Film tf = film_sub(R.film, task, R.sd.num_tasks);
    RNG rng(task);
    size_t xs = R.sd.x_samples, ys = R.sd.y_samples, n = xs * ys;
    size_t nl = R.S->lights.size(), na = integrator_floats(nl);
    std::vector<float> buf, cs(5 * n), arr(na * n + 1);
    std::vector<uint32_t> todo;
    Counters C, Cs;
    uint64_t ncam = 0, nshadow = 0;
    for (int32_t y = w[2]; y < w[3]; ++y)
        for (int32_t x = w[0]; x < w[1]; ++x) {
            pixel_samples(rng, x, y, xs, ys, R.sd.jitter != 0, R.sd.shutter_open, R.sd.shutter_close, nl, buf,
                          cs.data(), arr.data());
            for (size_t i = 0; i < n; ++i) {
                const float* c = &cs[5 * i];
                Ray ray = camera_ray(R.cam, c[0], c[1], c[2], c[3]);
                float L[3];
                li_direct(*R.S, ray, &arr[na * i], L, C, Cs, todo, &nshadow);
                ncam++;
                if (dump) {
                    for (int k = 0; k < 5; ++k) dump->push_back(c[k]);
                    for (size_t k = 0; k < na; ++k) dump->push_back(arr[na * i + k]);
                    dump->push_back(ray.o.x);
                    dump->push_back(ray.o.y);
                    dump->push_back(ray.o.z);
                    dump->push_back(ray.d.x);
                    dump->push_back(ray.d.y);
                    dump->push_back(ray.d.z);
                    for (int k = 0; k < 3; ++k) dump->push_back(L[k]);
                }
                film_add_sample(tf, c[0], c[1], L);
            }
        }
    if (!dump) film_add_sub(R.film, tf, nullptr);
    if (stats) {
        __atomic_fetch_add(&stats[0], ncam, __ATOMIC_RELAXED);
        __atomic_fetch_add(&stats[1], nshadow, __ATOMIC_RELAXED);
        __atomic_fetch_add(&stats[2], C.nodes, __ATOMIC_RELAXED);
        __atomic_fetch_add(&stats[3], C.tris, __ATOMIC_RELAXED);
        __atomic_fetch_add(&stats[4], C.spheres, __ATOMIC_RELAXED);
        __atomic_fetch_add(&stats[5], Cs.nodes, __ATOMIC_RELAXED);
        __atomic_fetch_add(&stats[6], Cs.tris, __ATOMIC_RELAXED);
        __atomic_fetch_add(&stats[7], Cs.spheres, __ATOMIC_RELAXED);
    }
}

Filter camera_filter(const PbrtCameraDesc& c) {
    return filter_new(c.filter_kind, c.filter_x_width, c.filter_y_width, c.filter_p0, c.filter_p1);
}

}  // namespace

// ================================================================ C API ===
extern "C" {

int oracle_bvh_create(const PbrtShapeDesc* shapes, uint32_t n_shapes, uint32_t mp, const char* sm, OracleBVH** out) {
    if (!out || (!shapes && n_shapes)) return PBRT_ERR_INVALID_ARGUMENT;
    OracleBVH* o = new OracleBVH();
    int st = build_aggregate(shapes, n_shapes, nullptr, 0, mp, parse_split(sm), o);
    if (st) {
        delete o;
        return st;
    }
    *out = o;
    return PBRT_OK;
}
int oracle_bvh_create_desc(const PbrtSceneDesc* d, OracleBVH** out) {
    if (!out || !d || (!d->shapes && d->n_shapes) || (!d->instances && d->n_instances))
        return PBRT_ERR_INVALID_ARGUMENT;
    OracleBVH* o = new OracleBVH();
    int st = build_aggregate(d->shapes, d->n_shapes, d->instances, d->n_instances, d->max_prims_in_node,
                             (SplitMethod)d->split_method, o);
    if (st) {
        delete o;
        return st;
    }
    *out = o;
    return PBRT_OK;
}
void oracle_bvh_destroy(OracleBVH* o) { delete o; }
int oracle_bvh_num_nodes(const OracleBVH* o, uint32_t* n) {
    *n = (uint32_t)o->nodes.size();
    return 0;
}
int oracle_bvh_num_primitives(const OracleBVH* o, uint32_t* n) {
    *n = (uint32_t)o->R.prims.size();
    return 0;
}
int oracle_bvh_depth(const OracleBVH* o, uint32_t* d) {
    *d = o->depth;
    return 0;
}
int oracle_bvh_get_nodes(const OracleBVH* o, PbrtPackedNode* out, uint32_t cap) {
    if (cap < o->nodes.size()) return PBRT_ERR_INVALID_ARGUMENT;
    for (size_t i = 0; i < o->nodes.size(); ++i) {
        const Packed& p = o->nodes[i];
        PbrtPackedNode& q = out[i];
        q.lo[0] = p.bounds.pmin.x;
        q.lo[1] = p.bounds.pmin.y;
        q.lo[2] = p.bounds.pmin.z;
        q.hi[0] = p.bounds.pmax.x;
        q.hi[1] = p.bounds.pmax.y;
        q.hi[2] = p.bounds.pmax.z;
        q.is_leaf = p.leaf ? 1 : 0;
        q.offset = p.offset;
        q.count = p.count;
    }
    return 0;
}
int oracle_bvh_get_primitive_order(const OracleBVH* o, uint32_t* out, uint32_t cap) {
    if (cap < o->ordered.size()) return PBRT_ERR_INVALID_ARGUMENT;
    memcpy(out, o->ordered.data(), o->ordered.size() * sizeof(uint32_t));
    return 0;
}
int oracle_bvh_world_bound(const OracleBVH* o, float lo[3], float hi[3]) {
    BBox b = o->nodes.empty() ? bbox_new() : o->nodes[0].bounds;  // bvh.rs:365-373
    lo[0] = b.pmin.x;
    lo[1] = b.pmin.y;
    lo[2] = b.pmin.z;
    hi[0] = b.pmax.x;
    hi[1] = b.pmax.y;
    hi[2] = b.pmax.z;
    return 0;
}
int oracle_bvh_triangle(const OracleBVH* o, uint32_t prim, float out[9]) {
    if (prim >= o->R.prims.size() || o->R.prims[prim].kind != KIND_TRI) return PBRT_ERR_INVALID_ARGUMENT;
    const Tri& t = o->R.prims[prim].tri;
    float v[9] = {t.p1.x, t.p1.y, t.p1.z, t.p2.x, t.p2.y, t.p2.z, t.p3.x, t.p3.y, t.p3.z};
    memcpy(out, v, sizeof(v));
    return 0;
}

static int intersect_impl(const OracleBVH* o, const PbrtRay* rays, uint32_t n, PbrtHit* hits, uint8_t* occ,
                          uint64_t* counters, int nthreads) {
    std::vector<Counters> cs(std::max(nthreads, 1));
    parallel_for(n, nthreads, [&](uint32_t lo, uint32_t hi, int t) {
        std::vector<uint32_t> todo;
        todo.reserve(128);
        Counters& C = cs[t];
        for (uint32_t i = lo; i < hi; ++i) {
            Ray r = to_ray(rays[i]);
            PbrtHit h;
            bool any = bvh_intersect(o, r, &h, C, todo);
            if (hits) hits[i] = h;
            if (occ) occ[i] = any ? 1 : 0;
        }
    });
    if (counters) {
        counters[0] = counters[1] = counters[2] = 0;
        for (auto& c : cs) {
            counters[0] += c.nodes;
            counters[1] += c.tris;
            counters[2] += c.spheres;
        }
    }
    return 0;
}
int oracle_count_first_hit(const OracleBVH* o, const PbrtRay* rays, uint32_t n, uint8_t* occ, uint64_t* counters,
                           int nthreads) {
    std::vector<Counters> cs(std::max(nthreads, 1));
    parallel_for(n, nthreads, [&](uint32_t lo, uint32_t hi, int t) {
        std::vector<uint32_t> todo;
        todo.reserve(128);
        for (uint32_t i = lo; i < hi; ++i) {
            Ray r = to_ray(rays[i]);
            PbrtHit h;
            int32_t compact;
            bool any = bvh_intersect_at(o, r, &h, cs[t], todo, &compact, true);
            if (occ) occ[i] = any ? 1 : 0;
        }
    });
    if (counters) {
        counters[0] = counters[1] = counters[2] = 0;
        for (auto& c : cs) {
            counters[0] += c.nodes;
            counters[1] += c.tris;
            counters[2] += c.spheres;
        }
    }
    return 0;
}
int oracle_intersect(const OracleBVH* o, const PbrtRay* rays, uint32_t n, PbrtHit* hits, uint64_t* counters,
                     int nthreads) {
    return intersect_impl(o, rays, n, hits, nullptr, counters, nthreads);
}
int oracle_intersect_p(const OracleBVH* o, const PbrtRay* rays, uint32_t n, uint8_t* occ, uint64_t* counters,
                       int nthreads) {
    return intersect_impl(o, rays, n, nullptr, occ, counters, nthreads);
}

struct OracleScene {
    SceneData S;
};

static int render_scene(const SceneData& S, const PbrtCameraDesc* camera, const PbrtSamplerDesc* sampler, float* rgb,
                        int nthreads, uint32_t task_lo, uint32_t task_hi, uint64_t* stats) {
    RenderCtx R;
    R.S = &S;
    R.cam = camera_new(*camera);
    R.film = film_image(camera->x_res, camera->y_res, camera_filter(*camera), camera->crop_window);
    R.sd = *sampler;
    if (stats)
        for (int k = 0; k < 8; ++k) stats[k] = 0;
    task_hi = std::min(task_hi, sampler->num_tasks);
    std::atomic<uint32_t> next(task_lo);
    auto worker = [&]() {
        for (;;) {
            uint32_t t = next.fetch_add(1);
            if (t >= task_hi) break;
            run_task(R, t, nullptr, stats);
        }
    };
    int nt = std::max(1, nthreads);
    std::vector<std::thread> th;
    for (int i = 1; i < nt; ++i) th.emplace_back(worker);
    worker();
    for (auto& t : th) t.join();
    film_write(R.film, rgb, 1.0f);
    return PBRT_OK;
}

int oracle_render(const PbrtSceneDesc* scene, const PbrtCameraDesc* camera, const PbrtSamplerDesc* sampler,
                  float* rgb, int nthreads, uint32_t task_lo, uint32_t task_hi, uint64_t* stats) {
    if (!scene || !camera || !sampler || !rgb || sampler->num_tasks == 0) return PBRT_ERR_INVALID_ARGUMENT;
    SceneData S;
    int st = scene_build(scene, &S);
    if (st) return st;
    return render_scene(S, camera, sampler, rgb, nthreads, task_lo, task_hi, stats);
}

int oracle_scene_create(const PbrtSceneDesc* scene, OracleScene** out) {
    if (!scene || !out) return PBRT_ERR_INVALID_ARGUMENT;
    OracleScene* o = new OracleScene();
    int st = scene_build(scene, &o->S);
    if (st) {
        delete o;
        return st;
    }
    *out = o;
    return PBRT_OK;
}
void oracle_scene_destroy(OracleScene* o) { delete o; }
int oracle_scene_render(const OracleScene* o, const PbrtCameraDesc* camera, const PbrtSamplerDesc* sampler,
                        float* rgb, int nthreads, uint32_t task_lo, uint32_t task_hi, uint64_t* stats) {
    if (!o || !camera || !sampler || !rgb || sampler->num_tasks == 0) return PBRT_ERR_INVALID_ARGUMENT;
    return render_scene(o->S, camera, sampler, rgb, nthreads, task_lo, task_hi, stats);
}

int oracle_task_samples(const PbrtSceneDesc* scene, const PbrtCameraDesc* camera, const PbrtSamplerDesc* sampler,
                        uint32_t task, float* out, uint64_t cap, uint32_t* n_out, uint32_t* stride) {
    SceneData S;
    int st = scene_build(scene, &S);
    if (st) return st;
    RenderCtx R;
    R.S = &S;
    R.cam = camera_new(*camera);
    R.film = film_image(camera->x_res, camera->y_res, camera_filter(*camera), camera->crop_window);
    R.sd = *sampler;
    std::vector<float> dump;
    run_task(R, task, &dump, nullptr);
    uint32_t s = (uint32_t)(5 + integrator_floats(S.lights.size()) + 6 + 3);
    *stride = s;
    *n_out = (uint32_t)(dump.size() / s);
    if (dump.size() > cap) return PBRT_ERR_INVALID_ARGUMENT;
    memcpy(out, dump.data(), dump.size() * sizeof(float));
    return PBRT_OK;
}

int oracle_quadratic(float a, float b, float c, float* t0, float* t1) { return quadratic(a, b, c, t0, t1) ? 1 : 0; }
void oracle_partition_by_f32(float* v, uint32_t n) {
    partition_by(v, n, [](float x) { return x; });
}
void oracle_partition_by_i64(int64_t* v, uint32_t n) {
    partition_by(v, n, [](int64_t x) { return x; });
}
void oracle_crop_window(uint32_t num, uint32_t count, float aspect, float out[4]) {
    crop_window(num, count, aspect, out);
}
void oracle_sub_window(int32_t xs, int32_t xe, int32_t ys, int32_t ye, uint32_t num, uint32_t count, int32_t out[4]) {
    sub_window(xs, xe, ys, ye, num, count, out);
}
int oracle_bbox_intersect(const float lo[3], const float hi[3], const PbrtRay* ray, float out[2]) {
    BBox b{mk(lo[0], lo[1], lo[2]), mk(hi[0], hi[1], hi[2])};
    return bbox_intersect(b, to_ray(*ray), &out[0], &out[1]) ? 1 : 0;
}
void oracle_bbox_metrics(const float lo[3], const float hi[3], float* area, int32_t* me) {
    BBox b{mk(lo[0], lo[1], lo[2]), mk(hi[0], hi[1], hi[2])};
    *area = surface_area(b);
    *me = max_extent(b);
}
int oracle_triangle_intersect(const float tri[9], const PbrtRay* ray, float out[3]) {
    Tri t{mk(tri[0], tri[1], tri[2]), mk(tri[3], tri[4], tri[5]), mk(tri[6], tri[7], tri[8]), false};
    return tri_hit(t, to_ray(*ray), &out[0], &out[1], &out[2]) ? 1 : 0;
}
int oracle_sphere_intersect(const PbrtTransform* o2w, float radius, float z0, float z1, float phimax,
                            const PbrtRay* ray, int mode, float out[16]) {
    Xf x = xf_from_desc(*o2w);
    Sphere s = sphere_new(x, xf_inverse(x), false, radius, z0, z1, phimax);
    Ray r = to_ray(*ray);
    Ray orr = xf_ray(s.w2o.m, r);
    float t, phi;
    if (!sphere_hit_obj(s, orr, &t, &phi)) return 0;
    if (mode == 1) {
        V3 p, nn, du, dv;
        float u, v;
        sphere_dg(s, orr, t, phi, &p, &nn, nullptr, &u, &v, &du, &dv);
        float o[16] = {t, t * 5e-4f, p.x, p.y, p.z, nn.x, nn.y, nn.z, u, v, du.x, du.y, du.z, dv.x, dv.y, dv.z};
        memcpy(out, o, sizeof(o));
    } else if (out) {
        out[0] = t;
    }
    return 1;
}
int oracle_quadric_intersect(int kind, const PbrtTransform* o2w, float a, float b, float c, float phimax,
                             const PbrtRay* ray, int mode, float out[16]) {
    Xf x = xf_from_desc(*o2w);
    Sphere s = kind == PBRT_SHAPE_DISK ? disk_new(x, xf_inverse(x), false, a, b, c, phimax)
                                       : cylinder_new(x, xf_inverse(x), false, a, b, c, phimax);
    Ray r = to_ray(*ray);
    Ray orr = xf_ray(s.w2o.m, r);
    float t, phi;
    if (!quad_hit_obj(s, orr, &t, &phi)) return 0;
    if (mode == 1) {
        V3 p, nn, du, dv;
        float u, v;
        quad_dg(s, orr, t, phi, &p, &nn, &u, &v, &du, &dv);
        float o[16] = {t, t * 5e-4f, p.x, p.y, p.z, nn.x, nn.y, nn.z, u, v, du.x, du.y, du.z, dv.x, dv.y, dv.z};
        memcpy(out, o, sizeof(o));
    } else if (out) {
        out[0] = t;
    }
    return 1;
}
int oracle_matrix_invert(const float m[16], float out[16]) {
    M4 a, r;
    memcpy(a.m, m, sizeof(a.m));
    if (!m4_invert(a, &r)) return 0;
    memcpy(out, r.m, sizeof(r.m));
    return 1;
}
void oracle_look_at(const float pos[3], const float look[3], const float up[3], PbrtTransform* out) {
    xf_to_desc(xf_look_at(mk(pos[0], pos[1], pos[2]), mk(look[0], look[1], look[2]), mk(up[0], up[1], up[2])), out);
}
void oracle_projection(uint32_t xres, uint32_t yres, const PbrtTransform* proj, const float screen[4],
                       PbrtTransform out[4]) {
    Xf o[4];
    projection(xres, yres, xf_from_desc(*proj), screen, o);
    for (int i = 0; i < 4; ++i) xf_to_desc(o[i], &out[i]);
}
void oracle_perspective(float fov, PbrtTransform* out) { xf_to_desc(perspective_xf(fov), out); }
void oracle_transform_point(const PbrtTransform* t, const float p[3], float out[3]) {
    V3 r = xf_point(xf_from_desc(*t).m, mk(p[0], p[1], p[2]));
    out[0] = r.x;
    out[1] = r.y;
    out[2] = r.z;
}
void oracle_transform_vector(const PbrtTransform* t, const float v[3], float out[3]) {
    V3 r = xf_vector(xf_from_desc(*t).m, mk(v[0], v[1], v[2]));
    out[0] = r.x;
    out[1] = r.y;
    out[2] = r.z;
}
// film.rs:280-309
void oracle_film_extents(uint32_t xres, uint32_t yres, const float crop[4], float xw, float yw, int32_t se[4],
                         int32_t pe[4]) {
    Film F = film_image(xres, yres, filter_new(0, xw, yw, 0, 0), crop, false);
    se[0] = f2i32(floorf((float)F.x_start + 0.5f - F.filter.xw));
    se[1] = f2i32(floorf((float)F.x_start + 0.5f + (float)F.x_count + F.filter.xw));
    se[2] = f2i32(floorf((float)F.y_start + 0.5f - F.filter.yw));
    se[3] = f2i32(floorf((float)F.y_start + 0.5f + (float)F.y_count + F.filter.yw));
    pe[0] = F.x_start;
    pe[1] = F.x_start + F.x_count;
    pe[2] = F.y_start;
    pe[3] = F.y_start + F.y_count;
}
float oracle_filter_eval(int kind, float xw, float yw, float p0, float p1, float x, float y) {
    return filter_eval(filter_new(kind, xw, yw, p0, p1), x, y);
}
void oracle_rng_words(uint64_t seed, uint64_t first, uint32_t n, uint32_t* out) {
    uint32_t key[8];
    seed_key(seed, key);
    uint32_t blk[16];
    uint64_t b = first / 16;
    int off = (int)(first % 16);
    chacha12_block(key, b, blk);
    for (uint32_t i = 0; i < n; ++i) {
        if (off == 16) {
            chacha12_block(key, ++b, blk);
            off = 0;
        }
        out[i] = blk[off++];
    }
}
void oracle_chacha_blocks(const uint32_t key[8], uint64_t counter, uint64_t stream, uint32_t rounds,
                          uint32_t n_blocks, uint32_t* out) {
    for (uint32_t i = 0; i < n_blocks; ++i) chacha_block(key, counter + i, stream, (int)rounds, out + 16 * (size_t)i);
}
void oracle_rng_key(uint64_t seed, uint32_t key[8]) { seed_key(seed, key); }
void oracle_rng_floats(uint64_t seed, uint32_t n, float* out) {
    RNG r(seed);
    for (uint32_t i = 0; i < n; ++i) out[i] = r.random_float();
}
void oracle_rng_uints(uint64_t seed, uint32_t n, uint64_t* out) {
    RNG r(seed);
    for (uint32_t i = 0; i < n; ++i) out[i] = r.random_uint();
}
void oracle_rng_shuffle_i64(uint64_t seed, int64_t* v, uint32_t n, uint32_t dims, uint32_t skip) {
    RNG r(seed);
    for (uint32_t i = 0; i < skip; ++i) r.random_uint();
    r.shuffle(v, n, dims);
}
void oracle_rng_permutation(uint64_t seed, uint64_t* v, uint32_t n) {  // rng.rs:35-42
    RNG r(seed);
    for (uint32_t i = 0; i < n; ++i) v[i] = i;
    r.shuffle(v, n, 1);
}
void oracle_stratified(uint64_t seed, const int32_t* calls, uint32_t n_calls, float* out) {
    RNG r(seed);
    size_t off = 0;
    for (uint32_t k = 0; k < n_calls; ++k) {
        const int32_t* c = calls + 4 * k;
        if (c[0] == 1) {
            stratified_1d(out + off, (size_t)c[1], r, c[3] != 0);
            off += (size_t)c[1];
        } else {
            stratified_2d(out + off, (size_t)c[1], (size_t)c[2], r, c[3] != 0);
            off += 2 * (size_t)c[1] * (size_t)c[2];
        }
    }
}
void oracle_latin_hypercube(uint64_t seed, uint32_t num, uint32_t dim, float* out) {
    RNG r(seed);
    latin_hypercube(out, num, dim, r);
}

}  // extern "C"
