// layout.h - device data layout of a flattened BVH scene (host + device).
//
// The reference keeps a depth-first array of PackedBVHNode
// (src/primitive/aggregates/bvh.rs:260-326): first child at n+1, second
// child at second_child_offset.  On the device the same tree is stored as
// sibling PAIRS: every inner node owns one 64-byte pair holding its two
// children's 32-byte records (child1 first), so one visit fetches both
// child boxes.  Pairs are numbered in the depth-first pre-order of their
// parents.  The root's own record travels in the kernel arguments.
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define PBRT_HD __host__ __device__ __forceinline__
#else
#define PBRT_HD inline
#endif

namespace pbrt {

// 32-byte child record: box + two words.
//   inner child: a = index of its own children's pair, b = its split axis
//   leaf child:  a = first ordered primitive,        b = kLeafBit | count
struct alignas(16) ChildRec {
    float lo_x, lo_y, lo_z;
    uint32_t a;
    float hi_x, hi_y, hi_z;
    uint32_t b;
};
static_assert(sizeof(ChildRec) == 32, "child record is 32 bytes");

struct alignas(64) NodePair {
    ChildRec c[2];
};
static_assert(sizeof(NodePair) == 64, "node pair is 64 bytes");

constexpr uint32_t kLeafBit = 0x80000000u;
constexpr uint32_t kCountMask = 0x7fffffffu;

// 4-wide node collapsed from two levels of the reference's binary tree.
// For a binary inner node N with children L (first) and R (second):
//   slot 0/1 = L's first/second child (slot 0 = L itself if L is a leaf,
//   slot 1 then empty), slot 2/3 = the same for R.
// Child record words: a = kNode4Leaf | first primitive, or the index of
// the child's own Node4, or kNode4Empty; b of slot 0 holds the node's
// three binary split axes: axis(N) | axis(L) << 2 | axis(R) << 4.
// The primitives of a leaf child end at the record that carries
// kPrimLastBit (PrimRec r2[3]).
struct alignas(128) Node4 {
    ChildRec c[4];
};
static_assert(sizeof(Node4) == 128, "4-wide node is 128 bytes");
constexpr uint32_t kNode4Leaf = 0x80000000u;
constexpr uint32_t kNode4Empty = 0xffffffffu;
constexpr uint32_t kPrimLastBit = 1u;

// 48-byte primitive record in BVH (ordered) order.  Triangle: p1 and the
// edges e1 = p2 - p1, e2 = p3 - p1, computed on the host with the same f32
// subtraction the reference does per test (src/shape/mesh.rs:45-46).
//   r0 = (p1.xyz, id)  id = refined input index | kSphereBit if a sphere
//   r1 = (e1.xyz, sphere index bits for spheres)
//   r2 = (e2.xyz, flags: kPrimLastBit on the last primitive of a leaf)
struct alignas(16) PrimRec {
    float r0[4];
    float r1[4];
    float r2[4];
};
static_assert(sizeof(PrimRec) == 48, "primitive record is 48 bytes");
constexpr uint32_t kSphereBit = 0x80000000u;

// An analytic shape - sphere (src/shape/sphere.rs:16-25), disk
// (src/shape/disk.rs:16-22) or cylinder (src/shape/cylinder.rs:16-23) -
// with its world-to-object and object-to-world matrix rows.  A disk keeps
// its height in z_min = z_max (its object bound, disk.rs:70-74).
// An instance (TransformedPrimitive) uses the same record: w2o / o2w are
// its world-to-primitive / primitive-to-world matrices and `instance`
// selects the definition's BVH.
enum { kQuadSphere = 0, kQuadDisk = 1, kQuadCylinder = 2, kQuadInstance = 3 };
struct alignas(16) SphereRec {
    float w2o[16];      // row-major world_to_object.m
    float o2w[16];      // row-major object_to_world.m
    float radius, z_min, z_max, phi_max;
    float theta_min, theta_max;
    uint32_t full;      // the phi (and for spheres the z) clip cannot reject
    uint32_t flip;      // reverse_orientation ^ transform_swaps_handedness
    uint32_t kind;      // kQuad*
    float height, inner_radius;
    uint32_t instance;  // kQuadInstance: definition index
};
static_assert(sizeof(SphereRec) == 176, "analytic shape record is 176 bytes");

}  // namespace pbrt
