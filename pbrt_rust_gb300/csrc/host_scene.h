// host_scene.h - host-side scene preparation for the device path.
//
// f32 math with the reference's operation order (no FMA: this file is
// compiled with -ffp-contract=off), primitive refinement, the reference
// SAH/middle/equal BVH build, its depth-first flattening, and the
// conversion to the device pair layout of layout.h.
#pragma once
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/pbrt_gpu.h"
#include "layout.h"

namespace pbrt {

struct V3 {
    float x, y, z;
};
inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
inline V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator*(V3 a, float f) { return v3(a.x * f, a.y * f, a.z * f); }
inline float dot3(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross3(V3 a, V3 b) {
    return v3((a.y * b.z) - (a.z * b.y), (a.z * b.x) - (a.x * b.z), (a.x * b.y) - (a.y * b.x));
}
inline float len3(V3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
inline V3 normalize3(V3 a) {  // geometry/normal.rs:181-186: v * (1 / |v|)
    float r = 1.0f / len3(a);
    return a * r;
}
inline float axis_of(V3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

struct Box {
    V3 lo, hi;
};
Box box_empty();
Box box_union(const Box& a, const Box& b);
Box box_union(const Box& a, V3 p);
float box_area(const Box& b);
int box_max_extent(const Box& b);

struct M4 {
    float m[4][4];
};
M4 m4_identity();
M4 m4_mul(const M4& a, const M4& b);
bool m4_inverse(const M4& a, M4* out);  // src/transform/matrix4x4.rs:66-160
V3 m4_point(const M4& m, V3 p);          // src/transform/transform.rs:195-208
V3 m4_vector(const M4& m, V3 v);         // src/transform/transform.rs:210-218
bool m4_swaps_handedness(const M4& m);   // src/transform/transform.rs:176-183

struct Xf {
    M4 m, mi;
};
Xf xf_from_desc(const PbrtTransform& t);
Xf xf_mul(const Xf& a, const Xf& b);
Xf xf_inverse(const Xf& a);

// One primitive of the fully refined list.
struct HostPrim {
    int kind;  // PBRT_SHAPE_TRIANGLE_MESH (triangle) or PBRT_SHAPE_SPHERE
    int shape;
    int material;
    int area_light;
    V3 p1, p2, p3;  // triangle vertices in refined order
    bool flip;
    int sphere;  // index into spheres
};

// Flattened reference node (PackedBVHNode, bvh.rs:260-272).
struct FlatNode {
    Box box;
    bool leaf;
    uint32_t offset;  // leaf: first prim; inner: second child
    uint32_t count;   // leaf: prim count; inner: axis
};

struct HostBVH {
    std::vector<HostPrim> prims;
    std::vector<SphereRec> spheres;
    std::vector<FlatNode> nodes;
    std::vector<uint32_t> ordered;  // ordered_prims: refined input index
    uint32_t depth = 0;
    // device layout
    ChildRec root{};
    std::vector<NodePair> pairs;
    std::vector<PrimRec> recs;
    bool has_spheres = false;
    // 4-wide layout (same tree, two binary levels per node)
    ChildRec root4{};
    std::vector<Node4> nodes4;
    uint32_t stack4_bound = 0;  // most entries a 4-wide traversal can push
    // instance definitions: one BVH each, shared by all their instances
    std::vector<HostBVH> insts;
    // With instances, the id a hit reports: refined primitives numbered in
    // order with each instance taking as many ids as its definition has
    // refined primitives (the ids of the same scene with every instance
    // copied out).  flat_id[i] = first id of refined primitive i; empty
    // without instances (id = refined index).
    std::vector<uint32_t> flat_id;
    uint64_t n_flat = 0;
};

// Fully refine shapes, build and flatten the BVH, and fill the device
// layout.  Returns a PbrtStatus; *err gets a message on failure.
int build_host_bvh(const PbrtShapeDesc* shapes, uint32_t n_shapes, uint32_t max_prims, const char* split_method,
                   HostBVH* out, std::string* err, bool on_device = false, const PbrtInstanceDesc* defs = nullptr,
                   uint32_t n_defs = 0);

// Bounds (mesh.rs:196-205, sphere.rs:111-126) and centroids (bvh.rs:77) of
// the refined primitives.
void prim_bounds(const HostBVH& H, std::vector<Box>* bounds, std::vector<float>* cx, std::vector<float>* cy,
                 std::vector<float>* cz);

// The tree of build_tree (H.nodes, H.ordered, H.depth) built on the current
// CUDA device (bvh_build.cu): identical nodes and primitive order.
int device_build_tree(HostBVH& H, uint32_t max_prims, int split, std::string* err);

int parse_split_method(const char* s);

// Camera set-up (src/camera/mod.rs:105-135, projective.rs:48-72): the
// raster-to-camera and camera-to-world matrices, row-major.
void camera_matrices(const PbrtCameraDesc& cam, float raster_to_camera[16], float camera_to_world[16]);

// The film's filter table (camera/film.rs:89-97, filter.rs:44-124); returns
// PBRT_ERR_INVALID_ARGUMENT for an unknown filter kind.
int filter_table(const PbrtCameraDesc& cam, float table[256]);

}  // namespace pbrt
