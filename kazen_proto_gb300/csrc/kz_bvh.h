// kz_bvh.h — host-side BVH builder for the device traversal kernels.
//
// Replaces the reference accelerators (BVHAccel, random-axis median split,
// src/core/accel.cpp:83-183; EmbreeAccel HIGH-quality build,
// src/core/accel.cpp:185-315) with a binned-SAH binary BVH whose nodes are
// laid out for 16-byte vector fetches on the GPU.
//
// Device node (64 bytes, 4 x float4), both children's boxes in one node:
//   n0 = (c0.lo.x, c0.hi.x, c0.lo.y, c0.hi.y)
//   n1 = (c1.lo.x, c1.hi.x, c1.lo.y, c1.hi.y)
//   n2 = (c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z)
//   n3 = (link0, link1, count0, count1) as int32
// link >= 0 is an inner node index; link < 0 is a leaf whose triangle records
// start at ~link and number `count`. An empty child has an inverted box.
// Triangle record (48 bytes, 3 x float4), in leaf order:
//   (v0.xyz, global triangle id), (v1.xyz, geom id), (v2.xyz, material id)
// with the integer fields stored as raw 32-bit patterns.
#pragma once

#include <cstdint>
#include <vector>

namespace kz {

struct BvhBuildInput {
    const float* tri_verts;        // ntris * 9 floats, world space
    uint32_t ntris;
    const uint32_t* tri_geom;      // geom id per triangle
    const int32_t* geom_material;  // material id per geom
};

struct BvhBuildOutput {
    std::vector<float> nodes;      // n_nodes * 16 floats
    std::vector<float> tris;       // ntris * 12 floats
    std::vector<uint32_t> order;   // record -> global triangle id
    uint32_t n_nodes = 0;
    uint32_t depth = 0;
};

// Binned SAH (32 bins per axis), at most `max_leaf` triangles per leaf
// (larger only when centroids coincide or the depth limit is hit). Depth is
// capped at kMaxBvhDepth so the fixed traversal stack cannot overflow.
constexpr int kMaxBvhDepth = 60;
void build_bvh(const BvhBuildInput& in, int max_leaf, BvhBuildOutput& out);

}  // namespace kz
