// kz_bvh.h — host-side BVH builder for the device traversal kernels.
//
// Replaces the reference accelerators (BVHAccel, random-axis median split,
// src/core/accel.cpp:83-183; EmbreeAccel HIGH-quality build,
// src/core/accel.cpp:185-315) with a binned-SAH binary BVH collapsed into an
// 8-wide BVH with quantized child boxes, laid out for 16-byte vector fetches
// on the GPU.
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

// The binary build: binned SAH (32 bins per axis), leaves of at most 3
// triangles (larger only where the depth cap kMaxBvhDepth is hit; the wide
// collapse halves those by count).
constexpr int kMaxBvhDepth = 60;

// 8-wide BVH with quantized child boxes, collapsed from a binned-SAH binary
// BVH (leaves of at most 3 triangles). Node = 80 bytes, 20 x 32-bit words:
//   w0..w2   p (float): lower corner of the node box
//   w3       ex | ey << 8 | ez << 16 | imask << 24; an axis' quantum is
//            2^(e - 127); imask bit s = slot s holds an inner node
//   w4       index of the first inner child (inner children are consecutive,
//            in slot order)
//   w5       first triangle record of the node's leaves
//   w6, w7   meta byte per slot: 0 empty; inner: 0x20 | (24 + s); leaf:
//            (unary triangle count: 1, 3 or 7) << 5 | offset from w5
//   w8..w19  per axis x, y, z: 8 low bytes (2 words) then 8 high bytes
//            (2 words): child box = p + [q_lo, q_hi] * quantum, rounded
//            outward so it contains the exact child box.
// Slots are assigned so that slot s's child lies towards the octant
// (+x if s & 1, +y if s & 2, +z if s & 4) of the node centre; a ray visits
// inner children in the order of slot ^ (its direction octant), which
// approximates near-first without sorting.
// Triangle record (48 bytes, 3 x float4), in the order the leaves reference
// them: (v0.xyz, global triangle id), (v1.xyz, geom id), (v2.xyz, material
// id), the integer fields stored as raw 32-bit patterns.
constexpr int kWideWords = 20;
// The builder rejects trees deeper than kWideDepthCap (binary depth cap + 32
// count splits); the traversal's group stack has kWideStack entries. They are
// equal in every product build. A test build may define KZ_WIDE_STACK smaller
// to drive the traversal into its stack-overflow path (KZ_ERR_STACK) on
// ordinary trees.
constexpr int kWideDepthCap = 96;
#ifndef KZ_WIDE_STACK
#define KZ_WIDE_STACK 96
#endif
constexpr int kWideStack = KZ_WIDE_STACK;
static_assert(kWideStack >= 1 && kWideStack <= kWideDepthCap, "traversal stack size out of range");

struct WideBvhOutput {
    std::vector<uint32_t> nodes;   // n_nodes * kWideWords
    std::vector<float> tris;       // ntris * 12 floats
    std::vector<uint32_t> order;   // record -> global triangle id
    uint32_t n_nodes = 0;
    uint32_t depth = 0;            // wide levels
};

// Collapse of the binary build into wide nodes: SAH-optimal slot assignment
// (default) or greedy (open the largest-area child until 8 slots). Costs are
// relative SAH weights of a wide-node visit and of one triangle test
// (KZ_BVH_TRI_COST).
// Relative cost of one triangle test against a wide-node visit in the SAH
// collapse. With the leaf tests shared by the warp (32 pairs per round), a
// triangle is cheap next to an eight-slot node test: on the terrain frame
// (1080p, 64 spp) the frame rate for 2.0 / 1.0 / 0.5 / 0.35 / 0.25 / 0.15
// was 1,665 / 1,690 / 1,732 / 1,744 / 1,747 / 1,743 Mpaths*bounces/s.
#ifndef KZ_BVH_BIN_LEAF
#define KZ_BVH_BIN_LEAF 1
#endif
#ifndef KZ_BVH_TRI_COST
#define KZ_BVH_TRI_COST 0.25f
#endif
struct WideBuildOptions {
    bool sah_collapse = true;
    float node_cost = 1.0f;
    float tri_cost = KZ_BVH_TRI_COST;
    int binary_max_leaf = KZ_BVH_BIN_LEAF;  // leaf size of the binary build the SAH collapse regroups (<= 3)
};

void build_wide_bvh(const BvhBuildInput& in, WideBvhOutput& out, const WideBuildOptions& opt = WideBuildOptions{});

}  // namespace kz
