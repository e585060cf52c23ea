// bvh_build.h — host-side BVH construction for the device scene.
#pragma once

#include <cstdint>
#include <vector>

#include "../../include/gartus_gpu.h"

namespace gt {

struct Aabb {
    double lo[3], hi[3];
};

// One node of the reference-layout binary BVH, in the reference's pre-order numbering
// (node 0 = root, a node's left subtree is numbered before its right subtree).
struct BuildNode {
    Aabb box;
    uint32_t first, count; // leaf range into `order` (count > 0 for a leaf)
    uint32_t left, right;  // children (internal nodes)
    bool leaf;
};

struct BuiltBvh {
    std::vector<BuildNode> nodes;
    std::vector<uint32_t> order; // leaf order -> primitive index
    uint32_t max_depth = 0;      // deepest node (root = 1)
};

// Padded bounds of one RayGeometry (object.rs:1015-1036, geometry.rs:197-203, 355-362).
Aabb geometry_aabb(const gt_geometry& g);

// Builds the binary SAH BVH of FlatBvh::build (raytracing/bvh.rs:233-288, 430-522):
// 12 centroid buckets along the largest centroid axis, first minimum of
// SA_L*n_L + SA_R*n_R, in-place swap partition, and a stable centroid-then-index
// midpoint split whenever the buckets cannot separate the primitives.
// `threads` host threads build the subtrees of ranges of at most `cut` primitives once
// the top of the tree is built (0: the machine's threads, at most 16, and a cut chosen
// from the count; serial below 65,536 primitives); the tree does not depend on either.
void build_reference_bvh(const gt_primitive* prims, uint32_t count, uint32_t leaf_size, BuiltBvh& out,
                         uint32_t threads = 0, uint32_t cut = 0);

// The same build over given boxes (a mesh's triangles, or world objects).
void build_bvh_from_boxes(const Aabb* boxes, uint32_t count, uint32_t leaf_size, BuiltBvh& out, uint32_t threads = 0,
                          uint32_t cut = 0);

} // namespace gt
