// Test shim: exposes the product's host BVH builder (gartus_gb300/csrc/bvh_build.cpp)
// through a C function so CPU tests can compare it node-for-node with the oracle.
#include <cstring>

#include "../../gartus_gb300/csrc/bvh_build.h"

// threads, cut: the parallel build's settings (0, 0: the library's defaults).
extern "C" int shim_build(const gt_primitive* prims, uint32_t count, uint32_t leaf, uint32_t* node_count,
                          double* bounds, uint32_t* info, uint32_t* order, uint32_t capacity, uint32_t* depth,
                          uint32_t threads, uint32_t cut) {
    gt::BuiltBvh b;
    gt::build_reference_bvh(prims, count, leaf, b, threads, cut);
    *node_count = uint32_t(b.nodes.size());
    *depth = b.max_depth;
    if (b.nodes.size() > capacity) return 1;
    for (size_t i = 0; i < b.nodes.size(); ++i) {
        for (int k = 0; k < 3; ++k) {
            bounds[i * 6 + k] = b.nodes[i].box.lo[k];
            bounds[i * 6 + 3 + k] = b.nodes[i].box.hi[k];
        }
        info[i * 3 + 0] = b.nodes[i].leaf ? 1u : 0u;
        info[i * 3 + 1] = b.nodes[i].leaf ? b.nodes[i].first : b.nodes[i].left;
        info[i * 3 + 2] = b.nodes[i].leaf ? b.nodes[i].count : b.nodes[i].right;
    }
    std::memcpy(order, b.order.data(), b.order.size() * sizeof(uint32_t));
    return 0;
}
