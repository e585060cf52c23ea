// wide_bvh.h — the eight-wide compressed BVH of the f32 throughput traversal.
//
// The tree is collapsed from the reference's binary SAH tree (so it covers exactly the same
// primitives in the same leaves) into nodes of up to eight children whose boxes are
// quantised to one byte per plane against a per-node origin and power-of-two scale, after
// Ylitie, Karras and Laine, "Efficient Incoherent Ray Traversal on GPUs Through Compressed
// Wide BVHs" (HPG 2017).  The byte layout here is this library's own: 80 bytes, five
// 16-byte loads per node.
#pragma once

#include <cstdint>
#include <vector>

namespace gt {

// Slot s of a node holds one child.  Plane q of axis a of slot s lies exactly at
// p[a] + q * 2^(e_a - 127) (q = qlo or qhi byte), which bounds the child's f32 box from
// outside.  Children are placed in slots so that a ray whose direction has sign bits
// `oct` (bit a set when the direction's a-component is negative) meets them roughly in
// the order slot oct ^ 0, oct ^ 1, ..., oct ^ 7.
struct alignas(16) WideNode {
    float p[3];          // quantisation origin, a multiple of the axis scale
    uint32_t e_imask;    // bits 0-7 / 8-15 / 16-23: biased exponent of the x / y / z scale;
                         // bits 24-31: slot s is an internal child
    uint32_t child_base; // node index of the first internal child; a node's internal
                         // children are consecutive, in slot order
    uint32_t prim_base;  // leaf slot of the first primitive of the node's leaf children,
                         // which are consecutive, in slot order
    uint32_t meta[2];    // byte s: leaf child = count << 5 | offset from prim_base; else 0
    uint32_t qlo[6];     // axis a's lower planes: slots 0-3 in qlo[2a], slots 4-7 in qlo[2a+1]
    uint32_t qhi[6];     // upper planes, same layout
};
static_assert(sizeof(WideNode) == 80, "WideNode is five 16-byte loads");

// Deepest wide tree the device traversal's stack holds (one entry per level).
constexpr uint32_t kWideStack = 32;

struct BuiltBvh;

struct WideBvh {
    std::vector<WideNode> nodes;  // node 0 is the root
    std::vector<uint32_t> order;  // new leaf slot -> leaf slot of the binary tree's order
    uint32_t depth = 0;           // levels, root = 1
    std::vector<uint32_t> source; // with keep_source: binary node of node * 8 + slot (~0u empty)
};

// Collapses `bvh` (binary, reference layout) into `out`.  Returns false when the tree has
// no wide form here: a leaf root, a leaf of more than four primitives, a tree deeper
// than kWideStack, or coordinates outside the range the scale exponents cover; the caller
// then keeps the binary traversal.
bool build_wide_bvh(const BuiltBvh& bvh, WideBvh& out, bool keep_source = false);

} // namespace gt
