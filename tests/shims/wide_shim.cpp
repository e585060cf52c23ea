// Test shim: builds the reference tree and the eight-wide tree collapsed from it with the
// product's host code (gartus_gb300/csrc/bvh_build.cpp, wide_bvh.cpp) and checks the wide
// tree's invariants exactly, so CPU tests can run them over many scenes.
#include <cmath>
#include <cstring>
#include <vector>

#include "../../gartus_gb300/csrc/bvh_build.h"
#include "../../gartus_gb300/csrc/wide_bvh.h"

namespace {

double down32(double v) {
    float f = float(v);
    if (double(f) > v) f = std::nextafter(f, -INFINITY);
    return double(f);
}
double up32(double v) {
    float f = float(v);
    if (double(f) < v) f = std::nextafter(f, INFINITY);
    return double(f);
}
uint32_t byte_of(const uint32_t* words, int a, int s) { return (words[2 * a + (s >> 2)] >> (8 * (s & 3))) & 0xffu; }

} // namespace

// Returns 0 when every invariant holds, else a code naming the first broken one:
//  1 the wide tree was not built, 2 the leaf order is not a permutation, 3 a slot's
//  plane does not bound its binary node's f32 box, 4 a leaf slot's primitives are not its
//  binary leaf's, 5 a node's internal children are not the nodes its slots name,
//  6 an empty slot carries a leaf, 7 a plane is not exactly representable.
// stats: nodes, depth, internal slots, leaf slots, empty slots.
extern "C" int shim_wide(const gt_primitive* prims, uint32_t count, uint32_t leaf, uint32_t* stats) {
    gt::BuiltBvh b;
    gt::build_reference_bvh(prims, count, leaf, b);
    gt::WideBvh w;
    if (!gt::build_wide_bvh(b, w, true)) return 1;
    stats[0] = uint32_t(w.nodes.size());
    stats[1] = w.depth;
    stats[2] = stats[3] = stats[4] = 0;
    std::vector<uint8_t> seen(count, 0);
    for (uint32_t j = 0; j < w.order.size(); ++j) {
        if (w.order[j] >= count || seen[w.order[j]]) return 2;
        seen[w.order[j]] = 1;
    }
    if (w.order.size() != count) return 2;
    // Binary node each wide node stands for (node 0: the root).
    std::vector<uint32_t> src_of_node(w.nodes.size(), ~0u);
    src_of_node[0] = 0;
    for (size_t n = 0; n < w.nodes.size(); ++n) {
        const gt::WideNode& nd = w.nodes[n];
        const uint32_t imask = nd.e_imask >> 24;
        uint32_t rank = 0, offset = 0;
        for (int s = 0; s < 8; ++s) {
            const uint32_t src = w.source[n * 8 + size_t(s)];
            const uint32_t m = (nd.meta[s >> 2] >> (8 * (s & 3))) & 0xffu;
            if (src == ~0u) {
                ++stats[4];
                if (m != 0 || (imask >> s & 1u)) return 6;
                continue;
            }
            const gt::BuildNode& bn = b.nodes[src];
            for (int a = 0; a < 3; ++a) {
                const int e = int((nd.e_imask >> (8 * a)) & 0xffu) - 127;
                const double sc = std::ldexp(1.0, e);
                const double lo = double(nd.p[a]) + double(byte_of(nd.qlo, a, s)) * sc;
                const double hi = double(nd.p[a]) + double(byte_of(nd.qhi, a, s)) * sc;
                // exact: the origin is a multiple of the scale below 2^24 steps
                if (std::fmod(double(nd.p[a]), sc) != 0.0 || std::fabs(double(nd.p[a]) / sc) >= 16777216.0) return 7;
                if (!(lo <= down32(bn.box.lo[a]) && hi >= up32(bn.box.hi[a]))) return 3;
            }
            if (imask >> s & 1u) {
                if (bn.leaf || m != 0) return 5;
                const uint32_t child = nd.child_base + rank++;
                if (child >= w.nodes.size()) return 5;
                src_of_node[child] = src;
                ++stats[2];
            } else {
                if (!bn.leaf) return 5;
                const uint32_t cnt = m >> 5, off = m & 31u;
                if (cnt != bn.count || off != offset) return 4;
                for (uint32_t k = 0; k < cnt; ++k)
                    if (w.order[nd.prim_base + off + k] != bn.first + k) return 4;
                offset += cnt;
                ++stats[3];
            }
        }
    }
    for (size_t n = 0; n < w.nodes.size(); ++n)
        if (src_of_node[n] == ~0u) return 5;
    return 0;
}
