// wide_bvh.cpp — collapse of the reference's binary SAH tree into the eight-wide
// compressed tree of the f32 traversal (layout and rules in wide_bvh.h).
#include "wide_bvh.h"

#include <algorithm>
#include <cmath>
#include <cstring>

#include "bvh_build.h"

namespace gt {
namespace {

// The f32 box the binary traversal uses for a node: its f64 box rounded outward.
struct Box32 {
    double lo[3], hi[3]; // f32 values, held in double
};

inline double down32(double v) {
    float f = float(v);
    if (double(f) > v) f = std::nextafter(f, -INFINITY);
    return double(f);
}
inline double up32(double v) {
    float f = float(v);
    if (double(f) < v) f = std::nextafter(f, INFINITY);
    return double(f);
}
Box32 box32(const Aabb& b) {
    Box32 r;
    for (int a = 0; a < 3; ++a) {
        r.lo[a] = down32(b.lo[a]);
        r.hi[a] = up32(b.hi[a]);
    }
    return r;
}

double area(const Aabb& b) {
    const double x = b.hi[0] - b.lo[0], y = b.hi[1] - b.lo[1], z = b.hi[2] - b.lo[2];
    return x * y + y * z + z * x;
}

// One axis of a node: the smallest scale 2^e (e in [-126, 127]) for which every child
// plane is a whole number of steps from an origin k0 * 2^e that f32 holds exactly, with
// at most 255 steps across the node.  Returns false when no exponent fits.
bool quantise_axis(double lo_min, double hi_max, int& e_out, double& k0_out) {
    const double ext = hi_max - lo_min;
    const double mag = std::max(std::fabs(lo_min), std::fabs(hi_max));
    int e = -126;
    if (ext > 0) e = std::max(e, int(std::ceil(std::log2(ext / 255.0))));
    if (mag > 0) e = std::max(e, int(std::ceil(std::log2(mag))) - 23);
    for (; e <= 127; ++e) {
        const double s = std::ldexp(1.0, e);
        const double k0 = std::floor(lo_min / s), k1 = std::ceil(hi_max / s);
        if (k1 - k0 <= 255.0 && std::fabs(k0) < 16777216.0) {
            e_out = e;
            k0_out = k0;
            return true;
        }
    }
    return false;
}

// Which binary nodes become wide nodes.  The leaves are the reference's, so the surface
// area heuristic of the wide tree (Ylitie et al. 2017, section 4.1) reduces to the summed
// area of its nodes: cost[n][j] is the least summed area of wide nodes inside binary
// subtree n when n's subtree takes at most j slots of the wide node above it, solved
// bottom-up over j = 1..8.
struct Collapse {
    enum : uint8_t { SLOT = 0xff, FEWER = 0xfe }; // else: split with k slots to the left
    std::vector<double> cost;   // [node * 8 + j - 1]
    std::vector<uint8_t> how;   // same index: SLOT, FEWER or k
    std::vector<uint8_t> split; // per node: k of the best eight-slot split of its children

    void solve(const BuiltBvh& bvh) {
        const size_t n = bvh.nodes.size();
        cost.assign(n * 8, 0.0);
        how.assign(n * 8, SLOT);
        split.assign(n, 0);
        for (size_t i = n; i-- > 0;) { // pre-order: children follow their parent
            const BuildNode& b = bvh.nodes[i];
            double* c = &cost[i * 8];
            uint8_t* h = &how[i * 8];
            if (b.leaf) continue; // a leaf is one slot at no node cost
            const double* cl = &cost[size_t(b.left) * 8];
            const double* cr = &cost[size_t(b.right) * 8];
            double best8 = INFINITY;
            for (int k = 1; k <= 7; ++k) {
                const double v = cl[k - 1] + cr[8 - k - 1];
                if (v < best8) {
                    best8 = v;
                    split[i] = uint8_t(k);
                }
            }
            c[0] = area(b.box) + best8; // its own wide node
            h[0] = SLOT;
            for (int j = 2; j <= 8; ++j) {
                c[j - 1] = c[j - 2];
                h[j - 1] = FEWER;
                for (int k = 1; k < j; ++k) {
                    const double v = cl[k - 1] + cr[j - k - 1];
                    if (v < c[j - 1]) {
                        c[j - 1] = v;
                        h[j - 1] = uint8_t(k);
                    }
                }
            }
        }
    }
    // The slots binary subtree m takes when it may use up to j of them.
    void expand(const BuiltBvh& bvh, uint32_t m, int j, std::vector<uint32_t>& out) const {
        while (how[size_t(m) * 8 + size_t(j) - 1] == FEWER) --j;
        const uint8_t h = how[size_t(m) * 8 + size_t(j) - 1];
        if (bvh.nodes[m].leaf || h == SLOT) {
            out.push_back(m);
            return;
        }
        expand(bvh, bvh.nodes[m].left, h, out);
        expand(bvh, bvh.nodes[m].right, j - h, out);
    }
    // The children (at most eight) of the wide node made from binary internal node b.
    void children(const BuiltBvh& bvh, uint32_t b, std::vector<uint32_t>& out) const {
        out.clear();
        const int k = split[b];
        expand(bvh, bvh.nodes[b].left, k, out);
        expand(bvh, bvh.nodes[b].right, 8 - k, out);
    }
};

struct Builder {
    const BuiltBvh& bvh;
    WideBvh& out;
    const Collapse& plan;
    uint32_t next_slot = 0; // next new leaf slot
    bool ok = true;
    bool keep_source = false;

    // Slot of each child: the child lying furthest against the diagonal direction of
    // octant s (signs of s's bits) goes to slot s, chosen greedily by that projection.
    void assign_slots(const std::vector<uint32_t>& ch, const Aabb& parent, int slot_of[8]) const {
        double pc[3];
        for (int a = 0; a < 3; ++a) pc[a] = 0.5 * (parent.lo[a] + parent.hi[a]);
        const size_t n = ch.size();
        double cost[8][8];
        for (size_t i = 0; i < n; ++i) {
            const Aabb& b = bvh.nodes[ch[i]].box;
            double c[3];
            for (int a = 0; a < 3; ++a) c[a] = 0.5 * (b.lo[a] + b.hi[a]) - pc[a];
            for (int s = 0; s < 8; ++s)
                cost[i][s] = ((s & 1) ? -c[0] : c[0]) + ((s & 2) ? -c[1] : c[1]) + ((s & 4) ? -c[2] : c[2]);
        }
        bool child_done[8] = {}, slot_used[8] = {};
        for (size_t k = 0; k < n; ++k) {
            int bi = -1, bs = -1;
            double bc = INFINITY;
            for (size_t i = 0; i < n; ++i) {
                if (child_done[i]) continue;
                for (int s = 0; s < 8; ++s)
                    if (!slot_used[s] && (bi < 0 || cost[i][s] < bc)) {
                        bi = int(i);
                        bs = s;
                        bc = cost[i][s];
                    }
            }
            child_done[bi] = true;
            slot_used[bs] = true;
            slot_of[bi] = bs;
        }
    }

    // Fills node w from binary internal node b; recurses into its internal children.
    void build(uint32_t w, uint32_t b, uint32_t depth) {
        if (!ok) return;
        out.depth = std::max(out.depth, depth);
        if (depth > kWideStack) {
            ok = false;
            return;
        }
        std::vector<uint32_t> ch;
        plan.children(bvh, b, ch);
        int slot_of[8];
        assign_slots(ch, bvh.nodes[b].box, slot_of);
        int child_in_slot[8];
        std::fill(child_in_slot, child_in_slot + 8, -1);
        for (size_t i = 0; i < ch.size(); ++i) child_in_slot[slot_of[i]] = int(i);

        WideNode nd;
        std::memset(&nd, 0, sizeof(nd));
        // Quantisation of the children's f32 boxes, per axis.
        Box32 cb[8];
        double lo_min[3] = {INFINITY, INFINITY, INFINITY}, hi_max[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (size_t i = 0; i < ch.size(); ++i) {
            cb[i] = box32(bvh.nodes[ch[i]].box);
            for (int a = 0; a < 3; ++a) {
                lo_min[a] = std::min(lo_min[a], cb[i].lo[a]);
                hi_max[a] = std::max(hi_max[a], cb[i].hi[a]);
            }
        }
        int e[3];
        double k0[3];
        for (int a = 0; a < 3; ++a) {
            if (!quantise_axis(lo_min[a], hi_max[a], e[a], k0[a])) {
                ok = false;
                return;
            }
            nd.p[a] = float(k0[a] * std::ldexp(1.0, e[a]));
        }
        uint32_t imask = 0;
        uint32_t n_internal = 0;
        for (int s = 0; s < 8; ++s) {
            const int i = child_in_slot[s];
            uint32_t lo8[3] = {255, 255, 255}, hi8[3] = {0, 0, 0}; // an empty slot: an empty box
            if (i >= 0) {
                for (int a = 0; a < 3; ++a) {
                    const double sc = std::ldexp(1.0, e[a]);
                    lo8[a] = uint32_t(std::floor(cb[i].lo[a] / sc) - k0[a]);
                    hi8[a] = uint32_t(std::ceil(cb[i].hi[a] / sc) - k0[a]);
                }
                if (!bvh.nodes[ch[size_t(i)]].leaf) {
                    imask |= 1u << s;
                    ++n_internal;
                }
            }
            for (int a = 0; a < 3; ++a) {
                nd.qlo[2 * a + (s >> 2)] |= lo8[a] << (8 * (s & 3));
                nd.qhi[2 * a + (s >> 2)] |= hi8[a] << (8 * (s & 3));
            }
        }
        nd.e_imask = uint32_t(e[0] + 127) | (uint32_t(e[1] + 127) << 8) | (uint32_t(e[2] + 127) << 16) | (imask << 24);
        // Leaf children: their primitives take the next new slots, in slot order.
        nd.prim_base = next_slot;
        uint32_t offset = 0;
        for (int s = 0; s < 8; ++s) {
            const int i = child_in_slot[s];
            if (i < 0) continue;
            const BuildNode& c = bvh.nodes[ch[size_t(i)]];
            if (!c.leaf) continue;
            if (c.count == 0 || c.count > 4) {
                ok = false;
                return;
            }
            nd.meta[s >> 2] |= ((c.count << 5) | offset) << (8 * (s & 3));
            for (uint32_t k = 0; k < c.count; ++k) out.order.push_back(c.first + k);
            offset += c.count;
            next_slot += c.count;
        }
        // Internal children: a block of consecutive nodes, filled depth first.
        nd.child_base = uint32_t(out.nodes.size());
        out.nodes.resize(out.nodes.size() + n_internal);
        out.nodes[w] = nd;
        if (keep_source) {
            out.source.resize(out.nodes.size() * 8, ~0u);
            for (int s = 0; s < 8; ++s)
                if (child_in_slot[s] >= 0) out.source[size_t(w) * 8 + size_t(s)] = ch[size_t(child_in_slot[s])];
        }
        uint32_t r = 0;
        for (int s = 0; s < 8; ++s) {
            const int i = child_in_slot[s];
            if (i < 0 || bvh.nodes[ch[size_t(i)]].leaf) continue;
            build(nd.child_base + r, ch[size_t(i)], depth + 1);
            ++r;
        }
    }
};

} // namespace

bool build_wide_bvh(const BuiltBvh& bvh, WideBvh& out, bool keep_source) {
    out = WideBvh();
    if (bvh.nodes.empty() || bvh.nodes[0].leaf) return false;
    out.nodes.resize(1);
    out.order.reserve(bvh.order.size());
    Collapse plan;
    plan.solve(bvh);
    Builder b{bvh, out, plan};
    b.keep_source = keep_source;
    b.build(0, 0, 1);
    if (!b.ok || out.order.size() != bvh.order.size()) {
        out = WideBvh();
        return false;
    }
    return true;
}

} // namespace gt
