// bvh_build.cpp — the reference's binary SAH BVH, built on the host in f64.
//
// The tree has to be node-for-node the reference's (its traversal statistics are part of
// the parity contract), so every choice below follows raytracing/bvh.rs: bucket index
// min(floor(offset*12), 11) with a saturating cast, strict `<` on cost so the first
// minimum wins, the in-place swap partition, and the midpoint split as a stable sort by
// centroid then primitive index.  The construction itself is an explicit work stack
// (left child processed first, so numbering is pre-order) instead of recursion, which
// keeps multi-million-primitive scenes off the call stack.
#include "bvh_build.h"

#include <algorithm>
#include <cmath>
#include <limits>
#include <numeric>
#include <stdexcept>

namespace gt {
namespace {

constexpr double kEps = 2.220446049250313e-16;
constexpr int kBuckets = 12;

Aabb point_box(const double* p) {
    Aabb b;
    for (int i = 0; i < 3; ++i) b.lo[i] = b.hi[i] = p[i];
    return b;
}
Aabb unite(const Aabb& a, const Aabb& b) {
    Aabb r;
    for (int i = 0; i < 3; ++i) {
        r.lo[i] = std::fmin(a.lo[i], b.lo[i]);
        r.hi[i] = std::fmax(a.hi[i], b.hi[i]);
    }
    return r;
}
Aabb grow(const Aabb& a, const double* p) { return unite(a, point_box(p)); }
Aabb pad(Aabb b, double eps) { // Bounds3::padded, polygon_matrix.rs:84-106
    double half = 0.5 * eps;
    for (int i = 0; i < 3; ++i)
        if (std::fabs(b.hi[i] - b.lo[i]) < eps) {
            b.lo[i] -= half;
            b.hi[i] += half;
        }
    return b;
}
double area(const Aabb& b) { // Bounds3::surface_area, polygon_matrix.rs:114-120
    double dx = std::fmax(b.hi[0] - b.lo[0], 0.0);
    double dy = std::fmax(b.hi[1] - b.lo[1], 0.0);
    double dz = std::fmax(b.hi[2] - b.lo[2], 0.0);
    return 2.0 * (dx * dy + dx * dz + dy * dz);
}
int widest(const Aabb& b) { // Bounds3::largest_axis, polygon_matrix.rs:122-134
    double dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
    if (dx >= dy && dx >= dz) return 0;
    return dy >= dz ? 1 : 2;
}
uint32_t bucket_of(double offset) { // `(offset * 12.0) as usize`, saturating, then min 11
    double v = offset * 12.0;
    uint64_t b = !(v > 0.0) ? 0 : (v >= 1.8e19 ? UINT64_MAX : uint64_t(v));
    return uint32_t(std::min<uint64_t>(b, kBuckets - 1));
}

struct Builder {
    const std::vector<Aabb>& box;
    std::vector<double> cx, cy, cz; // centroids
    std::vector<uint32_t>& order;

    double c(uint32_t p, int axis) const { return axis == 0 ? cx[p] : (axis == 1 ? cy[p] : cz[p]); }

    uint32_t midpoint(uint32_t* idx, uint32_t n, int axis) const { // bvh.rs:508-522
        std::stable_sort(idx, idx + n, [&](uint32_t a, uint32_t b) {
            double ca = c(a, axis), cb = c(b, axis);
            if (ca != cb) return ca < cb;
            return a < b;
        });
        return n / 2;
    }

    // split_bvh_indices (bvh.rs:430-496); returns 0 when the range stays a leaf.
    uint32_t split(uint32_t* idx, uint32_t n, uint32_t leaf_size) const {
        if (n <= leaf_size) return 0;
        double p0[3] = {cx[idx[0]], cy[idx[0]], cz[idx[0]]};
        Aabb cb = point_box(p0);
        for (uint32_t i = 1; i < n; ++i) {
            double p[3] = {cx[idx[i]], cy[idx[i]], cz[idx[i]]};
            cb = grow(cb, p);
        }
        const int axis = widest(cb);
        const double lo = cb.lo[axis];
        const double extent = cb.hi[axis] - lo;
        if (extent <= kEps) return midpoint(idx, n, axis);
        uint32_t cnt[kBuckets] = {0};
        Aabb bb[kBuckets];
        for (uint32_t i = 0; i < n; ++i) {
            uint32_t k = bucket_of((c(idx[i], axis) - lo) / extent);
            bb[k] = cnt[k] ? unite(bb[k], box[idx[i]]) : box[idx[i]];
            cnt[k]++;
        }
        // Left merges as prefix folds (min/max are exact, so fold order is immaterial).
        Aabb lb[kBuckets];
        uint32_t lc[kBuckets];
        bool lh[kBuckets];
        for (int k = 0; k < kBuckets; ++k) {
            lc[k] = (k ? lc[k - 1] : 0) + cnt[k];
            lh[k] = (k ? lh[k - 1] : false) || cnt[k];
            if (cnt[k]) lb[k] = (k && lh[k - 1]) ? unite(lb[k - 1], bb[k]) : bb[k];
            else if (k) lb[k] = lb[k - 1];
        }
        // The right side folds buckets s+1..11 left to right, so build it per split.
        uint32_t best = 0;
        double best_cost = std::numeric_limits<double>::infinity();
        for (int s = 0; s < kBuckets - 1; ++s) {
            uint32_t r_count = 0;
            bool r_has = false;
            Aabb r_box;
            for (int k = s + 1; k < kBuckets; ++k) {
                r_count += cnt[k];
                if (cnt[k]) {
                    r_box = r_has ? unite(r_box, bb[k]) : bb[k];
                    r_has = true;
                }
            }
            if (lc[s] == 0 || r_count == 0) continue;
            double cost = area(lb[s]) * double(lc[s]) + area(r_box) * double(r_count);
            if (cost < best_cost) {
                best_cost = cost;
                best = uint32_t(s);
            }
        }
        if (!std::isfinite(best_cost)) return midpoint(idx, n, axis);
        uint32_t left = 0;
        for (uint32_t next = 0; next < n; ++next) {
            if (bucket_of((c(idx[next], axis) - lo) / extent) <= best) {
                std::swap(idx[left], idx[next]);
                ++left;
            }
        }
        if (left == 0 || left == n) return midpoint(idx, n, axis);
        return left;
    }
};

} // namespace

Aabb geometry_aabb(const gt_geometry& g) {
    switch (g.kind) {
    case GT_GEOM_SPHERE: {
        double r = std::fmax(g.p[3], 0.0);
        Aabb b;
        for (int i = 0; i < 3; ++i) {
            double lo = g.p[i] - r, hi = g.p[i] + r;
            b.lo[i] = std::fmin(lo, hi);
            b.hi[i] = std::fmax(lo, hi);
        }
        return b;
    }
    case GT_GEOM_MOVING_SPHERE: {
        double r = std::fmax(g.p[6], 0.0);
        Aabb a, b;
        for (int i = 0; i < 3; ++i) {
            double lo = g.p[i] - r, hi = g.p[i] + r;
            a.lo[i] = std::fmin(lo, hi);
            a.hi[i] = std::fmax(lo, hi);
            lo = g.p[3 + i] - r;
            hi = g.p[3 + i] + r;
            b.lo[i] = std::fmin(lo, hi);
            b.hi[i] = std::fmax(lo, hi);
        }
        return unite(a, b);
    }
    case GT_GEOM_TRIANGLE: {
        Aabb b = grow(grow(point_box(g.p), g.p + 3), g.p + 6);
        return pad(b, 1e-10);
    }
    case GT_GEOM_QUAD: {
        double c[3], cu[3], cv[3], cuv[3];
        for (int i = 0; i < 3; ++i) {
            c[i] = g.p[i];
            cu[i] = g.p[i] + g.p[3 + i];
            cv[i] = g.p[i] + g.p[6 + i];
            cuv[i] = (g.p[i] + g.p[3 + i]) + g.p[6 + i];
        }
        return pad(grow(grow(grow(point_box(c), cu), cv), cuv), 1e-4);
    }
    default:
        throw std::invalid_argument("unknown geometry kind");
    }
}

void build_reference_bvh(const gt_primitive* prims, uint32_t count, uint32_t leaf_size, BuiltBvh& out) {
    std::vector<Aabb> box(count);
    for (uint32_t i = 0; i < count; ++i) box[i] = geometry_aabb(prims[i].geometry);
    build_bvh_from_boxes(box.data(), count, leaf_size, out);
}

void build_bvh_from_boxes(const Aabb* boxes, uint32_t count, uint32_t leaf_size, BuiltBvh& out) {
    out.nodes.clear();
    out.order.resize(count);
    std::iota(out.order.begin(), out.order.end(), 0u);
    out.max_depth = 0;
    if (count == 0) return;
    if (leaf_size == 0) leaf_size = 1;
    std::vector<Aabb> box(boxes, boxes + count);
    Builder b{box, {}, {}, {}, out.order};
    b.cx.resize(count);
    b.cy.resize(count);
    b.cz.resize(count);
    for (uint32_t i = 0; i < count; ++i) {
        b.cx[i] = 0.5 * (box[i].lo[0] + box[i].hi[0]); // Bounds3::centroid
        b.cy[i] = 0.5 * (box[i].lo[1] + box[i].hi[1]);
        b.cz[i] = 0.5 * (box[i].lo[2] + box[i].hi[2]);
    }
    out.nodes.reserve(size_t(count) * 2);
    struct Task {
        uint32_t first, count, parent, depth;
        bool is_right;
    };
    std::vector<Task> work;
    work.push_back({0, count, UINT32_MAX, 1, false});
    while (!work.empty()) {
        Task t = work.back();
        work.pop_back();
        Aabb nb = box[out.order[t.first]];
        for (uint32_t i = 1; i < t.count; ++i) nb = unite(nb, box[out.order[t.first + i]]);
        const uint32_t id = uint32_t(out.nodes.size());
        out.nodes.push_back(BuildNode{nb, t.first, t.count, 0, 0, true});
        out.max_depth = std::max(out.max_depth, t.depth);
        if (t.parent != UINT32_MAX) {
            if (t.is_right) out.nodes[t.parent].right = id;
            else out.nodes[t.parent].left = id;
        }
        const uint32_t left = b.split(out.order.data() + t.first, t.count, leaf_size);
        if (left == 0) continue;
        out.nodes[id].leaf = false;
        // Right task below left task on the stack: the left subtree is numbered first.
        work.push_back({t.first + left, t.count - left, id, t.depth + 1, true});
        work.push_back({t.first, left, id, t.depth + 1, false});
    }
}

} // namespace gt
