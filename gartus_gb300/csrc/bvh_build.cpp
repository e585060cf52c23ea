// bvh_build.cpp — the reference's binary SAH BVH, built on the host in f64.
//
// The tree has to be node-for-node the reference's (its traversal statistics are part of
// the parity contract), so every choice below follows raytracing/bvh.rs: bucket index
// min(floor(offset*12), 11) with a saturating cast, strict `<` on cost so the first
// minimum wins, the in-place swap partition, and the midpoint split as a stable sort by
// centroid then primitive index.  The construction itself is an explicit work stack
// (left child processed first, so numbering is pre-order) instead of recursion, which
// keeps multi-million-primitive scenes off the call stack.
//
// Large scenes build in parallel: the top of the tree is built on the calling thread
// until a range holds at most `cut` primitives; those ranges are disjoint slices of the
// leaf order, so host threads build their subtrees independently, and the pieces are
// then emitted in the serial build's pre-order.  Every split sees exactly the range it
// sees in the serial build, so the tree is the same node for node.
#include "bvh_build.h"

#include <algorithm>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <functional>
#include <limits>
#include <memory>
#include <mutex>
#include <numeric>
#include <stdexcept>
#include <system_error>
#include <thread>

namespace gt {
namespace {

constexpr double kEps = 2.220446049250313e-16;
constexpr int kBuckets = 12;
constexpr uint32_t kParallelMin = 1u << 16; // primitives below which the build stays serial

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

// Runs f(part, lo, hi) over `parts` contiguous chunks of [0, n): chunk 0 on the calling
// thread, the others on their own (or on the calling thread if none can be started).
template <class F> void par_chunks(uint32_t n, uint32_t parts, F&& f) {
    const uint32_t step = (n + parts - 1) / parts;
    std::vector<std::thread> pool;
    for (uint32_t p = 1; p < parts; ++p) {
        const uint32_t lo = std::min(n, p * step), hi = std::min(n, lo + step);
        try {
            pool.emplace_back(std::ref(f), p, lo, hi);
        } catch (const std::system_error&) {
            f(p, lo, hi);
        }
    }
    f(0u, 0u, std::min(n, step));
    for (std::thread& th : pool) th.join();
}

// Ranges from this size up split with `par` threads: the scans whose results do not
// depend on the order of the elements (centroid bounds, bucket counts and boxes: min, max
// and integer sums) run in chunks; the swap partition stays one sequential pass.
constexpr uint32_t kParSplit = 1u << 17;

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
    uint32_t split(uint32_t* idx, uint32_t n, uint32_t leaf_size, uint32_t par = 1) const {
        if (n <= leaf_size) return 0;
        const uint32_t parts = par > 1 && n >= kParSplit ? par : 1u;
        double p0[3] = {cx[idx[0]], cy[idx[0]], cz[idx[0]]};
        Aabb cb = point_box(p0);
        if (parts > 1) {
            std::vector<Aabb> pb(parts, cb);
            par_chunks(n, parts, [&](uint32_t p, uint32_t lo, uint32_t hi) {
                Aabb r = cb;
                for (uint32_t i = lo; i < hi; ++i) {
                    double q[3] = {cx[idx[i]], cy[idx[i]], cz[idx[i]]};
                    r = grow(r, q);
                }
                pb[p] = r;
            });
            for (const Aabb& r : pb) cb = unite(cb, r);
        } else {
            for (uint32_t i = 1; i < n; ++i) {
                double p[3] = {cx[idx[i]], cy[idx[i]], cz[idx[i]]};
                cb = grow(cb, p);
            }
        }
        const int axis = widest(cb);
        const double lo = cb.lo[axis];
        const double extent = cb.hi[axis] - lo;
        if (extent <= kEps) return midpoint(idx, n, axis);
        uint32_t cnt[kBuckets] = {0};
        Aabb bb[kBuckets];
        std::vector<uint8_t> bk; // each position's bucket (parallel scans only)
        if (parts > 1) {
            bk.resize(n);
            std::vector<uint32_t> pc(size_t(parts) * kBuckets, 0u);
            std::vector<Aabb> pbb(size_t(parts) * kBuckets);
            par_chunks(n, parts, [&](uint32_t p, uint32_t lo_i, uint32_t hi_i) {
                uint32_t* c_ = pc.data() + size_t(p) * kBuckets;
                Aabb* b_ = pbb.data() + size_t(p) * kBuckets;
                for (uint32_t i = lo_i; i < hi_i; ++i) {
                    const uint32_t k = bucket_of((c(idx[i], axis) - lo) / extent);
                    bk[i] = uint8_t(k);
                    b_[k] = c_[k] ? unite(b_[k], box[idx[i]]) : box[idx[i]];
                    c_[k]++;
                }
            });
            for (uint32_t p = 0; p < parts; ++p)
                for (int k = 0; k < kBuckets; ++k) {
                    const uint32_t m = pc[size_t(p) * kBuckets + k];
                    if (!m) continue;
                    const Aabb& r = pbb[size_t(p) * kBuckets + k];
                    bb[k] = cnt[k] ? unite(bb[k], r) : r;
                    cnt[k] += m;
                }
        } else {
            for (uint32_t i = 0; i < n; ++i) {
                uint32_t k = bucket_of((c(idx[i], axis) - lo) / extent);
                bb[k] = cnt[k] ? unite(bb[k], box[idx[i]]) : box[idx[i]];
                cnt[k]++;
            }
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
        if (parts > 1) { // the same pass, each position's bucket carried with its element
            for (uint32_t next = 0; next < n; ++next) {
                if (bk[next] <= best) {
                    std::swap(idx[left], idx[next]);
                    std::swap(bk[left], bk[next]);
                    ++left;
                }
            }
        } else {
            for (uint32_t next = 0; next < n; ++next) {
                if (bucket_of((c(idx[next], axis) - lo) / extent) <= best) {
                    std::swap(idx[left], idx[next]);
                    ++left;
                }
            }
        }
        if (left == 0 || left == n) return midpoint(idx, n, axis);
        return left;
    }
};

// A range left to the parallel phase: the placeholder node standing for it, its slice of
// the leaf order and its depth.
struct Deferred {
    uint32_t node, first, count, depth;
};

// The explicit-stack build of order[first, first + count) from depth `depth`, its nodes
// numbered from 0 in `nodes` (child links local to `nodes`, leaf ranges absolute).  With
// `defer`, a range of at most `cut` primitives below the root becomes a placeholder leaf
// handed to it instead of being built.
void grow_tree(const Builder& b, const std::vector<Aabb>& box, std::vector<uint32_t>& order, uint32_t first,
               uint32_t count, uint32_t depth, uint32_t leaf_size, std::vector<BuildNode>& nodes, uint32_t& max_depth,
               const std::function<void(const Deferred&)>* defer = nullptr, uint32_t cut = 0, uint32_t par = 1) {
    struct Task {
        uint32_t first, count, parent, depth;
        bool is_right;
    };
    std::vector<Task> work;
    work.push_back({first, count, UINT32_MAX, depth, false});
    while (!work.empty()) {
        Task t = work.back();
        work.pop_back();
        const uint32_t id = uint32_t(nodes.size());
        if (t.parent != UINT32_MAX) {
            if (t.is_right) nodes[t.parent].right = id;
            else nodes[t.parent].left = id;
        }
        if (defer && t.parent != UINT32_MAX && t.count <= cut) {
            nodes.push_back(BuildNode{Aabb{}, t.first, t.count, 0, 0, true});
            (*defer)(Deferred{id, t.first, t.count, t.depth});
            continue;
        }
        Aabb nb = box[order[t.first]];
        if (par > 1 && t.count >= kParSplit) {
            std::vector<Aabb> pb(par, nb);
            par_chunks(t.count, par, [&](uint32_t p, uint32_t lo, uint32_t hi) {
                Aabb r = nb;
                for (uint32_t i = lo; i < hi; ++i) r = unite(r, box[order[t.first + i]]);
                pb[p] = r;
            });
            for (const Aabb& r : pb) nb = unite(nb, r);
        } else {
            for (uint32_t i = 1; i < t.count; ++i) nb = unite(nb, box[order[t.first + i]]);
        }
        nodes.push_back(BuildNode{nb, t.first, t.count, 0, 0, true});
        max_depth = std::max(max_depth, t.depth);
        const uint32_t left = b.split(order.data() + t.first, t.count, leaf_size, par);
        if (left == 0) continue;
        nodes[id].leaf = false;
        // Right task below left task on the stack: the left subtree is numbered first.
        work.push_back({t.first + left, t.count - left, id, t.depth + 1, true});
        work.push_back({t.first, left, id, t.depth + 1, false});
    }
}

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

void build_reference_bvh(const gt_primitive* prims, uint32_t count, uint32_t leaf_size, BuiltBvh& out,
                         uint32_t threads, uint32_t cut) {
    std::vector<Aabb> box(count);
    for (uint32_t i = 0; i < count; ++i) box[i] = geometry_aabb(prims[i].geometry);
    build_bvh_from_boxes(box.data(), count, leaf_size, out, threads, cut);
}

void build_bvh_from_boxes(const Aabb* boxes, uint32_t count, uint32_t leaf_size, BuiltBvh& out, uint32_t threads,
                          uint32_t cut) {
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
    if (threads == 0) threads = std::min(16u, std::max(1u, std::thread::hardware_concurrency()));
    if (cut == 0) cut = count >= kParallelMin ? std::max<uint32_t>(count / (threads * 4u), 4096u) : 0u;
    if (threads <= 1 || cut == 0 || count <= cut) { // serial
        out.nodes.reserve(size_t(count) * 2);
        grow_tree(b, box, out.order, 0, count, 1, leaf_size, out.nodes, out.max_depth);
        return;
    }
    // The top of the tree on this thread; each range of at most `cut` primitives it leaves
    // as a placeholder is queued at once, and host threads build its subtree from its own
    // root while the top goes on.
    struct Piece {
        Deferred d;
        std::vector<BuildNode> nodes;
        uint32_t depth = 0;
    };
    std::vector<BuildNode> top;
    uint32_t top_depth = 0;
    std::vector<std::unique_ptr<Piece>> pieces; // appended under `mu`
    std::deque<Piece*> queue;
    std::mutex mu;
    std::condition_variable cv;
    bool top_done = false;
    auto worker = [&]() {
        for (;;) {
            Piece* pc = nullptr;
            {
                std::unique_lock<std::mutex> lk(mu);
                cv.wait(lk, [&] { return !queue.empty() || top_done; });
                if (queue.empty()) return;
                pc = queue.front();
                queue.pop_front();
            }
            pc->nodes.reserve(size_t(pc->d.count) * 2);
            grow_tree(b, box, out.order, pc->d.first, pc->d.count, pc->d.depth, leaf_size, pc->nodes, pc->depth);
        }
    };
    std::vector<std::thread> pool;
    auto finish_top = [&]() { // wakes the threads to drain the queue and end
        {
            std::lock_guard<std::mutex> lk(mu);
            top_done = true;
        }
        cv.notify_all();
    };
    for (uint32_t k = 1; k < threads; ++k) {
        try {
            pool.emplace_back(worker);
        } catch (const std::system_error&) { // fewer threads: this one takes the rest
            break;
        }
    }
    const std::function<void(const Deferred&)> defer = [&](const Deferred& d) {
        std::lock_guard<std::mutex> lk(mu);
        pieces.push_back(std::make_unique<Piece>());
        pieces.back()->d = d;
        queue.push_back(pieces.back().get());
        cv.notify_one();
    };
    try {
        grow_tree(b, box, out.order, 0, count, 1, leaf_size, top, top_depth, &defer, cut, threads);
    } catch (...) {
        finish_top();
        for (std::thread& th : pool) th.join();
        throw;
    }
    finish_top();
    worker();
    for (std::thread& th : pool) th.join();
    // Emitted in pre-order, left subtree first, exactly as the serial build numbers them.
    std::vector<int32_t> piece_of(top.size(), -1);
    size_t total = top.size();
    out.max_depth = top_depth;
    for (size_t i = 0; i < pieces.size(); ++i) {
        piece_of[pieces[i]->d.node] = int32_t(i);
        total += pieces[i]->nodes.size();
        out.max_depth = std::max(out.max_depth, pieces[i]->depth);
    }
    out.nodes.clear();
    out.nodes.reserve(total);
    struct Ref {
        int32_t piece; // -1: the top
        uint32_t id, parent;
        bool is_right;
    };
    std::vector<Ref> stack;
    stack.push_back({-1, 0, UINT32_MAX, false});
    while (!stack.empty()) {
        Ref r = stack.back();
        stack.pop_back();
        if (r.piece < 0 && piece_of[r.id] >= 0) { // a placeholder: its subtree's root
            r.piece = piece_of[r.id];
            r.id = 0;
        }
        const BuildNode& src = r.piece < 0 ? top[r.id] : pieces[size_t(r.piece)]->nodes[r.id];
        const uint32_t id = uint32_t(out.nodes.size());
        out.nodes.push_back(src);
        if (r.parent != UINT32_MAX) {
            if (r.is_right) out.nodes[r.parent].right = id;
            else out.nodes[r.parent].left = id;
        }
        if (!src.leaf) {
            stack.push_back({r.piece, src.right, id, true});
            stack.push_back({r.piece, src.left, id, false});
        }
    }
}

} // namespace gt
