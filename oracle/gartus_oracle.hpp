// gartus_oracle.hpp — TEST INFRASTRUCTURE ONLY.
//
// A CPU restatement of the gartus path tracer's hot path (the Rust reference is not
// buildable here: no cargo/rustc).  It exists to check the GPU library, to pin its
// outputs against the reference's own known-answer tests, and to serve as the timed
// CPU baseline.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
// may load it; the product never links or calls it.
//
// Oracle<double> mirrors the reference's f64 arithmetic operation for operation:
// same evaluation order, no FMA contraction (build with -ffp-contract=off, no
// -ffast-math), glibc's libm for the transcendentals (which is what Rust's f64::sin
// etc. call on Linux).  Oracle<float> runs the same code in f32 to separate f32
// rounding effects from bugs.  Citations are file:line within the gartus crate.
#pragma once

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <memory>
#include <numeric>
#include <optional>
#include <stdexcept>
#include <thread>
#include <utility>
#include <vector>

#include "../include/gartus_gpu.h"

namespace oracle {

constexpr double kPi = 3.141592653589793;      // std::f64::consts::PI
constexpr double kTau = 6.283185307179586;     // std::f64::consts::TAU
constexpr double kEps = 2.220446049250313e-16; // f64::EPSILON
constexpr double kShadowAcne = 0.001;          // SHADOW_ACNE_EPSILON, raytracing.rs:146
constexpr double kShadowAcnePdf = 0.001;       // SHADOW_ACNE_PDF_EPSILON, object.rs:1163
constexpr double kTriHitEps = 1e-10;           // geometry.rs:10
constexpr double kTriBoundsEps = 1e-10;        // geometry.rs:9
constexpr double kQuadHitEps = 1e-8;           // geometry.rs:12
constexpr double kQuadBoundsEps = 1e-4;        // geometry.rs:11
constexpr double kGgxMinAlpha = 1.0e-4;        // sampling.rs:12
constexpr double kRrMin = 0.05, kRrMax = 0.95; // camera.rs:31-32
constexpr int kBvhBuckets = 12;                // bvh.rs:4

// Rust's f64::clamp: NaN passes through (core::f64::clamp).
template <class R> inline R rclamp(R x, R lo, R hi) {
    if (x < lo) x = lo;
    if (x > hi) x = hi;
    return x;
}
// Rust's f64::min / f64::max ignore a NaN operand like fmin/fmax.
template <class R> inline R rmin(R a, R b) { return std::fmin(a, b); }
template <class R> inline R rmax(R a, R b) { return std::fmax(a, b); }
// `x as usize` / `x as u32`: truncation toward zero, saturating, NaN -> 0.
inline uint64_t as_usize(double x) {
    if (!(x > 0.0)) return 0;
    if (x >= 18446744073709551615.0) return UINT64_MAX;
    return static_cast<uint64_t>(x);
}
inline uint32_t as_u32(double x) {
    if (!(x > 0.0)) return 0;
    if (x >= 4294967295.0) return UINT32_MAX;
    return static_cast<uint32_t>(x);
}
inline int32_t as_i32(double x) { // Rust `as i32`: saturating, NaN -> 0
    if (std::isnan(x)) return 0;
    if (x >= 2147483647.0) return INT32_MAX;
    if (x <= -2147483648.0) return INT32_MIN;
    return static_cast<int32_t>(x);
}
inline int64_t as_i64(double x) {
    if (std::isnan(x)) return 0;
    if (x >= 9223372036854775807.0) return INT64_MAX;
    if (x <= -9223372036854775808.0) return INT64_MIN;
    return static_cast<int64_t>(x);
}
// f64::rem_euclid (core): r = a % b; if r < 0 { r + |b| } else { r }.
template <class R> inline R rem_euclid(R a, R b) {
    R r = std::fmod(a, b);
    return r < R(0) ? r + std::fabs(b) : r;
}
// powi(x, 5) as LLVM expands a constant exponent: x * ((x*x)*(x*x)).
template <class R> inline R powi5(R x) {
    R x2 = x * x;
    R x4 = x2 * x2;
    return x * x4;
}

// ------------------------------------------------------------------ vector maths
// Vector/Point ops, gmath/vector.rs:121-173, 175-300.
template <class R> struct V3 {
    R x{0}, y{0}, z{0};
    V3() = default;
    V3(R a, R b, R c) : x(a), y(b), z(c) {}
    R operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template <class R> inline V3<R> operator+(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R> inline V3<R> operator-(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class R> inline V3<R> operator-(V3<R> a) { return {-a.x, -a.y, -a.z}; }
template <class R> inline V3<R> operator*(V3<R> a, R s) { return {a.x * s, a.y * s, a.z * s}; }
template <class R> inline V3<R> operator*(R s, V3<R> a) { return a * s; }
template <class R> inline V3<R> vdiv(V3<R> a, R s) { return {a.x / s, a.y / s, a.z / s}; } // vector.rs:255-262
template <class R> inline R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R> inline V3<R> cross(V3<R> a, V3<R> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class R> inline R length_squared(V3<R> a) { return dot(a, a); }
template <class R> inline R length(V3<R> a) { return std::sqrt(length_squared(a)); }
template <class R> inline V3<R> normalized(V3<R> a) { // vector.rs:147-155
    R len = length(a);
    if (len < R(kEps)) return V3<R>();
    return vdiv(a, len);
}
template <class R> inline V3<R> reflected(V3<R> v, V3<R> n) { // vector.rs:157-160
    R k = R(2) * dot(v, n);
    return v - n * k;
}
template <class R> inline V3<R> refracted(V3<R> v, V3<R> n, R eta) { // vector.rs:162-173
    R cos_theta = rmin(dot(-v, n), R(1));
    V3<R> perp = (v + n * cos_theta) * eta;
    R s = -std::sqrt(std::fabs(R(1) - length_squared(perp)));
    V3<R> par = n * s;
    return perp + par;
}
template <class R> inline bool finite3(V3<R> a) {
    return std::isfinite(a.x) && std::isfinite(a.y) && std::isfinite(a.z);
}
// LinearRgb ops (graphics/colors.rs:116-190).  Division multiplies by the reciprocal.
template <class R> inline V3<R> cmul(V3<R> a, V3<R> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class R> inline V3<R> cdiv(V3<R> a, R s) { return a * (R(1) / s); }
template <class R> inline R max_component(V3<R> a) { return rmax(rmax(a.x, a.y), a.z); }

template <class R> struct Ray {
    V3<R> o, d;
    R time{0};
    V3<R> at(R t) const { return o + d * t; } // ray.rs:108-111
};

// ------------------------------------------------------------------------- RNG
// SampleRng, gmath/random.rs:16-153 (SplitMix64).
struct SampleRng {
    uint64_t state;
    explicit SampleRng(uint64_t seed) : state(seed) {}
    uint64_t next_u64() { // random.rs:23-29
        state += 0x9e3779b97f4a7c15ULL;
        uint64_t v = state;
        v = (v ^ (v >> 30)) * 0xbf58476d1ce4e5b9ULL;
        v = (v ^ (v >> 27)) * 0x94d049bb133111ebULL;
        return v ^ (v >> 31);
    }
    template <class R> R random_double();
    template <class R> R random_range(R lo, R hi) { return lo + (hi - lo) * random_double<R>(); }
    template <class R> V3<R> random_vector() {
        R a = random_double<R>(), b = random_double<R>(), c = random_double<R>();
        return {a, b, c};
    }
    template <class R> V3<R> random_vector_range(R lo, R hi) {
        R a = random_range<R>(lo, hi), b = random_range<R>(lo, hi), c = random_range<R>(lo, hi);
        return {a, b, c};
    }
    template <class R> V3<R> random_unit_vector_spherical() { // random.rs:107-115
        R r1 = random_double<R>();
        R r2 = random_double<R>();
        R z = R(1) - R(2) * r2;
        R radius = std::sqrt(R(1) - z * z);
        R phi = R(kTau) * r1;
        return {std::cos(phi) * radius, std::sin(phi) * radius, z};
    }
    template <class R> V3<R> random_cosine_direction() { // random.rs:119-126
        R r1 = random_double<R>();
        R r2 = random_double<R>();
        R phi = R(kTau) * r1;
        R radius = std::sqrt(r2);
        return {std::cos(phi) * radius, std::sin(phi) * radius, std::sqrt(R(1) - r2)};
    }
    template <class R> V3<R> random_in_unit_disk() { // random.rs:141-152
        for (;;) {
            R a = random_range<R>(R(-1), R(1));
            R b = random_range<R>(R(-1), R(1));
            V3<R> p(a, b, R(0));
            if (length_squared(p) < R(1)) return p;
        }
    }
};
// random.rs:56-59: (u64 >> 11) * 2^-53.
template <> inline double SampleRng::random_double<double>() {
    return static_cast<double>(next_u64() >> 11) * (1.0 / 9007199254740992.0);
}
// f32 variant: the top 24 bits, (u64 >> 40) * 2^-24, exact and in [0, 1).
template <> inline float SampleRng::random_double<float>() {
    return static_cast<float>(next_u64() >> 40) * (1.0f / 16777216.0f);
}

// RayCamera::pixel_seed, graphics/camera.rs:1720-1727.
inline uint64_t pixel_seed(uint64_t seed, uint32_t x, uint32_t y) {
    uint64_t z = seed ^ (uint64_t(x) * 0x9E3779B97F4A7C15ULL) ^ (uint64_t(y) * 0xD1B54A32D192ED03ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

// The throughput mode's per-sample substream key (no reference counterpart): SplitMix64's
// output for state (s + 1) * golden gamma; sample s of pixel (x, y) starts its own stream
// at pixel_seed(seed, x, y) ^ sample_key(s).
inline uint64_t sample_key(uint64_t s) {
    uint64_t z = (s + 1) * 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

// -------------------------------------------------------------------- bounds
// Bounds3, gmath/polygon_matrix.rs:19-140 (always f64: the BVH is built in f64).
struct Bounds {
    double mn[3] = {0, 0, 0}, mx[3] = {0, 0, 0};
    static Bounds from_points(V3<double> a, V3<double> b) {
        Bounds r;
        for (int i = 0; i < 3; ++i) {
            r.mn[i] = std::fmin(a[i], b[i]);
            r.mx[i] = std::fmax(a[i], b[i]);
        }
        return r;
    }
    Bounds unite(const Bounds& o) const {
        Bounds r;
        for (int i = 0; i < 3; ++i) {
            r.mn[i] = std::fmin(mn[i], o.mn[i]);
            r.mx[i] = std::fmax(mx[i], o.mx[i]);
        }
        return r;
    }
    Bounds union_point(V3<double> p) const { return unite(from_points(p, p)); }
    Bounds padded(double eps) const { // polygon_matrix.rs:84-106
        eps = std::fabs(eps);
        double half = 0.5 * eps;
        Bounds r = *this;
        for (int i = 0; i < 3; ++i)
            if (std::fabs(r.mx[i] - r.mn[i]) < eps) {
                r.mn[i] -= half;
                r.mx[i] += half;
            }
        return r;
    }
    V3<double> centroid() const {
        return {0.5 * (mn[0] + mx[0]), 0.5 * (mn[1] + mx[1]), 0.5 * (mn[2] + mx[2])};
    }
    double surface_area() const { // polygon_matrix.rs:114-120
        double dx = std::fmax(mx[0] - mn[0], 0.0), dy = std::fmax(mx[1] - mn[1], 0.0),
               dz = std::fmax(mx[2] - mn[2], 0.0);
        return 2.0 * (dx * dy + dx * dz + dy * dz);
    }
    int largest_axis() const { // polygon_matrix.rs:122-134
        double dx = mx[0] - mn[0], dy = mx[1] - mn[1], dz = mx[2] - mn[2];
        if (dx >= dy && dx >= dz) return 0;
        if (dy >= dz) return 1;
        return 2;
    }
};

// ----------------------------------------------------------------- primitives
template <class R> inline V3<R> v3(const double* p) { return {R(p[0]), R(p[1]), R(p[2])}; }

template <class R> struct Prim {
    int kind = 0;
    uint32_t material = 0;
    V3<R> a, b, c; // sphere: centre; moving: c0, c1; triangle: p0, p1, p2; quad: corner, u, v
    R radius{0};
    // QuadGeometry::new derived fields (geometry.rs:271-301)
    V3<R> qnormal, qw;
    R qplane_d{0}, qarea_sq{0};

    static Prim from_geometry(const gt_geometry& g, uint32_t material) {
        Prim p;
        p.kind = int(g.kind);
        p.material = material;
        switch (g.kind) {
        case GT_GEOM_SPHERE:
            p.a = v3<R>(g.p);
            p.radius = rmax(R(g.p[3]), R(0)); // geometry.rs:425-430
            break;
        case GT_GEOM_MOVING_SPHERE:
            p.a = v3<R>(g.p);
            p.b = v3<R>(g.p + 3);
            p.radius = rmax(R(g.p[6]), R(0));
            break;
        case GT_GEOM_TRIANGLE:
            p.a = v3<R>(g.p);
            p.b = v3<R>(g.p + 3);
            p.c = v3<R>(g.p + 6);
            break;
        case GT_GEOM_QUAD: {
            p.a = v3<R>(g.p);
            p.b = v3<R>(g.p + 3);
            p.c = v3<R>(g.p + 6);
            V3<R> n = cross(p.b, p.c);
            p.qnormal = normalized(n);
            p.qplane_d = dot(p.qnormal, p.a);
            R nl2 = length_squared(n);
            p.qw = nl2 <= R(kEps) ? V3<R>() : vdiv(n, nl2);
            p.qarea_sq = length_squared(cross(p.b, p.c));
            break;
        }
        default:
            throw std::invalid_argument("unknown geometry kind");
        }
        return p;
    }
    V3<R> center_at(R t) const { return a + (b - a) * t; } // geometry.rs:510-513
};

// Bounding boxes in f64 (object.rs:1015-1036, geometry.rs:197-203, 355-362).
inline Bounds geometry_bounds(const gt_geometry& g) {
    switch (g.kind) {
    case GT_GEOM_SPHERE: {
        V3<double> c = v3<double>(g.p);
        double r = std::fmax(g.p[3], 0.0);
        V3<double> rv(r, r, r);
        return Bounds::from_points(c - rv, c + rv);
    }
    case GT_GEOM_MOVING_SPHERE: {
        V3<double> c0 = v3<double>(g.p), c1 = v3<double>(g.p + 3);
        double r = std::fmax(g.p[6], 0.0);
        V3<double> rv(r, r, r);
        return Bounds::from_points(c0 - rv, c0 + rv).unite(Bounds::from_points(c1 - rv, c1 + rv));
    }
    case GT_GEOM_TRIANGLE: {
        V3<double> p0 = v3<double>(g.p), p1 = v3<double>(g.p + 3), p2 = v3<double>(g.p + 6);
        return Bounds::from_points(p0, p0).union_point(p1).union_point(p2).padded(kTriBoundsEps);
    }
    case GT_GEOM_QUAD: {
        V3<double> c = v3<double>(g.p), u = v3<double>(g.p + 3), v = v3<double>(g.p + 6);
        V3<double> p1 = c + u, p2 = c + v, p3 = (c + u) + v;
        return Bounds::from_points(c, c).union_point(p1).union_point(p2).union_point(p3).padded(kQuadBoundsEps);
    }
    default:
        throw std::invalid_argument("unknown geometry kind");
    }
}

template <class R> struct Hit {
    V3<R> point, normal; // normal is oriented against the ray (SurfaceHit::with_uv)
    V3<R> shading;       // HitRecord::shading_normal (the normal unless a mesh bends it)
    R t{0}, u{0}, v{0};
    bool front_face = false;
    int prim = -1;
    uint32_t material = 0;
    R margin{1}; // decision trace only: min(|cos| of the ray against the normal, edge distance in (u, v))
};

// Decision trace (test infrastructure).  When g_trace is set, the renderer records every
// discrete decision of a pixel's samples in order: which primitive a ray hits, what a
// material does, the Schlick/TIR choice, Russian roulette, the mixture choice, the pdf
// cut-offs, the next-event shadow tests, texture cells, environment texel picks and each
// sample's end.  An f32 and an f64 run of one pixel are then compared decision by
// decision: the first pair that differs names the decision f32 rounding flipped.  `value`
// is the decision's margin where it has one (0 at the decision's boundary).
struct TraceEvent {
    int32_t type, outcome;
    double value;
};
enum : int32_t {
    TR_SAMPLE = 1, // outcome: 1 finite sample, 0 dropped; value the sample's channel sum
    TR_HIT,        // outcome: primitive (media -2 - k), -1 miss; value the hit's margin
    TR_SCATTER,    // outcome: SCATTER_* kind
    TR_DIELECTRIC, // outcome: 0 refract, 1 Schlick reflection, 2 total internal reflection
    TR_RR,         // outcome: 1 survives, 0 terminated, 2 black throughput; value u - p
    TR_MIXTURE,    // outcome: 1 light target, 0 material; value u - weight
    TR_PDF,        // outcome: 0 continuation pdf cut, 1 scattering pdf cut; value the pdf
    TR_NEE_AREA,   // outcome: primitive the shadow ray hits, -1 none, -3 sample rejected; value its margin
    TR_NEE_ENV,    // outcome: 1 unoccluded, 0 occluded, -3 sample rejected; value the occluder's margin
    TR_LIGHT_PICK, // outcome: target index; value the pick's remainder over the total weight
    TR_TEXTURE,    // outcome: checker parity; value the coordinates' distance to a cell boundary
    TR_ENV_PICK,   // outcome: environment texel; value the draw's distance to a CDF step over the total
    TR_THROUGHPUT, // not a decision (outcome 0): the path throughput's largest channel after a scatter
    TR_ADAPTIVE    // outcome: 1 the pixel stops, 0 it continues; value (error - threshold) / threshold
};
inline thread_local std::vector<TraceEvent>* g_trace = nullptr;
inline void trace_note(int32_t type, int32_t outcome, double value = 0.0) {
    if (g_trace) g_trace->push_back(TraceEvent{type, outcome, value});
}

// Origin of a ray leaving hit h in direction dir.  f64: the hit point, the reference's
// rule (Ray::new(rec.point, ...), camera.rs:1799-1861, material.rs:2087-2351).  f32: the
// point moved off the surface by 2^-19 (max|p| + 1) along the oriented normal, on the side
// the ray leaves to, as the f32 device path does, so that the f32 oracle restates the f32
// device algorithm (f32 hit points are too coarse for t_min = 0.001 at grazing angles).
template <class R> inline V3<R> spawn_origin(const Hit<R>& h, V3<R> dir);
template <> inline V3<double> spawn_origin<double>(const Hit<double>& h, V3<double>) { return h.point; }
template <> inline V3<float> spawn_origin<float>(const Hit<float>& h, V3<float> dir) {
    const float m = std::fmax(std::fmax(std::fabs(h.point.x), std::fabs(h.point.y)), std::fabs(h.point.z)) + 1.0f;
    const float e = dot(dir, h.normal) >= 0.0f ? m * 0x1p-19f : -m * 0x1p-19f;
    return h.point + h.normal * e;
}

// f32 roots of hit_sphere_in_interval with less rounding, as the f32 device path computes
// them.  The discriminant is a (r^2 - |l|^2) with l = oc - (h / a) d, the centre's offset
// from the ray's closest approach (Haines, Guenther, Akenine-Moeller, "Precision
// Improvements for Ray/Sphere Intersection", Ray Tracing Gems, 2019): h^2 - a c cancels
// for a sphere small against its distance.  c = |oc|^2 - r^2 keeps its products' rounding
// errors (two-product by fused multiply-add) and its sums' (two-sum), so it stays accurate
// near a large sphere, and each root comes from the cancellation-free form
// (q = h + sign(h) sqrt(disc): the roots are c / q and q / a).  In exact arithmetic these
// are the reference's roots, tested in the reference's order.
inline float two_sum_err(float a, float b, float s) {
    const float bb = s - a;
    return (a - (s - bb)) + (b - bb);
}

// Interval::surrounds (object.rs:56-58).
template <class R> inline bool surrounds(R lo, R hi, R x) { return lo < x && x < hi; }

inline bool sphere_roots_f32(V3<float> center, float radius, const Ray<float>& ray, float& first, float& second) {
    const V3<float> oc = center - ray.o;
    const float a = length_squared(ray.d);
    if (a <= float(kEps)) return false;
    const float h = dot(ray.d, oc);
    const float tc = h / a;
    const V3<float> l{std::fma(-ray.d.x, tc, oc.x), std::fma(-ray.d.y, tc, oc.y), std::fma(-ray.d.z, tc, oc.z)};
    const float disc_a = std::fma(radius, radius, -length_squared(l));
    if (disc_a < 0.0f) return false;
    const float px = oc.x * oc.x, py = oc.y * oc.y, pz = oc.z * oc.z, rr = radius * radius;
    const float e = (std::fma(oc.x, oc.x, -px) + std::fma(oc.y, oc.y, -py)) + (std::fma(oc.z, oc.z, -pz) -
                                                                               std::fma(radius, radius, -rr));
    const float s1 = px + py, s2 = s1 + pz, s3 = s2 - rr;
    const float c = s3 + (((two_sum_err(px, py, s1) + two_sum_err(s1, pz, s2)) + two_sum_err(s2, -rr, s3)) + e);
    const float sq = std::sqrt(a * disc_a);
    const float q = h >= 0.0f ? h + sq : h - sq;
    if (q == 0.0f) {
        first = second = 0.0f;
    } else if (h >= 0.0f) {
        first = c / q;
        second = q / a;
    } else {
        first = q / a;
        second = c / q;
    }
    return true;
}

// hit_sphere_in_interval, object.rs:986-1013.
template <class R> inline bool hit_sphere_root(V3<R> center, R radius, const Ray<R>& ray, R tmin, R tmax, R& root) {
    if constexpr (sizeof(R) == 4) {
        float first, second;
        if (!sphere_roots_f32(center, radius, ray, first, second)) return false;
        if (surrounds(tmin, tmax, first)) {
            root = first;
            return true;
        }
        if (surrounds(tmin, tmax, second)) {
            root = second;
            return true;
        }
        return false;
    }
    V3<R> oc = center - ray.o;
    R a = length_squared(ray.d);
    if (a <= R(kEps)) return false;
    R h = dot(ray.d, oc);
    R c = length_squared(oc) - radius * radius;
    R disc = h * h - a * c;
    if (disc < R(0)) return false;
    R sq = std::sqrt(disc);
    R first = (h - sq) / a;
    if (surrounds(tmin, tmax, first)) {
        root = first;
        return true;
    }
    R second = (h + sq) / a;
    if (surrounds(tmin, tmax, second)) {
        root = second;
        return true;
    }
    return false;
}

// sphere_uv, object.rs:1038-1042.
template <class R> inline void sphere_uv(V3<R> p, R& u, R& v) {
    R theta = std::acos(-p.y);
    R phi = std::atan2(-p.z, p.x) + R(kPi);
    u = phi / (R(2) * R(kPi));
    v = theta / R(kPi);
}

template <class R> inline void set_face(Hit<R>& h, const Ray<R>& ray, V3<R> outward) { // object.rs:127-149
    h.front_face = dot(ray.d, outward) < R(0);
    h.normal = h.front_face ? outward : -outward;
    h.shading = h.normal;
}

// MovingSphereGeometry::outward_normal_at / SphereGeometry (geometry.rs:476-484, 530-538).
template <class R> inline V3<R> sphere_outward(V3<R> point, V3<R> center, R radius) {
    V3<R> out = point - center;
    if (std::fabs(radius) <= R(kEps)) return normalized(out);
    return vdiv(out, radius);
}

// TriangleGeometry::hit_ray (geometry.rs:239-265).
template <class R> inline bool triangle_hit_ray(V3<R> p0, V3<R> p1, V3<R> p2, const Ray<R>& ray, R tmin, R tmax,
                                                R& t, R& u, R& v) {
    V3<R> e1 = p1 - p0, e2 = p2 - p0;
    V3<R> pvec = cross(ray.d, e2);
    R det = dot(e1, pvec);
    if (std::fabs(det) < R(kTriHitEps)) return false;
    R inv_det = R(1) / det;
    V3<R> tvec = ray.o - p0;
    u = dot(tvec, pvec) * inv_det;
    if (!(u >= R(0) && u <= R(1))) return false;
    V3<R> qvec = cross(tvec, e1);
    v = dot(ray.d, qvec) * inv_det;
    if (v < R(0) || u + v > R(1)) return false;
    t = dot(e2, qvec) * inv_det;
    return tmin < t && t < tmax;
}

// QuadGeometry::hit_ray (geometry.rs:394-415).
template <class R> inline bool quad_hit_ray(const Prim<R>& q, const Ray<R>& ray, R tmin, R tmax, R& t, R& u, R& v) {
    if (q.qarea_sq <= R(kEps)) return false;
    R denom = dot(q.qnormal, ray.d);
    if (std::fabs(denom) < R(kQuadHitEps)) return false;
    t = (q.qplane_d - dot(q.qnormal, ray.o)) / denom;
    if (!(tmin < t && t < tmax)) return false;
    V3<R> planar = ray.at(t) - q.a; // plane_coordinates, geometry.rs:385-392
    u = dot(q.qw, cross(planar, q.c));
    v = dot(q.qw, cross(q.b, planar));
    if (!(u >= R(0) && u <= R(1)) || !(v >= R(0) && v <= R(1))) return false;
    return true;
}

// RayGeometry::intersect (object.rs:338-346 and the Intersect impls 160-234).
template <class R> inline bool intersect(const Prim<R>& p, const Ray<R>& ray, R tmin, R tmax, Hit<R>& h) {
    switch (p.kind) {
    case GT_GEOM_SPHERE:
    case GT_GEOM_MOVING_SPHERE: {
        V3<R> center = p.kind == GT_GEOM_SPHERE ? p.a : p.center_at(ray.time);
        R root;
        if (!hit_sphere_root(center, p.radius, ray, tmin, tmax, root)) return false;
        V3<R> point = ray.at(root);
        V3<R> center2 = p.kind == GT_GEOM_SPHERE ? p.a : p.center_at(ray.time);
        V3<R> outward = sphere_outward(point, center2, p.radius);
        sphere_uv(outward, h.u, h.v);
        h.point = point;
        h.t = root;
        set_face(h, ray, outward);
        if (g_trace) h.margin = std::fabs(dot(normalized(ray.d), outward));
        return true;
    }
    case GT_GEOM_TRIANGLE: {
        R t, u, v;
        if (!triangle_hit_ray(p.a, p.b, p.c, ray, tmin, tmax, t, u, v)) return false;
        V3<R> n = normalized(cross(p.b - p.a, p.c - p.a));
        if (length_squared(n) <= R(kEps)) return false;
        h.point = ray.at(t);
        h.t = t;
        h.u = u;
        h.v = v;
        set_face(h, ray, n);
        if (g_trace)
            h.margin = rmin(std::fabs(dot(normalized(ray.d), normalized(n))), rmin(rmin(u, v), R(1) - u - v));
        return true;
    }
    case GT_GEOM_QUAD: {
        R t, u, v;
        if (!quad_hit_ray(p, ray, tmin, tmax, t, u, v)) return false;
        V3<R> n = p.qnormal;
        if (length_squared(n) <= R(kEps)) return false;
        h.point = ray.at(t);
        h.t = t;
        h.u = u;
        h.v = v;
        set_face(h, ray, n);
        if (g_trace)
            h.margin = rmin(std::fabs(dot(normalized(ray.d), normalized(n))),
                            rmin(rmin(u, R(1) - u), rmin(v, R(1) - v)));
        return true;
    }
    }
    return false;
}

// ------------------------------------------------------------------- media
// ConstantMedium (raytracing/volume/medium.rs) around a Sphere or a box_object
// (object.rs:930-976), wrapped as Translate(RotateY(shape)) (instance.rs).
template <class R> struct Medium {
    std::vector<Prim<R>> parts; // the sphere, or the box's six sides in box_object's order
    uint32_t material = 0;
    bool rotate = false, translate = false;
    R sin_theta{0}, cos_theta{1};
    V3<R> offset;
    R neg_inv_density{-1};

    static Medium from_desc(const gt_medium& m) {
        Medium md;
        md.material = m.material;
        md.rotate = (m.transform & GT_MEDIUM_ROTATE_Y) != 0;
        md.translate = (m.transform & GT_MEDIUM_TRANSLATE) != 0;
        const double radians = m.rotate_y * kPi / 180.0; // degrees_to_radians, raytracing.rs:150-152
        md.sin_theta = R(std::sin(radians));
        md.cos_theta = R(std::cos(radians));
        md.offset = v3<R>(m.translate);
        md.neg_inv_density = R(-1.0 / m.density);
        auto quad = [&](double qx, double qy, double qz, const double* u, const double* v) {
            gt_geometry g{};
            g.kind = GT_GEOM_QUAD;
            g.p[0] = qx, g.p[1] = qy, g.p[2] = qz;
            for (int k = 0; k < 3; ++k) g.p[3 + k] = u[k], g.p[6 + k] = v[k];
            md.parts.push_back(Prim<R>::from_geometry(g, m.material));
        };
        if (m.shape == GT_MEDIUM_SPHERE) {
            gt_geometry g{};
            g.kind = GT_GEOM_SPHERE;
            for (int k = 0; k < 4; ++k) g.p[k] = m.p[k];
            md.parts.push_back(Prim<R>::from_geometry(g, m.material));
        } else {
            double lo[3], hi[3];
            for (int k = 0; k < 3; ++k) {
                lo[k] = std::fmin(m.p[k], m.p[3 + k]);
                hi[k] = std::fmax(m.p[k], m.p[3 + k]);
            }
            const double dx[3] = {hi[0] - lo[0], 0, 0}, dy[3] = {0, hi[1] - lo[1], 0}, dz[3] = {0, 0, hi[2] - lo[2]};
            const double mdx[3] = {-dx[0], -dx[1], -dx[2]}, mdz[3] = {-dz[0], -dz[1], -dz[2]};
            quad(lo[0], lo[1], hi[2], dx, dy);  // front
            quad(hi[0], lo[1], hi[2], mdz, dy); // right
            quad(hi[0], lo[1], lo[2], mdx, dy); // back
            quad(lo[0], lo[1], lo[2], dz, dy);  // left
            quad(lo[0], hi[1], hi[2], dx, mdz); // top
            quad(lo[0], lo[1], lo[2], dx, dz);  // bottom
        }
        return md;
    }

    // The boundary's closest hit in (tmin, tmax), through Translate then RotateY.
    bool boundary(const Ray<R>& world, R tmin, R tmax, R& t) const {
        Ray<R> r = world;
        if (translate) r.o = r.o - offset;
        if (rotate) { // rotate_y_point_inverse / rotate_y_vector_inverse
            r.o = V3<R>(cos_theta * r.o.x - sin_theta * r.o.z, r.o.y, sin_theta * r.o.x + cos_theta * r.o.z);
            r.d = V3<R>(cos_theta * r.d.x - sin_theta * r.d.z, r.d.y, sin_theta * r.d.x + cos_theta * r.d.z);
        }
        bool any = false;
        for (const Prim<R>& p : parts) { // HittableList: each later side must be closer
            Hit<R> h;
            if (intersect(p, r, tmin, tmax, h)) {
                tmax = h.t;
                t = h.t;
                any = true;
            }
        }
        return any;
    }

    // ConstantMedium::hit_with_rng with boundary_interval (medium.rs:119-187).
    bool hit(const Ray<R>& ray, R tmin, R tmax, SampleRng& rng, R& t) const {
        const R inf = std::numeric_limits<R>::infinity();
        R entry, exit;
        if (!boundary(ray, -inf, inf, entry)) return false;
        entry = std::fmax(entry, tmin);
        if (!boundary(ray, entry + R(0.0001), inf, exit)) return false;
        exit = std::fmin(exit, tmax);
        if (entry >= exit) return false;
        entry = std::fmax(entry, R(0));
        const R len = std::sqrt(length_squared(ray.d));
        if (len <= R(kEps)) return false;
        const R inside = (exit - entry) * len;
        const R sample = std::fmax(rng.random_double<R>(), std::numeric_limits<R>::min());
        const R distance = neg_inv_density * std::log(sample);
        if (distance > inside) return false;
        t = entry + distance / len;
        return true;
    }
};

// ----------------------------------------------------------------------- BVH
struct BvhStats { // BvhTraversalStats, bvh.rs:9-52
    uint64_t rays = 0, node_bounds_tests = 0, node_bounds_hits = 0, leaf_visits = 0, primitive_candidates = 0,
             leaf_hit_results = 0, max_stack_depth = 0;
    void merge(const BvhStats& o) {
        rays += o.rays;
        node_bounds_tests += o.node_bounds_tests;
        node_bounds_hits += o.node_bounds_hits;
        leaf_visits += o.leaf_visits;
        primitive_candidates += o.primitive_candidates;
        leaf_hit_results += o.leaf_hit_results;
        max_stack_depth = std::max(max_stack_depth, o.max_stack_depth);
    }
};

struct BvhNode {
    Bounds bounds;
    bool leaf;
    uint32_t a, b; // leaf: first, count; internal: left, right
};

// FlatBvh::build / build_range / split_bvh_indices (bvh.rs:233-288, 430-522).
struct FlatBvh {
    std::vector<BvhNode> nodes;
    std::vector<uint32_t> indices;
    std::vector<Bounds> prim_bounds;
    std::vector<V3<double>> centroids;

    void build(const std::vector<Bounds>& bounds, uint32_t leaf_size) {
        nodes.clear();
        prim_bounds = bounds;
        centroids.resize(bounds.size());
        for (size_t i = 0; i < bounds.size(); ++i) centroids[i] = bounds[i].centroid();
        indices.resize(bounds.size());
        std::iota(indices.begin(), indices.end(), 0u);
        if (bounds.empty()) return;
        nodes.reserve(bounds.size() * 2);
        build_range(leaf_size, 0, uint32_t(bounds.size()));
    }

    uint32_t build_range(uint32_t leaf_size, uint32_t first, uint32_t count) {
        Bounds b = prim_bounds[indices[first]];
        for (uint32_t i = 1; i < count; ++i) b = b.unite(prim_bounds[indices[first + i]]);
        uint32_t node_index = uint32_t(nodes.size());
        nodes.push_back(BvhNode{b, true, first, count});
        uint32_t left_count;
        if (split(indices.data() + first, count, leaf_size, left_count)) {
            uint32_t right_count = count - left_count;
            uint32_t l = build_range(leaf_size, first, left_count);
            uint32_t r = build_range(leaf_size, first + left_count, right_count);
            nodes[node_index].leaf = false;
            nodes[node_index].a = l;
            nodes[node_index].b = r;
        }
        return node_index;
    }

    static uint32_t bucket_index(double offset) { // bvh.rs:498-501
        uint64_t b = as_usize(offset * 12.0);
        return uint32_t(std::min<uint64_t>(b, kBvhBuckets - 1));
    }

    uint32_t midpoint_split(uint32_t* idx, uint32_t n, int axis) { // bvh.rs:508-522
        std::stable_sort(idx, idx + n, [&](uint32_t l, uint32_t r) {
            double la = centroids[l][axis], ra = centroids[r][axis];
            if (la < ra) return true;
            if (la > ra) return false;
            return l < r;
        });
        return n / 2;
    }

    bool split(uint32_t* idx, uint32_t n, uint32_t leaf_size, uint32_t& left_count) {
        if (n <= leaf_size) return false;
        Bounds cb = Bounds::from_points(centroids[idx[0]], centroids[idx[0]]);
        for (uint32_t i = 1; i < n; ++i) cb = cb.union_point(centroids[idx[i]]);
        int axis = cb.largest_axis();
        double extent = cb.mx[axis] - cb.mn[axis];
        if (extent <= kEps) {
            left_count = midpoint_split(idx, n, axis);
            return true;
        }
        uint32_t counts[kBvhBuckets] = {0};
        bool has[kBvhBuckets] = {false};
        Bounds bb[kBvhBuckets];
        for (uint32_t i = 0; i < n; ++i) {
            double off = (centroids[idx[i]][axis] - cb.mn[axis]) / extent;
            uint32_t k = bucket_index(off);
            counts[k]++;
            bb[k] = has[k] ? bb[k].unite(prim_bounds[idx[i]]) : prim_bounds[idx[i]];
            has[k] = true;
        }
        uint32_t best_split = 0;
        double best_cost = std::numeric_limits<double>::infinity();
        for (int s = 0; s < kBvhBuckets - 1; ++s) {
            uint32_t lc = 0, rc = 0;
            bool lh = false, rh = false;
            Bounds lb, rb;
            for (int k = 0; k <= s; ++k) {
                lc += counts[k];
                if (has[k]) {
                    lb = lh ? lb.unite(bb[k]) : bb[k];
                    lh = true;
                }
            }
            for (int k = s + 1; k < kBvhBuckets; ++k) {
                rc += counts[k];
                if (has[k]) {
                    rb = rh ? rb.unite(bb[k]) : bb[k];
                    rh = true;
                }
            }
            if (lc == 0 || rc == 0) continue;
            double cost = lb.surface_area() * double(lc) + rb.surface_area() * double(rc);
            if (cost < best_cost) {
                best_cost = cost;
                best_split = uint32_t(s);
            }
        }
        if (!std::isfinite(best_cost)) {
            left_count = midpoint_split(idx, n, axis);
            return true;
        }
        uint32_t lc = 0;
        for (uint32_t next = 0; next < n; ++next) {
            uint32_t index = idx[next];
            double off = (centroids[index][axis] - cb.mn[axis]) / extent;
            if (bucket_index(off) <= best_split) {
                std::swap(idx[lc], idx[next]);
                ++lc;
            }
        }
        if (lc == 0 || lc == n) {
            left_count = midpoint_split(idx, n, axis);
            return true;
        }
        left_count = lc;
        return true;
    }
};

// RayTraversal::new / hit_bounds (bvh.rs:99-146).
template <class R> struct RayTraversal {
    R o[3], inv[3];
    bool par[3];
    explicit RayTraversal(const Ray<R>& ray) {
        R d[3] = {ray.d.x, ray.d.y, ray.d.z};
        R org[3] = {ray.o.x, ray.o.y, ray.o.z};
        for (int i = 0; i < 3; ++i) {
            o[i] = org[i];
            par[i] = std::fabs(d[i]) <= R(kEps);
            inv[i] = par[i] ? R(0) : R(1) / d[i];
        }
    }
    bool hit_bounds(const Bounds& b, R tmin, R tmax, R& entry_out) const {
        R entry = tmin, exit = tmax;
        for (int axis = 0; axis < 3; ++axis) {
            R mn = R(b.mn[axis]), mx = R(b.mx[axis]);
            if (par[axis]) {
                if (o[axis] < mn || o[axis] > mx) return false;
                continue;
            }
            R t0 = (mn - o[axis]) * inv[axis];
            R t1 = (mx - o[axis]) * inv[axis];
            if (inv[axis] < R(0)) std::swap(t0, t1);
            entry = rmax(entry, t0);
            exit = rmin(exit, t1);
            if (exit <= entry) return false;
        }
        entry_out = entry;
        return true;
    }
};

// ------------------------------------------------------------------ Perlin noise
// Perlin (gmath/perlin.rs:8-137).  The tables are made in f64 as in the reference and
// read as R when evaluated.
struct Perlin {
    double grad[256][3];
    int perm[3][256];
    explicit Perlin(uint64_t seed = 1) { // Perlin::new, perlin.rs:19-31
        SampleRng rng(seed);
        for (auto& g : grad) { // random_unit_vector = the spherical form, random.rs:88-91
            V3<double> v = rng.random_unit_vector_spherical<double>();
            g[0] = v.x;
            g[1] = v.y;
            g[2] = v.z;
        }
        for (auto& p : perm) { // generate_permutation / permute, perlin.rs:83-101
            for (int i = 0; i < 256; ++i) p[i] = i;
            for (int i = 255; i > 0; --i) {
                int target = int(rng.random_double<double>() * (double(i) + 1.0));
                std::swap(p[i], p[target]);
            }
        }
    }
    template <class R> R noise(V3<R> p) const { // perlin.rs:36-58, perlin_interp 106-124
        R fx = p.x - std::floor(p.x), fy = p.y - std::floor(p.y), fz = p.z - std::floor(p.z);
        int32_t bx = as_i32(double(std::floor(p.x))), by = as_i32(double(std::floor(p.y))),
                bz = as_i32(double(std::floor(p.z)));
        R uu = fx * fx * (R(3) - R(2) * fx);
        R vv = fy * fy * (R(3) - R(2) * fy);
        R ww = fz * fz * (R(3) - R(2) * fz);
        R accum = R(0);
        for (int ox = 0; ox < 2; ++ox)
            for (int oy = 0; oy < 2; ++oy)
                for (int oz = 0; oz < 2; ++oz) {
                    // (base + offset) & 255 on i32 (wrapping add in release builds)
                    auto idx = [](int32_t b, int o) { return int((uint32_t(b) + uint32_t(o)) & 255u); };
                    int gi = perm[0][idx(bx, ox)] ^ perm[1][idx(by, oy)] ^ perm[2][idx(bz, oz)];
                    R gx = R(grad[gi][0]), gy = R(grad[gi][1]), gz = R(grad[gi][2]);
                    R wx = fx - R(ox), wy = fy - R(oy), wz = fz - R(oz);
                    R dot = gx * wx + gy * wy + gz * wz;
                    R bxw = ox ? uu : R(1) - uu; // blend, perlin.rs:130-136
                    R byw = oy ? vv : R(1) - vv;
                    R bzw = oz ? ww : R(1) - ww;
                    accum = accum + bxw * byw * bzw * dot;
                }
        return accum;
    }
    template <class R> R turbulence(V3<R> p, int depth) const { // perlin.rs:61-74
        R accum = R(0), weight = R(1);
        for (int k = 0; k < depth; ++k) {
            accum = accum + weight * noise(p);
            weight = weight * R(0.5);
            p = V3<R>{p.x * R(2), p.y * R(2), p.z * R(2)};
        }
        return std::fabs(accum);
    }
};

// ------------------------------------------------------------------ materials
// A bitmap texture (graphics/texture.rs Texture) and Texture::sample (texture.rs:202-208):
// 8-bit texels, nearest or bilinear, clamp or repeat per axis, t = 1 at the top row.
struct ImageData {
    uint32_t w = 0, h = 0;
    std::vector<uint8_t> rgb;
    int filter = GT_FILTER_NEAREST, wrap_s = GT_WRAP_CLAMP, wrap_t = GT_WRAP_CLAMP;

    // f64::rem_euclid(value, 1.0)
    static double rem1(double x) {
        double r = std::fmod(x, 1.0);
        return r < 0.0 ? r + 1.0 : r;
    }
    static double wrap(double x, int mode) { return mode == GT_WRAP_REPEAT ? rem1(x) : rclamp(x, 0.0, 1.0); }
    // Rust `f64 as u32` for the finite, non-negative values here (saturating).
    static uint32_t to_u32(double x) { return x <= 0.0 ? 0u : (x >= 4294967295.0 ? 4294967295u : uint32_t(x)); }
    const uint8_t* at(uint32_t x, uint32_t y) const { return rgb.data() + (size_t(y) * w + x) * 3; }
    // linear_axis (texture.rs:737-752): (coordinate, low texel, high texel)
    void axis(double value, uint32_t size, int mode, double& coord, uint32_t& lo, uint32_t& hi) const {
        if (mode == GT_WRAP_CLAMP) {
            coord = rclamp(value, 0.0, 1.0) * double(size - 1);
            lo = to_u32(std::floor(coord));
            hi = std::min(lo + 1, size - 1);
        } else {
            coord = rem1(value) * double(size);
            lo = std::min(to_u32(std::floor(coord)), size - 1);
            hi = lo + 1 == size ? 0 : lo + 1;
        }
    }
    // Rgb::lerp (colors.rs:525-537): per channel round(a + (b - a) t) as u8, t clamped.
    static void lerp(const uint8_t* a, const uint8_t* b, double t, uint8_t* out) {
        t = rclamp(t, 0.0, 1.0);
        for (int k = 0; k < 3; ++k) {
            const double v = std::round(double(a[k]) + double(int(b[k]) - int(a[k])) * t);
            out[k] = uint8_t(v <= 0.0 ? 0 : (v >= 255.0 ? 255 : v));
        }
    }
    // NormalMap::sample_tangent_normal (raytracing/texture.rs:254-275).
    template <class R> V3<R> tangent_normal(R u, R v, R strength, bool neg_y) const {
        if (w == 0 || h == 0) return V3<R>(0, 0, 1);
        uint8_t c[3];
        rgb8(double(u), double(v), c);
        auto dec = [](uint8_t ch) { return R(2.0 * (double(ch) / 255.0) - 1.0); };
        const R green = neg_y ? -dec(c[1]) : dec(c[1]);
        const V3<R> n(strength * dec(c[0]), strength * green, std::fmax(dec(c[2]), R(0)));
        return length_squared(n) <= R(kEps) ? V3<R>(0, 0, 1) : normalized(n);
    }
    // Texture::sample (graphics/texture.rs:202-208) of a non-empty bitmap: the u8 texel.
    void rgb8(double s, double t, uint8_t* c) const {
        c[0] = c[1] = c[2] = 0;
        if (!(std::isfinite(s) && std::isfinite(t))) return;
        if (filter == GT_FILTER_NEAREST) { // sample_nearest, texture.rs:716-722
            const double ws = wrap(s, wrap_s), wt = wrap(t, wrap_t);
            const uint32_t x = to_u32(std::round(ws * double(w - 1)));
            const uint32_t y = to_u32(std::round((1.0 - wt) * double(h - 1)));
            std::memcpy(c, at(x, y), 3);
        } else { // sample_linear, texture.rs:724-735
            double x, y;
            uint32_t x0, x1, y0, y1;
            axis(s, w, wrap_s, x, x0, x1);
            axis(1.0 - t, h, wrap_t, y, y0, y1);
            const double tx = x - double(x0), ty = y - double(y0);
            uint8_t top[3], bottom[3];
            lerp(at(x0, y0), at(x1, y0), tx, top);
            lerp(at(x0, y1), at(x1, y1), tx, bottom);
            lerp(top, bottom, ty, c);
        }
    }
    // ImageTexture::sample_linear (raytracing/texture.rs:148-155) then from_rgb_srgb.
    template <class R> V3<R> sample(R u, R v) const {
        uint8_t c[3] = {0, 0, 0};
        if (w == 0 || h == 0) {
            c[1] = c[2] = 255; // Rgb::CYAN
        } else if (std::isfinite(double(u)) && std::isfinite(double(v))) {
            const double s = double(u), t = double(v);
            if (filter == GT_FILTER_NEAREST) { // sample_nearest, texture.rs:716-722
                const double ws = wrap(s, wrap_s), wt = wrap(t, wrap_t);
                const uint32_t x = to_u32(std::round(ws * double(w - 1)));
                const uint32_t y = to_u32(std::round((1.0 - wt) * double(h - 1)));
                std::memcpy(c, at(x, y), 3);
            } else { // sample_linear, texture.rs:724-735
                double x, y;
                uint32_t x0, x1, y0, y1;
                axis(s, w, wrap_s, x, x0, x1);
                axis(1.0 - t, h, wrap_t, y, y0, y1);
                const double tx = x - double(x0), ty = y - double(y0);
                uint8_t top[3], bottom[3];
                lerp(at(x0, y0), at(x1, y0), tx, top);
                lerp(at(x0, y1), at(x1, y1), tx, bottom);
                lerp(top, bottom, ty, c);
            }
        }
        auto dec = [](uint8_t ch) { // LinearRgb::from_rgb_srgb, colors.rs:78-84
            const double x = double(ch) / 255.0;
            return R(x * x);
        };
        return V3<R>(dec(c[0]), dec(c[1]), dec(c[2]));
    }
};

template <class R> struct Material {
    int kind = GT_MAT_LAMBERTIAN;
    int texture = GT_TEX_SOLID;
    V3<R> color;
    R param{0};
    R tex_inv_scale{1};
    V3<R> even, odd;
    R noise_scale{1};
    int noise_variant = 0, noise_depth = 0;
    std::shared_ptr<Perlin> perlin;
    std::shared_ptr<const ImageData> image;
    std::shared_ptr<const ImageData> normal_map; // Lambertian / GgxMicrofacet::with_shared_normal_map
    R normal_strength{1};
    bool normal_neg_y = false;
    static Material from_desc(const gt_material& m) {
        Material r;
        r.kind = int(m.kind);
        r.texture = int(m.texture_kind);
        r.color = v3<R>(m.color);
        r.param = R(m.param);
        if (m.kind == GT_MAT_GGX || m.kind == GT_MAT_METAL) r.param = rclamp(R(m.param), R(0), R(1)); // material.rs:1386, 1972
        if (m.texture_kind == GT_TEX_CHECKER) { // CheckerTexture::new, raytracing/texture.rs:71-82
            double sc = m.tex[0];
            r.tex_inv_scale = R((std::isfinite(sc) && std::fabs(sc) > kEps) ? 1.0 / std::fabs(sc) : 1.0);
            r.even = v3<R>(m.tex + 1);
            r.odd = v3<R>(m.tex + 4);
        }
        if (m.texture_kind == GT_TEX_NOISE) { // NoiseTexture::{new, turbulence, marble}, texture.rs:293-322
            r.noise_scale = R(m.tex[0]);
            r.noise_variant = int(m.tex[1]);
            r.noise_depth = int(m.tex[2]);
            r.perlin = std::make_shared<Perlin>(uint64_t(m.tex[3]) | (uint64_t(m.tex[4]) << 32));
        }
        return r;
    }
    // MaterialColorSource::sample (material.rs:307-314): SolidColor or CheckerTexture
    // (raytracing/texture.rs:97-108: parity of floor(p * inv_scale) summed over axes).
    V3<R> sample(const Hit<R>& h) const {
        if (texture == GT_TEX_NOISE) { // NoiseTexture::sample_linear, texture.rs:337-352
            V3<R> q{h.point.x * noise_scale, h.point.y * noise_scale, h.point.z * noise_scale};
            R i;
            if (noise_variant == GT_NOISE_TURBULENCE) i = perlin->turbulence(q, noise_depth);
            else if (noise_variant == GT_NOISE_MARBLE)
                i = R(0.5) * (R(1) + std::sin(q.z + R(10) * perlin->turbulence(q, noise_depth)));
            else i = R(0.5) * (R(1) + perlin->noise(q));
            return V3<R>{i, i, i};
        }
        if (texture == GT_TEX_IMAGE) return image ? image->sample<R>(h.u, h.v) : V3<R>(0, 1, 1);
        if (texture == GT_TEX_CHECKER) {
            int64_t xi = as_i64(double(std::floor(tex_inv_scale * h.point.x)));
            int64_t yi = as_i64(double(std::floor(tex_inv_scale * h.point.y)));
            int64_t zi = as_i64(double(std::floor(tex_inv_scale * h.point.z)));
            bool is_even = ((xi + yi + zi) % 2) == 0;
            if (g_trace) {
                auto edge = [](double c) { return std::fabs(c - std::round(c)); };
                trace_note(TR_TEXTURE, is_even ? 0 : 1,
                           std::fmin(std::fmin(edge(double(tex_inv_scale * h.point.x)),
                                               edge(double(tex_inv_scale * h.point.y))),
                                     edge(double(tex_inv_scale * h.point.z))));
            }
            return is_even ? even : odd;
        }
        return color;
    }
};

// OrthonormalBasis::from_w (geometry.rs:93-112).
template <class R> struct Onb {
    V3<R> u, v, w;
    static bool from_w(V3<R> axis, Onb& out) {
        V3<R> w = normalized(axis);
        if (length_squared(w) <= R(kEps)) return false;
        V3<R> a = std::fabs(w.x) > R(0.9) ? V3<R>(0, 1, 0) : V3<R>(1, 0, 0);
        V3<R> v = normalized(cross(w, a));
        V3<R> u = cross(w, v);
        out = {u, v, w};
        return true;
    }
    V3<R> local(V3<R> l) const { return (u * l.x + v * l.y) + w * l.z; } // geometry.rs:125-128
};

template <class R> inline R ggx_alpha(R roughness) { // sampling.rs:310-312
    R r = rclamp(roughness, R(0), R(1));
    return rmax(r * r, R(kGgxMinAlpha));
}
template <class R> inline R ggx_d(R ndh, R roughness) { // sampling.rs:212-225
    if (!std::isfinite(ndh) || ndh <= R(0) || !std::isfinite(roughness)) return R(0);
    R alpha = ggx_alpha(roughness);
    R a2 = alpha * alpha;
    R cos2 = ndh * ndh;
    R denom = cos2 * (a2 - R(1)) + R(1);
    if (denom <= R(kEps)) return R(0);
    return a2 / (R(kPi) * denom * denom);
}
template <class R> inline R smith_g1(R nd, R roughness) { // sampling.rs:314-322
    if (!std::isfinite(nd) || nd <= R(0) || !std::isfinite(roughness)) return R(0);
    R alpha = ggx_alpha(roughness);
    R a2 = alpha * alpha;
    R cos2 = nd * nd;
    return R(2) * nd / (nd + std::sqrt(a2 + (R(1) - a2) * cos2));
}
template <class R> inline R schlick(R cosine, R f0) { // sampling.rs:240-247
    if (!std::isfinite(cosine) || !std::isfinite(f0)) return R(0);
    f0 = rclamp(f0, R(0), R(1));
    return f0 + (R(1) - f0) * powi5(R(1) - rclamp(cosine, R(0), R(1)));
}
template <class R> inline R specular_luminance(V3<R> c) { // material.rs:1760-1762
    return rclamp(R(0.2126) * c.x + R(0.7152) * c.y + R(0.0722) * c.z, R(0), R(1));
}

// HenyeyGreensteinPdf::phase_value (gmath/sampling.rs:126-136), SPHERE_AREA = 4 pi.
template <class R> inline R hg_phase(R cosine, R g) {
    if (!std::isfinite(cosine) || !std::isfinite(g) || std::fabs(g) >= R(1)) return R(0);
    R den = (R(1) + g * g) - (R(2) * g) * rclamp(cosine, R(-1), R(1));
    if (den <= R(kEps)) return R(0);
    return (R(1) - g * g) / (R(4.0 * kPi) * std::pow(den, R(1.5)));
}

// MaterialPdf (pdf.rs:46-104) restricted to Sphere / Cosine / GgxReflection /
// HenyeyGreenstein.
enum PdfKind { PDF_SPHERE = 0, PDF_COSINE = 1, PDF_GGX = 2, PDF_HG = 3 };
template <class R> struct MatPdf {
    int kind = PDF_SPHERE;
    Onb<R> basis;
    V3<R> outgoing;
    R roughness{0}, alpha{0};

    R value(V3<R> dir) const {
        if (kind == PDF_SPHERE) return R(1) / R(4.0 * kPi); // sampling.rs:31-41
        if (kind == PDF_HG) {                               // sampling.rs:139-147; roughness holds g
            R len = length(dir);
            if (len <= R(kEps)) return R(0);
            return hg_phase(dot(dir, basis.w) / len, roughness);
        }
        if (kind == PDF_COSINE) {                         // sampling.rs:66-78
            R len = length(dir);
            if (len <= R(kEps)) return R(0);
            R c = dot(dir, basis.w) / len;
            return c <= R(0) ? R(0) : c / R(kPi);
        }
        // GgxReflectionPdf::value, sampling.rs:257-272
        V3<R> in = normalized(dir);
        if (length_squared(in) <= R(kEps) || dot(in, basis.w) <= R(0)) return R(0);
        V3<R> half = normalized(in + outgoing);
        R odh = dot(outgoing, half);
        if (length_squared(half) <= R(kEps) || odh <= R(kEps)) return R(0);
        R ndh = dot(half, basis.w);
        R hp = ggx_d(ndh, roughness) * rmax(ndh, R(0));
        return hp / (R(4) * std::fabs(odh));
    }
    V3<R> generate(SampleRng& rng) const {
        if (kind == PDF_SPHERE) return rng.random_unit_vector_spherical<R>();
        if (kind == PDF_HG) { // sampling.rs:149-164
            const R g = roughness;
            R r1 = rng.random_double<R>();
            R r2 = rng.random_double<R>();
            R cos_t;
            if (std::fabs(g) < R(1e-3)) {
                cos_t = R(1) - R(2) * r1;
            } else {
                R term = (R(1) - g * g) / ((R(1) - g) + (R(2) * g) * r1);
                cos_t = rclamp(((R(1) + g * g) - term * term) / (R(2) * g), R(-1), R(1));
            }
            R sin_t = std::sqrt(rmax(R(1) - cos_t * cos_t, R(0)));
            R phi = R(2.0 * kPi) * r2;
            return basis.local(V3<R>(std::cos(phi) * sin_t, std::sin(phi) * sin_t, cos_t));
        }
        if (kind == PDF_COSINE) return basis.local(rng.random_cosine_direction<R>());
        // sampling.rs:274-298
        R r1 = rng.random_double<R>();
        R r2 = rng.random_double<R>();
        R phi = R(2) * R(kPi) * r1;
        R a2 = alpha * alpha;
        R cr2 = rmin(r2, R(1) - R(kEps));
        R tan2 = a2 * cr2 / (R(1) - cr2);
        R cos_t = R(1) / std::sqrt(R(1) + tan2);
        R sin_t = std::sqrt(rmax(R(1) - cos_t * cos_t, R(0)));
        V3<R> half = basis.local(V3<R>(std::cos(phi) * sin_t, std::sin(phi) * sin_t, cos_t));
        V3<R> refl = reflected(-outgoing, normalized(half));
        return dot(refl, basis.w) > R(0) ? refl : outgoing;
    }
};

enum ScatterKind { SCATTER_NONE = 0, SCATTER_SPECULAR = 1, SCATTER_PDF = 2 };
template <class R> struct Scatter {
    int kind = SCATTER_NONE;
    Ray<R> ray;      // specular
    V3<R> att;       // both
    MatPdf<R> pdf;   // scattering
};

// Material::scatter for the six variants.
template <class R> inline Scatter<R> scatter(const Material<R>& m, const Ray<R>& in, const Hit<R>& h, SampleRng& rng) {
    Scatter<R> s;
    switch (m.kind) {
    case GT_MAT_LAMBERTIAN: { // material.rs:508-521
        if (!Onb<R>::from_w(h.shading, s.pdf.basis)) return s;
        s.kind = SCATTER_PDF;
        s.pdf.kind = PDF_COSINE;
        s.att = m.sample(h);
        return s;
    }
    case GT_MAT_ISOTROPIC: // material.rs:1124-1137
        s.kind = SCATTER_PDF;
        s.pdf.kind = PDF_SPHERE;
        s.att = m.sample(h);
        return s;
    case GT_MAT_HENYEY_GREENSTEIN: // material.rs:1281-1295: around the incoming direction
        if (!Onb<R>::from_w(in.d, s.pdf.basis)) return s;
        s.kind = SCATTER_PDF;
        s.pdf.kind = PDF_HG;
        s.pdf.roughness = m.param;
        s.att = m.sample(h);
        return s;
    case GT_MAT_GGX: { // material.rs:1583-1597, GgxReflectionPdf::new sampling.rs:146-170
        V3<R> outgoing = -normalized(in.d);
        MatPdf<R> p;
        p.kind = PDF_GGX;
        if (!Onb<R>::from_w(h.shading, p.basis)) return s;
        p.outgoing = normalized(outgoing);
        if (length_squared(p.outgoing) <= R(kEps) || dot(p.outgoing, p.basis.w) <= R(0)) return s;
        p.roughness = rclamp(m.param, R(0), R(1));
        p.alpha = ggx_alpha(p.roughness);
        s.kind = SCATTER_PDF;
        s.pdf = p;
        s.att = m.sample(h);
        return s;
    }
    case GT_MAT_METAL: { // material.rs:2087-2106
        V3<R> refl = reflected(normalized(in.d), h.shading);
        V3<R> dir = refl + rng.random_unit_vector_spherical<R>() * m.param;
        if (dot(dir, h.normal) <= R(0)) return s;
        s.kind = SCATTER_SPECULAR;
        s.ray = Ray<R>{spawn_origin(h, dir), dir, in.time};
        s.att = m.color;
        return s;
    }
    case GT_MAT_DIELECTRIC: { // material.rs:2321-2351
        R ior = m.param;
        R ratio = h.front_face ? R(1) / ior : ior;
        V3<R> unit = normalized(in.d);
        R cos_t = rmin(dot(-unit, h.normal), R(1));
        R sin_t = std::sqrt(R(1) - cos_t * cos_t);
        bool cannot = ratio * sin_t > R(1);
        V3<R> dir;
        bool reflect = cannot;
        if (!reflect) {
            R r0 = (R(1) - ratio) / (R(1) + ratio); // Dielectric::reflectance, material.rs:2213-2219
            r0 = r0 * r0;
            R refl = r0 + (R(1) - r0) * powi5(R(1) - cos_t);
            const R u = rng.random_double<R>();
            reflect = refl > u;
            trace_note(TR_DIELECTRIC, reflect ? 1 : 0, double(u) - double(refl));
        } else {
            trace_note(TR_DIELECTRIC, 2, double(ratio * sin_t) - 1.0);
        }
        dir = reflect ? reflected(unit, h.normal) : refracted(unit, h.normal, ratio);
        s.kind = SCATTER_SPECULAR;
        s.ray = Ray<R>{spawn_origin(h, dir), dir, in.time};
        s.att = V3<R>(1, 1, 1);
        return s;
    }
    default: // DiffuseLight: no scatter (material.rs:1008-1028)
        return s;
    }
}

// Material::scattering_pdf.
template <class R> inline R scattering_pdf(const Material<R>& m, const Ray<R>& in, const Hit<R>& h, V3<R> out_dir) {
    switch (m.kind) {
    case GT_MAT_LAMBERTIAN: { // material.rs:523-530
        R c = dot(h.shading, normalized(out_dir));
        return c <= R(0) ? R(0) : c / R(kPi);
    }
    case GT_MAT_ISOTROPIC:
        return R(1) / (R(4) * R(kPi)); // material.rs:1139-1141
    case GT_MAT_HENYEY_GREENSTEIN: {  // material.rs:1297-1302
        MatPdf<R> p;
        p.kind = PDF_HG;
        p.roughness = m.param;
        if (!Onb<R>::from_w(in.d, p.basis)) return R(0);
        return p.value(out_dir);
    }
    case GT_MAT_GGX: {                  // material.rs:1599-1617, 1717-1758
        V3<R> outgoing = -normalized(in.d);
        V3<R> incoming = normalized(out_dir);
        if (dot(incoming, h.normal) <= R(0) || dot(outgoing, h.normal) <= R(0)) return R(0);
        R f0 = specular_luminance(m.sample(h));
        V3<R> n = normalized(h.shading);
        V3<R> o = normalized(outgoing);
        V3<R> i = normalized(incoming);
        R ndi = dot(n, i), ndo = dot(n, o);
        if (ndi <= R(0) || ndo <= R(0)) return R(0);
        V3<R> half = normalized(i + o);
        if (length_squared(half) <= R(kEps)) return R(0);
        R ndh = dot(n, half), odh = dot(o, half);
        if (ndh <= R(0) || odh <= R(0)) return R(0);
        R rough = m.param;
        R D = ggx_d(ndh, rough);
        R G = smith_g1(ndi, rough) * smith_g1(ndo, rough);
        f0 = rclamp(f0, R(0), R(1));
        if (f0 <= R(kEps)) return R(0);
        R F = schlick(odh, f0) / f0;
        return D * G * F / (R(4) * ndo);
    }
    default:
        return R(0);
    }
}

// Material::emitted (DiffuseLight front face only, material.rs:1008-1022).
template <class R> inline V3<R> emitted(const Material<R>& m, const Hit<R>& h) {
    if (m.kind == GT_MAT_DIFFUSE_LIGHT && h.front_face) return m.sample(h);
    return V3<R>();
}

// Material::denoise_albedo (material.rs:2698-2708 and the variants).
template <class R> inline V3<R> denoise_albedo(const Material<R>& m, const Hit<R>& h) {
    switch (m.kind) {
    case GT_MAT_METAL:
        return m.color;
    case GT_MAT_DIELECTRIC:
        return V3<R>(1, 1, 1);
    default:
        return m.sample(h);
    }
}

// ------------------------------------------------------------- light targets
template <class R> struct LightTarget {
    Prim<R> geom;
    R weight{1};
};

// sphere_pdf_value / quad_pdf_value / triangle_pdf_value / area_pdf_value (object.rs:1044-1111).
template <class R> inline R area_pdf_value(V3<R> dir, R t, V3<R> normal, R area) {
    if (area <= R(kEps)) return R(0);
    R d2 = length_squared(dir * t);
    R cosine = std::fabs(dot(normalized(dir), normal));
    if (cosine <= R(kEps)) return R(0);
    return d2 / (cosine * area);
}

template <class R> inline R geometry_pdf_value(const Prim<R>& g, V3<R> origin, R time, V3<R> dir) {
    Ray<R> r{origin, dir, R(0)};
    switch (g.kind) {
    case GT_GEOM_SPHERE:
    case GT_GEOM_MOVING_SPHERE: {
        V3<R> center = g.kind == GT_GEOM_SPHERE ? g.a : g.center_at(time);
        R root;
        if (!hit_sphere_root(center, g.radius, r, R(kShadowAcnePdf), std::numeric_limits<R>::infinity(), root))
            return R(0);
        V3<R> cd = center - origin;
        R d2 = length_squared(cd);
        R r2 = g.radius * g.radius;
        if (d2 <= r2) return R(1) / (R(4) * R(kPi));
        R cos_max = std::sqrt(R(1) - r2 / d2);
        R solid = R(2) * R(kPi) * (R(1) - cos_max);
        return solid <= R(kEps) ? R(0) : R(1) / solid;
    }
    case GT_GEOM_QUAD: {
        R t, u, v;
        if (!quad_hit_ray(g, r, R(kShadowAcnePdf), std::numeric_limits<R>::infinity(), t, u, v)) return R(0);
        R area = std::sqrt(g.qarea_sq);
        return area_pdf_value(dir, t, g.qnormal, area);
    }
    case GT_GEOM_TRIANGLE: {
        R t, u, v;
        if (!triangle_hit_ray(g.a, g.b, g.c, r, R(kShadowAcnePdf), std::numeric_limits<R>::infinity(), t, u, v))
            return R(0);
        V3<R> awn = cross(g.b - g.a, g.c - g.a);
        R area = R(0.5) * std::sqrt(length_squared(awn));
        return area_pdf_value(dir, t, normalized(awn), area);
    }
    }
    return R(0);
}

template <class R> inline V3<R> geometry_random_direction(const Prim<R>& g, V3<R> origin, R time, SampleRng& rng) {
    switch (g.kind) {
    case GT_GEOM_SPHERE:
    case GT_GEOM_MOVING_SPHERE: { // random_direction_to_sphere, object.rs:1113-1128
        V3<R> center = g.kind == GT_GEOM_SPHERE ? g.a : g.center_at(time);
        V3<R> dir = center - origin;
        R d2 = length_squared(dir);
        R r2 = g.radius * g.radius;
        if (d2 <= r2 || d2 <= R(kEps)) return rng.random_unit_vector_spherical<R>();
        R r1 = rng.random_double<R>(); // random_to_sphere, object.rs:1153-1161
        R rr2 = rng.random_double<R>();
        R z = R(1) + rr2 * (std::sqrt(R(1) - g.radius * g.radius / d2) - R(1));
        R phi = R(2) * R(kPi) * r1;
        R rz = std::sqrt(R(1) - z * z);
        V3<R> local(std::cos(phi) * rz, std::sin(phi) * rz, z);
        Onb<R> b;
        if (!Onb<R>::from_w(dir, b)) return local;
        return b.local(local);
    }
    case GT_GEOM_QUAD: { // object.rs:1130-1134
        R r1 = rng.random_double<R>();
        V3<R> p = g.a + g.b * r1;
        R r2 = rng.random_double<R>();
        p = p + g.c * r2;
        return p - origin;
    }
    case GT_GEOM_TRIANGLE: { // object.rs:1136-1151
        R a = rng.random_double<R>();
        R b = rng.random_double<R>();
        if (a + b > R(1)) {
            a = R(1) - a;
            b = R(1) - b;
        }
        V3<R> p = (g.a + (g.b - g.a) * a) + (g.c - g.a) * b;
        return p - origin;
    }
    }
    return V3<R>(1, 0, 0);
}

template <class R> struct LightList { // WeightedSamplingTargetList, scene.rs:423-497
    std::vector<LightTarget<R>> targets;
    R total{0};
    bool empty() const { return targets.empty(); }
    R pdf_value(V3<R> origin, R time, V3<R> dir) const {
        if (targets.empty() || total <= R(0)) return R(0);
        R sum = R(-0.0);
        for (const auto& t : targets) sum = sum + (t.weight / total) * geometry_pdf_value(t.geom, origin, time, dir);
        return sum;
    }
    V3<R> random_direction(V3<R> origin, R time, SampleRng& rng) const {
        if (targets.empty() || total <= R(0)) return V3<R>(1, 0, 0);
        R pick = rng.random_range<R>(R(0), total);
        for (size_t k = 0; k < targets.size(); ++k) {
            pick -= targets[k].weight;
            if (pick <= R(0)) {
                trace_note(TR_LIGHT_PICK, int32_t(k), double(pick) / double(total));
                return geometry_random_direction(targets[k].geom, origin, time, rng);
            }
        }
        trace_note(TR_LIGHT_PICK, int32_t(targets.size()) - 1, double(pick) / double(total));
        return geometry_random_direction(targets.back().geom, origin, time, rng);
    }
};

// ---------------------------------------------------------- environment light
// EnvironmentLight (raytracing/environment.rs:22-202).  SRGB8 is the reference; RGB32F is
// the linear f32 extension (same distribution and addressing, f64 bilinear of f32 texels,
// no 8-bit rounding and no gamma decode).
template <class R> struct Environment {
    int format = GT_ENV_SRGB8;
    uint32_t width = 0, height = 0;
    std::vector<uint8_t> px8;
    std::vector<float> px32;
    std::vector<double> weights, cdf;
    double total = 0;

    static double luminance(double r, double g, double b) { return 0.2126 * r + 0.7152 * g + 0.0722 * b; }
    void texel_linear(uint32_t x, uint32_t y, double out[3]) const {
        size_t i = (size_t(y) * width + x) * 3;
        for (int c = 0; c < 3; ++c) {
            if (format == GT_ENV_SRGB8) {
                double v = double(px8[i + c]) / 255.0; // colors.rs:78-84
                out[c] = v * v;
            } else {
                out[c] = double(px32[i + c]);
            }
        }
    }
    void build() { // environment.rs:155-185
        weights.clear();
        cdf.clear();
        total = 0;
        if (width == 0 || height == 0) return;
        for (uint32_t y = 0; y < height; ++y) {
            double theta = kPi * ((double(y) + 0.5) / double(height));
            double s = std::fmax(std::sin(theta), 0.0);
            for (uint32_t x = 0; x < width; ++x) {
                double c[3];
                texel_linear(x, y, c);
                double w = std::fmax(luminance(c[0], c[1], c[2]), 0.0) * s;
                total += w;
                weights.push_back(w);
                cdf.push_back(total);
            }
        }
    }
    double pixel_solid_angle(uint32_t y) const { // environment.rs:187-191
        double t0 = kPi * (double(y) / double(height));
        double t1 = kPi * (double(y + 1) / double(height));
        return (kTau / double(width)) * std::fmax(std::cos(t0) - std::cos(t1), 0.0);
    }
    R pdf_value(V3<R> dir_r) const { // environment.rs:133-153 (evaluated in f64)
        if (total <= kEps || weights.empty()) return R(1.0 / (4.0 * kPi));
        V3<double> d = normalized(V3<double>(double(dir_r.x), double(dir_r.y), double(dir_r.z)));
        double theta = std::acos(rclamp(d.y, -1.0, 1.0));
        double phi = rem_euclid(std::atan2(d.z, d.x), kTau);
        uint64_t x = as_usize(std::floor((phi / kTau) * double(width)));
        uint64_t y = as_usize(std::floor((theta / kPi) * double(height)));
        x = std::min<uint64_t>(x, width - 1);
        y = std::min<uint64_t>(y, height - 1);
        double prob = weights[y * width + x] / total;
        double sa = pixel_solid_angle(uint32_t(y));
        return sa <= kEps ? R(0) : R(prob / sa);
    }
    void sample_direction(SampleRng& rng, V3<R>& dir, R& pdf) const { // environment.rs:107-131
        if (total <= kEps || weights.empty()) {
            dir = rng.random_unit_vector_spherical<R>();
            pdf = R(1) / R(4.0 * kPi);
            return;
        }
        double target = double(rng.random_double<R>()) * total;
        size_t idx = size_t(std::lower_bound(cdf.begin(), cdf.end(), target) - cdf.begin());
        idx = std::min(idx, weights.size() - 1);
        if (g_trace) {
            const double lo = idx > 0 ? cdf[idx - 1] : 0.0;
            trace_note(TR_ENV_PICK, int32_t(idx), std::fmin(target - lo, cdf[idx] - target) / total);
        }
        size_t x = idx % width, y = idx / width;
        double u = (double(x) + double(rng.random_double<R>())) / double(width);
        double t0 = kPi * (double(y) / double(height));
        double t1 = kPi * (double(y + 1) / double(height));
        double c0 = std::cos(t0), c1 = std::cos(t1);
        double ct = c0 + double(rng.random_double<R>()) * (c1 - c0);
        double st = std::sqrt(std::fmax(1.0 - ct * ct, 0.0));
        double phi = kTau * u;
        V3<double> d(st * std::cos(phi), ct, st * std::sin(phi));
        dir = V3<R>(R(d.x), R(d.y), R(d.z));
        pdf = pdf_value(dir);
    }
    static uint8_t lerp_u8(uint8_t a, uint8_t b, double t) { // colors.rs:525-537
        t = rclamp(t, 0.0, 1.0);
        double v = std::round(double(a) + double(int(b) - int(a)) * t);
        if (!(v > 0.0)) return 0;
        if (v >= 255.0) return 255;
        return uint8_t(v);
    }
    V3<R> radiance(V3<R> dir_r) const { // environment.rs:98-105, texture.rs:657-711
        V3<double> d = normalized(V3<double>(double(dir_r.x), double(dir_r.y), double(dir_r.z)));
        double phi = rem_euclid(std::atan2(d.z, d.x), kTau);
        double theta = std::acos(rclamp(d.y, -1.0, 1.0));
        double s = phi / kTau, t = 1.0 - theta / kPi;
        if (width == 0 || height == 0 || !std::isfinite(s) || !std::isfinite(t)) return V3<R>();
        double xc = rem_euclid(s, 1.0) * double(width); // Repeat
        uint32_t x0 = std::min<uint32_t>(as_u32(std::floor(xc)), width - 1);
        uint32_t x1 = x0 + 1 == width ? 0 : x0 + 1;
        double yc = rclamp(1.0 - t, 0.0, 1.0) * double(height - 1); // Clamp
        uint32_t y0 = as_u32(std::floor(yc));
        uint32_t y1 = std::min<uint32_t>(y0 + 1, height - 1);
        double tx = xc - double(x0), ty = yc - double(y0);
        if (format == GT_ENV_SRGB8) {
            double out[3];
            for (int c = 0; c < 3; ++c) {
                auto p = [&](uint32_t xx, uint32_t yy) { return px8[(size_t(yy) * width + xx) * 3 + c]; };
                uint8_t top = lerp_u8(p(x0, y0), p(x1, y0), tx);
                uint8_t bot = lerp_u8(p(x0, y1), p(x1, y1), tx);
                double v = double(lerp_u8(top, bot, ty)) / 255.0;
                out[c] = v * v;
            }
            return V3<R>(R(out[0]), R(out[1]), R(out[2]));
        }
        double out[3];
        double ctx = rclamp(tx, 0.0, 1.0), cty = rclamp(ty, 0.0, 1.0);
        for (int c = 0; c < 3; ++c) {
            auto p = [&](uint32_t xx, uint32_t yy) { return double(px32[(size_t(yy) * width + xx) * 3 + c]); };
            double top = p(x0, y0) + (p(x1, y0) - p(x0, y0)) * ctx;
            double bot = p(x0, y1) + (p(x1, y1) - p(x0, y1)) * ctx;
            out[c] = top + (bot - top) * cty;
        }
        return V3<R>(R(out[0]), R(out[1]), R(out[2]));
    }
};

// --------------------------------------------------------------------- scene
// ------------------------------------------------------------ meshes, instances
// TriangleMesh (raytracing/mesh.rs): object-space primitives with optional per-triangle
// texture coordinates and vertex normals.  Its hit is the closest over all primitives in
// order (the mesh BVH of mesh.rs:640-668 returns the same hit up to exact ties).
template <class R> struct MeshObj {
    std::vector<Prim<R>> prims;
    std::vector<double> uv, vn; // 6 / 9 per primitive or empty
    std::vector<uint8_t> attr;  // bit 0 texcoords, bit 1 normals

    // MeshTriangle::hit (mesh.rs:56-101) with the material's normal map
    // (material.rs:1663-1684) for a closest hit `h` on primitive i.
    void finish(const Material<R>& m, uint32_t i, const Ray<R>& ray, Hit<R>& h) const {
        const Prim<R>& p = prims[i];
        if (p.kind != GT_GEOM_TRIANGLE || attr.empty() || attr[i] == 0) return;
        // the barycentrics of the hit: triangle_hit_ray's u, v (Hit u, v of a plain triangle)
        const R bu = h.u, bv = h.v, bw = R(1) - bu - bv;
        const double* tc = uv.empty() ? nullptr : uv.data() + size_t(i) * 6;
        if (attr[i] & 1) {
            h.u = bw * R(tc[0]) + bu * R(tc[2]) + bv * R(tc[4]);
            h.v = bw * R(tc[1]) + bu * R(tc[3]) + bv * R(tc[5]);
        }
        if (attr[i] & 2) { // shading_normal + set_shading_normal (object.rs:469-479)
            const double* n = vn.data() + size_t(i) * 9;
            const V3<R> s = V3<R>(R(n[0]), R(n[1]), R(n[2])) * bw + V3<R>(R(n[3]), R(n[4]), R(n[5])) * bu +
                            V3<R>(R(n[6]), R(n[7]), R(n[8])) * bv;
            if (length_squared(s) > R(kEps)) h.shading = h.front_face ? normalized(s) : -normalized(s);
        }
        if (!(attr[i] & 1) || !m.normal_map) return;
        // tangent_frame (mesh.rs:121-141)
        const V3<R> e1 = p.b - p.a, e2 = p.c - p.a;
        const R du1 = R(tc[2]) - R(tc[0]), dv1 = R(tc[3]) - R(tc[1]);
        const R du2 = R(tc[4]) - R(tc[0]), dv2 = R(tc[5]) - R(tc[1]);
        const R det = du1 * dv2 - du2 * dv1;
        if (std::fabs(det) <= R(kEps)) return;
        const R inv = R(1) / det;
        const V3<R> tangent = (e1 * dv2 - e2 * dv1) * inv, bitangent = (e2 * du1 - e1 * du2) * inv;
        if (!(length_squared(tangent) > R(kEps) && length_squared(bitangent) > R(kEps))) return;
        // set_tangent_frame (object.rs:495-517)
        const V3<R> n = h.shading;
        V3<R> t = tangent - n * dot(tangent, n);
        if (length_squared(t) <= R(kEps)) return;
        t = normalized(t);
        const V3<R> ref = cross(n, t);
        V3<R> b = bitangent - n * dot(bitangent, n);
        b = b - t * dot(b, t);
        if (length_squared(b) <= R(kEps)) b = ref;
        const R hand = dot(b, ref) < R(0) ? R(-1) : R(1);
        b = normalized(ref * hand);
        // normal_map_world_normal + set_oriented_shading_normal (object.rs:481-493)
        const V3<R> tn = m.normal_map->template tangent_normal<R>(h.u, h.v, m.normal_strength, m.normal_neg_y);
        V3<R> world = t * tn.x + b * tn.y + n * tn.z;
        if (length_squared(world) <= R(kEps)) return;
        world = normalized(world);
        if (dot(world, n) < R(0)) world = -world;
        if (length_squared(world) > R(kEps)) h.shading = normalized(world);
    }
};

// A world object: a mesh, or MatrixInstance(mesh) (raytracing/instance.rs:205-317).
template <class R> struct WorldObject {
    uint32_t mesh = 0;
    bool transformed = false;
    R xf[16], inv[16];
    static V3<R> point(const R* m, V3<R> p) { // transform_point, instance.rs:355-364
        R r[4];
        for (int i = 0; i < 4; ++i) r[i] = m[4 * i] * p.x + m[4 * i + 1] * p.y + m[4 * i + 2] * p.z + m[4 * i + 3] * R(1);
        if (std::fabs(r[3]) > R(kEps)) return V3<R>(r[0] / r[3], r[1] / r[3], r[2] / r[3]);
        return V3<R>(r[0], r[1], r[2]);
    }
    static V3<R> vector(const R* m, V3<R> v) { // transform_vector, instance.rs:366-369
        R r[3];
        for (int i = 0; i < 3; ++i) r[i] = m[4 * i] * v.x + m[4 * i + 1] * v.y + m[4 * i + 2] * v.z + m[4 * i + 3] * R(0);
        return V3<R>(r[0], r[1], r[2]);
    }
};

template <class R> struct Scene {
    std::vector<Prim<R>> prims;
    std::vector<gt_geometry> geoms;
    std::vector<Material<R>> materials;
    std::vector<Medium<R>> media;
    std::vector<MeshObj<R>> meshes;
    std::vector<WorldObject<R>> objects;
    FlatBvh bvh;

    void load(const gt_scene_desc& d) {
        prims.clear();
        geoms.clear();
        materials.clear();
        media.clear();
        meshes.clear();
        objects.clear();
        for (uint32_t k = 0; k < (d.meshes ? d.num_meshes : 0u); ++k) {
            const gt_mesh& gm = d.meshes[k];
            MeshObj<R> m;
            const size_t n = gm.num_primitives;
            for (size_t i = 0; i < n; ++i) {
                if (gm.primitives[i].material >= d.num_materials) throw std::invalid_argument("mesh material id");
                m.prims.push_back(Prim<R>::from_geometry(gm.primitives[i].geometry, gm.primitives[i].material));
            }
            if (gm.texcoords) m.uv.assign(gm.texcoords, gm.texcoords + n * 6);
            if (gm.normals) m.vn.assign(gm.normals, gm.normals + n * 9);
            m.attr.resize(n);
            for (size_t i = 0; i < n; ++i) {
                const uint8_t given = uint8_t((gm.texcoords ? 1 : 0) | (gm.normals ? 2 : 0));
                m.attr[i] = gm.attribute_flags ? uint8_t(gm.attribute_flags[i] & given) : given;
            }
            meshes.push_back(std::move(m));
        }
        for (uint32_t k = 0; k < (d.objects ? d.num_objects : 0u); ++k) {
            const gt_object& go = d.objects[k];
            if (go.mesh >= meshes.size()) throw std::invalid_argument("object mesh index");
            WorldObject<R> o;
            o.mesh = go.mesh;
            o.transformed = go.transformed != 0;
            for (int a = 0; a < 16; ++a) {
                o.xf[a] = R(go.transform[a]);
                o.inv[a] = R(go.inverse[a]);
            }
            objects.push_back(o);
        }
        for (uint32_t i = 0; i < (d.media ? d.num_media : 0u); ++i) {
            const gt_medium& m = d.media[i];
            if (m.material >= d.num_materials || !(std::isfinite(m.density) && m.density > 0.0) ||
                m.shape > GT_MEDIUM_BOX)
                throw std::invalid_argument("invalid medium");
            media.push_back(Medium<R>::from_desc(m));
        }
        std::vector<std::shared_ptr<const ImageData>> images;
        for (uint32_t i = 0; i < (d.images ? d.num_images : 0u); ++i) {
            auto im = std::make_shared<ImageData>();
            const gt_image& g = d.images[i];
            im->w = g.width;
            im->h = g.height;
            im->filter = int(g.filter);
            im->wrap_s = int(g.wrap_s);
            im->wrap_t = int(g.wrap_t);
            if (g.rgb) im->rgb.assign(g.rgb, g.rgb + size_t(g.width) * g.height * 3);
            images.push_back(im);
        }
        for (uint32_t i = 0; i < d.num_materials; ++i) {
            materials.push_back(Material<R>::from_desc(d.materials[i]));
            if (d.materials[i].normal_map) {
                const gt_material& gm = d.materials[i];
                if (gm.normal_map > images.size()) throw std::invalid_argument("normal map index out of range");
                materials.back().normal_map = images[gm.normal_map - 1];
                materials.back().normal_strength = R(std::fmax(gm.normal_map_strength, 0.0)); // with_strength
                materials.back().normal_neg_y = (gm.normal_map_flags & GT_NORMAL_MAP_NEGATIVE_Y) != 0;
            }
            if (d.materials[i].texture_kind == GT_TEX_IMAGE) {
                const double k = d.materials[i].tex[0];
                if (!(k >= 0 && k < double(images.size())) || k != std::floor(k))
                    throw std::invalid_argument("image texture index out of range");
                materials.back().image = images[size_t(k)];
            }
        }
        std::vector<Bounds> bounds;
        for (uint32_t i = 0; i < d.num_primitives; ++i) {
            const gt_primitive& p = d.primitives[i];
            if (p.material >= d.num_materials) throw std::invalid_argument("material id out of bounds");
            prims.push_back(Prim<R>::from_geometry(p.geometry, p.material));
            geoms.push_back(p.geometry);
            bounds.push_back(geometry_bounds(p.geometry));
        }
        bvh.build(bounds, d.bvh_leaf_size == 0 ? 4u : d.bvh_leaf_size);
    }

    // hit_ray_scene_indices (scene.rs:849-874).
    bool hit_leaf(const uint32_t* idx, uint32_t n, const Ray<R>& ray, R tmin, R tmax, Hit<R>& best) const {
        R closest = tmax;
        bool any = false;
        for (uint32_t i = 0; i < n; ++i) {
            Hit<R> h;
            if (intersect(prims[idx[i]], ray, tmin, closest, h)) {
                closest = h.t;
                h.prim = int(idx[i]);
                h.material = prims[idx[i]].material;
                best = h;
                any = true;
            }
        }
        return any;
    }

    // HittableList::hit_with_rng over [this RayScene, media...] (scene.rs:177-197): the
    // surfaces' closest hit, then each medium in order, clipped to the closest so far.  A
    // medium hit is the medium_hit_record of medium.rs:152-168.
    // The world objects come between the surfaces and the media.
    bool object_hit(const WorldObject<R>& o, const Ray<R>& ray, R tmin, R tmax, Hit<R>& out) const {
        Ray<R> r = ray;
        if (o.transformed) { // MatrixInstance::hit_with_rng (instance.rs:266-289)
            r.o = WorldObject<R>::point(o.inv, ray.o);
            r.d = WorldObject<R>::vector(o.inv, ray.d);
        }
        const MeshObj<R>& m = meshes[o.mesh];
        R closest = tmax;
        int best = -1;
        Hit<R> h;
        for (size_t i = 0; i < m.prims.size(); ++i) {
            Hit<R> c;
            if (intersect(m.prims[i], r, tmin, closest, c)) {
                closest = c.t;
                best = int(i);
                h = c;
            }
        }
        if (best < 0) return false;
        h.prim = best;
        h.material = m.prims[size_t(best)].material;
        m.finish(materials[h.material], uint32_t(best), r, h);
        if (o.transformed) { // (u, v) kept; set_face_normal resets the shading normal (object.rs:455-467)
            const V3<R> outward_obj = h.front_face ? h.normal : -h.normal;
            h.point = WorldObject<R>::point(o.xf, h.point);
            R nt[16]; // normal_transform = inverse.transpose()
            for (int i = 0; i < 4; ++i)
                for (int j = 0; j < 4; ++j) nt[4 * i + j] = o.inv[4 * j + i];
            set_face(h, ray, normalized(WorldObject<R>::vector(nt, outward_obj)));
        }
        out = h;
        return true;
    }

    bool world_hit(const Ray<R>& ray, R tmin, R tmax, Hit<R>& out, SampleRng& rng) const {
        bool any = hit(ray, tmin, tmax, out);
        R closest = any ? out.t : tmax;
        for (const WorldObject<R>& o : objects) {
            Hit<R> h;
            if (object_hit(o, ray, tmin, closest, h)) {
                closest = h.t;
                out = h;
                any = true;
            }
        }
        for (size_t k = 0; k < media.size(); ++k) {
            R t;
            if (!media[k].hit(ray, tmin, closest, rng, t)) continue;
            closest = t;
            out = Hit<R>();
            out.point = ray.at(t);
            out.normal = V3<R>(1, 0, 0);
            out.shading = out.normal;
            out.t = t;
            out.front_face = true;
            out.prim = -2 - int(k);
            out.material = media[k].material;
            any = true;
        }
        return any;
    }

    // FlatBvh::hit_with_stats (bvh.rs:306-399) over RayScene primitives.
    bool hit(const Ray<R>& ray, R tmin, R tmax, Hit<R>& out, BvhStats* stats = nullptr) const {
        if (bvh.nodes.empty()) return false;
        BvhStats local;
        BvhStats& st = stats ? *stats : local;
        RayTraversal<R> tr(ray);
        st.rays += 1;
        st.node_bounds_tests += 1;
        R root_entry;
        if (!tr.hit_bounds(bvh.nodes[0].bounds, tmin, tmax, root_entry)) return false;
        st.node_bounds_hits += 1;
        // TraversalStack: 64 inline entries, then a heap overflow (bvh.rs:174-220).
        struct Entry {
            uint32_t node;
            R t;
        };
        struct Stack {
            Entry inl[64];
            size_t n = 0;
            std::vector<Entry> over;
            void push_back(Entry e) {
                if (over.empty() && n < 64) inl[n++] = e;
                else over.push_back(e);
            }
            Entry back() const { return over.empty() ? inl[n - 1] : over.back(); }
            void pop_back() {
                if (!over.empty()) over.pop_back();
                else --n;
            }
            bool empty() const { return n == 0 && over.empty(); }
            size_t size() const { return n + over.size(); }
        } stack;
        stack.push_back({0, root_entry});
        st.max_stack_depth = std::max<uint64_t>(st.max_stack_depth, stack.size());
        R closest = tmax;
        bool any = false;
        while (!stack.empty()) {
            Entry e = stack.back();
            stack.pop_back();
            if (e.t >= closest) continue;
            const BvhNode& n = bvh.nodes[e.node];
            if (n.leaf) {
                st.leaf_visits += 1;
                st.primitive_candidates += n.b;
                Hit<R> h;
                if (hit_leaf(bvh.indices.data() + n.a, n.b, ray, tmin, closest, h)) {
                    st.leaf_hit_results += 1;
                    closest = h.t;
                    out = h;
                    any = true;
                }
            } else {
                st.node_bounds_tests += 2;
                R le, re;
                bool lh = tr.hit_bounds(bvh.nodes[n.a].bounds, tmin, closest, le);
                bool rh = tr.hit_bounds(bvh.nodes[n.b].bounds, tmin, closest, re);
                st.node_bounds_hits += uint64_t(lh) + uint64_t(rh);
                if (lh && rh) {
                    if (re < le) {
                        stack.push_back({n.a, le});
                        stack.push_back({n.b, re});
                    } else {
                        stack.push_back({n.b, re});
                        stack.push_back({n.a, le});
                    }
                } else if (lh) {
                    stack.push_back({n.a, le});
                } else if (rh) {
                    stack.push_back({n.b, re});
                }
                st.max_stack_depth = std::max<uint64_t>(st.max_stack_depth, stack.size());
            }
        }
        return any;
    }

    // RayScene::hit_bruteforce (scene.rs:1459-1467).
    bool hit_bruteforce(const Ray<R>& ray, R tmin, R tmax, Hit<R>& out) const {
        std::vector<uint32_t> all(prims.size());
        std::iota(all.begin(), all.end(), 0u);
        return hit_leaf(all.data(), uint32_t(all.size()), ray, tmin, tmax, out);
    }
};

// -------------------------------------------------------------------- camera
template <class R> struct Camera {
    gt_camera_desc desc;
    uint32_t width = 0, height = 0;
    V3<R> center, pixel00, du, dv, ddu, ddv;
    V3<R> p00_rel; // pixel00 - center in f64, reduced to R (used by the f32 evaluation)

    // RayCamera::initialized (camera.rs:1068-1130); computed in f64 then reduced to R.
    void init(const gt_camera_desc& d) {
        desc = d;
        desc.samples_per_pixel = std::max<uint32_t>(d.samples_per_pixel, 1u); // camera.rs:1085
        width = d.image_width;
        height = std::max<uint32_t>(as_u32(double(d.image_width) / d.aspect_ratio), 1u);
        double theta = d.vertical_fov * kPi / 180.0;
        double h = std::tan(theta * 0.5);
        double vh = 2.0 * h * d.focus_distance;
        double vw = vh * (double(d.image_width) / double(height));
        V3<double> c = v3<double>(d.lookfrom);
        V3<double> fwd = normalized(v3<double>(d.lookat) - c); // CameraBasis::looking_at, geometry.rs:23-37
        V3<double> right = normalized(cross(fwd, v3<double>(d.view_up)));
        V3<double> up = cross(right, fwd);
        V3<double> w = -fwd, u = right, v = up;
        V3<double> vu = u * vw;
        V3<double> vv = (-v) * vh;
        V3<double> pdu = vdiv(vu, double(d.image_width));
        V3<double> pdv = vdiv(vv, double(height));
        V3<double> ul = ((c - w * d.focus_distance) - vdiv(vu, 2.0)) - vdiv(vv, 2.0);
        V3<double> p00 = ul + (pdu + pdv) * 0.5;
        double dr = d.focus_distance * std::tan((d.defocus_angle * 0.5) * kPi / 180.0);
        auto cv = [](V3<double> a) { return V3<R>(R(a.x), R(a.y), R(a.z)); };
        center = cv(c);
        pixel00 = cv(p00);
        p00_rel = cv(p00 - c);
        du = cv(pdu);
        dv = cv(pdv);
        ddu = cv(u * dr);
        ddv = cv(v * dr);
    }
    uint32_t grid_width() const { // camera.rs:1706-1708, 3028-3034
        if (desc.pixel_sample_mode == GT_SAMPLE_RANDOM) return 1;
        if (desc.pixel_sample_mode == GT_SAMPLE_STRATIFIED)
            return std::max<uint32_t>(as_u32(std::sqrt(double(desc.samples_per_pixel))), 1u);
        return std::max<uint32_t>(desc.grid_width, 1u);
    }
    uint32_t effective_spp() const { // camera.rs:1547-1556
        if (desc.pixel_sample_mode == GT_SAMPLE_RANDOM) return desc.samples_per_pixel;
        uint64_t g = desc.pixel_sample_mode == GT_SAMPLE_STRATIFIED ? grid_width() : desc.grid_width;
        uint64_t s = g * g;
        return s > UINT32_MAX ? UINT32_MAX : uint32_t(s);
    }
    Ray<R> ray_for_pixel(uint32_t x, uint32_t y) const { // camera.rs:1641-1653
        V3<R> pc = (pixel00 + du * R(x)) + dv * R(y);
        return Ray<R>{center, pc - center, R(desc.shutter_start)};
    }
    // camera.rs:1658-1670 tail.  In f64 the direction is pixel_sample - origin as the
    // reference computes it.  In f32 that difference of two points far from the origin
    // cancels (a camera 800 units out with a viewport 1 unit ahead loses ~1e-4), so the
    // f32 evaluation forms the same vector from center-relative terms instead.
    Ray<R> finish_ray(R sx, R sy, SampleRng& rng) const {
        const bool defocus = !(desc.defocus_angle <= 0.0);
        V3<R> p;
        if (defocus) p = rng.random_in_unit_disk<R>();
        R time = rng.random_range<R>(R(desc.shutter_start), R(desc.shutter_end));
        if (sizeof(R) == sizeof(double)) {
            V3<R> ps = (pixel00 + du * sx) + dv * sy;
            V3<R> origin = defocus ? (center + ddu * p.x) + ddv * p.y : center;
            return Ray<R>{origin, ps - origin, time};
        }
        V3<R> off = defocus ? ddu * p.x + ddv * p.y : V3<R>();
        return Ray<R>{center + off, ((p00_rel + du * sx) + dv * sy) - off, time};
    }
    Ray<R> ray_for_pixel_sample(uint32_t x, uint32_t y, SampleRng& rng) const {
        R ox = rng.random_double<R>() - R(0.5);
        R oy = rng.random_double<R>() - R(0.5);
        return finish_ray(R(x) + ox, R(y) + oy, rng);
    }
    Ray<R> ray_for_pixel_stratified(uint32_t x, uint32_t y, uint32_t sx, uint32_t sy, uint32_t g,
                                    SampleRng& rng) const { // camera.rs:1672-1704
        R rec = R(1) / R(g);
        R ox = ((R(sx) + rng.random_double<R>()) * rec) - R(0.5);
        R oy = ((R(sy) + rng.random_double<R>()) * rec) - R(0.5);
        return finish_ray(R(x) + ox, R(y) + oy, rng);
    }
};

// RayBackground::radiance (camera.rs:301-322).
template <class R> inline V3<R> background_radiance(const gt_camera_desc& d, V3<R> dir) {
    if (d.background_kind == GT_BG_CONSTANT) return v3<R>(d.background);
    V3<R> nadir = v3<R>(d.background), horizon = v3<R>(d.background + 3), zenith = v3<R>(d.background + 6);
    R t = R(0.5) * (normalized(dir).y + R(1));
    if (t < R(0.5)) {
        R b = R(2) * t;
        return nadir * (R(1) - b) + horizon * b;
    }
    R b = R(2) * (t - R(0.5));
    return horizon * (R(1) - b) + zenith * b;
}

// RayCamera::power_heuristic (camera.rs:2486-2496).
template <class R> inline R power_heuristic(R a, R b) {
    if (!std::isfinite(a) || a <= R(kEps)) return R(0);
    if (!std::isfinite(b) || b <= R(kEps)) return R(1);
    R sa = a * a, sb = b * b;
    return sa / (sa + sb);
}

// ------------------------------------------------------------------ renderer
template <class R> struct Renderer {
    const Scene<R>* scene = nullptr;
    const LightList<R>* lights = nullptr; // nullptr = None
    const Environment<R>* env = nullptr;  // nullptr = None
    Camera<R> cam;
    bool nee = false;
    R light_pdf_weight{0.5};
    int rr_min_depth = 5;
    // Throughput mode: every sample draws from its own (pixel, sample) substream instead
    // of continuing the pixel's one stream (statistically equivalent, not stream-identical).
    bool substreams = false;

    void setup(const gt_camera_desc& d) {
        cam.init(d);
        // The environment entry points force NEE (camera.rs:4171-4173), which also sets
        // light_pdf_weight to 0 via SamplingStrategy::next_event_estimation (camera.rs:75-80).
        nee = d.direct_lighting_mode == GT_DIRECT_NEXT_EVENT_ESTIMATION || env != nullptr;
        light_pdf_weight = nee ? R(0) : rclamp(R(d.light_pdf_weight), R(0), R(1));
        rr_min_depth = d.russian_roulette_min_depth;
    }

    bool rr_survives(uint32_t bounce, V3<R>& att, SampleRng& rng) const { // camera.rs:2498-2523
        if (rr_min_depth < 0 || bounce < uint32_t(rr_min_depth)) return true;
        R m = max_component(att);
        if (!std::isfinite(m) || m <= R(kEps)) {
            trace_note(TR_RR, 2, double(m));
            return false;
        }
        R p = rclamp(m, R(kRrMin), R(kRrMax));
        const R u = rng.random_double<R>();
        trace_note(TR_RR, u >= p ? 0 : 1, double(u) - double(p));
        if (u >= p) return false;
        att = cdiv(att, p);
        return true;
    }

    V3<R> miss_radiance(V3<R> dir) const {
        if (env) return env->radiance(dir);
        return background_radiance<R>(cam.desc, dir);
    }

    // RayCamera::ray_color (camera.rs:1730-1862).
    V3<R> ray_color(Ray<R> ray, SampleRng& rng) const {
        V3<R> att(1, 1, 1), color;
        bool allow_emitted = true;
        R miss_w = R(1);
        const R inf = std::numeric_limits<R>::infinity();
        for (uint32_t bounce = 0; bounce < cam.desc.max_depth; ++bounce) {
            Hit<R> rec;
            if (!scene->world_hit(ray, R(kShadowAcne), inf, rec, rng)) {
                trace_note(TR_HIT, -1);
                V3<R> miss = miss_radiance(ray.d) * miss_w;
                return color + cmul(att, miss);
            }
            trace_note(TR_HIT, rec.prim, double(rec.margin));
            const Material<R>& m = scene->materials[rec.material];
            if (allow_emitted) color = color + cmul(att, emitted(m, rec));
            Scatter<R> s = scatter(m, ray, rec, rng);
            trace_note(TR_SCATTER, int32_t(s.kind));
            if (s.kind == SCATTER_NONE) return color;
            if (s.kind == SCATTER_SPECULAR) {
                att = cmul(att, s.att);
                ray = s.ray;
                allow_emitted = true;
                miss_w = R(1);
                if (!rr_survives(bounce, att, rng)) return color;
                continue;
            }
            if (nee) {
                // Both shadow rays of a bounce leave from one origin: the side of the area
                // light's direction when that sample is valid, else the environment's.
                const V3<R>* area_dir = nullptr;
                V3<R> adir;
                if (lights) color = color + cmul(att, direct_lighting(ray, rec, m, s.att, rng, adir, area_dir));
                if (env) color = color + cmul(att, environment_lighting(ray, rec, m, s.att, rng, area_dir));
            }
            // SamplingStrategy::continuation_sample (camera.rs:165-195)
            V3<R> dir;
            R pdf;
            bool suppress = false, weight_env = false;
            if (!nee && lights) {
                R w = light_pdf_weight;
                const R u = rng.random_double<R>();
                trace_note(TR_MIXTURE, u < w ? 1 : 0, double(u) - double(w));
                if (u < w)
                    dir = lights->random_direction(rec.point, ray.time, rng);
                else
                    dir = s.pdf.generate(rng);
                pdf = w * lights->pdf_value(rec.point, ray.time, dir) + (R(1) - w) * s.pdf.value(dir);
            } else {
                dir = s.pdf.generate(rng);
                pdf = s.pdf.value(dir);
                suppress = nee && lights;
                weight_env = nee && env;
            }
            if (!std::isfinite(pdf) || pdf <= R(kEps)) {
                trace_note(TR_PDF, 0, double(pdf));
                return color;
            }
            Ray<R> scattered{spawn_origin(rec, dir), dir, ray.time};
            R sp = scattering_pdf(m, ray, rec, dir);
            if (!std::isfinite(sp) || sp <= R(0)) {
                trace_note(TR_PDF, 1, double(sp));
                return color;
            }
            R next_miss_w = R(1);
            if (weight_env && env) next_miss_w = power_heuristic(pdf, env->pdf_value(dir));
            att = cmul(att, s.att * (sp / pdf));
            trace_note(TR_THROUGHPUT, 0, double(max_component(att)));
            ray = scattered;
            allow_emitted = !suppress;
            miss_w = next_miss_w;
            if (!rr_survives(bounce, att, rng)) return color;
        }
        return color;
    }

    // estimate_direct_lighting (camera.rs:2225-2262).
    // valid_dir is set to &dir_out when the sample passes both pdf tests (its shadow ray is
    // traced).
    V3<R> direct_lighting(const Ray<R>& in, const Hit<R>& rec, const Material<R>& m, V3<R> satt, SampleRng& rng,
                          V3<R>& dir_out, const V3<R>*& valid_dir) const {
        V3<R> dir = lights->random_direction(rec.point, in.time, rng);
        R lp = lights->pdf_value(rec.point, in.time, dir);
        if (!std::isfinite(lp) || lp <= R(kEps)) {
            trace_note(TR_NEE_AREA, -3, double(lp));
            return V3<R>();
        }
        Ray<R> shadow{spawn_origin(rec, dir), dir, in.time};
        R sp = scattering_pdf(m, in, rec, dir);
        if (!std::isfinite(sp) || sp <= R(0)) {
            trace_note(TR_NEE_AREA, -3, double(sp));
            return V3<R>();
        }
        dir_out = dir;
        valid_dir = &dir_out;
        Hit<R> lh;
        const bool lit = scene->world_hit(shadow, R(kShadowAcne), std::numeric_limits<R>::infinity(), lh, rng);
        trace_note(TR_NEE_AREA, lit ? lh.prim : -1, lit ? double(lh.margin) : 1.0);
        if (!lit) return V3<R>();
        V3<R> e = emitted(scene->materials[lh.material], lh);
        if (!finite3(e)) return V3<R>();
        return cmul(satt, e) * (sp / lp);
    }

    // estimate_environment_lighting (camera.rs:2264-2297).
    V3<R> environment_lighting(const Ray<R>& in, const Hit<R>& rec, const Material<R>& m, V3<R> satt,
                               SampleRng& rng, const V3<R>* area_dir) const {
        V3<R> dir;
        R ep;
        env->sample_direction(rng, dir, ep);
        if (!std::isfinite(ep) || ep <= R(kEps)) {
            trace_note(TR_NEE_ENV, -3, double(ep));
            return V3<R>();
        }
        Ray<R> shadow{spawn_origin(rec, area_dir ? *area_dir : dir), dir, in.time};
        R sp = scattering_pdf(m, in, rec, dir);
        if (!std::isfinite(sp) || sp <= R(0)) {
            trace_note(TR_NEE_ENV, -3, double(sp));
            return V3<R>();
        }
        R mis = power_heuristic(ep, sp);
        Hit<R> sh;
        const bool occluded = scene->world_hit(shadow, R(kShadowAcne), std::numeric_limits<R>::infinity(), sh, rng);
        trace_note(TR_NEE_ENV, occluded ? 0 : 1, occluded ? double(sh.margin) : 1.0);
        if (occluded) return V3<R>();
        return cmul(satt, env->radiance(dir)) * (mis * sp / ep);
    }

    // render_world_linear_pixel_with_context (camera.rs:2660-2723) plus adaptive
    // sampling (2937-2982).  Returns the pixel colour and the accepted-sample count.
    V3<R> pixel(uint32_t x, uint32_t y, uint32_t& accepted) const {
        const uint64_t seed = pixel_seed(cam.desc.rng_seed, x, y);
        SampleRng rng(seed);
        // Sample i's stream: the pixel's, continued; or its own substream.
        auto start_sample = [&](uint32_t i) {
            if (substreams) rng = SampleRng(seed ^ sample_key(i));
        };
        V3<R> sum;
        accepted = 0;
        if (cam.desc.pixel_sample_mode == GT_SAMPLE_RANDOM) {
            if (cam.desc.adaptive) {
                uint32_t mn = std::max<uint32_t>(cam.desc.adaptive_min_samples, 1u);
                uint32_t mx = std::max<uint32_t>(cam.desc.adaptive_max_samples, mn);
                V3<R> mean, m2;
                for (uint32_t i = 0; i < mx; ++i) {
                    start_sample(i);
                    V3<R> s = ray_color(cam.ray_for_pixel_sample(x, y, rng), rng);
                    trace_note(TR_SAMPLE, finite3(s) ? 1 : 0, finite3(s) ? double(s.x + s.y + s.z) : 0.0);
                    if (!finite3(s)) continue;
                    accepted += 1;
                    R count = R(accepted);
                    V3<R> delta = s - mean;
                    mean = mean + cdiv(delta, count);
                    V3<R> delta2 = s - mean;
                    m2 = m2 + cmul(delta, delta2);
                    if (accepted >= mn) {
                        const R err = adaptive_error(m2, accepted), thr = R(cam.desc.adaptive_error_threshold);
                        trace_note(TR_ADAPTIVE, err < thr ? 1 : 0, thr > R(0) ? double((err - thr) / thr) : double(err));
                        if (err < thr) break;
                    }
                }
                return mean;
            }
            for (uint32_t i = 0; i < cam.desc.samples_per_pixel; ++i) {
                start_sample(i);
                V3<R> s = ray_color(cam.ray_for_pixel_sample(x, y, rng), rng);
                trace_note(TR_SAMPLE, finite3(s) ? 1 : 0, finite3(s) ? double(s.x + s.y + s.z) : 0.0);
                if (finite3(s)) {
                    sum = sum + s;
                    accepted += 1;
                }
            }
        } else {
            uint32_t g = cam.grid_width();
            for (uint32_t sy = 0; sy < g; ++sy)
                for (uint32_t sx = 0; sx < g; ++sx) {
                    start_sample(sy * g + sx);
                    V3<R> s = ray_color(cam.ray_for_pixel_stratified(x, y, sx, sy, g, rng), rng);
                    trace_note(TR_SAMPLE, finite3(s) ? 1 : 0, finite3(s) ? double(s.x + s.y + s.z) : 0.0);
                    if (finite3(s)) {
                        sum = sum + s;
                        accepted += 1;
                    }
                }
        }
        return accepted == 0 ? V3<R>() : cdiv(sum, R(accepted)); // camera.rs:2984-2999
    }

    static R adaptive_error(V3<R> m2, uint32_t n) { // camera.rs:2962-2972
        if (n <= 1) return std::numeric_limits<R>::infinity();
        V3<R> var = cdiv(m2, R(n - 1));
        return std::sqrt(rmax(max_component(cdiv(var, R(n))), R(0)));
    }

    // render_denoising_aov_linear_pixel (camera.rs:3064-3116): kind 0 = albedo, 1 = normal.
    V3<R> aov_pixel(uint32_t x, uint32_t y, int kind) const {
        SampleRng rng(pixel_seed(cam.desc.rng_seed, x, y));
        V3<R> sum;
        uint32_t n = cam.effective_spp();
        auto sample = [&](const Ray<R>& ray) {
            Hit<R> rec;
            if (!scene->world_hit(ray, R(kShadowAcne), std::numeric_limits<R>::infinity(), rec, rng)) return V3<R>();
            if (kind == 0) return denoise_albedo(scene->materials[rec.material], rec);
            return (rec.shading + V3<R>(1, 1, 1)) * R(0.5);
        };
        if (cam.desc.pixel_sample_mode == GT_SAMPLE_RANDOM) {
            for (uint32_t i = 0; i < n; ++i) sum = sum + sample(cam.ray_for_pixel_sample(x, y, rng));
        } else {
            uint32_t g = cam.grid_width();
            for (uint32_t sy = 0; sy < g; ++sy)
                for (uint32_t sx = 0; sx < g; ++sx) sum = sum + sample(cam.ray_for_pixel_stratified(x, y, sx, sy, g, rng));
        }
        return cdiv(sum, R(n));
    }

    // Tiled render over a std::thread pool (render_values_tiled, camera.rs:3134-3170).
    template <class F> void for_tiles(uint32_t threads, F&& fn) const {
        const uint32_t tile = 16;
        uint32_t tx = (cam.width + tile - 1) / tile, ty = (cam.height + tile - 1) / tile;
        uint32_t total = tx * ty;
        std::atomic<uint32_t> next{0};
        auto worker = [&]() {
            for (;;) {
                uint32_t t = next.fetch_add(1);
                if (t >= total) return;
                uint32_t x0 = (t % tx) * tile, y0 = (t / tx) * tile;
                for (uint32_t y = y0; y < std::min(y0 + tile, cam.height); ++y)
                    for (uint32_t x = x0; x < std::min(x0 + tile, cam.width); ++x) fn(x, y);
            }
        };
        if (threads <= 1) {
            worker();
            return;
        }
        std::vector<std::thread> pool;
        for (uint32_t i = 0; i < threads; ++i) pool.emplace_back(worker);
        for (auto& t : pool) t.join();
    }
};

} // namespace oracle
