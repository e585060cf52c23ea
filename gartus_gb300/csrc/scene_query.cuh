// scene_query.cuh — device-side scene queries: BVH traversal (with the reference's
// visiting order and statistics), primitive intersection, hit records, materials,
// sampling targets, the environment light and camera rays.
#pragma once

#include "device_math.cuh"

namespace gt {

// Vector loads of 4 scalars (one LDG.128 in f32, two in f64).
template <class R> GT_DEV R4<R> ld4(const R* p) { return *reinterpret_cast<const R4<R>*>(p); }
template <class R> GT_DEV R4<R> ldg4(const R* p);
template <> GT_DEV R4<float> ldg4<float>(const float* p) {
    float4 v = __ldg(reinterpret_cast<const float4*>(p));
    return R4<float>{v.x, v.y, v.z, v.w};
}
template <> GT_DEV R4<double> ldg4<double>(const double* p) {
    double2 a = __ldg(reinterpret_cast<const double2*>(p));
    double2 b = __ldg(reinterpret_cast<const double2*>(p) + 1);
    return R4<double>{a.x, a.y, b.x, b.y};
}
template <class R> GT_DEV V3<R> xyz(R4<R> v) { return V3<R>{v.x, v.y, v.z}; }

// The f32 slab test widens the exit distance by 1 + 2*gamma(3) (gamma(n) = n u / (1 - n u),
// u = 2^-24) so rounding never culls a box the ray passes through (Ize, "Robust BVH Ray
// Traversal", JCGT 2013).  The f64 test is the reference's exactly (bvh.rs:119-146).
template <class R> struct SlabPad;
template <> struct SlabPad<float> {
    static GT_DEV float pad(float t) { return t * 1.00000036f; }
};
template <> struct SlabPad<double> {
    static GT_DEV double pad(double t) { return t; }
};

template <class R> struct RayT {
    R o[3], inv[3];
    bool par[3];
};
template <class R> GT_DEV RayT<R> make_rayt(V3<R> o, V3<R> d) { // RayTraversal::new, bvh.rs:99-117
    RayT<R> r;
    R dd[3] = {d.x, d.y, d.z};
    r.o[0] = o.x;
    r.o[1] = o.y;
    r.o[2] = o.z;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        r.par[i] = Num<R>::fabs(dd[i]) <= R(kEps);
        r.inv[i] = r.par[i] ? R(0) : R(1) / dd[i];
    }
    return r;
}
// RayTraversal::hit_bounds (bvh.rs:119-146): box = {min xyz, max xyz}.
template <class R> GT_DEV bool hit_box(const RayT<R>& r, const R* mn, const R* mx, R tmin, R tmax, R& entry) {
    R en = tmin, ex = tmax;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (r.par[a]) {
            if (r.o[a] < mn[a] || r.o[a] > mx[a]) return false;
            continue;
        }
        R t0 = (mn[a] - r.o[a]) * r.inv[a];
        R t1 = (mx[a] - r.o[a]) * r.inv[a];
        if (r.inv[a] < R(0)) {
            R tmp = t0;
            t0 = t1;
            t1 = tmp;
        }
        en = Num<R>::fmax(en, t0);
        ex = Num<R>::fmin(ex, SlabPad<R>::pad(t1));
        if (ex <= en) return false;
    }
    entry = en;
    return true;
}

// --------------------------------------------------------------- intersection
template <class R> GT_DEV bool sphere_root(V3<R> center, R radius, V3<R> o, V3<R> d, R tmin, R tmax, R& root) {
    V3<R> oc = center - o; // hit_sphere_in_interval, object.rs:986-1013
    R a = len2(d);
    if (a <= R(kEps)) return false;
    R h = dot(d, oc);
    R c = len2(oc) - radius * radius;
    R disc = h * h - a * c;
    if (disc < R(0)) return false;
    R sq = Num<R>::sqrt(disc);
    R first = (h - sq) / a;
    if (tmin < first && first < tmax) {
        root = first;
        return true;
    }
    R second = (h + sq) / a;
    if (tmin < second && second < tmax) {
        root = second;
        return true;
    }
    return false;
}

// f32: the same roots with less rounding.  The discriminant is a (r^2 - |l|^2) with
// l = oc - (h / a) d, the centre's offset from the ray's closest approach (Haines,
// Guenther, Akenine-Moeller, "Precision Improvements for Ray/Sphere Intersection", Ray
// Tracing Gems, 2019): the reference's h^2 - a c cancels when a sphere is small against
// its distance, which moved f32 hit normals by ~1e-3 on the final scene's small spheres.
// c = |oc|^2 - r^2 keeps its products' rounding errors (two-product) and its sums' (two-
// sum), so it stays accurate near a large sphere, and each root comes from the
// cancellation-free form (q = h + sign(h) sqrt(disc): roots c / q and q / a).  In exact
// arithmetic these are the reference's roots, tested in the reference's order.  The
// products whose errors are recovered use __fmul_rn so that no multiply-add absorbs them.
GT_DEV float two_sum_err(float a, float b, float s) {
    const float bb = __fsub_rn(s, a);
    return __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
template <> GT_DEV bool sphere_root<float>(V3<float> center, float radius, V3<float> o, V3<float> d, float tmin,
                                           float tmax, float& root) {
    const V3<float> oc = center - o;
    const float a = len2(d);
    if (a <= float(kEps)) return false;
    const float h = dot(d, oc);
    const float tc = h / a;
    const V3<float> l{__fmaf_rn(-d.x, tc, oc.x), __fmaf_rn(-d.y, tc, oc.y), __fmaf_rn(-d.z, tc, oc.z)};
    const float disc_a = __fmaf_rn(radius, radius, -len2(l));
    if (disc_a < 0.0f) return false;
    const float px = __fmul_rn(oc.x, oc.x), py = __fmul_rn(oc.y, oc.y), pz = __fmul_rn(oc.z, oc.z);
    const float rr = __fmul_rn(radius, radius);
    const float e = __fadd_rn(__fadd_rn(__fmaf_rn(oc.x, oc.x, -px), __fmaf_rn(oc.y, oc.y, -py)),
                              __fsub_rn(__fmaf_rn(oc.z, oc.z, -pz), __fmaf_rn(radius, radius, -rr)));
    const float s1 = __fadd_rn(px, py), s2 = __fadd_rn(s1, pz), s3 = __fsub_rn(s2, rr);
    const float c = __fadd_rn(s3, __fadd_rn(__fadd_rn(__fadd_rn(two_sum_err(px, py, s1), two_sum_err(s1, pz, s2)),
                                                      two_sum_err(s2, -rr, s3)),
                                            e));
    const float sq = sqrtf(a * disc_a);
    const float q = h >= 0.0f ? h + sq : h - sq;
    float first, second;
    if (q == 0.0f) {
        first = second = 0.0f;
    } else if (h >= 0.0f) {
        first = c / q;
        second = q / a;
    } else {
        first = q / a;
        second = c / q;
    }
    if (tmin < first && first < tmax) {
        root = first;
        return true;
    }
    if (tmin < second && second < tmax) {
        root = second;
        return true;
    }
    return false;
}

// Möller–Trumbore with the reference's tolerances (geometry.rs:239-265), edges given.
template <class R> GT_DEV bool tri_hit(V3<R> p0, V3<R> e1, V3<R> e2, V3<R> o, V3<R> d, R tmin, R tmax, R& t) {
    V3<R> pvec = cross(d, e2);
    R det = dot(e1, pvec);
    if (Num<R>::fabs(det) < R(kTriHitEps)) return false;
    R inv_det = R(1) / det;
    V3<R> tvec = o - p0;
    R u = dot(tvec, pvec) * inv_det;
    if (!(u >= R(0) && u <= R(1))) return false;
    V3<R> qvec = cross(tvec, e1);
    R v = dot(d, qvec) * inv_det;
    if (v < R(0) || u + v > R(1)) return false;
    t = dot(e2, qvec) * inv_det;
    return tmin < t && t < tmax;
}

// QuadGeometry::hit_ray (geometry.rs:394-415); the degenerate-area test is folded into
// the K_NEVER kind at upload.
template <class R> GT_DEV bool quad_hit(V3<R> corner, V3<R> u, V3<R> v, V3<R> n, V3<R> w, R plane_d, V3<R> o,
                                        V3<R> d, R tmin, R tmax, R& t) {
    R denom = dot(n, d);
    if (Num<R>::fabs(denom) < R(kQuadHitEps)) return false;
    t = (plane_d - dot(n, o)) / denom;
    if (!(tmin < t && t < tmax)) return false;
    V3<R> planar = (o + d * t) - corner;
    R a = dot(w, cross(planar, v));
    R b = dot(w, cross(u, planar));
    return (a >= R(0) && a <= R(1)) && (b >= R(0) && b <= R(1));
}

// RayGeometry::intersect for leaf-order primitive `i` (object.rs:338-346).
template <class R> GT_DEV bool prim_hit(const SceneDev<R>& sc, uint32_t i, V3<R> o, V3<R> d, R time, R tmin, R tmax,
                                        R& t) {
    const uint32_t kind = __ldg(&sc.meta[i].x) & 7u;
    const R* rec = sc.prims[i].v;
    switch (kind) {
    case K_SPHERE: {
        R4<R> s = ldg4(rec);
        return sphere_root(xyz(s), s.w, o, d, tmin, tmax, t);
    }
    case K_MOVING: {
        R4<R> s = ldg4(rec), dl = ldg4(rec + 4);
        V3<R> c = xyz(s) + xyz(dl) * time; // center_at, geometry.rs:510-513
        return sphere_root(c, s.w, o, d, tmin, tmax, t);
    }
    case K_TRIANGLE: {
        R4<R> a = ldg4(rec), b = ldg4(rec + 4), c = ldg4(rec + 8);
        return tri_hit(xyz(a), xyz(b), xyz(c), o, d, tmin, tmax, t);
    }
    case K_QUAD: {
        R4<R> a = ldg4(rec), b = ldg4(rec + 4), c = ldg4(rec + 8), e = ldg4(rec + 12);
        return quad_hit(xyz(a), xyz(b), xyz(c), V3<R>{b.w, c.w, e.w}, xyz(e), a.w, o, d, tmin, tmax, t);
    }
    default:
        return false;
    }
}

// The closest hit of a scene of at most 32 primitives for one warp whose lanes all trace
// the same ray (a path finished cooperatively): lane i tests leaf-order primitive i with
// the traversal's own prim_hit, then a warp arg-min (ties to the lower index) replaces the
// serial walk of the tree, whose dependent steps a lone warp cannot hide.  Only the
// order of visits differs from the traversal: exactly equal distances may resolve to
// another primitive.  Returns the primitive (all lanes) or -1; sets t_out on a hit.
template <class R>
GT_DEV int warp_closest(const SceneDev<R>& sc, V3<R> o, V3<R> d, R time, R tmin, R tmax, R& t_out) {
    const uint32_t lane = threadIdx.x & 31u;
    R t = tmax;
    int best = -1;
    if (lane < sc.num_prims) {
        R th;
        if (prim_hit(sc, lane, o, d, time, tmin, tmax, th)) {
            t = th;
            best = int(lane);
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const R ot = __shfl_xor_sync(0xffffffffu, t, off);
        const int ob = __shfl_xor_sync(0xffffffffu, best, off);
        if (ob >= 0 && (best < 0 || ot < t || (ot == t && ob < best))) {
            t = ot;
            best = ob;
        }
    }
    if (best >= 0) t_out = t;
    return best;
}

struct TraceStats {
    unsigned long long node_tests, node_hits, leaf_visits, candidates, leaf_hits;
    uint32_t max_depth;
};

constexpr int kStackSize = 64;

// ----------------------------------------------------------- near-decision test
// Check mode only: whether f32 rounding could change primitive i's hit decision for this
// ray — its hit point within a few dozen f32 ulps (of the coordinates involved, scaled up
// at grazing angles) of an edge, a determinant or plane angle near the reference's
// rejection threshold, a sphere root near the tangent, or a distance near t_min.  Rays
// with such a candidate (up to `tlim`) are re-traced in f64.
template <class R> GT_DEV R amax3(V3<R> a) {
    return Num<R>::fmax(Num<R>::fmax(Num<R>::fabs(a.x), Num<R>::fabs(a.y)), Num<R>::fabs(a.z));
}
template <class R>
GT_DEV bool prim_near(const SceneDev<R>& sc, uint32_t i, V3<R> o, V3<R> d, R time, R tmin, R tlim) {
    constexpr float kUlps = 64.0f * 5.9604645e-8f; // 64 units of 2^-24
    const uint32_t kind = __ldg(&sc.meta[i].x) & 7u;
    const R* rec = sc.prims[i].v;
    const R dl = Num<R>::sqrt(len2(d));
    if (!(dl > R(0))) return false;
    if (kind == K_TRIANGLE) {
        const V3<R> p0 = xyz(ldg4(rec)), e1 = xyz(ldg4(rec + 4)), e2 = xyz(ldg4(rec + 8));
        const V3<R> pvec = cross(d, e2);
        const R det = dot(e1, pvec);
        const R nl = Num<R>::sqrt(len2(cross(e1, e2)));
        if (Num<R>::fabs(det) < R(4e-10)) return true;
        const R inv = R(1) / det;
        const V3<R> tv = o - p0;
        const R u = dot(tv, pvec) * inv;
        const V3<R> qv = cross(tv, e1);
        const R v = dot(d, qv) * inv;
        const R t = dot(e2, qv) * inv;
        const R w = R(1) - u - v;
        const R graze = nl * dl / Num<R>::fabs(det); // 1 / |cos| of the ray against the plane
        const R tol = R(kUlps) * (amax3(o) + Num<R>::fabs(t) * amax3(d) + amax3(p0)) * R(1.7320508) * graze;
        const R hu = nl / Num<R>::sqrt(len2(e2)), hv = nl / Num<R>::sqrt(len2(e1)), hw = nl / Num<R>::sqrt(len2(e2 - e1));
        const R du = u * hu, dv = v * hv, dw = w * hw;
        if (!(du > -tol && dv > -tol && dw > -tol)) return false;
        const R ttol = tol / dl;
        if (!(t > tmin - ttol && t < tlim + ttol)) return false;
        const R edge = Num<R>::fmin(Num<R>::fmin(Num<R>::fabs(du), Num<R>::fabs(dv)), Num<R>::fabs(dw));
        return edge < tol || Num<R>::fabs(t - tmin) < ttol;
    }
    if (kind == K_SPHERE || kind == K_MOVING) {
        R4<R> sp = ldg4(rec);
        V3<R> c = xyz(sp);
        if (kind == K_MOVING) c = c + xyz(ldg4(rec + 4)) * time;
        const V3<R> oc = c - o;
        const R a = len2(d);
        const R h = dot(d, oc);
        const R l2 = len2(oc);
        const R cc = l2 - sp.w * sp.w;
        const R disc = h * h - a * cc;
        const R scale = h * h + a * (l2 + sp.w * sp.w);
        const R ttol = R(kUlps) * (Num<R>::fabs(h) + Num<R>::sqrt(Num<R>::fabs(disc)) + Num<R>::sqrt(scale)) / a +
                       R(kUlps) * (amax3(o) + amax3(c) + Num<R>::fabs(sp.w)) / dl;
        if (Num<R>::fabs(disc) <= R(kUlps) * scale) { // tangent: both roots near h / a
            const R tm = h / a;
            return tm > tmin - ttol && tm < tlim + ttol;
        }
        if (disc < R(0)) return false;
        const R sq = Num<R>::sqrt(disc);
        const R r1 = (h - sq) / a, r2 = (h + sq) / a;
        return Num<R>::fabs(r1 - tmin) < ttol || Num<R>::fabs(r2 - tmin) < ttol;
    }
    if (kind == K_QUAD) {
        R4<R> A = ldg4(rec), B = ldg4(rec + 4), Cq = ldg4(rec + 8), E = ldg4(rec + 12);
        const V3<R> corner = xyz(A), u = xyz(B), v = xyz(Cq), w = xyz(E), n = V3<R>{B.w, Cq.w, E.w};
        const R denom = dot(n, d);
        if (Num<R>::fabs(denom) < R(2e-8)) return true;
        const R t = (A.w - dot(n, o)) / denom;
        const V3<R> planar = (o + d * t) - corner;
        const R al = dot(w, cross(planar, v));
        const R be = dot(w, cross(u, planar));
        const R uxv = R(1) / Num<R>::sqrt(len2(w));
        const R ha = uxv / Num<R>::sqrt(len2(v)), hb = uxv / Num<R>::sqrt(len2(u));
        const R graze = dl / Num<R>::fabs(denom);
        const R tol = R(kUlps) * (amax3(o) + Num<R>::fabs(t) * amax3(d) + amax3(corner)) * R(1.7320508) * graze;
        const R d0 = al * ha, d1 = (R(1) - al) * ha, d2 = be * hb, d3 = (R(1) - be) * hb;
        if (!(d0 > -tol && d1 > -tol && d2 > -tol && d3 > -tol)) return false;
        const R ttol = tol / dl;
        if (!(t > tmin - ttol && t < tlim + ttol)) return false;
        const R edge = Num<R>::fmin(Num<R>::fmin(Num<R>::fabs(d0), Num<R>::fabs(d1)),
                                    Num<R>::fmin(Num<R>::fabs(d2), Num<R>::fabs(d3)));
        return edge < tol || Num<R>::fabs(t - tmin) < ttol;
    }
    return false;
}

// Estimated absolute error of the f32 distance t at which ray (o, d) meets primitive i
// (eight ulps of the quantities the distance is computed from: large for a big sphere
// seen at a distance, whose root suffers cancellation, and at grazing angles).
template <class R> GT_DEV R prim_t_err(const SceneDev<R>& sc, uint32_t i, V3<R> o, V3<R> d, R time, R t) {
    constexpr float kUlps = 8.0f * 5.9604645e-8f;
    const uint32_t kind = __ldg(&sc.meta[i].x) & 7u;
    const R* rec = sc.prims[i].v;
    const R dl = Num<R>::sqrt(len2(d));
    const R pos = amax3(o) + Num<R>::fabs(t) * amax3(d);
    if (kind == K_SPHERE || kind == K_MOVING) {
        R4<R> sp = ldg4(rec);
        V3<R> c = xyz(sp);
        if (kind == K_MOVING) c = c + xyz(ldg4(rec + 4)) * time;
        const V3<R> oc = c - o;
        const R a = len2(d), h = dot(d, oc), l2 = len2(oc);
        const R disc = Num<R>::fabs(h * h - a * (l2 - sp.w * sp.w));
        const R ddisc = R(kUlps) * (h * h + a * (l2 + sp.w * sp.w));
        const R dh = R(kUlps) * dl * (Num<R>::sqrt(l2) + amax3(c));
        return (dh + ddisc / (R(2) * Num<R>::sqrt(Num<R>::fmax(disc, ddisc)))) / a + R(kUlps) * (pos + amax3(c)) / dl;
    }
    if (kind == K_TRIANGLE) {
        const V3<R> p0 = xyz(ldg4(rec)), e1 = xyz(ldg4(rec + 4)), e2 = xyz(ldg4(rec + 8));
        const R det = Num<R>::fabs(dot(e1, cross(d, e2)));
        const R graze = Num<R>::sqrt(len2(cross(e1, e2))) * dl / Num<R>::fmax(det, R(1e-30));
        return R(kUlps) * (pos + amax3(p0)) * R(1.7320508) * graze / dl;
    }
    if (kind == K_QUAD) {
        R4<R> A = ldg4(rec), B = ldg4(rec + 4), Cq = ldg4(rec + 8), E = ldg4(rec + 12);
        const V3<R> n = V3<R>{B.w, Cq.w, E.w};
        const R denom = Num<R>::fmax(Num<R>::fabs(dot(n, d)), R(1e-30));
        return R(kUlps) * (Num<R>::fabs(A.w) + amax3(o) + pos + amax3(xyz(A))) * R(1.7320508) / denom;
    }
    return R(0);
}

// Check mode state of one ray: whether a near decision was seen, and the estimated error
// of the closest distance so far.
template <class R> struct CheckState {
    bool near;
    R best_err;
};

// Check mode's culling distance: boxes are visited up to this far beyond the closest hit,
// so that candidates whose distance may tie with it within f32 error are tested.
template <class R> GT_DEV R check_limit(R closest, R best_err) {
    return closest + Num<R>::fabs(closest) * R(0.00390625) + R(4) * best_err;
}

// One leaf primitive against the running closest hit.  Rendering: the reference's
// interval (t_min, closest).  Check mode: the same decision (a primitive replaces the
// closest only when nearer), plus the near flag when the two distances lie within their
// estimated f32 errors (or 2^-16 relative) of each other, and for near-boundary candidates.
template <class R, bool CHECK>
GT_DEV bool leaf_test(const SceneDev<R>& sc, uint32_t i, V3<R> o, V3<R> d, R time, R tmin, R& closest,
                      CheckState<R>* ck) {
    R t;
    if constexpr (!CHECK) {
        if (prim_hit(sc, i, o, d, time, tmin, closest, t)) {
            closest = t;
            return true;
        }
        return false;
    } else {
        bool nearer = false;
        const R inf = Num<R>::inf();
        if (prim_hit(sc, i, o, d, time, tmin, inf, t)) {
            const R e = prim_t_err(sc, i, o, d, time, t);
            const R window = R(2) * (e + ck->best_err) + Num<R>::fabs(t) * R(1.52587890625e-5);
            if (t < closest) {
                if (closest < inf && closest - t <= window) ck->near = true;
                closest = t;
                ck->best_err = e;
                nearer = true;
            } else if (t - closest <= window) {
                ck->near = true;
            }
        }
        if (!ck->near && prim_near(sc, i, o, d, time, tmin, check_limit(closest, ck->best_err))) ck->near = true;
        return nearer;
    }
}

// ----------------------------------------------------- eight-wide traversal (f32)
// Byte k (0-3) of w as an exact float: 0x4B0000kk is 2^23 + kk.
template <int K> GT_DEV float byte_f(uint32_t w) {
    return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7440u | uint32_t(K))) - 8388608.0f;
}

// Closest (or, with any_hit, first) hit over the compressed wide tree, with the same
// semantics as the binary walk below: the same leaf test and interval, boxes that never
// cull a primitive the f32 child box contains.  Per node one box test of up to eight
// children: plane q of axis a lies at p_a + q s_a, so its distance is q (s_a / d_a) +
// (p_a - o_a) / d_a, one fused multiply-add per plane.  The second term's rounding
// (relative to itself, not to the distance) is covered by widening it per node by 4 ulps
// of its own size; the far distance is then widened by 1 + 2^-21 as in the binary test.
// Children are visited nearest-octant first: hit internal children form a group (node
// index of the first child, 8 bits in visiting order, the internal-slot mask) of which
// the first is descended into and the rest wait on a stack of at most kWideStack groups;
// hit leaf children's primitives are tested at once.
template <bool CHECK>
GT_DEV int traverse_wide(const SceneDev<float>& sc, V3<float> o, V3<float> d, float time, float tmin, float tmax,
                         float& t_out, uint32_t* err, bool any_hit, CheckState<float>* ck) {
    const RayT<float> rt = make_rayt(o, d);
    float root_entry;
    if (!hit_box(rt, sc.root_box, sc.root_box + 3, tmin, tmax, root_entry)) return -1;
    const uint32_t oct = (rt.inv[0] < 0.0f ? 1u : 0u) | (rt.inv[1] < 0.0f ? 2u : 0u) | (rt.inv[2] < 0.0f ? 4u : 0u);
    const bool any_par = rt.par[0] || rt.par[1] || rt.par[2];
    uint2 stack[kWideStack];
    int sp = 0;
    uint32_t node = 0;
    float closest = tmax;
    int best = -1;
    for (;;) {
        const uint4* np = reinterpret_cast<const uint4*>(sc.wnodes + node);
        const uint4 c0 = __ldg(np), c1 = __ldg(np + 1), c2 = __ldg(np + 2), c3 = __ldg(np + 3), c4 = __ldg(np + 4);
        const float cull = CHECK ? check_limit(closest, ck->best_err) : closest;
        // Per axis: scale over direction, and the origin term widened for near and far planes.
        float ax[3], bn[3], bf[3];
        const uint32_t pw[3] = {c0.x, c0.y, c0.z};
        const float ov[3] = {o.x, o.y, o.z};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float sa = __uint_as_float(((c0.w >> (8 * a)) & 0xffu) << 23);
            if (rt.par[a]) { // no distance bound from this axis; containment is tested below
                ax[a] = 0.0f;
                bn[a] = -Num<float>::inf();
                bf[a] = Num<float>::inf();
            } else {
                ax[a] = sa * rt.inv[a];
                const float b = (__uint_as_float(pw[a]) - ov[a]) * rt.inv[a];
                const float pad = fabsf(b) * 2.3841858e-7f; // 4 ulps of b
                bn[a] = b - pad;
                bf[a] = b + pad;
            }
        }
        // Near and far plane words per axis (qlo for a positive direction component).
        const bool nx = rt.inv[0] < 0.0f, ny = rt.inv[1] < 0.0f, nz = rt.inv[2] < 0.0f;
        const uint32_t nx0 = nx ? c3.z : c2.x, nx1 = nx ? c3.w : c2.y, fx0 = nx ? c2.x : c3.z, fx1 = nx ? c2.y : c3.w;
        const uint32_t ny0 = ny ? c4.x : c2.z, ny1 = ny ? c4.y : c2.w, fy0 = ny ? c2.z : c4.x, fy1 = ny ? c2.w : c4.y;
        const uint32_t nz0 = nz ? c4.z : c3.x, nz1 = nz ? c4.w : c3.y, fz0 = nz ? c3.x : c4.z, fz1 = nz ? c3.y : c4.w;
        const uint32_t imask = c0.w >> 24;
        const uint32_t meta0 = c1.z, meta1 = c1.w;
        uint32_t hits = 0;
#define GT_WIDE_SLOT(S, WN_X, WF_X, WN_Y, WF_Y, WN_Z, WF_Z)                                                  \
    {                                                                                                     \
        const float tnx = fmaf(byte_f<(S)&3>(WN_X), ax[0], bn[0]), tfx = fmaf(byte_f<(S)&3>(WF_X), ax[0], bf[0]); \
        const float tny = fmaf(byte_f<(S)&3>(WN_Y), ax[1], bn[1]), tfy = fmaf(byte_f<(S)&3>(WF_Y), ax[1], bf[1]); \
        const float tnz = fmaf(byte_f<(S)&3>(WN_Z), ax[2], bn[2]), tfz = fmaf(byte_f<(S)&3>(WF_Z), ax[2], bf[2]); \
        const float en = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, tmin));                                        \
        const float ex = fminf(fminf(fminf(tfx, tfy), tfz) * 1.00000048f, cull);                           \
        hits |= (ex > en ? 1u : 0u) << (S);                                                               \
    }
        GT_WIDE_SLOT(0, nx0, fx0, ny0, fy0, nz0, fz0)
        GT_WIDE_SLOT(1, nx0, fx0, ny0, fy0, nz0, fz0)
        GT_WIDE_SLOT(2, nx0, fx0, ny0, fy0, nz0, fz0)
        GT_WIDE_SLOT(3, nx0, fx0, ny0, fy0, nz0, fz0)
        GT_WIDE_SLOT(4, nx1, fx1, ny1, fy1, nz1, fz1)
        GT_WIDE_SLOT(5, nx1, fx1, ny1, fy1, nz1, fz1)
        GT_WIDE_SLOT(6, nx1, fx1, ny1, fy1, nz1, fz1)
        GT_WIDE_SLOT(7, nx1, fx1, ny1, fy1, nz1, fz1)
#undef GT_WIDE_SLOT
        if (any_par) { // parallel axes: the origin must lie within the slab (one step of slack)
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                if (!rt.par[a]) continue;
                const float sa = __uint_as_float(((c0.w >> (8 * a)) & 0xffu) << 23);
                const float q = (ov[a] - __uint_as_float(pw[a])) / sa;
                const uint32_t lo0 = a == 0 ? c2.x : a == 1 ? c2.z : c3.x, lo1 = a == 0 ? c2.y : a == 1 ? c2.w : c3.y;
                const uint32_t hi0 = a == 0 ? c3.z : a == 1 ? c4.x : c4.z, hi1 = a == 0 ? c3.w : a == 1 ? c4.y : c4.w;
#pragma unroll
                for (int s = 0; s < 8; ++s) {
                    const uint32_t lw = s < 4 ? lo0 : lo1, hw = s < 4 ? hi0 : hi1;
                    const float lo = float((lw >> (8 * (s & 3))) & 0xffu), hi = float((hw >> (8 * (s & 3))) & 0xffu);
                    if (!(q >= lo - 1.0f && q <= hi + 1.0f)) hits &= ~(1u << s);
                }
            }
        }
        // Leaf children: their primitives, at once.
        uint32_t pm = 0;
#pragma unroll
        for (int s = 0; s < 8; ++s) {
            const uint32_t m = ((s < 4 ? meta0 : meta1) >> (8 * (s & 3))) & 0xffu;
            if ((hits >> s) & 1u) pm |= ((1u << (m >> 5)) - 1u) << (m & 31u);
        }
        const uint32_t pbase = c1.y;
        while (pm) {
            const uint32_t k = uint32_t(__ffs(pm)) - 1u;
            pm &= pm - 1u;
            if (leaf_test<float, CHECK>(sc, pbase + k, o, d, time, tmin, closest, ck)) {
                best = int(pbase + k);
                if (any_hit) {
                    t_out = closest;
                    return best;
                }
            }
        }
        // Internal children, in visiting order (bit i = slot i ^ oct).
        const uint32_t ih = hits & imask;
        uint32_t order = 0;
#pragma unroll
        for (int s = 0; s < 8; ++s) order |= ((ih >> s) & 1u) << (uint32_t(s) ^ oct);
        uint32_t gbase, gbits;
        if (order) {
            gbase = c1.x;
            gbits = order | (imask << 8);
            const uint32_t rest = gbits & ~(1u << (__ffs(order) - 1));
            if (rest & 0xffu) {
                if (sp >= int(kWideStack)) {
                    atomicOr(err, E_STACK_OVERFLOW);
                    break;
                }
                stack[sp++] = make_uint2(gbase, rest);
            }
        } else {
            if (sp == 0) break;
            const uint2 top = stack[sp - 1];
            gbase = top.x;
            gbits = top.y;
            const uint32_t rest = gbits & ~(1u << (__ffs(gbits & 0xffu) - 1));
            if (rest & 0xffu)
                stack[sp - 1].y = rest;
            else
                --sp;
        }
        const uint32_t slot = (uint32_t(__ffs(gbits & 0xffu)) - 1u) ^ oct;
        node = gbase + uint32_t(__popc((gbits >> 8) & ((1u << slot) - 1u)));
    }
    t_out = closest;
    return best;
}

// FlatBvh::hit_with_stats (bvh.rs:306-399): root test, LIFO stack of (node, entry t),
// skip entries at or beyond the closest hit, test both children of an internal node and
// push the farther first.  ANY = stop at the first hit (occlusion).  Returns the leaf-
// order primitive index of the closest hit or -1; sets *err on stack overflow.  An f32
// scene with a wide tree is traversed by traverse_wide instead (same result semantics),
// except for the statistics, which are defined by this walk.  CHECK (f32 primary-hit
// check): candidates slightly beyond the closest hit are tested too and *near reports
// near ties and near-boundary candidates in ck; the result is the rendering walk's.
// BINARY: this walk even where the scene has a wide tree.
template <class R, bool STATS, bool ANY, bool CHECK = false, bool BINARY = false>
GT_DEV int traverse(const SceneDev<R>& sc, V3<R> o, V3<R> d, R time, R tmin, R tmax, R& t_out, TraceStats* st,
                    uint32_t* err, bool any_hit = ANY, CheckState<R>* ck = nullptr) {
    if constexpr (sizeof(R) == 4 && !STATS && !BINARY) {
        if (sc.wnodes) return traverse_wide<CHECK>(sc, o, d, time, tmin, tmax, t_out, err, any_hit, ck);
    }
    RayT<R> rt = make_rayt(o, d);
    if (STATS) st->node_tests += 1;
    R root_entry;
    if (!hit_box(rt, sc.root_box, sc.root_box + 3, tmin, tmax, root_entry)) return -1;
    if (STATS) st->node_hits += 1;
    int32_t s_link[kStackSize];
    int32_t s_count[kStackSize];
    R s_t[kStackSize];
    int sp = 0;
    s_link[0] = sc.root_link;
    s_count[0] = sc.root_count;
    s_t[0] = root_entry;
    sp = 1;
    if (STATS) st->max_depth = max(st->max_depth, 1u);
    R closest = tmax;
    int best = -1;
    while (sp > 0) {
        --sp;
        const int32_t link = s_link[sp];
        const int32_t count = s_count[sp];
        const R et = s_t[sp];
        const R cull = CHECK ? check_limit(closest, ck->best_err) : closest;
        if (et >= cull) continue;
        if (link < 0) {
            // hit_ray_scene_indices (scene.rs:849-874) with Interval(t_min, closest).
            const uint32_t first = uint32_t(~link);
            if (STATS) {
                st->leaf_visits += 1;
                st->candidates += uint32_t(count);
            }
            bool leaf_hit = false;
            for (int k = 0; k < count; ++k) {
                if (leaf_test<R, CHECK>(sc, first + k, o, d, time, tmin, closest, ck)) {
                    best = int(first + k);
                    leaf_hit = true;
                    if (any_hit) {
                        t_out = closest;
                        return best;
                    }
                }
            }
            if (STATS && leaf_hit) st->leaf_hits += 1;
            continue;
        }
        const Node<R>& nd = sc.nodes[link];
        R b[12];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            R4<R> v = ldg4(nd.box + 4 * q);
            b[4 * q] = v.x;
            b[4 * q + 1] = v.y;
            b[4 * q + 2] = v.z;
            b[4 * q + 3] = v.w;
        }
        const int4 ln = __ldg(reinterpret_cast<const int4*>(nd.link));
        R le, re;
        const R ccull = CHECK ? check_limit(closest, ck->best_err) : closest;
        const bool lh = hit_box(rt, b, b + 3, tmin, ccull, le);
        const bool rh = hit_box(rt, b + 6, b + 9, tmin, ccull, re);
        if (STATS) {
            st->node_tests += 2;
            st->node_hits += uint32_t(lh) + uint32_t(rh);
        }
        if (sp + 2 > kStackSize) {
            atomicOr(err, E_STACK_OVERFLOW);
            break;
        }
        if (lh && rh) {
            if (re < le) {
                s_link[sp] = ln.x, s_count[sp] = ln.y, s_t[sp] = le, ++sp;
                s_link[sp] = ln.z, s_count[sp] = ln.w, s_t[sp] = re, ++sp;
            } else {
                s_link[sp] = ln.z, s_count[sp] = ln.w, s_t[sp] = re, ++sp;
                s_link[sp] = ln.x, s_count[sp] = ln.y, s_t[sp] = le, ++sp;
            }
        } else if (lh) {
            s_link[sp] = ln.x, s_count[sp] = ln.y, s_t[sp] = le, ++sp;
        } else if (rh) {
            s_link[sp] = ln.z, s_count[sp] = ln.w, s_t[sp] = re, ++sp;
        }
        if (STATS) st->max_depth = max(st->max_depth, uint32_t(sp));
    }
    t_out = closest;
    return best;
}

// ------------------------------------------------------------------ hit record
template <class R> struct HitRec {
    V3<R> p, n; // n oriented against the ray (SurfaceHit::with_uv, object.rs:127-149)
    V3<R> ns;   // shading normal (HitRecord::shading_normal): n except at mesh triangles with
                // vertex normals or a normal map
    R u, v;     // texture coordinates, computed for image-textured materials only
    bool front;
    uint32_t mat;
};
template <class R> GT_DEV HitRec<R> make_hit(const SceneDev<R>& sc, uint32_t i, V3<R> o, V3<R> d, R time, R t) {
    HitRec<R> h;
    const uint32_t m = __ldg(&sc.meta[i].x);
    const uint32_t kind = m & 7u;
    h.mat = m >> 3;
    h.p = o + d * t; // Ray::at
    const R* rec = sc.prims[i].v;
    V3<R> out;
    if (kind == K_SPHERE || kind == K_MOVING) {
        R4<R> s = ldg4(rec);
        V3<R> c = xyz(s);
        if (kind == K_MOVING) c = c + xyz(ldg4(rec + 4)) * time;
        V3<R> diff = h.p - c; // outward_normal_at, geometry.rs:476-484
        out = Num<R>::fabs(s.w) <= R(kEps) ? normalize(diff) : vdiv(diff, s.w);
    } else if (kind == K_TRIANGLE) {
        out = xyz(ldg4(rec + 12));
    } else {
        out = V3<R>{rec[7], rec[11], rec[15]};
    }
    h.front = dot(d, out) < R(0);
    h.n = h.front ? out : -out;
    h.ns = h.n;
    h.u = h.v = R(0);
    if (sc.mats[h.mat].tex == GT_TEX_IMAGE) {
        if (kind == K_SPHERE || kind == K_MOVING) { // sphere_uv, object.rs:1038-1042
            const R theta = Num<R>::acos(-out.y);
            const R phi = Num<R>::atan2(-out.z, out.x) + R(kPi);
            h.u = phi / R(2.0 * kPi);
            h.v = theta / R(kPi);
        } else if (kind == K_TRIANGLE) { // the Moller-Trumbore barycentrics of tri_hit
            const V3<R> p0 = xyz(ldg4(rec)), e1 = xyz(ldg4(rec + 4)), e2 = xyz(ldg4(rec + 8));
            const V3<R> pvec = cross(d, e2);
            const R inv_det = R(1) / dot(e1, pvec);
            const V3<R> tvec = o - p0;
            h.u = dot(tvec, pvec) * inv_det;
            h.v = dot(d, cross(tvec, e1)) * inv_det;
        } else { // QuadGeometry::plane_coordinates, geometry.rs:384-390
            const V3<R> corner = xyz(ldg4(rec)), qu = xyz(ldg4(rec + 4)), qv = xyz(ldg4(rec + 8));
            const V3<R> qw = xyz(ldg4(rec + 12));
            const V3<R> planar = h.p - corner;
            h.u = dot(qw, cross(planar, qv));
            h.v = dot(qw, cross(qu, planar));
        }
    }
    return h;
}

// ------------------------------------------------------------------------ media
// rotate_y_point_inverse / rotate_y_vector_inverse (instance.rs): world into object space.
template <class R> GT_DEV V3<R> rot_y_inv(V3<R> p, R s, R c) { return V3<R>{c * p.x - s * p.z, p.y, s * p.x + c * p.z}; }

// The closest hit of a medium's boundary in (tmin, tmax), object space: a sphere, or
// box_object's HittableList of six quads (scene.rs:177-197: a later quad must be strictly
// closer to replace an earlier one).
template <class R> GT_DEV bool boundary_hit(const MediumDev<R>& M, V3<R> o, V3<R> d, R tmin, R tmax, R& t) {
    bool any = false;
    for (uint32_t i = 0; i < M.parts; ++i) {
        const R* rec = M.part[i].v;
        R ti = R(0);
        bool h = false;
        if (M.kind[i] == K_SPHERE) {
            h = sphere_root(V3<R>{rec[0], rec[1], rec[2]}, rec[3], o, d, tmin, tmax, ti);
        } else if (M.kind[i] == K_QUAD) {
            h = quad_hit(V3<R>{rec[0], rec[1], rec[2]}, V3<R>{rec[4], rec[5], rec[6]}, V3<R>{rec[8], rec[9], rec[10]},
                         V3<R>{rec[7], rec[11], rec[15]}, V3<R>{rec[12], rec[13], rec[14]}, rec[3], o, d, tmin, tmax,
                         ti);
        }
        if (h) {
            tmax = ti;
            t = ti;
            any = true;
        }
    }
    return any;
}

// The media of HittableList::hit_with_rng after the surfaces (scene.rs:177-197), each one
// ConstantMedium::hit_with_rng (volume/medium.rs:119-187) through its Translate / RotateY:
// the boundary's first hit anywhere on the line, clamped to tmin, and its next hit
// 0.0001 further, clipped to the closest hit so far, bound the interval; a non-empty one
// draws a sample and scatters at distance -ln(sample) / density when that falls inside.
// `t` is the closest hit so far (infinity if none); returns -2 - index of the medium hit
// last, or `prim` unchanged.
template <class R> GT_DEV int media_hit(const SceneDev<R>& sc, V3<R> o, V3<R> d, R tmin, R& t, int prim, Rng& g) {
    const R inf = Num<R>::inf();
    for (uint32_t k = 0; k < sc.num_media; ++k) {
        const MediumDev<R>& M = sc.media[k];
        V3<R> oo = o, od = d;
        if (M.transform & GT_MEDIUM_TRANSLATE) oo = oo - V3<R>{M.off[0], M.off[1], M.off[2]};
        if (M.transform & GT_MEDIUM_ROTATE_Y) {
            oo = rot_y_inv(oo, M.sin_t, M.cos_t);
            od = rot_y_inv(od, M.sin_t, M.cos_t);
        }
        R entry = R(0), exit = R(0);
        if (!boundary_hit(M, oo, od, -inf, inf, entry)) continue;
        entry = Num<R>::fmax(entry, tmin);
        if (!boundary_hit(M, oo, od, entry + R(0.0001), inf, exit)) continue;
        exit = Num<R>::fmin(exit, t);
        if (entry >= exit) continue;
        entry = Num<R>::fmax(entry, R(0));
        const R len = Num<R>::sqrt(len2(d));
        if (len <= R(kEps)) continue;
        const R inside = (exit - entry) * len;
        const R sample = Num<R>::fmax(rnd<R>(g), Num<R>::min_positive());
        const R dist = M.neg_inv_density * Num<R>::log(sample);
        if (dist > inside) continue;
        t = entry + dist / len;
        prim = -2 - int(k);
    }
    return prim;
}

// medium_hit_record (volume/medium.rs:152-168): the world ray's point, normal +x, front face.
template <class R> GT_DEV HitRec<R> make_medium_hit(const SceneDev<R>& sc, int prim, V3<R> o, V3<R> d, R t) {
    HitRec<R> h;
    h.p = o + d * t;
    h.n = V3<R>{R(1), R(0), R(0)};
    h.ns = h.n;
    h.u = h.v = R(0);
    h.front = true;
    h.mat = sc.media[-2 - prim].mat;
    return h;
}

// -------------------------------------------------------------- world objects
// Matrix::transform_homogeneous_point with w = 1 (then transform_point's division by w when
// |w| > EPSILON) and with w = 0 (transform_vector), instance.rs:355-369.
template <class R> GT_DEV V3<R> xf_point(const R* m, V3<R> p) {
    R r[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) r[i] = m[4 * i] * p.x + m[4 * i + 1] * p.y + m[4 * i + 2] * p.z + m[4 * i + 3] * R(1);
    if (Num<R>::fabs(r[3]) > R(kEps)) return V3<R>{r[0] / r[3], r[1] / r[3], r[2] / r[3]};
    return V3<R>{r[0], r[1], r[2]};
}
template <class R> GT_DEV V3<R> xf_vector(const R* m, V3<R> v) {
    R r[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) r[i] = m[4 * i] * v.x + m[4 * i + 1] * v.y + m[4 * i + 2] * v.z + m[4 * i + 3] * R(0);
    return V3<R>{r[0], r[1], r[2]};
}
// transform_vector by the normal transform, the inverse's transpose: column i of `inv`.
template <class R> GT_DEV V3<R> xf_normal(const R* inv, V3<R> v) {
    R r[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) r[i] = inv[i] * v.x + inv[4 + i] * v.y + inv[8 + i] * v.z + inv[12 + i] * R(0);
    return V3<R>{r[0], r[1], r[2]};
}

// The closest object hit in (tmin, t): the objects' tree, then each object's mesh tree in
// object space (MatrixInstance::hit_with_rng transforms the ray by the inverse; the ray
// parameter is unchanged, instance.rs:266-289).  On a closer hit sets t, obj (leaf-order
// object index) and leaf (primitive in the mesh's leaf order).  BINARY: the meshes' binary
// trees even where they have wide ones (the persistent world variant, whose registers are
// already spent: its frames ran 23% slower with the wide walk inside).
template <class R, bool BINARY = false>
GT_DEV bool objects_hit(const SceneDev<R>& sc, V3<R> o, V3<R> d, R time, R tmin, R& t, int& obj, int& leaf,
                        uint32_t* err) {
    if (sc.num_objects == 0) return false;
    bool any = false;
    const RayT<R> rt = make_rayt(o, d);
    struct Entry {
        int32_t link, count;
        R entry;
    };
    Entry stack[32];
    int sp = 0;
    R e0;
    if (!hit_box(rt, sc.tlas_box, sc.tlas_box + 3, tmin, t, e0)) return false;
    stack[sp++] = Entry{sc.tlas_link, sc.tlas_count, e0};
    while (sp > 0) {
        const Entry en = stack[--sp];
        if (en.entry >= t) continue;
        if (en.link < 0) { // a leaf: its objects
            for (int32_t i = 0; i < en.count; ++i) {
                const int k = ~en.link + i;
                const ObjectDev<R>& ob = sc.objects[k];
                const V3<R> oo = ob.transformed ? xf_point(ob.inv, o) : o;
                const V3<R> od = ob.transformed ? xf_vector(ob.inv, d) : d;
                R tt = t;
                const int j =
                    traverse<R, false, false, false, BINARY>(sc.meshes[ob.mesh].view, oo, od, time, tmin, t, tt, nullptr, err);
                if (j >= 0 && tt < t) {
                    t = tt;
                    obj = k;
                    leaf = j;
                    any = true;
                }
            }
            continue;
        }
        const Node<R>& nd = sc.tlas[en.link];
        R el, er;
        const bool hl = hit_box(rt, nd.box, nd.box + 3, tmin, t, el);
        const bool hr = hit_box(rt, nd.box + 6, nd.box + 9, tmin, t, er);
        if (sp + 2 > 32) { // deeper than the host build allows; recorded, never expected
            if (err) atomicOr(err, 1u);
            break;
        }
        if (hl && hr) { // the nearer child on top
            if (el <= er) {
                stack[sp++] = Entry{nd.link[2], nd.link[3], er};
                stack[sp++] = Entry{nd.link[0], nd.link[1], el};
            } else {
                stack[sp++] = Entry{nd.link[0], nd.link[1], el};
                stack[sp++] = Entry{nd.link[2], nd.link[3], er};
            }
        } else if (hl) {
            stack[sp++] = Entry{nd.link[0], nd.link[1], el};
        } else if (hr) {
            stack[sp++] = Entry{nd.link[2], nd.link[3], er};
        }
    }
    return any;
}

// The hit record of mesh primitive `leaf` of leaf-order object `obj` at ray parameter t
// (world ray o, d).  A mesh triangle (MeshTriangle::hit, mesh.rs:56-101): texture
// coordinates interpolated from its vertices' (else the barycentrics), the shading normal
// interpolated from its vertex normals (set_shading_normal, object.rs:469-479), and with
// texture coordinates a tangent frame (mesh.rs:121-141, set_tangent_frame object.rs:495-517)
// through which the material's normal map bends the shading normal (material.rs:1663-1684,
// set_oriented_shading_normal object.rs:481-493).  Through a MatrixInstance the point and
// the normal go back to world space and set_face_normal resets the shading normal to the
// geometric one (instance.rs:277-288, object.rs:455-467); (u, v) are kept.
template <class R>
GT_DEV HitRec<R> make_mesh_hit(const SceneDev<R>& sc, int obj, int leaf, V3<R> o, V3<R> d, R time, R t) {
    const ObjectDev<R>& ob = sc.objects[obj];
    const MeshDev<R>& me = sc.meshes[ob.mesh];
    const V3<R> oo = ob.transformed ? xf_point(ob.inv, o) : o;
    const V3<R> od = ob.transformed ? xf_vector(ob.inv, d) : d;
    HitRec<R> h = make_hit(me.view, uint32_t(leaf), oo, od, time, t);
    const uint32_t kind = __ldg(&me.view.meta[leaf].x) & 7u;
    const uint32_t attr = me.attr ? me.attr[leaf] : 0u;
    if (kind == K_TRIANGLE && attr) {
        const R* rec = me.view.prims[leaf].v;
        const V3<R> p0 = xyz(ldg4(rec)), e1 = xyz(ldg4(rec + 4)), e2 = xyz(ldg4(rec + 8));
        const V3<R> pvec = cross(od, e2);
        const R inv_det = R(1) / dot(e1, pvec);
        const V3<R> tvec = oo - p0;
        const R bu = dot(tvec, pvec) * inv_det;
        const R bv = dot(od, cross(tvec, e1)) * inv_det;
        const R bw = R(1) - bu - bv;
        const R* tc = me.uv + size_t(leaf) * 6;
        if (attr & 1u) {
            h.u = bw * tc[0] + bu * tc[2] + bv * tc[4];
            h.v = bw * tc[1] + bu * tc[3] + bv * tc[5];
        }
        if (!ob.transformed) {
            if (attr & 2u) {
                const R* vn = me.vn + size_t(leaf) * 9;
                const V3<R> sn = V3<R>{vn[0], vn[1], vn[2]} * bw + V3<R>{vn[3], vn[4], vn[5]} * bu +
                                 V3<R>{vn[6], vn[7], vn[8]} * bv;
                if (len2(sn) > R(kEps)) {
                    const V3<R> u = normalize(sn);
                    h.ns = h.front ? u : -u;
                }
            }
            const MatDev<R>& m = me.view.mats[h.mat];
            if ((attr & 1u) && m.normal_map) {
                const R du1 = tc[2] - tc[0], dv1 = tc[3] - tc[1], du2 = tc[4] - tc[0], dv2 = tc[5] - tc[1];
                const R det = du1 * dv2 - du2 * dv1;
                if (Num<R>::fabs(det) > R(kEps)) {
                    const R inv = R(1) / det;
                    const V3<R> tg = (e1 * dv2 - e2 * dv1) * inv;
                    const V3<R> bt = (e2 * du1 - e1 * du2) * inv;
                    if (len2(tg) > R(kEps) && len2(bt) > R(kEps)) {
                        const V3<R> n = h.ns; // set_tangent_frame around the shading normal
                        V3<R> T = tg - n * dot(tg, n);
                        if (len2(T) > R(kEps)) {
                            T = normalize(T);
                            const V3<R> ref = cross(n, T);
                            V3<R> B = bt - n * dot(bt, n);
                            B = B - T * dot(B, T);
                            if (len2(B) <= R(kEps)) B = ref;
                            const R hand = dot(B, ref) < R(0) ? R(-1) : R(1);
                            B = normalize(ref * hand);
                            const V3<R> tn = normal_map_sample(m.normal_map, m.normal_strength, m.normal_neg_y != 0, h.u, h.v);
                            V3<R> nm = T * tn.x + B * tn.y + n * tn.z;
                            if (len2(nm) > R(kEps)) {
                                nm = normalize(nm);
                                if (dot(nm, n) < R(0)) nm = -nm;
                                if (len2(nm) > R(kEps)) h.ns = normalize(nm);
                            }
                        }
                    }
                }
            }
        }
    }
    if (ob.transformed) {
        const V3<R> outward_obj = h.front ? h.n : -h.n;
        h.p = xf_point(ob.xf, h.p);
        const V3<R> outward = normalize(xf_normal(ob.inv, outward_obj));
        h.front = dot(d, outward) < R(0);
        h.n = h.front ? outward : -outward;
        h.ns = h.n;
    }
    return h;
}

// HittableList::hit_with_rng over the whole world (scene.rs:177-197): the RayScene's
// surfaces, then the objects, then the media in order (each clipped to the closest hit so
// far; the media draw from g).  Fills h and returns true on a hit.
template <class R>
GT_DEV bool world_hit(const SceneDev<R>& sc, V3<R> o, V3<R> d, R time, R tmin, Rng& g, HitRec<R>& h, uint32_t* err) {
    const R inf = Num<R>::inf();
    R t = inf;
    int prim = traverse<R, false, false>(sc, o, d, time, tmin, inf, t, nullptr, err);
    if (prim < 0) t = inf;
    int obj = -1, leaf = -1;
    objects_hit<R, true>(sc, o, d, time, tmin, t, obj, leaf, err);
    const int med = media_hit(sc, o, d, tmin, t, -1, g);
    if (med <= -2) h = make_medium_hit(sc, med, o, d, t);
    else if (obj >= 0) h = make_mesh_hit(sc, obj, leaf, o, d, time, t);
    else if (prim >= 0) h = make_hit(sc, uint32_t(prim), o, d, time, t);
    else return false;
    return true;
}

// Origin of a ray that leaves the surface at h.  In f32 the hit point and the primitives'
// stored corners and edges carry rounding errors of a few ulps of the coordinates (about
// 1e-4 at 500 units), more than t_min = 0.001 covers for a grazing ray near the edge
// between two faces: such a ray can start just behind the neighbouring face's plane and
// hit it from inside, after which the path is trapped in a closed object and its
// throughput compounds without bound.  The f32 path therefore starts new rays
// 2^-19 (max |p| + 1) off the surface, on the side the ray leaves towards (a scaled form
// of the offset of Waechter and Binder, "A Fast and Robust Method for Avoiding
// Self-Intersection", Ray Tracing Gems, 2019).  The f64 path keeps the reference's h.p.
template <class R> GT_DEV V3<R> spawn_origin(const HitRec<R>& h, V3<R> dir);
template <> GT_DEV V3<double> spawn_origin(const HitRec<double>& h, V3<double>) { return h.p; }
template <> GT_DEV V3<float> spawn_origin(const HitRec<float>& h, V3<float> dir) {
    const float m = fmaxf(fmaxf(fabsf(h.p.x), fabsf(h.p.y)), fabsf(h.p.z)) + 1.0f;
    const float e = dot(dir, h.n) >= 0.0f ? m * 0x1p-19f : -m * 0x1p-19f;
    return h.p + h.n * e;
}

// ------------------------------------------------------------------ materials
// Perlin::noise (gmath/perlin.rs:36-58) and perlin_interp (106-124): the eight corner
// gradients picked through the three permutations, weighted by smoothstep blends, summed
// x-major in the reference's order.
template <class R> GT_DEV R perlin_noise(const PerlinDev<R>* t, V3<R> p) {
    const R fx = Num<R>::floor(p.x), fy = Num<R>::floor(p.y), fz = Num<R>::floor(p.z);
    const R u = p.x - fx, v = p.y - fy, w = p.z - fz;
    const uint32_t bx = uint32_t(Num<R>::to_i32(fx)), by = uint32_t(Num<R>::to_i32(fy)),
                   bz = uint32_t(Num<R>::to_i32(fz));
    const R uu = u * u * (R(3) - R(2) * u);
    const R vv = v * v * (R(3) - R(2) * v);
    const R ww = w * w * (R(3) - R(2) * w);
    R accum = R(0);
#pragma unroll
    for (uint32_t ox = 0; ox < 2; ++ox)
#pragma unroll
        for (uint32_t oy = 0; oy < 2; ++oy)
#pragma unroll
            for (uint32_t oz = 0; oz < 2; ++oz) {
                const uint32_t gi = uint32_t(t->perm[0][(bx + ox) & 255u]) ^ uint32_t(t->perm[1][(by + oy) & 255u]) ^
                                    uint32_t(t->perm[2][(bz + oz) & 255u]);
                const R wx = u - R(ox), wy = v - R(oy), wz = w - R(oz);
                const R dot = t->gx[gi] * wx + t->gy[gi] * wy + t->gz[gi] * wz;
                const R bxw = ox ? uu : R(1) - uu, byw = oy ? vv : R(1) - vv, bzw = oz ? ww : R(1) - ww;
                accum = accum + bxw * byw * bzw * dot;
            }
    return accum;
}

// Perlin::turbulence (perlin.rs:61-74).
template <class R> GT_DEV R perlin_turbulence(const PerlinDev<R>* t, V3<R> p, int32_t depth) {
    R accum = R(0), weight = R(1);
    for (int32_t k = 0; k < depth; ++k) {
        accum = accum + weight * perlin_noise(t, p);
        weight = weight * R(0.5);
        p = V3<R>{p.x * R(2), p.y * R(2), p.z * R(2)};
    }
    return Num<R>::fabs(accum);
}

// NoiseTexture::sample_linear (graphics/raytracing/texture.rs:337-352).
template <class R> GT_DEV R noise_intensity(const MatDev<R>& m, V3<R> p) {
    const V3<R> q{p.x * m.inv_scale, p.y * m.inv_scale, p.z * m.inv_scale};
    if (m.noise_variant == GT_NOISE_TURBULENCE) return perlin_turbulence(m.noise, q, m.noise_depth);
    if (m.noise_variant == GT_NOISE_MARBLE)
        return R(0.5) * (R(1) + Num<R>::sin(q.z + R(10) * perlin_turbulence(m.noise, q, m.noise_depth)));
    return R(0.5) * (R(1) + perlin_noise(m.noise, q));
}

// ImageTexture::sample_linear (raytracing/texture.rs:148-155) through Texture::sample
// (graphics/texture.rs:202-208, 716-752): nearest or bilinear with Rgb::lerp's rounding to
// bytes, clamp or repeat per axis, t = 1 at the top row, then (c / 255)^2.
template <class R> GT_DEV R rem1(R x) { // f64::rem_euclid(x, 1.0)
    const R r = Num<R>::fmod(x, R(1));
    return r < R(0) ? r + R(1) : r;
}
template <class R> GT_DEV uint32_t to_u32(R x) { // `as u32` for the finite values here
    return x <= R(0) ? 0u : (x >= R(4294967295.0) ? 4294967295u : uint32_t(x));
}
template <class R> GT_DEV void tex_axis(R value, uint32_t size, uint32_t mode, R& coord, uint32_t& lo, uint32_t& hi) {
    if (mode == GT_WRAP_CLAMP) {
        coord = clampr(value, R(0), R(1)) * R(size - 1);
        lo = to_u32(Num<R>::floor(coord));
        hi = min(lo + 1, size - 1);
    } else {
        coord = rem1(value) * R(size);
        lo = min(to_u32(Num<R>::floor(coord)), size - 1);
        hi = lo + 1 == size ? 0u : lo + 1;
    }
}
template <class R> GT_DEV void texel_lerp(const uint8_t* a, const uint8_t* b, R t, uint8_t* out) {
    t = clampr(t, R(0), R(1));
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const R v = Num<R>::round(R(a[k]) + R(int(b[k]) - int(a[k])) * t);
        out[k] = uint8_t(v <= R(0) ? 0 : (v >= R(255) ? 255 : int(v)));
    }
}
// Texture::sample (graphics/texture.rs:202-208, 696-752) of a non-empty bitmap: the 8-bit
// texel (nearest) or the u8 lerps of four (linear); black at a non-finite (u, v).
template <class R> GT_DEV void image_rgb8(const ImageDev* im, R u, R v, uint8_t* c) {
    c[0] = c[1] = c[2] = 0;
    if (!(Num<R>::finite(u) && Num<R>::finite(v))) return;
    const uint8_t* px = im->rgb;
    const uint32_t w = im->w, h = im->h;
    if (im->filter == GT_FILTER_NEAREST) {
        const R ws = im->wrap_s == GT_WRAP_REPEAT ? rem1(u) : clampr(u, R(0), R(1));
        const R wt = im->wrap_t == GT_WRAP_REPEAT ? rem1(v) : clampr(v, R(0), R(1));
        const uint32_t x = to_u32(Num<R>::round(ws * R(w - 1)));
        const uint32_t y = to_u32(Num<R>::round((R(1) - wt) * R(h - 1)));
        const uint8_t* t = px + (size_t(y) * w + x) * 3;
        c[0] = t[0];
        c[1] = t[1];
        c[2] = t[2];
    } else {
        R x, y;
        uint32_t x0, x1, y0, y1;
        tex_axis(u, w, im->wrap_s, x, x0, x1);
        tex_axis(R(1) - v, h, im->wrap_t, y, y0, y1);
        const R tx = x - R(x0), ty = y - R(y0);
        uint8_t top[3], bottom[3];
        texel_lerp(px + (size_t(y0) * w + x0) * 3, px + (size_t(y0) * w + x1) * 3, tx, top);
        texel_lerp(px + (size_t(y1) * w + x0) * 3, px + (size_t(y1) * w + x1) * 3, tx, bottom);
        texel_lerp(top, bottom, ty, c);
    }
}

// ImageTexture::sample_linear (raytracing/texture.rs:148-155): cyan for an empty bitmap,
// else the texel decoded as (c / 255)^2 (LinearRgb::from_rgb_srgb).
template <class R> GT_DEV V3<R> image_color(const ImageDev* im, R u, R v) {
    uint8_t c[3] = {0, 255, 255}; // Rgb::CYAN
    if (im != nullptr && im->w != 0 && im->h != 0) image_rgb8(im, u, v, c);
    const R r = R(c[0]) / R(255), g = R(c[1]) / R(255), b = R(c[2]) / R(255);
    return V3<R>{r * r, g * g, b * b};
}

// NormalMap::sample_tangent_normal (raytracing/texture.rs:254-275): channels decoded as
// 2 c / 255 - 1, x and y scaled by the strength, y negated for a -Y green channel, z
// clamped at 0, normalised; +z for an empty bitmap or a near-zero result.
template <class R> GT_DEV V3<R> normal_map_sample(const ImageDev* im, R strength, bool neg_y, R u, R v) {
    const V3<R> up{R(0), R(0), R(1)};
    if (im->w == 0 || im->h == 0) return up;
    uint8_t c[3];
    image_rgb8(im, u, v, c);
    auto dec = [](uint8_t ch) { return R(2) * (R(ch) / R(255)) - R(1); };
    const R green = neg_y ? -dec(c[1]) : dec(c[1]);
    const V3<R> n{strength * dec(c[0]), strength * green, Num<R>::fmax(dec(c[2]), R(0))};
    return len2(n) <= R(kEps) ? up : vdiv(n, Num<R>::sqrt(len2(n)));
}

template <class R> GT_DEV V3<R> mat_color(const MatDev<R>& m, const HitRec<R>& h) {
    if (m.tex == GT_TEX_IMAGE) return image_color(m.image, h.u, h.v);
    const V3<R> p = h.p;
    if (m.tex == GT_TEX_NOISE) {
        const R i = noise_intensity(m, p);
        return V3<R>{i, i, i};
    }
    if (m.tex == 1) { // CheckerTexture::sample_linear (raytracing/texture.rs:97-108)
        long long xi = (long long)Num<R>::floor(m.inv_scale * p.x);
        long long yi = (long long)Num<R>::floor(m.inv_scale * p.y);
        long long zi = (long long)Num<R>::floor(m.inv_scale * p.z);
        return ((xi + yi + zi) % 2) == 0 ? load3(m.even) : load3(m.odd);
    }
    return load3(m.color);
}

enum : int { SC_NONE = 0, SC_SPECULAR = 1, SC_PDF = 2 };
template <class R> struct ScatterRec {
    int kind;
    V3<R> dir; // specular direction
    V3<R> att;
    MatPdf<R> pdf;
};

template <class R> GT_DEV ScatterRec<R> mat_scatter(const MatDev<R>& m, V3<R> din, const HitRec<R>& h, Rng& g) {
    ScatterRec<R> s;
    s.kind = SC_NONE;
    switch (m.kind) {
    case 0: // Lambertian, material.rs:508-521
        if (!onb_from_w(h.ns, s.pdf.basis)) return s;
        s.kind = SC_PDF;
        s.pdf.kind = PDF_COSINE;
        s.att = mat_color(m, h);
        return s;
    case 2: // Isotropic, material.rs:1124-1137
        s.kind = SC_PDF;
        s.pdf.kind = PDF_SPHERE;
        s.att = mat_color(m, h);
        return s;
    case 6: // HenyeyGreenstein, material.rs:1281-1295: the phase function around the incoming ray
        if (!onb_from_w(din, s.pdf.basis)) return s;
        s.kind = SC_PDF;
        s.pdf.kind = PDF_HG;
        s.pdf.rough = m.param;
        s.att = mat_color(m, h);
        return s;
    case 3: { // GgxMicrofacet, material.rs:1583-1597; GgxReflectionPdf::new sampling.rs:146-170
        V3<R> outgoing = -normalize(din);
        if (!onb_from_w(h.ns, s.pdf.basis)) return s;
        s.pdf.out = normalize(outgoing);
        if (len2(s.pdf.out) <= R(kEps) || dot(s.pdf.out, s.pdf.basis.w) <= R(0)) return s;
        s.pdf.rough = clampr(m.param, R(0), R(1));
        s.pdf.alpha = ggx_alpha(s.pdf.rough);
        s.pdf.kind = PDF_GGX;
        s.kind = SC_PDF;
        s.att = mat_color(m, h);
        return s;
    }
    case 4: { // Metal, material.rs:2087-2106
        V3<R> refl = reflect(normalize(din), h.ns);
        V3<R> dir = refl + unit_vector_spherical<R>(g) * m.param;
        if (dot(dir, h.n) <= R(0)) return s;
        s.kind = SC_SPECULAR;
        s.dir = dir;
        s.att = load3(m.color);
        return s;
    }
    case 5: { // Dielectric, material.rs:2321-2351
        R ratio = h.front ? R(1) / m.param : m.param;
        V3<R> unit = normalize(din);
        R ct = Num<R>::fmin(dot(-unit, h.n), R(1));
        R st = Num<R>::sqrt(R(1) - ct * ct);
        bool refl = ratio * st > R(1);
        if (!refl) {
            R r0 = (R(1) - ratio) / (R(1) + ratio); // Dielectric::reflectance, material.rs:2213-2219
            r0 = r0 * r0;
            R rf = r0 + (R(1) - r0) * pow5(R(1) - ct);
            refl = rf > rnd<R>(g);
        }
        s.dir = refl ? reflect(unit, h.n) : refract(unit, h.n, ratio);
        s.kind = SC_SPECULAR;
        s.att = V3<R>{1, 1, 1};
        return s;
    }
    default: // DiffuseLight: no scatter
        return s;
    }
}

template <class R> GT_DEV R mat_scattering_pdf(const MatDev<R>& m, V3<R> din, const HitRec<R>& h, V3<R> dout) {
    switch (m.kind) {
    case 0: { // material.rs:523-530
        R c = dot(h.ns, normalize(dout));
        return c <= R(0) ? R(0) : c / R(kPi);
    }
    case 2:
        return R(1) / (R(4) * R(kPi));
    case 6: { // material.rs:1297-1302
        MatPdf<R> p;
        p.kind = PDF_HG;
        p.rough = m.param;
        if (!onb_from_w(din, p.basis)) return R(0);
        return matpdf_value(p, dout);
    }
    case 3: { // material.rs:1599-1617 and ggx_reflection_scattering_weight 1717-1758
        V3<R> outgoing = -normalize(din);
        V3<R> incoming = normalize(dout);
        if (dot(incoming, h.n) <= R(0) || dot(outgoing, h.n) <= R(0)) return R(0);
        V3<R> sc = mat_color(m, h); // specular_luminance, material.rs:1760-1762
        R f0 = clampr(R(0.2126) * sc.x + R(0.7152) * sc.y + R(0.0722) * sc.z, R(0), R(1));
        V3<R> n = normalize(h.ns), o = normalize(outgoing), i = normalize(incoming);
        R ndi = dot(n, i), ndo = dot(n, o);
        if (ndi <= R(0) || ndo <= R(0)) return R(0);
        V3<R> half = normalize(i + o);
        if (len2(half) <= R(kEps)) return R(0);
        R ndh = dot(n, half), odh = dot(o, half);
        if (ndh <= R(0) || odh <= R(0)) return R(0);
        R D = ggx_D(ndh, m.param);
        R G = smith_G1(ndi, m.param) * smith_G1(ndo, m.param);
        f0 = clampr(f0, R(0), R(1));
        if (f0 <= R(kEps)) return R(0);
        R F = schlick_f(odh, f0) / f0;
        return D * G * F / (R(4) * ndo);
    }
    default:
        return R(0);
    }
}

template <class R> GT_DEV V3<R> mat_emitted(const MatDev<R>& m, const HitRec<R>& h) {
    if (m.kind == 1 && h.front) return mat_color(m, h); // material.rs:1008-1022
    return V3<R>{0, 0, 0};
}

template <class R> GT_DEV V3<R> mat_albedo(const MatDev<R>& m, const HitRec<R>& h) { // denoise_albedo
    if (m.kind == 4) return load3(m.color);
    if (m.kind == 5) return V3<R>{1, 1, 1};
    return mat_color(m, h);
}

// ------------------------------------------------------------- light targets
template <class R> GT_DEV R area_pdf(V3<R> dir, R t, V3<R> n, R area) { // object.rs:1100-1111
    if (area <= R(kEps)) return R(0);
    R d2 = len2(dir * t);
    R cosine = Num<R>::fabs(dot(normalize(dir), n));
    if (cosine <= R(kEps)) return R(0);
    return d2 / (cosine * area);
}

template <class R> GT_DEV R light_pdf_one(const LightDev<R>& L, V3<R> origin, R time, V3<R> dir) {
    const R inf = Num<R>::inf();
    switch (L.kind) {
    case K_SPHERE:
    case K_MOVING: { // sphere_pdf_value, object.rs:1044-1070
        V3<R> c = load3(L.a);
        if (L.kind == K_MOVING) c = c + load3(L.b) * time;
        R root;
        if (!sphere_root(c, L.radius, origin, dir, R(kShadowAcnePdf), inf, root)) return R(0);
        V3<R> cd = c - origin;
        R d2 = len2(cd);
        R r2 = L.radius * L.radius;
        if (d2 <= r2) return R(1) / (R(4) * R(kPi));
        R cmax = Num<R>::sqrt(R(1) - r2 / d2);
        R solid = R(2) * R(kPi) * (R(1) - cmax);
        return solid <= R(kEps) ? R(0) : R(1) / solid;
    }
    case K_QUAD: { // quad_pdf_value, object.rs:1072-1084
        if (L.area_sq <= R(kEps)) return R(0);
        R t;
        if (!quad_hit(load3(L.a), load3(L.b), load3(L.c), load3(L.n), load3(L.w), L.plane_d, origin, dir,
                      R(kShadowAcnePdf), inf, t))
            return R(0);
        return area_pdf(dir, t, load3(L.n), L.area);
    }
    case K_TRIANGLE: { // triangle_pdf_value, object.rs:1086-1098
        V3<R> p0 = load3(L.a);
        R t;
        if (!tri_hit(p0, load3(L.b) - p0, load3(L.c) - p0, origin, dir, R(kShadowAcnePdf), inf, t)) return R(0);
        return area_pdf(dir, t, load3(L.n), L.area);
    }
    }
    return R(0);
}

template <class R> GT_DEV V3<R> light_dir_one(const LightDev<R>& L, V3<R> origin, R time, Rng& g) {
    switch (L.kind) {
    case K_SPHERE:
    case K_MOVING: { // random_direction_to_sphere, object.rs:1113-1128
        V3<R> c = load3(L.a);
        if (L.kind == K_MOVING) c = c + load3(L.b) * time;
        V3<R> dir = c - origin;
        R d2 = len2(dir);
        R r2 = L.radius * L.radius;
        if (d2 <= r2 || d2 <= R(kEps)) return unit_vector_spherical<R>(g);
        R r1 = rnd<R>(g); // random_to_sphere, object.rs:1153-1161
        R rr2 = rnd<R>(g);
        R z = R(1) + rr2 * (Num<R>::sqrt(R(1) - L.radius * L.radius / d2) - R(1));
        R phi = R(2) * R(kPi) * r1;
        R rz = Num<R>::sqrt(R(1) - z * z);
        R s, cc;
        Num<R>::sincos(phi, &s, &cc);
        V3<R> local{cc * rz, s * rz, z};
        Onb<R> b;
        if (!onb_from_w(dir, b)) return local;
        return onb_local(b, local);
    }
    case K_QUAD: { // object.rs:1130-1134
        R r1 = rnd<R>(g);
        V3<R> p = load3(L.a) + load3(L.b) * r1;
        R r2 = rnd<R>(g);
        p = p + load3(L.c) * r2;
        return p - origin;
    }
    case K_TRIANGLE: { // object.rs:1136-1151
        R a = rnd<R>(g);
        R b = rnd<R>(g);
        if (a + b > R(1)) {
            a = R(1) - a;
            b = R(1) - b;
        }
        V3<R> p0 = load3(L.a);
        V3<R> p = (p0 + (load3(L.b) - p0) * a) + (load3(L.c) - p0) * b;
        return p - origin;
    }
    }
    return V3<R>{1, 0, 0};
}

// WeightedSamplingTargetList::pdf_value / random_direction (scene.rs:479-497).
template <class R> GT_DEV R lights_pdf(const LightsDev<R>& L, V3<R> origin, R time, V3<R> dir) {
    if (L.count == 0 || L.total <= R(0)) return R(0);
    R sum = R(-0.0);
    for (uint32_t i = 0; i < L.count; ++i) sum = sum + (L.t[i].weight / L.total) * light_pdf_one(L.t[i], origin, time, dir);
    return sum;
}
template <class R> GT_DEV V3<R> lights_dir(const LightsDev<R>& L, V3<R> origin, R time, Rng& g) {
    if (L.count == 0 || L.total <= R(0)) return V3<R>{1, 0, 0};
    R pick = rnd_range<R>(g, R(0), L.total);
    for (uint32_t i = 0; i < L.count; ++i) {
        pick -= L.t[i].weight;
        if (pick <= R(0)) return light_dir_one(L.t[i], origin, time, g);
    }
    return light_dir_one(L.t[L.count - 1], origin, time, g);
}

// --------------------------------------------------------------- environment
template <class R> GT_DEV R env_pdf(const EnvDev<R>& E, V3<R> dir) { // environment.rs:133-153
    if (E.total <= R(kEps) || E.width == 0) return R(1) / R(4.0 * kPi);
    V3<R> d = normalize(dir);
    R theta = Num<R>::acos(clampr(d.y, R(-1), R(1)));
    R phi = rem_euclid(Num<R>::atan2(d.z, d.x), R(kTau));
    R fx = Num<R>::floor((phi / R(kTau)) * R(E.width));
    R fy = Num<R>::floor((theta / R(kPi)) * R(E.height));
    uint32_t x = fx > R(0) ? (uint32_t)fx : 0u;
    uint32_t y = fy > R(0) ? (uint32_t)fy : 0u;
    x = min(x, E.width - 1);
    y = min(y, E.height - 1);
    R prob = E.weights[size_t(y) * E.width + x] / E.total;
    R t0 = R(kPi) * (R(y) / R(E.height));
    R t1 = R(kPi) * (R(y + 1) / R(E.height));
    R s0, c0, s1, c1;
    Num<R>::sincos(t0, &s0, &c0);
    Num<R>::sincos(t1, &s1, &c1);
    R sa = (R(kTau) / R(E.width)) * Num<R>::fmax(c0 - c1, R(0));
    return sa <= R(kEps) ? R(0) : prob / sa;
}

template <class R> GT_DEV void env_sample(const EnvDev<R>& E, Rng& g, V3<R>& dir, R& pdf) { // environment.rs:107-131
    if (E.total <= R(kEps) || E.width == 0) {
        dir = unit_vector_spherical<R>(g);
        pdf = R(1) / R(4.0 * kPi);
        return;
    }
    R target = rnd<R>(g) * E.total;
    // partition_point(cdf < target): first index whose running sum is >= target.
    uint32_t lo = 0, hi = E.width * E.height;
    while (lo < hi) {
        uint32_t mid = lo + (hi - lo) / 2;
        if (E.cdf[mid] < target) lo = mid + 1;
        else hi = mid;
    }
    uint32_t idx = min(lo, E.width * E.height - 1);
    uint32_t x = idx % E.width, y = idx / E.width;
    R u = (R(x) + rnd<R>(g)) / R(E.width);
    R t0 = R(kPi) * (R(y) / R(E.height));
    R t1 = R(kPi) * (R(y + 1) / R(E.height));
    R s0, c0, s1, c1;
    Num<R>::sincos(t0, &s0, &c0);
    Num<R>::sincos(t1, &s1, &c1);
    R ct = c0 + rnd<R>(g) * (c1 - c0);
    R st = Num<R>::sqrt(Num<R>::fmax(R(1) - ct * ct, R(0)));
    R phi = R(kTau) * u;
    R sp, cp;
    Num<R>::sincos(phi, &sp, &cp);
    dir = V3<R>{st * cp, ct, st * sp};
    pdf = env_pdf(E, dir);
}

template <class R> GT_DEV uint8_t lerp_u8(uint8_t a, uint8_t b, R t) { // Rgb::lerp, colors.rs:525-537
    t = clampr(t, R(0), R(1));
    R v = Num<R>::round(R(a) + R(int(b) - int(a)) * t);
    if (!(v > R(0))) return 0;
    if (v >= R(255)) return 255;
    return (uint8_t)v;
}

// EnvironmentLight::radiance (environment.rs:98-105) through the bilinear texture
// sampler (graphics/texture.rs:657-711): Repeat in u, Clamp in v.
template <class R> GT_DEV V3<R> env_radiance(const EnvDev<R>& E, V3<R> dir) {
    V3<R> d = normalize(dir);
    R phi = rem_euclid(Num<R>::atan2(d.z, d.x), R(kTau));
    R theta = Num<R>::acos(clampr(d.y, R(-1), R(1)));
    R s = phi / R(kTau), t = R(1) - theta / R(kPi);
    if (E.width == 0 || !Num<R>::finite(s) || !Num<R>::finite(t)) return V3<R>{0, 0, 0};
    R xc = rem_euclid(s, R(1)) * R(E.width);
    R fx = Num<R>::floor(xc);
    uint32_t x0 = min(fx > R(0) ? (uint32_t)fx : 0u, E.width - 1);
    uint32_t x1 = x0 + 1 == E.width ? 0 : x0 + 1;
    R yc = clampr(R(1) - t, R(0), R(1)) * R(E.height - 1);
    R fy = Num<R>::floor(yc);
    uint32_t y0 = fy > R(0) ? (uint32_t)fy : 0u;
    uint32_t y1 = min(y0 + 1, E.height - 1);
    R tx = xc - R(x0), ty = yc - R(y0);
    size_t i00 = (size_t(y0) * E.width + x0) * 3, i10 = (size_t(y0) * E.width + x1) * 3;
    size_t i01 = (size_t(y1) * E.width + x0) * 3, i11 = (size_t(y1) * E.width + x1) * 3;
    R out[3];
    if (E.format == 0) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            uint8_t top = lerp_u8<R>(E.px8[i00 + c], E.px8[i10 + c], tx);
            uint8_t bot = lerp_u8<R>(E.px8[i01 + c], E.px8[i11 + c], tx);
            R v = R(lerp_u8<R>(top, bot, ty)) / R(255);
            out[c] = v * v; // gamma-2 decode, colors.rs:78-84
        }
    } else {
        R ctx = clampr(tx, R(0), R(1)), cty = clampr(ty, R(0), R(1));
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            R p00 = R(E.px32[i00 + c]), p10 = R(E.px32[i10 + c]);
            R p01 = R(E.px32[i01 + c]), p11 = R(E.px32[i11 + c]);
            R top = p00 + (p10 - p00) * ctx;
            R bot = p01 + (p11 - p01) * ctx;
            out[c] = top + (bot - top) * cty;
        }
    }
    return V3<R>{out[0], out[1], out[2]};
}

// ----------------------------------------------------------------- background
template <class R> GT_DEV V3<R> background(const CamDev<R>& c, V3<R> dir) { // camera.rs:301-322
    if (c.bg_kind == 0) return load3(c.bg);
    V3<R> nadir = load3(c.bg), hor = load3(c.bg + 3), zen = load3(c.bg + 6);
    R t = R(0.5) * (normalize(dir).y + R(1));
    if (t < R(0.5)) {
        R b = R(2) * t;
        return nadir * (R(1) - b) + hor * b;
    }
    R b = R(2) * (t - R(0.5));
    return hor * (R(1) - b) + zen * b;
}

// -------------------------------------------------------------------- camera
// ray_for_pixel_sample / ray_for_pixel_stratified_sample (camera.rs:1658-1704): jitter,
// optional defocus-disk origin, shutter time.  In f64 the direction is the reference's
// pixel_sample - origin.  In f32 that difference of two points far from the world origin
// cancels (a camera 800 units out with its viewport 1 unit ahead loses ~1e-4 relative),
// so the f32 path builds the same vector from center-relative terms whose base,
// pixel00 - center, was computed in f64.
template <class R> GT_DEV void camera_ray(const CamDev<R>& c, uint32_t x, uint32_t y, uint32_t sample, Rng& g,
                                          V3<R>& o, V3<R>& d, R& time) {
    R ox, oy;
    if (c.mode == 0) {
        ox = rnd<R>(g) - R(0.5);
        oy = rnd<R>(g) - R(0.5);
    } else {
        uint32_t sx = sample % c.grid, sy = sample / c.grid;
        R rec = R(1) / R(c.grid);
        ox = ((R(sx) + rnd<R>(g)) * rec) - R(0.5);
        oy = ((R(sy) + rnd<R>(g)) * rec) - R(0.5);
    }
    const R fx = R(x) + ox, fy = R(y) + oy;
    // Rejection sampling of the unit disk (random.rs:141-152); each try is accepted with
    // probability pi/4, so the cap of 4096 tries (reached with probability ~1e-2700)
    // only bounds the loop.
    V3<R> p{0, 0, 0};
    if (c.defocus) {
        for (int tries = 0; tries < 4096; ++tries) {
            R a = rnd_range<R>(g, R(-1), R(1));
            R b = rnd_range<R>(g, R(-1), R(1));
            p = V3<R>{a, b, R(0)};
            if (len2(p) < R(1)) break;
        }
    }
    time = rnd_range<R>(g, c.shutter0, c.shutter1);
    if (sizeof(R) == sizeof(double)) {
        V3<R> ps = (load3(c.pixel00) + load3(c.du) * fx) + load3(c.dv) * fy;
        V3<R> org = load3(c.center);
        if (c.defocus) org = (org + load3(c.ddu) * p.x) + load3(c.ddv) * p.y; // camera.rs:1710-1713
        o = org;
        d = ps - org;
    } else {
        V3<R> off{0, 0, 0};
        if (c.defocus) off = load3(c.ddu) * p.x + load3(c.ddv) * p.y;
        o = load3(c.center) + off;
        d = ((load3(c.p00_rel) + load3(c.du) * fx) + load3(c.dv) * fy) - off;
    }
}

} // namespace gt
