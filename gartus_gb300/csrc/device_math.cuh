// device_math.cuh — device-side arithmetic of the path tracer, templated on the scalar
// type R.  R = double follows the reference's f64 arithmetic operation for operation
// (the f64 translation unit is compiled with -fmad=false, so nothing is fused);
// R = float is the throughput path.  Citations are file:line within the gartus crate.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "layout.h"

namespace gt {

#define GT_DEV __device__ __forceinline__

constexpr double kPi = 3.141592653589793;
constexpr double kTau = 6.283185307179586;
constexpr double kEps = 2.220446049250313e-16; // f64::EPSILON (pdf and degeneracy tests)
constexpr double kShadowAcne = 0.001;          // raytracing.rs:146
constexpr double kShadowAcnePdf = 0.001;       // object.rs:1163
constexpr double kTriHitEps = 1e-10;           // geometry.rs:10
constexpr double kQuadHitEps = 1e-8;           // geometry.rs:12
constexpr double kGgxMinAlpha = 1.0e-4;        // sampling.rs:12

template <class R> struct Num;
template <> struct Num<float> {
    static GT_DEV float inf() { return __int_as_float(0x7f800000); }
    static GT_DEV float sqrt(float x) { return sqrtf(x); }
    static GT_DEV float acos(float x) { return acosf(x); }
    static GT_DEV float pow(float x, float y) { return powf(x, y); }
    static GT_DEV float atan2(float y, float x) { return atan2f(y, x); }
    static GT_DEV void sincos(float x, float* s, float* c) { sincosf(x, s, c); }
    static GT_DEV float fabs(float x) { return fabsf(x); }
    static GT_DEV float fmin(float a, float b) { return fminf(a, b); }
    static GT_DEV float fmax(float a, float b) { return fmaxf(a, b); }
    static GT_DEV float floor(float x) { return floorf(x); }
    static GT_DEV float sin(float x) { return sinf(x); }
    static GT_DEV int32_t to_i32(float x) { return __float2int_rz(x); } // saturating, NaN -> 0 (Rust `as`)
    static GT_DEV float fmod(float a, float b) { return fmodf(a, b); }
    static GT_DEV float log(float x) { return logf(x); }
    static GT_DEV float min_positive() { return 0x1p-126f; } // f32::MIN_POSITIVE
    static GT_DEV float round(float x) { return roundf(x); }
    static GT_DEV bool finite(float x) { return isfinite(x); }
};
template <> struct Num<double> {
    static GT_DEV double inf() { return __longlong_as_double(0x7ff0000000000000ULL); }
    static GT_DEV double sqrt(double x) { return ::sqrt(x); }
    static GT_DEV double acos(double x) { return ::acos(x); }
    static GT_DEV double pow(double x, double y) { return ::pow(x, y); }
    static GT_DEV double atan2(double y, double x) { return ::atan2(y, x); }
    static GT_DEV void sincos(double x, double* s, double* c) { ::sincos(x, s, c); }
    static GT_DEV double fabs(double x) { return ::fabs(x); }
    static GT_DEV double fmin(double a, double b) { return ::fmin(a, b); }
    static GT_DEV double fmax(double a, double b) { return ::fmax(a, b); }
    static GT_DEV double floor(double x) { return ::floor(x); }
    static GT_DEV double sin(double x) { return ::sin(x); }
    static GT_DEV int32_t to_i32(double x) { return __double2int_rz(x); } // saturating, NaN -> 0 (Rust `as`)
    static GT_DEV double fmod(double a, double b) { return ::fmod(a, b); }
    static GT_DEV double log(double x) { return ::log(x); }
    static GT_DEV double min_positive() { return 0x1p-1022; } // f64::MIN_POSITIVE
    static GT_DEV double round(double x) { return ::round(x); }
    static GT_DEV bool finite(double x) { return isfinite(x); }
};

// Rust f64::clamp keeps NaN; min/max ignore a NaN operand.
template <class R> GT_DEV R clampr(R x, R lo, R hi) {
    if (x < lo) x = lo;
    if (x > hi) x = hi;
    return x;
}
// Constant powi(x, 5) as LLVM lowers it: x * ((x*x)*(x*x)).
template <class R> GT_DEV R pow5(R x) {
    R x2 = x * x;
    R x4 = x2 * x2;
    return x * x4;
}
template <class R> GT_DEV R rem_euclid(R a, R b) {
    R r = Num<R>::fmod(a, b);
    return r < R(0) ? r + Num<R>::fabs(b) : r;
}

// ------------------------------------------------------------------- vectors
template <class R> struct V3 {
    R x, y, z;
};
template <class R> GT_DEV V3<R> v3(R x, R y, R z) { return V3<R>{x, y, z}; }
template <class R> GT_DEV V3<R> operator+(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R> GT_DEV V3<R> operator-(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class R> GT_DEV V3<R> operator-(V3<R> a) { return {-a.x, -a.y, -a.z}; }
template <class R> GT_DEV V3<R> operator*(V3<R> a, R s) { return {a.x * s, a.y * s, a.z * s}; }
template <class R> GT_DEV V3<R> vdiv(V3<R> a, R s) { return {a.x / s, a.y / s, a.z / s}; }
template <class R> GT_DEV R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R> GT_DEV V3<R> cross(V3<R> a, V3<R> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class R> GT_DEV R len2(V3<R> a) { return dot(a, a); }
template <class R> GT_DEV V3<R> normalize(V3<R> a) { // vector.rs:147-155
    R l = Num<R>::sqrt(len2(a));
    if (l < R(kEps)) return V3<R>{0, 0, 0};
    return vdiv(a, l);
}
template <class R> GT_DEV V3<R> reflect(V3<R> v, V3<R> n) { return v - n * (R(2) * dot(v, n)); }
template <class R> GT_DEV V3<R> refract(V3<R> v, V3<R> n, R eta) { // vector.rs:162-173
    R c = Num<R>::fmin(dot(-v, n), R(1));
    V3<R> perp = (v + n * c) * eta;
    R s = -Num<R>::sqrt(Num<R>::fabs(R(1) - len2(perp)));
    return perp + n * s;
}
template <class R> GT_DEV bool finite3(V3<R> a) {
    return Num<R>::finite(a.x) && Num<R>::finite(a.y) && Num<R>::finite(a.z);
}
// LinearRgb arithmetic (colors.rs:116-190): division is a reciprocal multiply.
template <class R> GT_DEV V3<R> cmul(V3<R> a, V3<R> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class R> GT_DEV V3<R> cdiv(V3<R> a, R s) { return a * (R(1) / s); }
template <class R> GT_DEV R maxc(V3<R> a) { return Num<R>::fmax(Num<R>::fmax(a.x, a.y), a.z); }
template <class R> GT_DEV V3<R> load3(const R* p) { return V3<R>{p[0], p[1], p[2]}; }

// ----------------------------------------------------------------------- RNG
// SplitMix64 sample stream (gmath/random.rs:16-29).
struct Rng {
    uint64_t s;
    GT_DEV uint64_t next() {
        s += 0x9e3779b97f4a7c15ULL;
        uint64_t v = s;
        v = (v ^ (v >> 30)) * 0xbf58476d1ce4e5b9ULL;
        v = (v ^ (v >> 27)) * 0x94d049bb133111ebULL;
        return v ^ (v >> 31);
    }
};
template <class R> GT_DEV R rnd(Rng& g);
// random.rs:56-59: (u64 >> 11) * 2^-53.
template <> GT_DEV double rnd<double>(Rng& g) { return double(g.next() >> 11) * (1.0 / 9007199254740992.0); }
// f32 stream: same draws, top 24 bits, (u64 >> 40) * 2^-24 (exact, in [0, 1)).
template <> GT_DEV float rnd<float>(Rng& g) { return float(uint32_t(g.next() >> 40)) * (1.0f / 16777216.0f); }
template <class R> GT_DEV R rnd_range(Rng& g, R lo, R hi) { return lo + (hi - lo) * rnd<R>(g); }

template <class R> GT_DEV V3<R> unit_vector_spherical(Rng& g) { // random.rs:107-115
    R r1 = rnd<R>(g);
    R r2 = rnd<R>(g);
    R z = R(1) - R(2) * r2;
    R radius = Num<R>::sqrt(R(1) - z * z);
    R phi = R(kTau) * r1;
    R s, c;
    Num<R>::sincos(phi, &s, &c);
    return {c * radius, s * radius, z};
}
template <class R> GT_DEV V3<R> cosine_direction(Rng& g) { // random.rs:119-126
    R r1 = rnd<R>(g);
    R r2 = rnd<R>(g);
    R phi = R(kTau) * r1;
    R radius = Num<R>::sqrt(r2);
    R s, c;
    Num<R>::sincos(phi, &s, &c);
    return {c * radius, s * radius, Num<R>::sqrt(R(1) - r2)};
}

// RayCamera::pixel_seed (camera.rs:1720-1727).
GT_DEV uint64_t pixel_seed(uint64_t seed, uint32_t x, uint32_t y) {
    uint64_t z = seed ^ (uint64_t(x) * 0x9E3779B97F4A7C15ULL) ^ (uint64_t(y) * 0xD1B54A32D192ED03ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

// --------------------------------------------------------------- onb / pdfs
template <class R> struct Onb {
    V3<R> u, v, w;
};
// OrthonormalBasis::from_w (geometry.rs:93-112).
template <class R> GT_DEV bool onb_from_w(V3<R> axis, Onb<R>& b) {
    V3<R> w = normalize(axis);
    if (len2(w) <= R(kEps)) return false;
    V3<R> a = Num<R>::fabs(w.x) > R(0.9) ? V3<R>{0, 1, 0} : V3<R>{1, 0, 0};
    V3<R> v = normalize(cross(w, a));
    b.u = cross(w, v);
    b.v = v;
    b.w = w;
    return true;
}
template <class R> GT_DEV V3<R> onb_local(const Onb<R>& b, V3<R> l) { return (b.u * l.x + b.v * l.y) + b.w * l.z; }

template <class R> GT_DEV R ggx_alpha(R rough) { // sampling.rs:310-312
    R r = clampr(rough, R(0), R(1));
    return Num<R>::fmax(r * r, R(kGgxMinAlpha));
}
template <class R> GT_DEV R ggx_D(R ndh, R rough) { // sampling.rs:212-225
    if (!Num<R>::finite(ndh) || ndh <= R(0) || !Num<R>::finite(rough)) return R(0);
    R alpha = ggx_alpha(rough);
    R a2 = alpha * alpha;
    R cos2 = ndh * ndh;
    R den = cos2 * (a2 - R(1)) + R(1);
    if (den <= R(kEps)) return R(0);
    return a2 / (R(kPi) * den * den);
}
template <class R> GT_DEV R smith_G1(R nd, R rough) { // sampling.rs:314-322
    if (!Num<R>::finite(nd) || nd <= R(0) || !Num<R>::finite(rough)) return R(0);
    R alpha = ggx_alpha(rough);
    R a2 = alpha * alpha;
    R cos2 = nd * nd;
    return R(2) * nd / (nd + Num<R>::sqrt(a2 + (R(1) - a2) * cos2));
}
template <class R> GT_DEV R schlick_f(R cosine, R f0) { // sampling.rs:240-247
    if (!Num<R>::finite(cosine) || !Num<R>::finite(f0)) return R(0);
    f0 = clampr(f0, R(0), R(1));
    return f0 + (R(1) - f0) * pow5(R(1) - clampr(cosine, R(0), R(1)));
}

// HenyeyGreensteinPdf::phase_value (gmath/sampling.rs:126-136), SPHERE_AREA = 4 pi.
template <class R> GT_DEV R hg_phase(R cosine, R g) {
    if (!Num<R>::finite(cosine) || !Num<R>::finite(g) || Num<R>::fabs(g) >= R(1)) return R(0);
    R den = (R(1) + g * g) - (R(2) * g) * clampr(cosine, R(-1), R(1));
    if (den <= R(kEps)) return R(0);
    return (R(1) - g * g) / (R(4.0 * kPi) * Num<R>::pow(den, R(1.5)));
}

// MaterialPdf on the path: Sphere, Cosine, GgxReflection, HenyeyGreenstein (pdf.rs:46-104).
enum : int { PDF_SPHERE = 0, PDF_COSINE = 1, PDF_GGX = 2, PDF_HG = 3 };
template <class R> struct MatPdf {
    int kind;
    Onb<R> basis;
    V3<R> out; // GGX outgoing
    R rough, alpha; // GGX roughness and alpha; HenyeyGreenstein: rough = g
};
template <class R> GT_DEV R matpdf_value(const MatPdf<R>& p, V3<R> dir) {
    if (p.kind == PDF_SPHERE) return R(1) / R(4.0 * kPi); // sampling.rs:31-41
    if (p.kind == PDF_HG) {                             // sampling.rs:139-147
        R l = Num<R>::sqrt(len2(dir));
        if (l <= R(kEps)) return R(0);
        return hg_phase(dot(dir, p.basis.w) / l, p.rough);
    }
    if (p.kind == PDF_COSINE) {                         // sampling.rs:66-78
        R l = Num<R>::sqrt(len2(dir));
        if (l <= R(kEps)) return R(0);
        R c = dot(dir, p.basis.w) / l;
        return c <= R(0) ? R(0) : c / R(kPi);
    }
    V3<R> in = normalize(dir); // sampling.rs:257-272
    if (len2(in) <= R(kEps) || dot(in, p.basis.w) <= R(0)) return R(0);
    V3<R> half = normalize(in + p.out);
    R odh = dot(p.out, half);
    if (len2(half) <= R(kEps) || odh <= R(kEps)) return R(0);
    R ndh = dot(half, p.basis.w);
    return (ggx_D(ndh, p.rough) * Num<R>::fmax(ndh, R(0))) / (R(4) * Num<R>::fabs(odh));
}
template <class R> GT_DEV V3<R> matpdf_generate(const MatPdf<R>& p, Rng& g) {
    if (p.kind == PDF_SPHERE) return unit_vector_spherical<R>(g);
    if (p.kind == PDF_HG) { // sampling.rs:149-164
        const R an = p.rough;
        R r1 = rnd<R>(g);
        R r2 = rnd<R>(g);
        R ct;
        if (Num<R>::fabs(an) < R(1e-3)) {
            ct = R(1) - R(2) * r1;
        } else {
            R term = (R(1) - an * an) / ((R(1) - an) + (R(2) * an) * r1);
            ct = clampr(((R(1) + an * an) - term * term) / (R(2) * an), R(-1), R(1));
        }
        R st = Num<R>::sqrt(Num<R>::fmax(R(1) - ct * ct, R(0)));
        R phi = R(2.0 * kPi) * r2;
        R s, c;
        Num<R>::sincos(phi, &s, &c);
        return onb_local(p.basis, V3<R>{c * st, s * st, ct});
    }
    if (p.kind == PDF_COSINE) return onb_local(p.basis, cosine_direction<R>(g));
    R r1 = rnd<R>(g); // sampling.rs:274-298
    R r2 = rnd<R>(g);
    R phi = R(2) * R(kPi) * r1;
    R a2 = p.alpha * p.alpha;
    R cr2 = Num<R>::fmin(r2, R(1) - R(kEps));
    R tan2 = a2 * cr2 / (R(1) - cr2);
    R ct = R(1) / Num<R>::sqrt(R(1) + tan2);
    R st = Num<R>::sqrt(Num<R>::fmax(R(1) - ct * ct, R(0)));
    R s, c;
    Num<R>::sincos(phi, &s, &c);
    V3<R> half = onb_local(p.basis, V3<R>{c * st, s * st, ct});
    V3<R> refl = reflect(-p.out, normalize(half));
    return dot(refl, p.basis.w) > R(0) ? refl : p.out;
}

template <class R> GT_DEV R power_heuristic(R a, R b) { // camera.rs:2486-2496
    if (!Num<R>::finite(a) || a <= R(kEps)) return R(0);
    if (!Num<R>::finite(b) || b <= R(kEps)) return R(1);
    R sa = a * a, sb = b * b;
    return sa / (sa + sb);
}

} // namespace gt
