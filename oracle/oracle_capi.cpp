// oracle_capi.cpp — TEST INFRASTRUCTURE ONLY: a C entry layer over gartus_oracle.hpp so
// the tests (and bench.py's CPU-baseline leg) can drive the oracle through ctypes with
// the same POD structs the product's C ABI takes.  Nothing in the product links this.
#include <chrono>
#include <memory>

#include "gartus_oracle.hpp"

using namespace oracle;

namespace {

struct OrcScene {
    Scene<double> s64;
    Scene<float> s32;
};

template <class R> void fill_stats(const BvhStats& st, gt_bvh_stats* out) {
    if (!out) return;
    out->rays = st.rays;
    out->node_bounds_tests = st.node_bounds_tests;
    out->node_bounds_hits = st.node_bounds_hits;
    out->leaf_visits = st.leaf_visits;
    out->primitive_candidates = st.primitive_candidates;
    out->leaf_hit_results = st.leaf_hit_results;
    out->max_stack_depth = st.max_stack_depth;
}

template <class R>
int render_impl(const Scene<R>& scene, const gt_light_target* lights, uint32_t nl, const gt_environment_desc* envd,
                const gt_camera_desc* cam, uint32_t rng_mode, uint32_t threads, uint32_t x0, uint32_t y0, uint32_t w,
                uint32_t h, int aovs, double* rgb, double* albedo, double* normal, uint32_t* accepted) {
    LightList<R> ll;
    for (uint32_t i = 0; i < nl; ++i) {
        LightTarget<R> t;
        t.geom = Prim<R>::from_geometry(lights[i].geometry, 0);
        t.weight = R(lights[i].weight);
        ll.total = ll.total + t.weight; // WeightedSamplingTargetList::add_target_weighted, scene.rs:460-476
        ll.targets.push_back(t);
    }
    Environment<R> env;
    if (envd) {
        env.format = int(envd->format);
        env.width = envd->width;
        env.height = envd->height;
        size_t n = size_t(env.width) * env.height * 3;
        if (env.format == GT_ENV_SRGB8) {
            const uint8_t* p = static_cast<const uint8_t*>(envd->texels);
            env.px8.assign(p, p + n);
        } else {
            const float* p = static_cast<const float*>(envd->texels);
            env.px32.assign(p, p + n);
        }
        env.build();
    }
    Renderer<R> r;
    r.scene = &scene;
    r.lights = lights ? &ll : nullptr;
    r.env = envd ? &env : nullptr;
    r.setup(*cam);
    r.substreams = rng_mode == 1;
    if (w == 0) w = r.cam.width;
    if (h == 0) h = r.cam.height;
    if (x0 + w > r.cam.width || y0 + h > r.cam.height) return 1;
    // Tile the requested window.
    const uint32_t tile = 16;
    uint32_t tx = (w + tile - 1) / tile, ty = (h + tile - 1) / tile, total = tx * ty;
    std::atomic<uint32_t> next{0};
    auto worker = [&]() {
        for (;;) {
            uint32_t t = next.fetch_add(1);
            if (t >= total) return;
            uint32_t bx = (t % tx) * tile, by = (t / tx) * tile;
            for (uint32_t yy = by; yy < std::min(by + tile, h); ++yy)
                for (uint32_t xx = bx; xx < std::min(bx + tile, w); ++xx) {
                    size_t o = size_t(yy) * w + xx;
                    uint32_t acc = 0;
                    V3<R> c = r.pixel(x0 + xx, y0 + yy, acc);
                    rgb[o * 3 + 0] = double(c.x);
                    rgb[o * 3 + 1] = double(c.y);
                    rgb[o * 3 + 2] = double(c.z);
                    if (accepted) accepted[o] = acc;
                    if (aovs && albedo) {
                        V3<R> a = r.aov_pixel(x0 + xx, y0 + yy, 0);
                        albedo[o * 3 + 0] = double(a.x);
                        albedo[o * 3 + 1] = double(a.y);
                        albedo[o * 3 + 2] = double(a.z);
                    }
                    if (aovs && normal) {
                        V3<R> nn = r.aov_pixel(x0 + xx, y0 + yy, 1);
                        normal[o * 3 + 0] = double(nn.x);
                        normal[o * 3 + 1] = double(nn.y);
                        normal[o * 3 + 2] = double(nn.z);
                    }
                }
        }
    };
    if (threads <= 1) {
        worker();
    } else {
        std::vector<std::thread> pool;
        for (uint32_t i = 0; i < threads; ++i) pool.emplace_back(worker);
        for (auto& th : pool) th.join();
    }
    return 0;
}

// The decision trace of one pixel (all its samples, in order): the set-up of render_impl
// for one pixel, with g_trace pointing at `out`.
template <class R>
int trace_impl(const Scene<R>& scene, const gt_light_target* lights, uint32_t nl, const gt_environment_desc* envd,
               const gt_camera_desc* cam, uint32_t rng_mode, uint32_t x, uint32_t y, std::vector<TraceEvent>& out) {
    LightList<R> ll;
    for (uint32_t i = 0; i < nl; ++i) {
        LightTarget<R> t;
        t.geom = Prim<R>::from_geometry(lights[i].geometry, 0);
        t.weight = R(lights[i].weight);
        ll.total = ll.total + t.weight;
        ll.targets.push_back(t);
    }
    Environment<R> env;
    if (envd) {
        env.format = int(envd->format);
        env.width = envd->width;
        env.height = envd->height;
        size_t n = size_t(env.width) * env.height * 3;
        if (env.format == GT_ENV_SRGB8) {
            const uint8_t* p = static_cast<const uint8_t*>(envd->texels);
            env.px8.assign(p, p + n);
        } else {
            const float* p = static_cast<const float*>(envd->texels);
            env.px32.assign(p, p + n);
        }
        env.build();
    }
    Renderer<R> r;
    r.scene = &scene;
    r.lights = lights ? &ll : nullptr;
    r.env = envd ? &env : nullptr;
    r.setup(*cam);
    r.substreams = rng_mode == 1;
    if (x >= r.cam.width || y >= r.cam.height) return 1;
    uint32_t acc = 0;
    g_trace = &out;
    r.pixel(x, y, acc);
    g_trace = nullptr;
    return 0;
}

} // namespace

extern "C" {

// Decision trace of pixel (x, y) (TraceEvent): up to `cap` events as (type, outcome)
// pairs and values; returns the number of events the pixel made (possibly above cap), or
// -1 on error.
int64_t orc_pixel_trace(void* sp, const gt_light_target* lights, uint32_t nl, const gt_environment_desc* env,
                        const gt_camera_desc* cam, int precision, uint32_t rng_mode, uint32_t x, uint32_t y,
                        int32_t* kinds, double* values, uint64_t cap) {
    auto* s = static_cast<OrcScene*>(sp);
    std::vector<TraceEvent> ev;
    try {
        const int rc = precision == 1 ? trace_impl<double>(s->s64, lights, nl, env, cam, rng_mode, x, y, ev)
                                      : trace_impl<float>(s->s32, lights, nl, env, cam, rng_mode, x, y, ev);
        if (rc) return -1;
    } catch (...) {
        g_trace = nullptr;
        return -1;
    }
    for (size_t i = 0; i < ev.size() && i < cap; ++i) {
        kinds[2 * i] = ev[i].type;
        kinds[2 * i + 1] = ev[i].outcome;
        values[i] = ev[i].value;
    }
    return int64_t(ev.size());
}

// RayTraversal::hit_bounds (bvh.rs:119-146) of one ray {o, d, time} against box6 {min, max}.
int orc_slab(const double* ray7, const double* box6, double tmin, double tmax, double* entry) {
    Ray<double> ray{{ray7[0], ray7[1], ray7[2]}, {ray7[3], ray7[4], ray7[5]}, ray7[6]};
    Bounds b;
    for (int i = 0; i < 3; ++i) {
        b.mn[i] = box6[i];
        b.mx[i] = box6[3 + i];
    }
    double e = 0.0;
    const bool hit = RayTraversal<double>(ray).hit_bounds(b, tmin, tmax, e);
    if (hit && entry) *entry = e;
    return hit ? 1 : 0;
}

void* orc_scene_create(const gt_scene_desc* d) {
    try {
        auto* s = new OrcScene();
        s->s64.load(*d);
        s->s32.load(*d);
        return s;
    } catch (...) {
        return nullptr;
    }
}

void orc_scene_destroy(void* s) { delete static_cast<OrcScene*>(s); }

uint32_t orc_scene_node_count(void* s) { return uint32_t(static_cast<OrcScene*>(s)->s64.bvh.nodes.size()); }

// Flattened reference-layout BVH: per node {min xyz, max xyz} bounds (6 doubles) and
// {leaf, a, b} (3 uint32); plus the primitive index permutation.
void orc_scene_bvh(void* s, double* bounds, uint32_t* info, uint32_t* indices) {
    const FlatBvh& b = static_cast<OrcScene*>(s)->s64.bvh;
    for (size_t i = 0; i < b.nodes.size(); ++i) {
        for (int k = 0; k < 3; ++k) {
            bounds[i * 6 + k] = b.nodes[i].bounds.mn[k];
            bounds[i * 6 + 3 + k] = b.nodes[i].bounds.mx[k];
        }
        info[i * 3 + 0] = b.nodes[i].leaf ? 1u : 0u;
        info[i * 3 + 1] = b.nodes[i].a;
        info[i * 3 + 2] = b.nodes[i].b;
    }
    for (size_t i = 0; i < b.indices.size(); ++i) indices[i] = b.indices[i];
}

// Closest hits (BVH or brute force) with stats; rays = n x {o, d, time}.
int orc_trace_rays(void* sp, const double* rays, uint32_t n, double tmin, double tmax, int bruteforce, int precision,
                   int32_t* ids, double* t, double* hitinfo, gt_bvh_stats* stats) {
    auto* s = static_cast<OrcScene*>(sp);
    BvhStats total;
    for (uint32_t i = 0; i < n; ++i) {
        const double* r = rays + size_t(i) * 7;
        BvhStats st;
        bool ok;
        double tt = 0, info[8] = {0};
        if (precision == 1) {
            Ray<double> ray{{r[0], r[1], r[2]}, {r[3], r[4], r[5]}, r[6]};
            Hit<double> h;
            ok = bruteforce ? s->s64.hit_bruteforce(ray, tmin, tmax, h) : s->s64.hit(ray, tmin, tmax, h, &st);
            if (ok) {
                tt = h.t;
                double tmp[8] = {h.point.x, h.point.y, h.point.z, h.normal.x, h.normal.y, h.normal.z, h.u, h.v};
                std::memcpy(info, tmp, sizeof(tmp));
                ids[i] = h.prim;
            }
        } else {
            Ray<float> ray{{float(r[0]), float(r[1]), float(r[2])}, {float(r[3]), float(r[4]), float(r[5])}, float(r[6])};
            Hit<float> h;
            ok = bruteforce ? s->s32.hit_bruteforce(ray, float(tmin), float(tmax), h)
                            : s->s32.hit(ray, float(tmin), float(tmax), h, &st);
            if (ok) {
                tt = h.t;
                double tmp[8] = {h.point.x, h.point.y, h.point.z, h.normal.x, h.normal.y, h.normal.z, h.u, h.v};
                std::memcpy(info, tmp, sizeof(tmp));
                ids[i] = h.prim;
            }
        }
        if (!ok) ids[i] = -1;
        if (t) t[i] = ok ? tt : 0.0;
        if (hitinfo) std::memcpy(hitinfo + size_t(i) * 8, info, sizeof(info));
        total.merge(st);
    }
    fill_stats<double>(total, stats);
    return 0;
}

// Camera derived vectors (center, pixel00, du, dv, ddu, ddv) and size.
int orc_camera(const gt_camera_desc* d, uint32_t* w, uint32_t* h, uint32_t* spp, double* out18) {
    Camera<double> c;
    c.init(*d);
    *w = c.width;
    *h = c.height;
    *spp = c.effective_spp();
    V3<double> vs[6] = {c.center, c.pixel00, c.du, c.dv, c.ddu, c.ddv};
    for (int i = 0; i < 6; ++i) {
        out18[i * 3 + 0] = vs[i].x;
        out18[i * 3 + 1] = vs[i].y;
        out18[i * 3 + 2] = vs[i].z;
    }
    return 0;
}

// Primary probe rays (RayCamera::ray_for_pixel) for every stride-th pixel, f64.
int orc_trace_primary(void* sp, const gt_camera_desc* d, uint32_t stride, int32_t* ids, double* t, gt_bvh_stats* stats) {
    auto* s = static_cast<OrcScene*>(sp);
    Camera<double> c;
    c.init(*d);
    if (stride == 0) stride = 1;
    BvhStats total;
    size_t k = 0;
    for (uint32_t y = 0; y < c.height; y += stride)
        for (uint32_t x = 0; x < c.width; x += stride) {
            Ray<double> ray = c.ray_for_pixel(x, y);
            Hit<double> h;
            BvhStats st;
            bool ok = s->s64.hit(ray, kShadowAcne, std::numeric_limits<double>::infinity(), h, &st);
            ids[k] = ok ? h.prim : -1;
            if (t) t[k] = ok ? h.t : 0.0;
            ++k;
            total.merge(st);
        }
    fill_stats<double>(total, stats);
    return 0;
}

// Renders the window [x0, x0+w) x [y0, y0+h) (w = h = 0: the whole image).
// precision: 1 = Oracle<double>, 0 = Oracle<float>; rng_mode: 0 = the pixel's one stream
// (the reference), 1 = a substream per sample.  Returns 0 on success.
int orc_render(void* sp, const gt_light_target* lights, uint32_t nl, const gt_environment_desc* env,
               const gt_camera_desc* cam, int precision, uint32_t rng_mode, uint32_t threads, uint32_t x0, uint32_t y0,
               uint32_t w, uint32_t h, int aovs, double* rgb, double* albedo, double* normal, uint32_t* accepted) {
    auto* s = static_cast<OrcScene*>(sp);
    try {
        if (precision == 1)
            return render_impl<double>(s->s64, lights, nl, env, cam, rng_mode, threads, x0, y0, w, h, aovs, rgb, albedo,
                                       normal, accepted);
        return render_impl<float>(s->s32, lights, nl, env, cam, rng_mode, threads, x0, y0, w, h, aovs, rgb, albedo,
                                  normal, accepted);
    } catch (...) {
        return 2;
    }
}

// ---------------------------------------------------------- known-answer probes
uint64_t orc_pixel_seed(uint64_t seed, uint32_t x, uint32_t y) { return pixel_seed(seed, x, y); }

void orc_rng_u64(uint64_t seed, uint32_t n, uint64_t* out) {
    SampleRng r(seed);
    for (uint32_t i = 0; i < n; ++i) out[i] = r.next_u64();
}

// Perlin::noise / turbulence at n points (xyz triples); depth < 0 = noise, else turbulence.
void orc_perlin(uint64_t seed, int precision, int depth, uint32_t n, const double* pts, double* out) {
    Perlin p(seed);
    for (uint32_t i = 0; i < n; ++i) {
        if (precision == 1) {
            V3<double> q{pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
            out[i] = depth < 0 ? p.noise(q) : p.turbulence(q, depth);
        } else {
            V3<float> q{float(pts[3 * i]), float(pts[3 * i + 1]), float(pts[3 * i + 2])};
            out[i] = depth < 0 ? double(p.noise(q)) : double(p.turbulence(q, depth));
        }
    }
}

// The permutation tables and gradients of Perlin::new(seed).
void orc_perlin_tables(uint64_t seed, double* grad768, int32_t* perm768) {
    Perlin p(seed);
    for (int i = 0; i < 256; ++i)
        for (int k = 0; k < 3; ++k) {
            grad768[i * 3 + k] = p.grad[i][k];
            perm768[k * 256 + i] = p.perm[k][i];
        }
}

void orc_rng_double(uint64_t seed, uint32_t n, double* out) {
    SampleRng r(seed);
    for (uint32_t i = 0; i < n; ++i) out[i] = r.random_double<double>();
}

// Single-primitive intersection: out = {t, u, v, px, py, pz, nx, ny, nz, front}.
int orc_intersect(const gt_geometry* g, const double* ray7, double tmin, double tmax, double* out) {
    Prim<double> p = Prim<double>::from_geometry(*g, 0);
    Ray<double> r{{ray7[0], ray7[1], ray7[2]}, {ray7[3], ray7[4], ray7[5]}, ray7[6]};
    Hit<double> h;
    if (!intersect(p, r, tmin, tmax, h)) return 0;
    double tmp[10] = {h.t, h.u, h.v, h.point.x, h.point.y, h.point.z, h.normal.x, h.normal.y, h.normal.z,
                      h.front_face ? 1.0 : 0.0};
    std::memcpy(out, tmp, sizeof(tmp));
    return 1;
}

void orc_geometry_bounds(const gt_geometry* g, double* out6) {
    Bounds b = geometry_bounds(*g);
    for (int k = 0; k < 3; ++k) {
        out6[k] = b.mn[k];
        out6[3 + k] = b.mx[k];
    }
}

double orc_geometry_pdf(const gt_geometry* g, const double* origin, double time, const double* dir) {
    Prim<double> p = Prim<double>::from_geometry(*g, 0);
    return geometry_pdf_value(p, V3<double>(origin[0], origin[1], origin[2]), time, V3<double>(dir[0], dir[1], dir[2]));
}

// Weighted target list: fraction of `n` random_direction draws that land on target 0.
double orc_lights_first_fraction(const gt_light_target* lights, uint32_t nl, const double* origin, uint64_t seed,
                                 uint32_t n) {
    LightList<double> ll;
    for (uint32_t i = 0; i < nl; ++i) {
        LightTarget<double> t;
        t.geom = Prim<double>::from_geometry(lights[i].geometry, 0);
        t.weight = lights[i].weight;
        ll.total += t.weight;
        ll.targets.push_back(t);
    }
    SampleRng rng(seed);
    uint32_t first = 0;
    V3<double> o(origin[0], origin[1], origin[2]);
    for (uint32_t i = 0; i < n; ++i) {
        V3<double> d = ll.random_direction(o, 0.0, rng);
        if (geometry_pdf_value(ll.targets[0].geom, o, 0.0, d) > 0.0) ++first;
    }
    return double(first) / double(n);
}

double orc_env_pdf(const gt_environment_desc* envd, const double* dir) {
    Environment<double> env;
    env.format = int(envd->format);
    env.width = envd->width;
    env.height = envd->height;
    size_t n = size_t(env.width) * env.height * 3;
    if (env.format == GT_ENV_SRGB8) {
        const uint8_t* p = static_cast<const uint8_t*>(envd->texels);
        env.px8.assign(p, p + n);
    } else {
        const float* p = static_cast<const float*>(envd->texels);
        env.px32.assign(p, p + n);
    }
    env.build();
    return env.pdf_value(V3<double>(dir[0], dir[1], dir[2]));
}

// Material probes: scatter (returns kind), scattering_pdf and the GGX helpers.
double orc_ggx_d(double ndh, double rough) { return ggx_d(ndh, rough); }
double orc_ggx_g(double ndi, double ndo, double rough) { return smith_g1(ndi, rough) * smith_g1(ndo, rough); }
double orc_schlick(double c, double f0) { return schlick(c, f0); }
double orc_dielectric_reflectance(double cosine, double ratio) {
    double r0 = (1.0 - ratio) / (1.0 + ratio);
    r0 = r0 * r0;
    return r0 + (1.0 - r0) * powi5(1.0 - cosine);
}
double orc_power_heuristic(double a, double b) { return power_heuristic(a, b); }
double orc_adaptive_error(const double* m2, uint32_t n) {
    return Renderer<double>::adaptive_error(V3<double>(m2[0], m2[1], m2[2]), n);
}
void orc_background(const gt_camera_desc* d, const double* dir, double* out) {
    V3<double> c = background_radiance<double>(*d, V3<double>(dir[0], dir[1], dir[2]));
    out[0] = c.x;
    out[1] = c.y;
    out[2] = c.z;
}
// Metal scatter direction with a given rng seed: returns 1 if scattered.
int orc_scatter(const gt_material* md, const double* ray7, const double* point, const double* normal, int front,
                uint64_t seed, double* out_dir, double* out_att, uint64_t* out_state) {
    Material<double> m = Material<double>::from_desc(*md);
    Ray<double> r{{ray7[0], ray7[1], ray7[2]}, {ray7[3], ray7[4], ray7[5]}, ray7[6]};
    Hit<double> h;
    h.point = V3<double>(point[0], point[1], point[2]);
    h.normal = V3<double>(normal[0], normal[1], normal[2]);
    h.shading = h.normal;
    h.front_face = front != 0;
    SampleRng rng(seed);
    Scatter<double> s = scatter(m, r, h, rng);
    *out_state = rng.state;
    if (s.kind == SCATTER_NONE) return 0;
    V3<double> d = s.kind == SCATTER_SPECULAR ? s.ray.d : s.pdf.generate(rng);
    out_dir[0] = d.x;
    out_dir[1] = d.y;
    out_dir[2] = d.z;
    out_att[0] = s.att.x;
    out_att[1] = s.att.y;
    out_att[2] = s.att.z;
    *out_state = rng.state;
    return s.kind;
}
double orc_scattering_pdf(const gt_material* md, const double* ray7, const double* point, const double* normal,
                          int front, const double* dir) {
    Material<double> m = Material<double>::from_desc(*md);
    Ray<double> r{{ray7[0], ray7[1], ray7[2]}, {ray7[3], ray7[4], ray7[5]}, ray7[6]};
    Hit<double> h;
    h.point = V3<double>(point[0], point[1], point[2]);
    h.normal = V3<double>(normal[0], normal[1], normal[2]);
    h.shading = h.normal;
    h.front_face = front != 0;
    return scattering_pdf(m, r, h, V3<double>(dir[0], dir[1], dir[2]));
}
// ConstantMedium::hit_with_rng of one medium alone on ray7 = {origin, direction, time} in
// (tmin, tmax) with a SampleRng seeded `seed`: 1 and *t on a scatter, else 0; *draws = the
// number of draws taken.
int orc_medium_hit(const gt_medium* m, const double* ray7, double tmin, double tmax, uint64_t seed, double* t,
                   uint32_t* draws) {
    const Medium<double> md = Medium<double>::from_desc(*m);
    Ray<double> r;
    r.o = V3<double>(ray7[0], ray7[1], ray7[2]);
    r.d = V3<double>(ray7[3], ray7[4], ray7[5]);
    r.time = ray7[6];
    SampleRng rng(seed);
    SampleRng start = rng;
    double th = 0.0;
    const bool hit = md.hit(r, tmin, tmax, rng, th);
    uint32_t n = 0;
    while (start.state != rng.state && n < 8) {
        start.next_u64();
        ++n;
    }
    *draws = n;
    *t = hit ? th : 0.0;
    return hit ? 1 : 0;
}

// The world's closest hit (surfaces, objects, media) of ray7 = {origin, direction, time} in
// (tmin, tmax), f64, media drawing from a SampleRng seeded `seed`.  out[14] = t, point,
// normal, shading normal, u, v, front face, material.  Returns 1 on a hit.
int orc_world_hit(void* sp, const double* ray7, double tmin, double tmax, uint64_t seed, double* out) {
    const Scene<double>& sc = static_cast<OrcScene*>(sp)->s64;
    Ray<double> r;
    r.o = V3<double>(ray7[0], ray7[1], ray7[2]);
    r.d = V3<double>(ray7[3], ray7[4], ray7[5]);
    r.time = ray7[6];
    SampleRng rng(seed);
    Hit<double> h;
    if (!sc.world_hit(r, tmin, tmax, h, rng)) return 0;
    const double v[14] = {h.t, h.point.x, h.point.y, h.point.z, h.normal.x, h.normal.y, h.normal.z,
                          h.shading.x, h.shading.y, h.shading.z, h.u, h.v, h.front_face ? 1.0 : 0.0,
                          double(h.material)};
    std::memcpy(out, v, sizeof(v));
    return 1;
}

// ImageTexture sampling at (u, v) into linear RGB.
void orc_image_sample(const gt_image* g, double u, double v, double* out) {
    ImageData im;
    im.w = g->width;
    im.h = g->height;
    im.filter = int(g->filter);
    im.wrap_s = int(g->wrap_s);
    im.wrap_t = int(g->wrap_t);
    if (g->rgb) im.rgb.assign(g->rgb, g->rgb + size_t(g->width) * g->height * 3);
    const V3<double> c = im.sample<double>(u, v);
    out[0] = c.x;
    out[1] = c.y;
    out[2] = c.z;
}
double orc_cosine_pdf(const double* normal, const double* dir) {
    MatPdf<double> p;
    p.kind = PDF_COSINE;
    if (!Onb<double>::from_w(V3<double>(normal[0], normal[1], normal[2]), p.basis)) return -1.0;
    return p.value(V3<double>(dir[0], dir[1], dir[2]));
}

} // extern "C"
