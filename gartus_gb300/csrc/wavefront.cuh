// wavefront.cuh — the wavefront integrator.  One path slot per pixel carries that pixel's
// sequential SplitMix64 stream from sample to sample (camera.rs:2669, 2685-2717).  Each
// iteration runs four kernels over compacted queues:
//   generate : finish the slot's previous sample (accumulate), start the next camera ray
//   trace    : closest hit for every queued ray, then bin the slot by material kind
//   shade    : one bounce of RayCamera::ray_color (camera.rs:1730-1862) per slot, with
//              warps reading one material's queue at a time
//   shadow   : the deferred next-event shadow queries of this bounce
// Queues are filled with warp-aggregated atomics (ballot / match_any + popc).
#pragma once

#include "scene_query.cuh"

namespace gt {

// One round of the throughput mode on the wavefront: slot i holds sample
// first + i / count of pixel list[i % count]; its radiance goes to out[i].
template <class R> struct SubRound {
    const uint32_t* list;
    R4<R>* out;
    uint32_t count, first;
};

template <class R> struct Params {
    SceneDev<R> sc;
    LightsDev<R> lights;
    EnvDev<R> env;
    CamDev<R> cam;
    PathState<R> ps;
    // Batched frames (kernels instantiated with BATCH = true): one camera per frame,
    // frame f owns the global pixel range [frame_start[f], frame_start[f + 1]).
    const CamDev<R>* cams;
    const uint32_t* frame_start;
    uint32_t num_frames;
    // Throughput mode (substreams) on the wavefront: the current round, in device memory
    // so that a stripe's cached graph serves every round; null in the reference mode.
    const SubRound<R>* sub;
};

// The camera of global pixel `pix` and the pixel's index within its frame: in a batch the
// frame is found by binary search over frame_start; otherwise it is the render's camera.
template <class R, bool BATCH> GT_DEV const CamDev<R>& cam_of(const Params<R>& P, uint32_t pix, uint32_t& local) {
    if constexpr (BATCH) {
        uint32_t lo = 0, hi = P.num_frames;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (__ldg(&P.frame_start[mid]) <= pix) lo = mid;
            else hi = mid;
        }
        local = pix - __ldg(&P.frame_start[lo]);
        return P.cams[lo];
    } else {
        local = pix;
        return P.cam;
    }
}

GT_DEV uint32_t lane_id() { return threadIdx.x & 31u; }
GT_DEV uint32_t lanemask_lt() { return (1u << lane_id()) - 1u; }

// All 32 lanes call; lanes with `want` append `value` to `queue`.
GT_DEV void warp_push(bool want, uint32_t value, uint32_t* queue, uint32_t* counter) {
    const unsigned m = __ballot_sync(0xffffffffu, want);
    if (m == 0) return;
    const uint32_t leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane_id() == leader) base = atomicAdd(counter, __popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (want) queue[base + __popc(m & lanemask_lt())] = value;
}

// All 32 lanes call; lanes with `want` append `value` to queue `key` (capacity `cap`).
GT_DEV void warp_push_keyed(bool want, uint32_t key, uint32_t value, uint32_t* queues, uint32_t cap,
                            uint32_t* counters) {
    const unsigned m = __ballot_sync(0xffffffffu, want);
    if (!want) return;
    const unsigned peers = __match_any_sync(m, key);
    const uint32_t leader = __ffs(peers) - 1;
    uint32_t base = 0;
    if (lane_id() == leader) base = atomicAdd(&counters[key], __popc(peers));
    base = __shfl_sync(peers, base, leader);
    queues[size_t(key) * cap + base + __popc(peers & lanemask_lt())] = value;
}

template <class R> GT_DEV void kahan_add(R4<R>& sum, R4<R>& c, V3<R> s);
// f32: Kahan-compensated running sum.
template <> GT_DEV void kahan_add<float>(R4<float>& sum, R4<float>& c, V3<float> s) {
    float in[3] = {s.x, s.y, s.z};
    float* sp[3] = {&sum.x, &sum.y, &sum.z};
    float* cp[3] = {&c.x, &c.y, &c.z};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float y = in[k] - *cp[k];
        float t = *sp[k] + y;
        *cp[k] = (t - *sp[k]) - y;
        *sp[k] = t;
    }
}
// f64: the reference's plain `pixel_color += sample` (camera.rs:2984-2991).
template <> GT_DEV void kahan_add<double>(R4<double>& sum, R4<double>& c, V3<double> s) {
    (void)c;
    sum.x = sum.x + s.x;
    sum.y = sum.y + s.y;
    sum.z = sum.z + s.z;
}

template <class R> GT_DEV R adaptive_error(V3<R> m2, uint32_t n) { // camera.rs:2962-2972
    if (n <= 1) return Num<R>::inf();
    V3<R> var = cdiv(m2, R(n - 1));
    return Num<R>::sqrt(Num<R>::fmax(maxc(cdiv(var, R(n))), R(0)));
}

template <class R, bool BATCH = false> __global__ void k_init(Params<R> P) {
    const uint32_t n = P.ps.n;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t local;
        const CamDev<R>& C = cam_of<R, BATCH>(P, i, local);
        const uint32_t x = local % C.width, y = local / C.width;
        const uint64_t s = pixel_seed(C.seed, x, y);
        P.ps.st[i] = make_uint4(uint32_t(s), uint32_t(s >> 32), F_NEWSAMPLE, 0u);
        P.ps.acc[i] = R4<R>{0, 0, 0, 0};
        P.ps.comp[i] = R4<R>{0, 0, 0, 0};
        P.ps.accepted[i] = 0;
    }
    if (blockIdx.x == 0 && threadIdx.x < C_COUNT) P.ps.counters[threadIdx.x] = 0;
    if (blockIdx.x == 0 && threadIdx.x < 8) P.ps.totals[threadIdx.x] = 0;
}

// Folds a finished sample into the pixel; returns true when adaptive sampling stops.
template <class R> GT_DEV bool finish_sample(const Params<R>& P, const CamDev<R>& C, uint32_t slot, V3<R> s) {
    if (!finite3(s)) return false; // non-finite samples are dropped (camera.rs:2984-2999, 2951-2953)
    R4<R> a = P.ps.acc[slot], c = P.ps.comp[slot];
    uint32_t acc_n = P.ps.accepted[slot] + 1;
    bool stop = false;
    if (C.adaptive) { // Welford update, camera.rs:2955-2960
        V3<R> mean = xyz(a), m2 = xyz(c);
        V3<R> delta = s - mean;
        mean = mean + cdiv(delta, R(acc_n));
        V3<R> delta2 = s - mean;
        m2 = m2 + cmul(delta, delta2);
        a = R4<R>{mean.x, mean.y, mean.z, R(0)};
        c = R4<R>{m2.x, m2.y, m2.z, R(0)};
        stop = acc_n >= C.adaptive_min && adaptive_error(m2, acc_n) < C.adaptive_threshold;
    } else {
        kahan_add(a, c, s);
    }
    P.ps.acc[slot] = a;
    P.ps.comp[slot] = c;
    P.ps.accepted[slot] = acc_n;
    return stop;
}

template <class R, bool BATCH = false> __global__ void __launch_bounds__(256) k_generate(Params<R> P, uint32_t cur) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        P.ps.counters[C_TRACE0 + (cur ^ 1u)] = 0;
        for (uint32_t k = 0; k < NUM_KEYS; ++k) P.ps.counters[C_MAT + k] = 0;
        P.ps.counters[C_SHADOW] = 0;
    }
    const uint32_t n = P.ps.local_n;
    const uint32_t warp0 = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u;
    const uint32_t stride = gridDim.x * blockDim.x;
    SubRound<R> sr{nullptr, nullptr, 0u, 0u};
    if constexpr (!BATCH) {
        if (P.sub) sr = *P.sub;
    }
    for (uint32_t base = warp0; base < n; base += stride) {
        const uint32_t j = base + lane_id();
        const uint32_t slot = j < n ? stripe_slot(P.ps, j) : 0u;
        bool push = false;
        if (j < n && sr.list) { // substreams: the slot's one sample, then its radiance out
            uint4 st = P.ps.st[slot];
            if (st.z & F_NEWSAMPLE) {
                uint32_t flags = F_DONE;
                Rng g{uint64_t(st.x) | (uint64_t(st.y) << 32)};
                if (st.w > 0) {
                    const R4<R> c = P.ps.col[slot];
                    sr.out[slot] = R4<R>{c.x, c.y, c.z, R(1)};
                } else {
                    const CamDev<R>& C = P.cam;
                    const uint32_t pix = sr.list[slot % sr.count], s = sr.first + slot / sr.count;
                    V3<R> o, d;
                    R time;
                    camera_ray(C, pix % C.width, pix / C.width, s, g, o, d, time);
                    if (C.max_depth == 0) { // the bounce loop never runs: a black sample
                        sr.out[slot] = R4<R>{0, 0, 0, R(1)};
                    } else {
                        P.ps.ray_o[slot] = R4<R>{o.x, o.y, o.z, time};
                        P.ps.ray_d[slot] = R4<R>{d.x, d.y, d.z, R(1)};
                        P.ps.att[slot] = R4<R>{1, 1, 1, 0};
                        P.ps.col[slot] = R4<R>{0, 0, 0, 0};
                        flags = F_TRACE | F_ALLOW_EMIT;
                        push = true;
                    }
                }
                if (!push) atomicAdd(&P.ps.counters[C_DONE], 1u);
                P.ps.st[slot] = make_uint4(uint32_t(g.s), uint32_t(g.s >> 32), flags, 1u);
            }
        } else if (j < n) {
            uint4 st = P.ps.st[slot];
            if (st.z & F_NEWSAMPLE) {
                uint32_t local;
                const CamDev<R>& C = cam_of<R, BATCH>(P, slot, local);
                const uint32_t limit = C.adaptive ? C.adaptive_max : C.spp;
                Rng g{uint64_t(st.x) | (uint64_t(st.y) << 32)};
                uint32_t started = st.w;
                bool stop = false;
                if (started > 0 && !(st.z & F_FRESH)) stop = finish_sample(P, C, slot, xyz(P.ps.col[slot]));
                const uint32_t x = local % C.width, y = local / C.width;
                uint32_t flags = F_DONE;
                while (!stop && started < limit) {
                    V3<R> o, d;
                    R time;
                    camera_ray(C, x, y, started, g, o, d, time);
                    ++started;
                    if (C.max_depth == 0) { // the bounce loop never runs: a black sample
                        stop = finish_sample(P, C, slot, V3<R>{0, 0, 0});
                        continue;
                    }
                    P.ps.ray_o[slot] = R4<R>{o.x, o.y, o.z, time};
                    P.ps.ray_d[slot] = R4<R>{d.x, d.y, d.z, R(1)};
                    P.ps.att[slot] = R4<R>{1, 1, 1, 0};
                    P.ps.col[slot] = R4<R>{0, 0, 0, 0};
                    flags = F_TRACE | F_ALLOW_EMIT;
                    push = true;
                    break;
                }
                if (!push) atomicAdd(&P.ps.counters[C_DONE], 1u);
                P.ps.st[slot] = make_uint4(uint32_t(g.s), uint32_t(g.s >> 32), flags, started);
            }
        }
        warp_push(push, slot, P.ps.q_trace[cur], &P.ps.counters[C_TRACE0 + cur]);
    }
}

// The per-iteration counter resets of k_generate, for substream iterations after the first
// in scenes without next-event queries (there k_shade writes each finished sample out, so
// no slot needs k_generate again).
template <class R> __global__ void k_iteration_reset(Params<R> P, uint32_t cur) {
    if (threadIdx.x == 0) P.ps.counters[C_TRACE0 + (cur ^ 1u)] = 0;
    if (threadIdx.x < NUM_KEYS) P.ps.counters[C_MAT + threadIdx.x] = 0;
    if (threadIdx.x == 0) P.ps.counters[C_SHADOW] = 0;
}

// Resident 256-thread blocks per SM of the f32 traversal and shade kernels (their launch
// bounds): more than the registers alone would allow, spilling into L1, because the
// stripes' launches then share the SMs better (mesh-heavy frame 297 -> 332 Msamples/s).
constexpr uint32_t kTraceBlocksPerSm = 6, kShadowBlocksPerSm = 5, kShadeBlocksPerSm = 4;

// OBJ: a world with objects and no media (whose hits draw no random numbers, so the
// deferred shadow queries keep the reference's order of draws): after the RayScene's tree
// the ray tests the objects (objects_hit, as world_hit does), and an object hit stores the
// object in hit_obj and the mesh's leaf in hit_prim.
template <class R, bool OBJ = false>
__global__ void __launch_bounds__(256, kTraceBlocksPerSm) k_trace(Params<R> P, uint32_t cur) {
    const uint32_t count = *reinterpret_cast<volatile uint32_t*>(&P.ps.counters[C_TRACE0 + cur]);
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&P.ps.totals[0], (unsigned long long)count);
    const uint32_t* q = P.ps.q_trace[cur];
    const uint32_t warp0 = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u;
    const uint32_t stride = gridDim.x * blockDim.x;
    const R inf = Num<R>::inf();
    for (uint32_t base = warp0; base < count; base += stride) {
        const uint32_t i = base + lane_id();
        const bool valid = i < count;
        uint32_t slot = 0, key = 0;
        if (valid) {
            slot = q[i];
            R4<R> o = P.ps.ray_o[slot], d = P.ps.ray_d[slot];
            R t = R(0);
            int prim = traverse<R, false, false>(P.sc, xyz(o), xyz(d), o.w, R(kShadowAcne), inf, t, nullptr,
                                                 &P.ps.counters[C_ERROR]);
            uint32_t mat = prim < 0 ? 0u : __ldg(&P.sc.meta[prim].x) >> 3;
            if constexpr (OBJ) {
                if (prim < 0) t = inf;
                int obj = -1, leaf = -1;
                objects_hit(P.sc, xyz(o), xyz(d), o.w, R(kShadowAcne), t, obj, leaf, &P.ps.counters[C_ERROR]);
                if (obj >= 0) {
                    prim = leaf;
                    mat = __ldg(&P.sc.meshes[P.sc.objects[obj].mesh].view.meta[leaf].x) >> 3;
                }
                P.ps.hit_obj[slot] = obj;
            }
            P.ps.hit_t[slot] = t;
            P.ps.hit_prim[slot] = prim;
            key = prim < 0 ? KEY_MISS : uint32_t(P.sc.mats[mat].kind);
        }
        warp_push_keyed(valid, key, slot, P.ps.q_mat, P.ps.qcap, &P.ps.counters[C_MAT]);
    }
}

template <class R> GT_DEV bool rr_survives(const CamDev<R>& cam, uint32_t bounce, V3<R>& att, Rng& g) {
    if (cam.rr_min_depth < 0 || bounce < uint32_t(cam.rr_min_depth)) return true; // camera.rs:2498-2523
    R m = maxc(att);
    if (!Num<R>::finite(m) || m <= R(kEps)) return false;
    R p = clampr(m, R(0.05), R(0.95));
    if (rnd<R>(g) >= p) return false;
    att = cdiv(att, p);
    return true;
}

// The in-flight state of one path (one sample of RayCamera::ray_color).
template <class R> struct Path {
    V3<R> o, d;
    R time;
    R miss_w; // miss_radiance_weight
    V3<R> att, col;
    uint32_t bounce;
    bool allow_emit;
};

// Next-event shadow queries produced by a bounce: k = 0 area light (closest hit, the hit's
// emission counts), k = 1 environment (occlusion only).  The contribution added to the
// sample is att * ((s * e) * ratio) with e the emission found (area) or 1 (environment).
template <class R> struct Shadow {
    bool valid[2];
    V3<R> o;
    R time;
    V3<R> dir[2];
    V3<R> att;
    V3<R> s[2];
    R ratio[2];
    uint32_t traced; // queries traced inline (scenes with media)
};

// Resolves shadow query k (after traversal) into the sample's radiance.
// `wh`: the hit record of an object hit (closest-hit query of a world with objects).
template <class R>
GT_DEV void apply_shadow(const Params<R>& P, V3<R>& col, const Shadow<R>& sh, int k, int prim, R t,
                         const HitRec<R>* wh = nullptr) {
    if (k == 0) { // closest hit; the emission of whatever is hit (camera.rs:2248-2261)
        if (prim < 0) return;
        HitRec<R> h = wh ? *wh : make_hit(P.sc, uint32_t(prim), sh.o, sh.dir[0], sh.time, t);
        V3<R> e = mat_emitted(P.sc.mats[h.mat], h);
        if (!finite3(e)) return;
        V3<R> direct = cmul(sh.s[0], e) * sh.ratio[0];
        col = col + cmul(sh.att, direct);
    } else { // occlusion only (camera.rs:2284-2293)
        if (prim >= 0) return;
        V3<R> direct = sh.s[1] * sh.ratio[1];
        col = col + cmul(sh.att, direct);
    }
}

// A next-event shadow query of a world with objects or media, traced where the reference
// traces it (inside estimate_direct_lighting / estimate_environment_lighting,
// camera.rs:2248, 2284): the world's closest hit, whose media draws come before the next
// sample of the bounce.  The environment query needs the closest hit too, since it clips
// the media's intervals.
template <class R> GT_DEV void shadow_now(const Params<R>& P, V3<R>& col, Shadow<R>& sh, int k, Rng& g) {
    HitRec<R> h;
    const bool hit = world_hit(P.sc, sh.o, sh.dir[k], sh.time, R(kShadowAcne), g, h, &P.ps.counters[C_ERROR]);
    sh.traced += 1;
    if (k == 0) {
        if (!hit) return;
        const V3<R> e = mat_emitted(P.sc.mats[h.mat], h);
        if (!finite3(e)) return;
        col = col + cmul(sh.att, cmul(sh.s[0], e) * sh.ratio[0]);
    } else if (!hit) {
        col = col + cmul(sh.att, sh.s[1] * sh.ratio[1]);
    }
}

// One iteration of the bounce loop of ray_color (camera.rs:1742-1859): miss radiance,
// emission, scatter, next-event sampling (camera.rs:2225-2297), continuation sample
// (camera.rs:165-195) and Russian roulette (camera.rs:2498-2523).  `prim` < 0 is a miss.
// Returns true if the path continues to another bounce.
// WORLD: a world with objects or media; the hit record comes from world_hit (`wh`, prim 0
// for a hit, -1 for a miss) and the shadow queries are traced here, in the reference's
// order of draws, instead of being left in `sh`.
// OBJ: the wavefront's world with objects; a non-null `wh` is an object hit's record,
// and the shadow queries are left in `sh` as usual.
template <class R, bool WORLD = false, bool OBJ = false>
GT_DEV bool integrate_bounce(const Params<R>& P, const CamDev<R>& cam, Path<R>& p, int prim, R t, Rng& g,
                             Shadow<R>& sh, const HitRec<R>* wh = nullptr) {
    sh.valid[0] = sh.valid[1] = false;
    sh.traced = 0;
    bool cont = false;
    if (prim < 0) {
        V3<R> bg = cam.use_env ? env_radiance(P.env, p.d) : background(cam, p.d);
        V3<R> miss = bg * p.miss_w;
        p.col = p.col + cmul(p.att, miss);
        return false;
    }
    const HitRec<R> h = WORLD || (OBJ && wh) ? *wh : make_hit(P.sc, uint32_t(prim), p.o, p.d, p.time, t);
    const MatDev<R> m = P.sc.mats[h.mat];
    if (p.allow_emit) p.col = p.col + cmul(p.att, mat_emitted(m, h));
    ScatterRec<R> s = mat_scatter(m, p.d, h, g);
    if (s.kind == SC_SPECULAR) {
        p.att = cmul(p.att, s.att);
        p.o = spawn_origin(h, s.dir);
        p.d = s.dir;
        p.allow_emit = true;
        p.miss_w = R(1);
        cont = rr_survives(cam, p.bounce, p.att, g);
    } else if (s.kind == SC_PDF) {
        if (cam.nee) {
            sh.o = h.p;
            sh.time = p.time;
            sh.att = p.att;
            if (cam.use_lights) { // estimate_direct_lighting, camera.rs:2225-2262
                V3<R> ldir = lights_dir(P.lights, h.p, p.time, g);
                R lp = lights_pdf(P.lights, h.p, p.time, ldir);
                if (Num<R>::finite(lp) && lp > R(kEps)) {
                    R sp = mat_scattering_pdf(m, p.d, h, ldir);
                    if (Num<R>::finite(sp) && sp > R(0)) {
                        sh.valid[0] = true;
                        sh.dir[0] = ldir;
                        sh.s[0] = s.att;
                        sh.ratio[0] = sp / lp;
                    }
                }
            }
            const bool area = sh.valid[0];
            if (WORLD && area) {
                sh.o = spawn_origin(h, sh.dir[0]);
                shadow_now(P, p.col, sh, 0, g);
                sh.valid[0] = false;
            }
            if (cam.use_env) { // estimate_environment_lighting, camera.rs:2264-2297
                V3<R> edir;
                R ep;
                env_sample(P.env, g, edir, ep);
                if (Num<R>::finite(ep) && ep > R(kEps)) {
                    R sp = mat_scattering_pdf(m, p.d, h, edir);
                    if (Num<R>::finite(sp) && sp > R(0)) {
                        R mis = power_heuristic(ep, sp);
                        sh.valid[1] = true;
                        sh.dir[1] = edir;
                        sh.s[1] = cmul(s.att, env_radiance(P.env, edir));
                        sh.ratio[1] = mis * sp / ep;
                    }
                }
            }
            if (WORLD) {
                if (sh.valid[1]) {
                    if (!area) sh.o = spawn_origin(h, sh.dir[1]);
                    shadow_now(P, p.col, sh, 1, g);
                    sh.valid[1] = false;
                }
            } else if (sh.valid[0] || sh.valid[1]) {
                sh.o = spawn_origin(h, sh.valid[0] ? sh.dir[0] : sh.dir[1]);
            }
        }
        V3<R> dir;
        R pdf;
        bool suppress = false, weight_env = false;
        if (!cam.nee && cam.use_lights) {
            const R w = cam.light_pdf_weight;
            if (rnd<R>(g) < w) dir = lights_dir(P.lights, h.p, p.time, g);
            else dir = matpdf_generate(s.pdf, g);
            pdf = w * lights_pdf(P.lights, h.p, p.time, dir) + (R(1) - w) * matpdf_value(s.pdf, dir);
        } else {
            dir = matpdf_generate(s.pdf, g);
            pdf = matpdf_value(s.pdf, dir);
            suppress = cam.nee && cam.use_lights;
            weight_env = cam.nee && cam.use_env;
        }
        if (Num<R>::finite(pdf) && pdf > R(kEps)) {
            R sp = mat_scattering_pdf(m, p.d, h, dir);
            if (Num<R>::finite(sp) && sp > R(0)) {
                R next_w = R(1);
                if (weight_env) next_w = power_heuristic(pdf, env_pdf(P.env, dir));
                p.att = cmul(p.att, s.att * (sp / pdf));
                p.o = spawn_origin(h, dir);
                p.d = dir;
                p.allow_emit = !suppress;
                p.miss_w = next_w;
                cont = rr_survives(cam, p.bounce, p.att, g);
            }
        }
    }
    if (cont && p.bounce + 1 >= cam.max_depth) cont = false; // the bounce loop is exhausted
    if (cont) p.bounce += 1;
    return cont;
}

// Wavefront shade step for `slot`: one bounce, pending shadow queries stored for k_shadow.
template <class R, bool BATCH, bool OBJ = false>
GT_DEV bool shade_slot(const Params<R>& P, uint32_t slot, uint32_t key, bool& shadow, bool& done) {
    uint4 st = P.ps.st[slot];
    Rng g{uint64_t(st.x) | (uint64_t(st.y) << 32)};
    uint32_t flags = st.z;
    R4<R> ro = P.ps.ray_o[slot], rd = P.ps.ray_d[slot];
    Path<R> p;
    p.o = xyz(ro);
    p.d = xyz(rd);
    p.time = ro.w;
    p.miss_w = rd.w;
    p.att = xyz(P.ps.att[slot]);
    p.col = xyz(P.ps.col[slot]);
    p.bounce = flags & F_BOUNCE_MASK;
    p.allow_emit = (flags & F_ALLOW_EMIT) != 0;
    Shadow<R> sh;
    const int prim = key == KEY_MISS ? -1 : P.ps.hit_prim[slot];
    const R t = key == KEY_MISS ? R(0) : P.ps.hit_t[slot];
    uint32_t local;
    HitRec<R> oh;
    const HitRec<R>* ohp = nullptr;
    if constexpr (OBJ) {
        const int obj = key == KEY_MISS ? -1 : P.ps.hit_obj[slot];
        if (obj >= 0) {
            oh = make_mesh_hit(P.sc, obj, prim, p.o, p.d, p.time, t);
            ohp = &oh;
        }
    }
    const bool cont = integrate_bounce<R, false, OBJ>(P, cam_of<R, BATCH>(P, slot, local), p, prim, t, g, sh, ohp);
    uint32_t sh_bits = 0;
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        if (!sh.valid[k]) continue;
        const size_t j = size_t(slot) * 2 + k;
        P.ps.sh_o[j] = R4<R>{sh.o.x, sh.o.y, sh.o.z, sh.time};
        P.ps.sh_d[j] = R4<R>{sh.dir[k].x, sh.dir[k].y, sh.dir[k].z, R(k + 1)};
        P.ps.sh_a[j] = R4<R>{sh.att.x, sh.att.y, sh.att.z, sh.ratio[k]};
        P.ps.sh_s[j] = R4<R>{sh.s[k].x, sh.s[k].y, sh.s[k].z, R(0)};
        sh_bits |= k == 0 ? F_SHADOW0 : F_SHADOW1;
    }
    flags &= ~(F_BOUNCE_MASK | F_TRACE | F_SHADOW0 | F_SHADOW1 | F_ALLOW_EMIT);
    flags |= sh_bits | (p.allow_emit ? F_ALLOW_EMIT : 0u);
    if (cont) {
        flags |= F_TRACE | (p.bounce & F_BOUNCE_MASK);
        P.ps.ray_o[slot] = R4<R>{p.o.x, p.o.y, p.o.z, p.time};
        P.ps.ray_d[slot] = R4<R>{p.d.x, p.d.y, p.d.z, p.miss_w};
        P.ps.att[slot] = R4<R>{p.att.x, p.att.y, p.att.z, R(0)};
    } else if (P.sub && sh_bits == 0) { // substreams: the slot's one sample is complete
        const R4<R> o = R4<R>{p.col.x, p.col.y, p.col.z, R(1)};
        P.sub->out[slot] = o;
        flags = F_DONE;
        done = true;
    } else {
        flags |= F_NEWSAMPLE;
    }
    P.ps.col[slot] = R4<R>{p.col.x, p.col.y, p.col.z, R(0)};
    P.ps.st[slot] = make_uint4(uint32_t(g.s), uint32_t(g.s >> 32), flags, st.w);
    shadow = sh_bits != 0;
    return cont;
}

template <class R, bool BATCH = false, bool OBJ = false>
__global__ void __launch_bounds__(256, BATCH ? 2u : kShadeBlocksPerSm) k_shade(Params<R> P, uint32_t cur) {
    uint32_t prefix[NUM_KEYS + 1];
    prefix[0] = 0;
#pragma unroll
    for (uint32_t k = 0; k < NUM_KEYS; ++k)
        prefix[k + 1] = prefix[k] + *reinterpret_cast<volatile uint32_t*>(&P.ps.counters[C_MAT + k]);
    const uint32_t total = prefix[NUM_KEYS];
    const uint32_t warp0 = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = warp0; base < total; base += stride) {
        const uint32_t i = base + lane_id();
        bool cont = false, shadow = false, done = false;
        uint32_t slot = 0;
        if (i < total) {
            uint32_t key = 0;
#pragma unroll
            for (uint32_t k = 1; k < NUM_KEYS; ++k)
                if (i >= prefix[k]) key = k;
            slot = P.ps.q_mat[size_t(key) * P.ps.qcap + (i - prefix[key])];
            cont = shade_slot<R, BATCH, OBJ>(P, slot, key, shadow, done);
        }
        warp_push(cont, slot, P.ps.q_trace[cur ^ 1u], &P.ps.counters[C_TRACE0 + (cur ^ 1u)]);
        warp_push(shadow, slot, P.ps.q_shadow, &P.ps.counters[C_SHADOW]);
        const unsigned fin = __ballot_sync(0xffffffffu, done);
        if (fin && lane_id() == 0) atomicAdd(&P.ps.counters[C_DONE], uint32_t(__popc(fin)));
    }
}

// OBJ: a world with objects: the closest-hit query (k = 0) also tests the objects below
// the RayScene's hit, the occlusion query (k = 1) the objects when the RayScene is clear.
template <class R, bool OBJ = false>
__global__ void __launch_bounds__(256, kShadowBlocksPerSm) k_shadow(Params<R> P) {
    const uint32_t count = *reinterpret_cast<volatile uint32_t*>(&P.ps.counters[C_SHADOW]);
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&P.ps.totals[1], (unsigned long long)count);
    const R inf = Num<R>::inf();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const uint32_t slot = P.ps.q_shadow[i];
        uint4 st = P.ps.st[slot];
        V3<R> col = xyz(P.ps.col[slot]);
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            if (!(st.z & (k == 0 ? F_SHADOW0 : F_SHADOW1))) continue;
            const size_t j = size_t(slot) * 2 + k;
            R4<R> so = P.ps.sh_o[j], sd = P.ps.sh_d[j], sa = P.ps.sh_a[j], ss = P.ps.sh_s[j];
            Shadow<R> sh;
            sh.o = xyz(so);
            sh.time = so.w;
            sh.att = xyz(sa);
            sh.dir[k] = xyz(sd);
            sh.s[k] = xyz(ss);
            sh.ratio[k] = sa.w;
            R t = R(0);
            int prim = k == 0 ? traverse<R, false, false>(P.sc, sh.o, sh.dir[k], sh.time, R(kShadowAcne), inf, t,
                                                          nullptr, &P.ps.counters[C_ERROR])
                              : traverse<R, false, true>(P.sc, sh.o, sh.dir[k], sh.time, R(kShadowAcne), inf, t,
                                                         nullptr, &P.ps.counters[C_ERROR]);
            if constexpr (OBJ) {
                int obj = -1, leaf = -1;
                if (k == 0) {
                    if (prim < 0) t = inf;
                    objects_hit(P.sc, sh.o, sh.dir[k], sh.time, R(kShadowAcne), t, obj, leaf, &P.ps.counters[C_ERROR]);
                    if (obj >= 0) {
                        const HitRec<R> oh = make_mesh_hit(P.sc, obj, leaf, sh.o, sh.dir[k], sh.time, t);
                        apply_shadow(P, col, sh, k, leaf, t, &oh);
                        continue;
                    }
                } else if (prim < 0) {
                    R to = inf;
                    if (objects_hit(P.sc, sh.o, sh.dir[k], sh.time, R(kShadowAcne), to, obj, leaf,
                                    &P.ps.counters[C_ERROR]))
                        prim = leaf;
                }
            }
            apply_shadow(P, col, sh, k, prim, t);
        }
        P.ps.col[slot] = R4<R>{col.x, col.y, col.z, R(0)};
        P.ps.st[slot].z = st.z & ~(F_SHADOW0 | F_SHADOW1);
    }
}

// Progressive preview: the estimate of every finished pixel, 0 elsewhere.
template <class R> __global__ void k_preview(Params<R> P, float* rgb) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < P.ps.n; i += gridDim.x * blockDim.x) {
        V3<R> c{0, 0, 0};
        if (P.ps.st[i].z & F_DONE) {
            const uint32_t a = P.ps.accepted[i];
            const V3<R> s = xyz(P.ps.acc[i]);
            c = P.cam.adaptive ? s : (a == 0 ? V3<R>{0, 0, 0} : cdiv(s, R(a)));
        }
        rgb[size_t(i) * 3 + 0] = float(c.x);
        rgb[size_t(i) * 3 + 1] = float(c.y);
        rgb[size_t(i) * 3 + 2] = float(c.z);
    }
}

// Pixel estimate: sum / accepted (camera.rs:2993-2999) or the Welford mean.
template <class R, bool BATCH = false>
__global__ void k_resolve(Params<R> P, float* rgb, double* rgb64, uint32_t* accepted) {
    const uint32_t n = P.ps.n;
    const uint32_t warp0 = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = warp0; base < n; base += stride) {
        const uint32_t i = base + lane_id();
        unsigned long long va = 0, vs = 0;
        if (i < n) {
            const uint32_t a = P.ps.accepted[i];
            V3<R> s = xyz(P.ps.acc[i]);
            V3<R> c;
            uint32_t local;
            if (cam_of<R, BATCH>(P, i, local).adaptive) c = s;
            else c = a == 0 ? V3<R>{0, 0, 0} : cdiv(s, R(a));
            if (rgb) {
                rgb[size_t(i) * 3 + 0] = float(c.x);
                rgb[size_t(i) * 3 + 1] = float(c.y);
                rgb[size_t(i) * 3 + 2] = float(c.z);
            }
            if (rgb64) {
                rgb64[size_t(i) * 3 + 0] = double(c.x);
                rgb64[size_t(i) * 3 + 1] = double(c.y);
                rgb64[size_t(i) * 3 + 2] = double(c.z);
            }
            if (accepted) accepted[i] = a;
            va = a;
            vs = P.ps.st[i].w;
        }
        // Sample totals for throughput reporting (warp-reduced, one atomic per warp).
        for (int off = 16; off > 0; off >>= 1) {
            va += __shfl_down_sync(0xffffffffu, va, off);
            vs += __shfl_down_sync(0xffffffffu, vs, off);
        }
        if (lane_id() == 0) {
            atomicAdd(&P.ps.totals[2], va);
            atomicAdd(&P.ps.totals[3], vs);
        }
    }
}

// Pixel estimate from the running sums (camera.rs:2993-2999) or the Welford mean.
template <class R> GT_DEV V3<R> pixel_estimate(const CamDev<R>& cam, R4<R> a, uint32_t acc_n) {
    if (cam.adaptive) return xyz(a);
    return acc_n == 0 ? V3<R>{0, 0, 0} : cdiv(xyz(a), R(acc_n));
}

// Register form of finish_sample: folds one sample into the pixel's sums.
template <class R> GT_DEV bool fold_sample(const CamDev<R>& cam, R4<R>& a, R4<R>& c, uint32_t& acc_n, V3<R> s) {
    if (!finite3(s)) return false;
    acc_n += 1;
    if (cam.adaptive) {
        V3<R> mean = xyz(a), m2 = xyz(c);
        V3<R> delta = s - mean;
        mean = mean + cdiv(delta, R(acc_n));
        V3<R> delta2 = s - mean;
        m2 = m2 + cmul(delta, delta2);
        a = R4<R>{mean.x, mean.y, mean.z, R(0)};
        c = R4<R>{m2.x, m2.y, m2.z, R(0)};
        return acc_n >= cam.adaptive_min && adaptive_error(m2, acc_n) < cam.adaptive_threshold;
    }
    kahan_add(a, c, s);
    return false;
}

// Cost classes for the persistent schedule's pixel order.  A pixel's samples form one
// sequential chain, so the frame can finish no sooner than its longest chain; pixels whose
// centre ray sees glass (long specular paths, Russian roulette surviving at 0.95) start
// first, then metal, glossy, diffuse, and emitters or misses last.
enum : uint32_t { NUM_COST_CLASSES = 5 };
GT_DEV uint32_t cost_class(int prim_kind_or_miss) {
    switch (prim_kind_or_miss) {
    case 5: return 0; // Dielectric
    case 4: return 1; // Metal
    case 3: return 2; // GGX
    case 0:           // Lambertian
    case 2:           // Isotropic
    case 6: return 3; // HenyeyGreenstein
    default: return 4; // DiffuseLight or a miss
    }
}

template <class R> __global__ void __launch_bounds__(256) k_classify(Params<R> P, uint32_t* queues, uint32_t* counts) {
    const uint32_t n = P.cam.width * P.cam.height;
    const uint32_t warp0 = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u;
    const uint32_t stride = gridDim.x * blockDim.x;
    const R inf = Num<R>::inf();
    for (uint32_t base = warp0; base < n; base += stride) {
        const uint32_t pix = base + lane_id();
        uint32_t key = 0;
        if (pix < n) {
            const R x = R(pix % P.cam.width), y = R(pix / P.cam.width);
            V3<R> d = (load3(P.cam.p00_rel) + load3(P.cam.du) * x) + load3(P.cam.dv) * y;
            R t;
            const int prim = traverse<R, false, false>(P.sc, load3(P.cam.center), d, P.cam.shutter0, R(kShadowAcne), inf,
                                                       t, nullptr, &P.ps.counters[C_ERROR]);
            key = cost_class(prim < 0 ? -1 : P.sc.mats[__ldg(&P.sc.meta[prim].x) >> 3].kind);
        }
        warp_push_keyed(pix < n, key, pix, queues, n, counts);
    }
}

// Persistent schedule: the whole frame in one launch.  Each thread takes pixels in cost
// order from a device counter and runs that pixel's samples in order in registers (the
// pixel's stream is sequential, camera.rs:2669).  Every loop iteration traces exactly one
// ray through one traversal call site — the live path's next ray or one of its pending
// next-event shadow rays — so lanes on different samples, pixels or ray kinds stay on the
// same instructions.  `cancel` is polled at each pixel fetch; `progress` receives the
// number of pixels handed out.
//
// RESUME = true finishes a wavefront render instead: `queues` is a list of the slots that
// are still running (class_counts[0] entries), each thread picks up a slot's saved state
// (its path mid-flight, or a finished sample waiting to be folded in) and, when the
// slot's pixel is done, stores the pixel sums back for k_resolve.
// Hand-over of a resume-mode k_persistent launch to a cooperative one (one warp per slot)
// once few slots are left; all zero = never.  `coop` makes the launch itself cooperative.
// Both modes run the same compiled code, so a slot's arithmetic does not depend on which
// mode finishes it.
struct HandOff {
    uint32_t* done = nullptr;  // slots this launch has finished
    uint32_t below = 0;        // hand over once (slots - done) <= below
    uint32_t* list = nullptr;  // slots handed over
    uint32_t* count = nullptr; // their number
    uint32_t coop = 0;         // 1 = one slot per warp (RESUME launches only)
};

// WORLD: a world with objects or participating media: every ray goes through world_hit
// (whose media draw from the pixel's stream), and shadow queries are traced inside
// integrate_bounce.
// COOP: the cooperative instantiation (one slot per warp, RESUME only), whose warps may
// also intersect small scenes lane-parallel (warp_closest); kept apart so the one-slot-per-
// lane launches keep their register budget.
template <class R, bool RESUME, bool BATCH = false, bool WORLD = false, bool COOP = false>
__global__ void __launch_bounds__(128, sizeof(R) == 8 ? 1 : 4) k_persistent(Params<R> P, uint32_t* next, const uint32_t* queues,
                                                    const uint32_t* class_counts, const volatile uint32_t* cancel,
                                                    volatile uint32_t* progress, float* rgb, double* rgb64,
                                                    uint32_t* accepted, HandOff ho = HandOff()) {
    const uint32_t n = RESUME ? class_counts[0] : (BATCH ? P.frame_start[P.num_frames] : P.cam.width * P.cam.height);
    const bool coop = RESUME && (COOP || ho.coop != 0); // warp-uniform
    // The camera of the pixel being rendered: the frame's in a batch, else the launch's.
    uint32_t frame = 0, local = 0;
    auto cam = [&]() -> const CamDev<R>& {
        if constexpr (BATCH) return P.cams[frame];
        else return P.cam;
    };
    // Global pixel -> (frame, pixel within the frame) by binary search over frame_start.
    auto locate = [&](uint32_t pix) {
        if constexpr (BATCH) {
            uint32_t lo = 0, hi = P.num_frames;
            while (hi - lo > 1) {
                const uint32_t mid = (lo + hi) >> 1;
                if (P.frame_start[mid] <= pix) lo = mid;
                else hi = mid;
            }
            frame = lo;
            local = pix - P.frame_start[lo];
        } else {
            local = pix;
        }
    };
    auto sample_limit = [&]() -> uint32_t { return cam().adaptive ? cam().adaptive_max : cam().spp; };
    const R inf = Num<R>::inf();
    uint32_t prefix[NUM_COST_CLASSES + 1];
    prefix[0] = 0;
#pragma unroll
    for (uint32_t k = 0; k < NUM_COST_CLASSES; ++k) prefix[k + 1] = prefix[k] + (RESUME ? 0u : class_counts[k]);
    auto fetch = [&]() -> uint32_t {
        uint32_t i;
        if (coop) { // one slot per warp: lane 0 decides for every lane, which then follow one path
            uint32_t v = 0;
            if (lane_id() == 0) v = (cancel && *cancel) ? n : atomicAdd(next, 1u);
            i = __shfl_sync(0xffffffffu, v, 0);
        } else {
            if (cancel && *cancel) return n;
            i = atomicAdd(next, 1u);
        }
        if (i >= n) return n;
        if (progress && (i & 1023u) == 0) *progress = i;
        if (RESUME || BATCH) return i;
        uint32_t k = 0;
#pragma unroll
        for (uint32_t c = 1; c < NUM_COST_CLASSES; ++c)
            if (i >= prefix[c]) k = c;
        return queues[size_t(k) * n + (i - prefix[k])];
    };
    unsigned long long n_rays = 0, n_shadow = 0, n_acc = 0, n_started = 0;
    uint32_t item = fetch();
    uint32_t pix = RESUME ? (item < n ? queues[item] : 0u) : item;
    Rng g{0};
    R4<R> a{0, 0, 0, 0}, c{0, 0, 0, 0};
    uint32_t acc_n = 0, started = 0;
    Path<R> p;
    Shadow<R> sh;
    uint32_t pending = 0; // bit k: shadow query k still to trace
    bool cont = false;
    bool need_sample = true;
    bool fresh = false; // resumed from an accumulator: no finished sample to fold in
    // Loads a wavefront slot's saved state (RESUME).
    auto resume = [&](uint32_t slot) {
        const uint4 st = P.ps.st[slot];
        fresh = (st.z & F_FRESH) != 0;
        g.s = uint64_t(st.x) | (uint64_t(st.y) << 32);
        started = st.w;
        a = P.ps.acc[slot];
        c = P.ps.comp[slot];
        acc_n = P.ps.accepted[slot];
        p.col = xyz(P.ps.col[slot]);
        need_sample = (st.z & F_TRACE) == 0;
        if (!need_sample) {
            const R4<R> ro = P.ps.ray_o[slot], rd = P.ps.ray_d[slot];
            p.o = xyz(ro);
            p.time = ro.w;
            p.d = xyz(rd);
            p.miss_w = rd.w;
            p.att = xyz(P.ps.att[slot]);
            p.bounce = st.z & F_BOUNCE_MASK;
            p.allow_emit = (st.z & F_ALLOW_EMIT) != 0;
        }
        pending = 0;
        cont = !need_sample;
    };
    // Saves the slot's state in the wavefront layout resume() reads (RESUME hand-over); a
    // migrated slot stays marked so that the tail's k_collect leaves it to the side stream.
    auto save = [&](uint32_t slot) {
        uint32_t flags = (P.ps.st[slot].z & F_MIGRATED) | (fresh ? F_FRESH : 0u);
        if (!need_sample) {
            flags = F_TRACE | (p.bounce & F_BOUNCE_MASK) | (p.allow_emit ? F_ALLOW_EMIT : 0u);
            P.ps.ray_o[slot] = R4<R>{p.o.x, p.o.y, p.o.z, p.time};
            P.ps.ray_d[slot] = R4<R>{p.d.x, p.d.y, p.d.z, p.miss_w};
            P.ps.att[slot] = R4<R>{p.att.x, p.att.y, p.att.z, R(0)};
        }
        P.ps.col[slot] = R4<R>{p.col.x, p.col.y, p.col.z, R(0)};
        P.ps.acc[slot] = a;
        P.ps.comp[slot] = c;
        P.ps.accepted[slot] = acc_n;
        P.ps.st[slot] = make_uint4(uint32_t(g.s), uint32_t(g.s >> 32), flags, started);
    };
    if (item < n) {
        locate(pix);
        if (RESUME) resume(pix);
        else g.s = pixel_seed(cam().seed, local % cam().width, local / cam().width);
    }
    bool alive = item < n;
    // The loop is warp-uniform and reconverges at each phase boundary (__syncwarp), so
    // the warp executes setup, one traversal and one integration step together instead
    // of drifting apart into sub-warps at different instructions.
    uint32_t iter = 0;
    while (__any_sync(0xffffffffu, alive)) {
        if (RESUME && !coop) {
            // Hand-over: once no more slots are left than the cooperative launch has warps,
            // lanes between samples or bounces save their slot, list it (with every slot not
            // yet taken) and stop; a slot then runs on a warp of its own, where it is not
            // slowed by other lanes' branches.
            if (ho.below && (iter & 15u) == 0u && alive && pending == 0 &&
                n - *reinterpret_cast<volatile uint32_t*>(ho.done) <= ho.below) {
                save(pix);
                ho.list[atomicAdd(ho.count, 1u)] = pix;
                for (uint32_t it = fetch(); it < n; it = fetch()) ho.list[atomicAdd(ho.count, 1u)] = queues[it];
                alive = false;
            }
        }
        ++iter;
        if (alive && need_sample) {
            bool stop = false;
            if (started > 0 && !fresh) stop = fold_sample(cam(), a, c, acc_n, p.col);
            fresh = false;
            bool got = false;
            for (;;) {
                const uint32_t x = local % cam().width, y = local / cam().width;
                const uint32_t limit = sample_limit();
                while (!stop && started < limit) {
                    camera_ray(cam(), x, y, started, g, p.o, p.d, p.time);
                    ++started;
                    if (cam().max_depth == 0) { // the bounce loop never runs: a black sample
                        stop = fold_sample(cam(), a, c, acc_n, V3<R>{0, 0, 0});
                        continue;
                    }
                    p.att = V3<R>{1, 1, 1};
                    p.col = V3<R>{0, 0, 0};
                    p.miss_w = R(1);
                    p.bounce = 0;
                    p.allow_emit = true;
                    got = true;
                    break;
                }
                if (got) break;
                // The pixel is finished: write it (or hand its sums back to the
                // wavefront's resolve) and take the next one.
                if (RESUME) {
                    if (!coop || lane_id() == 0) {
                        P.ps.acc[pix] = a;
                        P.ps.comp[pix] = c;
                        P.ps.accepted[pix] = acc_n;
                        P.ps.st[pix] = make_uint4(uint32_t(g.s), uint32_t(g.s >> 32), F_DONE, started);
                        if (ho.done) atomicAdd(ho.done, 1u);
                    }
                } else {
                    const V3<R> v = pixel_estimate(cam(), a, acc_n);
                    if (rgb) {
                        rgb[size_t(pix) * 3 + 0] = float(v.x);
                        rgb[size_t(pix) * 3 + 1] = float(v.y);
                        rgb[size_t(pix) * 3 + 2] = float(v.z);
                    }
                    if (rgb64) {
                        rgb64[size_t(pix) * 3 + 0] = double(v.x);
                        rgb64[size_t(pix) * 3 + 1] = double(v.y);
                        rgb64[size_t(pix) * 3 + 2] = double(v.z);
                    }
                    if (accepted) accepted[pix] = acc_n;
                    n_acc += acc_n;
                    n_started += started;
                }
                item = fetch();
                if (item >= n) {
                    alive = false;
                    break;
                }
                if (RESUME) {
                    pix = queues[item];
                    locate(pix);
                    resume(pix);
                    if (!need_sample) break; // a path in flight: trace it
                    stop = false;
                    got = false;
                    // a finished sample: fold it in before starting the next one
                    if (started > 0 && !fresh) stop = fold_sample(cam(), a, c, acc_n, p.col);
                    fresh = false;
                    continue;
                }
                pix = item;
                locate(pix);
                g.s = pixel_seed(cam().seed, local % cam().width, local / cam().width);
                a = R4<R>{0, 0, 0, 0};
                c = R4<R>{0, 0, 0, 0};
                acc_n = 0;
                started = 0;
                stop = false;
            }
            need_sample = false;
        }
        __syncwarp();
        // One traversal per iteration: a pending shadow query first (area, then
        // environment, in the reference's order), otherwise the path's next ray.
        const int which = (pending & 1u) ? 0 : ((pending & 2u) ? 1 : -1);
        R t = R(0);
        int prim = -1;
        HitRec<R> wrec;
        if (alive) {
            const V3<R> ro = which >= 0 ? sh.o : p.o;
            const V3<R> rd = which >= 0 ? sh.dir[which] : p.d;
            const R rt = which >= 0 ? sh.time : p.time;
            if constexpr (WORLD) { // no query is ever pending here
                prim = world_hit(P.sc, ro, rd, rt, R(kShadowAcne), g, wrec, &P.ps.counters[C_ERROR]) ? 0 : -1;
            } else if (COOP && sizeof(R) == 4 && P.sc.num_prims <= 32u) { // warp-uniform
                prim = warp_closest(P.sc, ro, rd, rt, R(kShadowAcne), inf, t);
            } else {
                prim = traverse<R, false, false>(P.sc, ro, rd, rt, R(kShadowAcne), inf, t, nullptr,
                                                 &P.ps.counters[C_ERROR], which == 1);
            }
        }
        __syncwarp();
        if (alive) {
            if (which >= 0) {
                apply_shadow(P, p.col, sh, which, prim, t);
                pending &= ~(1u << which);
                ++n_shadow;
            } else {
                ++n_rays;
                cont = integrate_bounce<R, WORLD>(P, cam(), p, prim, t, g, sh, &wrec);
                pending = (sh.valid[0] ? 1u : 0u) | (sh.valid[1] ? 2u : 0u);
                if constexpr (WORLD) n_shadow += sh.traced;
            }
            if (pending == 0 && !cont) need_sample = true;
        }
        __syncwarp();
    }
    // Throughput totals: warp-reduce, one atomic per warp (every lane of the launch's
    // full warps arrives here); a cooperative warp counted its one path in every lane.
    __syncwarp();
    for (int off = 16; off > 0 && !coop; off >>= 1) {
        n_rays += __shfl_down_sync(0xffffffffu, n_rays, off);
        n_shadow += __shfl_down_sync(0xffffffffu, n_shadow, off);
        n_acc += __shfl_down_sync(0xffffffffu, n_acc, off);
        n_started += __shfl_down_sync(0xffffffffu, n_started, off);
    }
    if (lane_id() == 0) {
        atomicAdd(&P.ps.totals[0], n_rays);
        atomicAdd(&P.ps.totals[1], n_shadow);
        atomicAdd(&P.ps.totals[2], n_acc);
        atomicAdd(&P.ps.totals[3], n_started);
        atomicAdd(&P.ps.totals[6], n_rays + n_shadow);
    }
}

// Resumable accumulation: slots start from an accumulator's streams and sums ...
template <class R>
__global__ void k_accum_load(Params<R> P, const uint64_t* rng, const R4<R>* sum, const R4<R>* comp,
                             const uint32_t* accepted, uint32_t started) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < P.ps.n; i += gridDim.x * blockDim.x) {
        const uint64_t s = rng[i];
        P.ps.st[i] = make_uint4(uint32_t(s), uint32_t(s >> 32), F_NEWSAMPLE | F_FRESH, started);
        P.ps.acc[i] = sum[i];
        P.ps.comp[i] = comp[i];
        P.ps.accepted[i] = accepted[i];
    }
}

// ... and hand them back when the frame is done.
template <class R>
__global__ void k_accum_store(Params<R> P, uint64_t* rng, R4<R>* sum, R4<R>* comp, uint32_t* accepted) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < P.ps.n; i += gridDim.x * blockDim.x) {
        const uint4 st = P.ps.st[i];
        rng[i] = uint64_t(st.x) | (uint64_t(st.y) << 32);
        sum[i] = P.ps.acc[i];
        comp[i] = P.ps.comp[i];
        accepted[i] = P.ps.accepted[i];
    }
}

// Every slot in order, and their number (a RESUME pass over the whole image).
static __global__ void k_list_all(uint32_t* list, uint32_t n, uint32_t* count) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) list[i] = i;
    if (blockIdx.x == 0 && threadIdx.x == 0) *count = n;
}

// Lists the wavefront slots that have not finished their pixel (for the RESUME pass).
template <class R> __global__ void __launch_bounds__(256) k_collect(Params<R> P, uint32_t* list, uint32_t* count) {
    const uint32_t n = P.ps.local_n;
    const uint32_t warp0 = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = warp0; base < n; base += stride) {
        const uint32_t j = base + lane_id();
        const uint32_t slot = j < n ? stripe_slot(P.ps, j) : 0u;
        const bool live = j < n && (P.ps.st[slot].z & (F_DONE | F_MIGRATED)) == 0;
        warp_push(live, slot, list, count);
    }
}

// Throughput mode (gt_render_opts.rng = GT_RNG_SUBSTREAMS; no reference counterpart).
// Sample s of pixel (x, y) draws from its own SplitMix64 stream, started at
// pixel_seed(seed, x, y) ^ sample_key(s), instead of continuing the pixel's one stream:
// statistically the reference's estimator, not its stream.  Samples are then independent,
// so every (pixel, sample) pair of a round is a work item and no pixel's samples form a
// chain.  k_substream traces a round's items; k_sub_fold adds each pixel's samples in
// sample order (Kahan sums, or Welford with the adaptive stop exactly where the reference
// would stop), so the image does not depend on the order in which items ran.
GT_DEV uint64_t sample_key(uint64_t s) {
    uint64_t z = (s + 1) * 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

// Items a lane claims at a time (one atomicAdd per claim).
constexpr uint32_t kSubClaim = 16;

// Round `first` .. first + S - 1 of the `count` pixels in `list`: item i is sample
// first + i / count of pixel list[i % count] (sample-major, so neighbouring lanes trace
// neighbouring pixels).  Its radiance goes to out[i] with w = 1, or w = 0 where the sample
// lies beyond the pixel's sample limit.  Each loop turn traces one ray per lane: a pending
// shadow query first, as k_persistent does, then the path's next ray.
template <class R, bool BATCH>
__global__ void __launch_bounds__(128, sizeof(R) == 8 ? 1 : 5)
    k_substream(Params<R> P, const uint32_t* list, uint32_t count, uint32_t first, uint32_t S, R4<R>* out,
                unsigned long long* next) {
    const unsigned long long items = (unsigned long long)count * S;
    const R inf = Num<R>::inf();
    unsigned long long item = 0, end = 0;
    unsigned long long n_rays = 0, n_shadow = 0;
    Path<R> p;
    Shadow<R> sh;
    Rng g{0};
    uint32_t pending = 0, pix = 0, frame = 0;
    bool cont = false; // the path has a next ray (once its pending shadow queries are traced)
    size_t slot_out = 0;
    // The camera of the item's pixel: its frame's in a batch, else the render's.
    auto cam = [&]() -> const CamDev<R>& {
        if constexpr (BATCH) return P.cams[frame];
        else return P.cam;
    };
    // Sets up the lane's next item that is a sample; false once the items are used up.
    auto start = [&]() -> bool {
        for (;;) {
            if (item == end) {
                item = atomicAdd(next, (unsigned long long)kSubClaim);
                if (item >= items) return false;
                end = item + kSubClaim < items ? item + kSubClaim : items;
            }
            const uint32_t j = uint32_t(item / count), k = uint32_t(item % count);
            slot_out = size_t(item);
            ++item;
            pix = list[k];
            uint32_t local = pix;
            if constexpr (BATCH) { // frame by binary search over the frame offsets
                uint32_t lo = 0, hi = P.num_frames;
                while (hi - lo > 1) {
                    const uint32_t mid = (lo + hi) >> 1;
                    if (__ldg(&P.frame_start[mid]) <= pix) lo = mid;
                    else hi = mid;
                }
                frame = lo;
                local = pix - __ldg(&P.frame_start[lo]);
            }
            const CamDev<R>& C = cam();
            const uint32_t s = first + j;
            if (s >= (C.adaptive ? C.adaptive_max : C.spp)) {
                out[slot_out] = R4<R>{0, 0, 0, 0};
                continue;
            }
            const uint32_t x = local % C.width, y = local / C.width;
            g.s = pixel_seed(C.seed, x, y) ^ sample_key(s);
            camera_ray(C, x, y, s, g, p.o, p.d, p.time);
            if (C.max_depth == 0) { // the bounce loop never runs: a black sample
                out[slot_out] = R4<R>{0, 0, 0, 1};
                continue;
            }
            p.att = V3<R>{1, 1, 1};
            p.col = V3<R>{0, 0, 0};
            p.miss_w = R(1);
            p.bounce = 0;
            p.allow_emit = true;
            pending = 0;
            cont = true;
            return true;
        }
    };
    bool alive = start();
    while (__any_sync(0xffffffffu, alive)) {
        const int which = (pending & 1u) ? 0 : ((pending & 2u) ? 1 : -1);
        R t = R(0);
        int prim = -1;
        if (alive) {
            const V3<R> ro = which >= 0 ? sh.o : p.o;
            const V3<R> rd = which >= 0 ? sh.dir[which] : p.d;
            const R rt = which >= 0 ? sh.time : p.time;
            prim = traverse<R, false, false>(P.sc, ro, rd, rt, R(kShadowAcne), inf, t, nullptr,
                                             &P.ps.counters[C_ERROR], which == 1);
        }
        __syncwarp();
        if (alive) {
            if (which >= 0) {
                apply_shadow(P, p.col, sh, which, prim, t);
                pending &= ~(1u << which);
                ++n_shadow;
            } else {
                HitRec<R> wrec;
                ++n_rays;
                cont = integrate_bounce<R, false>(P, cam(), p, prim, t, g, sh, &wrec);
                pending = (sh.valid[0] ? 1u : 0u) | (sh.valid[1] ? 2u : 0u);
            }
            if (pending == 0 && !cont) {
                out[slot_out] = R4<R>{p.col.x, p.col.y, p.col.z, R(1)};
                alive = start();
            }
        }
        __syncwarp();
    }
    for (int off = 16; off > 0; off >>= 1) {
        n_rays += __shfl_down_sync(0xffffffffu, n_rays, off);
        n_shadow += __shfl_down_sync(0xffffffffu, n_shadow, off);
    }
    if (lane_id() == 0) {
        atomicAdd(&P.ps.totals[0], n_rays);
        atomicAdd(&P.ps.totals[1], n_shadow);
        atomicAdd(&P.ps.totals[6], n_rays + n_shadow);
    }
}

// Folds round first .. first + S - 1 into each listed pixel's sums in sample order; pixels
// that neither stopped (adaptive) nor reached their sample limit go to next_list.
template <class R, bool BATCH>
__global__ void __launch_bounds__(256) k_sub_fold(Params<R> P, const uint32_t* list, uint32_t count, uint32_t first,
                                                  uint32_t S, const R4<R>* out, uint32_t* next_list,
                                                  uint32_t* next_count) {
    const uint32_t warp0 = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = warp0; base < count; base += stride) {
        const uint32_t k = base + lane_id();
        bool more = false;
        uint32_t pix = 0;
        if (k < count) {
            pix = list[k];
            uint32_t local;
            const CamDev<R>& C = cam_of<R, BATCH>(P, pix, local);
            const uint32_t limit = C.adaptive ? C.adaptive_max : C.spp;
            R4<R> a = P.ps.acc[pix], c = P.ps.comp[pix];
            uint32_t acc_n = P.ps.accepted[pix], started = P.ps.st[pix].w;
            bool stop = false;
            for (uint32_t j = 0; j < S && first + j < limit && !stop; ++j) {
                const R4<R> v = out[size_t(j) * count + k];
                started = first + j + 1;
                stop = fold_sample(C, a, c, acc_n, xyz(v));
            }
            P.ps.acc[pix] = a;
            P.ps.comp[pix] = c;
            P.ps.accepted[pix] = acc_n;
            P.ps.st[pix].w = started;
            more = !stop && started < limit;
        }
        warp_push(more, pix, next_list, next_count);
    }
}

// Progress image of the throughput mode (one frame): every pixel's estimate from the
// samples folded so far.
template <class R> __global__ void __launch_bounds__(256) k_sub_preview(Params<R> P, float* rgb) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < P.ps.n; i += gridDim.x * blockDim.x) {
        const V3<R> c = pixel_estimate(P.cam, P.ps.acc[i], P.ps.accepted[i]);
        rgb[size_t(i) * 3 + 0] = float(c.x);
        rgb[size_t(i) * 3 + 1] = float(c.y);
        rgb[size_t(i) * 3 + 2] = float(c.z);
    }
}

// Round set-up of the throughput mode on the wavefront: slot i gets its sample's own
// stream, or is done at once (w = 0 in out) when the sample lies beyond the pixel's limit.
template <class R> __global__ void __launch_bounds__(256) k_sub_init(Params<R> P) {
    const SubRound<R> sr = *P.sub;
    const uint32_t n = P.ps.local_n;
    const uint32_t warp0 = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = warp0; base < n; base += stride) {
        const uint32_t j = base + lane_id();
        const uint32_t slot = j < n ? stripe_slot(P.ps, j) : 0u;
        bool done = false;
        if (j < n) {
            const uint32_t pix = sr.list[slot % sr.count], s = sr.first + slot / sr.count;
            const CamDev<R>& C = P.cam;
            if (s >= (C.adaptive ? C.adaptive_max : C.spp)) {
                sr.out[slot] = R4<R>{0, 0, 0, 0};
                P.ps.st[slot] = make_uint4(0u, 0u, F_DONE, 0u);
                done = true;
            } else {
                const uint64_t seed = pixel_seed(C.seed, pix % C.width, pix / C.width) ^ sample_key(s);
                P.ps.st[slot] = make_uint4(uint32_t(seed), uint32_t(seed >> 32), F_NEWSAMPLE, 0u);
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, done);
        if (m && lane_id() == 0) atomicAdd(&P.ps.counters[C_DONE], uint32_t(__popc(m)));
    }
}

// Slow-slot migration.  A wavefront slot advances one bounce per iteration, so a frame
// lasts as long as its longest per-pixel sample chain (pixels behind glass run several
// times the median number of bounces).  Early in the frame the slots whose sample rate
// is far below the mean move to a persistent kernel on a second stream, which runs them
// concurrently with the wavefront at one bounce per loop instead of one per iteration.
//
// Pass 1: samples started by unfinished slots, and their number, into mstat[0], [1].
template <class R> __global__ void __launch_bounds__(256) k_progress_sum(Params<R> P) {
    const uint32_t n = P.ps.local_n;
    unsigned long long s = 0, c = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint4 st = P.ps.st[stripe_slot(P.ps, i)];
        if ((st.z & (F_DONE | F_MIGRATED)) == 0) {
            s += st.w;
            c += 1;
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        s += __shfl_down_sync(0xffffffffu, s, off);
        c += __shfl_down_sync(0xffffffffu, c, off);
    }
    if (lane_id() == 0 && c) {
        atomicAdd(&P.ps.mstat[0], s);
        atomicAdd(&P.ps.mstat[1], c);
    }
}

// Pass 2: marks every unfinished slot with started * ratio < mean started as migrated,
// lists it in q_migrate and counts it as done for the wavefront's termination test.
// A migrated slot keeps its path state; clearing F_NEWSAMPLE keeps k_generate away.
template <class R> __global__ void __launch_bounds__(256) k_migrate(Params<R> P, float ratio) {
    const uint32_t n = P.ps.local_n;
    const double sum = double(P.ps.mstat[0]), live = double(P.ps.mstat[1]);
    const uint32_t warp0 = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = warp0; base < n; base += stride) {
        const uint32_t j = base + lane_id();
        const uint32_t slot = j < n ? stripe_slot(P.ps, j) : 0u;
        bool mig = false;
        if (j < n && live > 0.0) {
            uint4 st = P.ps.st[slot];
            mig = (st.z & (F_DONE | F_MIGRATED)) == 0 && double(st.w) * double(ratio) * live < sum;
            if (mig) {
                st.z = (st.z & ~F_NEWSAMPLE) | F_MIGRATED;
                P.ps.st[slot] = st;
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, mig);
        if (m && lane_id() == 0) atomicAdd(&P.ps.counters[C_DONE], uint32_t(__popc(m)));
        warp_push(mig, slot, P.ps.q_migrate, &P.ps.counters[C_MIGRATED]);
    }
}

// Pass 3: the trace queue the next iteration starts from, q_trace[0], without migrated
// slots: survivors go to q_trace[1] (its counter zeroed before) ...
template <class R> __global__ void __launch_bounds__(256) k_drop_migrated(Params<R> P) {
    const uint32_t count = P.ps.counters[C_TRACE0];
    const uint32_t warp0 = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = warp0; base < count; base += stride) {
        const uint32_t i = base + lane_id();
        uint32_t slot = 0;
        bool keep = false;
        if (i < count) {
            slot = P.ps.q_trace[0][i];
            keep = (P.ps.st[slot].z & F_MIGRATED) == 0;
        }
        warp_push(keep, slot, P.ps.q_trace[1], &P.ps.counters[C_TRACE1]);
    }
}

// ... and are copied back.
template <class R> __global__ void __launch_bounds__(256) k_restore_queue(Params<R> P) {
    const uint32_t count = P.ps.counters[C_TRACE1];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
        P.ps.q_trace[0][i] = P.ps.q_trace[1][i];
    if (blockIdx.x == 0 && threadIdx.x == 0) P.ps.counters[C_TRACE0] = count;
}

// Denoising AOVs (camera.rs:3064-3116): first-hit albedo and 0.5 (n + 1), same per-pixel
// stream as the beauty pass, divided by the sample count.
template <class R> __global__ void k_aov(Params<R> P, float* albedo, float* normal) {
    const uint32_t n = P.cam.width * P.cam.height;
    const R inf = Num<R>::inf();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t x = i % P.cam.width, y = i / P.cam.width;
        Rng g{pixel_seed(P.cam.seed, x, y)};
        V3<R> sa{0, 0, 0}, sn{0, 0, 0};
        for (uint32_t k = 0; k < P.cam.spp; ++k) {
            V3<R> o, d;
            R time, t;
            camera_ray(P.cam, x, y, k, g, o, d, time);
            HitRec<R> h;
            if (P.sc.num_media || P.sc.num_objects) { // media draw from the same stream (camera.rs:3104-3106)
                if (!world_hit(P.sc, o, d, time, R(kShadowAcne), g, h, &P.ps.counters[C_ERROR])) continue;
            } else {
                const int prim = traverse<R, false, false>(P.sc, o, d, time, R(kShadowAcne), inf, t, nullptr,
                                                           &P.ps.counters[C_ERROR]);
                if (prim < 0) continue; // black on a miss
                h = make_hit(P.sc, uint32_t(prim), o, d, time, t);
            }
            sa = sa + mat_albedo(P.sc.mats[h.mat], h);
            sn = sn + (h.ns + V3<R>{1, 1, 1}) * R(0.5); // the shading normal (camera.rs:3112-3114)
        }
        sa = cdiv(sa, R(P.cam.spp));
        sn = cdiv(sn, R(P.cam.spp));
        if (albedo) {
            albedo[size_t(i) * 3 + 0] = float(sa.x);
            albedo[size_t(i) * 3 + 1] = float(sa.y);
            albedo[size_t(i) * 3 + 2] = float(sa.z);
        }
        if (normal) {
            normal[size_t(i) * 3 + 0] = float(sn.x);
            normal[size_t(i) * 3 + 1] = float(sn.y);
            normal[size_t(i) * 3 + 2] = float(sn.z);
        }
    }
}

// Closest-hit queries with BvhTraversalStats (bvh.rs:9-52, 306-399); rays are
// {origin xyz, direction xyz, time} in f64.  stats: [0..5) sums, [5] max stack depth.
template <class R>
__global__ void k_trace_rays(SceneDev<R> sc, const double* rays, uint32_t count, double tmin, double tmax,
                             int32_t* ids, double* tout, unsigned long long* stats, uint32_t* err) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const double* r = rays + size_t(i) * 7;
        V3<R> o{R(r[0]), R(r[1]), R(r[2])}, d{R(r[3]), R(r[4]), R(r[5])};
        TraceStats st{0, 0, 0, 0, 0, 0};
        R t = R(0);
        int prim = traverse<R, true, false>(sc, o, d, R(r[6]), R(tmin), R(tmax), t, &st, err);
        ids[i] = prim < 0 ? -1 : int32_t(__ldg(&sc.meta[prim].y));
        if (tout) tout[i] = prim < 0 ? 0.0 : double(t);
        atomicAdd(&stats[0], st.node_tests);
        atomicAdd(&stats[1], st.node_hits);
        atomicAdd(&stats[2], st.leaf_visits);
        atomicAdd(&stats[3], st.candidates);
        atomicAdd(&stats[4], st.leaf_hits);
        atomicMax(&stats[5], (unsigned long long)st.max_depth);
    }
}

// The f32 primary-hit check: each ray through the f32 rendering walk (the wide tree where
// the scene has one) in its check mode, which returns the rendering walk's closest hit
// and flags rays whose decision f32 rounding may have changed (near ties, near edges,
// near t_min) for an f64 re-trace.
template <class R>
__global__ void k_trace_rays_check(SceneDev<R> sc, const double* rays, uint32_t count, double tmin, double tmax,
                                   int32_t* ids, double* tout, uint8_t* near_out, uint32_t* err) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const double* r = rays + size_t(i) * 7;
        const V3<R> o{R(r[0]), R(r[1]), R(r[2])}, d{R(r[3]), R(r[4]), R(r[5])};
        R t = R(0);
        CheckState<R> ck{false, R(0)};
        const int prim = traverse<R, false, false, true>(sc, o, d, R(r[6]), R(tmin), R(tmax), t, nullptr, err, false,
                                                         &ck);
        ids[i] = prim < 0 ? -1 : int32_t(__ldg(&sc.meta[prim].y));
        tout[i] = prim < 0 ? 0.0 : double(t);
        near_out[i] = ck.near ? 1 : 0;
    }
}

} // namespace gt
