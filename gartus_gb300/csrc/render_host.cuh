// render_host.cuh — per-precision host orchestration: scene/light/environment upload,
// the wavefront loop (captured as a CUDA graph of two iterations and replayed until every
// pixel slot has finished), resolve, AOVs, and the statistics trace.  Included by exactly
// one translation unit per precision.
#pragma once

#include <time.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "internal.h"
#include "scene_tables.h"
#include "wavefront.cuh"

namespace gt {

#define GT_CUDA(call)                                                   \
    do {                                                                \
        cudaError_t e_ = (call);                                        \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);             \
    } while (0)

template <class R> inline void put3(R* dst, const double* src) {
    dst[0] = R(src[0]);
    dst[1] = R(src[1]);
    dst[2] = R(src[2]);
}

// f32 child boxes are rounded outward so the f32 slab test never culls a primitive the
// f64 box contains; f64 boxes are the reference's exactly.
template <class R> inline R round_down(double v);
template <class R> inline R round_up(double v);
template <> inline double round_down<double>(double v) { return v; }
template <> inline double round_up<double>(double v) { return v; }
template <> inline float round_down<float>(double v) {
    float f = float(v);
    return double(f) > v ? std::nextafter(f, -INFINITY) : f;
}
template <> inline float round_up<float>(double v) {
    float f = float(v);
    return double(f) < v ? std::nextafter(f, INFINITY) : f;
}

template <class R> inline void put_box(R* dst, const Aabb& b) {
    for (int i = 0; i < 3; ++i) {
        dst[i] = round_down<R>(b.lo[i]);
        dst[3 + i] = round_up<R>(b.hi[i]);
    }
}

template <class R> GpuScene<R>& gpu_of(gt_scene* s);
template <> inline GpuScene<float>& gpu_of<float>(gt_scene* s) { return s->f32; }
template <> inline GpuScene<double>& gpu_of<double>(gt_scene* s) { return s->f64; }
template <class R> GpuLights<R>& lights_of(gt_lights* l);
template <> inline GpuLights<float>& lights_of<float>(gt_lights* l) { return l->f32; }
template <> inline GpuLights<double>& lights_of<double>(gt_lights* l) { return l->f64; }
template <class R> GpuEnv<R>& env_of(gt_environment* e);
template <> inline GpuEnv<float>& env_of<float>(gt_environment* e) { return e->f32; }
template <> inline GpuEnv<double>& env_of<double>(gt_environment* e) { return e->f64; }

template <class R> void free_gpu(gt_scene* s) {
    GpuScene<R>& g = gpu_of<R>(s);
    cudaFree(g.prims);
    cudaFree(g.meta);
    cudaFree(g.nodes);
    cudaFree(g.wnodes);
    cudaFree(g.mats);
    cudaFree(g.perlin);
    cudaFree(g.texels);
    cudaFree(g.images);
    cudaFree(g.media);
    cudaFree(g.meshes);
    cudaFree(g.objects);
    cudaFree(g.tlas);
    for (void* p : g.mesh_allocs) cudaFree(p);
    cudaFree(g.parent_leaf);
    cudaFree(g.parent_int);
    cudaFree(g.arrivals);
    cudaFree(g.int_box);
    cudaFree(g.leaf_box);
    cudaFree(g.leaf_of);
    g = GpuScene<R>();
}

// One primitive's PrimRec (layout.h) from its gt_geometry, derived quantities in f64:
// returns its kind (K_NEVER for the degenerate quads and triangles every query rejects,
// geometry.rs:394-397, object.rs:192-203) or kBadKind for an unknown geometry kind.
constexpr uint32_t kBadKind = 0xFFFFFFFFu;
template <class R> uint32_t pack_prim(const gt_geometry& g, R* v) {
    const double* q = g.p;
    std::fill(v, v + 16, R(0));
    uint32_t kind = g.kind;
    switch (g.kind) {
    case GT_GEOM_SPHERE:
        put3(v, q);
        v[3] = R(std::fmax(q[3], 0.0));
        break;
    case GT_GEOM_MOVING_SPHERE: {
        put3(v, q);
        v[3] = R(std::fmax(q[6], 0.0));
        double dl[3] = {q[3] - q[0], q[4] - q[1], q[5] - q[2]};
        put3(v + 4, dl);
        break;
    }
    case GT_GEOM_TRIANGLE: {
        double e1[3] = {q[3] - q[0], q[4] - q[1], q[5] - q[2]};
        double e2[3] = {q[6] - q[0], q[7] - q[1], q[8] - q[2]};
        double c[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        double len = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
        double nrm[3] = {0, 0, 0};
        if (!(len < 2.220446049250313e-16))
            for (int k = 0; k < 3; ++k) nrm[k] = c[k] / len;
        put3(v, q);
        put3(v + 4, e1);
        put3(v + 8, e2);
        put3(v + 12, nrm);
        if (nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2] <= 2.220446049250313e-16) kind = K_NEVER;
        break;
    }
    case GT_GEOM_QUAD: {
        const double* u = q + 3;
        const double* w = q + 6;
        double c[3] = {u[1] * w[2] - u[2] * w[1], u[2] * w[0] - u[0] * w[2], u[0] * w[1] - u[1] * w[0]};
        double l2 = c[0] * c[0] + c[1] * c[1] + c[2] * c[2];
        double len = std::sqrt(l2);
        double nrm[3] = {0, 0, 0};
        if (!(len < 2.220446049250313e-16))
            for (int k = 0; k < 3; ++k) nrm[k] = c[k] / len;
        double pd = nrm[0] * q[0] + nrm[1] * q[1] + nrm[2] * q[2];
        double ww[3] = {0, 0, 0};
        if (!(l2 <= 2.220446049250313e-16))
            for (int k = 0; k < 3; ++k) ww[k] = c[k] / l2;
        put3(v, q);
        v[3] = R(pd);
        put3(v + 4, u);
        v[7] = R(nrm[0]);
        put3(v + 8, w);
        v[11] = R(nrm[1]);
        put3(v + 12, ww);
        v[15] = R(nrm[2]);
        if (l2 <= 2.220446049250313e-16) kind = K_NEVER; // area_squared() <= EPS
        if (nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2] <= 2.220446049250313e-16) kind = K_NEVER;
        break;
    }
    default:
        return kBadKind;
    }
    return kind;
}

// A medium's boundary as primitives: its sphere, or box_object's six quads in their order
// (object.rs:930-976: corners sorted per axis, sides spanned by dx, dy, dz and their
// negations).  Returns the count.
inline uint32_t medium_parts(const gt_medium& m, gt_geometry* out) {
    std::memset(out, 0, 6 * sizeof(gt_geometry));
    if (m.shape == GT_MEDIUM_SPHERE) {
        out[0].kind = GT_GEOM_SPHERE;
        for (int a = 0; a < 4; ++a) out[0].p[a] = m.p[a];
        return 1;
    }
    const double mn[3] = {std::fmin(m.p[0], m.p[3]), std::fmin(m.p[1], m.p[4]), std::fmin(m.p[2], m.p[5])};
    const double mx[3] = {std::fmax(m.p[0], m.p[3]), std::fmax(m.p[1], m.p[4]), std::fmax(m.p[2], m.p[5])};
    const double dx[3] = {mx[0] - mn[0], 0.0, 0.0}, dy[3] = {0.0, mx[1] - mn[1], 0.0}, dz[3] = {0.0, 0.0, mx[2] - mn[2]};
    const double ndx[3] = {-dx[0], -dx[1], -dx[2]}, ndz[3] = {-dz[0], -dz[1], -dz[2]};
    const double q[6][3] = {{mn[0], mn[1], mx[2]}, {mx[0], mn[1], mx[2]}, {mx[0], mn[1], mn[2]},
                            {mn[0], mn[1], mn[2]}, {mn[0], mx[1], mx[2]}, {mn[0], mn[1], mn[2]}};
    const double* u[6] = {dx, ndz, ndx, dz, dx, dx};
    const double* v[6] = {dy, dy, dy, dy, ndz, dz};
    for (int i = 0; i < 6; ++i) {
        out[i].kind = GT_GEOM_QUAD;
        for (int a = 0; a < 3; ++a) {
            out[i].p[a] = q[i][a];
            out[i].p[3 + a] = u[i][a];
            out[i].p[6 + a] = v[i][a];
        }
    }
    return 6;
}

// A reference-layout tree as device nodes: internal nodes renumbered densely in pre-order,
// leaf children as links (~first, count); also the root's box and link (a root box no ray
// enters for an empty tree).  `slot_of` maps leaf slots to the device primitive order when
// that order is the wide tree's (each leaf's primitives stay consecutive and in order).
template <class R>
void flatten_tree(const BuiltBvh& bvh, std::vector<Node<R>>& nodes, R* root_box, int32_t& root_link,
                  int32_t& root_count, const std::vector<uint32_t>* slot_of = nullptr) {
    std::vector<int32_t> internal_id(bvh.nodes.size(), -1);
    int32_t ni = 0;
    for (size_t i = 0; i < bvh.nodes.size(); ++i)
        if (!bvh.nodes[i].leaf) internal_id[i] = ni++;
    nodes.assign(size_t(ni), Node<R>());
    auto link_of = [&](uint32_t child, int32_t& link, int32_t& count) {
        const BuildNode& c = bvh.nodes[child];
        link = c.leaf ? ~int32_t(slot_of ? (*slot_of)[c.first] : c.first) : internal_id[child];
        count = c.leaf ? int32_t(c.count) : 0;
    };
    for (size_t i = 0; i < bvh.nodes.size(); ++i) {
        const BuildNode& b = bvh.nodes[i];
        if (b.leaf) continue;
        Node<R>& nd = nodes[size_t(internal_id[i])];
        put_box<R>(nd.box, bvh.nodes[b.left].box);
        put_box<R>(nd.box + 6, bvh.nodes[b.right].box);
        link_of(b.left, nd.link[0], nd.link[1]);
        link_of(b.right, nd.link[2], nd.link[3]);
    }
    if (bvh.nodes.empty()) {
        for (int k = 0; k < 3; ++k) {
            root_box[k] = R(1);
            root_box[3 + k] = R(-1);
        }
        root_link = ~0;
        root_count = 0;
    } else {
        put_box<R>(root_box, bvh.nodes[0].box);
        link_of(0, root_link, root_count);
    }
}

// transform_point (raytracing/instance.rs:355-364): the homogeneous product, divided by w
// when |w| > EPSILON.
inline void xf_point_host(const double* m, const double* p, double* out) {
    double r[4];
    for (int i = 0; i < 4; ++i) r[i] = m[4 * i] * p[0] + m[4 * i + 1] * p[1] + m[4 * i + 2] * p[2] + m[4 * i + 3] * 1.0;
    const bool div = std::fabs(r[3]) > 2.220446049250313e-16;
    for (int i = 0; i < 3; ++i) out[i] = div ? r[i] / r[3] : r[i];
}

// Meshes (their primitives in their own tree's leaf order, attributes alongside) and world
// objects (in the leaf order of a tree over their world boxes: the mesh's box, through
// the instance transform's eight corners as transform_bounds does, instance.rs:319-335).
// In f32 a mesh's tree is collapsed to the eight-wide form as the RayScene's is (its
// primitives then in the wide tree's leaf order), unless the scene asks for binary trees.
template <class R> gt_status upload_meshes(gt_scene* s, GpuScene<R>& g, cudaStream_t st) {
    SceneDev<R>& v = g.view;
    v.num_objects = 0;
    if (s->objects.empty()) return GT_OK;
    auto dput = [&](const void* src, size_t bytes, void** dst) -> gt_status {
        *dst = nullptr;
        if (bytes == 0) return GT_OK;
        GT_CUDA(cudaMalloc(dst, bytes));
        g.mesh_allocs.push_back(*dst);
        GT_CUDA(cudaMemcpyAsync(*dst, src, bytes, cudaMemcpyHostToDevice, st));
        return GT_OK;
    };
    std::vector<MeshDev<R>> md(s->meshes.size());
    // Host staging stays alive until the copies finish (synchronised below).
    std::vector<std::vector<PrimRec<R>>> keep_rec(md.size());
    std::vector<std::vector<uint2>> keep_meta(md.size());
    std::vector<std::vector<Node<R>>> keep_nodes(md.size());
    std::vector<std::vector<R>> keep_uv(md.size()), keep_vn(md.size());
    std::vector<std::vector<uint8_t>> keep_attr(md.size());
    std::vector<WideBvh> keep_wide(md.size());
    gt_status rc;
    for (size_t k = 0; k < md.size(); ++k) {
        const MeshHost& mh = s->meshes[k];
        const size_t mn = mh.prims.size();
        auto& rec = keep_rec[k];
        auto& meta = keep_meta[k];
        auto& uv = keep_uv[k];
        auto& vn = keep_vn[k];
        auto& attr = keep_attr[k];
        rec.resize(mn);
        meta.resize(mn);
        attr.resize(mn);
        if (!mh.uv.empty()) uv.resize(mn * 6);
        if (!mh.vn.empty()) vn.resize(mn * 9);
        WideBvh& wide = keep_wide[k];
        const bool use_wide = sizeof(R) == 4 && s->f32_tree == GT_F32_TREE_WIDE && build_wide_bvh(mh.bvh, wide);
        std::vector<uint32_t> slot_of;
        if (use_wide) {
            slot_of.resize(mn);
            for (size_t j = 0; j < mn; ++j) slot_of[wide.order[j]] = uint32_t(j);
        }
        for (size_t j = 0; j < mn; ++j) {
            const uint32_t pi = mh.bvh.order[use_wide ? wide.order[j] : j];
            const gt_primitive& p = mh.prims[pi];
            const uint32_t kind = pack_prim<R>(p.geometry, rec[j].v);
            if (kind == kBadKind) return fail(GT_ERR_INVALID_ARG, "unknown geometry kind");
            meta[j] = make_uint2(kind | (p.material << 3), pi);
            attr[j] = mh.attr[pi];
            for (int a = 0; a < 6 && !uv.empty(); ++a) uv[j * 6 + a] = R(mh.uv[size_t(pi) * 6 + a]);
            for (int a = 0; a < 9 && !vn.empty(); ++a) vn[j * 9 + a] = R(mh.vn[size_t(pi) * 9 + a]);
        }
        SceneDev<R> mv;
        std::memset(&mv, 0, sizeof(mv));
        flatten_tree<R>(mh.bvh, keep_nodes[k], mv.root_box, mv.root_link, mv.root_count, use_wide ? &slot_of : nullptr);
        void *dp, *dm, *dn, *du, *dv, *da, *dw = nullptr;
        if ((rc = dput(rec.data(), mn * sizeof(PrimRec<R>), &dp)) != GT_OK) return rc;
        if ((rc = dput(meta.data(), mn * sizeof(uint2), &dm)) != GT_OK) return rc;
        if ((rc = dput(keep_nodes[k].data(), keep_nodes[k].size() * sizeof(Node<R>), &dn)) != GT_OK) return rc;
        if ((rc = dput(uv.data(), uv.size() * sizeof(R), &du)) != GT_OK) return rc;
        if ((rc = dput(vn.data(), vn.size() * sizeof(R), &dv)) != GT_OK) return rc;
        if ((rc = dput(attr.data(), attr.size(), &da)) != GT_OK) return rc;
        if (use_wide && (rc = dput(wide.nodes.data(), wide.nodes.size() * sizeof(WideNode), &dw)) != GT_OK) return rc;
        mv.wnodes = static_cast<const WideNode*>(dw);
        mv.prims = static_cast<const PrimRec<R>*>(dp);
        mv.meta = static_cast<const uint2*>(dm);
        mv.nodes = static_cast<const Node<R>*>(dn);
        mv.mats = g.mats;
        mv.num_prims = uint32_t(mn);
        mv.num_nodes = uint32_t(keep_nodes[k].size());
        md[k] = MeshDev<R>{mv, static_cast<const R*>(du), static_cast<const R*>(dv), static_cast<const uint8_t*>(da)};
    }
    const size_t no = s->objects.size();
    std::vector<Aabb> boxes(no);
    for (size_t k = 0; k < no; ++k) {
        const gt_object& o = s->objects[k];
        const BuiltBvh& mb = s->meshes[o.mesh].bvh;
        Aabb b = mb.nodes.empty() ? Aabb{{0, 0, 0}, {0, 0, 0}} : mb.nodes[0].box;
        if (o.transformed && !mb.nodes.empty()) {
            Aabb t{{1e300, 1e300, 1e300}, {-1e300, -1e300, -1e300}};
            for (int c = 0; c < 8; ++c) {
                const double p[3] = {(c & 1) ? b.hi[0] : b.lo[0], (c & 2) ? b.hi[1] : b.lo[1], (c & 4) ? b.hi[2] : b.lo[2]};
                double q[3];
                xf_point_host(o.transform, p, q);
                for (int a = 0; a < 3; ++a) {
                    t.lo[a] = std::fmin(t.lo[a], q[a]);
                    t.hi[a] = std::fmax(t.hi[a], q[a]);
                }
            }
            b = t;
        }
        boxes[k] = b;
    }
    BuiltBvh tl;
    build_bvh_from_boxes(boxes.data(), uint32_t(no), 2, tl);
    if (tl.max_depth + 1 > 30) return fail(GT_ERR_UNSUPPORTED, "object tree deeper than the device traversal stack");
    std::vector<ObjectDev<R>> od(no);
    for (size_t j = 0; j < no; ++j) {
        const gt_object& o = s->objects[tl.order[j]];
        std::memset(&od[j], 0, sizeof(od[j]));
        od[j].mesh = o.mesh;
        od[j].transformed = o.transformed;
        for (int a = 0; a < 16; ++a) {
            od[j].xf[a] = R(o.transform[a]);
            od[j].inv[a] = R(o.inverse[a]);
        }
    }
    std::vector<Node<R>> tnodes;
    flatten_tree<R>(tl, tnodes, v.tlas_box, v.tlas_link, v.tlas_count);
    GT_CUDA(cudaMalloc(&g.meshes, std::max<size_t>(md.size(), 1) * sizeof(MeshDev<R>)));
    GT_CUDA(cudaMalloc(&g.objects, no * sizeof(ObjectDev<R>)));
    GT_CUDA(cudaMalloc(&g.tlas, std::max<size_t>(tnodes.size(), 1) * sizeof(Node<R>)));
    if (!md.empty())
        GT_CUDA(cudaMemcpyAsync(g.meshes, md.data(), md.size() * sizeof(MeshDev<R>), cudaMemcpyHostToDevice, st));
    GT_CUDA(cudaMemcpyAsync(g.objects, od.data(), no * sizeof(ObjectDev<R>), cudaMemcpyHostToDevice, st));
    if (!tnodes.empty())
        GT_CUDA(cudaMemcpyAsync(g.tlas, tnodes.data(), tnodes.size() * sizeof(Node<R>), cudaMemcpyHostToDevice, st));
    GT_CUDA(cudaStreamSynchronize(st));
    v.meshes = g.meshes;
    v.objects = g.objects;
    v.tlas = g.tlas;
    v.num_objects = uint32_t(no);
    return GT_OK;
}

// Flattens the primitives into leaf order with derived quantities computed in f64
// (QuadGeometry::new, geometry.rs:271-301; TriangleGeometry::geometric_normal 171-179).
template <class R> gt_status upload_scene(gt_scene* s) {
    GpuScene<R>& g = gpu_of<R>(s);
    if (g.ready) return GT_OK;
    // The f32 path of a GT_BVH_GPU_LBVH scene builds its tree on the device from the
    // primitives in their given order; everything else uses the reference's SAH tree.
    const bool gpu_bvh = sizeof(R) == 4 && s->bvh_builder == GT_BVH_GPU_LBVH;
    if (!gpu_bvh) {
        const gt_status rc = ensure_reference_bvh(s);
        if (rc != GT_OK) return rc;
    }
    const BuiltBvh& bvh = s->bvh;
    const size_t n = s->prims.size();
    // The f32 path of a reference-SAH scene traverses the eight-wide tree collapsed from it;
    // its primitives then lie in the wide tree's leaf order (the binary tree's leaves keep
    // their primitives consecutive in that order, so both trees index one array).
    WideBvh wide;
    const bool use_wide =
        sizeof(R) == 4 && !gpu_bvh && s->f32_tree == GT_F32_TREE_WIDE && build_wide_bvh(bvh, wide);
    std::vector<uint32_t> slot_of;
    if (use_wide) {
        slot_of.resize(n);
        for (size_t j = 0; j < n; ++j) slot_of[wide.order[j]] = uint32_t(j);
    }
    std::vector<PrimRec<R>> recs(n);
    std::vector<uint2> meta(n);
    std::vector<float> boxes(gpu_bvh ? n * 6 : 0); // f32 bounds, rounded outward
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};   // bounds of the box centres
    if (gpu_bvh) {
        for (int a = 0; a < 3; ++a) {
            lo[a] = 1e300;
            hi[a] = -1e300;
        }
        for (size_t j = 0; j < n; ++j) {
            const Aabb b = geometry_aabb(s->prims[j].geometry);
            put_box<float>(boxes.data() + j * 6, b);
            for (int a = 0; a < 3; ++a) {
                const double c = 0.5 * (b.lo[a] + b.hi[a]);
                lo[a] = std::fmin(lo[a], c);
                hi[a] = std::fmax(hi[a], c);
            }
        }
    }
    for (size_t j = 0; j < n; ++j) {
        const uint32_t pi = gpu_bvh ? uint32_t(j) : bvh.order[use_wide ? wide.order[j] : j];
        const gt_primitive& p = s->prims[pi];
        const uint32_t kind = pack_prim<R>(p.geometry, recs[j].v);
        if (kind == kBadKind) return fail(GT_ERR_INVALID_ARG, "unknown geometry kind");
        meta[j] = make_uint2(kind | (p.material << 3), pi);
    }
    // Internal nodes, renumbered densely in pre-order; leaf children become links.
    std::vector<Node<R>> nodes;
    R root_box[6];
    int32_t root_link = ~0, root_count = 0;
    if (!gpu_bvh) flatten_tree<R>(bvh, nodes, root_box, root_link, root_count, use_wide ? &slot_of : nullptr);
    std::vector<MatDev<R>> mats(s->mats.size());
    std::vector<PerlinDev<R>> perlin;
    std::vector<size_t> perlin_of; // material index of each table set
    for (size_t i = 0; i < s->mats.size(); ++i) {
        const gt_material& m = s->mats[i];
        MatDev<R>& d = mats[i];
        std::memset(&d, 0, sizeof(d));
        d.kind = int32_t(m.kind);
        d.tex = int32_t(m.texture_kind);
        put3(d.color, m.color);
        d.param = R(m.param);
        if (m.kind == GT_MAT_GGX || m.kind == GT_MAT_METAL) // material.rs:1386, 1972
            d.param = R(std::fmin(std::fmax(m.param, 0.0), 1.0));
        if (m.texture_kind == GT_TEX_CHECKER) { // CheckerTexture::new, raytracing/texture.rs:71-82
            double sc = m.tex[0];
            d.inv_scale = R((std::isfinite(sc) && std::fabs(sc) > 2.220446049250313e-16) ? 1.0 / std::fabs(sc) : 1.0);
            put3(d.even, m.tex + 1);
            put3(d.odd, m.tex + 4);
        }
        if (m.texture_kind == GT_TEX_NOISE) { // NoiseTexture (graphics/raytracing/texture.rs:293-322)
            d.inv_scale = R(m.tex[0]);
            d.noise_variant = int32_t(m.tex[1]);
            d.noise_depth = int32_t(m.tex[2]);
            PerlinTables t;
            make_perlin_tables(uint64_t(m.tex[3]) | (uint64_t(m.tex[4]) << 32), t);
            PerlinDev<R> pd;
            for (int k = 0; k < 256; ++k) {
                pd.gx[k] = R(t.grad[k][0]);
                pd.gy[k] = R(t.grad[k][1]);
                pd.gz[k] = R(t.grad[k][2]);
            }
            std::memcpy(pd.perm, t.perm, sizeof(pd.perm));
            perlin.push_back(pd);
            perlin_of.push_back(i);
        }
    }
    free_gpu<R>(s);
    if (!perlin.empty()) {
        GT_CUDA(cudaMalloc(&g.perlin, perlin.size() * sizeof(PerlinDev<R>)));
        for (size_t k = 0; k < perlin.size(); ++k) mats[perlin_of[k]].noise = g.perlin + k;
    }
    std::vector<ImageDev> idev(s->images.size());
    if (!s->images.empty()) { // the bitmaps back to back, one descriptor each
        size_t total = 0;
        for (const ImageHost& im : s->images) total += im.rgb.size();
        GT_CUDA(cudaMalloc(&g.texels, std::max<size_t>(total, 16)));
        GT_CUDA(cudaMalloc(&g.images, idev.size() * sizeof(ImageDev)));
        size_t off = 0;
        for (size_t k = 0; k < idev.size(); ++k) {
            const ImageHost& im = s->images[k];
            idev[k] = ImageDev{g.texels + off, im.w, im.h, im.filter, im.wrap_s, im.wrap_t, 0u};
            off += im.rgb.size();
        }
        for (size_t i = 0; i < s->mats.size(); ++i) {
            const gt_material& m = s->mats[i];
            if (m.texture_kind == GT_TEX_IMAGE) mats[i].image = g.images + size_t(m.tex[0]);
            if (m.normal_map) { // NormalMap::with_strength clamps at 0 (raytracing/texture.rs:198-202)
                mats[i].normal_map = g.images + size_t(m.normal_map - 1);
                mats[i].normal_strength = R(std::fmax(m.normal_map_strength, 0.0));
                mats[i].normal_neg_y = (m.normal_map_flags & GT_NORMAL_MAP_NEGATIVE_Y) ? 1 : 0;
            }
        }
    }
    // Media: boundary shapes in PrimRec layout, the RotateY sine and cosine of
    // degrees_to_radians (raytracing.rs:150-152) and -1/density (medium.rs:97-101), in f64.
    std::vector<MediumDev<R>> mdev(s->media.size());
    for (size_t k = 0; k < mdev.size(); ++k) {
        const gt_medium& gm = s->media[k];
        MediumDev<R>& M = mdev[k];
        std::memset(&M, 0, sizeof(M));
        M.mat = gm.material;
        M.transform = gm.transform;
        M.neg_inv_density = R(-1.0 / gm.density);
        const double rad = gm.rotate_y * 3.141592653589793 / 180.0;
        M.sin_t = R(std::sin(rad));
        M.cos_t = R(std::cos(rad));
        for (int a = 0; a < 3; ++a) M.off[a] = R(gm.translate[a]);
        gt_geometry parts[6];
        M.parts = medium_parts(gm, parts);
        for (uint32_t i = 0; i < M.parts; ++i) M.kind[i] = pack_prim<R>(parts[i], M.part[i].v);
    }
    if (!mdev.empty()) GT_CUDA(cudaMalloc(&g.media, mdev.size() * sizeof(MediumDev<R>)));
    GT_CUDA(cudaMalloc(&g.prims, std::max<size_t>(n, 1) * sizeof(PrimRec<R>)));
    GT_CUDA(cudaMalloc(&g.meta, std::max<size_t>(n, 1) * sizeof(uint2)));
    GT_CUDA(cudaMalloc(&g.nodes, std::max<size_t>(nodes.size(), 1) * sizeof(Node<R>)));
    GT_CUDA(cudaMalloc(&g.mats, std::max<size_t>(mats.size(), 1) * sizeof(MatDev<R>)));
    if (use_wide) GT_CUDA(cudaMalloc(&g.wnodes, wide.nodes.size() * sizeof(WideNode)));
    cudaStream_t st = s->ctx->stream;
    if (n) {
        GT_CUDA(cudaMemcpyAsync(g.prims, recs.data(), n * sizeof(PrimRec<R>), cudaMemcpyHostToDevice, st));
        GT_CUDA(cudaMemcpyAsync(g.meta, meta.data(), n * sizeof(uint2), cudaMemcpyHostToDevice, st));
    }
    if (!nodes.empty())
        GT_CUDA(cudaMemcpyAsync(g.nodes, nodes.data(), nodes.size() * sizeof(Node<R>), cudaMemcpyHostToDevice, st));
    if (use_wide)
        GT_CUDA(cudaMemcpyAsync(g.wnodes, wide.nodes.data(), wide.nodes.size() * sizeof(WideNode),
                                cudaMemcpyHostToDevice, st));
    if (!mats.empty())
        GT_CUDA(cudaMemcpyAsync(g.mats, mats.data(), mats.size() * sizeof(MatDev<R>), cudaMemcpyHostToDevice, st));
    if (!perlin.empty())
        GT_CUDA(cudaMemcpyAsync(g.perlin, perlin.data(), perlin.size() * sizeof(PerlinDev<R>), cudaMemcpyHostToDevice,
                                st));
    for (size_t k = 0; k < idev.size(); ++k)
        if (!s->images[k].rgb.empty())
            GT_CUDA(cudaMemcpyAsync(const_cast<uint8_t*>(idev[k].rgb), s->images[k].rgb.data(), s->images[k].rgb.size(),
                                    cudaMemcpyHostToDevice, st));
    if (!idev.empty())
        GT_CUDA(cudaMemcpyAsync(g.images, idev.data(), idev.size() * sizeof(ImageDev), cudaMemcpyHostToDevice, st));
    if (!mdev.empty())
        GT_CUDA(cudaMemcpyAsync(g.media, mdev.data(), mdev.size() * sizeof(MediumDev<R>), cudaMemcpyHostToDevice, st));
    GT_CUDA(cudaStreamSynchronize(st));
    SceneDev<R>& v = g.view;
    v.prims = g.prims;
    v.meta = g.meta;
    v.nodes = g.nodes;
    v.mats = g.mats;
    v.media = g.media;
    v.num_media = uint32_t(mdev.size());
    v.num_prims = uint32_t(n);
    v.num_nodes = uint32_t(nodes.size());
    v.wnodes = use_wide ? g.wnodes : nullptr;
    g.wide_depth = use_wide ? wide.depth : 0u;
    g.wide_nodes = use_wide ? uint32_t(wide.nodes.size()) : 0u;
    if (gpu_bvh && n > 0) {
        cudaFree(g.nodes); // the device builder allocates its own node array
        g.nodes = nullptr;
        v.nodes = nullptr;
        const int sms = s->ctx->num_sms > 0 ? s->ctx->num_sms : 1;
        if constexpr (sizeof(R) == 4) {
            const gt_status rc = build_lbvh_f32(g, uint32_t(n), boxes.data(), lo, hi, st, sms);
            if (rc != GT_OK) return rc;
        }
    } else if (!gpu_bvh && !bvh.nodes.empty()) {
        for (int a = 0; a < 6; ++a) v.root_box[a] = root_box[a];
        v.root_link = root_link;
        v.root_count = root_count;
    } else { // an empty scene: a root box that no ray can enter
        for (int k = 0; k < 3; ++k) {
            v.root_box[k] = R(1);
            v.root_box[3 + k] = R(-1);
        }
        v.root_link = ~0;
        v.root_count = 0;
    }
    const gt_status mrc = upload_meshes<R>(s, g, st);
    if (mrc != GT_OK) return mrc;
    g.ready = true;
    return GT_OK;
}

template <class R> gt_status upload_lights(gt_lights* l) {
    GpuLights<R>& g = lights_of<R>(l);
    if (g.ready) return GT_OK;
    std::vector<LightDev<R>> t(l->targets.size());
    for (size_t i = 0; i < t.size(); ++i) {
        const gt_geometry& geo = l->targets[i].geometry;
        const double* q = geo.p;
        LightDev<R>& d = t[i];
        std::memset(&d, 0, sizeof(d));
        d.kind = int32_t(geo.kind);
        d.weight = R(l->targets[i].weight);
        switch (geo.kind) {
        case GT_GEOM_SPHERE:
            put3(d.a, q);
            d.radius = R(std::fmax(q[3], 0.0));
            break;
        case GT_GEOM_MOVING_SPHERE: {
            put3(d.a, q);
            double dl[3] = {q[3] - q[0], q[4] - q[1], q[5] - q[2]};
            put3(d.b, dl);
            d.radius = R(std::fmax(q[6], 0.0));
            break;
        }
        case GT_GEOM_QUAD: {
            const double* u = q + 3;
            const double* w = q + 6;
            double c[3] = {u[1] * w[2] - u[2] * w[1], u[2] * w[0] - u[0] * w[2], u[0] * w[1] - u[1] * w[0]};
            double l2 = c[0] * c[0] + c[1] * c[1] + c[2] * c[2];
            double len = std::sqrt(l2);
            double nrm[3] = {0, 0, 0}, ww[3] = {0, 0, 0};
            if (!(len < 2.220446049250313e-16))
                for (int k = 0; k < 3; ++k) nrm[k] = c[k] / len;
            if (!(l2 <= 2.220446049250313e-16))
                for (int k = 0; k < 3; ++k) ww[k] = c[k] / l2;
            put3(d.a, q);
            put3(d.b, u);
            put3(d.c, w);
            put3(d.n, nrm);
            put3(d.w, ww);
            d.plane_d = R(nrm[0] * q[0] + nrm[1] * q[1] + nrm[2] * q[2]);
            d.area_sq = R(l2);
            d.area = R(std::sqrt(l2));
            break;
        }
        case GT_GEOM_TRIANGLE: {
            double e1[3] = {q[3] - q[0], q[4] - q[1], q[5] - q[2]};
            double e2[3] = {q[6] - q[0], q[7] - q[1], q[8] - q[2]};
            double c[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
            double l2 = c[0] * c[0] + c[1] * c[1] + c[2] * c[2];
            double len = std::sqrt(l2);
            double nrm[3] = {0, 0, 0};
            if (!(len < 2.220446049250313e-16))
                for (int k = 0; k < 3; ++k) nrm[k] = c[k] / len;
            put3(d.a, q);
            put3(d.b, q + 3);
            put3(d.c, q + 6);
            put3(d.n, nrm);
            d.area = R(0.5 * std::sqrt(l2));
            break;
        }
        default:
            return fail(GT_ERR_INVALID_ARG, "unknown light geometry kind");
        }
    }
    cudaFree(g.t);
    g.t = nullptr;
    GT_CUDA(cudaMalloc(&g.t, std::max<size_t>(t.size(), 1) * sizeof(LightDev<R>)));
    if (!t.empty())
        GT_CUDA(cudaMemcpyAsync(g.t, t.data(), t.size() * sizeof(LightDev<R>), cudaMemcpyHostToDevice, l->ctx->stream));
    GT_CUDA(cudaStreamSynchronize(l->ctx->stream));
    g.view.t = g.t;
    g.view.count = uint32_t(t.size());
    g.view.total = R(l->total);
    g.ready = true;
    return GT_OK;
}

template <class R> gt_status upload_env(gt_environment* e) {
    GpuEnv<R>& g = env_of<R>(e);
    if (g.ready) return GT_OK;
    const size_t n = e->weights.size();
    std::vector<R> w(n), c(n);
    for (size_t i = 0; i < n; ++i) {
        w[i] = R(e->weights[i]);
        c[i] = R(e->cdf[i]);
    }
    cudaFree(g.weights);
    cudaFree(g.cdf);
    g.weights = g.cdf = nullptr;
    GT_CUDA(cudaMalloc(&g.weights, std::max<size_t>(n, 1) * sizeof(R)));
    GT_CUDA(cudaMalloc(&g.cdf, std::max<size_t>(n, 1) * sizeof(R)));
    if (n) {
        GT_CUDA(cudaMemcpyAsync(g.weights, w.data(), n * sizeof(R), cudaMemcpyHostToDevice, e->ctx->stream));
        GT_CUDA(cudaMemcpyAsync(g.cdf, c.data(), n * sizeof(R), cudaMemcpyHostToDevice, e->ctx->stream));
    }
    GT_CUDA(cudaStreamSynchronize(e->ctx->stream));
    g.view.format = int32_t(e->format);
    g.view.width = e->width;
    g.view.height = e->height;
    g.view.px8 = e->d_px8;
    g.view.px32 = e->d_px32;
    g.view.weights = g.weights;
    g.view.cdf = g.cdf;
    g.view.total = R(e->total);
    g.ready = true;
    return GT_OK;
}

template <class R> CamDev<R> cam_dev(const CamHost& h, bool use_lights, bool use_env) {
    CamDev<R> c;
    std::memset(&c, 0, sizeof(c));
    put3(c.center, h.center);
    put3(c.pixel00, h.pixel00);
    put3(c.du, h.du);
    put3(c.dv, h.dv);
    put3(c.ddu, h.ddu);
    put3(c.ddv, h.ddv);
    double rel[3] = {h.pixel00[0] - h.center[0], h.pixel00[1] - h.center[1], h.pixel00[2] - h.center[2]};
    put3(c.p00_rel, rel);
    const gt_camera_desc& d = h.desc;
    c.shutter0 = R(d.shutter_start);
    c.shutter1 = R(d.shutter_end);
    c.light_pdf_weight = R(h.light_pdf_weight);
    c.adaptive_threshold = R(d.adaptive_error_threshold);
    for (int i = 0; i < 9; ++i) c.bg[i] = R(d.background[i]);
    c.seed = d.rng_seed;
    c.width = h.width;
    c.height = h.height;
    c.spp = h.spp;
    c.mode = d.pixel_sample_mode;
    c.grid = h.grid;
    c.adaptive = (d.adaptive && d.pixel_sample_mode == GT_SAMPLE_RANDOM) ? 1u : 0u;
    c.adaptive_min = std::max<uint32_t>(d.adaptive_min_samples, 1u);
    c.adaptive_max = std::max<uint32_t>(d.adaptive_max_samples, c.adaptive_min);
    c.max_depth = d.max_depth;
    c.rr_min_depth = d.russian_roulette_min_depth;
    c.defocus = d.defocus_angle <= 0.0 ? 0u : 1u;
    c.bg_kind = d.background_kind;
    c.nee = h.nee ? 1u : 0u;
    c.use_lights = use_lights ? 1u : 0u;
    c.use_env = use_env ? 1u : 0u;
    return c;
}

// Bump allocator over the context workspace.
struct Bump {
    char* base;
    size_t off = 0;
    template <class T> T* take(size_t count) {
        off = (off + 255) & ~size_t(255);
        T* p = reinterpret_cast<T*>(base ? base + off : nullptr);
        off += count * sizeof(T);
        return p;
    }
};

// Per-slot path state, shared by every stripe (slot = pixel index).
template <class R> void layout_slots(Bump& b, PathState<R>& ps, uint32_t n, bool nee, bool objects = false) {
    ps.n = n;
    ps.ray_o = b.take<R4<R>>(n);
    ps.ray_d = b.take<R4<R>>(n);
    ps.att = b.take<R4<R>>(n);
    ps.col = b.take<R4<R>>(n);
    ps.st = b.take<uint4>(n);
    ps.hit_t = b.take<R>(n);
    ps.hit_prim = b.take<int32_t>(n);
    ps.hit_obj = objects ? b.take<int32_t>(n) : nullptr;
    ps.acc = b.take<R4<R>>(n);
    ps.comp = b.take<R4<R>>(n);
    ps.accepted = b.take<uint32_t>(n);
    const size_t ns = nee ? size_t(n) * 2 : 2;
    ps.sh_o = b.take<R4<R>>(ns);
    ps.sh_d = b.take<R4<R>>(ns);
    ps.sh_a = b.take<R4<R>>(ns);
    ps.sh_s = b.take<R4<R>>(ns);
    ps.totals = b.take<unsigned long long>(8);
    ps.stripe = 0;
    ps.stripes = 1;
    ps.row = 0;
    ps.local_n = n;
}

// One stripe's queues and counters, `cap` entries per queue.
template <class R> void layout_queues(Bump& b, PathState<R>& ps, uint32_t cap, bool nee) {
    ps.qcap = cap;
    ps.q_trace[0] = b.take<uint32_t>(cap);
    ps.q_trace[1] = b.take<uint32_t>(cap);
    ps.q_mat = b.take<uint32_t>(size_t(cap) * NUM_KEYS);
    ps.q_shadow = b.take<uint32_t>(nee ? cap : 1);
    ps.q_migrate = b.take<uint32_t>(cap);
    ps.q_handoff = b.take<uint32_t>(cap);
    ps.counters = b.take<uint32_t>(C_COUNT);
    ps.mstat = b.take<unsigned long long>(2);
}

inline gt_status ensure_workspace(gt_context* ctx, size_t bytes) {
    if (ctx->ws_bytes >= bytes) return GT_OK;
    if (ctx->ws) {
        cudaStreamSynchronize(ctx->stream);
        cudaStreamSynchronize(ctx->side);
        for (int k = 0; k < gt_context::kMaxStripes; ++k) {
            cudaStreamSynchronize(ctx->stripe_stream[k]);
            cudaStreamSynchronize(ctx->stripe_side[k]);
        }
        cudaFree(ctx->ws);
        ctx->ws = nullptr;
        ctx->ws_bytes = 0;
    }
    cudaError_t e = cudaMalloc(&ctx->ws, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(GT_ERR_OOM, "cannot allocate the render workspace");
    }
    ctx->ws_bytes = bytes;
    return GT_OK;
}

// CUDA events for whole-render timing and, in profile mode, per-kernel timing.
struct EventPool {
    cudaEvent_t begin = nullptr, end = nullptr;
    struct Rec {
        int kernel;
        cudaEvent_t a, z;
    };
    std::vector<cudaEvent_t> free_events;
    std::vector<Rec> pending;
    gt_status init() {
        if (cudaEventCreate(&begin) != cudaSuccess || cudaEventCreate(&end) != cudaSuccess)
            return fail(GT_ERR_CUDA, "cudaEventCreate");
        return GT_OK;
    }
    cudaError_t get(cudaEvent_t& e) {
        if (!free_events.empty()) {
            e = free_events.back();
            free_events.pop_back();
            return cudaSuccess;
        }
        return cudaEventCreate(&e);
    }
    cudaError_t pair(cudaEvent_t& a, cudaEvent_t& z) {
        cudaError_t r = get(a);
        return r == cudaSuccess ? get(z) : r;
    }
    void note(int kernel, cudaEvent_t a, cudaEvent_t z) { pending.push_back(Rec{kernel, a, z}); }
    // Call after a stream synchronize: folds finished pairs into the per-kernel times.
    void harvest(double* ms) {
        for (const Rec& r : pending) {
            float t = 0.f;
            if (cudaEventElapsedTime(&t, r.a, r.z) == cudaSuccess) ms[r.kernel] += t;
            free_events.push_back(r.a);
            free_events.push_back(r.z);
        }
        pending.clear();
    }
    ~EventPool() {
        for (const Rec& r : pending) {
            free_events.push_back(r.a);
            free_events.push_back(r.z);
        }
        for (cudaEvent_t e : free_events) cudaEventDestroy(e);
        if (begin) cudaEventDestroy(begin);
        if (end) cudaEventDestroy(end);
    }
};

// Persistent schedule: one launch sized to fill every SM; with a progress callback the
// host polls the mapped pixel counter while the kernel runs and can raise the cancel word.
template <class R>
gt_status run_persistent(gt_context* ctx, Params<R>& P, uint32_t* d_next, float* o_rgb, double* o_rgb64,
                         uint32_t* o_acc, const gt_render_opts& opts, EventPool& ev, double* kms, uint64_t* klaunch) {
    cudaStream_t st = ctx->stream;
    const uint32_t n = P.ps.n;
    GT_CUDA(cudaMemsetAsync(P.ps.counters, 0, C_COUNT * sizeof(uint32_t), st));
    GT_CUDA(cudaMemsetAsync(P.ps.totals, 0, 8 * sizeof(unsigned long long), st));
    GT_CUDA(cudaMemsetAsync(d_next, 0, sizeof(uint32_t), st));
    // Cost-ordered pixel queues (the C_MAT counters hold the class sizes).
    const uint32_t sms0 = uint32_t(ctx->num_sms > 0 ? ctx->num_sms : 1);
    const uint32_t cblocks = std::max<uint32_t>(1u, std::min<uint32_t>((n + 255) / 256, sms0 * 8));
    k_classify<R><<<cblocks, 256, 0, st>>>(P, P.ps.q_mat, P.ps.counters + C_MAT);
    GT_CUDA(cudaGetLastError());
    klaunch[GT_KERNEL_OTHER] += 1;
    ctx->mapped[0] = 0;
    ctx->mapped[1] = 0;
    if (opts.progress && opts.progress_rgb && o_rgb) // unfinished pixels read as 0 in progress images
        GT_CUDA(cudaMemsetAsync(o_rgb, 0, size_t(n) * 3 * sizeof(float), st));
    int per_sm = 0;
    const bool world = P.sc.num_media != 0 || P.sc.num_objects != 0;
    GT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, world ? k_persistent<R, false, false, true> : k_persistent<R, false>, 128, 0));
    const uint32_t sms = uint32_t(ctx->num_sms > 0 ? ctx->num_sms : 1);
    const uint32_t blocks = std::max<uint32_t>(1u, std::min<uint32_t>(sms * uint32_t(std::max(per_sm, 1)), (n + 127) / 128));
    const bool profile = opts.profile != 0;
    cudaEvent_t a = nullptr, z = nullptr;
    GT_CUDA(ev.pair(a, z));
    GT_CUDA(cudaEventRecord(a, st));
    if (world)
        k_persistent<R, false, false, true><<<blocks, 128, 0, st>>>(P, d_next, P.ps.q_mat, P.ps.counters + C_MAT,
                                                                   ctx->mapped_dev, ctx->mapped_dev + 1, o_rgb, o_rgb64,
                                                                   o_acc);
    else
        k_persistent<R, false><<<blocks, 128, 0, st>>>(P, d_next, P.ps.q_mat, P.ps.counters + C_MAT, ctx->mapped_dev,
                                                       ctx->mapped_dev + 1, o_rgb, o_rgb64, o_acc);
    GT_CUDA(cudaGetLastError());
    klaunch[GT_KERNEL_PERSISTENT] += 1;
    GT_CUDA(cudaEventRecord(z, st));
    bool cancelled = false;
    if (opts.progress) {
        const uint32_t limit = P.cam.adaptive ? P.cam.adaptive_max : P.cam.spp;
        for (;;) {
            cudaError_t q = cudaEventQuery(z);
            if (q == cudaSuccess) break;
            if (q != cudaErrorNotReady) return cuda_fail(q, "persistent render");
            struct timespec ts{0, 2000000};
            nanosleep(&ts, nullptr);
            const uint32_t handed = std::min<uint32_t>(uint32_t(ctx->mapped[1]), n);
            if (opts.progress_rgb && o_rgb) { // copied beside the running launch, on the side stream
                GT_CUDA(cudaMemcpyAsync(opts.progress_rgb, o_rgb, size_t(n) * 3 * sizeof(float),
                                        cudaMemcpyDeviceToHost, ctx->side));
                GT_CUDA(cudaStreamSynchronize(ctx->side));
            }
            if (!cancelled && call_progress(ctx, opts, uint64_t(handed) * limit, uint64_t(n) * limit)) {
                ctx->mapped[0] = 1; // raise the cancel word: threads stop taking pixels
                cancelled = true;
            }
        }
    }
    GT_CUDA(cudaEventSynchronize(z));
    if (profile) {
        ev.note(GT_KERNEL_PERSISTENT, a, z);
        ev.harvest(kms);
    } else {
        ev.free_events.push_back(a);
        ev.free_events.push_back(z);
    }
    if (cancelled) return fail(GT_ERR_CANCELLED, "render cancelled by the progress callback");
    return GT_OK;
}

// Copies results to host buffers, checks the device error word and fills the stats.
template <class R>
gt_status finish_render(gt_context* ctx, const Params<R>& P, gt_frame* frame, const gt_render_opts& opts,
                        bool host_out, uint32_t n, float* o_rgb, double* o_rgb64, uint32_t* o_acc, float* o_alb,
                        float* o_nrm, EventPool& ev, double* kms, uint64_t* klaunch, uint64_t iters) {
    cudaStream_t st = ctx->stream;
    GT_CUDA(cudaEventRecord(ev.end, st));
    if (host_out) {
        GT_CUDA(cudaMemcpyAsync(frame->rgb, o_rgb, size_t(n) * 3 * sizeof(float), cudaMemcpyDeviceToHost, st));
        if (frame->rgb64)
            GT_CUDA(cudaMemcpyAsync(frame->rgb64, o_rgb64, size_t(n) * 3 * sizeof(double), cudaMemcpyDeviceToHost, st));
        if (frame->accepted)
            GT_CUDA(cudaMemcpyAsync(frame->accepted, o_acc, size_t(n) * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        if (opts.aovs && frame->albedo)
            GT_CUDA(cudaMemcpyAsync(frame->albedo, o_alb, size_t(n) * 3 * sizeof(float), cudaMemcpyDeviceToHost, st));
        if (opts.aovs && frame->normal)
            GT_CUDA(cudaMemcpyAsync(frame->normal, o_nrm, size_t(n) * 3 * sizeof(float), cudaMemcpyDeviceToHost, st));
    }
    // totals[0..3] and [6] into pinned words 2..9 and 14..15
    unsigned long long tot[4], prays = 0;
    GT_CUDA(cudaMemcpyAsync(ctx->pinned + 2, P.ps.totals, sizeof(tot), cudaMemcpyDeviceToHost, st));
    GT_CUDA(cudaMemcpyAsync(ctx->pinned + 14, P.ps.totals + 6, sizeof(prays), cudaMemcpyDeviceToHost, st));
    // counters[C_ERROR .. C_TAIL] into pinned words 10..13
    GT_CUDA(cudaMemcpyAsync(ctx->pinned + 10, P.ps.counters + C_ERROR, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    GT_CUDA(cudaStreamSynchronize(st));
    if (ctx->pinned[10]) return fail(GT_ERR_INTERNAL, "traversal stack overflow (BVH deeper than the device stack)");
    std::memcpy(tot, ctx->pinned + 2, sizeof(tot));
    std::memcpy(&prays, ctx->pinned + 14, sizeof(prays));
    if (opts.stats) {
        gt_render_stats& o = *opts.stats;
        std::memset(&o, 0, sizeof(o));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev.begin, ev.end);
        o.gpu_ms = ms;
        o.iterations = iters;
        o.rays = tot[0];
        o.shadow_rays = tot[1];
        o.samples = tot[2];
        o.samples_started = tot[3];
        o.migrated_pixels = ctx->pinned[10 + (C_MIGRATED - C_ERROR)];
        o.tail_pixels = ctx->pinned[10 + (C_TAIL - C_ERROR)];
        o.persistent_rays = prays;
        if (opts.profile) ev.harvest(kms);
        for (int k = 0; k < GT_KERNEL_COUNT; ++k) {
            o.kernel_ms[k] = opts.profile ? kms[k] : 0.0;
            o.kernel_launches[k] = klaunch[k];
        }
    }
    return GT_OK;
}

// Throughput mode: rounds of samples for every pixel still sampling, as many samples per
// round as keep the round near kSubItems items (so rounds grow as adaptive pixels stop).
// Each round traces its (pixel, sample) items in one k_substream launch and folds them into
// the pixels' sums in sample order (k_sub_fold), which also lists the pixels that go on.
constexpr uint64_t kSubItems = uint64_t(1) << 26; // work items per round, at most (or one per pixel)

// With adaptive sampling a pixel may stop at any sample of a round, and the round's later
// samples of that pixel are traced for nothing: rounds then take at most
// kSubAdaptiveRound samples per pixel.
constexpr uint32_t kSubAdaptiveRound = 8;

inline uint32_t sub_round_size(uint32_t count, uint32_t remaining, bool adaptive) {
    const uint64_t r = std::min<uint64_t>(remaining, kSubItems / std::max<uint32_t>(count, 1u));
    return std::max<uint32_t>(1u, uint32_t(adaptive ? std::min<uint64_t>(r, kSubAdaptiveRound) : r));
}

// Before a progress call of the throughput mode: the frame as far as its folded samples
// know it, copied into opts.progress_rgb (single frames).
template <class R>
gt_status sub_progress_image(gt_context* ctx, Params<R>& P, float* o_rgb, uint32_t n, const gt_render_opts& opts) {
    if (!opts.progress_rgb || !o_rgb) return GT_OK;
    const uint32_t sms = uint32_t(ctx->num_sms > 0 ? ctx->num_sms : 1);
    k_sub_preview<R><<<std::max<uint32_t>(1u, std::min<uint32_t>((n + 255) / 256, sms * 8)), 256, 0, ctx->stream>>>(
        P, o_rgb);
    GT_CUDA(cudaGetLastError());
    GT_CUDA(cudaMemcpyAsync(opts.progress_rgb, o_rgb, size_t(n) * 3 * sizeof(float), cudaMemcpyDeviceToHost,
                            ctx->stream));
    GT_CUDA(cudaStreamSynchronize(ctx->stream));
    return GT_OK;
}

template <class R, bool BATCH>
gt_status run_substreams(gt_context* ctx, Params<R>& P, uint32_t* const list[2], R4<R>* out, unsigned long long* next,
                         uint32_t n, uint32_t limit_max, bool adaptive, float* o_rgb, const gt_render_opts& opts,
                         EventPool& ev, double* kms, uint64_t* klaunch, uint64_t& rounds) {
    cudaStream_t st = ctx->stream;
    const uint32_t sms = uint32_t(ctx->num_sms > 0 ? ctx->num_sms : 1);
    int per_sm = 0;
    GT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_substream<R, BATCH>, 128, 0));
    const uint32_t blocks = sms * uint32_t(std::max(per_sm, 1));
    const uint32_t fblocks = std::max<uint32_t>(1u, std::min<uint32_t>((n + 255) / 256, sms * 8));
    const bool profile = opts.profile != 0;
    k_list_all<<<fblocks, 256, 0, st>>>(list[0], n, P.ps.counters + C_TRACE0);
    GT_CUDA(cudaGetLastError());
    klaunch[GT_KERNEL_OTHER] += 1;
    uint32_t count = n, cur = 0;
    for (uint32_t first = 0, round = 0; count > 0 && first < limit_max; first += round, cur ^= 1u) {
        round = sub_round_size(count, limit_max - first, adaptive);
        cudaEvent_t a = nullptr, z = nullptr;
        GT_CUDA(cudaMemsetAsync(next, 0, sizeof(unsigned long long), st));
        GT_CUDA(cudaMemsetAsync(P.ps.counters + C_TRACE0 + (cur ^ 1u), 0, sizeof(uint32_t), st));
        if (profile) {
            GT_CUDA(ev.pair(a, z));
            GT_CUDA(cudaEventRecord(a, st));
        }
        k_substream<R, BATCH><<<blocks, 128, 0, st>>>(P, list[cur], count, first, round, out, next);
        GT_CUDA(cudaGetLastError());
        klaunch[GT_KERNEL_PERSISTENT] += 1;
        if (profile) {
            GT_CUDA(cudaEventRecord(z, st));
            ev.note(GT_KERNEL_PERSISTENT, a, z);
            GT_CUDA(ev.pair(a, z));
            GT_CUDA(cudaEventRecord(a, st));
        }
        k_sub_fold<R, BATCH><<<fblocks, 256, 0, st>>>(P, list[cur], count, first, round, out, list[cur ^ 1u],
                                                      P.ps.counters + C_TRACE0 + (cur ^ 1u));
        GT_CUDA(cudaGetLastError());
        klaunch[GT_KERNEL_OTHER] += 1;
        if (profile) {
            GT_CUDA(cudaEventRecord(z, st));
            ev.note(GT_KERNEL_OTHER, a, z);
        }
        GT_CUDA(cudaMemcpyAsync(ctx->pinned, P.ps.counters + C_TRACE0 + (cur ^ 1u), sizeof(uint32_t),
                                cudaMemcpyDeviceToHost, st));
        GT_CUDA(cudaStreamSynchronize(st));
        count = ctx->pinned[0];
        ++rounds;
        const uint64_t done = std::min<uint64_t>(uint64_t(first) + round, limit_max);
        if (opts.progress) {
            if constexpr (!BATCH) {
                gt_status prc;
                if ((prc = sub_progress_image<R>(ctx, P, o_rgb, n, opts)) != GT_OK) return prc;
            }
            if (call_progress(ctx, opts, done * n, uint64_t(limit_max) * n))
                return fail(GT_ERR_CANCELLED, "render cancelled by the progress callback");
        }
    }
    return GT_OK;
}

// Throughput mode on the wavefront (one frame): each round's (pixel, sample) items are the
// wavefront's slots.  k_sub_init seeds every slot's own stream, k_generate starts each
// slot's one sample and, when its path has ended, writes its radiance out; the bounces run
// through k_trace, k_shade and k_shadow as in the reference mode, sorted by material, and
// a round ends when every slot is done (at most max_depth + 1 iterations, as no slot
// starts a second sample).  k_sub_fold then adds the round to the pixels' sums.
constexpr uint64_t kSubWaveItems = uint64_t(1) << 24; // slots of one round (or one per pixel)

template <class R>
gt_status run_sub_wavefront(gt_context* ctx, Params<R>& P, std::vector<Params<R>>& SW, SubRound<R>* d_sub,
                            uint32_t* const list[2], R4<R>* out, uint32_t cap, uint32_t n, uint32_t limit_max, bool nee,
                            bool objects, float* o_rgb, const gt_render_opts& opts, EventPool& ev, double* kms,
                            uint64_t* klaunch, uint64_t& rounds) {
    cudaStream_t st = ctx->stream;
    const uint32_t sms = uint32_t(ctx->num_sms > 0 ? ctx->num_sms : 1), threads = 256;
    const uint32_t gen_per_sm = opts.generate_blocks_per_sm ? std::min<uint32_t>(opts.generate_blocks_per_sm, 32u) : 8u;
    const uint32_t wave_per_sm = opts.trace_blocks_per_sm ? std::min<uint32_t>(opts.trace_blocks_per_sm, 32u) : 6u;
    const bool profile = opts.profile != 0;
    const uint32_t K = uint32_t(SW.size());
    const uint32_t fblocks = std::max<uint32_t>(1u, std::min<uint32_t>((n + 255) / 256, sms * 8));
    // the fold's pixel lists count into words the wavefront does not use in this mode
    uint32_t* list_count[2] = {P.ps.counters + C_SIDE_DONE, P.ps.counters + C_SIDE_COOP};
    for (uint32_t k = 0; k < K; ++k) GT_CUDA(cudaMemsetAsync(SW[k].ps.counters, 0, C_COUNT * sizeof(uint32_t), st));
    k_list_all<<<fblocks, 256, 0, st>>>(list[0], n, list_count[0]);
    GT_CUDA(cudaGetLastError());
    klaunch[GT_KERNEL_OTHER] += 1;
    uint32_t count = n, cur = 0;
    for (uint32_t first = 0, round = 0; count > 0 && first < limit_max; first += round, cur ^= 1u) {
        round = std::max<uint32_t>(1u, std::min<uint32_t>(limit_max - first, cap / count));
        if (P.cam.adaptive) round = std::min(round, kSubAdaptiveRound);
        const uint32_t items = count * round;
        const uint32_t kk = std::min(K, round); // stripes with rows this round
        const SubRound<R> h{list[cur], out, count, first};
        GT_CUDA(cudaMemcpyAsync(d_sub, &h, sizeof(h), cudaMemcpyHostToDevice, st));
        for (uint32_t k = 0; k < kk; ++k)
            GT_CUDA(cudaMemsetAsync(SW[k].ps.counters, 0, (C_DONE + 1) * sizeof(uint32_t), st));
        cudaEvent_t ready = nullptr;
        GT_CUDA(ev.get(ready));
        GT_CUDA(cudaEventRecord(ready, st));
        ev.free_events.push_back(ready);
        std::vector<cudaStream_t> ss(kk);
        std::vector<uint32_t> local(kk), lblocks(kk), wblocks(kk);
        for (uint32_t k = 0; k < kk; ++k) {
            Params<R>& Q = SW[k];
            Q.ps.n = items;
            Q.ps.stripe = k;
            Q.ps.stripes = kk;
            Q.ps.row = count;
            Q.ps.local_n = local[k] = ((round - k + kk - 1) / kk) * count;
            lblocks[k] = std::max<uint32_t>(1u, std::min<uint32_t>((local[k] + threads - 1) / threads, sms * gen_per_sm));
            wblocks[k] = std::max<uint32_t>(1u, std::min<uint32_t>((local[k] + threads - 1) / threads, sms * wave_per_sm));
            ss[k] = profile ? st : ctx->stripe_stream[k];
            GT_CUDA(cudaStreamWaitEvent(ss[k], ready, 0));
            k_sub_init<R><<<lblocks[k], threads, 0, ss[k]>>>(Q);
            GT_CUDA(cudaGetLastError());
            klaunch[GT_KERNEL_OTHER] += 1;
        }
        // Iterations in batches between checks of the done counts: a path lasts at most
        // max_depth + 1 iterations (camera ray, bounces, and its radiance written out).
        const uint32_t max_iters = 2u * (P.cam.max_depth + 2u) + 8u;
        std::vector<bool> running(kk, true);
        std::vector<uint32_t> q(kk, 0u);
        uint32_t iters = 0, active = kk;
        // The first batch of iterations of stripe k, launched directly or (outside profile
        // mode) captured once as a graph that is relaunched while the stripe's kernel
        // parameters and launch sizes stay the same (rounds of one size, renders of one frame).
        // Without next-event queries k_shade writes each finished sample out, so after the
        // first iteration only k_generate's counter resets are needed.
        // trace (1), shade (2) or shadow (3) of stripe k; a world with objects runs the
        // kernels' OBJ instantiations
        auto launch_kind = [&](int kind, uint32_t k, uint32_t qq) {
            if (objects) {
                if (kind == 1) k_trace<R, true><<<wblocks[k], threads, 0, ss[k]>>>(SW[k], qq);
                else if (kind == 2) k_shade<R, false, true><<<wblocks[k], threads, 0, ss[k]>>>(SW[k], qq);
                else k_shadow<R, true><<<wblocks[k], threads, 0, ss[k]>>>(SW[k]);
            } else {
                if (kind == 1) k_trace<R><<<wblocks[k], threads, 0, ss[k]>>>(SW[k], qq);
                else if (kind == 2) k_shade<R><<<wblocks[k], threads, 0, ss[k]>>>(SW[k], qq);
                else k_shadow<R><<<wblocks[k], threads, 0, ss[k]>>>(SW[k]);
            }
        };
        auto launch_iterations = [&](uint32_t k, uint32_t batch) -> cudaError_t {
            for (uint32_t b = 0; b < batch; ++b) {
                const uint32_t qq = (q[k] + b) & 1u;
                if (b == 0 || nee) k_generate<R><<<lblocks[k], threads, 0, ss[k]>>>(SW[k], qq);
                else k_iteration_reset<R><<<1, 32, 0, ss[k]>>>(SW[k], qq);
                launch_kind(1, k, qq);
                launch_kind(2, k, qq);
                if (nee) launch_kind(3, k, qq);
            }
            return cudaGetLastError();
        };
        auto graph_batch = [&](uint32_t k, uint32_t batch) -> gt_status {
            std::vector<unsigned char> key(sizeof(Params<R>) + 5 * sizeof(uint32_t));
            std::memcpy(key.data(), &SW[k], sizeof(Params<R>));
            const uint32_t extra[5] = {batch, lblocks[k], wblocks[k], nee ? 1u : 0u, 0x5B5u};
            std::memcpy(key.data() + sizeof(Params<R>), extra, sizeof(extra));
            gt_context::CachedGraph& cg = ctx->graphs[k];
            if (!(cg.exec && cg.key == key)) {
                if (cg.exec) cudaGraphExecDestroy(cg.exec);
                cg.exec = nullptr;
                cg.key.clear();
                cudaGraph_t graph = nullptr;
                GT_CUDA(cudaStreamBeginCapture(ss[k], cudaStreamCaptureModeThreadLocal));
                const cudaError_t le = launch_iterations(k, batch);
                const cudaError_t ce = cudaStreamEndCapture(ss[k], &graph);
                if (le != cudaSuccess || ce != cudaSuccess) {
                    if (graph) cudaGraphDestroy(graph);
                    return cuda_fail(le != cudaSuccess ? le : ce, "substream graph capture");
                }
                const cudaError_t ie = cudaGraphInstantiate(&cg.exec, graph, 0);
                cudaGraphDestroy(graph);
                if (ie != cudaSuccess) {
                    cg.exec = nullptr;
                    return cuda_fail(ie, "cudaGraphInstantiate");
                }
                cg.key = std::move(key);
            }
            GT_CUDA(cudaGraphLaunch(cg.exec, ss[k]));
            return GT_OK;
        };
        while (active > 0) {
            const uint32_t batch = iters == 0 ? std::min<uint32_t>(P.cam.max_depth + 2u, 16u) : 2u;
            for (uint32_t k = 0; k < kk; ++k) {
                if (!running[k]) continue;
                if (iters == 0 && !profile) {
                    gt_status grc;
                    if ((grc = graph_batch(k, batch)) != GT_OK) return grc;
                    q[k] ^= batch & 1u;
                    klaunch[GT_KERNEL_GENERATE] += nee ? batch : 1u;
                    klaunch[GT_KERNEL_OTHER] += nee ? 0u : batch - 1u;
                    klaunch[GT_KERNEL_TRACE] += batch;
                    klaunch[GT_KERNEL_SHADE] += batch;
                    if (nee) klaunch[GT_KERNEL_SHADOW] += batch;
                    GT_CUDA(cudaMemcpyAsync(ctx->pinned + 64 + k, SW[k].ps.counters + C_DONE, sizeof(uint32_t),
                                            cudaMemcpyDeviceToHost, ss[k]));
                    continue;
                }
                for (uint32_t b = 0; b < batch; ++b, q[k] ^= 1u) {
                    for (int kind = 0; kind < (nee ? 4 : 3); ++kind) {
                        cudaEvent_t a = nullptr, z = nullptr;
                        if (profile) {
                            GT_CUDA(ev.pair(a, z));
                            GT_CUDA(cudaEventRecord(a, ss[k]));
                        }
                        const bool gen = iters + b == 0 || nee;
                        if (kind == 0 && gen) k_generate<R><<<lblocks[k], threads, 0, ss[k]>>>(SW[k], q[k]);
                        else if (kind == 0) k_iteration_reset<R><<<1, 32, 0, ss[k]>>>(SW[k], q[k]);
                        else launch_kind(kind, k, q[k]);
                        GT_CUDA(cudaGetLastError());
                        if (profile) {
                            GT_CUDA(cudaEventRecord(z, ss[k]));
                            ev.note(kind == 0 ? GT_KERNEL_GENERATE
                                              : kind == 1 ? GT_KERNEL_TRACE : kind == 2 ? GT_KERNEL_SHADE : GT_KERNEL_SHADOW,
                                    a, z);
                        }
                    }
                    klaunch[iters + b == 0 || nee ? GT_KERNEL_GENERATE : GT_KERNEL_OTHER] += 1;
                    klaunch[GT_KERNEL_TRACE] += 1;
                    klaunch[GT_KERNEL_SHADE] += 1;
                    if (nee) klaunch[GT_KERNEL_SHADOW] += 1;
                }
                GT_CUDA(cudaMemcpyAsync(ctx->pinned + 64 + k, SW[k].ps.counters + C_DONE, sizeof(uint32_t),
                                        cudaMemcpyDeviceToHost, ss[k]));
            }
            iters += batch;
            for (uint32_t k = 0; k < kk; ++k)
                if (running[k]) GT_CUDA(cudaStreamSynchronize(ss[k]));
            for (uint32_t k = 0; k < kk; ++k)
                if (running[k] && ctx->pinned[64 + k] >= local[k]) {
                    running[k] = false;
                    --active;
                }
            if (active > 0 && iters > max_iters)
                return fail(GT_ERR_INTERNAL, "substream round did not finish within its iteration bound");
        }
        rounds += iters;
        GT_CUDA(cudaMemsetAsync(list_count[cur ^ 1u], 0, sizeof(uint32_t), st));
        k_sub_fold<R, false><<<fblocks, 256, 0, st>>>(P, list[cur], count, first, round, out, list[cur ^ 1u],
                                                      list_count[cur ^ 1u]);
        GT_CUDA(cudaGetLastError());
        klaunch[GT_KERNEL_OTHER] += 1;
        GT_CUDA(cudaMemcpyAsync(ctx->pinned, list_count[cur ^ 1u], sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        GT_CUDA(cudaStreamSynchronize(st));
        count = ctx->pinned[0];
        const uint64_t done = std::min<uint64_t>(uint64_t(first) + round, limit_max);
        if (opts.progress) {
            gt_status prc;
            if ((prc = sub_progress_image<R>(ctx, P, o_rgb, n, opts)) != GT_OK) return prc;
            if (call_progress(ctx, opts, done * n, uint64_t(limit_max) * n))
                return fail(GT_ERR_CANCELLED, "render cancelled by the progress callback");
        }
    }
    // the stripes' stack-overflow flags
    for (uint32_t k = 0; k < K; ++k)
        GT_CUDA(cudaMemcpyAsync(ctx->pinned + 64 + k, SW[k].ps.counters + C_ERROR, sizeof(uint32_t),
                                cudaMemcpyDeviceToHost, st));
    GT_CUDA(cudaStreamSynchronize(st));
    for (uint32_t k = 0; k < K; ++k)
        if (ctx->pinned[64 + k]) return fail(GT_ERR_INTERNAL, "traversal stack overflow (BVH deeper than the device stack)");
    return GT_OK;
}

// One frame (BATCH = false) or, with BATCH = true, the frames bcams[0 .. bcount) of equal
// width as one image of their rows stacked in order: every wavefront kernel then looks up
// each slot's frame camera, and each frame's slice of the result goes to bframes[i].
template <class R, bool BATCH = false>
gt_status render_impl(gt_scene* s, const gt_lights* l, gt_environment* e, const CamHost& cam,
                      const gt_render_opts& opts, gt_frame* frame, gt_accumulator* accum = nullptr,
                      uint32_t add_samples = 0, const CamHost* bcams = nullptr, uint32_t bcount = 0,
                      gt_frame* const* bframes = nullptr) {
    gt_context* ctx = s->ctx;
    cudaStream_t st = ctx->stream;
    gt_status rc;
    if ((rc = upload_scene<R>(s)) != GT_OK) return rc;
    const bool use_lights = l != nullptr;
    const bool use_env = e != nullptr;
    Params<R> P;
    std::memset(&P, 0, sizeof(P));
    P.sc = gpu_of<R>(s).view;
    if (use_lights) {
        if ((rc = upload_lights<R>(const_cast<gt_lights*>(l))) != GT_OK) return rc;
        P.lights = lights_of<R>(const_cast<gt_lights*>(l)).view;
    }
    if (use_env) {
        if ((rc = upload_env<R>(e)) != GT_OK) return rc;
        P.env = env_of<R>(e).view;
    }
    P.cam = cam_dev<R>(cam, use_lights, use_env);
    if (accum) P.cam.spp = accum->samples + add_samples; // the streams run on to the new total
    uint32_t n_pix = cam.width * cam.height;
    uint32_t img_h = cam.height; // rows the stripes deal out
    uint32_t limit_max = P.cam.adaptive ? P.cam.adaptive_max : P.cam.spp, depth_max = P.cam.max_depth;
    bool any_nee = P.cam.nee && (use_lights || use_env), want64 = false, any_adaptive = P.cam.adaptive != 0;
    std::vector<CamDev<R>> bcd;
    std::vector<uint32_t> bstart;
    if constexpr (BATCH) {
        bcd.resize(bcount);
        bstart.resize(size_t(bcount) + 1);
        uint64_t total = 0;
        img_h = 0;
        for (uint32_t i = 0; i < bcount; ++i) {
            bcd[i] = cam_dev<R>(bcams[i], use_lights, use_env);
            bstart[i] = uint32_t(total);
            total += uint64_t(bcams[i].width) * bcams[i].height;
            if (total >= (1ull << 31)) return fail(GT_ERR_INVALID_ARG, "a batch holds fewer than 2^31 pixels");
            img_h += bcams[i].height;
            limit_max = std::max(limit_max, bcd[i].adaptive ? bcd[i].adaptive_max : bcd[i].spp);
            depth_max = std::max(depth_max, bcd[i].max_depth);
            any_nee = any_nee || (bcd[i].nee && (use_lights || use_env));
            any_adaptive = any_adaptive || bcd[i].adaptive != 0;
            want64 = want64 || bframes[i]->rgb64 != nullptr;
        }
        bstart[bcount] = uint32_t(total);
        n_pix = uint32_t(total);
        P.num_frames = bcount;
    }
    const uint32_t n = n_pix;
    const bool nee = any_nee;

    // Workspace: path state (wavefront only), per-stripe queues and counters, and device
    // staging for host outputs.
    // A world with media renders on the persistent schedule, whose WORLD variant traces
    // shadow queries in the reference's order of draws (a medium's hit draws from the
    // pixel's stream); accumulation resumes wavefront state in that variant's RESUME mode.
    // A world with objects and no media draws nothing in its hits, so it renders on the
    // wavefront (OBJ kernels: the rays also test the objects), single frames and batches,
    // and its tail in the world variant.
    const bool world = P.sc.num_media != 0 || P.sc.num_objects != 0;
    const bool media = P.sc.num_media != 0;
    const bool obj_wave = world && !media;
    if (BATCH && media) return fail(GT_ERR_UNSUPPORTED, "a scene with media does not render as a wavefront batch");
    // Throughput mode: every (pixel, sample) pair of a round is a work item.
    const bool subs = opts.rng == GT_RNG_SUBSTREAMS;
    if (BATCH && subs && world) return fail(GT_ERR_UNSUPPORTED, "a substream batch does not render a scene with objects");
    if (subs && (media || accum))
        return fail(GT_ERR_UNSUPPORTED, "substreams render neither worlds with media nor accumulations");
    // A single frame of a scene with objects or with more than kSubWaveMinPrims primitives
    // runs its rounds through the wavefront kernels (k_generate starts each slot's one
    // sample); a batch, or a small scene, through k_substream.  Measured (Msamples/s, wavefront / k_substream):
    // final scene (485 spheres) 933 / 669, mesh-heavy 332 / 185, Cornell box (13) 1,376 /
    // 1,804: with a tiny tree the one-kernel path loop is cheaper than the wavefront's
    // path-state traffic.
    constexpr uint32_t kSubWaveMinPrims = 64;
    const bool sub_wave = subs && !BATCH && (P.sc.num_prims > kSubWaveMinPrims || obj_wave);
    // one round's items at most: the cap, or the frame's samples when it has fewer
    const uint64_t sub_items = std::max<uint64_t>(
        std::min<uint64_t>(sub_wave ? kSubWaveItems : kSubItems, uint64_t(n_pix) * std::max(limit_max, 1u)), n_pix);
    const bool persistent = !subs && ((!BATCH && opts.schedule == GT_SCHEDULE_PERSISTENT && !accum) || (media && !accum));
    const bool host_out = BATCH || frame->device_buffers == 0;
    // Wavefront stripes: rows are dealt round-robin to K independent wavefronts on their
    // own streams, whose kernels then overlap on the GPU (each kernel alone leaves SMs
    // waiting on memory).
    uint32_t K = opts.stripes ? opts.stripes : 4u;
    K = std::max<uint32_t>(1u, std::min<uint32_t>({K, uint32_t(gt_context::kMaxStripes), img_h}));
    if (persistent || media || subs) K = 1;
    const uint32_t qcap = ((img_h + K - 1) / K) * cam.width;
    std::vector<Params<R>> SP(K);
    CamDev<R>* d_cams = nullptr;
    uint32_t* d_start = nullptr;
    uint32_t* sub_list[2] = {nullptr, nullptr};
    R4<R>* sub_out = nullptr;
    unsigned long long* sub_next = nullptr;
    Params<R> W = P;               // substream wavefront: one round's item slots
    SubRound<R>* d_sub = nullptr;
    // its stripes (sample rows dealt round-robin, as pixel rows are in the reference mode)
    // (default 2: final scene 928 / 995 / 876 / 704 Msamples/s with 1 / 2 / 4 / 8 stripes,
    // mesh-heavy 332 / 399 / 405 / 399)
    const uint32_t sub_k = std::max<uint32_t>(1u, std::min<uint32_t>(opts.stripes ? opts.stripes : 2u,
                                                                      uint32_t(gt_context::kMaxStripes)));
    std::vector<Params<R>> SW(sub_wave ? sub_k : 0u);
    auto lay = [&](Bump& bb) {
        if constexpr (BATCH) {
            d_cams = bb.take<CamDev<R>>(bcount);
            d_start = bb.take<uint32_t>(size_t(bcount) + 1);
            P.cams = d_cams;
            P.frame_start = d_start;
        }
        if (subs) { // per-pixel sums, two pixel lists, one round's sample radiance
            layout_slots<R>(bb, P.ps, n, false);
            P.ps.counters = bb.take<uint32_t>(C_COUNT);
            sub_list[0] = bb.take<uint32_t>(n);
            sub_list[1] = bb.take<uint32_t>(n);
            sub_out = bb.take<R4<R>>(sub_items);
            sub_next = bb.take<unsigned long long>(1);
            if (sub_wave) { // the wavefront's slots are a round's items, rows dealt to stripes
                W = P;
                layout_slots<R>(bb, W.ps, uint32_t(sub_items), nee, obj_wave);
                W.ps.totals = P.ps.totals;
                d_sub = bb.take<SubRound<R>>(1);
                W.sub = d_sub;
                for (uint32_t k = 0; k < sub_k; ++k) {
                    SW[k] = W;
                    layout_queues<R>(bb, SW[k].ps, uint32_t(sub_items / sub_k + n), nee);
                }
            }
            SP[0] = P;
        } else if (persistent) {
            P.ps.n = n;
            P.ps.counters = bb.take<uint32_t>(C_COUNT);
            P.ps.totals = bb.take<unsigned long long>(8);
            P.ps.q_mat = bb.take<uint32_t>(size_t(n) * NUM_COST_CLASSES); // cost-ordered pixel queues
        } else {
            layout_slots<R>(bb, P.ps, n, nee, obj_wave);
            for (uint32_t k = 0; k < K; ++k) {
                SP[k] = P;
                layout_queues<R>(bb, SP[k].ps, qcap, nee);
                SP[k].ps.stripe = k;
                SP[k].ps.stripes = K;
                SP[k].ps.row = cam.width;
                SP[k].ps.local_n = ((img_h - k + K - 1) / K) * cam.width;
            }
            P.ps.counters = SP[0].ps.counters; // the error word k_resolve-side checks read
        }
        return bb.take<uint32_t>(K); // persistent pixel counters (one per stripe's tail)
    };
    Bump sizing{nullptr};
    lay(sizing);
    sizing.take<float>(size_t(n) * 3 * 3);
    sizing.take<double>(size_t(n) * 3);
    sizing.take<uint32_t>(n);
    if ((rc = ensure_workspace(ctx, sizing.off + 4096)) != GT_OK) return rc;
    Bump b{static_cast<char*>(ctx->ws)};
    uint32_t* d_next = lay(b);
    float* d_rgb = b.take<float>(size_t(n) * 3);
    float* d_alb = b.take<float>(size_t(n) * 3);
    float* d_nrm = b.take<float>(size_t(n) * 3);
    double* d_rgb64 = b.take<double>(size_t(n) * 3);
    uint32_t* d_acc = b.take<uint32_t>(n);
    float* o_rgb = d_rgb;
    float *o_alb = nullptr, *o_nrm = nullptr;
    double* o_rgb64 = want64 ? d_rgb64 : nullptr;
    uint32_t* o_acc = d_acc;
    if constexpr (!BATCH) {
        o_rgb = host_out ? d_rgb : frame->rgb;
        o_alb = host_out ? (frame->albedo ? d_alb : nullptr) : frame->albedo;
        o_nrm = host_out ? (frame->normal ? d_nrm : nullptr) : frame->normal;
        o_rgb64 = host_out ? (frame->rgb64 ? d_rgb64 : nullptr) : frame->rgb64;
        o_acc = host_out ? (frame->accepted ? d_acc : nullptr) : frame->accepted;
    }

    const int sms = ctx->num_sms > 0 ? ctx->num_sms : 1;
    const uint32_t threads = 256;
    const uint32_t slot_blocks = std::max<uint32_t>(1u, std::min<uint32_t>((n + threads - 1) / threads, uint32_t(sms) * 8));

    // Device time of the whole render, and in profile mode of every kernel launch.
    EventPool ev;
    if ((rc = ev.init()) != GT_OK) return rc;
    const bool profile = opts.profile != 0;
    double kms[GT_KERNEL_COUNT] = {0};
    uint64_t klaunch[GT_KERNEL_COUNT] = {0};
    GT_CUDA(cudaEventRecord(ev.begin, st));
    if (persistent) {
        rc = run_persistent<R>(ctx, P, d_next, o_rgb, o_rgb64, o_acc, opts, ev, kms, klaunch);
        if (rc != GT_OK) return rc;
        if (opts.aovs && (o_alb || o_nrm)) {
            cudaEvent_t a = nullptr, z = nullptr;
            if (profile) GT_CUDA(ev.pair(a, z));
            if (profile) GT_CUDA(cudaEventRecord(a, st));
            k_aov<R><<<slot_blocks, threads, 0, st>>>(P, o_alb, o_nrm);
            GT_CUDA(cudaGetLastError());
            klaunch[GT_KERNEL_OTHER] += 1;
            if (profile) {
                GT_CUDA(cudaEventRecord(z, st));
                ev.note(GT_KERNEL_OTHER, a, z);
            }
        }
        return finish_render<R>(ctx, P, frame, opts, host_out, n, o_rgb, o_rgb64, o_acc, o_alb, o_nrm, ev, kms,
                                klaunch, 1);
    }
    {
        cudaEvent_t a = nullptr, z = nullptr;
        if (profile) GT_CUDA(ev.pair(a, z));
        if (profile) GT_CUDA(cudaEventRecord(a, st));
        for (uint32_t k = 0; k < K; ++k)
            GT_CUDA(cudaMemsetAsync(SP[k].ps.counters, 0, C_COUNT * sizeof(uint32_t), st));
        if constexpr (BATCH) {
            GT_CUDA(cudaMemcpyAsync(d_cams, bcd.data(), bcd.size() * sizeof(CamDev<R>), cudaMemcpyHostToDevice, st));
            GT_CUDA(cudaMemcpyAsync(d_start, bstart.data(), bstart.size() * sizeof(uint32_t), cudaMemcpyHostToDevice,
                                    st));
        }
        k_init<R, BATCH><<<slot_blocks, threads, 0, st>>>(P);
        GT_CUDA(cudaGetLastError());
        klaunch[GT_KERNEL_OTHER] += 1;
        if (accum && accum->samples > 0) {
            k_accum_load<R><<<slot_blocks, threads, 0, st>>>(P, accum->rng, static_cast<const R4<R>*>(accum->sum),
                                                             static_cast<const R4<R>*>(accum->comp), accum->accepted,
                                                             accum->samples);
            GT_CUDA(cudaGetLastError());
            klaunch[GT_KERNEL_OTHER] += 1;
        }
        if (profile) {
            GT_CUDA(cudaEventRecord(z, st));
            ev.note(GT_KERNEL_OTHER, a, z);
        }
    }

    if (subs) {
        uint64_t rounds = 0;
        if (sub_wave)
            rc = run_sub_wavefront<R>(ctx, P, SW, d_sub, sub_list, sub_out, uint32_t(sub_items), n, limit_max, nee,
                                      obj_wave, o_rgb, opts, ev, kms, klaunch, rounds);
        else
            rc = run_substreams<R, BATCH>(ctx, P, sub_list, sub_out, sub_next, n, limit_max, any_adaptive, o_rgb,
                                          opts, ev, kms, klaunch, rounds);
        if (rc != GT_OK) return rc;
        k_resolve<R, BATCH><<<slot_blocks, threads, 0, st>>>(P, o_rgb, o_rgb64, o_acc);
        GT_CUDA(cudaGetLastError());
        klaunch[GT_KERNEL_OTHER] += 1;
        if (!BATCH && opts.aovs && (o_alb || o_nrm)) { // the AOV pass keeps the reference's pixel streams
            k_aov<R><<<slot_blocks, threads, 0, st>>>(P, o_alb, o_nrm);
            GT_CUDA(cudaGetLastError());
            klaunch[GT_KERNEL_OTHER] += 1;
        }
        if constexpr (BATCH) {
            for (uint32_t i = 0; i < bcount; ++i) {
                gt_frame* f = bframes[i];
                const size_t o = bstart[i], np = size_t(bstart[i + 1]) - bstart[i];
                const cudaMemcpyKind kind = f->device_buffers ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
                GT_CUDA(cudaMemcpyAsync(f->rgb, d_rgb + o * 3, np * 3 * sizeof(float), kind, st));
                if (f->rgb64) GT_CUDA(cudaMemcpyAsync(f->rgb64, d_rgb64 + o * 3, np * 3 * sizeof(double), kind, st));
                if (f->accepted) GT_CUDA(cudaMemcpyAsync(f->accepted, d_acc + o, np * sizeof(uint32_t), kind, st));
            }
            return finish_render<R>(ctx, P, nullptr, opts, false, n, o_rgb, o_rgb64, o_acc, o_alb, o_nrm, ev, kms,
                                    klaunch, rounds);
        } else {
            return finish_render<R>(ctx, P, frame, opts, host_out, n, o_rgb, o_rgb64, o_acc, o_alb, o_nrm, ev, kms,
                                    klaunch, rounds);
        }
    }

    if constexpr (!BATCH) {
        if (media) { // accumulated world with media: every pixel's chain continues from the
                     // state just loaded in the RESUME mode of the persistent kernel's world variant
            Params<R> Q = SP[0];
            uint32_t* list = Q.ps.q_handoff; // n entries: one stripe
            uint32_t* count = Q.ps.counters + C_TAIL;
            GT_CUDA(cudaMemsetAsync(d_next, 0, sizeof(uint32_t), st));
            k_list_all<<<slot_blocks, threads, 0, st>>>(list, n, count);
            GT_CUDA(cudaGetLastError());
            int per_sm = 0;
            GT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_persistent<R, true, false, true>, 128, 0));
            const uint32_t blocks =
                std::max<uint32_t>(1u, std::min<uint32_t>(uint32_t(sms) * uint32_t(std::max(per_sm, 1)), (n + 127) / 128));
            cudaEvent_t a = nullptr, z = nullptr;
            if (profile) GT_CUDA(ev.pair(a, z));
            if (profile) GT_CUDA(cudaEventRecord(a, st));
            k_persistent<R, true, false, true><<<blocks, 128, 0, st>>>(Q, d_next, list, count, nullptr, nullptr, nullptr,
                                                                       nullptr, nullptr);
            GT_CUDA(cudaGetLastError());
            klaunch[GT_KERNEL_PERSISTENT] += 2;
            if (profile) {
                GT_CUDA(cudaEventRecord(z, st));
                ev.note(GT_KERNEL_PERSISTENT, a, z);
            }
            k_resolve<R, false><<<slot_blocks, threads, 0, st>>>(P, o_rgb, o_rgb64, o_acc);
            GT_CUDA(cudaGetLastError());
            if (opts.aovs && (o_alb || o_nrm)) {
                k_aov<R><<<slot_blocks, threads, 0, st>>>(P, o_alb, o_nrm);
                GT_CUDA(cudaGetLastError());
                klaunch[GT_KERNEL_OTHER] += 1;
            }
            k_accum_store<R><<<slot_blocks, threads, 0, st>>>(P, accum->rng, static_cast<R4<R>*>(accum->sum),
                                                              static_cast<R4<R>*>(accum->comp), accum->accepted);
            GT_CUDA(cudaGetLastError());
            klaunch[GT_KERNEL_OTHER] += 2;
            rc = finish_render<R>(ctx, P, frame, opts, host_out, n, o_rgb, o_rgb64, o_acc, o_alb, o_nrm, ev, kms, klaunch, 0);
            if (rc == GT_OK) {
                accum->samples += add_samples;
                accum->seed = cam.desc.rng_seed;
            }
            return rc;
        }
    }

    // Per-stripe launch sizes: a stripe owns about 1/K of the GPU.
    int tail_per_sm = 0, coop_per_sm = 0;
    GT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&tail_per_sm, k_persistent<R, true, BATCH>, 128, 0));
    GT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&coop_per_sm, k_persistent<R, true, BATCH, false, true>, 128, 0));
    const uint32_t full_persist = uint32_t(sms) * uint32_t(std::max(tail_per_sm, 1));
    const uint32_t full_coop = uint32_t(sms) * uint32_t(std::max(coop_per_sm, 1));
    const uint32_t gen_per_sm = opts.generate_blocks_per_sm ? std::min<uint32_t>(opts.generate_blocks_per_sm, 32u) : 8u;
    const uint32_t wave_per_sm = opts.trace_blocks_per_sm ? std::min<uint32_t>(opts.trace_blocks_per_sm, 32u) : 6u;
    const uint32_t lblocks =
        std::max<uint32_t>(1u, std::min<uint32_t>((qcap + threads - 1) / threads, uint32_t(sms) * gen_per_sm));
    const uint32_t wblocks =
        std::max<uint32_t>(1u, std::min<uint32_t>((qcap + threads - 1) / threads, uint32_t(sms) * wave_per_sm));
    const uint32_t tblocks = std::max<uint32_t>(uint32_t(sms), full_persist / K);
    const uint32_t coop_blocks = std::max<uint32_t>(uint32_t(sms), full_coop / K);
    const uint32_t side_blocks = std::max<uint32_t>(uint32_t(sms) / 2u, full_persist / K);
    const uint32_t side_coop_blocks = std::max<uint32_t>(uint32_t(sms) / 2u, uint32_t(sms) * 2u / K);
    uint32_t tail_slots = 0;
    if (opts.schedule == GT_SCHEDULE_AUTO)
        tail_slots = opts.tail_slots ? (opts.tail_slots + K - 1) / K : tblocks * 128u;
    // Slow-slot migration: once per stripe, after kMigrateAfter iterations, the slots
    // progressing at less than 1/kMigrateRatio of the stripe's mean sample rate move to
    // k_persistent (resume mode) on the stripe's side stream.  By default only in scenes
    // of at most kMigrateMaxPrims primitives: on the 2.36 M-triangle frame the migrated
    // slots' persistent walks ran slower than the wavefront (267 against 297 Msamples/s),
    // while small scenes gain (64 adaptive batch frames: 1,177 against 1,075).
    constexpr uint64_t kMigrateAfter = 60;
    constexpr float kMigrateRatio = 2.0f;
    constexpr uint32_t kMigrateMaxPrims = 65536;
    // (not in a world with objects: the side kernel is the plain persistent variant)
    const bool may_migrate =
        opts.schedule == GT_SCHEDULE_AUTO && !obj_wave &&
        (opts.migrate == GT_MIGRATE_ON || (opts.migrate == GT_MIGRATE_DEFAULT && P.sc.num_prims <= kMigrateMaxPrims));
    ctx->mapped[0] = 0; // the side kernels' cancel word

    // One iteration = generate, trace, shade (+ shadow); two iterations (ping-pong trace
    // queues) are captured once per stripe as a graph and replayed.
    const int kernels_per_iteration = nee ? 4 : 3;
    struct Stripe {
        cudaStream_t st, side;
        cudaGraphExec_t exec = nullptr;
        uint64_t iters = 0;
        uint32_t batch = 2;
        bool running = true, migrated = false, tail = false;
        cudaEvent_t fork = nullptr, join = nullptr;
    };
    std::vector<Stripe> S(K);
    auto launch_iteration = [&](uint32_t k, uint32_t cur, bool timed) -> cudaError_t {
        const cudaStream_t s = S[k].st;
        for (int q = 0; q < kernels_per_iteration; ++q) {
            cudaEvent_t a = nullptr, z = nullptr;
            if (timed) {
                cudaError_t e = ev.pair(a, z);
                if (e != cudaSuccess) return e;
                cudaEventRecord(a, s);
            }
            // shade and shadow grids at most their resident blocks (one wave)
            const uint32_t shade_blocks = std::min<uint32_t>(wblocks, uint32_t(sms) * kShadeBlocksPerSm);
            const uint32_t shadow_blocks = std::min<uint32_t>(wblocks, uint32_t(sms) * kShadowBlocksPerSm);
            if (q == 0) k_generate<R, BATCH><<<lblocks, threads, 0, s>>>(SP[k], cur);
            else if (obj_wave) {
                if (q == 1) k_trace<R, true><<<wblocks, threads, 0, s>>>(SP[k], cur);
                else if (q == 2) k_shade<R, BATCH, true><<<shade_blocks, threads, 0, s>>>(SP[k], cur);
                else k_shadow<R, true><<<shadow_blocks, threads, 0, s>>>(SP[k]);
            } else if (q == 1) k_trace<R><<<wblocks, threads, 0, s>>>(SP[k], cur);
            else if (q == 2) k_shade<R, BATCH><<<shade_blocks, threads, 0, s>>>(SP[k], cur);
            else k_shadow<R><<<shadow_blocks, threads, 0, s>>>(SP[k]);
            if (timed) {
                cudaEventRecord(z, s);
                ev.note(q == 0 ? GT_KERNEL_GENERATE : q == 1 ? GT_KERNEL_TRACE : q == 2 ? GT_KERNEL_SHADE : GT_KERNEL_SHADOW,
                        a, z);
            }
        }
        return cudaGetLastError();
    };
    auto cleanup = [&]() {}; // the graphs stay cached in the context
    cudaEvent_t init_done = nullptr;
    GT_CUDA(ev.get(init_done));
    GT_CUDA(cudaEventRecord(init_done, st));
    for (uint32_t k = 0; k < K; ++k) {
        // Profile mode issues every launch on the context stream, so launches run one at a
        // time and each kernel's event pair measures that kernel alone.
        S[k].st = profile ? st : ctx->stripe_stream[k];
        S[k].side = profile ? st : ctx->stripe_side[k];
        GT_CUDA(cudaStreamWaitEvent(S[k].st, init_done, 0));
        if (!profile) {
            // Reuse the stripe's graph from the previous render when nothing it captured
            // changed: its key is the stripe's kernel parameters and launch sizes.
            std::vector<unsigned char> key(sizeof(Params<R>) + 4 * sizeof(uint32_t));
            std::memcpy(key.data(), &SP[k], sizeof(Params<R>));
            const uint32_t extra[4] = {lblocks, wblocks, uint32_t(kernels_per_iteration), uint32_t(sizeof(R))};
            std::memcpy(key.data() + sizeof(Params<R>), extra, sizeof(extra));
            gt_context::CachedGraph& cg = ctx->graphs[k];
            if (cg.exec && cg.key == key) {
                S[k].exec = cg.exec;
                continue;
            }
            if (cg.exec) cudaGraphExecDestroy(cg.exec);
            cg.exec = nullptr;
            cg.key.clear();
            cudaGraph_t graph = nullptr;
            GT_CUDA(cudaStreamBeginCapture(S[k].st, cudaStreamCaptureModeThreadLocal));
            cudaError_t le = launch_iteration(k, 0, false);
            if (le == cudaSuccess) le = launch_iteration(k, 1, false);
            cudaError_t ce = cudaStreamEndCapture(S[k].st, &graph);
            if (le != cudaSuccess || ce != cudaSuccess) {
                if (graph) cudaGraphDestroy(graph);
                cleanup();
                return cuda_fail(le != cudaSuccess ? le : ce, "wavefront graph capture");
            }
            ce = cudaGraphInstantiate(&S[k].exec, graph, 0);
            cudaGraphDestroy(graph);
            if (ce != cudaSuccess) {
                S[k].exec = nullptr;
                return cuda_fail(ce, "cudaGraphInstantiate");
            }
            cg.exec = S[k].exec;
            cg.key = std::move(key);
        }
    }

    auto migrate = [&](uint32_t k) -> gt_status {
        Params<R>& Q = SP[k];
        const cudaStream_t s = S[k].st;
        GT_CUDA(cudaMemsetAsync(Q.ps.mstat, 0, 2 * sizeof(unsigned long long), s));
        GT_CUDA(cudaMemsetAsync(Q.ps.counters + C_MIGRATED, 0, 2 * sizeof(uint32_t), s));
        GT_CUDA(cudaMemsetAsync(Q.ps.counters + C_SIDE_DONE, 0, 3 * sizeof(uint32_t), s));
        GT_CUDA(cudaMemsetAsync(Q.ps.counters + C_TRACE1, 0, sizeof(uint32_t), s));
        k_progress_sum<R><<<lblocks, threads, 0, s>>>(Q);
        k_migrate<R><<<lblocks, threads, 0, s>>>(Q, kMigrateRatio);
        k_drop_migrated<R><<<wblocks, threads, 0, s>>>(Q);
        k_restore_queue<R><<<wblocks, threads, 0, s>>>(Q);
        GT_CUDA(cudaGetLastError());
        klaunch[GT_KERNEL_OTHER] += 4;
        GT_CUDA(ev.pair(S[k].fork, S[k].join));
        GT_CUDA(cudaEventRecord(S[k].fork, s));
        GT_CUDA(cudaStreamWaitEvent(S[k].side, S[k].fork, 0));
        HandOff ho;
        ho.done = Q.ps.counters + C_SIDE_DONE;
        ho.below = side_coop_blocks * 4u;
        ho.list = Q.ps.q_handoff;
        ho.count = Q.ps.counters + C_SIDE_COOP;
        k_persistent<R, true, BATCH><<<side_blocks, 128, 0, S[k].side>>>(Q, Q.ps.counters + C_MIGRATE_NEXT, Q.ps.q_migrate,
                                                                   Q.ps.counters + C_MIGRATED, ctx->mapped_dev,
                                                                   nullptr, nullptr, nullptr, nullptr, ho);
        HandOff coop;
        coop.coop = 1;
        k_persistent<R, true, BATCH, false, true><<<side_coop_blocks, 128, 0, S[k].side>>>(
            Q, Q.ps.counters + C_SIDE_COOP_NEXT, Q.ps.q_handoff, Q.ps.counters + C_SIDE_COOP, ctx->mapped_dev, nullptr,
            nullptr, nullptr, nullptr, coop);
        GT_CUDA(cudaGetLastError());
        klaunch[GT_KERNEL_PERSISTENT] += 2;
        GT_CUDA(cudaEventRecord(S[k].join, S[k].side));
        S[k].migrated = true;
        return GT_OK;
    };
    // The last pixels of a stripe are its longest sample chains; once no more than one
    // persistent launch's worth of its slots is left, per-bounce launches would run
    // nearly empty, so the remaining slots finish in k_persistent's RESUME mode: one slot
    // per lane, then one slot per warp for the last ones.
    auto run_tail = [&](uint32_t k) -> gt_status {
        Params<R>& Q = SP[k];
        const cudaStream_t s = S[k].st;
        cudaEvent_t a = nullptr, z = nullptr;
        if (profile) GT_CUDA(ev.pair(a, z));
        if (profile) GT_CUDA(cudaEventRecord(a, s));
        uint32_t* list = Q.ps.q_trace[0];
        uint32_t* count = Q.ps.counters + C_TAIL;
        GT_CUDA(cudaMemsetAsync(count, 0, sizeof(uint32_t), s));
        GT_CUDA(cudaMemsetAsync(Q.ps.counters + C_TAIL_DONE, 0, 3 * sizeof(uint32_t), s));
        GT_CUDA(cudaMemsetAsync(d_next + k, 0, sizeof(uint32_t), s));
        k_collect<R><<<lblocks, threads, 0, s>>>(Q, list, count);
        if (obj_wave) { // the world variant, one slot per lane to the end
            k_persistent<R, true, BATCH, true><<<tblocks, 128, 0, s>>>(Q, d_next + k, list, count, nullptr, nullptr,
                                                                       nullptr, nullptr, nullptr);
            GT_CUDA(cudaGetLastError());
            klaunch[GT_KERNEL_OTHER] += 1;
            klaunch[GT_KERNEL_PERSISTENT] += 1;
            if (profile) {
                GT_CUDA(cudaEventRecord(z, s));
                ev.note(GT_KERNEL_PERSISTENT, a, z);
            }
            S[k].tail = true;
            return GT_OK;
        }
        HandOff ho;
        ho.done = Q.ps.counters + C_TAIL_DONE;
        ho.below = coop_blocks * 4u;
        ho.list = Q.ps.q_trace[1];
        ho.count = Q.ps.counters + C_TAIL_COOP;
        k_persistent<R, true, BATCH><<<tblocks, 128, 0, s>>>(Q, d_next + k, list, count, nullptr, nullptr, nullptr, nullptr,
                                                      nullptr, ho);
        HandOff coop;
        coop.coop = 1;
        k_persistent<R, true, BATCH, false, true><<<coop_blocks, 128, 0, s>>>(
            Q, Q.ps.counters + C_TAIL_COOP_NEXT, Q.ps.q_trace[1], Q.ps.counters + C_TAIL_COOP, nullptr, nullptr, nullptr,
            nullptr, nullptr, coop);
        GT_CUDA(cudaGetLastError());
        klaunch[GT_KERNEL_OTHER] += 1;
        klaunch[GT_KERNEL_PERSISTENT] += 2;
        if (profile) {
            GT_CUDA(cudaEventRecord(z, s));
            ev.note(GT_KERNEL_PERSISTENT, a, z);
        }
        S[k].tail = true;
        return GT_OK;
    };

    const uint32_t limit = limit_max;
    const uint64_t max_iters = uint64_t(limit) * uint64_t(std::max<uint32_t>(depth_max, 1u)) + 8;
    uint64_t iters = 0;
    rc = GT_OK;
    for (uint32_t active = K; active > 0 && rc == GT_OK;) {
        cudaError_t ce = cudaSuccess;
        for (uint32_t k = 0; k < K && ce == cudaSuccess; ++k) {
            if (!S[k].running) continue;
            for (uint32_t i = 0; i < S[k].batch && ce == cudaSuccess; ++i) {
                if (profile) {
                    ce = launch_iteration(k, 0, true);
                    if (ce == cudaSuccess) ce = launch_iteration(k, 1, true);
                } else {
                    ce = cudaGraphLaunch(S[k].exec, S[k].st);
                }
                for (int q = 0; q < kernels_per_iteration; ++q) klaunch[GT_KERNEL_GENERATE + q] += 2;
            }
            S[k].iters += 2ull * S[k].batch;
            iters = std::max(iters, S[k].iters);
            if (ce == cudaSuccess)
                ce = cudaMemcpyAsync(ctx->pinned + 64 + 2 * k, SP[k].ps.counters + C_DONE, 2 * sizeof(uint32_t),
                                     cudaMemcpyDeviceToHost, S[k].st);
        }
        for (uint32_t k = 0; k < K && ce == cudaSuccess; ++k)
            if (S[k].running) ce = cudaStreamSynchronize(S[k].st);
        if (ce != cudaSuccess) {
            rc = cuda_fail(ce, "wavefront launch");
            break;
        }
        if (profile) ev.harvest(kms);
        uint64_t done_all = 0;
        for (uint32_t k = 0; k < K; ++k) {
            const uint32_t local = SP[k].ps.local_n;
            if (!S[k].running) {
                done_all += local;
                continue;
            }
            const uint32_t done = ctx->pinned[64 + 2 * k], err = ctx->pinned[64 + 2 * k + 1];
            done_all += std::min(done, local);
            if (err) {
                rc = fail(GT_ERR_INTERNAL, "traversal stack overflow (BVH deeper than the device stack)");
                break;
            }
            if (done >= local) {
                S[k].running = false;
                --active;
            } else if (local - done <= tail_slots) { // few pixels left: finish them in a persistent launch
                if ((rc = run_tail(k)) != GT_OK) break;
                S[k].running = false;
                --active;
            } else {
                if (may_migrate && !S[k].migrated && S[k].iters >= kMigrateAfter && (rc = migrate(k)) != GT_OK) break;
                if (S[k].iters > max_iters) {
                    rc = fail(GT_ERR_INTERNAL, "wavefront did not terminate within its iteration bound");
                    break;
                }
                S[k].batch = std::min<uint32_t>(S[k].batch * 2, profile ? 8u : 64u);
            }
        }
        if (rc != GT_OK || active == 0) break;
        if (!BATCH && opts.progress && opts.progress_rgb) { // the image as far as it is known
            k_preview<R><<<slot_blocks, threads, 0, st>>>(P, o_rgb);
            klaunch[GT_KERNEL_OTHER] += 1;
            if ((ce = cudaMemcpyAsync(opts.progress_rgb, o_rgb, size_t(n) * 3 * sizeof(float), cudaMemcpyDeviceToHost,
                                      st)) == cudaSuccess)
                ce = cudaStreamSynchronize(st);
            if (ce != cudaSuccess) {
                rc = cuda_fail(ce, "progress image");
                break;
            }
        }
        if (opts.progress && call_progress(ctx, opts, done_all * limit, uint64_t(n) * limit)) {
            rc = fail(GT_ERR_CANCELLED, "render cancelled by the progress callback");
            break;
        }
    }
    cleanup();
    if (rc != GT_OK) {
        ctx->mapped[0] = 1; // the side kernels stop taking slots
        cudaDeviceSynchronize();
        return rc;
    }
    // Join every stripe (and its side stream) before the resolve reads every slot.
    for (uint32_t k = 0; k < K; ++k) {
        cudaEvent_t end = nullptr;
        GT_CUDA(ev.get(end));
        GT_CUDA(cudaEventRecord(end, S[k].st));
        GT_CUDA(cudaStreamWaitEvent(st, end, 0));
        ev.free_events.push_back(end);
        if (S[k].migrated) {
            GT_CUDA(cudaStreamWaitEvent(st, S[k].join, 0));
            ev.note(GT_KERNEL_PERSISTENT, S[k].fork, S[k].join);
        }
    }
    ev.free_events.push_back(init_done);

    {
        cudaEvent_t a = nullptr, z = nullptr;
        if (profile) GT_CUDA(ev.pair(a, z));
        if (profile) GT_CUDA(cudaEventRecord(a, st));
        k_resolve<R, BATCH><<<slot_blocks, threads, 0, st>>>(P, o_rgb, o_rgb64, o_acc);
        GT_CUDA(cudaGetLastError());
        klaunch[GT_KERNEL_OTHER] += 1;
        if (!BATCH && opts.aovs && (o_alb || o_nrm)) {
            k_aov<R><<<slot_blocks, threads, 0, st>>>(P, o_alb, o_nrm);
            GT_CUDA(cudaGetLastError());
            klaunch[GT_KERNEL_OTHER] += 1;
        }
        if (profile) {
            GT_CUDA(cudaEventRecord(z, st));
            ev.note(GT_KERNEL_OTHER, a, z);
        }
    }
    if (accum) {
        k_accum_store<R><<<slot_blocks, threads, 0, st>>>(P, accum->rng, static_cast<R4<R>*>(accum->sum),
                                                          static_cast<R4<R>*>(accum->comp), accum->accepted);
        GT_CUDA(cudaGetLastError());
        klaunch[GT_KERNEL_OTHER] += 1;
    }
    // Per-stripe counters into the frame's: stack overflow flags, migrated and tail pixels.
    Params<R> F = P;
    F.ps.counters = SP[0].ps.counters;
    std::vector<uint32_t> words(size_t(K) * C_COUNT);
    for (uint32_t k = 0; k < K; ++k)
        GT_CUDA(cudaMemcpyAsync(words.data() + size_t(k) * C_COUNT, SP[k].ps.counters, C_COUNT * sizeof(uint32_t),
                                cudaMemcpyDeviceToHost, st));
    if constexpr (BATCH) { // each frame's slice of the batch buffers into its own outputs
        for (uint32_t i = 0; i < bcount; ++i) {
            gt_frame* f = bframes[i];
            const size_t o = bstart[i], np = size_t(bstart[i + 1]) - bstart[i];
            const cudaMemcpyKind kind = f->device_buffers ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
            GT_CUDA(cudaMemcpyAsync(f->rgb, d_rgb + o * 3, np * 3 * sizeof(float), kind, st));
            if (f->rgb64) GT_CUDA(cudaMemcpyAsync(f->rgb64, d_rgb64 + o * 3, np * 3 * sizeof(double), kind, st));
            if (f->accepted) GT_CUDA(cudaMemcpyAsync(f->accepted, d_acc + o, np * sizeof(uint32_t), kind, st));
        }
        rc = finish_render<R>(ctx, F, nullptr, opts, false, n, o_rgb, o_rgb64, o_acc, o_alb, o_nrm, ev, kms, klaunch,
                              iters);
    } else {
        rc = finish_render<R>(ctx, F, frame, opts, host_out, n, o_rgb, o_rgb64, o_acc, o_alb, o_nrm, ev, kms, klaunch,
                              iters);
    }
    if (rc == GT_OK) {
        uint64_t migrated_px = 0, tail_px = 0;
        for (uint32_t k = 0; k < K; ++k) {
            const uint32_t* w = words.data() + size_t(k) * C_COUNT;
            if (w[C_ERROR]) rc = fail(GT_ERR_INTERNAL, "traversal stack overflow (BVH deeper than the device stack)");
            migrated_px += w[C_MIGRATED];
            tail_px += w[C_TAIL];
        }
        if (rc == GT_OK && opts.stats) {
            opts.stats->migrated_pixels = migrated_px;
            opts.stats->tail_pixels = tail_px;
        }
    }
    if (rc == GT_OK && accum) {
        accum->samples += add_samples;
        accum->seed = cam.desc.rng_seed;
    }
    return rc;
}

// Batched frames (many small frames of one scene, each with its own camera, sample count
// and adaptive settings): every frame's pixels in one k_persistent launch in BATCH mode,
// each pixel rendered with its frame's camera.  Pixels are taken in frame order; the
// images equal one gt_render per frame.
template <class R>
gt_status render_batch_impl(gt_scene* s, const gt_lights* l, gt_environment* e, const CamHost* cams, uint32_t count,
                            const gt_render_opts& opts, gt_frame* const* frames) {
    gt_context* ctx = s->ctx;
    cudaStream_t st = ctx->stream;
    gt_status rc;
    if ((rc = upload_scene<R>(s)) != GT_OK) return rc;
    const bool use_lights = l != nullptr;
    const bool use_env = e != nullptr;
    Params<R> P;
    std::memset(&P, 0, sizeof(P));
    P.sc = gpu_of<R>(s).view;
    if (use_lights) {
        if ((rc = upload_lights<R>(const_cast<gt_lights*>(l))) != GT_OK) return rc;
        P.lights = lights_of<R>(const_cast<gt_lights*>(l)).view;
    }
    if (use_env) {
        if ((rc = upload_env<R>(e)) != GT_OK) return rc;
        P.env = env_of<R>(e).view;
    }
    std::vector<CamDev<R>> cd(count);
    std::vector<uint32_t> start(size_t(count) + 1);
    uint64_t total = 0;
    bool want64 = false;
    for (uint32_t i = 0; i < count; ++i) {
        cd[i] = cam_dev<R>(cams[i], use_lights, use_env);
        start[i] = uint32_t(total);
        total += uint64_t(cams[i].width) * cams[i].height;
        if (total >= (1ull << 32)) return fail(GT_ERR_INVALID_ARG, "a batch holds fewer than 2^32 pixels");
        want64 = want64 || frames[i]->rgb64 != nullptr;
    }
    start[count] = uint32_t(total);
    const uint32_t n = uint32_t(total);
    P.cam = cd[0];
    P.num_frames = count;
    P.ps.n = n;

    auto lay = [&](Bump& bb, CamDev<R>** dcams, uint32_t** dstart, uint32_t** next, float** rgb, double** rgb64,
                   uint32_t** acc) {
        *dcams = bb.take<CamDev<R>>(count);
        *dstart = bb.take<uint32_t>(size_t(count) + 1);
        P.ps.counters = bb.take<uint32_t>(C_COUNT);
        P.ps.totals = bb.take<unsigned long long>(8);
        *next = bb.take<uint32_t>(1);
        *rgb = bb.take<float>(size_t(n) * 3);
        *rgb64 = want64 ? bb.take<double>(size_t(n) * 3) : nullptr;
        *acc = bb.take<uint32_t>(size_t(n));
    };
    CamDev<R>* d_cams;
    uint32_t *d_start, *d_next, *d_acc;
    float* d_rgb;
    double* d_rgb64;
    Bump sizing{nullptr};
    lay(sizing, &d_cams, &d_start, &d_next, &d_rgb, &d_rgb64, &d_acc);
    if ((rc = ensure_workspace(ctx, sizing.off + 4096)) != GT_OK) return rc;
    Bump b{static_cast<char*>(ctx->ws)};
    lay(b, &d_cams, &d_start, &d_next, &d_rgb, &d_rgb64, &d_acc);
    P.cams = d_cams;
    P.frame_start = d_start;

    EventPool ev;
    if ((rc = ev.init()) != GT_OK) return rc;
    double kms[GT_KERNEL_COUNT] = {0};
    uint64_t klaunch[GT_KERNEL_COUNT] = {0};
    GT_CUDA(cudaEventRecord(ev.begin, st));
    GT_CUDA(cudaMemcpyAsync(d_cams, cd.data(), cd.size() * sizeof(CamDev<R>), cudaMemcpyHostToDevice, st));
    GT_CUDA(cudaMemcpyAsync(d_start, start.data(), start.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    GT_CUDA(cudaMemsetAsync(P.ps.counters, 0, C_COUNT * sizeof(uint32_t), st));
    GT_CUDA(cudaMemsetAsync(P.ps.totals, 0, 8 * sizeof(unsigned long long), st));
    GT_CUDA(cudaMemsetAsync(d_next, 0, sizeof(uint32_t), st));
    ctx->mapped[0] = 0;
    ctx->mapped[1] = 0;
    int per_sm = 0;
    const bool world = P.sc.num_media != 0 || P.sc.num_objects != 0;
    GT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, world ? k_persistent<R, false, true, true> : k_persistent<R, false, true>, 128, 0));
    const uint32_t sms = uint32_t(ctx->num_sms > 0 ? ctx->num_sms : 1);
    const uint32_t blocks = std::max<uint32_t>(1u, std::min<uint32_t>(sms * uint32_t(std::max(per_sm, 1)), (n + 127) / 128));
    cudaEvent_t a = nullptr, z = nullptr;
    GT_CUDA(ev.pair(a, z));
    GT_CUDA(cudaEventRecord(a, st));
    if (world)
        k_persistent<R, false, true, true><<<blocks, 128, 0, st>>>(P, d_next, nullptr, nullptr, ctx->mapped_dev,
                                                                   ctx->mapped_dev + 1, d_rgb, d_rgb64, d_acc);
    else
        k_persistent<R, false, true><<<blocks, 128, 0, st>>>(P, d_next, nullptr, nullptr, ctx->mapped_dev,
                                                             ctx->mapped_dev + 1, d_rgb, d_rgb64, d_acc);
    GT_CUDA(cudaGetLastError());
    klaunch[GT_KERNEL_PERSISTENT] += 1;
    GT_CUDA(cudaEventRecord(z, st));
    bool cancelled = false;
    if (opts.progress) { // the host polls the mapped pixel counter while the launch runs
        for (;;) {
            cudaError_t q = cudaEventQuery(z);
            if (q == cudaSuccess) break;
            if (q != cudaErrorNotReady) return cuda_fail(q, "batched render");
            struct timespec ts{0, 2000000};
            nanosleep(&ts, nullptr);
            const uint32_t handed = std::min<uint32_t>(uint32_t(ctx->mapped[1]), n);
            if (!cancelled && call_progress(ctx, opts, handed, n)) {
                ctx->mapped[0] = 1;
                cancelled = true;
            }
        }
    }
    ev.note(GT_KERNEL_PERSISTENT, a, z);
    // Each frame's slice of the batch buffers into its own outputs.
    for (uint32_t i = 0; i < count; ++i) {
        gt_frame* f = frames[i];
        const size_t o = start[i], np = size_t(start[i + 1]) - start[i];
        const cudaMemcpyKind kind = f->device_buffers ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
        GT_CUDA(cudaMemcpyAsync(f->rgb, d_rgb + o * 3, np * 3 * sizeof(float), kind, st));
        if (f->rgb64) GT_CUDA(cudaMemcpyAsync(f->rgb64, d_rgb64 + o * 3, np * 3 * sizeof(double), kind, st));
        if (f->accepted) GT_CUDA(cudaMemcpyAsync(f->accepted, d_acc + o, np * sizeof(uint32_t), kind, st));
    }
    GT_CUDA(cudaEventRecord(ev.end, st));
    unsigned long long tot[8];
    GT_CUDA(cudaMemcpyAsync(ctx->pinned + 2, P.ps.totals, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    GT_CUDA(cudaMemcpyAsync(ctx->pinned + 10, P.ps.counters + C_ERROR, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    GT_CUDA(cudaStreamSynchronize(st));
    if (ctx->pinned[10]) return fail(GT_ERR_INTERNAL, "traversal stack overflow (BVH deeper than the device stack)");
    if (cancelled) return fail(GT_ERR_CANCELLED, "render cancelled by the progress callback");
    std::memcpy(tot, ctx->pinned + 2, 4 * sizeof(unsigned long long));
    if (opts.stats) {
        gt_render_stats& o = *opts.stats;
        std::memset(&o, 0, sizeof(o));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev.begin, ev.end);
        o.gpu_ms = ms;
        o.iterations = 1;
        o.rays = tot[0];
        o.shadow_rays = tot[1];
        o.samples = tot[2];
        o.samples_started = tot[3];
        o.persistent_rays = tot[0] + tot[1];
        if (opts.profile) ev.harvest(kms);
        for (int k = 0; k < GT_KERNEL_COUNT; ++k) {
            o.kernel_ms[k] = opts.profile ? kms[k] : 0.0;
            o.kernel_launches[k] = klaunch[k];
        }
    }
    return GT_OK;
}

template <class R>
gt_status trace_impl(gt_scene* s, const double* rays, uint32_t count, double tmin, double tmax, int32_t* ids,
                     double* t, gt_bvh_stats* stats) {
    gt_context* ctx = s->ctx;
    cudaStream_t st = ctx->stream;
    gt_status rc;
    if ((rc = upload_scene<R>(s)) != GT_OK) return rc;
    Bump sizing{nullptr};
    sizing.take<double>(size_t(count) * 7);
    sizing.take<int32_t>(count);
    sizing.take<double>(count);
    sizing.take<unsigned long long>(8);
    if ((rc = ensure_workspace(ctx, sizing.off + 4096)) != GT_OK) return rc;
    Bump b{static_cast<char*>(ctx->ws)};
    double* d_rays = b.take<double>(size_t(count) * 7);
    int32_t* d_ids = b.take<int32_t>(count);
    double* d_t = b.take<double>(count);
    unsigned long long* d_stats = b.take<unsigned long long>(8);
    if (count) GT_CUDA(cudaMemcpyAsync(d_rays, rays, size_t(count) * 7 * sizeof(double), cudaMemcpyHostToDevice, st));
    GT_CUDA(cudaMemsetAsync(d_stats, 0, 8 * sizeof(unsigned long long), st));
    if (count) {
        const uint32_t blocks = std::min<uint32_t>((count + 127) / 128, uint32_t(std::max(ctx->num_sms, 1)) * 8);
        k_trace_rays<R><<<blocks, 128, 0, st>>>(gpu_of<R>(s).view, d_rays, count, tmin, tmax, d_ids, d_t, d_stats,
                                                reinterpret_cast<uint32_t*>(d_stats + 7));
        GT_CUDA(cudaGetLastError());
        GT_CUDA(cudaMemcpyAsync(ids, d_ids, size_t(count) * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
        if (t) GT_CUDA(cudaMemcpyAsync(t, d_t, size_t(count) * sizeof(double), cudaMemcpyDeviceToHost, st));
    }
    unsigned long long h[8];
    GT_CUDA(cudaMemcpyAsync(h, d_stats, sizeof(h), cudaMemcpyDeviceToHost, st));
    GT_CUDA(cudaStreamSynchronize(st));
    if (h[7] & 0xffffffffull) return fail(GT_ERR_INTERNAL, "traversal stack overflow");
    if (stats) {
        stats->rays = count;
        stats->node_bounds_tests = h[0];
        stats->node_bounds_hits = h[1];
        stats->leaf_visits = h[2];
        stats->primitive_candidates = h[3];
        stats->leaf_hit_results = h[4];
        stats->max_stack_depth = h[5];
    }
    return GT_OK;
}

} // namespace gt
