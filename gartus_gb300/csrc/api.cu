// api.cu — the extern "C" boundary of include/gartus_gpu.h: argument validation (the
// reference's assert! panics become GT_ERR_INVALID_ARG), handle lifetimes, camera set-up
// in f64 on the host, and dispatch to the f32 or f64 wavefront.
#include <cmath>
#include <cstddef>
#include <cstring>
#include <initializer_list>
#include <exception>
#include <new>

#include "internal.h"

namespace gt {

namespace {
thread_local std::string g_last_error;
constexpr double kEps = 2.220446049250313e-16;

struct D3 {
    double x, y, z;
};
D3 d3(const double* p) { return D3{p[0], p[1], p[2]}; }
D3 sub(D3 a, D3 b) { return D3{a.x - b.x, a.y - b.y, a.z - b.z}; }
D3 add(D3 a, D3 b) { return D3{a.x + b.x, a.y + b.y, a.z + b.z}; }
D3 mul(D3 a, double s) { return D3{a.x * s, a.y * s, a.z * s}; }
D3 divs(D3 a, double s) { return D3{a.x / s, a.y / s, a.z / s}; }
double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
D3 cross(D3 a, D3 b) { return D3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
D3 normalized(D3 a) { // vector.rs:147-155
    double l = std::sqrt(dot(a, a));
    return l < kEps ? D3{0, 0, 0} : divs(a, l);
}
void put(double* dst, D3 v) {
    dst[0] = v.x;
    dst[1] = v.y;
    dst[2] = v.z;
}
bool finite3(const double* p) { return std::isfinite(p[0]) && std::isfinite(p[1]) && std::isfinite(p[2]); }

uint32_t image_height(const gt_camera_desc& d) { // `(w / aspect) as u32`, then max(1)
    double h = double(d.image_width) / d.aspect_ratio;
    uint32_t v = !(h > 0.0) ? 0u : (h >= 4294967295.0 ? UINT32_MAX : uint32_t(h));
    return v < 1 ? 1 : v;
}

// RayCamera::validate_view (camera.rs:1161-1201) plus the builder clamps.
gt_status validate_camera(const gt_camera_desc& d) {
    if (d.struct_size < sizeof(gt_camera_desc)) return fail(GT_ERR_INVALID_ARG, "camera struct_size too small");
    if (d.image_width == 0) return fail(GT_ERR_INVALID_ARG, "image width must be positive");
    if (!std::isfinite(d.aspect_ratio) || !(d.aspect_ratio > 0.0))
        return fail(GT_ERR_INVALID_ARG, "aspect ratio must be positive and finite");
    if (!std::isfinite(d.vertical_fov) || !(0.0 < d.vertical_fov && d.vertical_fov < 180.0))
        return fail(GT_ERR_INVALID_ARG, "vertical field of view must be finite and in 0..180 degrees");
    D3 w = sub(d3(d.lookfrom), d3(d.lookat));
    if (!(dot(w, w) > kEps)) return fail(GT_ERR_INVALID_ARG, "lookfrom and lookat must be distinct");
    D3 vup = d3(d.view_up);
    if (!(dot(vup, vup) > kEps)) return fail(GT_ERR_INVALID_ARG, "view-up vector must be nonzero");
    D3 fwd = normalized(sub(d3(d.lookat), d3(d.lookfrom)));
    D3 right = normalized(cross(fwd, vup));
    if (dot(fwd, fwd) <= kEps || dot(right, right) <= kEps)
        return fail(GT_ERR_INVALID_ARG, "view-up vector must not be parallel to the viewing direction");
    if (!std::isfinite(d.defocus_angle) || !(d.defocus_angle >= 0.0 && d.defocus_angle < 180.0))
        return fail(GT_ERR_INVALID_ARG, "defocus angle must be finite and in 0..180 degrees");
    if (!std::isfinite(d.focus_distance) || !(d.focus_distance > 0.0))
        return fail(GT_ERR_INVALID_ARG, "focus distance must be positive and finite");
    if (!std::isfinite(d.shutter_start) || !std::isfinite(d.shutter_end) || !(d.shutter_start <= d.shutter_end))
        return fail(GT_ERR_INVALID_ARG, "shutter interval must be finite and ordered");
    if (d.background_kind > GT_BG_VERTICAL_GRADIENT)
        return fail(GT_ERR_UNSUPPORTED, "only constant and vertical-gradient backgrounds cross the ABI");
    for (int i = 0; i < 9; ++i)
        if (!std::isfinite(d.background[i])) return fail(GT_ERR_INVALID_ARG, "background color components must be finite");
    if (d.pixel_sample_mode > GT_SAMPLE_STRATIFIED_GRID) return fail(GT_ERR_INVALID_ARG, "unknown pixel sample mode");
    if (d.direct_lighting_mode > GT_DIRECT_NEXT_EVENT_ESTIMATION)
        return fail(GT_ERR_INVALID_ARG, "unknown direct lighting mode");
    if (!std::isfinite(d.light_pdf_weight)) return fail(GT_ERR_INVALID_ARG, "light PDF weight must be finite");
    if (d.adaptive && (!std::isfinite(d.adaptive_error_threshold) || !(d.adaptive_error_threshold > 0.0)))
        return fail(GT_ERR_INVALID_ARG, "adaptive sampling error threshold must be positive and finite");
    uint64_t pixels = uint64_t(d.image_width) * image_height(d);
    if (pixels > (1ull << 30)) return fail(GT_ERR_INVALID_ARG, "image is too large");
    return GT_OK;
}

// RayCamera::initialized (camera.rs:1068-1130), in f64.
CamHost init_camera(const gt_camera_desc& d, bool env) {
    CamHost c;
    std::memset(&c, 0, sizeof(c));
    c.desc = d;
    c.desc.samples_per_pixel = d.samples_per_pixel < 1 ? 1 : d.samples_per_pixel;
    c.width = d.image_width;
    c.height = image_height(d);
    const double pi = 3.141592653589793;
    double theta = d.vertical_fov * pi / 180.0;
    double h = std::tan(theta * 0.5);
    double vh = 2.0 * h * d.focus_distance;
    double vw = vh * (double(d.image_width) / double(c.height));
    D3 center = d3(d.lookfrom);
    D3 fwd = normalized(sub(d3(d.lookat), center)); // CameraBasis::looking_at, geometry.rs:23-37
    D3 right = normalized(cross(fwd, d3(d.view_up)));
    D3 up = cross(right, fwd);
    D3 w = D3{-fwd.x, -fwd.y, -fwd.z};
    D3 vu = mul(right, vw);
    D3 vv = mul(D3{-up.x, -up.y, -up.z}, vh);
    D3 pdu = divs(vu, double(d.image_width));
    D3 pdv = divs(vv, double(c.height));
    D3 ul = sub(sub(sub(center, mul(w, d.focus_distance)), divs(vu, 2.0)), divs(vv, 2.0));
    D3 p00 = add(ul, mul(add(pdu, pdv), 0.5));
    double dr = d.focus_distance * std::tan((d.defocus_angle * 0.5) * pi / 180.0);
    put(c.center, center);
    put(c.pixel00, p00);
    put(c.du, pdu);
    put(c.dv, pdv);
    put(c.ddu, mul(right, dr));
    put(c.ddv, mul(up, dr));
    // Samples the loops run (effective_samples_per_pixel, camera.rs:1547-1556) and the
    // stratified grid (camera.rs:1706-1708, 3028-3034); a zero grid width is clamped to 1
    // as RayCamera::with_stratified_grid_width does.
    if (d.pixel_sample_mode == GT_SAMPLE_RANDOM) {
        c.grid = 1;
        c.spp = c.desc.samples_per_pixel;
    } else if (d.pixel_sample_mode == GT_SAMPLE_STRATIFIED) {
        double r = std::sqrt(double(c.desc.samples_per_pixel));
        uint32_t g = !(r > 0.0) ? 0u : uint32_t(r);
        c.grid = g < 1 ? 1 : g;
        c.spp = c.grid * c.grid;
    } else {
        c.grid = d.grid_width < 1 ? 1 : d.grid_width;
        c.spp = c.grid * c.grid;
    }
    // The environment entry points switch to next-event estimation
    // (environment_importance_camera, camera.rs:4171-4173).
    c.nee = d.direct_lighting_mode == GT_DIRECT_NEXT_EVENT_ESTIMATION || env;
    c.light_pdf_weight = c.nee ? 0.0 : std::fmin(std::fmax(d.light_pdf_weight, 0.0), 1.0);
    return c;
}

gt_status validate_geometry(const gt_geometry& g) {
    if (g.kind > GT_GEOM_QUAD) return fail(GT_ERR_INVALID_ARG, "unknown geometry kind");
    for (int i = 0; i < 9; ++i)
        if (!std::isfinite(g.p[i])) return fail(GT_ERR_INVALID_ARG, "geometry parameters must be finite");
    return GT_OK;
}

} // namespace

void set_error(const std::string& msg) { g_last_error = msg; }
CamHost camera_setup(const gt_camera_desc& d, bool env) { return init_camera(d, env); }
gt_status fail(gt_status status, const std::string& msg) {
    g_last_error = msg;
    return status;
}
gt_status ensure_reference_bvh(gt_scene* s) {
    if (s->bvh_ready) return GT_OK;
    build_reference_bvh(s->prims.data(), uint32_t(s->prims.size()), s->leaf_size, s->bvh);
    if (s->bvh.max_depth + 1 > 62) return fail(GT_ERR_UNSUPPORTED, "BVH deeper than the device traversal stack");
    s->bvh_ready = true;
    return GT_OK;
}

gt_status cuda_fail(cudaError_t e, const char* what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? GT_ERR_OOM : GT_ERR_CUDA;
}

} // namespace gt

using namespace gt;

extern "C" {

uint32_t gt_abi_version(void) { return GT_ABI_VERSION; }

const char* gt_last_error(void) { return g_last_error.c_str(); }

gt_status gt_camera_default(uint32_t image_width, double aspect_ratio, gt_camera_desc* c) {
    if (!c) return fail(GT_ERR_INVALID_ARG, "null camera");
    if (image_width == 0) return fail(GT_ERR_INVALID_ARG, "image width must be positive");
    if (!std::isfinite(aspect_ratio) || !(aspect_ratio > 0.0))
        return fail(GT_ERR_INVALID_ARG, "aspect ratio must be positive and finite");
    std::memset(c, 0, sizeof(*c));
    c->struct_size = sizeof(gt_camera_desc);
    c->image_width = image_width;
    c->aspect_ratio = aspect_ratio;
    c->samples_per_pixel = 1;
    c->pixel_sample_mode = GT_SAMPLE_RANDOM;
    c->grid_width = 1;
    c->direct_lighting_mode = GT_DIRECT_CURRENT_PATH_CONTINUATION;
    c->light_pdf_weight = 0.5;
    c->max_depth = 10;
    c->russian_roulette_min_depth = 5;
    c->rng_seed = 1;
    c->vertical_fov = 90.0;
    c->lookat[2] = -1.0;
    c->view_up[1] = 1.0;
    c->focus_distance = 1.0;
    c->shutter_end = 1.0;
    c->background_kind = GT_BG_CONSTANT;
    c->background[0] = 0.70;
    c->background[1] = 0.80;
    c->background[2] = 1.00;
    return GT_OK;
}

gt_status gt_camera_image_size(const gt_camera_desc* c, uint32_t* w, uint32_t* h, uint32_t* spp) {
    if (!c) return fail(GT_ERR_INVALID_ARG, "null camera");
    gt_status rc = validate_camera(*c);
    if (rc != GT_OK) return rc;
    CamHost ch = init_camera(*c, false);
    if (w) *w = ch.width;
    if (h) *h = ch.height;
    if (spp) *spp = ch.spp;
    return GT_OK;
}

gt_status gt_context_create(int device, gt_context** out) {
    GT_GUARD_BEGIN
    if (!out) return fail(GT_ERR_INVALID_ARG, "null output handle");
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        cudaGetLastError();
        return fail(GT_ERR_NO_DEVICE, "no CUDA device available");
    }
    if (device < 0 || device >= count) return fail(GT_ERR_INVALID_ARG, "device index out of range");
    e = cudaSetDevice(device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    auto* ctx = new gt_context();
    ctx->device = device;
    cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking);
    for (int k = 0; k < gt_context::kMaxStripes && e == cudaSuccess; ++k) {
        e = cudaStreamCreateWithFlags(&ctx->stripe_stream[k], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stripe_side[k], cudaStreamNonBlocking);
    }
    if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&ctx->pinned), 1024);
    void* mapped = nullptr;
    if (e == cudaSuccess) e = cudaHostAlloc(&mapped, 64, cudaHostAllocMapped);
    if (e == cudaSuccess) {
        std::memset(mapped, 0, 64);
        ctx->mapped = static_cast<volatile uint32_t*>(mapped);
        e = cudaHostGetDevicePointer(reinterpret_cast<void**>(&ctx->mapped_dev), mapped, 0);
    }
    if (e != cudaSuccess) {
        if (ctx->stream) cudaStreamDestroy(ctx->stream);
        if (ctx->side) cudaStreamDestroy(ctx->side);
        for (int k = 0; k < gt_context::kMaxStripes; ++k) {
            if (ctx->stripe_stream[k]) cudaStreamDestroy(ctx->stripe_stream[k]);
            if (ctx->stripe_side[k]) cudaStreamDestroy(ctx->stripe_side[k]);
        }
        if (ctx->pinned) cudaFreeHost(ctx->pinned);
        if (ctx->mapped) cudaFreeHost(const_cast<uint32_t*>(ctx->mapped));
        delete ctx;
        return cuda_fail(e, "context creation");
    }
    *out = ctx;
    return GT_OK;
    GT_GUARD_END
}

void gt_context_destroy(gt_context* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaDeviceSynchronize();
    for (auto& g : ctx->graphs)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    cudaFree(ctx->ws);
    cudaFreeHost(ctx->pinned);
    cudaFreeHost(const_cast<uint32_t*>(ctx->mapped));
    cudaStreamDestroy(ctx->stream);
    cudaStreamDestroy(ctx->side);
    for (int k = 0; k < gt_context::kMaxStripes; ++k) {
        cudaStreamDestroy(ctx->stripe_stream[k]);
        cudaStreamDestroy(ctx->stripe_side[k]);
    }
    delete ctx;
}

gt_status gt_scene_create(gt_context* ctx, const gt_scene_desc* d, gt_scene** out) {
    GT_GUARD_BEGIN
    if (!ctx || !d || !out) return fail(GT_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    if (d->struct_size < sizeof(gt_scene_desc)) return fail(GT_ERR_INVALID_ARG, "scene struct_size too small");
    if ((d->num_primitives && !d->primitives) || (d->num_materials && !d->materials) || (d->num_images && !d->images))
        return fail(GT_ERR_INVALID_ARG, "null primitive, material or image array");
    if (d->num_primitives > (1u << 28)) return fail(GT_ERR_INVALID_ARG, "too many primitives");
    for (uint32_t i = 0; i < d->num_materials; ++i) {
        const gt_material& m = d->materials[i];
        if (m.kind > GT_MAT_HENYEY_GREENSTEIN) return fail(GT_ERR_INVALID_ARG, "unknown material kind");
        if (m.texture_kind > GT_TEX_IMAGE) return fail(GT_ERR_INVALID_ARG, "unknown texture kind");
        if (m.texture_kind == GT_TEX_IMAGE) {
            const double k = m.tex[0];
            if (!(k >= 0.0 && k < double(d->num_images)) || k != std::floor(k))
                return fail(GT_ERR_INVALID_ARG, "image texture index out of range");
        }
        if (m.texture_kind == GT_TEX_NOISE) {
            const double v = m.tex[1], depth = m.tex[2], lo = m.tex[3], hi = m.tex[4];
            if (!std::isfinite(m.tex[0]) || !(v == 0.0 || v == 1.0 || v == 2.0) || !(depth >= 0.0 && depth <= 64.0) ||
                depth != std::floor(depth) || !(lo >= 0.0 && lo < 4294967296.0) || lo != std::floor(lo) ||
                !(hi >= 0.0 && hi < 4294967296.0) || hi != std::floor(hi))
                return fail(GT_ERR_INVALID_ARG, "noise texture needs a finite scale, variant 0-2, integer depth "
                                                "0-64 and a seed split into two 32-bit halves");
        }
        if (!finite3(m.color) || !std::isfinite(m.param)) return fail(GT_ERR_INVALID_ARG, "material values must be finite");
        if (m.kind == GT_MAT_DIELECTRIC && !(m.param > 0.0))
            return fail(GT_ERR_INVALID_ARG, "refractive index must be positive and finite");
        if (m.kind == GT_MAT_HENYEY_GREENSTEIN && !(std::fabs(m.param) < 1.0)) // material.rs:1334-1343
            return fail(GT_ERR_INVALID_ARG, "Henyey-Greenstein anisotropy must be finite and in (-1, 1)");
        if (m.normal_map) { // only Lambertian and GgxMicrofacet carry one (material.rs:456-460, 1505-1520)
            if (m.normal_map > d->num_images || !(m.kind == GT_MAT_LAMBERTIAN || m.kind == GT_MAT_GGX) ||
                !std::isfinite(m.normal_map_strength) || m.normal_map_flags > GT_NORMAL_MAP_NEGATIVE_Y)
                return fail(GT_ERR_INVALID_ARG, "a normal map needs an image index, a Lambertian or GGX material, "
                                                "a finite strength and flags 0-1");
        }
    }
    if ((d->num_meshes && !d->meshes) || (d->num_objects && !d->objects))
        return fail(GT_ERR_INVALID_ARG, "null mesh or object array");
    for (uint32_t k = 0; k < d->num_meshes; ++k) {
        const gt_mesh& mh = d->meshes[k];
        if (mh.num_primitives && !mh.primitives) return fail(GT_ERR_INVALID_ARG, "null mesh primitives");
        if (mh.num_primitives > (1u << 28)) return fail(GT_ERR_INVALID_ARG, "too many mesh primitives");
        for (uint32_t i = 0; i < mh.num_primitives; ++i) {
            gt_status rc = validate_geometry(mh.primitives[i].geometry);
            if (rc != GT_OK) return rc;
            if (mh.primitives[i].material >= d->num_materials)
                return fail(GT_ERR_INVALID_ARG, "mesh material id out of bounds");
        }
        const size_t nuv = mh.texcoords ? size_t(mh.num_primitives) * 6 : 0, nvn = mh.normals ? size_t(mh.num_primitives) * 9 : 0;
        for (size_t i = 0; i < nuv; ++i)
            if (!std::isfinite(mh.texcoords[i])) return fail(GT_ERR_INVALID_ARG, "mesh texture coordinates must be finite");
        for (size_t i = 0; i < nvn; ++i)
            if (!std::isfinite(mh.normals[i])) return fail(GT_ERR_INVALID_ARG, "mesh vertex normals must be finite");
    }
    for (uint32_t k = 0; k < d->num_objects; ++k) {
        const gt_object& o = d->objects[k];
        if (o.mesh >= d->num_meshes || o.transformed > 1) return fail(GT_ERR_INVALID_ARG, "object needs a mesh index and transformed 0-1");
        for (int a = 0; a < 16; ++a)
            if (o.transformed && !(std::isfinite(o.transform[a]) && std::isfinite(o.inverse[a])))
                return fail(GT_ERR_INVALID_ARG, "object matrices must be finite");
    }
    if (d->num_media && !d->media) return fail(GT_ERR_INVALID_ARG, "null media array");
    if (d->num_media > kMaxMedia) return fail(GT_ERR_INVALID_ARG, "at most 64 media per scene");
    for (uint32_t i = 0; i < d->num_media; ++i) {
        const gt_medium& m = d->media[i];
        bool finite = std::isfinite(m.rotate_y) && finite3(m.translate);
        for (int k = 0; k < 6; ++k) finite = finite && std::isfinite(m.p[k]);
        if (m.shape > GT_MEDIUM_BOX || m.transform > (GT_MEDIUM_ROTATE_Y | GT_MEDIUM_TRANSLATE) || !finite)
            return fail(GT_ERR_INVALID_ARG, "medium needs shape 0-1, transform bits 0-3 and finite values");
        if (!(std::isfinite(m.density) && m.density > 0.0)) // medium.rs:93-96
            return fail(GT_ERR_INVALID_ARG, "medium density must be positive and finite");
        if (m.material >= d->num_materials) return fail(GT_ERR_INVALID_ARG, "medium material id out of bounds");
    }
    for (uint32_t i = 0; i < d->num_primitives; ++i) {
        gt_status rc = validate_geometry(d->primitives[i].geometry);
        if (rc != GT_OK) return rc;
        if (d->primitives[i].material >= d->num_materials)
            return fail(GT_ERR_INVALID_ARG, "ray scene material id out of bounds"); // scene.rs:1158-1161
    }
    GT_CONTEXT_LOCK(ctx);
    const uint32_t builder = d->struct_size >= sizeof(gt_scene_desc) ? d->bvh_builder : 0u;
    if (builder > GT_BVH_GPU_LBVH) return fail(GT_ERR_INVALID_ARG, "unknown BVH builder");
    if (d->f32_tree > GT_F32_TREE_BINARY) return fail(GT_ERR_INVALID_ARG, "unknown f32 tree");
    auto* s = new gt_scene();
    s->ctx = ctx;
    s->f32_tree = d->f32_tree;
    s->prims.assign(d->primitives, d->primitives + d->num_primitives);
    s->mats.assign(d->materials, d->materials + d->num_materials);
    s->bvh_builder = builder;
    s->media.assign(d->media, d->media + d->num_media);
    s->objects.assign(d->objects, d->objects + d->num_objects);
    for (uint32_t k = 0; k < d->num_meshes; ++k) { // TriangleBvh::build (mesh.rs:645-652)
        const gt_mesh& mh = d->meshes[k];
        MeshHost m;
        const size_t n = mh.num_primitives;
        m.prims.assign(mh.primitives, mh.primitives + n);
        if (mh.texcoords) m.uv.assign(mh.texcoords, mh.texcoords + n * 6);
        if (mh.normals) m.vn.assign(mh.normals, mh.normals + n * 9);
        m.attr.resize(n);
        for (size_t i = 0; i < n; ++i) {
            const uint8_t given = uint8_t((mh.texcoords ? 1 : 0) | (mh.normals ? 2 : 0));
            m.attr[i] = mh.attribute_flags ? uint8_t(mh.attribute_flags[i] & given) : given;
        }
        m.leaf_size = mh.bvh_leaf_size ? mh.bvh_leaf_size : 4u;
        build_reference_bvh(m.prims.data(), uint32_t(n), m.leaf_size, m.bvh);
        if (m.bvh.max_depth + 1 > 62) {
            delete s;
            return fail(GT_ERR_UNSUPPORTED, "mesh BVH deeper than the device traversal stack");
        }
        s->meshes.push_back(std::move(m));
    }
    for (uint32_t i = 0; i < d->num_images; ++i) {
        const gt_image& g = d->images[i];
        const uint64_t texels = uint64_t(g.width) * g.height;
        if (g.filter > GT_FILTER_LINEAR || g.wrap_s > GT_WRAP_REPEAT || g.wrap_t > GT_WRAP_REPEAT ||
            texels > (1ull << 28) || (texels && !g.rgb)) {
            delete s;
            return fail(GT_ERR_INVALID_ARG, "image needs filter and wrap modes 0-1, at most 2^28 texels and its data");
        }
        ImageHost im;
        im.w = texels ? g.width : 0u;
        im.h = texels ? g.height : 0u;
        im.filter = g.filter;
        im.wrap_s = g.wrap_s;
        im.wrap_t = g.wrap_t;
        if (texels) im.rgb.assign(g.rgb, g.rgb + texels * 3);
        s->images.push_back(std::move(im));
    }
    s->leaf_size = d->bvh_leaf_size ? d->bvh_leaf_size : 4u;
    if (builder == GT_BVH_REFERENCE_SAH) {
        const gt_status rc = ensure_reference_bvh(s);
        if (rc != GT_OK) {
            delete s;
            return rc;
        }
    }
    *out = s;
    return GT_OK;
    GT_GUARD_END
}

void gt_scene_destroy(gt_scene* s) {
    if (!s) return;
    gt::destroy_or_defer(s->ctx, [s] {
        cudaSetDevice(s->ctx->device);
        cudaStreamSynchronize(s->ctx->stream);
        free_gpu_f32(s);
        free_gpu_f64(s);
        delete s;
    });
}

gt_status gt_scene_update_primitives(gt_scene* s, uint32_t first, uint32_t count, const gt_primitive* prims) {
    GT_GUARD_BEGIN
    if (!s || (count && !prims)) return fail(GT_ERR_INVALID_ARG, "null argument");
    if (uint64_t(first) + count > s->prims.size()) return fail(GT_ERR_INVALID_ARG, "primitive range out of bounds");
    for (uint32_t i = 0; i < count; ++i) {
        gt_status rc = validate_geometry(prims[i].geometry);
        if (rc != GT_OK) return rc;
        if (prims[i].material >= s->mats.size())
            return fail(GT_ERR_INVALID_ARG, "ray scene material id out of bounds"); // scene.rs:1158-1161
    }
    GT_CONTEXT_LOCK(s->ctx);
    cudaError_t ce = cudaSetDevice(s->ctx->device);
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaSetDevice");
    ce = cudaStreamSynchronize(s->ctx->stream); // no render of this context still reads the old data
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamSynchronize");
    std::copy(prims, prims + count, s->prims.begin() + first);
    // The reference tree is rebuilt when next needed (the f64 path, statistics, the
    // reference builder's f32 path); a GPU-built f32 tree is refitted now.
    s->bvh_ready = false;
    free_gpu_f64(s);
    gt_status rc = update_f32(s, first, count);
    if (rc != GT_OK) {
        free_gpu_f32(s);
        return rc;
    }
    if (s->bvh_builder == GT_BVH_REFERENCE_SAH) return ensure_reference_bvh(s);
    return GT_OK;
    GT_GUARD_END
}

gt_status gt_scene_bvh_node_count(const gt_scene* s, uint32_t* count) {
    GT_GUARD_BEGIN
    if (!s || !count) return fail(GT_ERR_INVALID_ARG, "null argument");
    gt_scene* m = const_cast<gt_scene*>(s);
    GT_CONTEXT_LOCK(m->ctx);
    const gt_status rc = ensure_reference_bvh(m);
    if (rc != GT_OK) return rc;
    *count = uint32_t(s->bvh.nodes.size());
    return GT_OK;
    GT_GUARD_END
}

gt_status gt_scene_emissive_targets(const gt_scene* s, gt_light_target* targets, uint32_t capacity, uint32_t* count) {
    if (!s || !count) return fail(GT_ERR_INVALID_ARG, "null argument");
    uint32_t n = 0;
    for (const gt_primitive& p : s->prims) {
        if (s->mats[p.material].kind != GT_MAT_DIFFUSE_LIGHT) continue; // RayMaterial::is_emissive
        if (targets && n < capacity) {
            targets[n].geometry = p.geometry;
            targets[n].weight = 1.0;
        }
        ++n;
    }
    *count = n;
    return GT_OK;
}

gt_status gt_lights_create(gt_context* ctx, const gt_light_target* t, uint32_t count, gt_lights** out) {
    GT_GUARD_BEGIN
    if (!ctx || !out || (count && !t)) return fail(GT_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    double total = 0.0;
    for (uint32_t i = 0; i < count; ++i) { // add_target_weighted, scene.rs:460-476
        gt_status rc = validate_geometry(t[i].geometry);
        if (rc != GT_OK) return rc;
        if (!std::isfinite(t[i].weight) || !(t[i].weight > 0.0))
            return fail(GT_ERR_INVALID_ARG, "sampling target weight must be finite and positive");
        total = total + t[i].weight;
        if (!std::isfinite(total)) return fail(GT_ERR_INVALID_ARG, "sampling target total weight must remain finite");
    }
    auto* l = new gt_lights();
    l->ctx = ctx;
    l->targets.assign(t, t + count);
    l->total = total;
    *out = l;
    return GT_OK;
    GT_GUARD_END
}

void gt_lights_destroy(gt_lights* l) {
    if (!l) return;
    gt::destroy_or_defer(l->ctx, [l] {
        cudaSetDevice(l->ctx->device);
        cudaStreamSynchronize(l->ctx->stream);
        free_lights_f32(l);
        free_lights_f64(l);
        delete l;
    });
}

gt_status gt_environment_create(gt_context* ctx, const gt_environment_desc* d, gt_environment** out) {
    GT_GUARD_BEGIN
    if (!ctx || !d || !out) return fail(GT_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    if (d->struct_size < sizeof(gt_environment_desc)) return fail(GT_ERR_INVALID_ARG, "environment struct_size too small");
    if (d->format > GT_ENV_RGB32F) return fail(GT_ERR_INVALID_ARG, "unknown environment format");
    if (d->width == 0 || d->height == 0 || !d->texels) return fail(GT_ERR_INVALID_ARG, "empty environment image");
    if (uint64_t(d->width) * d->height > (1ull << 27)) return fail(GT_ERR_INVALID_ARG, "environment image too large");
    GT_CONTEXT_LOCK(ctx);
    auto* e = new gt_environment();
    e->ctx = ctx;
    e->format = d->format;
    e->width = d->width;
    e->height = d->height;
    const size_t n = size_t(d->width) * d->height;
    if (d->format == GT_ENV_SRGB8) {
        const uint8_t* p = static_cast<const uint8_t*>(d->texels);
        e->px8.assign(p, p + n * 3);
    } else {
        const float* p = static_cast<const float*>(d->texels);
        e->px32.assign(p, p + n * 3);
        for (float v : e->px32)
            if (!std::isfinite(v)) {
                delete e;
                return fail(GT_ERR_INVALID_ARG, "environment texels must be finite");
            }
    }
    // EnvironmentLight::rebuild_distribution (environment.rs:155-185): weight =
    // max(luminance(texel), 0) * sin(theta at the row centre), running-sum CDF.
    const double pi = 3.141592653589793;
    e->weights.reserve(n);
    e->cdf.reserve(n);
    for (uint32_t y = 0; y < d->height; ++y) {
        double theta = pi * ((double(y) + 0.5) / double(d->height));
        double s = std::fmax(std::sin(theta), 0.0);
        for (uint32_t x = 0; x < d->width; ++x) {
            size_t i = (size_t(y) * d->width + x) * 3;
            double c[3];
            for (int k = 0; k < 3; ++k) {
                if (d->format == GT_ENV_SRGB8) {
                    double v = double(e->px8[i + k]) / 255.0;
                    c[k] = v * v;
                } else {
                    c[k] = double(e->px32[i + k]);
                }
            }
            double lum = 0.2126 * c[0] + 0.7152 * c[1] + 0.0722 * c[2];
            double w = std::fmax(lum, 0.0) * s;
            e->total += w;
            e->weights.push_back(w);
            e->cdf.push_back(e->total);
        }
    }
    cudaSetDevice(ctx->device);
    cudaError_t ce;
    if (d->format == GT_ENV_SRGB8) {
        ce = cudaMalloc(&e->d_px8, n * 3);
        if (ce == cudaSuccess) ce = cudaMemcpy(e->d_px8, e->px8.data(), n * 3, cudaMemcpyHostToDevice);
    } else {
        ce = cudaMalloc(&e->d_px32, n * 3 * sizeof(float));
        if (ce == cudaSuccess) ce = cudaMemcpy(e->d_px32, e->px32.data(), n * 3 * sizeof(float), cudaMemcpyHostToDevice);
    }
    if (ce != cudaSuccess) {
        cudaFree(e->d_px8);
        cudaFree(e->d_px32);
        delete e;
        return cuda_fail(ce, "environment upload");
    }
    *out = e;
    return GT_OK;
    GT_GUARD_END
}

void gt_environment_destroy(gt_environment* e) {
    if (!e) return;
    gt::destroy_or_defer(e->ctx, [e] {
        cudaSetDevice(e->ctx->device);
        cudaStreamSynchronize(e->ctx->stream);
        free_env_f32(e);
        free_env_f64(e);
        cudaFree(e->d_px8);
        cudaFree(e->d_px32);
        delete e;
    });
}

// ------------------------------------------------------------ accumulators
namespace {
size_t accum_scalar(uint32_t precision) { return precision == GT_PRECISION_F64 ? sizeof(double) : sizeof(float); }
// Checkpoint blob: header, then rng[n], sum[n], comp[n] (4 scalars each), accepted[n].
struct AccumHeader {
    uint32_t magic, version, width, height, precision, samples;
    uint64_t seed;
};
constexpr uint32_t kAccumMagic = 0x47544143u; // "GTAC"
uint64_t accum_payload(const gt_accumulator* a) {
    const uint64_t n = uint64_t(a->width) * a->height;
    return n * (sizeof(uint64_t) + 8 * accum_scalar(a->precision) + sizeof(uint32_t));
}
} // namespace

gt_status gt_accumulator_create(gt_context* ctx, uint32_t width, uint32_t height, uint32_t precision,
                                gt_accumulator** out) {
    GT_GUARD_BEGIN
    if (!ctx || !out) return fail(GT_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    if (width == 0 || height == 0 || uint64_t(width) * height > (1ull << 31))
        return fail(GT_ERR_INVALID_ARG, "accumulator size must be positive and at most 2^31 pixels");
    if (precision > GT_PRECISION_F64) return fail(GT_ERR_INVALID_ARG, "unknown precision");
    GT_CONTEXT_LOCK(ctx);
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    auto* a = new gt_accumulator();
    a->ctx = ctx;
    a->width = width;
    a->height = height;
    a->precision = precision;
    const size_t n = size_t(width) * height, r4 = 4 * accum_scalar(precision);
    e = cudaMalloc(&a->rng, n * sizeof(uint64_t));
    if (e == cudaSuccess) e = cudaMalloc(&a->sum, n * r4);
    if (e == cudaSuccess) e = cudaMalloc(&a->comp, n * r4);
    if (e == cudaSuccess) e = cudaMalloc(&a->accepted, n * sizeof(uint32_t));
    if (e != cudaSuccess) {
        cudaFree(a->rng);
        cudaFree(a->sum);
        cudaFree(a->comp);
        cudaFree(a->accepted);
        delete a;
        return cuda_fail(e, "accumulator allocation");
    }
    *out = a;
    return GT_OK;
    GT_GUARD_END
}

void gt_accumulator_destroy(gt_accumulator* a) {
    if (!a) return;
    gt::destroy_or_defer(a->ctx, [a] {
        cudaSetDevice(a->ctx->device);
        cudaStreamSynchronize(a->ctx->stream);
        cudaFree(a->rng);
        cudaFree(a->sum);
        cudaFree(a->comp);
        cudaFree(a->accepted);
        delete a;
    });
}

gt_status gt_accumulator_samples(const gt_accumulator* a, uint32_t* samples) {
    if (!a || !samples) return fail(GT_ERR_INVALID_ARG, "null argument");
    *samples = a->samples;
    return GT_OK;
}

gt_status gt_accumulator_save(const gt_accumulator* a, void* host, uint64_t capacity, uint64_t* size) {
    GT_GUARD_BEGIN
    if (!a || !size) return fail(GT_ERR_INVALID_ARG, "null argument");
    const uint64_t need = sizeof(AccumHeader) + accum_payload(a);
    *size = need;
    if (!host) return GT_OK;
    if (capacity < need) return fail(GT_ERR_INVALID_ARG, "checkpoint buffer too small");
    GT_CONTEXT_LOCK(a->ctx);
    cudaError_t e = cudaSetDevice(a->ctx->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    AccumHeader h{kAccumMagic, 1u, a->width, a->height, a->precision, a->samples, a->seed};
    auto* p = static_cast<char*>(host);
    std::memcpy(p, &h, sizeof(h));
    p += sizeof(h);
    const size_t n = size_t(a->width) * a->height, r4 = 4 * accum_scalar(a->precision);
    const void* src[4] = {a->rng, a->sum, a->comp, a->accepted};
    const size_t bytes[4] = {n * sizeof(uint64_t), n * r4, n * r4, n * sizeof(uint32_t)};
    for (int k = 0; k < 4; ++k) {
        e = cudaMemcpy(p, src[k], bytes[k], cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(e, "checkpoint copy");
        p += bytes[k];
    }
    return GT_OK;
    GT_GUARD_END
}

gt_status gt_accumulator_load(gt_accumulator* a, const void* host, uint64_t size) {
    GT_GUARD_BEGIN
    if (!a || !host) return fail(GT_ERR_INVALID_ARG, "null argument");
    AccumHeader h;
    if (size < sizeof(h)) return fail(GT_ERR_INVALID_ARG, "checkpoint too small");
    std::memcpy(&h, host, sizeof(h));
    if (h.magic != kAccumMagic || h.version != 1u) return fail(GT_ERR_INVALID_ARG, "not an accumulator checkpoint");
    if (h.width != a->width || h.height != a->height || h.precision != a->precision)
        return fail(GT_ERR_INVALID_ARG, "checkpoint size or precision differs from the accumulator's");
    if (size < sizeof(h) + accum_payload(a)) return fail(GT_ERR_INVALID_ARG, "checkpoint truncated");
    GT_CONTEXT_LOCK(a->ctx);
    cudaError_t e = cudaSetDevice(a->ctx->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    const char* p = static_cast<const char*>(host) + sizeof(h);
    const size_t n = size_t(a->width) * a->height, r4 = 4 * accum_scalar(a->precision);
    void* dst[4] = {a->rng, a->sum, a->comp, a->accepted};
    const size_t bytes[4] = {n * sizeof(uint64_t), n * r4, n * r4, n * sizeof(uint32_t)};
    for (int k = 0; k < 4; ++k) {
        e = cudaMemcpy(dst[k], p, bytes[k], cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cuda_fail(e, "checkpoint copy");
        p += bytes[k];
    }
    a->samples = h.samples;
    a->seed = h.seed;
    return GT_OK;
    GT_GUARD_END
}

gt_status gt_render_accumulate(gt_scene* s, const gt_lights* l, const gt_environment* e, const gt_camera_desc* c,
                               uint32_t samples, gt_accumulator* acc, const gt_render_opts* o, gt_frame* f) {
    GT_GUARD_BEGIN
    if (!s || !c || !acc || !f) return fail(GT_ERR_INVALID_ARG, "null argument");
    if (acc->ctx != s->ctx) return fail(GT_ERR_INVALID_ARG, "accumulator and scene must share a context");
    if (f->struct_size < sizeof(gt_frame)) return fail(GT_ERR_INVALID_ARG, "frame struct_size too small");
    gt_render_opts opts;
    std::memset(&opts, 0, sizeof(opts));
    if (o) {
        if (o->struct_size < sizeof(gt_render_opts)) return fail(GT_ERR_INVALID_ARG, "options struct_size too small");
        opts = *o;
    }
    if (opts.schedule == GT_SCHEDULE_PERSISTENT || opts.schedule > GT_SCHEDULE_PERSISTENT)
        return fail(GT_ERR_INVALID_ARG, "accumulation runs the auto or wavefront schedule");
    if (opts.rng != GT_RNG_PIXEL) return fail(GT_ERR_UNSUPPORTED, "accumulation continues the pixels' own streams");
    opts.precision = acc->precision;
    if ((l && l->ctx != s->ctx) || (e && e->ctx != s->ctx))
        return fail(GT_ERR_INVALID_ARG, "lights, environment and scene must share a context");
    if (c->pixel_sample_mode != GT_SAMPLE_RANDOM || c->adaptive)
        return fail(GT_ERR_UNSUPPORTED, "accumulation needs random pixel sampling without adaptive stopping");
    if (samples == 0 || uint64_t(acc->samples) + samples > 0xFFFFFFFFull)
        return fail(GT_ERR_INVALID_ARG, "sample count must be positive and the total below 2^32");
    if (acc->samples > 0 && c->rng_seed != acc->seed)
        return fail(GT_ERR_INVALID_ARG, "the camera's rng_seed differs from the one the accumulation started with");
    gt_camera_desc cd = *c;
    cd.samples_per_pixel = 1; // validated as a plain random-sampling camera; the loop count is set below
    gt_status rc = validate_camera(cd);
    if (rc != GT_OK) return rc;
    CamHost cam = init_camera(cd, e != nullptr);
    if (cam.width != acc->width || cam.height != acc->height)
        return fail(GT_ERR_INVALID_ARG, "the camera's image size differs from the accumulator's");
    if (f->width != cam.width || f->height != cam.height)
        return fail(GT_ERR_INVALID_ARG, "frame size does not match the camera's image size");
    if (!f->rgb) return fail(GT_ERR_INVALID_ARG, "frame has no rgb buffer");
    GT_CONTEXT_LOCK(s->ctx);
    gt::DeferredDestroys deferred_destroys{s->ctx};
    cudaError_t ce = cudaSetDevice(s->ctx->device);
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaSetDevice");
    auto* env = const_cast<gt_environment*>(e);
    if (acc->precision == GT_PRECISION_F64) return render_accumulate_f64(s, l, env, cam, opts, f, acc, samples);
    return render_accumulate_f32(s, l, env, cam, opts, f, acc, samples);
    GT_GUARD_END
}

gt_status gt_render_batch(gt_scene* s, const gt_lights* l, const gt_environment* e, const gt_frame_job* jobs,
                          uint32_t count, const gt_render_opts* o) {
    GT_GUARD_BEGIN
    if (!s || (!jobs && count)) return fail(GT_ERR_INVALID_ARG, "null argument");
    if (count == 0) return fail(GT_ERR_INVALID_ARG, "a batch needs at least one frame");
    gt_render_opts opts;
    std::memset(&opts, 0, sizeof(opts));
    if (o) {
        if (o->struct_size < sizeof(gt_render_opts)) return fail(GT_ERR_INVALID_ARG, "options struct_size too small");
        opts = *o;
    }
    if (opts.precision > GT_PRECISION_F64) return fail(GT_ERR_INVALID_ARG, "unknown precision");
    if (opts.aovs) return fail(GT_ERR_UNSUPPORTED, "denoising AOVs are not rendered in batches");
    if (opts.rng > GT_RNG_SUBSTREAMS) return fail(GT_ERR_INVALID_ARG, "unknown rng mode");
    if (opts.rng == GT_RNG_SUBSTREAMS && opts.precision == GT_PRECISION_F64)
        return fail(GT_ERR_UNSUPPORTED, "substream batches render in f32");
    if ((l && l->ctx != s->ctx) || (e && e->ctx != s->ctx))
        return fail(GT_ERR_INVALID_ARG, "lights, environment and scene must share a context");
    std::vector<CamHost> cams(count);
    std::vector<gt_frame*> frames(count);
    for (uint32_t i = 0; i < count; ++i) {
        const gt_frame_job& j = jobs[i];
        if (!j.camera || !j.frame) return fail(GT_ERR_INVALID_ARG, "batch job without a camera or a frame");
        if (j.frame->struct_size < sizeof(gt_frame)) return fail(GT_ERR_INVALID_ARG, "frame struct_size too small");
        gt_status rc = validate_camera(*j.camera);
        if (rc != GT_OK) return rc;
        cams[i] = init_camera(*j.camera, e != nullptr);
        if (j.frame->width != cams[i].width || j.frame->height != cams[i].height)
            return fail(GT_ERR_INVALID_ARG, "frame size does not match the camera's image size");
        if (!j.frame->rgb) return fail(GT_ERR_INVALID_ARG, "frame has no rgb buffer");
        frames[i] = j.frame;
    }
    GT_CONTEXT_LOCK(s->ctx);
    gt::DeferredDestroys deferred_destroys{s->ctx};
    cudaError_t ce = cudaSetDevice(s->ctx->device);
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaSetDevice");
    auto* env = const_cast<gt_environment*>(e);
    if (opts.precision == GT_PRECISION_F64) return render_batch_f64(s, l, env, cams.data(), count, opts, frames.data());
    return render_batch_f32(s, l, env, cams.data(), count, opts, frames.data());
    GT_GUARD_END
}

gt_status gt_render(gt_scene* s, const gt_lights* l, const gt_environment* e, const gt_camera_desc* c,
                    const gt_render_opts* o, gt_frame* f) {
    GT_GUARD_BEGIN
    if (!s || !c || !f) return fail(GT_ERR_INVALID_ARG, "null argument");
    if (f->struct_size < sizeof(gt_frame)) return fail(GT_ERR_INVALID_ARG, "frame struct_size too small");
    gt_render_opts opts;
    std::memset(&opts, 0, sizeof(opts));
    if (o) {
        if (o->struct_size < sizeof(gt_render_opts)) return fail(GT_ERR_INVALID_ARG, "options struct_size too small");
        opts = *o;
    }
    if (opts.precision > GT_PRECISION_F64) return fail(GT_ERR_INVALID_ARG, "unknown precision");
    if (opts.struct_size >= offsetof(gt_render_opts, schedule) + sizeof(uint32_t) &&
        opts.schedule > GT_SCHEDULE_PERSISTENT)
        return fail(GT_ERR_INVALID_ARG, "unknown schedule");
    if (opts.struct_size < offsetof(gt_render_opts, schedule) + sizeof(uint32_t)) opts.schedule = GT_SCHEDULE_AUTO;
    if (opts.migrate > GT_MIGRATE_OFF) return fail(GT_ERR_INVALID_ARG, "unknown migrate mode");
    if (opts.rng > GT_RNG_SUBSTREAMS) return fail(GT_ERR_INVALID_ARG, "unknown rng mode");
    if ((l && l->ctx != s->ctx) || (e && e->ctx != s->ctx))
        return fail(GT_ERR_INVALID_ARG, "lights, environment and scene must share a context");
    gt_status rc = validate_camera(*c);
    if (rc != GT_OK) return rc;
    CamHost cam = init_camera(*c, e != nullptr);
    if (f->width != cam.width || f->height != cam.height)
        return fail(GT_ERR_INVALID_ARG, "frame size does not match the camera's image size");
    if (!f->rgb) return fail(GT_ERR_INVALID_ARG, "frame has no rgb buffer");
    GT_CONTEXT_LOCK(s->ctx);
    gt::DeferredDestroys deferred_destroys{s->ctx};
    cudaError_t ce = cudaSetDevice(s->ctx->device);
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaSetDevice");
    auto* env = const_cast<gt_environment*>(e);
    if (opts.precision == GT_PRECISION_F64) return render_f64(s, l, env, cam, opts, f);
    return render_f32(s, l, env, cam, opts, f);
    GT_GUARD_END
}

gt_status gt_autotune(gt_scene* s, const gt_lights* l, const gt_environment* e, const gt_frame_job* jobs,
                      uint32_t count, gt_render_opts* opts, gt_autotune_report* report) {
    GT_GUARD_BEGIN
    if (!s || !jobs || !opts || count == 0) return fail(GT_ERR_INVALID_ARG, "null argument");
    if (opts->struct_size < sizeof(gt_render_opts)) return fail(GT_ERR_INVALID_ARG, "options struct_size too small");
    if (report && report->struct_size < sizeof(gt_autotune_report))
        return fail(GT_ERR_INVALID_ARG, "report struct_size too small");
    if (opts->schedule > GT_SCHEDULE_PERSISTENT) return fail(GT_ERR_INVALID_ARG, "unknown schedule");
    // PERSISTENT (for instance the outcome of an earlier tune) is tuned as AUTO, whose last
    // candidate is PERSISTENT again.
    const uint32_t given_schedule = opts->schedule == GT_SCHEDULE_PERSISTENT ? GT_SCHEDULE_AUTO : opts->schedule;
    uint32_t trials = 0;
    // Device time of the second of two renders with `o` (the first captures its graphs).
    auto timed = [&](const gt_render_opts& cand, double& ms) -> gt_status {
        gt_render_opts o = cand;
        gt_render_stats st;
        o.stats = &st;
        o.profile = 0;
        o.progress = nullptr;
        o.progress_rgb = nullptr;
        for (int rep = 0; rep < 2; ++rep) {
            const gt_status rc = count == 1 ? gt_render(s, l, e, jobs[0].camera, &o, jobs[0].frame)
                                            : gt_render_batch(s, l, e, jobs, count, &o);
            if (rc != GT_OK) return rc;
        }
        ++trials;
        ms = st.gpu_ms;
        return GT_OK;
    };
    gt_render_opts best = *opts;
    best.schedule = given_schedule;
    double best_ms = 0.0;
    gt_status rc = timed(best, best_ms);
    if (rc != GT_OK) return rc;
    const double given_ms = best_ms;
    auto sweep = [&](uint32_t gt_render_opts::*field, std::initializer_list<uint32_t> values) -> gt_status {
        const gt_render_opts start = best;
        for (uint32_t v : values) {
            if (start.*field == v) continue;
            gt_render_opts cand = start;
            cand.*field = v;
            double ms = 0.0;
            const gt_status r = timed(cand, ms);
            if (r != GT_OK) return r;
            if (ms < 0.99 * best_ms) {
                best = cand;
                best_ms = ms;
            }
        }
        return GT_OK;
    };
    // Candidates around the library's defaults (0 = default).
    if ((rc = sweep(&gt_render_opts::stripes, {1u, 2u, 3u, 4u, 6u, 8u})) != GT_OK) return rc;
    if ((rc = sweep(&gt_render_opts::tail_slots, {0u, 4096u, 16384u, 65536u, 262144u})) != GT_OK) return rc;
    if ((rc = sweep(&gt_render_opts::trace_blocks_per_sm, {4u, 6u, 8u, 12u})) != GT_OK) return rc;
    if ((rc = sweep(&gt_render_opts::generate_blocks_per_sm, {4u, 8u, 16u})) != GT_OK) return rc;
    if (best.schedule == GT_SCHEDULE_AUTO &&
        (rc = sweep(&gt_render_opts::migrate, {uint32_t(GT_MIGRATE_ON), uint32_t(GT_MIGRATE_OFF)})) != GT_OK)
        return rc;
    // Last, the persistent schedule alone (it wins for small frames, whose wavefront
    // iterations are launch-bound); only when the caller left the choice to AUTO.
    if (given_schedule == GT_SCHEDULE_AUTO) {
        gt_render_opts cand = best;
        cand.schedule = GT_SCHEDULE_PERSISTENT;
        double ms = 0.0;
        if ((rc = timed(cand, ms)) != GT_OK) return rc;
        if (ms < 0.99 * best_ms) {
            best = cand;
            best_ms = ms;
        }
    }
    best.stats = opts->stats;
    best.profile = opts->profile;
    best.progress = opts->progress;
    best.progress_user = opts->progress_user;
    best.progress_rgb = opts->progress_rgb;
    *opts = best;
    if (report) {
        report->trials = trials;
        report->given_ms = given_ms;
        report->best_ms = best_ms;
    }
    return GT_OK;
    GT_GUARD_END
}

gt_status gt_trace_rays(gt_scene* s, const double* rays, uint32_t count, double tmin, double tmax, int32_t* ids,
                        double* t, gt_bvh_stats* stats) {
    GT_GUARD_BEGIN
    if (!s || (count && (!rays || !ids))) return fail(GT_ERR_INVALID_ARG, "null argument");
    GT_CONTEXT_LOCK(s->ctx);
    cudaError_t ce = cudaSetDevice(s->ctx->device);
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaSetDevice");
    if (s->prims.empty()) { // no BVH: RayScene counts a linear scan of zero primitives
        for (uint32_t i = 0; i < count; ++i) {
            ids[i] = -1;
            if (t) t[i] = 0.0;
        }
        if (stats) {
            std::memset(stats, 0, sizeof(*stats));
            stats->rays = count;
        }
        return GT_OK;
    }
    return trace_rays_f64(s, rays, count, tmin, tmax, ids, t, stats);
    GT_GUARD_END
}

// Probe rays RayCamera::ray_for_pixel (camera.rs:1641-1653) in f64 for every `stride`-th
// pixel, row-major: {origin, direction, time} per ray.
static std::vector<double> primary_rays(const gt_camera_desc& c, uint32_t stride) {
    CamHost cam = init_camera(c, false);
    std::vector<double> rays;
    for (uint32_t y = 0; y < cam.height; y += stride)
        for (uint32_t x = 0; x < cam.width; x += stride) {
            double pc[3];
            for (int k = 0; k < 3; ++k) pc[k] = (cam.pixel00[k] + cam.du[k] * double(x)) + cam.dv[k] * double(y);
            rays.push_back(cam.center[0]);
            rays.push_back(cam.center[1]);
            rays.push_back(cam.center[2]);
            for (int k = 0; k < 3; ++k) rays.push_back(pc[k] - cam.center[k]);
            rays.push_back(c.shutter_start);
        }
    return rays;
}

gt_status gt_trace_primary(gt_scene* s, const gt_camera_desc* c, uint32_t stride, int32_t* ids, double* t,
                           gt_bvh_stats* stats) {
    GT_GUARD_BEGIN
    if (!s || !c || !ids) return fail(GT_ERR_INVALID_ARG, "null argument");
    gt_status rc = validate_camera(*c);
    if (rc != GT_OK) return rc;
    const std::vector<double> rays = primary_rays(*c, stride ? stride : 1u);
    return gt_trace_rays(s, rays.data(), uint32_t(rays.size() / 7), 0.001, INFINITY, ids, t, stats);
    GT_GUARD_END
}

gt_status gt_trace_rays_f32(gt_scene* s, const double* rays, uint32_t count, double tmin, double tmax, int32_t* ids,
                            double* t, uint8_t* refined, gt_trace_report* report) {
    GT_GUARD_BEGIN
    if (!s || (count && (!rays || !ids))) return fail(GT_ERR_INVALID_ARG, "null argument");
    if (report && report->struct_size < sizeof(gt_trace_report))
        return fail(GT_ERR_INVALID_ARG, "report struct_size too small");
    if (report) {
        std::memset(reinterpret_cast<char*>(report) + sizeof(uint32_t), 0, sizeof(gt_trace_report) - sizeof(uint32_t));
        report->rays = count;
    }
    GT_CONTEXT_LOCK(s->ctx);
    cudaError_t ce = cudaSetDevice(s->ctx->device);
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaSetDevice");
    if (s->prims.empty()) {
        for (uint32_t i = 0; i < count; ++i) {
            ids[i] = -1;
            if (t) t[i] = 0.0;
            if (refined) refined[i] = 0;
        }
        return GT_OK;
    }
    return trace_rays_f32(s, rays, count, tmin, tmax, ids, t, refined, report);
    GT_GUARD_END
}

gt_status gt_trace_primary_f32(gt_scene* s, const gt_camera_desc* c, uint32_t stride, int32_t* ids, double* t,
                               uint8_t* refined, gt_trace_report* report) {
    GT_GUARD_BEGIN
    if (!s || !c || !ids) return fail(GT_ERR_INVALID_ARG, "null argument");
    gt_status rc = validate_camera(*c);
    if (rc != GT_OK) return rc;
    const std::vector<double> rays = primary_rays(*c, stride ? stride : 1u);
    return gt_trace_rays_f32(s, rays.data(), uint32_t(rays.size() / 7), 0.001, INFINITY, ids, t, refined, report);
    GT_GUARD_END
}

} // extern "C"
