// internal.h — host-side objects behind the opaque handles of gartus_gpu.h.
#pragma once

#include <cuda_runtime.h>

#include <functional>
#include <mutex>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/gartus_gpu.h"
#include "bvh_build.h"
#include "layout.h"

namespace gt {

// Media per scene: each ray tests all of them in order.
constexpr uint32_t kMaxMedia = 64;

// A mesh copied from gt_mesh, with its tree (built at scene creation).
struct MeshHost {
    std::vector<gt_primitive> prims;
    std::vector<double> uv, vn;  // 6 / 9 per primitive, or empty
    std::vector<uint8_t> attr;   // presence bits per primitive
    uint32_t leaf_size = 4;
    BuiltBvh bvh;
};

// A scene's bitmap texture, copied from gt_image.
struct ImageHost {
    uint32_t w = 0, h = 0, filter = 0, wrap_s = 0, wrap_t = 0;
    std::vector<uint8_t> rgb;
};

template <class R> struct GpuScene {
    bool ready = false;
    uint8_t* texels = nullptr;     // every image's texels, back to back
    ImageDev* images = nullptr;
    MediumDev<R>* media = nullptr;
    MeshDev<R>* meshes = nullptr;
    ObjectDev<R>* objects = nullptr;
    Node<R>* tlas = nullptr;
    std::vector<void*> mesh_allocs; // every mesh's device arrays
    // GT_BVH_GPU_LBVH (f32 only): the tree's bottom-up links and leaf boxes, kept so that
    // gt_scene_update_primitives can refit it in place.
    int32_t* parent_leaf = nullptr;
    int32_t* parent_int = nullptr;
    uint32_t* arrivals = nullptr;
    float* int_box = nullptr;
    float* leaf_box = nullptr;
    uint32_t* leaf_of = nullptr; // original primitive index -> leaf position
    PrimRec<R>* prims = nullptr;
    uint2* meta = nullptr;
    Node<R>* nodes = nullptr;
    WideNode* wnodes = nullptr; // f32 only: the wide tree (null when the scene has none)
    uint32_t wide_depth = 0, wide_nodes = 0;
    MatDev<R>* mats = nullptr;
    PerlinDev<R>* perlin = nullptr; // one table set per noise-textured material
    SceneDev<R> view{};
};

template <class R> struct GpuLights {
    bool ready = false;
    LightDev<R>* t = nullptr;
    LightsDev<R> view{};
};

template <class R> struct GpuEnv {
    bool ready = false;
    R* weights = nullptr;
    R* cdf = nullptr;
    EnvDev<R> view{};
};

// Camera after RayCamera::initialized (camera.rs:1068-1130), in f64.
struct CamHost {
    double center[3], pixel00[3], du[3], dv[3], ddu[3], ddv[3];
    uint32_t width, height;
    uint32_t spp;  // samples per pixel the loops run (effective count)
    uint32_t grid; // stratified grid width (1 in random mode)
    gt_camera_desc desc;
    bool nee;
    double light_pdf_weight;
};

void set_error(const std::string& msg);
// RayCamera::initialized in f64 for an already validated camera (api.cu).
CamHost camera_setup(const gt_camera_desc& d, bool env);
gt_status fail(gt_status status, const std::string& msg);
gt_status cuda_fail(cudaError_t e, const char* what);

} // namespace gt

// Every extern "C" entry point runs its body inside these, so no C++ exception crosses the C ABI.
#define GT_GUARD_BEGIN try {
#define GT_GUARD_END                                                  \
    }                                                                 \
    catch (const std::bad_alloc&) {                                   \
        return gt::fail(GT_ERR_OOM, "host allocation failed");        \
    }                                                                 \
    catch (const std::exception& ex) {                                \
        return gt::fail(GT_ERR_INTERNAL, ex.what());                  \
    }


struct gt_context {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr; // concurrent persistent kernel for migrated wavefront slots
    // Wavefront stripes: each runs its kernels on its own stream and its migrated slots on
    // its own side stream.
    static constexpr int kMaxStripes = 8;
    cudaStream_t stripe_stream[kMaxStripes] = {};
    cudaStream_t stripe_side[kMaxStripes] = {};
    // Each stripe's instantiated two-iteration graph, reused while its kernel parameters
    // (scene, camera, workspace, launch sizes) stay the same from one render to the next.
    struct CachedGraph {
        std::vector<unsigned char> key;
        cudaGraphExec_t exec = nullptr;
    };
    CachedGraph graphs[kMaxStripes];
    // Held by every call that touches the context's device state.  A progress callback runs
    // on the rendering thread while the render holds it, so the lock is recursive and the
    // callback is counted: a destroy called from inside the callback (a handle that the
    // host language's garbage collector finalises there, say) is deferred to the end of the
    // render, and every other call fails instead of deadlocking or disturbing the render.
    std::recursive_mutex mu;
    int in_callback = 0;
    std::vector<std::function<void()>> deferred;
    void* ws = nullptr; // render workspace (path state, queues, staging)
    size_t ws_bytes = 0;
    uint32_t* pinned = nullptr; // host-pinned copy of the loop counters (256 words)
    // Host memory mapped into the device: [0] cancel word, [1] pixels handed out.
    volatile uint32_t* mapped = nullptr;
    uint32_t* mapped_dev = nullptr;
};

namespace gt {
// Calls the render's progress callback with the context marked as inside it.
inline int call_progress(gt_context* ctx, const gt_render_opts& o, uint64_t done, uint64_t total) {
    ++ctx->in_callback;
    const int r = o.progress(o.progress_user, done, total);
    --ctx->in_callback;
    return r;
}

// Runs, when a render entry point returns, the destroys its progress callbacks deferred.
struct DeferredDestroys {
    gt_context* ctx;
    ~DeferredDestroys() {
        if (ctx->in_callback) return;
        std::vector<std::function<void()>> list;
        list.swap(ctx->deferred);
        for (auto& f : list) f();
    }
};

// Destroys now, or at the end of the render whose progress callback this is.
inline void destroy_or_defer(gt_context* ctx, std::function<void()> destroy) {
    std::lock_guard<std::recursive_mutex> lock(ctx->mu);
    if (ctx->in_callback) ctx->deferred.push_back(std::move(destroy));
    else destroy();
}
} // namespace gt

// Takes the context lock for the rest of the scope; from inside a progress callback of a
// render on this context, returns GT_ERR_INVALID_ARG instead.
#define GT_CONTEXT_LOCK(ctxp)                                                                          \
    std::lock_guard<std::recursive_mutex> gt_context_lock_(ctxp->mu);                                   \
    if ((ctxp)->in_callback)                                                                           \
    return gt::fail(GT_ERR_INVALID_ARG, "called from inside a progress callback of a render on this context")

// Resumable accumulation state in device memory (one entry per pixel, in the
// accumulator's precision): stream position, radiance sums, Kahan compensation, accepted.
struct gt_accumulator {
    gt_context* ctx = nullptr;
    uint32_t width = 0, height = 0, precision = 0;
    uint32_t samples = 0;  // samples per pixel accumulated
    uint64_t seed = 0;     // the camera rng_seed the streams started from
    uint64_t* rng = nullptr;
    void* sum = nullptr;   // R4<R> per pixel
    void* comp = nullptr;  // R4<R> per pixel
    uint32_t* accepted = nullptr;
};

struct gt_scene {
    gt_context* ctx = nullptr;
    std::vector<gt_primitive> prims;
    std::vector<gt_material> mats;
    std::vector<gt::ImageHost> images;
    std::vector<gt_medium> media;
    std::vector<gt::MeshHost> meshes;
    std::vector<gt_object> objects;
    uint32_t bvh_builder = GT_BVH_REFERENCE_SAH;
    uint32_t f32_tree = GT_F32_TREE_WIDE;
    uint32_t leaf_size = 4;
    bool bvh_ready = false; // `bvh` has been built (eagerly for the reference builder)
    gt::BuiltBvh bvh;
    gt::GpuScene<float> f32;
    gt::GpuScene<double> f64;
};

struct gt_lights {
    gt_context* ctx = nullptr;
    std::vector<gt_light_target> targets;
    double total = 0.0;
    gt::GpuLights<float> f32;
    gt::GpuLights<double> f64;
};

struct gt_environment {
    gt_context* ctx = nullptr;
    uint32_t format = 0, width = 0, height = 0;
    uint8_t* d_px8 = nullptr;
    float* d_px32 = nullptr;
    std::vector<uint8_t> px8;
    std::vector<float> px32;
    std::vector<double> weights, cdf;
    double total = 0.0;
    gt::GpuEnv<float> f32;
    gt::GpuEnv<double> f64;
};

namespace gt {

// Per-precision entry points (render_f32.cu / render_f64.cu).
gt_status render_f32(gt_scene* s, const gt_lights* l, gt_environment* e, const CamHost& cam,
                     const gt_render_opts& opts, gt_frame* frame);
gt_status render_f64(gt_scene* s, const gt_lights* l, gt_environment* e, const CamHost& cam,
                     const gt_render_opts& opts, gt_frame* frame);
gt_status render_accumulate_f32(gt_scene* s, const gt_lights* l, gt_environment* e, const CamHost& cam,
                                const gt_render_opts& opts, gt_frame* frame, gt_accumulator* acc, uint32_t samples);
gt_status render_accumulate_f64(gt_scene* s, const gt_lights* l, gt_environment* e, const CamHost& cam,
                                const gt_render_opts& opts, gt_frame* frame, gt_accumulator* acc, uint32_t samples);
gt_status render_batch_f32(gt_scene* s, const gt_lights* l, gt_environment* e, const CamHost* cams, uint32_t count,
                           const gt_render_opts& opts, gt_frame* const* frames);
gt_status render_batch_f64(gt_scene* s, const gt_lights* l, gt_environment* e, const CamHost* cams, uint32_t count,
                           const gt_render_opts& opts, gt_frame* const* frames);
gt_status trace_rays_f32(gt_scene* s, const double* rays, uint32_t count, double tmin, double tmax, int32_t* ids,
                         double* t, uint8_t* refined, gt_trace_report* rep);
gt_status trace_rays_f64(gt_scene* s, const double* rays, uint32_t count, double tmin, double tmax,
                         int32_t* ids, double* t, gt_bvh_stats* stats);
void free_gpu_f32(gt_scene* s);
void free_gpu_f64(gt_scene* s);
void free_lights_f32(gt_lights* l);
void free_lights_f64(gt_lights* l);
void free_env_f32(gt_environment* e);
void free_env_f64(gt_environment* e);

} // namespace gt

namespace gt {
// The reference-layout SAH tree of `s`, built on first use (api.cu).
gt_status ensure_reference_bvh(gt_scene* s);
gt_status refit_lbvh_f32(GpuScene<float>& g, uint32_t n, uint32_t count, const uint32_t* index,
                         const PrimRec<float>* recs, const uint2* meta, const float* boxes, cudaStream_t st, int sms);
gt_status update_f32(gt_scene* s, uint32_t first, uint32_t count);
// A linear BVH for the f32 path built on the device from f32 primitive bounds; permutes
// g.prims / g.meta into leaf order and sets the view's nodes and root (lbvh.cu).
gt_status build_lbvh_f32(GpuScene<float>& g, uint32_t n, const float* boxes_host, const double* bounds_lo,
                         const double* bounds_hi, cudaStream_t st, int sms);
} // namespace gt
