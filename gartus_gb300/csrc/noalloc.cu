// noalloc.cu — gt_render_noalloc: an f32 render that allocates nothing.
//
// Some callers cannot allocate device memory when they render: a real-time loop that
// must not hit cudaMalloc's synchronisation and latency, a host runtime whose allocator
// owns all device memory, or code that runs where allocation is forbidden.  For them this
// entry point runs the persistent schedule (k_classify + k_persistent, f32) with all of
// its scratch — counters, sample totals, the pixel counter and the cost-ordered pixel
// queues — in one file-scope device array of fixed size, reserved when the library's
// device code is loaded onto a GPU and held until the process exits.
#include <mutex>
#include <string>

#include "render_host.cuh"

namespace gt {
namespace {

constexpr uint32_t kNoAllocMaxPixels = GT_NOALLOC_MAX_PIXELS;
// Header: counters at 0 (C_COUNT words), totals at 128 (8 x 8 B), pixel counter at 192.
constexpr size_t kHeaderBytes = 512;
static_assert(C_COUNT * sizeof(uint32_t) <= 128, "counters overlap the totals in the scratch header");
constexpr size_t kScratchBytes = kHeaderBytes + size_t(kNoAllocMaxPixels) * NUM_COST_CLASSES * sizeof(uint32_t);

// The shared scratch.  Host code must not use this name as an address: on the host it
// is only a stand-in symbol, so device code gets its address from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
void* g_scratch_ptr[kMaxDevices] = {nullptr};

// Once per device, with that device current: the device address of g_scratch.
gt_status scratch_for_device(int device, unsigned char** out) {
    if (device < 0 || device >= kMaxDevices) return fail(GT_ERR_UNSUPPORTED, "device index too large for gt_render_noalloc");
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch_ptr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess || !p) return cuda_fail(e == cudaSuccess ? cudaErrorInvalidSymbol : e, "cudaGetSymbolAddress");
        g_scratch_ptr[device] = p;
    }
    *out = static_cast<unsigned char*>(g_scratch_ptr[device]);
    return GT_OK;
}

} // namespace
} // namespace gt

using namespace gt;

extern "C" gt_status gt_render_noalloc(gt_scene* scene, const gt_lights* lights, const gt_environment* environment,
                                       const gt_camera_desc* camera, float* rgb, uint32_t* accepted) {
    try {
        if (!scene || !camera || !rgb) return fail(GT_ERR_INVALID_ARG, "null argument");
        if ((lights && lights->ctx != scene->ctx) || (environment && environment->ctx != scene->ctx))
            return fail(GT_ERR_INVALID_ARG, "lights, environment and scene must share a context");
        uint32_t w = 0, h = 0, spp = 0;
        gt_status rc = gt_camera_image_size(camera, &w, &h, &spp);
        if (rc != GT_OK) return rc;
        const uint64_t n64 = uint64_t(w) * h;
        if (n64 > kNoAllocMaxPixels)
            return fail(GT_ERR_INVALID_ARG, "image has more pixels than gt_render_noalloc's scratch holds (" +
                                                std::to_string(kNoAllocMaxPixels) + ")");
        // The device copies must already exist: creating them would allocate.
        if (!scene->f32.ready)
            return fail(GT_ERR_INVALID_ARG, "scene is not resident on the device in f32; render it once with gt_render first");
        if (lights && !lights->f32.ready)
            return fail(GT_ERR_INVALID_ARG, "lights are not resident on the device in f32; render once with gt_render first");
        if (environment && !environment->f32.ready)
            return fail(GT_ERR_INVALID_ARG,
                        "environment is not resident on the device in f32; render once with gt_render first");
        gt_context* ctx = scene->ctx;
        GT_CONTEXT_LOCK(ctx);
        cudaError_t ce = cudaSetDevice(ctx->device);
        if (ce != cudaSuccess) return cuda_fail(ce, "cudaSetDevice");
        unsigned char* base = nullptr;
        if ((rc = scratch_for_device(ctx->device, &base)) != GT_OK) return rc;

        // The same set-up as gt_render's persistent path, with scratch from g_scratch.
        const uint32_t n = uint32_t(n64);
        const CamHost cam = camera_setup(*camera, environment != nullptr); // validated above
        Params<float> P;
        std::memset(&P, 0, sizeof(P));
        P.sc = scene->f32.view;
        if (lights) P.lights = lights->f32.view;
        if (environment) P.env = environment->f32.view;
        P.cam = cam_dev<float>(cam, lights != nullptr, environment != nullptr);
        P.ps.n = n;
        P.ps.counters = reinterpret_cast<uint32_t*>(base);
        P.ps.totals = reinterpret_cast<unsigned long long*>(base + 128);
        uint32_t* next = reinterpret_cast<uint32_t*>(base + 192);
        uint32_t* queues = reinterpret_cast<uint32_t*>(base + kHeaderBytes);
        cudaStream_t st = ctx->stream;
        // Every call shares g_scratch and it keeps the last call's contents: the header
        // (queue sizes, counters, error word) starts at zero each call; the queues are
        // fully rewritten before they are read.
        ce = cudaMemsetAsync(base, 0, kHeaderBytes, st);
        if (ce != cudaSuccess) return cuda_fail(ce, "cudaMemsetAsync");
        const uint32_t sms = uint32_t(ctx->num_sms > 0 ? ctx->num_sms : 1);
        const uint32_t cblocks = std::max<uint32_t>(1u, std::min<uint32_t>((n + 255) / 256, sms * 8));
        k_classify<float><<<cblocks, 256, 0, st>>>(P, queues, P.ps.counters + C_MAT);
        int per_sm = 0;
        const bool world = P.sc.num_media != 0 || P.sc.num_objects != 0;
        ce = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &per_sm, world ? k_persistent<float, false, false, true> : k_persistent<float, false>, 128, 0);
        if (ce != cudaSuccess) return cuda_fail(ce, "occupancy query");
        const uint32_t blocks = std::max<uint32_t>(1u, std::min<uint32_t>(sms * uint32_t(std::max(per_sm, 1)), (n + 127) / 128));
        if (world)
            k_persistent<float, false, false, true><<<blocks, 128, 0, st>>>(P, next, queues, P.ps.counters + C_MAT, nullptr,
                                                                           nullptr, rgb, nullptr, accepted);
        else
            k_persistent<float, false><<<blocks, 128, 0, st>>>(P, next, queues, P.ps.counters + C_MAT, nullptr, nullptr,
                                                               rgb, nullptr, accepted);
        ce = cudaGetLastError();
        if (ce != cudaSuccess) return cuda_fail(ce, "gt_render_noalloc launch");
        ce = cudaMemcpyAsync(ctx->pinned, P.ps.counters + C_ERROR, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
        if (ce != cudaSuccess) return cuda_fail(ce, "gt_render_noalloc");
        const uint32_t word = ctx->pinned[0];
        if (word & E_STACK_OVERFLOW)
            return fail(GT_ERR_INTERNAL, "traversal stack overflow (BVH deeper than the device stack)");
        if (word) return fail(GT_ERR_INTERNAL, "device error word " + std::to_string(word));
        return GT_OK;
    } catch (const std::exception& ex) {
        return fail(GT_ERR_INTERNAL, ex.what());
    }
}
