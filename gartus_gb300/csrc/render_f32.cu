// render_f32.cu — the f32 throughput instantiation of the wavefront integrator.
#include "render_host.cuh"

namespace gt {

gt_status render_f32(gt_scene* s, const gt_lights* l, gt_environment* e, const CamHost& cam,
                     const gt_render_opts& opts, gt_frame* frame) {
    return render_impl<float>(s, l, e, cam, opts, frame);
}

gt_status render_accumulate_f32(gt_scene* s, const gt_lights* l, gt_environment* e, const CamHost& cam,
                                const gt_render_opts& opts, gt_frame* frame, gt_accumulator* acc, uint32_t samples) {
    return render_impl<float>(s, l, e, cam, opts, frame, acc, samples);
}

// Frames of one width run through the striped wavefront as one image of their rows; the
// persistent schedule, or frames of different widths, use the one-launch persistent batch.
gt_status render_batch_f32(gt_scene* s, const gt_lights* l, gt_environment* e, const CamHost* cams, uint32_t count,
                           const gt_render_opts& opts, gt_frame* const* frames) {
    bool same_width = true;
    for (uint32_t i = 1; i < count; ++i) same_width = same_width && cams[i].width == cams[0].width;
    if (opts.schedule != GT_SCHEDULE_PERSISTENT && same_width && s->media.empty())
        return render_impl<float, true>(s, l, e, cams[0], opts, nullptr, nullptr, 0, cams, count, frames);
    return render_batch_impl<float>(s, l, e, cams, count, opts, frames);
}

void free_gpu_f32(gt_scene* s) { free_gpu<float>(s); }

void free_lights_f32(gt_lights* l) {
    cudaFree(l->f32.t);
    l->f32 = GpuLights<float>();
}

void free_env_f32(gt_environment* e) {
    cudaFree(e->f32.weights);
    cudaFree(e->f32.cdf);
    e->f32 = GpuEnv<float>();
}

} // namespace gt
