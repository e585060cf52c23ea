// render_f64.cu — the reference-exact f64 instantiation.  This translation unit is built
// with -fmad=false so no multiply-add is fused: every operation rounds as the reference's
// f64 arithmetic does.
#include "render_host.cuh"

namespace gt {

gt_status render_f64(gt_scene* s, const gt_lights* l, gt_environment* e, const CamHost& cam,
                     const gt_render_opts& opts, gt_frame* frame) {
    return render_impl<double>(s, l, e, cam, opts, frame);
}

gt_status render_accumulate_f64(gt_scene* s, const gt_lights* l, gt_environment* e, const CamHost& cam,
                                const gt_render_opts& opts, gt_frame* frame, gt_accumulator* acc, uint32_t samples) {
    return render_impl<double>(s, l, e, cam, opts, frame, acc, samples);
}

gt_status render_batch_f64(gt_scene* s, const gt_lights* l, gt_environment* e, const CamHost* cams, uint32_t count,
                           const gt_render_opts& opts, gt_frame* const* frames) {
    return render_batch_impl<double>(s, l, e, cams, count, opts, frames);
}

gt_status trace_rays_f64(gt_scene* s, const double* rays, uint32_t count, double tmin, double tmax,
                         int32_t* ids, double* t, gt_bvh_stats* stats) {
    return trace_impl<double>(s, rays, count, tmin, tmax, ids, t, stats);
}

void free_gpu_f64(gt_scene* s) { free_gpu<double>(s); }

void free_lights_f64(gt_lights* l) {
    cudaFree(l->f64.t);
    l->f64 = GpuLights<double>();
}

void free_env_f64(gt_environment* e) {
    cudaFree(e->f64.weights);
    cudaFree(e->f64.cdf);
    e->f64 = GpuEnv<double>();
}

} // namespace gt
