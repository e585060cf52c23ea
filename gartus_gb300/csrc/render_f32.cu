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
    if (opts.schedule != GT_SCHEDULE_PERSISTENT && same_width && s->media.empty() && s->objects.empty())
        return render_impl<float, true>(s, l, e, cams[0], opts, nullptr, nullptr, 0, cams, count, frames);
    return render_batch_impl<float>(s, l, e, cams, count, opts, frames);
}

void free_gpu_f32(gt_scene* s) { free_gpu<float>(s); }

// After s->prims[first, first + count) changed: a resident GPU-built tree is refitted in
// place (records, metadata and boxes of those primitives, then every internal box); any
// other resident f32 copy is dropped and rebuilt from the reference tree at the next render.
gt_status update_f32(gt_scene* s, uint32_t first, uint32_t count) {
    GpuScene<float>& g = s->f32;
    if (!g.ready) return GT_OK;
    if (s->bvh_builder != GT_BVH_GPU_LBVH || !g.leaf_of) {
        free_gpu<float>(s);
        return GT_OK;
    }
    std::vector<uint32_t> index(count);
    std::vector<PrimRec<float>> recs(count);
    std::vector<uint2> meta(count);
    std::vector<float> boxes(size_t(count) * 6);
    for (uint32_t i = 0; i < count; ++i) {
        const uint32_t pi = first + i;
        const gt_primitive& p = s->prims[pi];
        const uint32_t kind = pack_prim<float>(p.geometry, recs[i].v);
        if (kind == kBadKind) return fail(GT_ERR_INVALID_ARG, "unknown geometry kind");
        index[i] = pi;
        meta[i] = make_uint2(kind | (p.material << 3), pi);
        put_box<float>(boxes.data() + size_t(i) * 6, geometry_aabb(p.geometry));
    }
    const int sms = s->ctx->num_sms > 0 ? s->ctx->num_sms : 1;
    return refit_lbvh_f32(g, uint32_t(s->prims.size()), count, index.data(), recs.data(), meta.data(), boxes.data(),
                          s->ctx->stream, sms);
}

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
