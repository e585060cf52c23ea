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

// Frames of one width run through the striped wavefront as one image of their rows (worlds
// with objects too); the persistent schedule, frames of different widths, or a world with
// media use the one-launch persistent batch.
gt_status render_batch_f32(gt_scene* s, const gt_lights* l, gt_environment* e, const CamHost* cams, uint32_t count,
                           const gt_render_opts& opts, gt_frame* const* frames) {
    bool same_width = true;
    for (uint32_t i = 1; i < count; ++i) same_width = same_width && cams[i].width == cams[0].width;
    // substreams: the frames' pixels are work items of one list, whatever their widths
    if (opts.rng == GT_RNG_SUBSTREAMS ||
        (opts.schedule != GT_SCHEDULE_PERSISTENT && same_width && s->media.empty()))
        return render_impl<float, true>(s, l, e, cams[0], opts, nullptr, nullptr, 0, cams, count, frames);
    return render_batch_impl<float>(s, l, e, cams, count, opts, frames);
}

void free_gpu_f32(gt_scene* s) { free_gpu<float>(s); }

// Check 1 on the f32 traversal: ids and distances from the f32 rendering walk; the rays
// it flags are re-traced by the f64 walk over the reference tree, whose ids are the
// reference's.  refined[i]: 0 = f32 result, 1 = re-traced in f64, same id, 2 = re-traced,
// id changed.
gt_status trace_rays_f32(gt_scene* s, const double* rays, uint32_t count, double tmin, double tmax, int32_t* ids,
                         double* t, uint8_t* refined, gt_trace_report* rep) {
    gt_context* ctx = s->ctx;
    cudaStream_t st = ctx->stream;
    gt_status rc;
    if ((rc = upload_scene<float>(s)) != GT_OK) return rc;
    Bump sizing{nullptr};
    sizing.take<double>(size_t(count) * 7);
    sizing.take<int32_t>(count);
    sizing.take<double>(count);
    sizing.take<uint8_t>(count);
    sizing.take<uint32_t>(4);
    if ((rc = ensure_workspace(ctx, sizing.off + 4096)) != GT_OK) return rc;
    Bump b{static_cast<char*>(ctx->ws)};
    double* d_rays = b.take<double>(size_t(count) * 7);
    int32_t* d_ids = b.take<int32_t>(count);
    double* d_t = b.take<double>(count);
    uint8_t* d_near = b.take<uint8_t>(count);
    uint32_t* d_err = b.take<uint32_t>(4);
    std::vector<double> tt(count);
    std::vector<uint8_t> near(count);
    GT_CUDA(cudaMemsetAsync(d_err, 0, 4 * sizeof(uint32_t), st));
    if (count) {
        GT_CUDA(cudaMemcpyAsync(d_rays, rays, size_t(count) * 7 * sizeof(double), cudaMemcpyHostToDevice, st));
        const uint32_t blocks = std::min<uint32_t>((count + 127) / 128, uint32_t(std::max(ctx->num_sms, 1)) * 8);
        k_trace_rays_check<float><<<blocks, 128, 0, st>>>(s->f32.view, d_rays, count, tmin, tmax, d_ids, d_t, d_near, d_err);
        GT_CUDA(cudaGetLastError());
        GT_CUDA(cudaMemcpyAsync(ids, d_ids, size_t(count) * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
        GT_CUDA(cudaMemcpyAsync(tt.data(), d_t, size_t(count) * sizeof(double), cudaMemcpyDeviceToHost, st));
        GT_CUDA(cudaMemcpyAsync(near.data(), d_near, count, cudaMemcpyDeviceToHost, st));
    }
    uint32_t err = 0;
    GT_CUDA(cudaMemcpyAsync(&err, d_err, sizeof(err), cudaMemcpyDeviceToHost, st));
    GT_CUDA(cudaStreamSynchronize(st));
    if (err) return fail(GT_ERR_INTERNAL, "traversal stack overflow");
    std::vector<uint32_t> which;
    std::vector<double> again;
    for (uint32_t i = 0; i < count; ++i)
        if (near[i]) {
            which.push_back(i);
            again.insert(again.end(), rays + size_t(i) * 7, rays + size_t(i) * 7 + 7);
        }
    uint64_t changed = 0;
    if (!which.empty()) {
        std::vector<int32_t> ids64(which.size());
        std::vector<double> t64(which.size());
        if ((rc = trace_rays_f64(s, again.data(), uint32_t(which.size()), tmin, tmax, ids64.data(), t64.data(),
                                 nullptr)) != GT_OK)
            return rc;
        for (size_t k = 0; k < which.size(); ++k) {
            const uint32_t i = which[k];
            if (ids[i] != ids64[k]) {
                ++changed;
                near[i] = 2;
            }
            ids[i] = ids64[k];
            tt[i] = t64[k];
        }
    }
    if (t) std::copy(tt.begin(), tt.end(), t);
    if (refined) std::copy(near.begin(), near.end(), refined);
    if (rep) {
        rep->tree = s->f32.view.wnodes ? GT_F32_TREE_WIDE : GT_F32_TREE_BINARY;
        rep->rays = count;
        rep->refined = which.size();
        rep->changed = changed;
        rep->wide_nodes = s->f32.wide_nodes;
        rep->wide_depth = s->f32.wide_depth;
    }
    return GT_OK;
}

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
