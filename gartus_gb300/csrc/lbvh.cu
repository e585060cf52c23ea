// lbvh.cu — a BVH built on the GPU for the f32 throughput path (gt_scene_desc.bvh_builder =
// GT_BVH_GPU_LBVH), for scenes too large for the host SAH build to be paid per upload.
//
// A linear BVH after Karras, "Maximizing Parallelism in the Construction of BVHs, Octrees,
// and k-d Trees" (HPG 2012): primitives sorted by the 30-bit Morton code of their box
// centres, one internal node per adjacent pair of sorted primitives whose split is found
// from the longest common prefixes of the codes, and boxes filled in bottom-up.  The result
// uses the same node layout as the host-built tree (both child boxes inline, leaf children
// as ~first primitive with a count), so the traversal kernels are unchanged; primitives and
// their metadata are permuted into the sorted (leaf) order on the device.  Boxes come from
// the host's padded f64 bounds rounded outward to f32, so they are as conservative as the
// host tree's.  The reference-layout SAH tree that f64 rendering and the traversal
// statistics need is then built on the host only when they are used.
#include <cub/cub.cuh>

#include "internal.h"

namespace gt {
namespace {

// 10 bits per axis interleaved (x in the highest position of each triple).
__device__ __forceinline__ uint32_t spread10(uint32_t v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

__global__ void k_morton(const float* boxes, uint32_t n, float3 lo, float3 inv_ext, uint32_t* codes,
                         uint32_t* index) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float* b = boxes + size_t(i) * 6;
        const float c[3] = {0.5f * (b[0] + b[3]), 0.5f * (b[1] + b[4]), 0.5f * (b[2] + b[5])};
        const float l[3] = {lo.x, lo.y, lo.z}, s[3] = {inv_ext.x, inv_ext.y, inv_ext.z};
        uint32_t q[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float t = (c[a] - l[a]) * s[a] * 1024.0f;
            q[a] = uint32_t(fminf(fmaxf(t, 0.0f), 1023.0f));
        }
        codes[i] = (spread10(q[0]) << 2) | (spread10(q[1]) << 1) | spread10(q[2]);
        index[i] = i;
    }
}

// Primitives, metadata and boxes gathered into the sorted order.
__global__ void k_permute(const PrimRec<float>* prims, const uint2* meta, const float* boxes, const uint32_t* order,
                          uint32_t n, PrimRec<float>* prims_out, uint2* meta_out, float* boxes_out) {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const uint32_t i = order[k];
        prims_out[k] = prims[i];
        meta_out[k] = meta[i];
#pragma unroll
        for (int a = 0; a < 6; ++a) boxes_out[size_t(k) * 6 + a] = boxes[size_t(i) * 6 + a];
    }
}

// Length of the common prefix of sorted codes i and j (ties broken by index), -1 outside.
__device__ __forceinline__ int delta(const uint32_t* codes, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    const uint32_t a = codes[i], b = codes[j];
    if (a == b) return 32 + __clz(uint32_t(i) ^ uint32_t(j));
    return __clz(a ^ b);
}

// Internal node i of n - 1: its range of sorted primitives, split and children (Karras 2012,
// algorithm 4).  Leaf children are written as ~primitive with count 1.
__global__ void k_karras(const uint32_t* codes, int n, Node<float>* nodes, int32_t* parent_leaf, int32_t* parent_int) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n - 1; i += gridDim.x * blockDim.x) {
        const int d = delta(codes, n, i, i + 1) - delta(codes, n, i, i - 1) >= 0 ? 1 : -1;
        const int dmin = delta(codes, n, i, i - d);
        int lmax = 2;
        while (delta(codes, n, i, i + lmax * d) > dmin) lmax <<= 1;
        int l = 0;
        for (int t = lmax >> 1; t >= 1; t >>= 1)
            if (delta(codes, n, i, i + (l + t) * d) > dmin) l += t;
        const int j = i + l * d;
        const int dnode = delta(codes, n, i, j);
        int s = 0, t = l;
        do {
            t = (t + 1) >> 1;
            if (delta(codes, n, i, i + (s + t) * d) > dnode) s += t;
        } while (t > 1);
        const int gamma = i + s * d + min(d, 0);
        const bool left_leaf = min(i, j) == gamma, right_leaf = max(i, j) == gamma + 1;
        Node<float>& nd = nodes[i];
        nd.link[0] = left_leaf ? ~gamma : gamma;
        nd.link[1] = left_leaf ? 1 : 0;
        nd.link[2] = right_leaf ? ~(gamma + 1) : gamma + 1;
        nd.link[3] = right_leaf ? 1 : 0;
        if (left_leaf) parent_leaf[gamma] = i;
        else parent_int[gamma] = i;
        if (right_leaf) parent_leaf[gamma + 1] = i;
        else parent_int[gamma + 1] = i;
        if (i == 0) parent_int[0] = -1;
    }
}

// Bottom-up boxes: each leaf walks towards the root; at every internal node the first of
// its two children to arrive stops and the second writes both child boxes and the node's
// own box for its parent.  A walk is at most the tree's depth.
__global__ void k_boxes(const float* leaf_box, int n, const int32_t* parent_leaf, const int32_t* parent_int,
                        uint32_t* arrivals, float* int_box, Node<float>* nodes) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        int node = parent_leaf[k];
        while (node >= 0) {
            __threadfence();
            if (atomicAdd(&arrivals[node], 1u) == 0u) break;
            Node<float>& nd = nodes[node];
            float u[6] = {3.0e38f, 3.0e38f, 3.0e38f, -3.0e38f, -3.0e38f, -3.0e38f};
#pragma unroll
            for (int side = 0; side < 2; ++side) {
                const int32_t link = nd.link[2 * side];
                const float* src = link < 0 ? leaf_box + size_t(~link) * 6 : int_box + size_t(link) * 6;
                float b[6];
#pragma unroll
                for (int a = 0; a < 6; ++a) b[a] = __ldcg(src + a);
#pragma unroll
                for (int a = 0; a < 6; ++a) nd.box[6 * side + a] = b[a];
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    u[a] = fminf(u[a], b[a]);
                    u[3 + a] = fmaxf(u[3 + a], b[3 + a]);
                }
            }
#pragma unroll
            for (int a = 0; a < 6; ++a) __stcg(int_box + size_t(node) * 6 + a, u[a]);
            __threadfence();
            node = parent_int[node];
        }
    }
}

// leaf_of[original index] = leaf position.
__global__ void k_invert(const uint32_t* order, uint32_t n, uint32_t* leaf_of) {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) leaf_of[order[k]] = k;
}

// Refit input: updated primitives (original index, record, metadata, box) scattered into
// their leaf positions.
__global__ void k_update(const uint32_t* index, const PrimRec<float>* recs, const uint2* meta, const float* boxes,
                         uint32_t count, const uint32_t* leaf_of, PrimRec<float>* prims, uint2* meta_out,
                         float* leaf_box) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const uint32_t k = leaf_of[index[i]];
        prims[k] = recs[i];
        meta_out[k] = meta[i];
#pragma unroll
        for (int a = 0; a < 6; ++a) leaf_box[size_t(k) * 6 + a] = boxes[size_t(i) * 6 + a];
    }
}

} // namespace

gt_status build_lbvh_f32(GpuScene<float>& g, uint32_t n, const float* boxes_host, const double* bounds_lo,
                         const double* bounds_hi, cudaStream_t st, int sms) {
    SceneDev<float>& v = g.view;
    if (n == 0) return GT_OK; // the caller set an empty root
    std::vector<void*> tmp;
    auto dmalloc = [&](void** p, size_t bytes) -> cudaError_t {
        const cudaError_t e = cudaMalloc(p, std::max<size_t>(bytes, 1));
        if (e == cudaSuccess) tmp.push_back(*p);
        return e;
    };
    auto cleanup = [&]() {
        cudaStreamSynchronize(st);
        for (void* p : tmp) cudaFree(p);
    };
    float *d_boxes = nullptr, *d_sorted_boxes = nullptr, *d_int_box = nullptr;
    uint32_t *d_codes = nullptr, *d_codes_sorted = nullptr, *d_index = nullptr, *d_order = nullptr, *d_arrivals = nullptr;
    int32_t *d_parent_leaf = nullptr, *d_parent_int = nullptr;
    PrimRec<float>* d_prims = nullptr;
    uint2* d_meta = nullptr;
    cudaError_t e = cudaSuccess;
    const uint32_t ni = n > 1 ? n - 1 : 1;
    if (e == cudaSuccess) e = dmalloc(reinterpret_cast<void**>(&d_boxes), size_t(n) * 6 * sizeof(float));
    // The tree's links and boxes stay with the scene for refits (freed with it).
    auto keep = [&](void** p, size_t bytes) -> cudaError_t { return cudaMalloc(p, std::max<size_t>(bytes, 1)); };
    if (e == cudaSuccess) e = keep(reinterpret_cast<void**>(&g.leaf_box), size_t(n) * 6 * sizeof(float));
    if (e == cudaSuccess) e = keep(reinterpret_cast<void**>(&g.int_box), size_t(ni) * 6 * sizeof(float));
    if (e == cudaSuccess) e = keep(reinterpret_cast<void**>(&g.arrivals), size_t(ni) * sizeof(uint32_t));
    if (e == cudaSuccess) e = keep(reinterpret_cast<void**>(&g.parent_leaf), size_t(n) * sizeof(int32_t));
    if (e == cudaSuccess) e = keep(reinterpret_cast<void**>(&g.parent_int), size_t(ni) * sizeof(int32_t));
    if (e == cudaSuccess) e = keep(reinterpret_cast<void**>(&g.leaf_of), size_t(n) * sizeof(uint32_t));
    d_sorted_boxes = g.leaf_box;
    d_int_box = g.int_box;
    d_arrivals = g.arrivals;
    d_parent_leaf = g.parent_leaf;
    d_parent_int = g.parent_int;
    if (e == cudaSuccess) e = dmalloc(reinterpret_cast<void**>(&d_codes), size_t(n) * sizeof(uint32_t));
    if (e == cudaSuccess) e = dmalloc(reinterpret_cast<void**>(&d_codes_sorted), size_t(n) * sizeof(uint32_t));
    if (e == cudaSuccess) e = dmalloc(reinterpret_cast<void**>(&d_index), size_t(n) * sizeof(uint32_t));
    if (e == cudaSuccess) e = dmalloc(reinterpret_cast<void**>(&d_order), size_t(n) * sizeof(uint32_t));
    if (e == cudaSuccess) e = dmalloc(reinterpret_cast<void**>(&d_prims), size_t(n) * sizeof(PrimRec<float>));
    if (e == cudaSuccess) e = dmalloc(reinterpret_cast<void**>(&d_meta), size_t(n) * sizeof(uint2));
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_boxes, boxes_host, size_t(n) * 6 * sizeof(float), cudaMemcpyHostToDevice, st);
    const float ext[3] = {float(bounds_hi[0] - bounds_lo[0]), float(bounds_hi[1] - bounds_lo[1]),
                          float(bounds_hi[2] - bounds_lo[2])};
    const float3 lo = make_float3(float(bounds_lo[0]), float(bounds_lo[1]), float(bounds_lo[2]));
    const float3 inv = make_float3(ext[0] > 0.f ? 1.f / ext[0] : 0.f, ext[1] > 0.f ? 1.f / ext[1] : 0.f,
                                   ext[2] > 0.f ? 1.f / ext[2] : 0.f);
    const int threads = 256;
    const int blocks = int(std::max<uint64_t>(1, std::min<uint64_t>((n + threads - 1) / threads, uint64_t(sms) * 8)));
    if (e == cudaSuccess) {
        k_morton<<<blocks, threads, 0, st>>>(d_boxes, n, lo, inv, d_codes, d_index);
        e = cudaGetLastError();
    }
    size_t temp_bytes = 0;
    if (e == cudaSuccess)
        e = cub::DeviceRadixSort::SortPairs(nullptr, temp_bytes, d_codes, d_codes_sorted, d_index, d_order, int(n), 0,
                                            30, st);
    void* d_temp = nullptr;
    if (e == cudaSuccess) e = dmalloc(&d_temp, temp_bytes);
    if (e == cudaSuccess)
        e = cub::DeviceRadixSort::SortPairs(d_temp, temp_bytes, d_codes, d_codes_sorted, d_index, d_order, int(n), 0,
                                            30, st);
    if (e == cudaSuccess) {
        k_permute<<<blocks, threads, 0, st>>>(g.prims, g.meta, d_boxes, d_order, n, d_prims, d_meta, d_sorted_boxes);
        k_invert<<<blocks, threads, 0, st>>>(d_order, n, g.leaf_of);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(g.prims, d_prims, size_t(n) * sizeof(PrimRec<float>), cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(g.meta, d_meta, size_t(n) * sizeof(uint2), cudaMemcpyDeviceToDevice, st);
    if (n == 1) {
        float b[6];
        for (int a = 0; a < 6; ++a) b[a] = boxes_host[a];
        for (int a = 0; a < 6; ++a) v.root_box[a] = b[a];
        v.root_link = ~0;
        v.root_count = 1;
        cleanup();
        if (e != cudaSuccess) return cuda_fail(e, "GPU BVH build");
        return GT_OK;
    }
    if (e == cudaSuccess) e = cudaMalloc(&g.nodes, size_t(ni) * sizeof(Node<float>));
    if (e == cudaSuccess) e = cudaMemsetAsync(d_arrivals, 0, size_t(ni) * sizeof(uint32_t), st);
    if (e == cudaSuccess) {
        k_karras<<<blocks, threads, 0, st>>>(d_codes_sorted, int(n), g.nodes, d_parent_leaf, d_parent_int);
        k_boxes<<<blocks, threads, 0, st>>>(d_sorted_boxes, int(n), d_parent_leaf, d_parent_int, d_arrivals, d_int_box,
                                            g.nodes);
        e = cudaGetLastError();
    }
    float root[6] = {0, 0, 0, 0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(root, d_int_box, sizeof(root), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cleanup();
    if (e != cudaSuccess) return cuda_fail(e, "GPU BVH build");
    for (int a = 0; a < 6; ++a) v.root_box[a] = root[a];
    v.root_link = 0;
    v.root_count = 0;
    v.nodes = g.nodes;
    v.num_nodes = ni;
    return GT_OK;
}

} // namespace gt

namespace gt {

// Refit after gt_scene_update_primitives: the updated primitives go to their leaf positions
// and every internal box is recomputed bottom-up along the kept links (the topology, and so
// the leaf order, stays that of the build).
gt_status refit_lbvh_f32(GpuScene<float>& g, uint32_t n, uint32_t count, const uint32_t* index,
                         const PrimRec<float>* recs, const uint2* meta, const float* boxes, cudaStream_t st, int sms) {
    if (count == 0 || n == 0) return GT_OK;
    if (!g.leaf_of) return fail(GT_ERR_INTERNAL, "GPU BVH refit without its build links");
    SceneDev<float>& v = g.view;
    uint32_t* d_index = nullptr;
    PrimRec<float>* d_recs = nullptr;
    uint2* d_meta = nullptr;
    float* d_boxes = nullptr;
    cudaError_t e = cudaMalloc(&d_index, size_t(count) * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&d_recs, size_t(count) * sizeof(PrimRec<float>));
    if (e == cudaSuccess) e = cudaMalloc(&d_meta, size_t(count) * sizeof(uint2));
    if (e == cudaSuccess) e = cudaMalloc(&d_boxes, size_t(count) * 6 * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_index, index, size_t(count) * sizeof(uint32_t), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_recs, recs, size_t(count) * sizeof(PrimRec<float>), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_meta, meta, size_t(count) * sizeof(uint2), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_boxes, boxes, size_t(count) * 6 * sizeof(float), cudaMemcpyHostToDevice, st);
    const int threads = 256;
    const int ublocks = int(std::max<uint64_t>(1, std::min<uint64_t>((count + threads - 1) / threads, uint64_t(sms) * 8)));
    const int blocks = int(std::max<uint64_t>(1, std::min<uint64_t>((n + threads - 1) / threads, uint64_t(sms) * 8)));
    if (e == cudaSuccess) {
        k_update<<<ublocks, threads, 0, st>>>(d_index, d_recs, d_meta, d_boxes, count, g.leaf_of, g.prims, g.meta,
                                              g.leaf_box);
        e = cudaGetLastError();
    }
    float root[6] = {0, 0, 0, 0, 0, 0};
    if (n == 1) {
        if (e == cudaSuccess) e = cudaMemcpyAsync(root, g.leaf_box, sizeof(root), cudaMemcpyDeviceToHost, st);
    } else {
        if (e == cudaSuccess) e = cudaMemsetAsync(g.arrivals, 0, size_t(n - 1) * sizeof(uint32_t), st);
        if (e == cudaSuccess) {
            k_boxes<<<blocks, threads, 0, st>>>(g.leaf_box, int(n), g.parent_leaf, g.parent_int, g.arrivals, g.int_box,
                                                g.nodes);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaMemcpyAsync(root, g.int_box, sizeof(root), cudaMemcpyDeviceToHost, st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(d_index);
    cudaFree(d_recs);
    cudaFree(d_meta);
    cudaFree(d_boxes);
    if (e != cudaSuccess) return cuda_fail(e, "GPU BVH refit");
    for (int a = 0; a < 6; ++a) v.root_box[a] = root[a];
    return GT_OK;
}

} // namespace gt
