// denoise.cu — the learned denoiser: network, training step and inference.
//
// The network is a 5-level U-Net of 3x3 convs (32/48/64/80/96 channels, ReLU, 2x2 average
// pooling, nearest 2x upsampling concatenated with the skip) that maps log(1 + beauty),
// albedo and normal to log(1 + radiance) as a residual over log(1 + beauty).  It is trained
// with L1 on log(1 + x) by Adam, entirely with the kernels of denoise_kernels.cuh.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "denoise_kernels.cuh"
#include "internal.h"

using namespace gt;
using namespace gt::dn;

namespace {

struct Layer {
    int cin, cout; // real channel counts
    int cin_p;     // input channels padded to 16
    int cout_p;    // rows of the forward weights (multiple of 8)
    int cout_pp;   // output channels padded to 16 (gradient width)
    bool relu;
    size_t w_off, b_off; // offsets into the flat FP32 parameter vector
};

constexpr int kLevels = 5;
constexpr int kCh[kLevels] = {32, 48, 64, 80, 96};

std::vector<Layer> make_layers() {
    std::vector<Layer> L;
    auto add = [&](int cin, int cout, bool relu) {
        Layer l;
        l.cin = cin;
        l.cout = cout;
        l.cin_p = (cin + 15) / 16 * 16;
        l.cout_p = (cout + 7) / 8 * 8;
        l.cout_pp = (cout + 15) / 16 * 16;
        l.relu = relu;
        L.push_back(l);
    };
    add(9, kCh[0], true);
    add(kCh[0], kCh[0], true);
    for (int lv = 1; lv < kLevels; ++lv) {
        add(kCh[lv - 1], kCh[lv], true);
        add(kCh[lv], kCh[lv], true);
    }
    for (int lv = kLevels - 2; lv >= 0; --lv) {
        add(kCh[lv + 1] + kCh[lv], kCh[lv], true);
        add(kCh[lv], kCh[lv], true);
    }
    add(kCh[0], 3, false);
    size_t off = 0;
    for (auto& l : L) {
        l.w_off = off;
        off += size_t(l.cout) * 9 * l.cin;
        l.b_off = off;
        off += size_t(l.cout);
    }
    return L;
}

int grid_for(long long count, int threads, int sms) {
    const long long b = (count + threads - 1) / threads;
    return int(std::max<long long>(1, std::min<long long>(b, (long long)sms * 16)));
}

// Layer index of each stage: encoder level lv = 2lv, 2lv+1; decoder level lv (deep to
// shallow) = dec_a(lv), dec_a(lv)+1; then the output conv.
constexpr int enc_a(int lv) { return 2 * lv; }
constexpr int dec_a(int lv) { return 2 * kLevels + 2 * (kLevels - 2 - lv); }
constexpr int kOut = 4 * kLevels - 2;

} // namespace

struct gt_denoiser {
    gt_context* ctx = nullptr;
    std::vector<Layer> layers;
    size_t nparams = 0;
    float* p = nullptr; // master parameters (FP32, flat)
    float* m = nullptr; // Adam moments
    float* v = nullptr;
    float* g = nullptr; // gradient (flat)
    long long step = 0;
    std::vector<__nv_bfloat16*> wb, wf; // forward / input-gradient BF16 weights
    std::vector<float*> dwp;             // padded FP32 weight gradients [cout_pp][9][cin_p]
    float* dbp = nullptr;                // bias gradients (each layer's at its b_off)
    int wg_blocks = 1;                   // weight-gradient CTAs per tap
    float* wpart = nullptr;              // their partial sums [9][wg_blocks][cout_pp][cin_p]
    int bg_blocks = 1;                   // bias-gradient blocks
    float* bpart = nullptr;              // their partial sums [bg_blocks][kBgMaxCh]
    // activations for the current (n, h, w)
    int n = 0, h = 0, w = 0;
    std::vector<void*> bufs;
    __nv_bfloat16* x0 = nullptr;
    float *lb = nullptr, *out = nullptr, *loss = nullptr;
    std::vector<__nv_bfloat16*> act, gact; // per layer output and its gradient
    __nv_bfloat16* pool[kLevels] = {};     // pooled inputs of levels 1..4
    __nv_bfloat16* gpool[kLevels] = {};
    __nv_bfloat16* cat[kLevels] = {};      // decoder concat inputs of levels 0..3
    __nv_bfloat16* gcat[kLevels] = {};
    __nv_bfloat16* gout = nullptr;         // loss gradient (16 channels)
    bool weights_dirty = true;
    // inference staging for the current frame size (h, w unpadded)
    int io_h = 0, io_w = 0;
    std::vector<void*> io;
    float *in_beauty = nullptr, *in_half = nullptr, *in_albedo = nullptr, *in_normal = nullptr;
    float *dn = nullptr, *res = nullptr;
    uint8_t* flags = nullptr;
    uint32_t* flag_count = nullptr;
    uint32_t* err = nullptr; // set by a tensor-core kernel whose mbarrier wait gave up
    bool launch_failed = false; // a convolution could not be launched (tensor map encoding)
};

namespace {

void free_bufs(gt_denoiser* d) {
    for (void* b : d->bufs) cudaFree(b);
    d->bufs.clear();
    d->n = d->h = d->w = 0;
}

void free_io(gt_denoiser* d) {
    for (void* b : d->io) cudaFree(b);
    d->io.clear();
    d->io_h = d->io_w = 0;
}

template <class T> gt_status dalloc(std::vector<void*>& list, T** out, size_t count) {
    void* ptr = nullptr;
    cudaError_t e = cudaMalloc(&ptr, std::max<size_t>(count, 1) * sizeof(T));
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(GT_ERR_OOM, "cannot allocate denoiser buffers");
    }
    list.push_back(ptr);
    *out = static_cast<T*>(ptr);
    return GT_OK;
}
template <class T> gt_status dalloc(gt_denoiser* d, T** out, size_t count) { return dalloc(d->bufs, out, count); }

// Staging for one frame of h x w pixels: inputs (host callers), the denoised image, the
// result and the tile flags (enough for the smallest tile, 4 x 4).
gt_status ensure_io(gt_denoiser* d, int h, int w) {
    if (d->io_h == h && d->io_w == w) return GT_OK;
    free_io(d);
    const size_t n3 = size_t(h) * w * 3;
    gt_status rc;
    if ((rc = dalloc(d->io, &d->in_beauty, n3)) != GT_OK) return rc;
    if ((rc = dalloc(d->io, &d->in_half, n3)) != GT_OK) return rc;
    if ((rc = dalloc(d->io, &d->in_albedo, n3)) != GT_OK) return rc;
    if ((rc = dalloc(d->io, &d->in_normal, n3)) != GT_OK) return rc;
    if ((rc = dalloc(d->io, &d->dn, n3)) != GT_OK) return rc;
    if ((rc = dalloc(d->io, &d->res, n3)) != GT_OK) return rc;
    if ((rc = dalloc(d->io, &d->flags, size_t((h + 3) / 4) * ((w + 3) / 4))) != GT_OK) return rc;
    if ((rc = dalloc(d->io, &d->flag_count, 1)) != GT_OK) return rc;
    d->io_h = h;
    d->io_w = w;
    return GT_OK;
}

gt_status ensure_bufs(gt_denoiser* d, int n, int h, int w) {
    if (d->n == n && d->h == h && d->w == w) return GT_OK;
    free_bufs(d);
    const size_t P0 = size_t(n) * h * w;
    auto P = [&](int lv) { return size_t(n) * (h >> lv) * (w >> lv); };
    gt_status rc;
    if ((rc = dalloc(d, &d->x0, P0 * 16)) != GT_OK) return rc;
    if ((rc = dalloc(d, &d->lb, P0 * 3)) != GT_OK) return rc;
    if ((rc = dalloc(d, &d->out, P0 * 3)) != GT_OK) return rc;
    if ((rc = dalloc(d, &d->loss, 1)) != GT_OK) return rc;
    if ((rc = dalloc(d, &d->gout, P0 * 16)) != GT_OK) return rc;
    d->act.assign(d->layers.size(), nullptr);
    d->gact.assign(d->layers.size(), nullptr);
    for (size_t i = 0; i < d->layers.size(); ++i) {
        if (int(i) == kOut) continue;
        const int lv = i < size_t(2 * kLevels) ? int(i) / 2 : kLevels - 2 - (int(i) - 2 * kLevels) / 2;
        const int c = d->layers[i].cout;
        if ((rc = dalloc(d, &d->act[i], P(lv) * c)) != GT_OK) return rc;
        if ((rc = dalloc(d, &d->gact[i], P(lv) * c)) != GT_OK) return rc;
    }
    for (int lv = 1; lv < kLevels; ++lv) {
        if ((rc = dalloc(d, &d->pool[lv], P(lv) * kCh[lv - 1])) != GT_OK) return rc;
        if ((rc = dalloc(d, &d->gpool[lv], P(lv) * kCh[lv - 1])) != GT_OK) return rc;
    }
    for (int lv = 0; lv < kLevels - 1; ++lv) {
        const int c = kCh[lv + 1] + kCh[lv];
        if ((rc = dalloc(d, &d->cat[lv], P(lv) * c)) != GT_OK) return rc;
        if ((rc = dalloc(d, &d->gcat[lv], P(lv) * c)) != GT_OK) return rc;
    }
    d->n = n;
    d->h = h;
    d->w = w;
    return GT_OK;
}

gt_status refresh_weights(gt_denoiser* d, cudaStream_t st) {
    if (!d->weights_dirty) return GT_OK;
    const int sms = d->ctx->num_sms > 0 ? d->ctx->num_sms : 1;
    for (size_t i = 0; i < d->layers.size(); ++i) {
        const Layer& l = d->layers[i];
        const long long cnt = (long long)l.cout_p * 9 * l.cin_p + (long long)l.cin_p * 9 * l.cout_pp;
        k_weights_bf16<<<grid_for(cnt, 256, sms), 256, 0, st>>>(d->p + l.w_off, l.cout, l.cin, d->wb[i], l.cout_p,
                                                                 l.cin_p, d->wf[i], l.cout_pp);
    }
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "denoiser weights");
    d->weights_dirty = false;
    return GT_OK;
}

// Tile shape of a tensor-core convolution with N output channels: rows per CTA (each row's
// accumulator takes a power-of-two range of TMEM columns, at most 512 in all) and pipeline
// stages (2 while two CTAs fit in an SM's tensor memory, else 3).
struct TcShape {
    int rows, stride, stages;
};
constexpr TcShape tc_shape_rows(int n, int rows) {
    return TcShape{rows, tc_pow2_cols(n), rows * tc_pow2_cols(n) <= 256 ? 2 : 3};
}
constexpr TcShape tc_shape(int n) { return tc_shape_rows(n, tc_pow2_cols(n) <= 128 ? 4 : 2); }
// Largest shared-memory request (N = 176, the input gradient of the deepest decoder layer,
// and N = 96).
constexpr int kTcSmemMax =
    tc_smem_bytes(176, tc_shape(176).rows, tc_shape(176).stages) > tc_smem_bytes(96, tc_shape(96).rows, tc_shape(96).stages)
        ? tc_smem_bytes(176, tc_shape(176).rows, tc_shape(176).stages)
        : tc_smem_bytes(96, tc_shape(96).rows, tc_shape(96).stages);
static_assert(kTcSmemMax <= 227 * 1024, "tensor-core convolution needs more shared memory than a CTA has");

// cuTensorMapEncodeTiled from the driver, looked up once through the runtime.
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled() {
    static EncodeTiledFn fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<EncodeTiledFn>(p);
    }();
    return fn;
}

// BF16 tensor map of `rank` dimensions (innermost first), unit element strides, no swizzle,
// zero fill outside the tensor.
bool encode_bf16(CUtensorMap* m, const void* base, int rank, const cuuint64_t* dims, const cuuint64_t* strides,
                 const cuuint32_t* box) {
    const EncodeTiledFn fn = encode_tiled();
    if (!fn) return false;
    const cuuint32_t es[5] = {1, 1, 1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, cuuint32_t(rank), const_cast<void*>(base), dims, strides, box, es,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Launches a tensor-core convolution: TMA staging when the input is one tensor, per-thread
// staging when it is read as an upsampled half plus a skip tensor.
gt_status launch_conv_tc(gt_denoiser* d, ConvTc a, cudaStream_t st) {
    a.n_mma = (a.cout_p + 15) / 16 * 16;
    // Rows per CTA: the most that tensor memory allows, halved while the grid would give
    // fewer than two CTAs per SM (the deep, small levels).
    TcShape sh = tc_shape(a.n_mma);
    const int sms = d->ctx->num_sms > 0 ? d->ctx->num_sms : 1;
    const int segs = (a.w + kTcM - 1) / kTcM;
    while (sh.rows > 1 && segs * ((a.h + sh.rows - 1) / sh.rows) * a.n < 2 * sms)
        sh = tc_shape_rows(a.n_mma, sh.rows / 2);
    a.rows = sh.rows;
    a.acc_stride = sh.stride;
    a.stages = sh.stages;
    a.tmem_cols = uint32_t(sh.rows * sh.stride);
    a.err = d->err;
    const int grid = (a.w + kTcM - 1) / kTcM * ((a.h + a.rows - 1) / a.rows) * a.n;
    const int smem = tc_smem_bytes(a.n_mma, a.rows, a.stages);
    if (!a.lo) {
        ConvTma t;
        std::memset(&t, 0, sizeof(t));
        const cuuint64_t xd[4] = {cuuint64_t(a.cin), cuuint64_t(a.w), cuuint64_t(a.h), cuuint64_t(a.n)};
        const cuuint64_t xs[3] = {cuuint64_t(a.cin) * 2, cuuint64_t(a.w) * a.cin * 2,
                                  cuuint64_t(a.h) * a.w * a.cin * 2};
        const cuuint32_t xb[4] = {8, 130, 1, 1};
        const cuuint64_t wd[3] = {cuuint64_t(a.cin), 9, cuuint64_t(a.cout_p)};
        const cuuint64_t ws[2] = {cuuint64_t(a.cin) * 2, cuuint64_t(a.cin) * 2 * 9};
        const cuuint32_t wb[3] = {8, 1, cuuint32_t(a.n_mma)};
        if (!encode_bf16(&t.x, a.x, 4, xd, xs, xb) || !encode_bf16(&t.wt, a.wt, 3, wd, ws, wb))
            return fail(GT_ERR_CUDA, "cannot encode the denoiser's tensor maps");
        t.cin = a.cin;
        t.cout_p = a.cout_p;
        t.n_mma = a.n_mma;
        t.cout = a.cout;
        t.bias = a.bias;
        t.y = a.y;
        t.ldy = a.ldy;
        t.yoff = a.yoff;
        t.yf = a.yf;
        t.res = a.res;
        t.relu = a.relu;
        t.n = a.n;
        t.h = a.h;
        t.w = a.w;
        t.rows = a.rows;
        t.acc_stride = a.acc_stride;
        t.stages = a.stages;
        t.tmem_cols = a.tmem_cols;
        t.err = a.err;
        k_conv_fwd_tma<<<grid, 128, smem, st>>>(t);
    } else {
        k_conv_fwd_tc<<<grid, 128, smem, st>>>(a);
    }
    return GT_OK;
}

void conv(gt_denoiser* d, int li, const __nv_bfloat16* x, __nv_bfloat16* y, int ldy, float* yf, const float* res,
          int lv, cudaStream_t st, const __nv_bfloat16* lo = nullptr, int cl = 0) {
    const Layer& l = d->layers[li];
    ConvTc a;
    std::memset(&a, 0, sizeof(a));
    a.x = x;
    a.lo = lo;
    a.cl = cl;
    a.cin = l.cin_p;
    a.wt = d->wb[li];
    a.bias = d->p + l.b_off;
    a.cout_p = l.cout_p;
    a.cout = l.cout;
    a.y = y;
    a.ldy = ldy;
    a.yf = yf;
    a.res = res;
    a.relu = l.relu ? 1 : 0;
    a.n = d->n;
    a.h = d->h >> lv;
    a.w = d->w >> lv;
    if (launch_conv_tc(d, a, st) != GT_OK) d->launch_failed = true;
}

// Input gradient: the same convolution over dY with the flipped, transposed weights, no
// bias or ReLU.
void conv_dgrad(gt_denoiser* d, int li, const __nv_bfloat16* dy, __nv_bfloat16* dx, int lv, cudaStream_t st) {
    const Layer& l = d->layers[li];
    ConvTc a;
    std::memset(&a, 0, sizeof(a));
    a.x = dy;
    a.cin = l.cout_pp;
    a.wt = d->wf[li];
    a.cout_p = l.cin_p;
    a.cout = l.cin;
    a.y = dx;
    a.ldy = l.cin;
    a.n = d->n;
    a.h = d->h >> lv;
    a.w = d->w >> lv;
    if (launch_conv_tc(d, a, st) != GT_OK) d->launch_failed = true;
}

gt_status check_err(gt_denoiser* d, cudaStream_t st) {
    if (d->launch_failed) {
        d->launch_failed = false;
        return fail(GT_ERR_CUDA, "cannot encode the denoiser's tensor maps");
    }
    cudaError_t e = cudaMemcpyAsync(d->ctx->pinned, d->err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "denoiser");
    if (d->ctx->pinned[0] & 2u) return fail(GT_ERR_INTERNAL, "denoiser shared memory is not 128-byte aligned");
    if (d->ctx->pinned[0]) return fail(GT_ERR_TIMEOUT, "denoiser tensor-core pipeline wait timed out");
    return GT_OK;
}

// Weight and bias gradients of layer li: per-CTA partial sums reduced in a fixed order, so
// the gradient does not depend on the order in which the CTAs run.
void conv_wgrad(gt_denoiser* d, int li, const __nv_bfloat16* dy, const __nv_bfloat16* x, int lv, cudaStream_t st) {
    const Layer& l = d->layers[li];
    ConvWgradTc a;
    a.dy = dy;
    a.cout = l.cout_pp;
    a.x = x;
    a.cin = l.cin_p;
    a.n = d->n;
    a.h = d->h >> lv;
    a.w = d->w >> lv;
    const long long P = (long long)a.n * a.h * a.w;
    const long long chunks = (P + kWgK - 1) / kWgK;
    a.blocks = int(std::max<long long>(1, std::min<long long>(chunks, d->wg_blocks)));
    a.part = d->wpart;
    a.tmem_cols = uint32_t(tc_pow2_cols(a.cin));
    a.err = d->err;
    // At 256 tensor-memory columns a CTA asks for a third of the SM's shared memory, so
    // that no more than two (512 columns) share an SM and none waits in tcgen05.alloc.
    const int smem = a.tmem_cols == 256 ? std::max(wg_smem_bytes(a.cin), kWgSmemTwoPerSm) : wg_smem_bytes(a.cin);
    k_conv_wgrad_tc<<<dim3(a.blocks, 9), 128, smem, st>>>(a);
    const int sms = d->ctx->num_sms > 0 ? d->ctx->num_sms : 1;
    k_wgrad_reduce<<<grid_for(9LL * a.cout * a.cin, 256, sms), 256, 0, st>>>(d->wpart, a.blocks, a.cout, a.cin,
                                                                             d->dwp[li]);
    const int bblocks = int(std::max<long long>(1, std::min<long long>(P, d->bg_blocks)));
    k_bias_grad<<<bblocks, 128, 0, st>>>(dy, l.cout_pp, l.cout, P, d->bpart);
    k_bias_reduce<<<1, 128, 0, st>>>(d->bpart, bblocks, l.cout, d->dbp + l.b_off);
}

// Forward pass (inputs already packed); d->out = log-space prediction.  Training keeps the
// decoder's concatenated inputs for the weight gradients; inference reads the upsampled
// half and the skip straight into the convolution's staging.
void forward(gt_denoiser* d, cudaStream_t st, bool training) {
    const int sms = d->ctx->num_sms > 0 ? d->ctx->num_sms : 1;
    const __nv_bfloat16* in = d->x0;
    for (int lv = 0; lv < kLevels; ++lv) {
        if (lv > 0) {
            const int c = kCh[lv - 1], hh = d->h >> (lv - 1), ww = d->w >> (lv - 1);
            k_pool<<<grid_for((long long)d->n * (hh / 2) * (ww / 2) * c, 256, sms), 256, 0, st>>>(
                d->act[enc_a(lv - 1) + 1], d->pool[lv], d->n, hh, ww, c);
            in = d->pool[lv];
        }
        conv(d, enc_a(lv), in, d->act[enc_a(lv)], kCh[lv], nullptr, nullptr, lv, st);
        conv(d, enc_a(lv) + 1, d->act[enc_a(lv)], d->act[enc_a(lv) + 1], kCh[lv], nullptr, nullptr, lv, st);
    }
    const __nv_bfloat16* lo = d->act[enc_a(kLevels - 1) + 1];
    for (int lv = kLevels - 2; lv >= 0; --lv) {
        const int cl = kCh[lv + 1], cs = kCh[lv], hh = d->h >> lv, ww = d->w >> lv;
        if (training) {
            k_upcat<<<grid_for((long long)d->n * hh * ww * (cl + cs), 256, sms), 256, 0, st>>>(
                lo, cl, d->act[enc_a(lv) + 1], cs, d->cat[lv], d->n, hh, ww);
            conv(d, dec_a(lv), d->cat[lv], d->act[dec_a(lv)], kCh[lv], nullptr, nullptr, lv, st);
        } else {
            conv(d, dec_a(lv), d->act[enc_a(lv) + 1], d->act[dec_a(lv)], kCh[lv], nullptr, nullptr, lv, st, lo, cl);
        }
        conv(d, dec_a(lv) + 1, d->act[dec_a(lv)], d->act[dec_a(lv) + 1], kCh[lv], nullptr, nullptr, lv, st);
        lo = d->act[dec_a(lv) + 1];
    }
    conv(d, kOut, lo, nullptr, 0, d->out, d->lb, 0, st);
}

// Backward pass from d->gout (the loss gradient); parameter gradients into d->g.
gt_status backward(gt_denoiser* d, cudaStream_t st) {
    const int sms = d->ctx->num_sms > 0 ? d->ctx->num_sms : 1;
    for (size_t i = 0; i < d->layers.size(); ++i) {
        const Layer& l = d->layers[i];
        cudaMemsetAsync(d->dwp[i], 0, size_t(l.cout_pp) * 9 * l.cin_p * sizeof(float), st);
    }
    cudaMemsetAsync(d->dbp, 0, d->nparams * sizeof(float), st);
    auto relu_bwd = [&](__nv_bfloat16* g, const __nv_bfloat16* y, long long count) {
        k_relu_bwd<<<grid_for(count, 256, sms), 256, 0, st>>>(g, y, count);
    };
    auto P = [&](int lv) { return (long long)d->n * (d->h >> lv) * (d->w >> lv); };
    // output conv
    conv_wgrad(d, kOut, d->gout, d->act[dec_a(0) + 1], 0, st);
    conv_dgrad(d, kOut, d->gout, d->gact[dec_a(0) + 1], 0, st);
    // decoder, shallowest level first
    for (int lv = 0; lv <= kLevels - 2; ++lv) {
        const int b = dec_a(lv);
        relu_bwd(d->gact[b + 1], d->act[b + 1], P(lv) * kCh[lv]);
        conv_wgrad(d, b + 1, d->gact[b + 1], d->act[b], lv, st);
        conv_dgrad(d, b + 1, d->gact[b + 1], d->gact[b], lv, st);
        relu_bwd(d->gact[b], d->act[b], P(lv) * kCh[lv]);
        conv_wgrad(d, b, d->gact[b], d->cat[lv], lv, st);
        conv_dgrad(d, b, d->gact[b], d->gcat[lv], lv, st);
        // the upsampled half feeds the deeper level's output, the skip half this level's
        // encoder output (written here; the pool's gradient is added below)
        const int cl = kCh[lv + 1], cs = kCh[lv];
        __nv_bfloat16* dlo = lv + 1 <= kLevels - 2 ? d->gact[dec_a(lv + 1) + 1] : d->gact[enc_a(kLevels - 1) + 1];
        k_upcat_bwd<<<grid_for(P(lv + 1) * cl + P(lv) * cs, 256, sms), 256, 0, st>>>(
            d->gcat[lv], cl, cs, dlo, d->gact[enc_a(lv) + 1], d->n, d->h >> lv, d->w >> lv);
    }
    // encoder, deepest level first
    for (int lv = kLevels - 1; lv >= 0; --lv) {
        const int a = enc_a(lv);
        relu_bwd(d->gact[a + 1], d->act[a + 1], P(lv) * kCh[lv]);
        conv_wgrad(d, a + 1, d->gact[a + 1], d->act[a], lv, st);
        conv_dgrad(d, a + 1, d->gact[a + 1], d->gact[a], lv, st);
        relu_bwd(d->gact[a], d->act[a], P(lv) * kCh[lv]);
        conv_wgrad(d, a, d->gact[a], lv > 0 ? d->pool[lv] : d->x0, lv, st);
        if (lv > 0) {
            conv_dgrad(d, a, d->gact[a], d->gpool[lv], lv, st);
            const int c = kCh[lv - 1], hh = d->h >> (lv - 1), ww = d->w >> (lv - 1);
            k_pool_bwd<<<grid_for(P(lv - 1) * c, 256, sms), 256, 0, st>>>(d->gpool[lv], d->gact[enc_a(lv - 1) + 1],
                                                                           d->n, hh, ww, c);
        }
    }
    for (size_t i = 0; i < d->layers.size(); ++i) {
        const Layer& l = d->layers[i];
        k_gather_grad<<<grid_for((long long)l.cout * 9 * l.cin + l.cout, 256, sms), 256, 0, st>>>(
            d->dwp[i], l.cout, l.cin, l.cin_p, d->dbp + l.b_off, d->g + l.w_off);
    }
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "denoiser backward");
    return GT_OK;
}

// He-normal initialisation from a SplitMix64 stream (Box-Muller); biases 0.  The output
// conv starts small, so the untrained network returns nearly its input.
void init_params(std::vector<float>& host, const std::vector<Layer>& L, uint64_t seed) {
    uint64_t s = seed;
    auto next = [&]() {
        s += 0x9e3779b97f4a7c15ULL;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
        return z ^ (z >> 31);
    };
    auto unit = [&]() { return (double(next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); };
    for (const Layer& l : L) {
        const double sd = std::sqrt(2.0 / (9.0 * l.cin)) * (l.relu ? 1.0 : 0.1);
        for (size_t i = 0; i < size_t(l.cout) * 9 * l.cin; ++i) {
            const double u1 = unit(), u2 = unit();
            host[l.w_off + i] = float(sd * std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2));
        }
        for (int i = 0; i < l.cout; ++i) host[l.b_off + i] = 0.f;
    }
}

gt_status check_image(long long n, long long h, long long w) {
    if (n <= 0 || h <= 0 || w <= 0 || h % 16 || w % 16)
        return fail(GT_ERR_INVALID_ARG, "denoiser images need a positive size with height and width multiples of 16");
    if (n * h * w > (1LL << 28)) return fail(GT_ERR_INVALID_ARG, "denoiser batch too large");
    return GT_OK;
}

} // namespace

extern "C" {

gt_status gt_denoiser_create(gt_context* ctx, uint64_t seed, gt_denoiser** out) {
    GT_GUARD_BEGIN
    if (!ctx || !out) return fail(GT_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    GT_CONTEXT_LOCK(ctx);
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    auto* d = new gt_denoiser();
    d->ctx = ctx;
    d->layers = make_layers();
    const Layer& last = d->layers.back();
    d->nparams = last.b_off + last.cout;
    std::vector<float> host(d->nparams);
    init_params(host, d->layers, seed);
    auto al = [&](void** p, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(p, bytes);
        if (e == cudaSuccess) e = cudaMemset(*p, 0, bytes);
    };
    al(reinterpret_cast<void**>(&d->p), d->nparams * sizeof(float));
    al(reinterpret_cast<void**>(&d->m), d->nparams * sizeof(float));
    al(reinterpret_cast<void**>(&d->v), d->nparams * sizeof(float));
    al(reinterpret_cast<void**>(&d->g), d->nparams * sizeof(float));
    al(reinterpret_cast<void**>(&d->dbp), d->nparams * sizeof(float));
    al(reinterpret_cast<void**>(&d->err), sizeof(uint32_t));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_conv_fwd_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmemMax);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_conv_fwd_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmemMax);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_conv_wgrad_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 std::max(wg_smem_bytes(kWgMaxN), kWgSmemTwoPerSm));
    // Two weight-gradient CTAs fit an SM (shared memory): about two per SM over the 9 taps.
    const int sms = ctx->num_sms > 0 ? ctx->num_sms : 1;
    d->wg_blocks = std::max(1, (2 * sms + 8) / 9);
    d->bg_blocks = sms * 8;
    size_t part_max = 0;
    for (const Layer& l : d->layers) part_max = std::max(part_max, size_t(l.cout_pp) * l.cin_p);
    al(reinterpret_cast<void**>(&d->wpart), 9 * size_t(d->wg_blocks) * part_max * sizeof(float));
    al(reinterpret_cast<void**>(&d->bpart), size_t(d->bg_blocks) * kBgMaxCh * sizeof(float));
    d->wb.assign(d->layers.size(), nullptr);
    d->wf.assign(d->layers.size(), nullptr);
    d->dwp.assign(d->layers.size(), nullptr);
    for (size_t i = 0; i < d->layers.size(); ++i) {
        const Layer& l = d->layers[i];
        al(reinterpret_cast<void**>(&d->wb[i]), size_t(l.cout_p) * 9 * l.cin_p * sizeof(__nv_bfloat16));
        al(reinterpret_cast<void**>(&d->wf[i]), size_t(l.cin_p) * 9 * l.cout_pp * sizeof(__nv_bfloat16));
        al(reinterpret_cast<void**>(&d->dwp[i]), size_t(l.cout_pp) * 9 * l.cin_p * sizeof(float));
    }
    if (e == cudaSuccess) e = cudaMemcpy(d->p, host.data(), d->nparams * sizeof(float), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        gt_denoiser_destroy(d);
        return cuda_fail(e, "denoiser allocation");
    }
    *out = d;
    return GT_OK;
    GT_GUARD_END
}

static void destroy_denoiser(gt_denoiser* d) {
    cudaSetDevice(d->ctx->device);
    cudaStreamSynchronize(d->ctx->stream);
    free_bufs(d);
    free_io(d);
    cudaFree(d->p);
    cudaFree(d->m);
    cudaFree(d->v);
    cudaFree(d->g);
    cudaFree(d->dbp);
    cudaFree(d->err);
    cudaFree(d->wpart);
    cudaFree(d->bpart);
    for (auto* p : d->wb) cudaFree(p);
    for (auto* p : d->wf) cudaFree(p);
    for (auto* p : d->dwp) cudaFree(p);
    delete d;
}

void gt_denoiser_destroy(gt_denoiser* d) {
    if (!d) return;
    gt::destroy_or_defer(d->ctx, [d] { destroy_denoiser(d); });
}


gt_status gt_denoiser_param_count(const gt_denoiser* d, uint64_t* count) {
    if (!d || !count) return fail(GT_ERR_INVALID_ARG, "null argument");
    *count = d->nparams;
    return GT_OK;
}

gt_status gt_denoiser_get_params(const gt_denoiser* d, float* host, uint64_t count) {
    GT_GUARD_BEGIN
    if (!d || !host) return fail(GT_ERR_INVALID_ARG, "null argument");
    if (count != d->nparams) return fail(GT_ERR_INVALID_ARG, "parameter count differs from the network's");
    GT_CONTEXT_LOCK(d->ctx);
    cudaSetDevice(d->ctx->device);
    const cudaError_t e = cudaMemcpy(host, d->p, count * sizeof(float), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "denoiser parameters");
    return GT_OK;
    GT_GUARD_END
}

gt_status gt_denoiser_set_params(gt_denoiser* d, const float* host, uint64_t count) {
    GT_GUARD_BEGIN
    if (!d || !host) return fail(GT_ERR_INVALID_ARG, "null argument");
    if (count != d->nparams) return fail(GT_ERR_INVALID_ARG, "parameter count differs from the network's");
    for (uint64_t i = 0; i < count; ++i)
        if (!std::isfinite(host[i])) return fail(GT_ERR_INVALID_ARG, "denoiser parameters must be finite");
    GT_CONTEXT_LOCK(d->ctx);
    cudaSetDevice(d->ctx->device);
    cudaError_t e = cudaMemcpy(d->p, host, count * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(d->m, 0, count * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(d->v, 0, count * sizeof(float));
    if (e != cudaSuccess) return cuda_fail(e, "denoiser parameters");
    d->step = 0;
    d->weights_dirty = true;
    return GT_OK;
    GT_GUARD_END
}

gt_status gt_denoiser_train_step(gt_denoiser* d, const float* beauty, const float* albedo, const float* normal,
                                 const float* target, uint32_t n, uint32_t h, uint32_t w, float lr, float* loss,
                                 float* grad) {
    GT_GUARD_BEGIN
    if (!d || !beauty || !target) return fail(GT_ERR_INVALID_ARG, "null argument");
    gt_status rc = check_image(n, h, w);
    if (rc != GT_OK) return rc;
    if (!(lr >= 0.f) || !std::isfinite(lr)) return fail(GT_ERR_INVALID_ARG, "learning rate must be finite and >= 0");
    GT_CONTEXT_LOCK(d->ctx);
    cudaSetDevice(d->ctx->device);
    const cudaStream_t st = d->ctx->stream;
    if ((rc = ensure_bufs(d, int(n), int(h), int(w))) != GT_OK) return rc;
    if ((rc = refresh_weights(d, st)) != GT_OK) return rc;
    const int sms = d->ctx->num_sms > 0 ? d->ctx->num_sms : 1;
    const long long P = (long long)n * h * w;
    cudaMemsetAsync(d->err, 0, sizeof(uint32_t), st);
    k_pack_input<<<grid_for(P, 256, sms), 256, 0, st>>>(beauty, albedo, normal, int(n), int(h), int(w), int(h),
                                                         int(w), d->x0, d->lb);
    forward(d, st, true);
    cudaMemsetAsync(d->loss, 0, sizeof(float), st);
    k_l1_log1p<<<grid_for(P, 256, sms), 256, 0, st>>>(d->out, target, P, d->loss, d->gout);
    if ((rc = backward(d, st)) != GT_OK) return rc;
    if (lr > 0.f) {
        d->step += 1;
        const float c1 = 1.f - std::pow(0.9f, float(d->step)), c2 = 1.f - std::pow(0.999f, float(d->step));
        k_adam<<<grid_for((long long)d->nparams, 256, sms), 256, 0, st>>>(d->p, d->m, d->v, d->g,
                                                                          (long long)d->nparams, lr, 0.9f, 0.999f,
                                                                          1e-8f, c1, c2);
        d->weights_dirty = true;
    }
    float l = 0.f;
    cudaError_t e = cudaMemcpyAsync(&l, d->loss, sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && grad)
        e = cudaMemcpyAsync(grad, d->g, d->nparams * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "denoiser training step");
    if ((rc = check_err(d, st)) != GT_OK) return rc;
    if (loss) *loss = l;
    return GT_OK;
    GT_GUARD_END
}

gt_status gt_denoise(gt_denoiser* d, const gt_denoise_input* in, uint32_t tile, float threshold, float* out,
                     uint8_t* tile_fallback, uint32_t* fallback_count) {
    GT_GUARD_BEGIN
    if (!d || !in || !out) return fail(GT_ERR_INVALID_ARG, "null argument");
    if (in->struct_size < sizeof(gt_denoise_input)) return fail(GT_ERR_INVALID_ARG, "gt_denoise_input.struct_size too small");
    if (!in->beauty) return fail(GT_ERR_INVALID_ARG, "beauty image is required");
    if (in->device_buffers > 1) return fail(GT_ERR_INVALID_ARG, "device_buffers must be 0 or 1");
    const long long h = in->height, w = in->width;
    if (h <= 0 || w <= 0 || h * w > (1LL << 26)) return fail(GT_ERR_INVALID_ARG, "image size out of range");
    if (tile == 0) tile = 16;
    if (tile < 4 || tile > 256) return fail(GT_ERR_INVALID_ARG, "tile must be 0 or in [4, 256]");
    if (threshold == 0.f) threshold = 3.f;
    if (!(threshold > 0.f) || !std::isfinite(threshold)) return fail(GT_ERR_INVALID_ARG, "threshold must be finite and > 0");
    const int hp = int((h + 15) / 16 * 16), wp = int((w + 15) / 16 * 16);
    const int tiles = int(((h + tile - 1) / tile) * ((w + tile - 1) / tile));
    GT_CONTEXT_LOCK(d->ctx);
    cudaError_t e = cudaSetDevice(d->ctx->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    const cudaStream_t st = d->ctx->stream;
    gt_status rc;
    if ((rc = ensure_bufs(d, 1, hp, wp)) != GT_OK) return rc;
    if ((rc = ensure_io(d, int(h), int(w))) != GT_OK) return rc;
    if ((rc = refresh_weights(d, st)) != GT_OK) return rc;
    const size_t bytes = size_t(h) * w * 3 * sizeof(float);
    const float *beauty = in->beauty, *half = in->beauty_half, *albedo = in->albedo, *normal = in->normal;
    if (!in->device_buffers) {
        auto up = [&](const float* src, float* dst) -> const float* {
            if (!src) return nullptr;
            if (e == cudaSuccess) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st);
            return dst;
        };
        beauty = up(beauty, d->in_beauty);
        half = up(half, d->in_half);
        albedo = up(albedo, d->in_albedo);
        normal = up(normal, d->in_normal);
        if (e != cudaSuccess) return cuda_fail(e, "denoiser input copy");
    }
    float* result = in->device_buffers ? out : d->res;
    const int sms = d->ctx->num_sms > 0 ? d->ctx->num_sms : 1;
    cudaMemsetAsync(d->err, 0, sizeof(uint32_t), st);
    k_pack_input<<<grid_for((long long)hp * wp, 256, sms), 256, 0, st>>>(beauty, albedo, normal, 1, int(h), int(w), hp,
                                                                          wp, d->x0, d->lb);
    forward(d, st, false);
    k_unpack_output<<<grid_for(h * w * 3, 256, sms), 256, 0, st>>>(d->out, int(h), int(w), wp, half ? d->dn : result);
    if (half) {
        cudaMemsetAsync(d->flag_count, 0, sizeof(uint32_t), st);
        k_tile_fallback<<<tiles, 256, 0, st>>>(d->dn, beauty, half, int(h), int(w), int(tile), threshold, result,
                                               d->flags, d->flag_count);
    }
    e = cudaGetLastError();
    if (e == cudaSuccess && !in->device_buffers) e = cudaMemcpyAsync(out, result, bytes, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && half && tile_fallback)
        e = cudaMemcpyAsync(tile_fallback, d->flags, size_t(tiles), cudaMemcpyDeviceToHost, st);
    uint32_t count = 0;
    if (e == cudaSuccess && half) e = cudaMemcpyAsync(d->ctx->pinned, d->flag_count, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "denoise");
    if (half) count = d->ctx->pinned[0];
    if ((rc = check_err(d, st)) != GT_OK) return rc;
    if (!half && tile_fallback) std::memset(tile_fallback, 0, size_t(tiles));
    if (fallback_count) *fallback_count = count;
    return GT_OK;
    GT_GUARD_END
}

} // extern "C"
