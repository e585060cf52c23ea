// denoise_kernels.cuh — kernels of the learned denoiser: a 5-level U-Net of 3x3 convs over
// the beauty / albedo / normal AOVs (render_denoising_aovs, renderer.rs:121-129).
//
// Tensors are NHWC.  Activations and weights are BF16; every product is accumulated in FP32
// on the tensor cores.  A 3x3 conv is an implicit GEMM: M = pixels, N = output channels,
// K = 9 taps x input channels (k_conv_fwd_tc: tcgen05.mma with the accumulator in tensor
// memory).  Its input gradient is the same GEMM with the taps flipped and the channel roles
// swapped; its weight gradient is a GEMM over pixels (M = output channels, N = input
// channels, K = pixels; k_conv_wgrad_tc, tcgen05.mma, reduced in a fixed order by
// k_wgrad_reduce).
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace gt {
namespace dn {

__device__ __forceinline__ uint32_t lane() { return threadIdx.x & 31u; }

__device__ __forceinline__ uint32_t pack_bf16(__nv_bfloat16 lo, __nv_bfloat16 hi) {
    return uint32_t(__bfloat16_as_ushort(lo)) | (uint32_t(__bfloat16_as_ushort(hi)) << 16);
}

// D += A (16x16, row) * B (16x8, col), BF16 in, FP32 accumulate.
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Two consecutive BF16 channels (c even) of pixel (n, y, x), 0 outside the image.
__device__ __forceinline__ uint32_t ld2(const __nv_bfloat16* t, int c_stride, int n, int y, int x, int h, int w,
                                        int c) {
    if (y < 0 || y >= h || x < 0 || x >= w) return 0u;
    return __ldg(reinterpret_cast<const unsigned int*>(t + ((size_t(n) * h + y) * w + x) * c_stride + c));
}

// ------------------------------------------------------------ tcgen05 convolution
// The 3x3 convolution on the 5th-generation tensor cores.  One CTA computes R consecutive
// output rows (R = 4, or 2 for wide layers) of 128 consecutive pixels (M = 128 per MMA)
// for all N output channels, each row's D[pixel][co] accumulating in its own range of
// tensor-memory columns (FP32).  K runs over 16-channel chunks of the input; each chunk is
// staged once in shared memory as
//   A: the R + 2 input rows y0-1 .. y0+R, pixels x0-1 .. x0+128 (130 staged rows per input
//      row),
//   B: the chunk's weights for all 9 taps,
// in the K-major no-swizzle core-matrix layout (8 rows x 16 bytes per core matrix).  The
// staged pixels of one input row are contiguous at 16 bytes per pixel within each
// 8-channel half, so the operand of horizontal tap dx is the same tile with its start
// address moved by (dx + 1) x 16 bytes, and vertical tap dy of output row r is staged row
// r + dy + 1: 9R MMAs per chunk read R + 2 staged rows and one set of weights.  Two or three
// stages overlap the next chunks' loads (cp.async, zero-filled outside the image) with the
// MMAs, which one thread issues and commits to a per-stage mbarrier.
constexpr int kTcM = 128;                     // pixels per MMA
constexpr int kTcRows = 136;                  // staged pixels per input row (130 used)
constexpr int kTcRowBytes = kTcRows * 16;     // one 8-channel half of one staged row
constexpr int kTcATile = 2 * kTcRowBytes;     // one input row, 16 channels
constexpr int kTcMaxStages = 3;
constexpr uint32_t kTcWaitLimit = 1u << 22;   // mbarrier polls before giving up

__host__ __device__ constexpr int tc_stage_bytes(int n, int rows) {
    return ((rows + 2) * kTcATile + 9 * n * 32 + 127) / 128 * 128;
}
__host__ __device__ constexpr int tc_smem_bytes(int n, int rows, int stages) {
    return 128 + stages * tc_stage_bytes(n, rows);
}
__host__ __device__ constexpr int tc_pow2_cols(int n) { return n <= 32 ? 32 : n <= 64 ? 64 : n <= 128 ? 128 : 256; }

struct ConvTc {
    const __nv_bfloat16* x; // [n][h][w][cin]
    int cin;                // multiple of 16
    const __nv_bfloat16* wt; // [cout_p][9][cin]
    const float* bias;      // [cout] or null
    int cout_p;             // rows of wt
    int n_mma;              // MMA N: cout_p rounded up to 16 (rows >= cout_p are zero)
    int cout;               // channels stored
    __nv_bfloat16* y;       // [n][h][w][ldy] at channel offset yoff, or null
    int ldy, yoff;
    float* yf;              // [n][h][w][cout] FP32 output, or null
    const float* res;       // FP32 residual added to yf, or null
    int relu;
    int n, h, w;
    const __nv_bfloat16* lo; // optional: input channels [0, cl) are the 2x nearest upsampling of
    int cl;                  // lo ([n][h/2][w/2][cl]) and the rest come from x ([n][h][w][cin - cl])
    int rows;               // output rows per CTA (R)
    int acc_stride;         // TMEM columns per row accumulator (power of two >= n_mma)
    int stages;             // 2 or 3
    uint32_t tmem_cols;     // TMEM columns allocated (rows * acc_stride)
    uint32_t* err;          // set to 1 if an mbarrier wait gave up
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return uint32_t(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, uint32_t bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(bytes) : "memory");
}

__device__ __forceinline__ void cp_async_wait_pending(int pending) {
    if (pending <= 0) asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    else if (pending == 1) asm volatile("cp.async.wait_group 1;\n" ::: "memory");
    else asm volatile("cp.async.wait_group 2;\n" ::: "memory");
}

// Shared-memory matrix descriptor (K-major, no swizzle): start, leading-dimension byte
// offset (between core matrices adjacent in K), stride byte offset (between 8-row groups),
// descriptor version 1 at bits 46-47, layout type 0 (no swizzle) at bits 61-63.
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return uint64_t((addr >> 4) & 0x3FFFu) | (uint64_t((lbo >> 4) & 0x3FFFu) << 16) |
           (uint64_t((sbo >> 4) & 0x3FFFu) << 32) | (uint64_t(1) << 46);
}

// Instruction descriptor, kind::f16: FP32 accumulator (bits 4-5 = 1), A and B BF16 (bits
// 7-9 and 10-12 = 1), both K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28.
__device__ __forceinline__ uint32_t tc_idesc(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(n >> 3) << 17) | (uint32_t(kTcM >> 4) << 24);
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t addr, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(addr), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait: false (and *err = 1) if the phase did not complete within the limit.
__device__ __forceinline__ bool mbar_wait(uint32_t addr, uint32_t parity, uint32_t* err) {
    for (uint32_t i = 0; i < kTcWaitLimit; ++i)
        if (mbar_try_wait(addr, parity)) return true;
    atomicOr(err, 1u);
    return false;
}

__global__ void __launch_bounds__(128) k_conv_fwd_tc(ConvTc a) {
    extern __shared__ __align__(128) uint8_t smem[];
    uint64_t* mbar = reinterpret_cast<uint64_t*>(smem); // kTcMaxStages barriers
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + 64);
    const int N = a.n_mma, R = a.rows, S = a.stages;
    const int stage_bytes = tc_stage_bytes(N, R);
    const int a_bytes = (R + 2) * kTcATile;
    uint8_t* stage_base = smem + 128;
    const int segs = (a.w + kTcM - 1) / kTcM, groups = (a.h + R - 1) / R;
    const int seg = blockIdx.x % segs, rg = (blockIdx.x / segs) % groups, img = blockIdx.x / (segs * groups);
    const int y0 = rg * R, x0 = seg * kTcM;
    const int tid = threadIdx.x, warp = tid >> 5;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tmem_slot)),
                     "r"(a.tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        for (int s = 0; s < S; ++s)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&mbar[s])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    auto load_chunk = [&](int c, int s) {
        uint8_t* A = stage_base + s * stage_bytes;
        const uint32_t a_base = smem_u32(A), b_base = a_base + a_bytes;
        // A: R + 2 input rows x 130 pixels x 2 halves of 8 channels
        for (int i = tid; i < (R + 2) * 260; i += blockDim.x) {
            const int ri = i / 260, rem = i % 260, r = rem >> 1, half = rem & 1;
            const int px = x0 - 1 + r, py = y0 + ri - 1;
            const bool ok = px >= 0 && px < a.w && py >= 0 && py < a.h;
            const int ch = c * 16 + half * 8;
            const __nv_bfloat16* src = a.x;
            if (ok) {
                if (!a.lo)
                    src = a.x + ((size_t(img) * a.h + py) * a.w + px) * a.cin + ch;
                else if (ch < a.cl)
                    src = a.lo + ((size_t(img) * (a.h >> 1) + (py >> 1)) * (a.w >> 1) + (px >> 1)) * a.cl + ch;
                else
                    src = a.x + ((size_t(img) * a.h + py) * a.w + px) * (a.cin - a.cl) + (ch - a.cl);
            }
            cp_async16(a_base + ri * kTcATile + half * kTcRowBytes + r * 16, src, ok ? 16u : 0u);
        }
        // B: 9 taps x N rows x 2 halves
        for (int i = tid; i < 9 * N * 2; i += blockDim.x) {
            const int tap = i / (2 * N), rem = i % (2 * N), nr = rem >> 1, half = rem & 1;
            const bool ok = nr < a.cout_p;
            const __nv_bfloat16* src = ok ? a.wt + (size_t(nr) * 9 + tap) * a.cin + c * 16 + half * 8 : a.wt;
            cp_async16(b_base + tap * N * 32 + half * N * 16 + nr * 16, src, ok ? 16u : 0u);
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    };

    const int nchunks = a.cin / 16;
    const uint32_t idesc = tc_idesc(N);
    bool ok = true;
    for (int c = 0; c < S - 1 && c < nchunks; ++c) load_chunk(c, c);
    for (int c = 0; c < nchunks; ++c) {
        const int s = c % S, cn = c + S - 1;
        if (cn < nchunks) {
            // stage cn % S was last read by chunk cn - S
            if (cn >= S) ok = mbar_wait(smem_u32(&mbar[cn % S]), uint32_t(((cn - S) / S) & 1), a.err);
            if (__syncthreads_or(!ok)) {
                ok = false;
                break;
            }
            load_chunk(cn, cn % S);
        }
        cp_async_wait_pending(min(S - 1, nchunks - 1 - c));
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const uint32_t A = smem_u32(stage_base + s * stage_bytes), B = A + a_bytes;
            for (int tap = 0; tap < 9; ++tap) {
                const int dyi = tap / 3, dxi = tap % 3;
                const uint64_t bd = tc_desc(B + tap * N * 32, N * 16, 128);
                const uint32_t acc = (c > 0 || tap > 0) ? 1u : 0u;
                for (int r = 0; r < R; ++r) {
                    const uint64_t ad = tc_desc(A + (r + dyi) * kTcATile + dxi * 16, kTcRowBytes, 128);
                    asm volatile(
                        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
                            tmem + uint32_t(r * a.acc_stride)),
                        "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                        : "memory");
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                             smem_u32(&mbar[s]))
                         : "memory");
        }
    }
    if (ok) {
        const int last = nchunks - 1;
        ok = mbar_wait(smem_u32(&mbar[last % S]), uint32_t((last / S) & 1), a.err);
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    if (__syncthreads_or(!ok) == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        // Epilogue: thread t owns D row t (TMEM lane t) of every row accumulator: pixel x0 + t.
        const int px = x0 + tid;
        for (int r = 0; r < R; ++r) {
            const int y = y0 + r;
            const size_t p = (size_t(img) * a.h + y) * a.w + px;
            const bool store = px < a.w && y < a.h;
            for (int cb = 0; cb < N; cb += 16) {
                uint32_t v[16];
                const uint32_t taddr = tmem + (uint32_t(warp * 32) << 16) + uint32_t(r * a.acc_stride + cb);
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
                    "%15}, [%16];\n"
                    : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
                      "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
                      "=r"(v[14]), "=r"(v[15])
                    : "r"(taddr)
                    : "memory");
                asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
                if (!store) continue;
                if (a.y && !a.yf && cb + 16 <= a.cout && ((a.ldy | a.yoff) & 7) == 0) {
                    // 16 channels = two 16-byte stores
                    uint32_t packed[8];
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        float f0 = __uint_as_float(v[2 * j]) + (a.bias ? a.bias[cb + 2 * j] : 0.f);
                        float f1 = __uint_as_float(v[2 * j + 1]) + (a.bias ? a.bias[cb + 2 * j + 1] : 0.f);
                        if (a.relu) {
                            f0 = fmaxf(f0, 0.f);
                            f1 = fmaxf(f1, 0.f);
                        }
                        packed[j] = pack_bf16(__float2bfloat16(f0), __float2bfloat16(f1));
                    }
                    uint4* dst = reinterpret_cast<uint4*>(a.y + p * a.ldy + a.yoff + cb);
                    dst[0] = make_uint4(packed[0], packed[1], packed[2], packed[3]);
                    dst[1] = make_uint4(packed[4], packed[5], packed[6], packed[7]);
                    continue;
                }
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int co = cb + j;
                    if (co >= a.cout) break;
                    float f = __uint_as_float(v[j]) + (a.bias ? a.bias[co] : 0.f);
                    if (a.relu) f = fmaxf(f, 0.f);
                    if (a.y) a.y[p * a.ldy + a.yoff + co] = __float2bfloat16(f);
                    if (a.yf) a.yf[p * a.cout + co] = f + (a.res ? a.res[p * a.cout + co] : 0.f);
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(a.tmem_cols) : "memory");
}

// The same convolution with its operands staged by TMA (cp.async.bulk.tensor) instead of
// per-thread copies.  A box of 8 channels x 130 pixels of one input row lands as 130
// consecutive 16-byte rows, which is exactly one 8-channel half of a staged row above; a
// box of 8 channels x 1 tap x N output channels of the weights lands as one half of one
// tap's B operand.  One thread produces and issues: per chunk it posts the chunk's byte
// count on the stage's `full` mbarrier, issues the 2(R + 2) + 18 boxes (zero-filled outside
// the image), waits for them, issues the chunk's 9R MMAs and commits them to the stage's
// `done` mbarrier; the stage is refilled once those MMAs have read it.  The other threads
// wait at a barrier until the last commit, then all read TMEM in the epilogue.
struct ConvTma {
    CUtensorMap x;          // [n][h][w][cin] BF16: dims (cin, w, h, n), box (8, 130, 1, 1)
    CUtensorMap wt;         // [cout_p][9][cin] BF16: dims (cin, 9, cout_p), box (8, 1, n_mma)
    int cin, cout_p, n_mma, cout;
    const float* bias;
    __nv_bfloat16* y;
    int ldy, yoff;
    float* yf;
    const float* res;
    int relu;
    int n, h, w;
    int rows, acc_stride, stages;
    uint32_t tmem_cols;
    uint32_t* err;
};

__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            uint32_t mbar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];\n" ::"r"(dst),
        "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(mbar)
        : "memory");
}
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, uint32_t mbar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];\n" ::"r"(dst),
        "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(mbar)
        : "memory");
}

__global__ void __launch_bounds__(128) k_conv_fwd_tma(const __grid_constant__ ConvTma a) {
    extern __shared__ __align__(128) uint8_t smem[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem);      // kTcMaxStages
    uint64_t* done = reinterpret_cast<uint64_t*>(smem + 32); // kTcMaxStages
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + 64);
    __shared__ int failed;
    const int N = a.n_mma, R = a.rows, S = a.stages;
    const int stage_bytes = tc_stage_bytes(N, R);
    const int a_bytes = (R + 2) * kTcATile;
    uint8_t* stage_base = smem + 128;
    const int segs = (a.w + kTcM - 1) / kTcM, groups = (a.h + R - 1) / R;
    const int seg = blockIdx.x % segs, rg = (blockIdx.x / segs) % groups, img = blockIdx.x / (segs * groups);
    const int y0 = rg * R, x0 = seg * kTcM;
    const int tid = threadIdx.x, warp = tid >> 5;
    const uint32_t chunk_bytes = uint32_t((R + 2) * 2 * 130 * 16 + 9 * 2 * N * 16);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tmem_slot)),
                     "r"(a.tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        failed = (smem_u32(stage_base) & 127u) != 0u; // TMA destinations must be 128-byte aligned
        for (int s = 0; s < S; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&full[s])) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&done[s])) : "memory");
        }
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        if (failed) atomicOr(a.err, 2u);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    const int nchunks = a.cin / 16;

    if (tid == 0 && !failed) {
        auto load = [&](int c, int s) {
            const uint32_t A = smem_u32(stage_base + s * stage_bytes), B = A + a_bytes;
            const uint32_t fb = smem_u32(&full[s]);
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(fb), "r"(chunk_bytes)
                         : "memory");
            for (int ri = 0; ri < R + 2; ++ri)
                for (int half = 0; half < 2; ++half)
                    tma_load_4d(A + ri * kTcATile + half * kTcRowBytes, &a.x, c * 16 + half * 8, x0 - 1, y0 + ri - 1,
                                img, fb);
            for (int tap = 0; tap < 9; ++tap)
                for (int half = 0; half < 2; ++half)
                    tma_load_3d(B + tap * N * 32 + half * N * 16, &a.wt, c * 16 + half * 8, tap, 0, fb);
        };
        const uint32_t idesc = tc_idesc(N);
        for (int c = 0; c < S && c < nchunks; ++c) load(c, c);
        bool ok = true;
        for (int c = 0; c < nchunks && ok; ++c) {
            const int s = c % S;
            ok = mbar_wait(smem_u32(&full[s]), uint32_t((c / S) & 1), a.err);
            if (!ok) break;
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const uint32_t A = smem_u32(stage_base + s * stage_bytes), B = A + a_bytes;
            for (int tap = 0; tap < 9; ++tap) {
                const int dyi = tap / 3, dxi = tap % 3;
                const uint64_t bd = tc_desc(B + tap * N * 32, N * 16, 128);
                const uint32_t acc = (c > 0 || tap > 0) ? 1u : 0u;
                for (int r = 0; r < R; ++r) {
                    const uint64_t ad = tc_desc(A + (r + dyi) * kTcATile + dxi * 16, kTcRowBytes, 128);
                    asm volatile(
                        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
                            tmem + uint32_t(r * a.acc_stride)),
                        "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                        : "memory");
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                             smem_u32(&done[s]))
                         : "memory");
            // refill the stage of the previous chunk once its MMAs have read it
            const int cp = c - 1, cn = cp + S;
            if (cp >= 0 && cn < nchunks) {
                ok = mbar_wait(smem_u32(&done[cp % S]), uint32_t((cp / S) & 1), a.err);
                if (ok) load(cn, cp % S);
            }
        }
        if (ok) {
            const int last = nchunks - 1;
            ok = mbar_wait(smem_u32(&done[last % S]), uint32_t((last / S) & 1), a.err);
        }
        if (!ok) failed = 1;
    }
    __syncthreads();
    if (!failed) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        const int px = x0 + tid;
        for (int r = 0; r < R; ++r) {
            const int y = y0 + r;
            const size_t p = (size_t(img) * a.h + y) * a.w + px;
            const bool store = px < a.w && y < a.h;
            for (int cb = 0; cb < N; cb += 16) {
                uint32_t v[16];
                const uint32_t taddr = tmem + (uint32_t(warp * 32) << 16) + uint32_t(r * a.acc_stride + cb);
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
                    "%15}, [%16];\n"
                    : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
                      "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
                      "=r"(v[14]), "=r"(v[15])
                    : "r"(taddr)
                    : "memory");
                asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
                if (!store) continue;
                if (a.y && !a.yf && cb + 16 <= a.cout && ((a.ldy | a.yoff) & 7) == 0) {
                    uint32_t packed[8];
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        float f0 = __uint_as_float(v[2 * j]) + (a.bias ? a.bias[cb + 2 * j] : 0.f);
                        float f1 = __uint_as_float(v[2 * j + 1]) + (a.bias ? a.bias[cb + 2 * j + 1] : 0.f);
                        if (a.relu) {
                            f0 = fmaxf(f0, 0.f);
                            f1 = fmaxf(f1, 0.f);
                        }
                        packed[j] = pack_bf16(__float2bfloat16(f0), __float2bfloat16(f1));
                    }
                    uint4* dst = reinterpret_cast<uint4*>(a.y + p * a.ldy + a.yoff + cb);
                    dst[0] = make_uint4(packed[0], packed[1], packed[2], packed[3]);
                    dst[1] = make_uint4(packed[4], packed[5], packed[6], packed[7]);
                    continue;
                }
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int co = cb + j;
                    if (co >= a.cout) break;
                    float f = __uint_as_float(v[j]) + (a.bias ? a.bias[co] : 0.f);
                    if (a.relu) f = fmaxf(f, 0.f);
                    if (a.y) a.y[p * a.ldy + a.yoff + co] = __float2bfloat16(f);
                    if (a.yf) a.yf[p * a.cout + co] = f + (a.res ? a.res[p * a.cout + co] : 0.f);
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(a.tmem_cols) : "memory");
}

// The weight gradient on the 5th-generation tensor cores: per tap, the GEMM
// D[co][ci] = sum over pixels p of dY[p][co] * X[p + tap][ci] with M = output channels
// (padded to 128 with zero rows), N = input channels (cin, a multiple of 16) and K = pixels.
// CTA (b, tap) takes the 64-pixel chunks b, b + B, b + 2B, ... of the pixels; each chunk is
// staged transposed into the K-major no-swizzle core-matrix layout (8 rows x 16 bytes:
// 8 channels x 8 pixels) — A = dY^T [kc][co/8][co%8][8 pixels], B = X^T [kc][ci/8][ci%8][8
// pixels] — and one thread issues its four K = 16 MMAs into the FP32 accumulator in tensor
// memory and commits them to the stage's mbarrier; two stages overlap staging and MMAs.
// The CTA writes its accumulator to its own slice of `part` ([tap][b][co][ci]); a second
// kernel adds the slices in order of b, so the gradient is the same on every run.
constexpr int kWgM = 128;            // MMA M (output channels, zero-padded)
constexpr int kWgK = 64;             // pixels per staged chunk
constexpr int kWgMaxN = 256;         // input channels (MMA N)
constexpr int kWgABytes = (kWgK / 8) * (kWgM / 8) * 128;
__host__ __device__ constexpr int wg_stage_bytes(int n) { return kWgABytes + (kWgK / 8) * (n / 8) * 128; }
__host__ __device__ constexpr int wg_smem_bytes(int n) { return 128 + 2 * wg_stage_bytes(n); }
constexpr int kWgSmemTwoPerSm = 78 * 1024; // three such CTAs exceed an SM's 228 KB

struct ConvWgradTc {
    const __nv_bfloat16* dy; // [P][cout] (pixels of n images of h x w)
    int cout;                // multiple of 16, at most 128
    const __nv_bfloat16* x;  // [P][cin]
    int cin;                 // multiple of 16, at most 256 (MMA N)
    float* part;             // [9][blocks][cout][cin]
    int blocks;              // CTAs per tap (gridDim.x)
    int n, h, w;
    uint32_t tmem_cols;      // power of two >= cin
    uint32_t* err;
};

__global__ void __launch_bounds__(128) k_conv_wgrad_tc(ConvWgradTc a) {
    extern __shared__ __align__(128) uint8_t smem[];
    uint64_t* mbar = reinterpret_cast<uint64_t*>(smem);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + 64);
    uint8_t* stage_base = smem + 128;
    const int N = a.cin, stage_bytes = wg_stage_bytes(N);
    const int tap = blockIdx.y, dy = tap / 3 - 1, dx = tap % 3 - 1;
    const int tid = threadIdx.x, warp = tid >> 5;
    const long long P = (long long)a.n * a.h * a.w;
    const long long chunks = (P + kWgK - 1) / kWgK;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tmem_slot)),
                     "r"(a.tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        for (int s = 0; s < 2; ++s)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&mbar[s])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    // A rows co >= cout stay zero in both stages.
    for (int i = tid; i < 2 * kWgABytes / 16; i += blockDim.x) {
        const int s = i / (kWgABytes / 16), q = i % (kWgABytes / 16);
        reinterpret_cast<uint4*>(stage_base + s * stage_bytes)[q] = make_uint4(0, 0, 0, 0);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    // Stages chunk `chunk` into stage s: dY^T into A, the tap-shifted X^T into B.
    auto stage = [&](long long chunk, int s) {
        uint8_t* A = stage_base + s * stage_bytes;
        uint8_t* B = A + kWgABytes;
        const long long p0 = chunk * kWgK;
        const int cg = a.cout / 8, ng = N / 8;
        for (int i = tid; i < kWgK * cg; i += blockDim.x) {
            const int pl = i % kWgK, g = i / kWgK;
            const long long p = p0 + pl;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (p < P) v = __ldg(reinterpret_cast<const uint4*>(a.dy + size_t(p) * a.cout + g * 8));
            const uint16_t* e = reinterpret_cast<const uint16_t*>(&v);
            uint8_t* dst = A + (pl >> 3) * ((kWgM / 8) * 128) + g * 128 + (pl & 7) * 2;
#pragma unroll
            for (int r = 0; r < 8; ++r) *reinterpret_cast<uint16_t*>(dst + r * 16) = e[r];
        }
        for (int i = tid; i < kWgK * ng; i += blockDim.x) {
            const int pl = i % kWgK, g = i / kWgK;
            const long long p = p0 + pl;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (p < P) {
                const int x = int(p % a.w), y = int((p / a.w) % a.h), img = int(p / ((long long)a.w * a.h));
                const int ys = y + dy, xs = x + dx;
                if (ys >= 0 && ys < a.h && xs >= 0 && xs < a.w)
                    v = __ldg(reinterpret_cast<const uint4*>(a.x + ((size_t(img) * a.h + ys) * a.w + xs) * N + g * 8));
            }
            const uint16_t* e = reinterpret_cast<const uint16_t*>(&v);
            uint8_t* dst = B + (pl >> 3) * (ng * 128) + g * 128 + (pl & 7) * 2;
#pragma unroll
            for (int r = 0; r < 8; ++r) *reinterpret_cast<uint16_t*>(dst + r * 16) = e[r];
        }
    };

    const uint32_t idesc = tc_idesc(N);
    bool ok = true;
    int issued = 0; // chunks whose MMAs were committed
    for (long long chunk = blockIdx.x; chunk < chunks; chunk += a.blocks, ++issued) {
        const int s = issued & 1;
        // stage s was last read by chunk issued - 2
        if (issued >= 2) ok = mbar_wait(smem_u32(&mbar[s]), uint32_t(((issued - 2) >> 1) & 1), a.err);
        if (__syncthreads_or(!ok)) {
            ok = false;
            break;
        }
        stage(chunk, s);
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const uint32_t A = smem_u32(stage_base + s * stage_bytes), B = A + kWgABytes;
#pragma unroll
            for (int k = 0; k < kWgK / 16; ++k) {
                const uint64_t ad = tc_desc(A + 2 * k * ((kWgM / 8) * 128), (kWgM / 8) * 128, 128);
                const uint64_t bd = tc_desc(B + 2 * k * ((N / 8) * 128), (N / 8) * 128, 128);
                const uint32_t acc = (issued > 0 || k > 0) ? 1u : 0u;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                             smem_u32(&mbar[s]))
                         : "memory");
        }
    }
    // The MMAs read shared memory and write tensor memory until their last commit
    // arrives: wait for it (bounded) also after a failed wait, before the memory is freed.
    if (issued > 0) {
        const int last = issued - 1;
        if (!mbar_wait(smem_u32(&mbar[last & 1]), uint32_t((last >> 1) & 1), a.err)) ok = false;
    }
    if (__syncthreads_or(!ok) == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        // Thread t holds row t of D (TMEM lane t): output channel t.
        const int co = tid;
        float* dst = a.part + ((size_t(tap) * a.blocks + blockIdx.x) * a.cout + co) * N;
        for (int cb = 0; cb < N; cb += 16) {
            uint32_t v[16];
            const uint32_t taddr = tmem + (uint32_t(warp * 32) << 16) + uint32_t(cb);
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
                "%15}, [%16];\n"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                  "=r"(v[15])
                : "r"(taddr)
                : "memory");
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            if (co >= a.cout) continue;
#pragma unroll
            for (int j = 0; j < 16; j += 4)
                *reinterpret_cast<float4*>(dst + cb + j) = make_float4(
                    issued ? __uint_as_float(v[j]) : 0.f, issued ? __uint_as_float(v[j + 1]) : 0.f,
                    issued ? __uint_as_float(v[j + 2]) : 0.f, issued ? __uint_as_float(v[j + 3]) : 0.f);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(a.tmem_cols) : "memory");
}

// dw[co][tap][ci] += sum over b = 0, 1, ... of part[tap][b][co][ci], in that order.
__global__ void k_wgrad_reduce(const float* part, int blocks, int cout, int cin, float* dw) {
    const long long count = 9LL * cout * cin;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x) {
        const int ci = int(i % cin), co = int((i / cin) % cout), tap = int(i / ((long long)cin * cout));
        float s = 0.f;
        for (int b = 0; b < blocks; ++b) s += part[((size_t(tap) * blocks + b) * cout + co) * cin + ci];
        dw[(size_t(co) * 9 + tap) * cin + ci] += s;
    }
}

// Bias gradient, sum_p dY[p][c] for the first `count` of `stride` channels: FP32 partial
// sums per block into part[block][c] (k_bias_reduce adds them in order of block).
constexpr int kBgMaxCh = 128; // channels of a bias-gradient partial row
__global__ void k_bias_grad(const __nv_bfloat16* dy, int stride, int count, long long P, float* part) {
    for (int ch = threadIdx.x; ch < count; ch += blockDim.x) {
        float s = 0.f;
        for (long long p = blockIdx.x; p < P; p += gridDim.x) s += __bfloat162float(dy[size_t(p) * stride + ch]);
        part[size_t(blockIdx.x) * kBgMaxCh + ch] = s;
    }
}

// db[ch] += the blocks' partial sums, in order of block.
__global__ void k_bias_reduce(const float* part, int blocks, int count, float* db) {
    for (int ch = threadIdx.x; ch < count; ch += blockDim.x) {
        float s = 0.f;
        for (int b = 0; b < blocks; ++b) s += part[size_t(b) * kBgMaxCh + ch];
        db[ch] += s;
    }
}

// g = g * (y > 0) elementwise (the output y was ReLU'd).
__global__ void k_relu_bwd(__nv_bfloat16* g, const __nv_bfloat16* y, long long count) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x)
        if (!(__bfloat162float(y[i]) > 0.f)) g[i] = __float2bfloat16(0.f);
}

// 2x2 average pool: [n][h][w][c] -> [n][h/2][w/2][c].
__global__ void k_pool(const __nv_bfloat16* x, __nv_bfloat16* y, int n, int h, int w, int c) {
    const long long count = (long long)n * (h / 2) * (w / 2) * c;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x) {
        const int ch = int(i % c);
        const long long q = i / c;
        const int xo = int(q % (w / 2)), yo = int((q / (w / 2)) % (h / 2)), nn = int(q / ((long long)(w / 2) * (h / 2)));
        float s = 0.f;
        for (int k = 0; k < 4; ++k)
            s += __bfloat162float(x[((size_t(nn) * h + 2 * yo + (k >> 1)) * w + 2 * xo + (k & 1)) * c + ch]);
        y[i] = __float2bfloat16(0.25f * s);
    }
}

// Backward of the pool, added into dx: dx[2y+i][2x+j] += dy[y][x] / 4.
__global__ void k_pool_bwd(const __nv_bfloat16* dy, __nv_bfloat16* dx, int n, int h, int w, int c) {
    const long long count = (long long)n * h * w * c;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x) {
        const int ch = int(i % c);
        const long long q = i / c;
        const int x = int(q % w), y = int((q / w) % h), nn = int(q / ((long long)w * h));
        const float g = __bfloat162float(dy[((size_t(nn) * (h / 2) + y / 2) * (w / 2) + x / 2) * c + ch]);
        dx[i] = __float2bfloat16(__bfloat162float(dx[i]) + 0.25f * g);
    }
}

// Concatenate the 2x nearest upsampling of `lo` ([n][h/2][w/2][cl]) with `skip` ([n][h][w][cs])
// into y ([n][h][w][cl + cs]).
__global__ void k_upcat(const __nv_bfloat16* lo, int cl, const __nv_bfloat16* skip, int cs, __nv_bfloat16* y, int n,
                        int h, int w) {
    const int c = cl + cs;
    const long long count = (long long)n * h * w * c;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x) {
        const int ch = int(i % c);
        const long long p = i / c;
        const int x = int(p % w), yy = int((p / w) % h), nn = int(p / ((long long)w * h));
        y[i] = ch < cl ? lo[((size_t(nn) * (h / 2) + yy / 2) * (w / 2) + x / 2) * cl + ch] : skip[size_t(p) * cs + ch - cl];
    }
}

// Backward of k_upcat: dlo[y][x] = sum of the four upsampled gradients; dskip = its slice.
__global__ void k_upcat_bwd(const __nv_bfloat16* dy, int cl, int cs, __nv_bfloat16* dlo, __nv_bfloat16* dskip, int n,
                            int h, int w) {
    const int c = cl + cs;
    const long long lo_count = (long long)n * (h / 2) * (w / 2) * cl;
    const long long sk_count = (long long)n * h * w * cs;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < lo_count + sk_count;
         i += (long long)gridDim.x * blockDim.x) {
        if (i < lo_count) {
            const int ch = int(i % cl);
            const long long q = i / cl;
            const int x = int(q % (w / 2)), yy = int((q / (w / 2)) % (h / 2)), nn = int(q / ((long long)(w / 2) * (h / 2)));
            float s = 0.f;
            for (int k = 0; k < 4; ++k)
                s += __bfloat162float(dy[((size_t(nn) * h + 2 * yy + (k >> 1)) * w + 2 * x + (k & 1)) * c + ch]);
            dlo[i] = __float2bfloat16(s);
        } else {
            const long long j = i - lo_count;
            const int ch = int(j % cs);
            const long long p = j / cs;
            dskip[j] = dy[size_t(p) * c + cl + ch];
        }
    }
}

// Network input: log(1 + beauty), albedo, normal (9 channels) into 16 BF16 channels, and
// log(1 + beauty) in FP32 for the residual output.  Sources are [n][h][w][3]; the network's
// images are [n][hp][wp] (hp >= h, wp >= w), the extra rows and columns repeating the last
// ones.
__global__ void k_pack_input(const float* beauty, const float* albedo, const float* normal, int n, int h, int w,
                             int hp, int wp, __nv_bfloat16* x, float* lb) {
    const long long P = (long long)n * hp * wp;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < P; p += (long long)gridDim.x * blockDim.x) {
        const int xx = min(int(p % wp), w - 1), yy = min(int((p / wp) % hp), h - 1);
        const long long nn = p / ((long long)wp * hp);
        const size_t s = ((size_t(nn) * h + yy) * w + xx) * 3;
        __nv_bfloat16* o = x + size_t(p) * 16;
        for (int k = 0; k < 3; ++k) {
            const float b = beauty[s + k];
            const float l = log1pf(isfinite(b) ? fmaxf(b, 0.f) : 0.f);
            lb[p * 3 + k] = l;
            o[k] = __float2bfloat16(l);
            o[3 + k] = __float2bfloat16(albedo ? albedo[s + k] : 0.f);
            o[6 + k] = __float2bfloat16(normal ? normal[s + k] : 0.f);
        }
        for (int k = 9; k < 16; ++k) o[k] = __float2bfloat16(0.f);
    }
}

// Loss: mean |out - log(1 + target)| over P x 3 values; its gradient into 16 BF16 channels.
__global__ void k_l1_log1p(const float* out, const float* target, long long P, float* loss, __nv_bfloat16* g) {
    const float inv = 1.f / float(P * 3);
    float s = 0.f;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < P; p += (long long)gridDim.x * blockDim.x) {
        for (int k = 0; k < 3; ++k) {
            const float tv = target[p * 3 + k];
            const float d = out[p * 3 + k] - log1pf(isfinite(tv) ? fmaxf(tv, 0.f) : 0.f);
            s += fabsf(d);
            g[size_t(p) * 16 + k] = __float2bfloat16(d > 0.f ? inv : (d < 0.f ? -inv : 0.f));
        }
        for (int k = 3; k < 16; ++k) g[size_t(p) * 16 + k] = __float2bfloat16(0.f);
    }
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, s * inv);
}

// Adam on the FP32 master parameters (Kingma & Ba 2015).
__global__ void k_adam(float* p, float* m, float* v, const float* g, long long count, float lr, float b1, float b2,
                       float eps, float c1, float c2) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

// Master weights W[co][9][cin] (FP32) -> forward BF16 [cout_p][9][cin_p] and the flipped,
// transposed input-gradient weights [cin_p][9][cout_pp]: Wf[ci][t][co] = W[co][8 - t][ci].
__global__ void k_weights_bf16(const float* w, int cout, int cin, __nv_bfloat16* wb, int cout_p, int cin_p,
                               __nv_bfloat16* wf, int cout_pp) {
    const long long nb = (long long)cout_p * 9 * cin_p, nf = (long long)cin_p * 9 * cout_pp;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nb + nf; i += (long long)gridDim.x * blockDim.x) {
        if (i < nb) {
            const int ci = int(i % cin_p), tap = int((i / cin_p) % 9), co = int(i / (9LL * cin_p));
            wb[i] = __float2bfloat16(co < cout && ci < cin ? w[(size_t(co) * 9 + tap) * cin + ci] : 0.f);
        } else {
            const long long j = i - nb;
            const int co = int(j % cout_pp), tap = int((j / cout_pp) % 9), ci = int(j / (9LL * cout_pp));
            wf[j] = __float2bfloat16(co < cout && ci < cin ? w[(size_t(co) * 9 + (8 - tap)) * cin + ci] : 0.f);
        }
    }
}

// Padded weight gradients -> flat gradient vector; the bias gradients are read in place.
__global__ void k_gather_grad(const float* dwp, int cout, int cin, int cin_p, const float* dbp, float* g) {
    const long long nw = (long long)cout * 9 * cin;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nw + cout; i += (long long)gridDim.x * blockDim.x) {
        if (i < nw) {
            const int ci = int(i % cin), tap = int((i / cin) % 9), co = int(i / (9LL * cin));
            g[i] = dwp[(size_t(co) * 9 + tap) * cin_p + ci];
        } else {
            g[i] = dbp[i - nw];
        }
    }
}

// Output: exp(out) - 1, clamped at 0, cropped from [hp][wp][3] to [h][w][3].
__global__ void k_unpack_output(const float* out, int h, int w, int wp, float* rgb) {
    const long long count = (long long)h * w * 3;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x) {
        const int k = int(i % 3);
        const long long q = i / 3;
        const int xx = int(q % w), yy = int(q / w);
        rgb[i] = fmaxf(expm1f(out[(size_t(yy) * wp + xx) * 3 + k]), 0.f);
    }
}

// Split-buffer residual test, one block per tile.  With p the render, a the mean of its
// first half of samples, d the denoised image and N the tile's pixel count, per channel c:
//     m_d = mean(d),  m_p = mean(p),  v = sum((a - p)^2) / N^2
// (v estimates the variance of m_p: (a - p)^2 = (a - b)^2 / 4 estimates each pixel's
// variance from its two halves).  The tile keeps p when the denoised tile's mean moved by
// more than `threshold` standard errors, with 1% of the mean as a floor:
//     sum_c (m_d - m_p)^2 > threshold^2 * sum_c (v + (0.01 m_p)^2)
// flags[tile] = 1 and *count += 1 for each tile that falls back.
constexpr float kFallbackRelFloor = 0.01f;
__global__ void __launch_bounds__(256) k_tile_fallback(const float* d, const float* p, const float* a, int h, int w,
                                                        int tile, float threshold, float* out, uint8_t* flags,
                                                        uint32_t* count) {
    __shared__ float red[3][3][8]; // [sum d, sum p, sum (a-p)^2][channel][warp]
    __shared__ int keep_plain;
    const int tiles_x = (w + tile - 1) / tile;
    const int tx = blockIdx.x % tiles_x, ty = blockIdx.x / tiles_x;
    const int x0 = tx * tile, y0 = ty * tile;
    const int tw = min(tile, w - x0), th = min(tile, h - y0);
    float sd[3] = {0.f, 0.f, 0.f}, sp[3] = {0.f, 0.f, 0.f}, sv[3] = {0.f, 0.f, 0.f};
    for (int q = threadIdx.x; q < tw * th; q += blockDim.x) {
        const size_t o = (size_t(y0 + q / tw) * w + x0 + q % tw) * 3;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float pv = isfinite(p[o + k]) ? p[o + k] : 0.f;
            const float av = isfinite(a[o + k]) ? a[o + k] : 0.f;
            sd[k] += d[o + k];
            sp[k] += pv;
            sv[k] += (av - pv) * (av - pv);
        }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        for (int off = 16; off > 0; off >>= 1) {
            sd[k] += __shfl_down_sync(0xffffffffu, sd[k], off);
            sp[k] += __shfl_down_sync(0xffffffffu, sp[k], off);
            sv[k] += __shfl_down_sync(0xffffffffu, sv[k], off);
        }
        if ((threadIdx.x & 31) == 0) {
            red[0][k][threadIdx.x >> 5] = sd[k];
            red[1][k][threadIdx.x >> 5] = sp[k];
            red[2][k][threadIdx.x >> 5] = sv[k];
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const float n = float(tw * th);
        float shift = 0.f, var = 0.f;
        for (int k = 0; k < 3; ++k) {
            float td = 0.f, tp = 0.f, tv = 0.f;
            for (int i = 0; i < int(blockDim.x >> 5); ++i) {
                td += red[0][k][i];
                tp += red[1][k][i];
                tv += red[2][k][i];
            }
            const float md = td / n, mp = tp / n;
            shift += (md - mp) * (md - mp);
            var += tv / (n * n) + (kFallbackRelFloor * mp) * (kFallbackRelFloor * mp);
        }
        keep_plain = shift > threshold * threshold * var ? 1 : 0;
        flags[blockIdx.x] = uint8_t(keep_plain);
        if (keep_plain) atomicAdd(count, 1u);
    }
    __syncthreads();
    const float* src = keep_plain ? p : d;
    for (int i = threadIdx.x; i < tw * th * 3; i += blockDim.x) {
        const int k = i % 3, q = i / 3;
        const size_t o = (size_t(y0 + q / tw) * w + x0 + q % tw) * 3 + k;
        out[o] = src[o];
    }
}

} // namespace dn
} // namespace gt
