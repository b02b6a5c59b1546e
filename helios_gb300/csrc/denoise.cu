// denoise.cu — the learned denoiser: a 5-level convolutional encoder-decoder
// (3x3 convolutions, 32 -> 128 channels, skip connections) over 1-spp
// radiance + albedo + normal + depth, trained and run entirely by this file's
// kernels.  No counterpart in the reference engine; the auxiliary inputs
// follow its AOV definitions (renderer.h:27-35, debug_visualization.frag:
// 142-161: albedo = base colour at the first hit, normal = shading normal).
//
// Tensor-core path (sm_103a): every convolution — forward, backward-data and
// backward-weights — is an implicit GEMM on tcgen05.mma with the FP32
// accumulator in TMEM and BF16 operands staged in shared memory by TMA:
//
//   forward / backward-data   D[128 px][N ch] += A[128 px][32 ch] * B[N][32]^T
//       A: an 8x16-pixel tile of an NHWC activation tensor shifted by the
//          tap — a descriptor offset into ONE 4-D TMA box per 32-channel
//          chunk that holds two tiles and their one-pixel halo; out-of-range
//          pixels read as zero (that is the convolution's zero padding);
//          K-major, 64-byte swizzle (k_conv_halo).
//       B: the tap's weights [N][32 ch], K-major, shared by the two tiles'
//          accumulators.  Backward-data runs the same kernel on the output
//          gradient with the weights transposed and the taps mirrored.
//   backward-weights          D[128 ci][N co] += X[px][ci]^T * G[px][co]
//       both operands MN-major straight from NHWC boxes — X as a halo box,
//          each tap of a group of taps reading its shifted view by
//          descriptor offset into its own accumulator (k_wgrad_halo); each
//          CTA reduces over a split of the pixel tiles and writes partials,
//          and a second kernel sums the partials in a fixed order.
//
// One CTA = 6 warps: warps 0-3 drain TMEM (tcgen05.ld, one TMEM lane quarter
// each) and run the fused epilogue (bias, ReLU, ReLU-mask of the gradient,
// BF16 pack, channel split for concatenated inputs); warp 4 issues TMA; warp
// 5 allocates TMEM and one of its threads issues the MMAs.  Stages are
// guarded by full/empty mbarriers; every wait is bounded (error bit, no trap).
//
// Activations and activation gradients are BF16 NHWC with channel counts that
// are multiples of 32; weights, biases, gradients of parameters and the Adam
// state are FP32 (BF16 copies of the weights in the two layouts the kernels
// read are refreshed by the Adam kernel).
#include "hx_internal.h"
#include "tc.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

namespace {

using bf16 = __nv_bfloat16;

constexpr int kChunk = 32;                // channels per K step (64-byte rows)
constexpr int kChunkBytes = 128 * 64;     // one 128-row x 64-byte operand tile
constexpr int kThreads = 192;
constexpr int kConvStages = 4;

enum Epi : int { EPI_RELU_BF16 = 0, EPI_LINEAR_F32 = 1, EPI_DGRAD = 2 };

struct ConvArgs {
    int W, H, nimg, tiles_x, tiles_y;
    int chunks0, chunks1;      // 32-channel K chunks of source 0 / source 1
    int N;                     // MMA N: output channels, multiple of 16
    int stages;
    uint32_t b_bytes;          // per-stage B tile (N rows x 64 B, rounded up to 1 KB)
    uint32_t tmem_cols;
    int mode;
    const float* bias;
    void* out0;
    void* out1;
    int och0, och1;            // channels of out0 / out1 (EPI_DGRAD splits at och0)
    const bf16* mask0;         // EPI_DGRAD: zero the gradient where mask <= 0
    const bf16* mask1;
    const bf16* resid;         // EPI_LINEAR_F32: network input (32 ch); channels 0-2 are added to the output
    int n_store;               // channels written (EPI_RELU_BF16)
    uint32_t* err;
    long long wait_cycles;     // budget of each pipeline wait
};

__device__ __forceinline__ void store16_bf16(bf16* dst, const float (&f)[16]) {
    uint32_t w[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        __nv_bfloat162 h = __floats2bfloat162_rn(f[2 * j], f[2 * j + 1]);
        w[j] = *reinterpret_cast<uint32_t*>(&h);
    }
    uint4* d = reinterpret_cast<uint4*>(dst);
    d[0] = make_uint4(w[0], w[1], w[2], w[3]);
    d[1] = make_uint4(w[4], w[5], w[6], w[7]);
}
__device__ __forceinline__ void load16_bf16(const bf16* src, float (&f)[16]) {
    const uint4* s = reinterpret_cast<const uint4*>(src);
    uint4 a = s[0], b = s[1];
    uint32_t w[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        __nv_bfloat162 h = *reinterpret_cast<__nv_bfloat162*>(&w[j]);
        f[2 * j] = __low2float(h);
        f[2 * j + 1] = __high2float(h);
    }
}

__device__ __forceinline__ uint8_t* align1k(uint8_t* p) {
    return reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(p) + 1023) & ~uintptr_t(1023));
}

// Before a CTA frees its TMEM and exits — normally or after a pipeline wait
// gave up — its own asynchronous work must have landed: the producer waits
// for the newest load of every stage it filled (older loads of a stage
// completed before the stage was refilled), the MMA issuer for `done`, which
// it committed after its last MMA.  These waits use the full budget; on the
// normal path they find the phases already complete.
__device__ __forceinline__ void drain(int warp, int lane, int issued, int stages, uint64_t* full, uint64_t* done,
                                      uint32_t* s_fail) {
    if (warp == 4 && lane == 0) {
        for (int i = issued > stages ? issued - stages : 0; i < issued; ++i)
            if (!tc::mbar_wait(&full[i % stages], (i / stages) & 1)) *s_fail = 1;
    } else if (warp == 5 && lane == 0) {
        if (!tc::mbar_wait(done, 0)) *s_fail = 1;
    }
}

// Forward / backward-data convolution over a halo: one CTA = two 8x16-pixel
// tiles stacked vertically (8 x 32 pixels, two 128-row accumulators in TMEM).
// Per 32-channel chunk ONE TMA box of the tiles and their one-pixel halo
// (32 ch x 10 x 34 pixels, 64-byte swizzle: 340 rows of 64 B) is loaded, and
// the nine taps are nine descriptor start offsets into it: tap (ky, kx) of
// tile m reads rows (m*16 + py + ky) * 10 + kx + px, i.e. 8-row groups one
// halo row (640 B) apart, K-major within each 64-byte row.  Each weight tile
// (one tap, one chunk) feeds both accumulators.  Activation bytes per pixel
// and chunk fall from 9 x 64 B to 340 x 64 / 256 B, weight bytes by half.
constexpr int kHX = 8, kHY = 16, kHMT = 2;                      // tile, tiles per CTA
constexpr int kHaloW = kHX + 2, kHaloH = kHMT * kHY + 2;
constexpr uint32_t kHaloBytes = kHaloW * kHaloH * 64;            // 21,760
constexpr uint32_t kHaloStride = (kHaloBytes + 1023) / 1024 * 1024;
constexpr uint32_t kHaloRowBytes = kHaloW * 64;                  // 640: stride of 8-row groups

// Epilogue of one halo-kernel CTA tile pair: TMEM lane r (pixel (r % 8,
// r / 8) of tile m) from the accumulator at column col0 + m * N, bias + ReLU /
// residual / gradient mask, stores.  Called by warps 0-3 (TMEM lane quarters).
__device__ __forceinline__ void halo_epilogue(const ConvArgs& a, uint32_t trow, uint32_t col0, int x0, int y0, int n,
                                              int r) {
    for (int m = 0; m < kHMT; ++m) {
        const int x = x0 + (r & (kHX - 1)), y = y0 + m * kHY + r / kHX;
        const bool inb = x < a.W && y < a.H;
        const size_t pix = ((size_t)n * a.H + y) * a.W + x;
        for (int col = 0; col < a.N; col += 16) {
            uint32_t v[16];
            __syncwarp();
            tc::tmem_ld16(trow + col0 + (uint32_t)(m * a.N + col), v);
            tc::tmem_wait_ld();
            float f[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) f[j] = __uint_as_float(v[j]);
            if (!inb) continue;
            if (a.mode == EPI_RELU_BF16) {
                if (col < a.n_store) {
#pragma unroll
                    for (int j = 0; j < 16; ++j) f[j] = fmaxf(f[j] + a.bias[col + j], 0.0f);
                    store16_bf16(reinterpret_cast<bf16*>(a.out0) + pix * a.och0 + col, f);
                }
            } else if (a.mode == EPI_LINEAR_F32) {
                if (col == 0) {
                    const __nv_bfloat162 r01 = *reinterpret_cast<const __nv_bfloat162*>(a.resid + pix * 32);
                    const float r2 = __bfloat162float(a.resid[pix * 32 + 2]);
                    reinterpret_cast<float4*>(a.out0)[pix] =
                        make_float4((f[0] + a.bias[0]) + __low2float(r01), (f[1] + a.bias[1]) + __high2float(r01),
                                    (f[2] + a.bias[2]) + r2, 0.0f);
                }
            } else {
                const bool hi = col >= a.och0;
                const int och = hi ? a.och1 : a.och0, lc = hi ? col - a.och0 : col;
                const bf16* mk = hi ? a.mask1 : a.mask0;
                if (mk) {
                    float mv[16];
                    load16_bf16(mk + pix * och + lc, mv);
#pragma unroll
                    for (int j = 0; j < 16; ++j) f[j] = mv[j] > 0.0f ? f[j] : 0.0f;
                }
                store16_bf16(reinterpret_cast<bf16*>(hi ? a.out1 : a.out0) + pix * och + lc, f);
            }
        }
    }
}

__global__ void __launch_bounds__(kThreads, 6)
    k_conv_halo(const __grid_constant__ CUtensorMap src0, const __grid_constant__ CUtensorMap src1,
                const __grid_constant__ CUtensorMap wmap, ConvArgs a) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = align1k(smem_raw);
    const int nch = a.chunks0 + a.chunks1;
    uint8_t* As = smem;                              // halo buffers: two (double-buffered over chunks), one
    uint8_t* Bs = smem + (nch > 1 ? 2 : 1) * kHaloStride;  // for a single chunk; then the weight stages
    uint64_t* a_full = reinterpret_cast<uint64_t*>(Bs + a.stages * a.b_bytes);
    uint64_t* a_empty = a_full + 2;
    uint64_t* b_full = a_empty + 2;
    uint64_t* b_empty = b_full + a.stages;
    uint64_t* done = b_empty + a.stages;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(done + 1);
    __shared__ uint32_t s_fail;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int per_img = a.tiles_x * a.tiles_y;
    const int n = blockIdx.x / per_img, rem = blockIdx.x % per_img;
    const int x0 = (rem % a.tiles_x) * kHX, y0 = (rem / a.tiles_x) * (kHMT * kHY);

    if (threadIdx.x == 0) {
        for (int s = 0; s < 2; ++s) {
            tc::mbar_init(&a_full[s], 1);
            tc::mbar_init(&a_empty[s], 1);
        }
        for (int s = 0; s < a.stages; ++s) {
            tc::mbar_init(&b_full[s], 1);
            tc::mbar_init(&b_empty[s], 1);
        }
        tc::mbar_init(done, 1);
        tc::fence_mbar_init();
        s_fail = 0;
    }
    if (warp == 5) {
        tc::tmem_alloc(tslot, a.tmem_cols);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tslot;

    int issued_a = 0, issued_b = 0;  // halo and weight loads issued by the producer (warp 4, lane 0)
    if (warp == 4) {
        if (lane == 0) {
            tc::tma_prefetch(&src0);
            if (a.chunks1) tc::tma_prefetch(&src1);
            tc::tma_prefetch(&wmap);
            const uint32_t wbytes = a.N * 64;
            bool stop = false;
            for (int c = 0; c < nch && !stop; ++c) {
                const int hb = c & 1;
                if (c >= 2 && !tc::mbar_wait(&a_empty[hb], ((c >> 1) - 1) & 1, a.wait_cycles)) {
                    s_fail = 1;
                    break;
                }
                issued_a = c + 1;
                tc::mbar_expect_tx(&a_full[hb], kHaloBytes);
                if (c < a.chunks0)
                    tc::tma_load_4d(As + hb * kHaloStride, &src0, &a_full[hb], c * kChunk, x0 - 1, y0 - 1, n);
                else
                    tc::tma_load_4d(As + hb * kHaloStride, &src1, &a_full[hb], (c - a.chunks0) * kChunk, x0 - 1,
                                    y0 - 1, n);
                for (int t = 0; t < 9; ++t) {
                    const int i = c * 9 + t, s = i % a.stages;
                    if (i >= a.stages && !tc::mbar_wait(&b_empty[s], ((i / a.stages) - 1) & 1, a.wait_cycles)) {
                        s_fail = 1;
                        stop = true;
                        break;
                    }
                    issued_b = i + 1;
                    tc::mbar_expect_tx(&b_full[s], wbytes);
                    tc::tma_load_3d(Bs + s * a.b_bytes, &wmap, &b_full[s], c * kChunk, 0, t);
                }
            }
        }
    } else if (warp == 5) {
        if (lane == 0) {
            const uint32_t idesc = tc::idesc_bf16(128, a.N, 0, 0);
            bool ok = true;
            for (int c = 0; c < nch && ok; ++c) {
                const int hb = c & 1;
                if (!tc::mbar_wait(&a_full[hb], (c >> 1) & 1, a.wait_cycles)) {
                    ok = false;
                    break;
                }
                tc::fence_after_sync();
                const uint32_t ab = tc::smem_u32(As + hb * kHaloStride);
                for (int t = 0; t < 9; ++t) {
                    const int i = c * 9 + t, s = i % a.stages;
                    if (!tc::mbar_wait(&b_full[s], (i / a.stages) & 1, a.wait_cycles)) {
                        ok = false;
                        break;
                    }
                    tc::fence_after_sync();
                    const int ky = t / 3, kx = t % 3;
                    const uint32_t bb = tc::smem_u32(Bs + s * a.b_bytes);
#pragma unroll
                    for (int m = 0; m < kHMT; ++m)
#pragma unroll
                        for (int k = 0; k < 2; ++k) {
                            const uint32_t aa = ab + (uint32_t)(m * kHY + ky) * kHaloRowBytes + kx * 64 + 32 * k;
                            tc::mma_bf16(tmem + (uint32_t)(m * a.N), tc::smem_desc(aa, 16, kHaloRowBytes, tc::kSwizzle64B),
                                         tc::smem_desc(bb + 32 * k, 16, 512, tc::kSwizzle64B), idesc, (c | t | k) != 0);
                        }
                    tc::mma_commit(&b_empty[s]);
                }
                if (ok) tc::mma_commit(&a_empty[hb]);
            }
            if (!ok) s_fail = 1;
            tc::mma_commit(done);
        }
    } else {
        bool ok = tc::mbar_wait(done, 0, a.wait_cycles);
        ok = __all_sync(0xffffffffu, ok);
        tc::fence_after_sync();
        if (ok) {
            halo_epilogue(a, tmem + ((uint32_t)(warp * 32) << 16), 0u, x0, y0, n, warp * 32 + lane);
        } else if (lane == 0) {
            s_fail = 1;
        }
    }
    // drain: the producer's newest halo and weight loads, the MMA issuer's `done`
    if (warp == 4 && lane == 0) {
        for (int c = issued_a > 2 ? issued_a - 2 : 0; c < issued_a; ++c)
            if (!tc::mbar_wait(&a_full[c & 1], (c >> 1) & 1)) s_fail = 1;
        for (int i = issued_b > a.stages ? issued_b - a.stages : 0; i < issued_b; ++i)
            if (!tc::mbar_wait(&b_full[i % a.stages], (i / a.stages) & 1)) s_fail = 1;
    } else if (warp == 5 && lane == 0) {
        if (!tc::mbar_wait(done, 0)) s_fail = 1;
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 5) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tmem, a.tmem_cols);
    }
    if (threadIdx.x == 0 && s_fail) atomicOr(a.err, 1u);
}

// Persistent form of k_conv_halo for single-chunk layers (32 input channels,
// N <= 64: the full-resolution layers): a CTA per SM slot loads the layer's
// nine weight tiles once, then walks tile pairs (blockIdx.x, + gridDim.x, ...)
// through a kPHaloStages-deep halo ring; two TMEM accumulator sets let the
// epilogue warps drain pair i while the MMAs of pair i + 1 run.  Barriers:
// w_full (weights), h_full / h_empty (halo ring), acc_full (MMA -> epilogue,
// one commit per pair) and acc_empty (epilogue -> MMA, one arrival per
// epilogue warp).
constexpr int kPHaloStages = 3;

__global__ void __launch_bounds__(kThreads, 1)
    k_conv_halo_p(const __grid_constant__ CUtensorMap src0, const __grid_constant__ CUtensorMap wmap, ConvArgs a) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = align1k(smem_raw);
    uint8_t* Ws = smem;                                    // nine weight tiles
    uint8_t* Hs = smem + 9 * a.b_bytes;                    // halo ring
    uint64_t* w_full = reinterpret_cast<uint64_t*>(Hs + kPHaloStages * kHaloStride);
    uint64_t* h_full = w_full + 1;
    uint64_t* h_empty = h_full + kPHaloStages;
    uint64_t* acc_full = h_empty + kPHaloStages;
    uint64_t* acc_empty = acc_full + 2;
    uint64_t* done = acc_empty + 2;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(done + 1);
    __shared__ uint32_t s_fail;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int per_img = a.tiles_x * a.tiles_y;
    const int ntiles = per_img * a.nimg;
    const uint32_t acc_cols = (uint32_t)(kHMT * a.N);  // one accumulator set (both tiles of a pair)

    if (threadIdx.x == 0) {
        tc::mbar_init(w_full, 1);
        for (int s = 0; s < kPHaloStages; ++s) {
            tc::mbar_init(&h_full[s], 1);
            tc::mbar_init(&h_empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(&acc_full[b], 1);
            tc::mbar_init(&acc_empty[b], 4);
        }
        tc::mbar_init(done, 1);
        tc::fence_mbar_init();
        s_fail = 0;
    }
    if (warp == 5) {
        tc::tmem_alloc(tslot, a.tmem_cols);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tslot;

    int issued = 0;  // halo loads issued by the producer (warp 4, lane 0)
    if (warp == 4) {
        if (lane == 0) {
            tc::tma_prefetch(&src0);
            tc::tma_prefetch(&wmap);
            tc::mbar_expect_tx(w_full, 9u * a.N * 64);
            for (int t = 0; t < 9; ++t) tc::tma_load_3d(Ws + t * a.b_bytes, &wmap, w_full, 0, 0, t);
            int i = 0;
            for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++i) {
                const int s = i % kPHaloStages;
                if (i >= kPHaloStages &&
                    !tc::mbar_wait(&h_empty[s], ((i / kPHaloStages) - 1) & 1, a.wait_cycles)) {
                    s_fail = 1;
                    break;
                }
                issued = i + 1;
                const int n = tile / per_img, rem = tile % per_img;
                const int x0 = (rem % a.tiles_x) * kHX, y0 = (rem / a.tiles_x) * (kHMT * kHY);
                tc::mbar_expect_tx(&h_full[s], kHaloBytes);
                tc::tma_load_4d(Hs + s * kHaloStride, &src0, &h_full[s], 0, x0 - 1, y0 - 1, n);
            }
        }
    } else if (warp == 5) {
        if (lane == 0) {
            const uint32_t idesc = tc::idesc_bf16(128, a.N, 0, 0);
            bool ok = tc::mbar_wait(w_full, 0, a.wait_cycles);
            const uint32_t wb = tc::smem_u32(Ws);
            int i = 0;
            for (int tile = blockIdx.x; ok && tile < ntiles; tile += gridDim.x, ++i) {
                const int s = i % kPHaloStages, b = i & 1;
                if (!tc::mbar_wait(&h_full[s], (i / kPHaloStages) & 1, a.wait_cycles) ||
                    (i >= 2 && !tc::mbar_wait(&acc_empty[b], ((i >> 1) - 1) & 1, a.wait_cycles))) {
                    ok = false;
                    break;
                }
                tc::fence_after_sync();
                const uint32_t hb = tc::smem_u32(Hs + s * kHaloStride);
                const uint32_t d = tmem + (uint32_t)b * acc_cols;
                for (int t = 0; t < 9; ++t) {
                    const int ky = t / 3, kx = t % 3;
                    const uint32_t bb = wb + (uint32_t)t * a.b_bytes;
#pragma unroll
                    for (int m = 0; m < kHMT; ++m)
#pragma unroll
                        for (int k = 0; k < 2; ++k) {
                            const uint32_t aa = hb + (uint32_t)(m * kHY + ky) * kHaloRowBytes + kx * 64 + 32 * k;
                            tc::mma_bf16(d + (uint32_t)(m * a.N), tc::smem_desc(aa, 16, kHaloRowBytes, tc::kSwizzle64B),
                                         tc::smem_desc(bb + 32 * k, 16, 512, tc::kSwizzle64B), idesc, (t | k) != 0);
                        }
                }
                tc::mma_commit(&h_empty[s]);
                tc::mma_commit(&acc_full[b]);
            }
            if (!ok) s_fail = 1;
            tc::mma_commit(done);
        }
    } else {
        int i = 0;
        for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++i) {
            const int b = i & 1;
            bool ok = tc::mbar_wait(&acc_full[b], (i >> 1) & 1, a.wait_cycles);
            ok = __all_sync(0xffffffffu, ok);
            if (!ok) {
                if (lane == 0) s_fail = 1;
                break;
            }
            tc::fence_after_sync();
            const int n = tile / per_img, rem = tile % per_img;
            const int x0 = (rem % a.tiles_x) * kHX, y0 = (rem / a.tiles_x) * (kHMT * kHY);
            halo_epilogue(a, tmem + ((uint32_t)(warp * 32) << 16), (uint32_t)b * acc_cols, x0, y0, n, warp * 32 + lane);
            tc::fence_before_sync();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&acc_empty[b]);
        }
    }
    // drain: the producer's weight load and newest halo loads, the MMA issuer's `done`
    if (warp == 4 && lane == 0) {
        if (!tc::mbar_wait(w_full, 0)) s_fail = 1;
        for (int i = issued > kPHaloStages ? issued - kPHaloStages : 0; i < issued; ++i)
            if (!tc::mbar_wait(&h_full[i % kPHaloStages], (i / kPHaloStages) & 1)) s_fail = 1;
    } else if (warp == 5 && lane == 0) {
        if (!tc::mbar_wait(done, 0)) s_fail = 1;
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 5) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tmem, a.tmem_cols);
    }
    if (threadIdx.x == 0 && s_fail) atomicOr(a.err, 1u);
}

// Backward-weights over a halo: CTA (split, 128-input-channel block, group of
// consecutive taps) walks the split's 8x16-pixel tiles; per tile it loads each
// input chunk ONCE as a tile + one-pixel-halo box (32 ch x 10 x 18, 64-byte
// swizzle) and the output gradient once (32 ch x 8 x 16), and every tap of
// the group reads its shifted input view from the halo box by descriptor
// offset (pixel rows 640 B apart) into its own TMEM accumulator D_t[ci][co]
// (the group's taps x N columns).  Both operands MN-major, as in k_wgrad.
constexpr uint32_t kWHaloBytes = kHaloW * (kHY + 2) * 64;                  // 11,520
constexpr uint32_t kWHaloStride = (kWHaloBytes + 1023) / 1024 * 1024;      // 12 KB

struct WgradHaloArgs {
    int W, H, tiles_x, tiles_y, ntiles;
    int chunks0, chunks1, gchunks;
    int splits, stages, taps;  // taps per CTA (grid.z groups)
    uint32_t a_bytes, b_bytes, tmem_cols;
    float* partial;            // [splits][9][N][cin]
    int cin;
    uint32_t* err;
    long long wait_cycles;
};

__global__ void __launch_bounds__(kThreads, 1)
    k_wgrad_halo(const __grid_constant__ CUtensorMap src0, const __grid_constant__ CUtensorMap src1,
                 const __grid_constant__ CUtensorMap gmap, WgradHaloArgs a) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = align1k(smem_raw);
    uint8_t* As = smem;
    uint8_t* Bs = smem + a.stages * a.a_bytes;
    uint64_t* full = reinterpret_cast<uint64_t*>(Bs + a.stages * a.b_bytes);
    uint64_t* empty = full + a.stages;
    uint64_t* done = empty + a.stages;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(done + 1);
    __shared__ uint32_t s_fail;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int sp = blockIdx.x, mb = blockIdx.y;
    const int tap0 = blockIdx.z * a.taps, ntap = min(a.taps, 9 - tap0);
    const int t_begin = (int)((long long)a.ntiles * sp / a.splits);
    const int t_end = (int)((long long)a.ntiles * (sp + 1) / a.splits);
    const int iters = t_end - t_begin;
    const int nch = a.chunks0 + a.chunks1;
    const int qa = min(4, nch - mb * 4);
    const int N = 32 * a.gchunks;
    const int per_img = a.tiles_x * a.tiles_y;

    if (threadIdx.x == 0) {
        for (int s = 0; s < a.stages; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        tc::mbar_init(done, 1);
        tc::fence_mbar_init();
        s_fail = 0;
    }
    if (warp == 5) {
        tc::tmem_alloc(tslot, a.tmem_cols);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tslot;

    int issued = 0;  // stages loaded by the producer (warp 4, lane 0)
    if (warp == 4) {
        if (lane == 0) {
            tc::tma_prefetch(&src0);
            if (a.chunks1) tc::tma_prefetch(&src1);
            tc::tma_prefetch(&gmap);
            const uint32_t bytes = (uint32_t)qa * kWHaloBytes + (uint32_t)a.gchunks * kChunkBytes;
            for (int i = 0; i < iters; ++i) {
                const int s = i % a.stages;
                if (i >= a.stages && !tc::mbar_wait(&empty[s], ((i / a.stages) - 1) & 1, a.wait_cycles)) {
                    s_fail = 1;
                    break;
                }
                issued = i + 1;
                const int t = t_begin + i, n = t / per_img, rem = t % per_img;
                const int x0 = (rem % a.tiles_x) * kHX, y0 = (rem / a.tiles_x) * kHY;
                tc::mbar_expect_tx(&full[s], bytes);
                for (int q = 0; q < qa; ++q) {
                    const int c = mb * 4 + q;
                    uint8_t* dst = As + s * a.a_bytes + q * kWHaloStride;
                    if (c < a.chunks0)
                        tc::tma_load_4d(dst, &src0, &full[s], c * kChunk, x0 - 1, y0 - 1, n);
                    else
                        tc::tma_load_4d(dst, &src1, &full[s], (c - a.chunks0) * kChunk, x0 - 1, y0 - 1, n);
                }
                for (int q = 0; q < a.gchunks; ++q)
                    tc::tma_load_4d(Bs + s * a.b_bytes + q * kChunkBytes, &gmap, &full[s], q * kChunk, x0, y0, n);
            }
        }
    } else if (warp == 5) {
        if (lane == 0) {
            const uint32_t idesc = tc::idesc_bf16(128, N, 1, 1);
            for (int i = 0; i < iters; ++i) {
                const int s = i % a.stages;
                if (!tc::mbar_wait(&full[s], (i / a.stages) & 1, a.wait_cycles)) {
                    s_fail = 1;
                    break;
                }
                tc::fence_after_sync();
                const uint32_t ab = tc::smem_u32(As + s * a.a_bytes), bb = tc::smem_u32(Bs + s * a.b_bytes);
                for (int j = 0; j < ntap; ++j) {
                    const int tap = tap0 + j, ky = tap / 3, kx = tap % 3;
#pragma unroll
                    for (int k = 0; k < 8; ++k)  // 16 pixels = tile rows 2k, 2k + 1
                        tc::mma_bf16(tmem + (uint32_t)(j * N),
                                     tc::smem_desc(ab + (uint32_t)((2 * k + ky) * kHaloW + kx) * 64, kWHaloStride,
                                                   kHaloRowBytes, tc::kSwizzle64B),
                                     tc::smem_desc(bb + 1024 * k, kChunkBytes, 512, tc::kSwizzle64B), idesc,
                                     (i | k) != 0);
                }
                tc::mma_commit(&empty[s]);
            }
            tc::mma_commit(done);
        }
    } else {
        bool ok = tc::mbar_wait(done, 0, a.wait_cycles);
        ok = __all_sync(0xffffffffu, ok);
        tc::fence_after_sync();
        if (ok) {
            const int ci = mb * 128 + warp * 32 + lane;
            const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
            for (int j = 0; j < ntap; ++j) {
                float* dst = a.partial + ((size_t)sp * 9 + tap0 + j) * N * a.cin;
                for (int col = 0; col < N; col += 16) {
                    uint32_t v[16];
                    __syncwarp();
                    tc::tmem_ld16(trow + (uint32_t)(j * N + col), v);
                    tc::tmem_wait_ld();
                    if (ci < a.cin) {
#pragma unroll
                        for (int e = 0; e < 16; ++e)
                            dst[(size_t)(col + e) * a.cin + ci] = iters > 0 ? __uint_as_float(v[e]) : 0.0f;
                    }
                }
            }
        } else if (lane == 0) {
            s_fail = 1;
        }
    }
    drain(warp, lane, issued, a.stages, full, done, &s_fail);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 5) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tmem, a.tmem_cols);
    }
    if (threadIdx.x == 0 && s_fail) atomicOr(a.err, 1u);
}

// grad[tap][co][ci] = scale * sum_split partial[split][tap][co][ci], co < cout.
// A block = 32 consecutive outputs (lanes) x 8 split groups (warps): warp j
// sums splits j, j + 8, ... in order, then the eight group sums are added in
// warp order — a fixed order, so the result is deterministic.
constexpr int kReduceGroups = 8;
__global__ void __launch_bounds__(32 * kReduceGroups) k_wgrad_reduce(const float* __restrict__ partial, int splits, int N,
                                                                      int cout, int cin, float scale,
                                                                      float* __restrict__ grad) {
    __shared__ float red[kReduceGroups][33];
    const int lane = threadIdx.x & 31, j = threadIdx.x >> 5;
    const size_t total = (size_t)9 * cout * cin;
    const size_t i = (size_t)blockIdx.x * 32 + lane;
    float s = 0.0f;
    if (i < total) {
        const size_t tap = i / ((size_t)cout * cin), rem = i % ((size_t)cout * cin);
        const size_t co = rem / cin, ci = rem % cin;
        for (int k = j; k < splits; k += kReduceGroups) s += partial[(((size_t)k * 9 + tap) * N + co) * cin + ci];
    }
    red[j][lane] = s;
    __syncthreads();
    if (j == 0 && i < total) {
        float t = 0.0f;
#pragma unroll
        for (int q = 0; q < kReduceGroups; ++q) t += red[q][lane];
        grad[i] = t * scale;
    }
}

// Per-channel sums of a [P][C] BF16 tensor (C a multiple of 8, at most 128) in
// two fixed-order passes: each of kColBlocks blocks sums its contiguous pixel
// range, every thread 8 channels of a pixel per 16-byte load, the block's
// lanes combined in lane order; then one block per channel sums the blocks'
// partials (fixed per-thread subsets, a fixed-order tree).
constexpr int kColBlocks = 1024, kColThreads = 256;
__global__ void __launch_bounds__(kColThreads) k_colsum_partial(const bf16* __restrict__ g, size_t P, int C,
                                                                float* __restrict__ part) {
    __shared__ float acc[kColThreads][8];
    const int ncg = C / 8;                  // 8-channel groups of a pixel
    const int lanes = kColThreads / ncg;    // pixel lanes of the block
    const int cg = threadIdx.x % ncg, lanep = threadIdx.x / ncg;
    const size_t p0 = P * blockIdx.x / gridDim.x, p1 = P * (blockIdx.x + 1) / gridDim.x;
    float s[8] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    if (lanep < lanes)
        for (size_t p = p0 + lanep; p < p1; p += lanes) {
            const uint4 v = __ldg(reinterpret_cast<const uint4*>(g + p * C) + cg);
            const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const __nv_bfloat162 h = *reinterpret_cast<const __nv_bfloat162*>(&w[j]);
                s[2 * j] += __low2float(h);
                s[2 * j + 1] += __high2float(h);
            }
        }
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[threadIdx.x][j] = s[j];
    __syncthreads();
    if (threadIdx.x < C) {
        const int c = threadIdx.x;
        float t = 0.0f;
        for (int k = 0; k < lanes; ++k) t += acc[k * ncg + c / 8][c % 8];
        part[(size_t)blockIdx.x * C + c] = t;
    }
}
__global__ void __launch_bounds__(kColThreads) k_colsum_final(const float* __restrict__ part, int blocks, int C,
                                                              float scale, float* __restrict__ out) {
    __shared__ float red[kColThreads];
    const int c = blockIdx.x;
    float t = 0.0f;
    for (int k = threadIdx.x; k < blocks; k += kColThreads) t += part[(size_t)k * C + c];
    red[threadIdx.x] = t;
    __syncthreads();
    for (int h = kColThreads / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[c] = red[0] * scale;
}

// 8-channel vector helpers
__device__ __forceinline__ void unpack8(uint4 u, float (&f)[8]) {
    uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        __nv_bfloat162 h = *reinterpret_cast<__nv_bfloat162*>(&w[j]);
        f[2 * j] = __low2float(h);
        f[2 * j + 1] = __high2float(h);
    }
}
__device__ __forceinline__ uint4 pack8(const float (&f)[8]) {
    uint32_t w[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        __nv_bfloat162 h = __floats2bfloat162_rn(f[2 * j], f[2 * j + 1]);
        w[j] = *reinterpret_cast<uint32_t*>(&h);
    }
    return make_uint4(w[0], w[1], w[2], w[3]);
}

// The resampling kernels below run one block row per image row of the
// half-resolution grid (grid.y = n * h) and one thread per 8-channel group of
// a half-resolution pixel (grid.x covers w * C / 8): 32-bit indices, one
// division per thread, each thread handling the pixel's 2x2 full-resolution
// block.  Sizes are checked on the host (n * h, w * C / 8 < 2^31).
struct RowIdx {
    int n, y, x, g;
    bool ok;
};
__device__ __forceinline__ RowIdx row_idx(int h, int w, int cg) {
    RowIdx r;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    r.ok = j < w * cg;
    r.x = j / cg;
    r.g = j - r.x * cg;
    r.n = blockIdx.y / h;
    r.y = blockIdx.y - r.n * h;
    return r;
}

// 2x2 average pool: out [n][H/2][W/2][C] from in [n][H][W][C].
__global__ void k_pool(const bf16* __restrict__ in, int H, int W, int C, int nimg, bf16* __restrict__ out) {
    const int h = H / 2, w = W / 2, cg = C / 8;
    const RowIdx r = row_idx(h, w, cg);
    if (!r.ok) return;
    float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int dy = 0; dy < 2; ++dy)
        for (int dx = 0; dx < 2; ++dx) {
            float f[8];
            const size_t q = ((size_t)(r.n * H + 2 * r.y + dy) * W + 2 * r.x + dx) * C;
            unpack8(reinterpret_cast<const uint4*>(in + q)[r.g], f);
#pragma unroll
            for (int j = 0; j < 8; ++j) s[j] += f[j];
        }
#pragma unroll
    for (int j = 0; j < 8; ++j) s[j] *= 0.25f;
    reinterpret_cast<uint4*>(out + ((size_t)(r.n * h + r.y) * w + r.x) * C)[r.g] = pack8(s);
}

// g_a += (a > 0) * g_p / 4 spread over each 2x2 block (pool backward into a
// ReLU output that also feeds a skip connection).
__global__ void k_pool_bwd_add(const bf16* __restrict__ gp, const bf16* __restrict__ act, int H, int W, int C,
                               int nimg, bf16* __restrict__ ga) {
    const int h = H / 2, w = W / 2, cg = C / 8;
    const RowIdx r = row_idx(h, w, cg);
    if (!r.ok) return;
    float fp[8];
    unpack8(reinterpret_cast<const uint4*>(gp + ((size_t)(r.n * h + r.y) * w + r.x) * C)[r.g], fp);
    for (int dy = 0; dy < 2; ++dy)
        for (int dx = 0; dx < 2; ++dx) {
            const size_t q = ((size_t)(r.n * H + 2 * r.y + dy) * W + 2 * r.x + dx) * C;
            float fa[8], fg[8];
            unpack8(reinterpret_cast<const uint4*>(act + q)[r.g], fa);
            unpack8(reinterpret_cast<const uint4*>(ga + q)[r.g], fg);
#pragma unroll
            for (int j = 0; j < 8; ++j) fg[j] = fg[j] + (fa[j] > 0.0f ? 0.25f * fp[j] : 0.0f);
            reinterpret_cast<uint4*>(ga + q)[r.g] = pack8(fg);
        }
}

// Nearest 2x upsampling: out [n][2h][2w][C].
__global__ void k_up(const bf16* __restrict__ in, int h, int w, int C, int nimg, bf16* __restrict__ out) {
    const int H = 2 * h, W = 2 * w, cg = C / 8;
    const RowIdx r = row_idx(h, w, cg);
    if (!r.ok) return;
    const uint4 v = reinterpret_cast<const uint4*>(in + ((size_t)(r.n * h + r.y) * w + r.x) * C)[r.g];
    for (int dy = 0; dy < 2; ++dy)
        for (int dx = 0; dx < 2; ++dx)
            reinterpret_cast<uint4*>(out + ((size_t)(r.n * H + 2 * r.y + dy) * W + 2 * r.x + dx) * C)[r.g] = v;
}

// Upsampling backward: sum of the 2x2 gradient block.
__global__ void k_up_bwd(const bf16* __restrict__ gin, int h, int w, int C, int nimg, bf16* __restrict__ gout) {
    const int H = 2 * h, W = 2 * w, cg = C / 8;
    const RowIdx r = row_idx(h, w, cg);
    if (!r.ok) return;
    float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int dy = 0; dy < 2; ++dy)
        for (int dx = 0; dx < 2; ++dx) {
            float f[8];
            const size_t q = ((size_t)(r.n * H + 2 * r.y + dy) * W + 2 * r.x + dx) * C;
            unpack8(reinterpret_cast<const uint4*>(gin + q)[r.g], f);
#pragma unroll
            for (int j = 0; j < 8; ++j) s[j] += f[j];
        }
    reinterpret_cast<uint4*>(gout + ((size_t)(r.n * h + r.y) * w + r.x) * C)[r.g] = pack8(s);
}

// Features [n][h][w][12] (radiance rgb, noise level, albedo rgb, depth, normal
// xyz, -) -> network input [n][H][W][32] BF16 (log1p radiance, albedo, normal,
// depth, noise level), zero outside h x w and beyond channel 10.
__global__ void k_pack_input(const float* __restrict__ feat, int h, int w, int H, int W, int nimg,
                             bf16* __restrict__ x) {
    const size_t total = (size_t)nimg * H * W;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < total; p += (size_t)gridDim.x * blockDim.x) {
        const int px = (int)(p % W), py = (int)((p / W) % H);
        const size_t n = p / ((size_t)W * H);
        float f[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) f[j] = 0.0f;
        if (px < w && py < h) {
            const float4* s = reinterpret_cast<const float4*>(feat + ((n * h + py) * w + px) * 12);
            float4 r = s[0], ad = s[1], nm = s[2];
            f[0] = log1pf(fmaxf(r.x, 0.0f));
            f[1] = log1pf(fmaxf(r.y, 0.0f));
            f[2] = log1pf(fmaxf(r.z, 0.0f));
            f[3] = ad.x;
            f[4] = ad.y;
            f[5] = ad.z;
            f[6] = nm.x;
            f[7] = nm.y;
            f[8] = nm.z;
            f[9] = ad.w;
            f[10] = r.w;
        }
        uint4* d = reinterpret_cast<uint4*>(x + p * 32);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            float g[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) g[j] = f[8 * q + j];
            d[q] = pack8(g);
        }
    }
}

// Network output (log1p radiance) -> RGBA radiance for the h x w crop.
__global__ void k_unpack_output(const float4* __restrict__ y, int h, int w, int H, int W, int nimg,
                                float4* __restrict__ out) {
    const size_t total = (size_t)nimg * h * w;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < total; p += (size_t)gridDim.x * blockDim.x) {
        const int px = (int)(p % w), py = (int)((p / w) % h);
        const size_t n = p / ((size_t)w * h);
        const float4 v = y[(n * H + py) * W + px];
        out[p] = make_float4(fmaxf(expm1f(v.x), 0.0f), fmaxf(expm1f(v.y), 0.0f), fmaxf(expm1f(v.z), 0.0f), 1.0f);
    }
}

// Loss and its gradient per pixel (3 colour channels), per-block sums:
//   HX_DN_LOSS_L1_LOG:   |y - log1p(t)|,               g_y = sign(y - log1p(t))
//   HX_DN_LOSS_L2_LINEAR: (expm1(y) - t)^2,            g_y = 2 (expm1(y) - t) exp(y)
// (t = max(target, 0); the 1 / (3 P) mean factor is applied to the parameter
// gradients).
constexpr int kLossBlocks = 256;
__global__ void k_loss(const float4* __restrict__ y, const float4* __restrict__ tgt, size_t P, uint32_t kind,
                       bf16* __restrict__ gy, float* __restrict__ part) {
    __shared__ float red[256];
    float s = 0.0f;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < P; p += (size_t)gridDim.x * blockDim.x) {
        const float4 v = y[p], t = tgt[p];
        const float yv[3] = {v.x, v.y, v.z}, tv[3] = {fmaxf(t.x, 0.0f), fmaxf(t.y, 0.0f), fmaxf(t.z, 0.0f)};
        float g[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            if (kind == HX_DN_LOSS_L2_LINEAR) {
                const float e = expf(yv[c]), d = (e - 1.0f) - tv[c];
                s += d * d;
                g[c] = 2.0f * d * e;
            } else {
                const float d = yv[c] - log1pf(tv[c]);
                s += fabsf(d);
                g[c] = d > 0.0f ? 1.0f : (d < 0.0f ? -1.0f : 0.0f);
            }
        }
        __nv_bfloat162 a = __floats2bfloat162_rn(g[0], g[1]), b = __floats2bfloat162_rn(g[2], 0.0f);
        uint2 w = make_uint2(*reinterpret_cast<uint32_t*>(&a), *reinterpret_cast<uint32_t*>(&b));
        *reinterpret_cast<uint2*>(gy + p * 32) = w;
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

struct AdamLayer {
    unsigned long long off;
    int cin, cout, nf, cd;
    bf16* wf;  // forward layout [9][nf][cin]
    bf16* wd;  // backward-data layout [9][cin][cd], taps mirrored
};
constexpr int kMaxLayers = 16;
struct AdamArgs {
    AdamLayer L[kMaxLayers];
    int nlayers;
    unsigned long long total;
    float lr, b1, b2, eps, c1, c2;  // c1 = 1 - b1^t, c2 = 1 - b2^t
    int update;                     // 0: only refresh the BF16 copies
};
__global__ void k_adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, AdamArgs a) {
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < a.total;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        float wi = w[i];
        if (a.update) {
            const float gi = g[i];
            const float mi = a.b1 * m[i] + (1.0f - a.b1) * gi;
            const float vi = a.b2 * v[i] + (1.0f - a.b2) * gi * gi;
            m[i] = mi;
            v[i] = vi;
            wi -= a.lr * (mi / a.c1) / (sqrtf(vi / a.c2) + a.eps);
            w[i] = wi;
        }
        int l = 0;
        while (l + 1 < a.nlayers && i >= a.L[l + 1].off) ++l;
        const AdamLayer& L = a.L[l];
        const unsigned long long e = i - L.off, nw = 9ull * L.cout * L.cin;
        if (e < nw) {
            const int tap = (int)(e / ((unsigned long long)L.cout * L.cin));
            const int rem = (int)(e % ((unsigned long long)L.cout * L.cin));
            const int co = rem / L.cin, ci = rem % L.cin;
            const bf16 b = __float2bfloat16_rn(wi);
            L.wf[((size_t)tap * L.nf + co) * L.cin + ci] = b;
            L.wd[((size_t)(8 - tap) * L.cin + ci) * L.cd + co] = b;
        }
    }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

hx_status get_encode() {
    static std::once_flag once;
    static cudaError_t err = cudaSuccess;
    std::call_once(once, [] {
        cudaDriverEntryPointQueryResult q;
        void* fn = nullptr;
        err = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
        if (err == cudaSuccess && q == cudaDriverEntryPointSuccess) g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
    });
    if (!g_encode) {
        hx_set_error("cuTensorMapEncodeTiled unavailable (%s)", cudaGetErrorString(err));
        return HX_ERR_DEVICE;
    }
    return HX_OK;
}

// NHWC BF16 activation: 4-D map (C, W, H, n), a box of 32 channels x bx x by pixels,
// 64-byte swizzle: (10, 34) for k_conv_halo (two
// 8x16 tiles and their one-pixel halo), (10, 18) and (8, 16) for
// k_wgrad_halo's input halo and output-gradient tile; out-of-range pixels
// read as zero.
hx_status make_halo_map(CUtensorMap* m, const bf16* p, int C, int W, int H, int n, int bx = kHaloW,
                        int by = kHaloH) {
    HX_TRY(get_encode());
    cuuint64_t dims[4] = {(cuuint64_t)C, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)n};
    cuuint64_t strides[3] = {(cuuint64_t)C * 2, (cuuint64_t)C * 2 * W, (cuuint64_t)C * 2 * W * H};
    cuuint32_t box[4] = {kChunk, (cuuint32_t)bx, (cuuint32_t)by, 1};
    cuuint32_t es[4] = {1, 1, 1, 1};
    CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, (void*)p, dims, strides, box, es,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        hx_set_error("cuTensorMapEncodeTiled (halo C=%d W=%d H=%d n=%d) failed: %d", C, W, H, n, (int)r);
        return HX_ERR_DEVICE;
    }
    return HX_OK;
}
// Weights [9][rows][K] BF16: 3-D map (K, rows, 9), box (32, rows, 1).
hx_status make_w_map(CUtensorMap* m, const bf16* p, int K, int rows) {
    HX_TRY(get_encode());
    cuuint64_t dims[3] = {(cuuint64_t)K, (cuuint64_t)rows, 9};
    cuuint64_t strides[2] = {(cuuint64_t)K * 2, (cuuint64_t)K * 2 * rows};
    cuuint32_t box[3] = {kChunk, (cuuint32_t)rows, 1};
    cuuint32_t es[3] = {1, 1, 1};
    CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, (void*)p, dims, strides, box, es,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        hx_set_error("cuTensorMapEncodeTiled (weights K=%d rows=%d) failed: %d", K, rows, (int)r);
        return HX_ERR_DEVICE;
    }
    return HX_OK;
}

// Tensors of the network.  Level = resolution level (0 = full).
enum Tid : int { X, A0, A0B, P0, A1, P1, A2, P2, A3, P3, A4, A4B, U3, D3, U2, D2, U1, D1, U0, D0, D0B, GYT, NT };
struct TensorSpec {
    int level, C;
};
const TensorSpec kTensors[NT] = {
    {0, 32}, {0, 32}, {0, 32}, {1, 32}, {1, 64}, {2, 64}, {2, 64}, {3, 64}, {3, 96}, {4, 96}, {4, 128},
    {4, 128}, {3, 128}, {3, 96}, {2, 96}, {2, 64}, {1, 64}, {1, 64}, {0, 64}, {0, 32}, {0, 32}, {0, 32}};

struct LayerSpec {
    int src0, src1;  // tensor ids (src1 = -1: single source)
    int out;         // output tensor id (-1: the FP32 network output)
    int cout;
    bool relu;
};
const LayerSpec kLayers[] = {
    {X, -1, A0, 32, true},     {A0, -1, A0B, 32, true},   {P0, -1, A1, 64, true},    {P1, -1, A2, 64, true},
    {P2, -1, A3, 96, true},    {P3, -1, A4, 128, true},   {A4, -1, A4B, 128, true},  {U3, A3, D3, 96, true},
    {U2, A2, D2, 64, true},    {U1, A1, D1, 64, true},    {U0, A0B, D0, 32, true},   {D0, -1, D0B, 32, true},
    {D0B, -1, -1, 3, false}};
constexpr int kNumLayers = sizeof(kLayers) / sizeof(kLayers[0]);

int round_up(int v, int m) { return (v + m - 1) / m * m; }
uint32_t pow2_cols(int n) {
    uint32_t c = 32;
    while ((int)c < n) c <<= 1;
    return c;
}

struct Layer {
    int cin, cout, nf, cd;
    size_t off;        // into the flat parameter vector
    bf16* wf = nullptr;
    bf16* wd = nullptr;
    CUtensorMap wf_map, wd_map;
};

// Work split of a layer's backward-weights pass (k_wgrad_halo): 8x16-pixel
// tiles; taps per CTA so the taps' accumulators (taps x N columns) fit 256
// TMEM columns, spread evenly over the groups; pixel-tile splits for about
// two CTAs per SM.
struct WgradPlan {
    int tiles_x, tiles_y, ntiles, mblocks, taps, groups, splits;
};
WgradPlan wgrad_plan(const Layer& L, int W, int H, int n, int sms) {
    WgradPlan w{};
    w.tiles_x = (W + kHX - 1) / kHX;
    w.tiles_y = (H + kHY - 1) / kHY;
    w.ntiles = w.tiles_x * w.tiles_y * n;
    w.mblocks = (L.cin + 127) / 128;
    const int fit = std::max(1, std::min(9, 256 / L.cd));
    w.groups = (9 + fit - 1) / fit;
    w.taps = (9 + w.groups - 1) / w.groups;
    w.groups = (9 + w.taps - 1) / w.taps;
    const int per = w.mblocks * w.groups;
    w.splits = std::max(1, std::min(w.ntiles, (2 * sms + per - 1) / per));
    return w;
}


struct Plan {
    int n = 0, H = 0, W = 0;  // padded network size (multiple of 16)
    bool train = false;
    bf16* t[NT] = {};
    bf16* g[NT] = {};
    CUtensorMap hm[NT], hgm[NT];  // k_conv_halo: two 8x16 tiles + halo (10 x 34) of activations / gradients
    CUtensorMap wxm[NT], wgm[NT]; // k_wgrad_halo: input halo (10 x 18), output-gradient tile (8 x 16)
    float4* y = nullptr;
    float* partial = nullptr;
    size_t partial_bytes = 0;
    float* colpart = nullptr;
    float* loss_part = nullptr;
    std::vector<void*> allocs;
};

}  // namespace

struct hx_denoiser {
    hx_context* ctx = nullptr;
    Layer layers[kNumLayers];
    size_t nparams = 0;
    float* params = nullptr;
    float* grads = nullptr;
    float* adam_m = nullptr;
    float* adam_v = nullptr;
    uint32_t* err = nullptr;
    long long wait_cycles = tc::kWaitCycles;  // pipeline-wait budget (hx_denoiser_set_wait_budget)
    int step = 0;
    uint32_t loss_kind = HX_DN_LOSS_L1_LOG;
    std::vector<void*> allocs;
    std::unique_ptr<Plan> train_plan;
    std::vector<std::unique_ptr<Plan>> infer_plans;  // most recently used first
    Plan* last_infer = nullptr;
};

namespace {

hx_status dn_alloc(hx_context* ctx, std::vector<void*>& list, void** p, size_t bytes) {
    HX_TRY(hx_alloc(ctx, p, bytes));
    list.push_back(*p);
    HX_CUDA(cudaMemsetAsync(*p, 0, bytes, ctx->stream));
    return HX_OK;
}

void free_plan(hx_context* ctx, Plan* p) {
    if (!p) return;
    for (void* a : p->allocs) hx_free(ctx, a);
    p->allocs.clear();
}

int level_dim(int d, int level) { return d >> level; }

hx_status build_plan(hx_denoiser* dn, Plan* p, int n, int H, int W, bool train) {
    hx_context* ctx = dn->ctx;
    p->n = n;
    p->H = H;
    p->W = W;
    p->train = train;
    for (int i = 0; i < NT; ++i) {
        const int h = level_dim(H, kTensors[i].level), w = level_dim(W, kTensors[i].level), C = kTensors[i].C;
        const size_t bytes = (size_t)n * h * w * C * sizeof(bf16);
        if (i != GYT) {
            HX_TRY(dn_alloc(ctx, p->allocs, (void**)&p->t[i], bytes));
            HX_TRY(make_halo_map(&p->hm[i], p->t[i], C, w, h, n));
            if (train) HX_TRY(make_halo_map(&p->wxm[i], p->t[i], C, w, h, n, kHaloW, kHY + 2));
        }
        if (train && i != X) {
            HX_TRY(dn_alloc(ctx, p->allocs, (void**)&p->g[i], bytes));
            HX_TRY(make_halo_map(&p->hgm[i], p->g[i], C, w, h, n));
            HX_TRY(make_halo_map(&p->wgm[i], p->g[i], C, w, h, n, kHX, kHY));
        }
    }
    HX_TRY(dn_alloc(ctx, p->allocs, (void**)&p->y, (size_t)n * H * W * sizeof(float4)));
    if (train) {
        size_t mx = 0;
        for (int l = 0; l < kNumLayers; ++l) {
            const Layer& L = dn->layers[l];
            const int lev = kTensors[kLayers[l].src0].level;
            const WgradPlan wp = wgrad_plan(L, level_dim(W, lev), level_dim(H, lev), n, ctx->num_sms);
            mx = std::max(mx, (size_t)wp.splits * 9 * L.cd * L.cin * sizeof(float));
        }
        p->partial_bytes = mx;
        HX_TRY(dn_alloc(ctx, p->allocs, (void**)&p->partial, mx));
        HX_TRY(dn_alloc(ctx, p->allocs, (void**)&p->colpart, (size_t)kColBlocks * 128 * sizeof(float)));
        HX_TRY(dn_alloc(ctx, p->allocs, (void**)&p->loss_part, kLossBlocks * sizeof(float)));
    }
    HX_CUDA(cudaStreamSynchronize(ctx->stream));
    return HX_OK;
}

// Training keeps one plan (one crop size); inference keeps the buffers of
// the last kMaxInferPlans image sizes, so serving a mix of resolutions does
// not reallocate per request.
constexpr size_t kMaxInferPlans = 4;

hx_status get_plan(hx_denoiser* dn, int n, int H, int W, bool train, Plan** out) {
    auto fits = [&](const Plan* p) { return p && p->n == n && p->H == H && p->W == W; };
    if (train) {
        if (!fits(dn->train_plan.get())) {
            if (dn->train_plan) {
                HX_CUDA(cudaStreamSynchronize(dn->ctx->stream));
                free_plan(dn->ctx, dn->train_plan.get());
            }
            dn->train_plan.reset(new Plan());
            hx_status s = build_plan(dn, dn->train_plan.get(), n, H, W, true);
            if (s != HX_OK) {
                free_plan(dn->ctx, dn->train_plan.get());
                dn->train_plan.reset();
                return s;
            }
        }
        *out = dn->train_plan.get();
        return HX_OK;
    }
    auto& v = dn->infer_plans;
    for (size_t i = 0; i < v.size(); ++i)
        if (fits(v[i].get())) {
            std::rotate(v.begin(), v.begin() + i, v.begin() + i + 1);
            *out = dn->last_infer = v.front().get();
            return HX_OK;
        }
    if (v.size() >= kMaxInferPlans) {
        HX_CUDA(cudaStreamSynchronize(dn->ctx->stream));
        free_plan(dn->ctx, v.back().get());
        v.pop_back();
    }
    std::unique_ptr<Plan> p(new Plan());
    hx_status s = build_plan(dn, p.get(), n, H, W, false);
    if (s != HX_OK) {
        free_plan(dn->ctx, p.get());
        return s;
    }
    v.insert(v.begin(), std::move(p));
    *out = dn->last_infer = v.front().get();
    return HX_OK;
}


int grid_for(size_t total, int threads, int sms) {
    return (int)std::max<size_t>(1, std::min<size_t>((total + threads - 1) / threads, (size_t)sms * 8));
}

// Launch k_conv for layer l.  dgrad = false: forward from the layer's
// sources into its output; dgrad = true: output gradient -> source gradients.
hx_status launch_conv(hx_denoiser* dn, Plan* p, int l, bool dgrad) {
    hx_context* ctx = dn->ctx;
    const LayerSpec& S = kLayers[l];
    const Layer& L = dn->layers[l];
    const int lev = kTensors[S.src0].level;
    const int H = level_dim(p->H, lev), W = level_dim(p->W, lev);
    ConvArgs a{};
    a.W = W;
    a.H = H;
    a.nimg = p->n;
    a.tiles_x = (W + kHX - 1) / kHX;
    a.tiles_y = (H + kHMT * kHY - 1) / (kHMT * kHY);
    a.stages = kConvStages;
    a.err = dn->err;
    a.wait_cycles = dn->wait_cycles;
    const CUtensorMap *m0, *m1, *wm;
    const CUtensorMap* act = p->hm;
    const CUtensorMap* gact = p->hgm;
    if (!dgrad) {
        m0 = &act[S.src0];
        m1 = S.src1 >= 0 ? &act[S.src1] : m0;
        wm = &L.wf_map;
        a.chunks0 = kTensors[S.src0].C / kChunk;
        a.chunks1 = S.src1 >= 0 ? kTensors[S.src1].C / kChunk : 0;
        a.N = L.nf;
        a.bias = dn->params + L.off + (size_t)9 * L.cout * L.cin;
        if (S.out >= 0) {
            a.mode = EPI_RELU_BF16;
            a.out0 = p->t[S.out];
            a.och0 = kTensors[S.out].C;
            a.n_store = L.cout;
        } else {
            a.mode = EPI_LINEAR_F32;
            a.out0 = p->y;
            a.och0 = 4;
            a.resid = p->t[X];
        }
    } else {
        const int gout = S.out >= 0 ? S.out : GYT;
        m0 = &gact[gout];
        m1 = m0;
        wm = &L.wd_map;
        a.chunks0 = L.cd / kChunk;
        a.chunks1 = 0;
        a.N = L.cin;
        a.mode = EPI_DGRAD;
        a.out0 = p->g[S.src0];
        a.och0 = kTensors[S.src0].C;
        a.out1 = S.src1 >= 0 ? p->g[S.src1] : nullptr;
        a.och1 = S.src1 >= 0 ? kTensors[S.src1].C : 0;
        // ReLU outputs (and their nearest upsamplings) mask the gradient here;
        // pooled inputs are masked by the pool-backward kernel instead.
        auto relu_src = [](int t) { return t != P0 && t != P1 && t != P2 && t != P3 && t != X; };
        a.mask0 = relu_src(S.src0) ? p->t[S.src0] : nullptr;
        a.mask1 = S.src1 >= 0 && relu_src(S.src1) ? p->t[S.src1] : nullptr;
    }
    HX_CHECK_ARG(a.N % 16 == 0 && a.N >= 16 && a.N <= 256, "conv N=%d out of range", a.N);
    a.b_bytes = (uint32_t)round_up(a.N * 64, 1024);
    const int grid = a.tiles_x * a.tiles_y * p->n;
    if (a.chunks0 + a.chunks1 == 1 && a.N <= 64) {
        // single-chunk layer: the persistent kernel (weights resident, halo ring,
        // two accumulator sets), two CTAs per SM
        a.tmem_cols = pow2_cols(2 * kHMT * a.N);
        const size_t smem = 1024 + 9 * (size_t)a.b_bytes + kPHaloStages * (size_t)kHaloStride + 256;
        HX_CUDA(cudaFuncSetAttribute(k_conv_halo_p, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        const int pgrid = std::min(grid, 2 * ctx->num_sms);
        k_conv_halo_p<<<pgrid, kThreads, smem, ctx->stream>>>(*m0, *wm, a);
        HX_CUDA(cudaGetLastError());
        return HX_OK;
    }
    a.tmem_cols = pow2_cols(kHMT * a.N);
    // one halo buffer for a single 32-channel chunk (more resident CTAs for the 32-channel layers)
    const int nhalo = a.chunks0 + a.chunks1 > 1 ? 2 : 1;
    const size_t smem = 1024 + nhalo * (size_t)kHaloStride + a.stages * (size_t)a.b_bytes + 256;
    HX_CUDA(cudaFuncSetAttribute(k_conv_halo, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_conv_halo<<<grid, kThreads, smem, ctx->stream>>>(*m0, *m1, *wm, a);
    HX_CUDA(cudaGetLastError());
    return HX_OK;
}

hx_status launch_wgrad(hx_denoiser* dn, Plan* p, int l, float scale) {
    hx_context* ctx = dn->ctx;
    const LayerSpec& S = kLayers[l];
    const Layer& L = dn->layers[l];
    const int lev = kTensors[S.src0].level;
    const int H = level_dim(p->H, lev), W = level_dim(p->W, lev);
    const int gout = S.out >= 0 ? S.out : GYT;
    const WgradPlan wp = wgrad_plan(L, W, H, p->n, ctx->num_sms);
    WgradHaloArgs a{};
    a.W = W;
    a.H = H;
    a.tiles_x = wp.tiles_x;
    a.tiles_y = wp.tiles_y;
    a.ntiles = wp.ntiles;
    a.chunks0 = kTensors[S.src0].C / kChunk;
    a.chunks1 = S.src1 >= 0 ? kTensors[S.src1].C / kChunk : 0;
    a.gchunks = L.cd / kChunk;
    a.splits = wp.splits;
    a.taps = wp.taps;
    const int qmax = std::min(4, a.chunks0 + a.chunks1);
    a.a_bytes = (uint32_t)qmax * kWHaloStride;
    a.b_bytes = a.gchunks * kChunkBytes;
    a.stages = a.a_bytes + a.b_bytes <= 40u * 1024 ? 3 : 2;
    a.tmem_cols = pow2_cols(wp.taps * L.cd);
    a.partial = p->partial;
    a.cin = L.cin;
    a.err = dn->err;
    a.wait_cycles = dn->wait_cycles;
    HX_CHECK_ARG((size_t)a.splits * 9 * L.cd * L.cin * sizeof(float) <= p->partial_bytes, "wgrad partial overflow");
    // the MMA's M = 128 input channels reads four chunk slots at kWHaloStride
    // apart even when a block has fewer chunks: cover the last stage's reach
    const size_t body = std::max<size_t>((size_t)a.stages * (a.a_bytes + a.b_bytes),
                                         (size_t)(a.stages - 1) * a.a_bytes + 4 * (size_t)kWHaloStride);
    const size_t smem = 1024 + body + 256;
    HX_CUDA(cudaFuncSetAttribute(k_wgrad_halo, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const CUtensorMap* m0 = &p->wxm[S.src0];
    const CUtensorMap* m1 = S.src1 >= 0 ? &p->wxm[S.src1] : m0;
    k_wgrad_halo<<<dim3(a.splits, wp.mblocks, wp.groups), kThreads, smem, ctx->stream>>>(*m0, *m1, p->wgm[gout], a);
    HX_CUDA(cudaGetLastError());
    float* gw = dn->grads + L.off;
    const size_t total = (size_t)9 * L.cout * L.cin;
    k_wgrad_reduce<<<(unsigned)((total + 31) / 32), 32 * kReduceGroups, 0, ctx->stream>>>(p->partial, a.splits, L.cd,
                                                                                           L.cout, L.cin, scale, gw);
    HX_CUDA(cudaGetLastError());
    // bias gradient
    const int C = kTensors[gout].C;
    const int lev_o = S.out >= 0 ? kTensors[S.out].level : 0;
    const size_t P = (size_t)p->n * level_dim(p->H, lev_o) * level_dim(p->W, lev_o);
    k_colsum_partial<<<kColBlocks, kColThreads, 0, ctx->stream>>>(p->g[gout], P, C, p->colpart);
    k_colsum_final<<<L.cout, kColThreads, 0, ctx->stream>>>(p->colpart, kColBlocks, C, scale, gw + total);
    HX_CUDA(cudaGetLastError());
    return HX_OK;
}

// Launch grid of the resampling kernels over an h x w half-resolution grid.
hx_status row_grid(int n, int h, int w, int C, dim3* g) {
    HX_CHECK_ARG((long long)n * h <= 65535 && (long long)w * (C / 8) < (1ll << 31), "resampling grid %d x %d x %d too large",
                 n, h, w);
    *g = dim3((unsigned)((w * (C / 8) + 255) / 256), (unsigned)(n * h));
    return HX_OK;
}

hx_status elementwise_pool(hx_denoiser* dn, Plan* p, int src, int dst) {
    const int lev = kTensors[src].level, C = kTensors[src].C;
    const int H = level_dim(p->H, lev), W = level_dim(p->W, lev);
    dim3 g;
    HX_TRY(row_grid(p->n, H / 2, W / 2, C, &g));
    k_pool<<<g, 256, 0, dn->ctx->stream>>>(p->t[src], H, W, C, p->n, p->t[dst]);
    HX_CUDA(cudaGetLastError());
    return HX_OK;
}
hx_status elementwise_up(hx_denoiser* dn, Plan* p, int src, int dst) {
    const int lev = kTensors[src].level, C = kTensors[src].C;
    const int h = level_dim(p->H, lev), w = level_dim(p->W, lev);
    dim3 g;
    HX_TRY(row_grid(p->n, h, w, C, &g));
    k_up<<<g, 256, 0, dn->ctx->stream>>>(p->t[src], h, w, C, p->n, p->t[dst]);
    HX_CUDA(cudaGetLastError());
    return HX_OK;
}

hx_status run_forward(hx_denoiser* dn, Plan* p) {
    const int pools[4][2] = {{A0B, P0}, {A1, P1}, {A2, P2}, {A3, P3}};
    const int ups[4][2] = {{A4B, U3}, {D3, U2}, {D2, U1}, {D1, U0}};
    for (int l = 0; l < kNumLayers; ++l) {
        if (l >= 2 && l <= 5) HX_TRY(elementwise_pool(dn, p, pools[l - 2][0], pools[l - 2][1]));
        if (l >= 7 && l <= 10) HX_TRY(elementwise_up(dn, p, ups[l - 7][0], ups[l - 7][1]));
        HX_TRY(launch_conv(dn, p, l, false));
    }
    return HX_OK;
}

hx_status run_backward(hx_denoiser* dn, Plan* p, float scale) {
    hx_context* ctx = dn->ctx;
    for (int l = kNumLayers - 1; l >= 0; --l) {
        const LayerSpec& S = kLayers[l];
        HX_TRY(launch_wgrad(dn, p, l, scale));
        if (l == 0) break;
        HX_TRY(launch_conv(dn, p, l, true));
        // route the source gradients
        for (int k = 0; k < 2; ++k) {
            const int s = k == 0 ? S.src0 : S.src1;
            if (s < 0) continue;
            const int lev = kTensors[s].level, C = kTensors[s].C;
            const int H = level_dim(p->H, lev), W = level_dim(p->W, lev);
            if (s == U3 || s == U2 || s == U1 || s == U0) {
                const int dst = s == U3 ? A4B : s == U2 ? D3 : s == U1 ? D2 : D1;
                dim3 g;
                HX_TRY(row_grid(p->n, H / 2, W / 2, C, &g));
                k_up_bwd<<<g, 256, 0, ctx->stream>>>(p->g[s], H / 2, W / 2, C, p->n, p->g[dst]);
                HX_CUDA(cudaGetLastError());
            } else if (s == P0 || s == P1 || s == P2 || s == P3) {
                const int a = s == P0 ? A0B : s == P1 ? A1 : s == P2 ? A2 : A3;
                const int Ha = 2 * H, Wa = 2 * W;
                dim3 g;
                HX_TRY(row_grid(p->n, H, W, C, &g));
                k_pool_bwd_add<<<g, 256, 0, ctx->stream>>>(p->g[s], p->t[a], Ha, Wa, C, p->n, p->g[a]);
                HX_CUDA(cudaGetLastError());
            }
        }
    }
    return HX_OK;
}

hx_status refresh_weights(hx_denoiser* dn, bool update, float lr) {
    AdamArgs a{};
    a.nlayers = kNumLayers;
    for (int l = 0; l < kNumLayers; ++l) {
        const Layer& L = dn->layers[l];
        a.L[l] = AdamLayer{(unsigned long long)L.off, L.cin, L.cout, L.nf, L.cd, L.wf, L.wd};
    }
    a.total = dn->nparams;
    a.b1 = 0.9f;
    a.b2 = 0.999f;
    a.eps = 1e-8f;
    a.lr = lr;
    a.update = update ? 1 : 0;
    if (update) {
        dn->step += 1;
        a.c1 = (float)(1.0 - std::pow(0.9, dn->step));
        a.c2 = (float)(1.0 - std::pow(0.999, dn->step));
    } else {
        a.c1 = a.c2 = 1.0f;
    }
    k_adam<<<grid_for(dn->nparams, 256, dn->ctx->num_sms), 256, 0, dn->ctx->stream>>>(dn->params, dn->grads,
                                                                                    dn->adam_m, dn->adam_v, a);
    HX_CUDA(cudaGetLastError());
    return HX_OK;
}

hx_status check_err(hx_denoiser* dn) {
    uint32_t e = 0;
    HX_CUDA(cudaMemcpyAsync(&e, dn->err, sizeof(e), cudaMemcpyDeviceToHost, dn->ctx->stream));
    HX_CUDA(cudaStreamSynchronize(dn->ctx->stream));
    if (e) {
        HX_CUDA(cudaMemsetAsync(dn->err, 0, sizeof(uint32_t), dn->ctx->stream));
        hx_set_error("denoiser: a tensor-core pipeline wait timed out (status 0x%x)", e);
        return HX_ERR_TIMEOUT;
    }
    return HX_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

hx_status hx_denoiser_create(hx_context* ctx, hx_denoiser** out) {
    HX_CHECK_ARG(ctx && out, "null argument");
    *out = nullptr;
    std::unique_ptr<hx_denoiser> dn(new hx_denoiser());
    dn->ctx = ctx;
    HX_CUDA(cudaSetDevice(ctx->device));
    size_t off = 0;
    for (int l = 0; l < kNumLayers; ++l) {
        Layer& L = dn->layers[l];
        const LayerSpec& S = kLayers[l];
        L.cin = kTensors[S.src0].C + (S.src1 >= 0 ? kTensors[S.src1].C : 0);
        L.cout = S.cout;
        L.nf = round_up(L.cout, 16);
        L.cd = round_up(L.cout, 32);
        L.off = off;
        off += (size_t)9 * L.cout * L.cin + L.cout;
    }
    dn->nparams = off;
    auto fail = [&](hx_status s) {
        for (void* a : dn->allocs) hx_free(ctx, a);
        return s;
    };
    hx_status s;
    if ((s = dn_alloc(ctx, dn->allocs, (void**)&dn->params, off * 4)) != HX_OK) return fail(s);
    if ((s = dn_alloc(ctx, dn->allocs, (void**)&dn->grads, off * 4)) != HX_OK) return fail(s);
    if ((s = dn_alloc(ctx, dn->allocs, (void**)&dn->adam_m, off * 4)) != HX_OK) return fail(s);
    if ((s = dn_alloc(ctx, dn->allocs, (void**)&dn->adam_v, off * 4)) != HX_OK) return fail(s);
    if ((s = dn_alloc(ctx, dn->allocs, (void**)&dn->err, 256)) != HX_OK) return fail(s);
    for (int l = 0; l < kNumLayers; ++l) {
        Layer& L = dn->layers[l];
        if ((s = dn_alloc(ctx, dn->allocs, (void**)&L.wf, (size_t)9 * L.nf * L.cin * 2)) != HX_OK) return fail(s);
        if ((s = dn_alloc(ctx, dn->allocs, (void**)&L.wd, (size_t)9 * L.cin * L.cd * 2)) != HX_OK) return fail(s);
        if ((s = make_w_map(&L.wf_map, L.wf, L.cin, L.nf)) != HX_OK) return fail(s);
        if ((s = make_w_map(&L.wd_map, L.wd, L.cd, L.cin)) != HX_OK) return fail(s);
    }
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) return fail(HX_ERR_DEVICE);
    *out = dn.release();
    return HX_OK;
}

hx_status hx_denoiser_destroy(hx_denoiser* dn) {
    if (!dn) return HX_OK;
    cudaStreamSynchronize(dn->ctx->stream);
    if (dn->train_plan) free_plan(dn->ctx, dn->train_plan.get());
    for (auto& p : dn->infer_plans) free_plan(dn->ctx, p.get());
    for (void* a : dn->allocs) hx_free(dn->ctx, a);
    delete dn;
    return HX_OK;
}

hx_status hx_denoiser_num_params(hx_denoiser* dn, uint64_t* n) {
    HX_CHECK_ARG(dn && n, "null argument");
    *n = dn->nparams;
    return HX_OK;
}

hx_status hx_denoiser_set_params(hx_denoiser* dn, const float* host, uint64_t n) {
    HX_CHECK_ARG(dn && host, "null argument");
    HX_CHECK_ARG(n == dn->nparams, "expected %llu parameters, got %llu", (unsigned long long)dn->nparams,
                 (unsigned long long)n);
    HX_CUDA(cudaSetDevice(dn->ctx->device));
    HX_CUDA(cudaMemcpyAsync(dn->params, host, n * 4, cudaMemcpyHostToDevice, dn->ctx->stream));
    HX_CUDA(cudaMemsetAsync(dn->adam_m, 0, n * 4, dn->ctx->stream));
    HX_CUDA(cudaMemsetAsync(dn->adam_v, 0, n * 4, dn->ctx->stream));
    dn->step = 0;
    HX_TRY(refresh_weights(dn, false, 0.0f));
    HX_CUDA(cudaStreamSynchronize(dn->ctx->stream));
    return HX_OK;
}

// He-uniform weights (bound sqrt(6 / fan_in), fan_in = 9 cin) from a
// SplitMix64 stream of the seed, zero biases; resets the Adam state.
hx_status hx_denoiser_init_params(hx_denoiser* dn, uint64_t seed) {
    HX_CHECK_ARG(dn, "null argument");
    std::vector<float> p(dn->nparams);
    uint64_t x = seed;
    auto next = [&]() {  // SplitMix64 (Steele, Lea, Flood 2014)
        uint64_t z = (x += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    };
    for (int l = 0; l < kNumLayers; ++l) {
        const Layer& L = dn->layers[l];
        const double bound = std::sqrt(6.0 / (9.0 * L.cin));
        float* w = p.data() + L.off;
        for (size_t k = 0; k < (size_t)9 * L.cout * L.cin; ++k)
            w[k] = (float)(((double)(next() >> 11) * 0x1.0p-53 * 2.0 - 1.0) * bound);
        for (int k = 0; k < L.cout; ++k) w[(size_t)9 * L.cout * L.cin + k] = 0.0f;
    }
    return hx_denoiser_set_params(dn, p.data(), p.size());
}

hx_status hx_denoiser_get_params(hx_denoiser* dn, float* host, uint64_t n) {
    HX_CHECK_ARG(dn && host && n == dn->nparams, "bad argument");
    HX_CUDA(cudaSetDevice(dn->ctx->device));
    HX_CUDA(cudaMemcpyAsync(host, dn->params, n * 4, cudaMemcpyDeviceToHost, dn->ctx->stream));
    HX_CUDA(cudaStreamSynchronize(dn->ctx->stream));
    return HX_OK;
}

hx_status hx_denoiser_get_gradients(hx_denoiser* dn, float* host, uint64_t n) {
    HX_CHECK_ARG(dn && host && n == dn->nparams, "bad argument");
    HX_CUDA(cudaSetDevice(dn->ctx->device));
    HX_CUDA(cudaMemcpyAsync(host, dn->grads, n * 4, cudaMemcpyDeviceToHost, dn->ctx->stream));
    HX_CUDA(cudaStreamSynchronize(dn->ctx->stream));
    return HX_OK;
}

hx_status hx_denoiser_forward_backward(hx_denoiser* dn, const float* d_features, const float* d_targets, uint32_t n,
                                       uint32_t h, uint32_t w, float* loss) {
    HX_CHECK_ARG(dn && d_features && d_targets, "null argument");
    HX_CHECK_ARG(n >= 1 && h >= 16 && w >= 16 && h % 16 == 0 && w % 16 == 0,
                 "training crops must be multiples of 16 pixels (got %ux%u)", w, h);
    hx_context* ctx = dn->ctx;
    HX_CUDA(cudaSetDevice(ctx->device));
    Plan* p = nullptr;
    HX_TRY(get_plan(dn, (int)n, (int)h, (int)w, true, &p));
    const size_t P = (size_t)n * h * w;
    k_pack_input<<<grid_for(P, 256, ctx->num_sms), 256, 0, ctx->stream>>>(d_features, h, w, h, w, n, p->t[X]);
    HX_CUDA(cudaGetLastError());
    HX_TRY(run_forward(dn, p));
    k_loss<<<kLossBlocks, 256, 0, ctx->stream>>>(p->y, reinterpret_cast<const float4*>(d_targets), P, dn->loss_kind,
                                                  p->g[GYT], p->loss_part);
    HX_CUDA(cudaGetLastError());
    HX_TRY(run_backward(dn, p, (float)(1.0 / (3.0 * (double)P))));
    if (loss) {
        float part[kLossBlocks];
        HX_CUDA(cudaMemcpyAsync(part, p->loss_part, sizeof(part), cudaMemcpyDeviceToHost, ctx->stream));
        HX_TRY(check_err(dn));
        double s = 0.0;
        for (int i = 0; i < kLossBlocks; ++i) s += part[i];
        *loss = (float)(s / (3.0 * (double)P));
    } else {
        HX_TRY(check_err(dn));
    }
    return HX_OK;
}

hx_status hx_denoiser_set_loss(hx_denoiser* dn, uint32_t kind) {
    HX_CHECK_ARG(dn && kind <= HX_DN_LOSS_L2_LINEAR, "hx_denoiser_set_loss: bad argument");
    dn->loss_kind = kind;
    return HX_OK;
}

hx_status hx_denoiser_adam_step(hx_denoiser* dn, float lr) {
    HX_CHECK_ARG(dn, "null argument");
    HX_CUDA(cudaSetDevice(dn->ctx->device));
    HX_TRY(refresh_weights(dn, true, lr));
    return HX_OK;
}

hx_status hx_denoiser_train_step(hx_denoiser* dn, const float* d_features, const float* d_targets, uint32_t n,
                                 uint32_t h, uint32_t w, float lr, float* loss) {
    HX_TRY(hx_denoiser_forward_backward(dn, d_features, d_targets, n, h, w, loss));
    return hx_denoiser_adam_step(dn, lr);
}

hx_status hx_denoiser_infer(hx_denoiser* dn, const float* d_features, uint32_t n, uint32_t h, uint32_t w,
                            float* d_out_rgba) {
    HX_CHECK_ARG(dn && d_features && d_out_rgba, "null argument");
    HX_CHECK_ARG(n >= 1 && h >= 1 && w >= 1, "empty image");
    hx_context* ctx = dn->ctx;
    HX_CUDA(cudaSetDevice(ctx->device));
    const int H = round_up((int)h, 16), W = round_up((int)w, 16);
    Plan* p = nullptr;
    HX_TRY(get_plan(dn, (int)n, H, W, false, &p));
    const size_t P = (size_t)n * H * W;
    k_pack_input<<<grid_for(P, 256, ctx->num_sms), 256, 0, ctx->stream>>>(d_features, h, w, H, W, n, p->t[X]);
    HX_CUDA(cudaGetLastError());
    HX_TRY(run_forward(dn, p));
    const size_t Po = (size_t)n * h * w;
    k_unpack_output<<<grid_for(Po, 256, ctx->num_sms), 256, 0, ctx->stream>>>(p->y, h, w, H, W, n,
                                                                             reinterpret_cast<float4*>(d_out_rgba));
    HX_CUDA(cudaGetLastError());
    return HX_OK;
}

hx_status hx_denoiser_check(hx_denoiser* dn) {
    HX_CHECK_ARG(dn, "null argument");
    return check_err(dn);
}

hx_status hx_denoiser_set_wait_budget(hx_denoiser* dn, uint64_t cycles) {
    HX_CHECK_ARG(dn, "null argument");
    HX_CHECK_ARG(cycles <= (uint64_t)tc::kWaitCycles, "wait budget above the default %lld cycles", tc::kWaitCycles);
    dn->wait_cycles = cycles ? (long long)cycles : tc::kWaitCycles;
    return HX_OK;
}

// Test access to a stored activation of the last forward pass (BF16 bits,
// NHWC at that tensor's level), by tensor index in network order.
hx_status hx_denoiser_read_tensor(hx_denoiser* dn, uint32_t training, uint32_t index, uint32_t gradient, void* host,
                                  uint64_t bytes) {
    HX_CHECK_ARG(dn && host, "null argument");
    HX_CHECK_ARG(index < NT, "tensor index %u out of range", index);
    Plan* p = training ? dn->train_plan.get() : dn->last_infer;
    HX_CHECK_ARG(p, "no %s pass has run", training ? "training" : "inference");
    const void* src = gradient ? (const void*)p->g[index] : (const void*)p->t[index];
    HX_CHECK_ARG(src, "tensor not stored");
    const int lev = kTensors[index].level;
    const size_t need = (size_t)p->n * level_dim(p->H, lev) * level_dim(p->W, lev) * kTensors[index].C * 2;
    HX_CHECK_ARG(bytes == need, "tensor %u holds %zu bytes", index, need);
    HX_CUDA(cudaSetDevice(dn->ctx->device));
    HX_CUDA(cudaMemcpyAsync(host, src, bytes, cudaMemcpyDeviceToHost, dn->ctx->stream));
    HX_CUDA(cudaStreamSynchronize(dn->ctx->stream));
    return HX_OK;
}

hx_status hx_denoiser_read_output(hx_denoiser* dn, uint32_t training, float* host, uint64_t count) {
    HX_CHECK_ARG(dn && host, "null argument");
    Plan* p = training ? dn->train_plan.get() : dn->last_infer;
    HX_CHECK_ARG(p, "no pass has run");
    HX_CHECK_ARG(count == (uint64_t)p->n * p->H * p->W * 4, "output holds %llu floats",
                 (unsigned long long)p->n * p->H * p->W * 4);
    HX_CUDA(cudaSetDevice(dn->ctx->device));
    HX_CUDA(cudaMemcpyAsync(host, p->y, count * 4, cudaMemcpyDeviceToHost, dn->ctx->stream));
    HX_CUDA(cudaStreamSynchronize(dn->ctx->stream));
    return HX_OK;
}

}  // extern "C"
