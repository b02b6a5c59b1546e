// integrator.cu — the wavefront path integrator (replaces the ray-tracing
// pipeline of src/engine/gfx/path_integrator.cpp and the shaders
// path_trace_*.glsl) and the accumulate / tone-map passes
// (path_trace_rgen.glsl:217-248, tone_map.frag).
//
// One progressive frame = one sample per pixel of the current tile.  Several
// frames can share one wavefront (paths p = pixel * nframes + frame); the
// accumulation then replays them in frame order, so the image is identical
// to frame-by-frame rendering.
//
// Per bounce:  k_extend (closest hit of this bounce's rays + any-hit
// visibility of the previous bounce's shadow rays, which add their NEE
// contribution)  ->  k_shade (surface, NEE sample, BSDF sample, Russian
// roulette; appends shadow rays and next-bounce rays with warp-aggregated
// atomics); a last k_extend traces the final bounce's shadow rays.  Queue
// lengths live in device memory and every kernel is a grid-stride or
// persistent loop over them, so a frame is enqueued without host round
// trips.
#include "wavefront.cuh"

#include <algorithm>
#include <cstring>
#include <vector>

namespace {

// Traversal records of caller rays (origin xyz, tmin, direction xyz, tmax)
// for the production traversal kernels; the queue holds n extension rays and
// no shadow ray.
__global__ void k_ray_records(const float* __restrict__ rays, uint32_t n, uint32_t any_hit, float4* __restrict__ qo,
                              float4* __restrict__ qr0, float4* __restrict__ qr1, uint32_t* counters) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float* r = rays + 8 * (size_t)i;
        float4 r0, r1;
        ray_record(v3(r[4], r[5], r[6]), r[7], any_hit != 0, r0, r1);
        qo[i] = make_float4(r[0], r[1], r[2], r[3]);
        qr0[i] = r0;
        qr1[i] = r1;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        counters[0] = n;
        counters[2] = 0;
        counters[4] = 0;
    }
}

__global__ void k_rng_streams(uint32_t kind, const uint32_t* seeds, uint32_t n, uint32_t draws, uint32_t* out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Rng r;
    if (kind == 0) {
        r.s0 = wang_hash(seeds[2 * i]);
        r.s1 = wang_hash(seeds[2 * i + 1]);
        rng_next<0>(r);
    } else {
        r.s0 = pcg_hash(pcg_hash(seeds[2 * i]) + seeds[2 * i + 1]);
        r.s1 = 0;
    }
    for (uint32_t k = 0; k < draws; ++k) out[(size_t)i * draws + k] = rng_next_k(kind, r);
}

// Hits / radiance of one W x H frame's paths (slot = path = pix in the
// rect's tiled pixel order, pix_xy) to row-major pixel order.  Caller-supplied
// rays pass W = n, H = 1, for which the order is the identity.
__global__ void k_hits_to_host_layout(const float4* __restrict__ hits, uint32_t W, uint32_t H, hx_hit* out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W * H) return;
    const Rect rect{0, 0, W, H};
    const float4 h = hits[pix_of_xy(rect, i % W, i / W)];
    out[i].t = h.x;
    out[i].prim = __float_as_uint(h.y);
    out[i].u = h.z;
    out[i].v = h.w;
}

__global__ void k_radiance_out(const float4* __restrict__ L, uint32_t W, uint32_t H, float* out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W * H) return;
    const Rect rect{0, 0, W, H};
    const float4 l = L[pix_of_xy(rect, i % W, i / W)];
    out[3 * (size_t)i] = l.x;
    out[3 * (size_t)i + 1] = l.y;
    out[3 * (size_t)i + 2] = l.z;
}

}  // namespace

// ---------------------------------------------------------------------------
// Integrator object.
// ---------------------------------------------------------------------------
struct hx_integrator {
    hx_context* ctx = nullptr;
    const hx_scene* scene = nullptr;
    hx_integrator_desc desc{};
    uint32_t capacity = 0;  // paths per wavefront
    Queues q{};
    std::vector<void*> allocs;
    float4* acc = nullptr;
    float4* comp = nullptr;
    uint32_t* count_map = nullptr;
    float4* resolved = nullptr;
    uchar4* ldr = nullptr;
    hx_hit* hits_host_layout = nullptr;
    float* rgb_tmp = nullptr;
    float4* aov_a = nullptr;      // accumulated first-hit albedo + depth feature (AOV accumulation on)
    float4* aov_n = nullptr;      // accumulated first-hit shading normal
    bool aov = false;
    uint32_t aov_frames = 0;      // frames in the AOV buffers since they were cleared
    float* feat = nullptr;        // denoiser features (12 floats per pixel), on first use
    float4* denoised = nullptr;
    // progressive state (path_integrator.h:46-53)
    uint32_t accumulated = 0, tile_idx = 0;
    std::vector<Rect> tiles;
    // timing / counting
    bool timing = false;
    bool counting = false;
    hx_stats stats{};
    int grid_trace = 0, grid_shade = 0, grid_gen = 0, grid_batched = 0;
    uint32_t* status_host = nullptr;  // pinned copy of the device status word
};

static void compute_tiles(hx_integrator* it) {  // path_integrator.cpp:312-336
    it->tiles.clear();
    const uint32_t T = 128;
    if (it->desc.tiled) {
        uint32_t nx = (it->desc.width + T - 1) / T, ny = (it->desc.height + T - 1) / T;
        for (uint32_t x = 0; x < nx; ++x)
            for (uint32_t y = 0; y < ny; ++y) {
                Rect r{x * T, y * T, std::min(T, it->desc.width - x * T), std::min(T, it->desc.height - y * T)};
                it->tiles.push_back(r);
            }
    } else {
        it->tiles.push_back(Rect{0, 0, it->desc.width, it->desc.height});
    }
}

extern "C" hx_status hx_integrator_create(hx_context* ctx, const hx_scene* scene, const hx_integrator_desc* desc,
                                          hx_integrator** out) {
    HX_CHECK_ARG(ctx && scene && desc && out, "hx_integrator_create: null argument");
    HX_CHECK_ARG(desc->width > 0 && desc->height > 0 && desc->width <= 16384 && desc->height <= 16384,
                 "hx_integrator_create: bad extents %ux%u", desc->width, desc->height);
    HX_CHECK_ARG(desc->policy.rng <= 1 && desc->policy.accumulation <= 1 && desc->policy.ray_offset <= 1,
                 "hx_integrator_create: bad policy");
    HX_CHECK_ARG(desc->max_ray_bounces <= 64, "hx_integrator_create: max_ray_bounces %u above 64",
                 desc->max_ray_bounces);
    HX_CHECK_ARG(!(desc->policy.visualize_nans && desc->policy.accumulation == HX_ACCUM_KAHAN),
                 "hx_integrator_create: visualize_nans needs running-mean accumulation");
    HX_CUDA(cudaSetDevice(ctx->device));
    hx_integrator* it = new hx_integrator();
    it->ctx = ctx;
    it->scene = scene;
    it->desc = *desc;
    uint64_t npix = (uint64_t)desc->width * desc->height;
    uint64_t cap = desc->max_paths_in_flight ? desc->max_paths_in_flight : std::max<uint64_t>(npix, 1u << 22);
    cap = std::max<uint64_t>(cap, std::min<uint64_t>(npix, 128 * 128));
    if (cap > 0x7fffffffull) cap = 0x7fffffffull;
    it->capacity = (uint32_t)cap;
    auto fail = [&](hx_status s) { hx_integrator_destroy(it); return s; };
    auto alloc = [&](void** p, size_t bytes) -> hx_status {
        hx_status s = hx_alloc(ctx, p, bytes);
        if (s == HX_OK) it->allocs.push_back(*p);
        return s;
    };
    hx_status s = HX_OK;
#define HX_A(ptr, bytes) if ((s = alloc((void**)&(ptr), (bytes))) != HX_OK) return fail(s)
    for (int k = 0; k < 2; ++k) {
        HX_A(it->q.o[k], 16 * cap);
        HX_A(it->q.d[k], 16 * cap);
        HX_A(it->q.r0[k], 16 * cap);  // FP32 payloads (the policy may change after creation)
        HX_A(it->q.r1[k], 16 * cap);
        HX_A(it->q.p[k], 4 * cap);
    }
    HX_A(it->q.hit, 16 * cap);
    HX_A(it->q.so, 16 * cap);
    HX_A(it->q.sr0, 16 * cap);
    HX_A(it->q.sr1, 16 * cap);
    HX_A(it->q.sc, 16 * cap);
    HX_A(it->q.T, 16 * cap);
    HX_A(it->q.L, 16 * cap);
    HX_A(it->q.rng, 8 * cap);
    HX_A(it->q.shade_list, 4 * cap);
    it->q.shade_cap = (uint32_t)cap;
    HX_A(it->q.part, 4 * (size_t)kPartBlocks);
    HX_A(it->q.counters, 64);
    HX_A(it->q.stats, 128);
    HX_A(it->q.status, 64);
    HX_A(it->acc, 16 * npix);
    HX_A(it->comp, 16 * npix);
    HX_A(it->count_map, 4 * npix);
    HX_A(it->resolved, 16 * npix);
    HX_A(it->ldr, 4 * npix);
    HX_A(it->hits_host_layout, sizeof(hx_hit) * npix);
    HX_A(it->rgb_tmp, 12 * npix);
#undef HX_A
    if (cudaHostAlloc((void**)&it->status_host, 64, cudaHostAllocDefault) != cudaSuccess) {
        it->status_host = nullptr;
        hx_set_error("hx_integrator_create: pinned status word allocation failed");
        return fail(HX_ERR_DEVICE);
    }
    *it->status_host = 0;
    cudaStream_t st = ctx->stream;
    HX_CUDA(cudaMemsetAsync(it->acc, 0, 16 * npix, st));
    HX_CUDA(cudaMemsetAsync(it->comp, 0, 16 * npix, st));
    HX_CUDA(cudaMemsetAsync(it->count_map, 0, 4 * npix, st));
    HX_CUDA(cudaMemsetAsync(it->q.stats, 0, 128, st));
    HX_CUDA(cudaMemsetAsync(it->q.status, 0, 64, st));
    int per_sm = 0;
    HX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_extend<false, false>, kTraceThreads, 0));
    it->grid_trace = std::max(1, per_sm) * ctx->num_sms;
    HX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_shade<false>, kShadeThreads, 0));
    it->grid_shade = std::max(1, per_sm) * ctx->num_sms;
    it->grid_gen = ctx->num_sms * 8;
    HX_CUDA(set_carveouts(k_extend_batched<false, false>, k_extend_batched<true, false>, k_extend_batched<false, true>,
                          k_extend_batched<true, true>, k_extend_batched<false, false, true>,
                          k_extend_batched<true, false, true>, k_extend_batched<false, true, true>,
                          k_extend_batched<true, true, true>));
    HX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_extend_batched<false>, kTraceThreads, 0));
    it->grid_batched = std::max(1, per_sm) * ctx->num_sms;
    compute_tiles(it);
    *out = it;
    return HX_OK;
}

extern "C" hx_status hx_integrator_destroy(hx_integrator* it) {
    if (!it) return HX_OK;
    if (it->ctx) cudaStreamSynchronize(it->ctx->stream);
    for (void* p : it->allocs) hx_free(it->ctx, p);
    if (it->status_host) cudaFreeHost(it->status_host);
    delete it;
    return HX_OK;
}

// The device status word: kernels set bit 0 (traversal-stack overflow or a
// malformed tree) and bit 1 (a shading list that does not cover a bounce's
// rays).  Calls that synchronise anyway queue a copy of the word into pinned
// memory before their wait (queue_status) and report it after
// (report_status), so the production path adds no synchronisation.
static hx_status queue_status(hx_integrator* it) {
    HX_CUDA(cudaMemcpyAsync(it->status_host, it->q.status, 4, cudaMemcpyDeviceToHost, it->ctx->stream));
    return HX_OK;
}
static hx_status report_status(hx_integrator* it) {
    const uint32_t st = *it->status_host;
    if (st & 3u) {
        *it->status_host = 0;
        hx_set_error((st & 1u) ? "BVH traversal stack overflow (status word 0x%x)"
                               : "shading list does not cover the bounce's rays (status word 0x%x)",
                     st);
        cudaMemsetAsync(it->q.status, 0, 4, it->ctx->stream);
        return HX_ERR_DEVICE;
    }
    return HX_OK;
}
static hx_status check_status(hx_integrator* it) {
    HX_TRY(queue_status(it));
    HX_CUDA(cudaStreamSynchronize(it->ctx->stream));
    return report_status(it);
}

struct StageTimer {
    hx_integrator* it;
    cudaEvent_t a = nullptr, b = nullptr;
    double* acc;
    StageTimer(hx_integrator* i, double* target) : it(i), acc(target) {
        if (it->timing) {
            cudaEventCreate(&a);
            cudaEventCreate(&b);
            cudaEventRecord(a, it->ctx->stream);
        }
    }
    ~StageTimer() {
        if (it->timing) {
            cudaEventRecord(b, it->ctx->stream);
            cudaEventSynchronize(b);
            float ms = 0;
            cudaEventElapsedTime(&ms, a, b);
            *acc += ms;
            cudaEventDestroy(a);
            cudaEventDestroy(b);
        }
    }
};

// Traces nframes frames of the rect through all bounces; leaves per-path
// radiance in q.L.  With accumulate, folds them into the image.
// Ray-debug launch (gather_debug_rays): n paths through one pixel, segments
// recorded by k_shade<false, true> into q's debug buffers; no accumulation.
struct DebugLaunch {
    uint32_t px, py, n;
};

static hx_status run_wavefront(hx_integrator* it, const hx_frame_desc& f, Rect rect, uint32_t frame0, uint32_t nframes,
                               bool accumulate, const DebugLaunch* dbg = nullptr) {
    hx_context* ctx = it->ctx;
    cudaStream_t st = ctx->stream;
    const DevScene& s = it->scene->d;
    Policy P = make_policy(it->desc.policy);
    uint32_t npix = rect.w * rect.h;
    uint32_t total = npix * nframes;
    const bool fp16 = it->desc.policy.payload == HX_PAYLOAD_FP16;
    Queues qs = it->q;
    qs.list_mode = shade_list_mode(total, fp16);
    if (qs.list_mode == 0u) qs.shade_list = nullptr;  // shade in queue order
    it->stats.paths += total;
    {
        StageTimer t(it, &it->stats.ms_raygen);
        if (dbg)
            k_raygen_debug<<<it->grid_gen, kGenThreads, 0, st>>>(f, dbg->px, dbg->py, it->desc.width, it->desc.height, dbg->n,
                                                                 frame0, P.rng, it->q);
        else if (fp16)
            k_raygen<true><<<it->grid_gen, kGenThreads, 0, st>>>(f, rect, it->desc.width, it->desc.height, frame0, nframes, 0,
                                                                 total, P.rng, it->q);
        else
            k_raygen<false><<<it->grid_gen, kGenThreads, 0, st>>>(f, rect, it->desc.width, it->desc.height, frame0, nframes, 0,
                                                                  total, P.rng, it->q);
        it->stats.kernel_launches++;
    }
    {
        // bounce b: k_extend traces the extension rays of b and the shadow
        // rays of b - 1; a last launch traces the final bounce's shadow rays.
        // The camera hit is always shaded (the closest-hit shader runs for
        // every traced ray; only the indirect ray obeys (depth + 1) <
        // max_ray_bounces, path_trace_rchit.glsl:577), so a limit of 0 traces
        // like 1.
        const uint32_t bounces = std::max<uint32_t>(1u, it->desc.max_ray_bounces);
        for (uint32_t b = 0; b <= bounces; ++b) {
            const int cur = b & 1;
            {
                StageTimer t(it, &it->stats.ms_trace);
                HX_CUDA(cudaMemsetAsync(it->q.counters + 4, 0, 24, st));  // fetch cursor, miss / hit counts
#define HX_EXTEND(COUNT, FP16)                                                                                 \
    launch_extend<COUNT, FP16>(s, qs, it->grid_batched, it->grid_trace, st, it->q.o[cur], it->q.r0[cur], it->q.r1[cur], \
                               it->q.p[cur], it->q.counters + cur, it->q.counters + 4)
                if (it->counting) {
                    if (fp16) HX_EXTEND(true, true);
                    else HX_EXTEND(true, false);
                } else {
                    if (fp16) HX_EXTEND(false, true);
                    else HX_EXTEND(false, false);
                }
#undef HX_EXTEND
                it->stats.trace_launches++;
                it->stats.kernel_launches++;
            }
            if (b == bounces) break;
            if (b == 0 && it->aov && accumulate) {
                if (fp16)
                    k_aov_accumulate<true><<<it->grid_gen, kGenThreads, 0, st>>>(s, rect, frame0, nframes, it->q.hit, it->aov_a,
                                                                              it->aov_n, it->desc.width);
                else
                    k_aov_accumulate<false><<<it->grid_gen, kGenThreads, 0, st>>>(s, rect, frame0, nframes, it->q.hit, it->aov_a,
                                                                               it->aov_n, it->desc.width);
                it->aov_frames += nframes;
                it->stats.kernel_launches++;
            }
            HX_CUDA(cudaMemsetAsync(it->q.counters + (cur ^ 1), 0, 4, st));
            HX_CUDA(cudaMemsetAsync(it->q.counters + 2, 0, 4, st));
            {
                StageTimer t(it, &it->stats.ms_shade);
                it->stats.kernel_launches += fp16 ? launch_shade_partition<true>(qs, cur, st)
                                                  : launch_shade_partition<false>(qs, cur, st);
                const float bias = it->desc.shadow_ray_bias;
                const uint32_t nb = it->desc.max_ray_bounces;
                if (P.ray_offset) {
                    if (dbg) k_shade<false, true, true><<<it->grid_shade, kShadeThreads, 0, st>>>(s, P, nb, bias, cur, qs);
                    else if (fp16) k_shade<true, false, true><<<it->grid_shade, kShadeThreads, 0, st>>>(s, P, nb, bias, cur, qs);
                    else k_shade<false, false, true><<<it->grid_shade, kShadeThreads, 0, st>>>(s, P, nb, bias, cur, qs);
                } else if (dbg) k_shade<false, true><<<it->grid_shade, kShadeThreads, 0, st>>>(s, P, nb, bias, cur, qs);
                else if (fp16) k_shade<true><<<it->grid_shade, kShadeThreads, 0, st>>>(s, P, nb, bias, cur, qs);
                else k_shade<false><<<it->grid_shade, kShadeThreads, 0, st>>>(s, P, nb, bias, cur, qs);
                it->stats.kernel_launches++;
            }
        }
    }
    if (accumulate) {
        StageTimer t(it, &it->stats.ms_accumulate);
        bool kahan = it->desc.policy.accumulation == HX_ACCUM_KAHAN;
        k_accumulate<<<it->grid_gen, kGenThreads, 0, st>>>(rect, it->desc.width, frame0, nframes, it->desc.policy.radiance_clamp,
                                                           kahan ? 1u : 0u, it->desc.policy.visualize_nans ? 1u : 0u, it->q.L,
                                                           it->acc, it->comp);
        k_count_add<<<it->grid_gen, kGenThreads, 0, st>>>(rect, it->desc.width, nframes, it->count_map);
        it->stats.kernel_launches += 2;
    }
    HX_CUDA(cudaGetLastError());
    return HX_OK;
}

static void clear_images(hx_integrator* it) {  // renderer.cpp:212-223
    size_t npix = (size_t)it->desc.width * it->desc.height;
    cudaMemsetAsync(it->acc, 0, 16 * npix, it->ctx->stream);
    cudaMemsetAsync(it->comp, 0, 16 * npix, it->ctx->stream);
    cudaMemsetAsync(it->count_map, 0, 4 * npix, it->ctx->stream);
    if (it->aov_a) {
        cudaMemsetAsync(it->aov_a, 0, 16 * npix, it->ctx->stream);
        cudaMemsetAsync(it->aov_n, 0, 16 * npix, it->ctx->stream);
    }
    it->aov_frames = 0;
}

extern "C" hx_status hx_integrator_set_aov_accumulation(hx_integrator* it, uint32_t enabled) {
    HX_CHECK_ARG(it, "null integrator");
    if (enabled && !it->aov_a) {
        const size_t npix = (size_t)it->desc.width * it->desc.height;
        HX_TRY(hx_alloc_t(it->ctx, &it->aov_a, npix));
        it->allocs.push_back(it->aov_a);
        HX_TRY(hx_alloc_t(it->ctx, &it->aov_n, npix));
        it->allocs.push_back(it->aov_n);
        HX_CUDA(cudaMemsetAsync(it->aov_a, 0, 16 * npix, it->ctx->stream));
        HX_CUDA(cudaMemsetAsync(it->aov_n, 0, 16 * npix, it->ctx->stream));
    }
    if ((enabled != 0) != it->aov) {  // AOVs must cover the same samples as the image
        it->accumulated = 0;
        it->tile_idx = 0;
    }
    it->aov = enabled != 0;
    return HX_OK;
}

extern "C" hx_status hx_integrator_render_frames(hx_integrator* it, const hx_frame_desc* frame, uint32_t num_frames) {
    HX_CHECK_ARG(it && frame, "hx_integrator_render_frames: null argument");
    HX_CUDA(cudaSetDevice(it->ctx->device));
    std::memset(&it->stats, 0, sizeof(it->stats));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (it->timing) {
        HX_CUDA(cudaEventCreate(&e0));
        HX_CUDA(cudaEventCreate(&e1));
        HX_CUDA(cudaEventRecord(e0, it->ctx->stream));
    }
    HX_CUDA(cudaMemsetAsync(it->q.stats, 0, 128, it->ctx->stream));
    uint32_t left = num_frames;
    while (left > 0 && it->tile_idx < it->tiles.size()) {
        Rect r = it->tiles[it->tile_idx];
        uint32_t npix = r.w * r.h;
        uint32_t remaining = it->desc.max_samples - it->accumulated;
        uint32_t batch = std::min(left, remaining);
        batch = std::min<uint32_t>(batch, std::max<uint32_t>(1, it->capacity / npix));
        if (batch == 0) break;
        if (it->accumulated == 0 && it->tile_idx == 0) clear_images(it);
        HX_TRY(run_wavefront(it, *frame, r, it->accumulated, batch, true));
        it->accumulated += batch;
        left -= batch;
        if (it->accumulated >= it->desc.max_samples) {  // path_integrator.cpp:78-82
            it->accumulated = 0;
            it->tile_idx++;
        }
    }
    if (it->timing || it->counting) {
        if (!it->timing) {
            HX_CUDA(cudaEventCreate(&e0));
            HX_CUDA(cudaEventCreate(&e1));
            HX_CUDA(cudaEventRecord(e0, it->ctx->stream));
        }
        HX_CUDA(cudaEventRecord(e1, it->ctx->stream));
        HX_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        HX_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        it->stats.ms_total = ms;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        unsigned long long h[9];
        HX_CUDA(cudaMemcpy(h, it->q.stats, sizeof(h), cudaMemcpyDeviceToHost));
        it->stats.extension_rays = h[0];
        it->stats.shadow_rays = h[1];
        it->stats.node_visits = h[2];
        it->stats.tri_tests = h[3];
        it->stats.warp_node_steps = h[4];
        it->stats.warp_tri_steps = h[5];
        it->stats.warp_loop_iters = h[6];
        it->stats.lane_loop_busy = h[7];
        it->stats.alpha_tests = h[8];
        HX_TRY(check_status(it));
    }
    return HX_OK;
}

extern "C" hx_status hx_integrator_render(hx_integrator* it, const hx_frame_desc* frame) {
    return hx_integrator_render_frames(it, frame, 1);
}

extern "C" hx_status hx_integrator_restart_bake(hx_integrator* it) {
    HX_CHECK_ARG(it, "null integrator");
    it->accumulated = 0;
    it->tile_idx = 0;
    return HX_OK;
}
extern "C" hx_status hx_integrator_set_max_ray_bounces(hx_integrator* it, uint32_t n) {
    HX_CHECK_ARG(it && n <= 64, "hx_integrator_set_max_ray_bounces: bad value");
    it->desc.max_ray_bounces = n;
    return HX_OK;
}
extern "C" hx_status hx_integrator_set_max_samples(hx_integrator* it, uint32_t n) {
    HX_CHECK_ARG(it && n >= 1, "hx_integrator_set_max_samples: bad value");
    it->desc.max_samples = n;
    return HX_OK;
}
extern "C" hx_status hx_integrator_set_shadow_ray_bias(hx_integrator* it, float bias) {
    HX_CHECK_ARG(it, "null integrator");
    it->desc.shadow_ray_bias = bias;
    return HX_OK;
}
extern "C" hx_status hx_integrator_set_tiled(hx_integrator* it, uint32_t tiled) {  // path_integrator.cpp:116-120
    HX_CHECK_ARG(it, "null integrator");
    it->desc.tiled = tiled ? 1u : 0u;
    compute_tiles(it);
    return HX_OK;
}
extern "C" hx_status hx_integrator_set_policy(hx_integrator* it, const hx_policy* p) {
    HX_CHECK_ARG(it && p && p->rng <= 1 && p->accumulation <= 1 && p->ray_offset <= 1,
                 "hx_integrator_set_policy: bad policy");
    HX_CHECK_ARG(!(p->visualize_nans && p->accumulation == HX_ACCUM_KAHAN),
                 "hx_integrator_set_policy: visualize_nans needs running-mean accumulation");
    it->desc.policy = *p;
    return HX_OK;
}
extern "C" hx_status hx_integrator_progress(const hx_integrator* it, uint32_t* acc, uint32_t* tile, uint32_t* target) {
    HX_CHECK_ARG(it, "null integrator");
    if (acc) *acc = it->desc.max_samples * it->tile_idx + it->accumulated;
    if (tile) *tile = it->tile_idx;
    if (target) *target = it->desc.max_samples * (uint32_t)it->tiles.size();
    return HX_OK;
}

extern "C" hx_status hx_integrator_tonemap(hx_integrator* it, uint32_t op, float exposure, uint8_t* host_rgba8) {
    HX_CHECK_ARG(it && op <= 2, "hx_integrator_tonemap: bad argument");
    uint32_t W = it->desc.width, H = it->desc.height;
    cudaStream_t st = it->ctx->stream;
    bool kahan = it->desc.policy.accumulation == HX_ACCUM_KAHAN;
    const float4* src = it->acc;
    if (kahan) {
        k_resolve<<<it->grid_gen, kGenThreads, 0, st>>>(it->acc, it->count_map, W * H, 1u, it->resolved);
        src = it->resolved;
    }
    k_tonemap<<<it->grid_gen, kGenThreads, 0, st>>>(src, nullptr, W, H, op, exposure, it->ldr);
    HX_CUDA(cudaGetLastError());
    if (host_rgba8) {
        HX_CUDA(cudaMemcpyAsync(host_rgba8, it->ldr, 4 * (size_t)W * H, cudaMemcpyDeviceToHost, st));
        HX_TRY(queue_status(it));
        HX_CUDA(cudaStreamSynchronize(st));
        return report_status(it);
    }
    return HX_OK;
}

extern "C" hx_status hx_integrator_read_accumulation(hx_integrator* it, float* host) {
    HX_CHECK_ARG(it && host, "hx_integrator_read_accumulation: null argument");
    uint32_t n = it->desc.width * it->desc.height;
    cudaStream_t st = it->ctx->stream;
    bool kahan = it->desc.policy.accumulation == HX_ACCUM_KAHAN;
    k_resolve<<<it->grid_gen, kGenThreads, 0, st>>>(it->acc, it->count_map, n, kahan ? 1u : 0u, it->resolved);
    HX_CUDA(cudaGetLastError());
    HX_CUDA(cudaMemcpyAsync(host, it->resolved, 16 * (size_t)n, cudaMemcpyDeviceToHost, st));
    HX_TRY(queue_status(it));
    HX_CUDA(cudaStreamSynchronize(st));
    return report_status(it);
}

// ---------------------------------------------------------------------------
// Bake checkpoint / resume: the progressive state (path_integrator.h:46-53 —
// the accumulation image, num_accumulated_samples, tile_idx) to host memory and
// back.  The next frame's seeds come from `accumulated` (frame0 of
// run_wavefront), so a restored integrator continues the same sample sequence.
// ---------------------------------------------------------------------------
static_assert(sizeof(hx_bake_checkpoint) == 64, "checkpoint header is 64 bytes");

// 64-bit payload hash: four independent lanes (h = rotl(h ^ w * K2, 31) * K1 per
// little-endian 8-byte word, lanes strided by 32 bytes), the tail bytes packed
// into a last word, the lanes and the length folded through the SplitMix64
// finaliser (Steele, Lea, Flood 2014).
static uint64_t checkpoint_hash(const unsigned char* p, size_t n) {
    const uint64_t K1 = 0x9E3779B97F4A7C15ull, K2 = 0xBF58476D1CE4E5B9ull;
    auto rotl = [](uint64_t x, int r) { return (x << r) | (x >> (64 - r)); };
    auto fin = [](uint64_t z) {
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    };
    uint64_t h[4] = {K1, K2, ~K1, ~K2};
    size_t i = 0;
    for (; i + 32 <= n; i += 32)
        for (int l = 0; l < 4; ++l) {
            uint64_t w;
            std::memcpy(&w, p + i + 8 * l, 8);
            h[l] = rotl(h[l] ^ (w * K2), 31) * K1;
        }
    uint64_t tail = 0;
    for (size_t k = 0; i + k < n; ++k) tail |= (uint64_t)p[i + k] << (8 * (k & 7));
    uint64_t r = fin(n ^ tail);
    for (int l = 0; l < 4; ++l) r = fin(r ^ h[l]);
    return r;
}

static size_t checkpoint_payload_bytes(uint32_t w, uint32_t h, bool aov) {
    const size_t npix = (size_t)w * h;
    return npix * (16 + 16 + 4) + (aov ? npix * 32 : 0);
}

extern "C" hx_status hx_integrator_checkpoint_size(const hx_integrator* it, size_t* bytes) {
    HX_CHECK_ARG(it && bytes, "hx_integrator_checkpoint_size: null argument");
    *bytes = sizeof(hx_bake_checkpoint) + checkpoint_payload_bytes(it->desc.width, it->desc.height, it->aov);
    return HX_OK;
}

extern "C" hx_status hx_integrator_save_checkpoint(hx_integrator* it, void* host, size_t bytes) {
    HX_CHECK_ARG(it && host, "hx_integrator_save_checkpoint: null argument");
    const size_t payload = checkpoint_payload_bytes(it->desc.width, it->desc.height, it->aov);
    HX_CHECK_ARG(bytes >= sizeof(hx_bake_checkpoint) + payload,
                 "hx_integrator_save_checkpoint: %zu bytes given, %zu needed", bytes,
                 sizeof(hx_bake_checkpoint) + payload);
    HX_CUDA(cudaSetDevice(it->ctx->device));
    const size_t npix = (size_t)it->desc.width * it->desc.height;
    unsigned char* out = (unsigned char*)host;
    unsigned char* d = out + sizeof(hx_bake_checkpoint);
    cudaStream_t st = it->ctx->stream;
    HX_CUDA(cudaMemcpyAsync(d, it->acc, 16 * npix, cudaMemcpyDeviceToHost, st));
    HX_CUDA(cudaMemcpyAsync(d + 16 * npix, it->comp, 16 * npix, cudaMemcpyDeviceToHost, st));
    HX_CUDA(cudaMemcpyAsync(d + 32 * npix, it->count_map, 4 * npix, cudaMemcpyDeviceToHost, st));
    if (it->aov) {
        HX_CUDA(cudaMemcpyAsync(d + 36 * npix, it->aov_a, 16 * npix, cudaMemcpyDeviceToHost, st));
        HX_CUDA(cudaMemcpyAsync(d + 52 * npix, it->aov_n, 16 * npix, cudaMemcpyDeviceToHost, st));
    }
    HX_TRY(queue_status(it));
    HX_CUDA(cudaStreamSynchronize(st));
    HX_TRY(report_status(it));
    hx_bake_checkpoint hdr{};
    hdr.magic = HX_BAKE_CHECKPOINT_MAGIC;
    hdr.version = HX_BAKE_CHECKPOINT_VERSION;
    hdr.width = it->desc.width;
    hdr.height = it->desc.height;
    hdr.max_samples = it->desc.max_samples;
    hdr.tiled = it->desc.tiled;
    hdr.accumulation = it->desc.policy.accumulation;
    hdr.accumulated = it->accumulated;
    hdr.tile_idx = it->tile_idx;
    hdr.aov = it->aov ? 1u : 0u;
    hdr.aov_frames = it->aov_frames;
    hdr.payload_bytes = payload;
    hdr.checksum = checkpoint_hash(d, payload);
    std::memcpy(out, &hdr, sizeof(hdr));
    return HX_OK;
}

extern "C" hx_status hx_integrator_load_checkpoint(hx_integrator* it, const void* host, size_t bytes) {
    HX_CHECK_ARG(it && host, "hx_integrator_load_checkpoint: null argument");
    HX_CHECK_ARG(bytes >= sizeof(hx_bake_checkpoint), "hx_integrator_load_checkpoint: %zu bytes, shorter than the header",
                 bytes);
    hx_bake_checkpoint hdr;
    std::memcpy(&hdr, host, sizeof(hdr));
    HX_CHECK_ARG(hdr.magic == HX_BAKE_CHECKPOINT_MAGIC && hdr.version == HX_BAKE_CHECKPOINT_VERSION,
                 "hx_integrator_load_checkpoint: not a version-%u bake checkpoint (magic 0x%08x, version %u)",
                 HX_BAKE_CHECKPOINT_VERSION, hdr.magic, hdr.version);
    HX_CHECK_ARG(hdr.width == it->desc.width && hdr.height == it->desc.height,
                 "hx_integrator_load_checkpoint: checkpoint is %ux%u, integrator %ux%u", hdr.width, hdr.height,
                 it->desc.width, it->desc.height);
    HX_CHECK_ARG(hdr.max_samples == it->desc.max_samples && hdr.tiled == it->desc.tiled &&
                     hdr.accumulation == it->desc.policy.accumulation,
                 "hx_integrator_load_checkpoint: max_samples/tiled/accumulation %u/%u/%u differ from the integrator's "
                 "%u/%u/%u", hdr.max_samples, hdr.tiled, hdr.accumulation, it->desc.max_samples, it->desc.tiled,
                 it->desc.policy.accumulation);
    HX_CHECK_ARG(hdr.aov <= 1 && hdr.tile_idx <= it->tiles.size() && hdr.accumulated < hdr.max_samples,
                 "hx_integrator_load_checkpoint: progress fields out of range");
    const size_t payload = checkpoint_payload_bytes(hdr.width, hdr.height, hdr.aov != 0);
    HX_CHECK_ARG(hdr.payload_bytes == payload && bytes >= sizeof(hdr) + payload,
                 "hx_integrator_load_checkpoint: payload %llu bytes recorded, %zu expected, %zu available",
                 (unsigned long long)hdr.payload_bytes, payload, bytes - sizeof(hdr));
    const unsigned char* d = (const unsigned char*)host + sizeof(hdr);
    HX_CHECK_ARG(checkpoint_hash(d, payload) == hdr.checksum, "hx_integrator_load_checkpoint: checksum mismatch");
    HX_CUDA(cudaSetDevice(it->ctx->device));
    HX_TRY(hx_integrator_set_aov_accumulation(it, hdr.aov));
    const size_t npix = (size_t)hdr.width * hdr.height;
    cudaStream_t st = it->ctx->stream;
    HX_CUDA(cudaMemcpyAsync(it->acc, d, 16 * npix, cudaMemcpyHostToDevice, st));
    HX_CUDA(cudaMemcpyAsync(it->comp, d + 16 * npix, 16 * npix, cudaMemcpyHostToDevice, st));
    HX_CUDA(cudaMemcpyAsync(it->count_map, d + 32 * npix, 4 * npix, cudaMemcpyHostToDevice, st));
    if (hdr.aov) {
        HX_CUDA(cudaMemcpyAsync(it->aov_a, d + 36 * npix, 16 * npix, cudaMemcpyHostToDevice, st));
        HX_CUDA(cudaMemcpyAsync(it->aov_n, d + 52 * npix, 16 * npix, cudaMemcpyHostToDevice, st));
    }
    HX_CUDA(cudaStreamSynchronize(st));  // the caller's buffer may go away after the return
    it->accumulated = hdr.accumulated;
    it->tile_idx = hdr.tile_idx;
    it->aov_frames = hdr.aov_frames;
    return HX_OK;
}

// Output-buffer views of Renderer::render_debug_visualization
// (renderer.cpp:491-545; debug_visualization.vert:54-64,
// debug_visualization.frag:71-161), rendered headless by ray casting: per
// pixel one camera ray through the pixel centre (the raster pass samples
// fragments there; pinhole, no jitter), the closest triangle with no alpha
// test (the fragment shader never discards), then the fragment shader's value:
//   albedo     material albedo or the bilinear texel RGB (level 0)
//   normals    the interpolated per-vertex normalize(mat3(normal_matrix) n),
//              not renormalised (no normal maps), * 0.5 + 0.5
//   roughness  material roughness or the selected texture channel (no
//              MIN_ROUGHNESS clamp), metallic likewise, emissive as albedo
// Misses keep the clear colour (0, 0, 0, 1).  Rows are in display order (the
// pass renders with a negative-height viewport, renderer.cpp:498-506): output
// row r is the camera row H - 1 - r of the path tracer's launch grid, the same
// orientation hx_integrator_tonemap returns.  HX_OUTPUT_FINAL is the resolved
// accumulation in that orientation.
__global__ void k_output_view(DevScene s, hx_frame_desc f, uint32_t W, uint32_t H, uint32_t which,
                              const float4* __restrict__ resolved, float4* __restrict__ out, uint32_t* status) {
    const uint32_t n = W * H;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t x = i % W, row = i / W, y = H - 1 - row;
        if (which == HX_OUTPUT_FINAL) {
            out[i] = resolved[(size_t)y * W + x];
            continue;
        }
        const float tx = ((float)x + 0.5f) / (float)W, ty = ((float)y + 0.5f) / (float)H;
        const float nx = tx * 2.0f - 1.0f, ny = ty * 2.0f - 1.0f;
        const float* m = f.view_proj_inverse;
        const float tw = mat4_row(m, 3, nx, ny, 0.0f, 1.0f);
        const V3 target = v3(mat4_row(m, 0, nx, ny, 0.0f, 1.0f) / tw, mat4_row(m, 1, nx, ny, 0.0f, 1.0f) / tw,
                             mat4_row(m, 2, nx, ny, 0.0f, 1.0f) / tw);
        const V3 cam = light_v3(f.camera_pos);
        const V3 d = normalize(target - cam);
        TravState st;
        uint2 stack[kStackSize];
        bool overflow = false;
        trav_init(st, s, cam, d, 0.001f, 10000.0f, false);
        while (!trav_step<false, true>(st, stack, s, overflow, nullptr)) {
        }
        if (overflow) atomicOr(status, 1u);
        float4 c = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
        if (st.best != kNoHit) {
            const uint4 pi = s.prim_info[st.best];
            const DevInstance& inst = s.inst[pi.x];
            const uint32_t i0 = s.indices[3 * pi.y], i1 = s.indices[3 * pi.y + 1], i2 = s.indices[3 * pi.y + 2];
            const float4 p0 = s.vtx[2 * (size_t)i0], n0 = s.vtx[2 * (size_t)i0 + 1];
            const float4 p1 = s.vtx[2 * (size_t)i1], n1 = s.vtx[2 * (size_t)i1 + 1];
            const float4 p2 = s.vtx[2 * (size_t)i2], n2 = s.vtx[2 * (size_t)i2 + 1];
            const float b0 = 1.0f - st.bu - st.bv, b1 = st.bu, b2 = st.bv;
            const float tu = p0.w * b0 + p1.w * b1 + p2.w * b2;
            const float tv = n0.w * b0 + n1.w * b1 + n2.w * b2;
            const hx_material& mt = s.materials[pi.z];
            V3 v = v3(0.0f);
            if (which == HX_OUTPUT_ALBEDO) {
                v = mt.texture_indices0[0] == -1 ? v3(mt.albedo[0], mt.albedo[1], mt.albedo[2])
                                                 : tex_bilinear_rgb(s, (uint32_t)mt.texture_indices0[0], tu, tv);
            } else if (which == HX_OUTPUT_NORMALS) {
                // FS_IN_* = interpolated normalize(mat3(normal_matrix) x) per vertex
                auto lerp_n = [&](V3 x0, V3 x1, V3 x2) {
                    const V3 a = normalize(mat3_mul(inst.normal, x0)), b = normalize(mat3_mul(inst.normal, x1)),
                             e = normalize(mat3_mul(inst.normal, x2));
                    return v3(a.x * b0 + b.x * b1 + e.x * b2, a.y * b0 + b.y * b1 + e.y * b2, a.z * b0 + b.z * b1 + e.z * b2);
                };
                V3 nn = lerp_n(v3(n0.x, n0.y, n0.z), v3(n1.x, n1.y, n1.z), v3(n2.x, n2.y, n2.z));
                if (mt.texture_indices0[1] != -1) {  // debug_visualization.frag:77-90
                    const float4 ta = s.vtx_tb[2 * (size_t)i0], ba = s.vtx_tb[2 * (size_t)i0 + 1];
                    const float4 tb = s.vtx_tb[2 * (size_t)i1], bb = s.vtx_tb[2 * (size_t)i1 + 1];
                    const float4 tc = s.vtx_tb[2 * (size_t)i2], bc = s.vtx_tb[2 * (size_t)i2 + 1];
                    const V3 T = normalize(lerp_n(v3(ta.x, ta.y, ta.z), v3(tb.x, tb.y, tb.z), v3(tc.x, tc.y, tc.z)));
                    const V3 B = normalize(lerp_n(v3(ba.x, ba.y, ba.z), v3(bb.x, bb.y, bb.z), v3(bc.x, bc.y, bc.z)));
                    const V3 N = normalize(nn);
                    const V3 mp = tex_bilinear_rgb(s, (uint32_t)mt.texture_indices0[1], tu, tv);
                    const V3 nm = normalize(mp * 2.0f - v3(1.0f));
                    nn = normalize(v3(T.x * nm.x + B.x * nm.y + N.x * nm.z, T.y * nm.x + B.y * nm.y + N.y * nm.z,
                                      T.z * nm.x + B.z * nm.y + N.z * nm.z));
                }
                v = nn * 0.5f + v3(0.5f);
            } else if (which == HX_OUTPUT_ROUGHNESS) {
                const float r = mt.texture_indices0[2] == -1
                                    ? mt.roughness_metallic[0]
                                    : tex_bilinear(s, (uint32_t)mt.texture_indices0[2], tu, tv, mt.texture_indices1[2]);
                v = v3(r);
            } else if (which == HX_OUTPUT_METALLIC) {
                const float r = mt.texture_indices0[3] == -1
                                    ? mt.roughness_metallic[1]
                                    : tex_bilinear(s, (uint32_t)mt.texture_indices0[3], tu, tv, mt.texture_indices1[3]);
                v = v3(r);
            } else {
                v = mt.texture_indices1[0] == -1 ? v3(mt.emissive[0], mt.emissive[1], mt.emissive[2])
                                                 : tex_bilinear_rgb(s, (uint32_t)mt.texture_indices1[0], tu, tv);
            }
            c = make_float4(v.x, v.y, v.z, 1.0f);
        }
        out[i] = c;
    }
}

extern "C" hx_status hx_integrator_render_output(hx_integrator* it, const hx_frame_desc* frame, uint32_t output_buffer,
                                                 float* host_rgba32f) {
    HX_CHECK_ARG(it && frame && host_rgba32f, "hx_integrator_render_output: null argument");
    HX_CHECK_ARG(output_buffer <= HX_OUTPUT_FINAL, "hx_integrator_render_output: output buffer %u (0..%u)", output_buffer,
                 (unsigned)HX_OUTPUT_FINAL);
    const uint32_t W = it->desc.width, H = it->desc.height, n = W * H;
    cudaStream_t st = it->ctx->stream;
    if (output_buffer == HX_OUTPUT_FINAL) {
        const bool kahan = it->desc.policy.accumulation == HX_ACCUM_KAHAN;
        k_resolve<<<it->grid_gen, kGenThreads, 0, st>>>(it->acc, it->count_map, n, kahan ? 1u : 0u, it->resolved);
        HX_CUDA(cudaGetLastError());
    }
    // the view goes to the flattened-hits staging buffer (sizeof(hx_hit) = 16 B per pixel)
    float4* out = reinterpret_cast<float4*>(it->hits_host_layout);
    k_output_view<<<it->grid_gen, kGenThreads, 0, st>>>(it->scene->d, *frame, W, H, output_buffer, it->resolved, out,
                                                         it->q.status);
    HX_CUDA(cudaGetLastError());
    it->stats.kernel_launches++;
    HX_CUDA(cudaMemcpyAsync(host_rgba32f, out, 16 * (size_t)n, cudaMemcpyDeviceToHost, st));
    return check_status(it);
}

// PathIntegrator::gather_debug_rays (path_integrator.cpp:88-104) with the
// RAY_DEBUG_VIEW shaders (path_trace_rgen.glsl:136-147,183-188,
// path_trace_rchit.glsl:548-567): num_debug_rays paths through the pixel
// (pixel_x, pixel_y) given in display coordinates (the launch row is
// height - pixel_y, path_integrator.cpp:146), seeded with the accumulated
// sample count like a frame; every hit of a ray after the camera ray adds a
// segment (two vertices: position, colour).  Segments appear in shading
// order.  *count receives the number of vertices recorded (capped at
// 2 * num_debug_rays * max_ray_bounces); at most capacity are copied out.
extern "C" hx_status hx_integrator_gather_debug_rays(hx_integrator* it, const hx_frame_desc* frame, uint32_t pixel_x,
                                                     uint32_t pixel_y, uint32_t num_debug_rays,
                                                     hx_debug_ray_vertex* host_vertices, uint32_t capacity, uint32_t* count) {
    HX_CHECK_ARG(it && frame && count && (host_vertices || capacity == 0), "hx_integrator_gather_debug_rays: null argument");
    HX_CHECK_ARG(num_debug_rays >= 1 && num_debug_rays <= it->capacity,
                 "hx_integrator_gather_debug_rays: %u rays (1..%u, the wavefront capacity)", num_debug_rays, it->capacity);
    HX_CHECK_ARG(pixel_x < it->desc.width && pixel_y < it->desc.height,
                 "hx_integrator_gather_debug_rays: pixel (%u, %u) outside %u x %u", pixel_x, pixel_y, it->desc.width,
                 it->desc.height);
    if (it->desc.policy.payload != HX_PAYLOAD_FP32) {
        hx_set_error("hx_integrator_gather_debug_rays: needs FP32 payloads (16-bit hit records carry no distance)");
        return HX_ERR_UNSUPPORTED;
    }
    const uint64_t max_vertices = 2ull * num_debug_rays * std::max<uint32_t>(1, it->desc.max_ray_bounces);
    HX_CHECK_ARG(max_vertices <= 0xffffffffull, "hx_integrator_gather_debug_rays: too many rays");
    cudaStream_t st = it->ctx->stream;
    float4 *color = nullptr, *verts = nullptr;
    uint32_t* cnt = nullptr;
    hx_status rs = hx_alloc_t(it->ctx, &color, num_debug_rays);
    if (rs == HX_OK) rs = hx_alloc_t(it->ctx, &verts, 2 * (size_t)max_vertices);
    if (rs == HX_OK) rs = hx_alloc_t(it->ctx, &cnt, 1);
    if (rs == HX_OK) {
        it->q.dbg_color = color;
        it->q.dbg_verts = verts;
        it->q.dbg_count = cnt;
        it->q.dbg_capacity = (uint32_t)max_vertices;
        cudaError_t e = cudaMemsetAsync(cnt, 0, 4, st);
        if (e != cudaSuccess) {
            hx_set_error("hx_integrator_gather_debug_rays: %s", cudaGetErrorString(e));
            rs = HX_ERR_DEVICE;
        }
        const DebugLaunch dl{pixel_x, it->desc.height - pixel_y, num_debug_rays};
        const Rect r{0, 0, num_debug_rays, 1};
        if (rs == HX_OK) rs = run_wavefront(it, *frame, r, it->accumulated, 1, false, &dl);
        uint32_t n = 0;
        if (rs == HX_OK && cudaMemcpyAsync(&n, cnt, 4, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
            cudaStreamSynchronize(st) == cudaSuccess) {
            n = std::min<uint32_t>(n, (uint32_t)max_vertices);
            *count = n;
            const uint32_t m = std::min(n, capacity);
            if (m && cudaMemcpyAsync(host_vertices, verts, 32 * (size_t)m, cudaMemcpyDeviceToHost, st) != cudaSuccess) {
                hx_set_error("hx_integrator_gather_debug_rays: copy failed");
                rs = HX_ERR_DEVICE;
            }
        } else if (rs == HX_OK) {
            hx_set_error("hx_integrator_gather_debug_rays: %s", cudaGetErrorString(cudaGetLastError()));
            rs = HX_ERR_DEVICE;
        }
        if (rs == HX_OK) rs = check_status(it);
        it->q.dbg_color = nullptr;
        it->q.dbg_verts = nullptr;
        it->q.dbg_count = nullptr;
        it->q.dbg_capacity = 0;
    }
    cudaStreamSynchronize(st);
    if (color) hx_free(it->ctx, color);
    if (verts) hx_free(it->ctx, verts);
    if (cnt) hx_free(it->ctx, cnt);
    return rs;
}

extern "C" hx_status hx_integrator_set_timing(hx_integrator* it, uint32_t enabled) {
    HX_CHECK_ARG(it, "null integrator");
    it->timing = enabled != 0;
    return HX_OK;
}
extern "C" hx_status hx_integrator_set_counting(hx_integrator* it, uint32_t enabled) {
    HX_CHECK_ARG(it, "null integrator");
    it->counting = enabled != 0;
    return HX_OK;
}
extern "C" hx_status hx_integrator_stats(const hx_integrator* it, hx_stats* out) {
    HX_CHECK_ARG(it && out, "null argument");
    *out = it->stats;
    return HX_OK;
}

// Closest hits of the primary rays k_raygen<false> just queued, with the
// kernel a frame's first bounce uses (no shadow rays are queued).
static void launch_primary_trace(hx_integrator* it, cudaStream_t st) {
    const DevScene& s = it->scene->d;
    launch_extend<false, false>(s, it->q, it->grid_batched, it->grid_trace, st, it->q.o[0], it->q.r0[0], it->q.r1[0],
                                it->q.p[0], it->q.counters, it->q.counters + 4);
}

extern "C" hx_status hx_integrator_primary_hits(hx_integrator* it, const hx_frame_desc* f, uint32_t frame_index,
                                                hx_hit* host) {
    HX_CHECK_ARG(it && f && host, "hx_integrator_primary_hits: null argument");
    cudaStream_t st = it->ctx->stream;
    uint32_t W = it->desc.width, H = it->desc.height;
    HX_CHECK_ARG((uint64_t)W * H <= it->capacity, "frame exceeds wavefront capacity");
    Rect r{0, 0, W, H};
    Policy P = make_policy(it->desc.policy);
    k_raygen<false><<<it->grid_gen, kGenThreads, 0, st>>>(*f, r, W, H, frame_index, 1, 0, W * H, P.rng, it->q);
    HX_CUDA(cudaMemsetAsync(it->q.counters + 4, 0, 24, st));
    launch_primary_trace(it, st);
    uint32_t n = W * H;
    k_hits_to_host_layout<<<(n + 255) / 256, 256, 0, st>>>(it->q.hit, W, H, it->hits_host_layout);
    HX_CUDA(cudaGetLastError());
    HX_CUDA(cudaMemcpyAsync(host, it->hits_host_layout, sizeof(hx_hit) * n, cudaMemcpyDeviceToHost, st));
    HX_TRY(check_status(it));
    return HX_OK;
}

extern "C" hx_status hx_integrator_features(hx_integrator* it, const hx_frame_desc* f, uint32_t frame_index,
                                            float* d_features) {
    HX_CHECK_ARG(it && f && d_features, "hx_integrator_features: null argument");
    cudaStream_t st = it->ctx->stream;
    uint32_t W = it->desc.width, H = it->desc.height, n = W * H;
    HX_CHECK_ARG((uint64_t)n <= it->capacity, "frame exceeds wavefront capacity");
    bool kahan = it->desc.policy.accumulation == HX_ACCUM_KAHAN;
    k_resolve<<<it->grid_gen, kGenThreads, 0, st>>>(it->acc, it->count_map, n, kahan ? 1u : 0u, it->resolved);
    // (the progressive counter wraps to 0 when max_samples is reached, the
    // image and AOV buffers keep the finished frame)
    if (it->aov && it->aov_frames > 0) {
        k_features_accumulated<<<it->grid_gen, kGenThreads, 0, st>>>(it->resolved, it->aov_a, it->aov_n, n, it->count_map,
                                                                     1u, d_features);
        HX_CUDA(cudaGetLastError());
        return HX_OK;
    }
    Rect r{0, 0, W, H};
    Policy P = make_policy(it->desc.policy);
    k_raygen<false><<<it->grid_gen, kGenThreads, 0, st>>>(*f, r, W, H, frame_index, 1, 0, W * H, P.rng, it->q);
    HX_CUDA(cudaMemsetAsync(it->q.counters + 4, 0, 24, st));
    launch_primary_trace(it, st);
    k_features<<<it->grid_gen, kGenThreads, 0, st>>>(it->scene->d, it->q.hit, it->resolved, W, H, it->count_map,
                                                      d_features);
    HX_CUDA(cudaGetLastError());
    HX_TRY(check_status(it));
    return HX_OK;
}

extern "C" hx_status hx_integrator_resolve(hx_integrator* it, float* d_rgba) {
    HX_CHECK_ARG(it && d_rgba, "hx_integrator_resolve: null argument");
    uint32_t n = it->desc.width * it->desc.height;
    bool kahan = it->desc.policy.accumulation == HX_ACCUM_KAHAN;
    k_resolve<<<it->grid_gen, kGenThreads, 0, it->ctx->stream>>>(it->acc, it->count_map, n, kahan ? 1u : 0u,
                                                                  reinterpret_cast<float4*>(d_rgba));
    HX_CUDA(cudaGetLastError());
    return HX_OK;
}

extern "C" hx_status hx_integrator_denoise(hx_integrator* it, hx_denoiser* dn, const hx_frame_desc* f, uint32_t op,
                                           float exposure, uint8_t* host_rgba8, float* host_rgba32f) {
    HX_CHECK_ARG(it && dn && f && op <= 2, "hx_integrator_denoise: bad argument");
    cudaStream_t st = it->ctx->stream;
    uint32_t W = it->desc.width, H = it->desc.height, n = W * H;
    if (!it->feat) {
        HX_TRY(hx_alloc_t(it->ctx, &it->feat, 12 * (size_t)it->capacity));
        it->allocs.push_back(it->feat);
        HX_TRY(hx_alloc_t(it->ctx, &it->denoised, (size_t)it->capacity));
        it->allocs.push_back(it->denoised);
    }
    HX_TRY(hx_integrator_features(it, f, 0, it->feat));
    HX_TRY(hx_denoiser_infer(dn, it->feat, 1, H, W, reinterpret_cast<float*>(it->denoised)));
    k_tonemap<<<it->grid_gen, kGenThreads, 0, st>>>(it->denoised, nullptr, W, H, op, exposure, it->ldr);
    HX_CUDA(cudaGetLastError());
    if (host_rgba8) HX_CUDA(cudaMemcpyAsync(host_rgba8, it->ldr, 4 * (size_t)n, cudaMemcpyDeviceToHost, st));
    if (host_rgba32f) HX_CUDA(cudaMemcpyAsync(host_rgba32f, it->denoised, 16 * (size_t)n, cudaMemcpyDeviceToHost, st));
    HX_TRY(hx_denoiser_check(dn));
    return HX_OK;
}

extern "C" hx_status hx_integrator_sample_radiance(hx_integrator* it, const hx_frame_desc* f, uint32_t frame_index,
                                                   float* host_rgb) {
    HX_CHECK_ARG(it && f && host_rgb, "hx_integrator_sample_radiance: null argument");
    uint32_t W = it->desc.width, H = it->desc.height;
    HX_CHECK_ARG((uint64_t)W * H <= it->capacity, "frame exceeds wavefront capacity");
    Rect r{0, 0, W, H};
    HX_TRY(run_wavefront(it, *f, r, frame_index, 1, false));
    uint32_t n = W * H;
    cudaStream_t st = it->ctx->stream;
    k_radiance_out<<<(n + 255) / 256, 256, 0, st>>>(it->q.L, W, H, it->rgb_tmp);
    HX_CUDA(cudaGetLastError());
    HX_CUDA(cudaMemcpyAsync(host_rgb, it->rgb_tmp, 12 * (size_t)n, cudaMemcpyDeviceToHost, st));
    HX_TRY(check_status(it));
    return HX_OK;
}

extern "C" hx_status hx_scene_trace(const hx_scene* scene, const float* host_rays, uint32_t n, uint32_t any_hit,
                                    hx_hit* host_hits) {
    HX_CHECK_ARG(scene && host_rays && host_hits, "hx_scene_trace: null argument");
    if (n == 0) return HX_OK;
    hx_context* ctx = scene->ctx;
    cudaStream_t st = ctx->stream;
    // the rays go through the kernels a frame's bounces use
    const size_t N = n;
    DevBuffer buf;
    HX_TRY(buf.reserve(ctx, 32 * N + 4 * 16 * N + sizeof(hx_hit) * N + 512));
    char* base = buf.as<char>();
    float* d_rays = reinterpret_cast<float*>(base);
    Queues q{};
    q.o[0] = reinterpret_cast<float4*>(base + 32 * N);
    q.r0[0] = q.o[0] + N;
    q.r1[0] = q.r0[0] + N;
    q.hit = q.r1[0] + N;
    hx_hit* d_hits = reinterpret_cast<hx_hit*>(q.hit + N);
    q.counters = reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(d_hits) + sizeof(hx_hit) * N);
    q.stats = reinterpret_cast<unsigned long long*>(q.counters + 16);
    q.status = reinterpret_cast<uint32_t*>(q.stats + 16);
    HX_CUDA(cudaMemcpyAsync(d_rays, host_rays, 32 * N, cudaMemcpyHostToDevice, st));
    HX_CUDA(cudaMemsetAsync(q.counters, 0, 64 + 128 + 4, st));
    k_ray_records<<<ctx->num_sms * 4, 256, 0, st>>>(d_rays, n, any_hit, q.o[0], q.r0[0], q.r1[0], q.counters);
    const DevScene& s = scene->d;
    const int grid = ctx->num_sms * kTraceMinBlocks;
    launch_extend<false, false>(s, q, grid, grid, st, q.o[0], q.r0[0], q.r1[0], nullptr, q.counters, q.counters + 4);
    k_hits_to_host_layout<<<(n + 255) / 256, 256, 0, st>>>(q.hit, n, 1, d_hits);
    HX_CUDA(cudaGetLastError());
    uint32_t status = 0;
    HX_CUDA(cudaMemcpyAsync(host_hits, d_hits, sizeof(hx_hit) * N, cudaMemcpyDeviceToHost, st));
    HX_CUDA(cudaMemcpyAsync(&status, q.status, 4, cudaMemcpyDeviceToHost, st));
    HX_CUDA(cudaStreamSynchronize(st));
    buf.release();
    if (status) {
        hx_set_error("BVH traversal stack overflow");
        return HX_ERR_DEVICE;
    }
    return HX_OK;
}

extern "C" hx_status hx_rng_streams(hx_context* ctx, uint32_t kind, const uint32_t* seeds, uint32_t n, uint32_t draws,
                                    uint32_t* host_out) {
    HX_CHECK_ARG(ctx && seeds && host_out && kind <= 1, "hx_rng_streams: bad argument");
    if (n == 0 || draws == 0) return HX_OK;
    cudaStream_t st = ctx->stream;
    DevBuffer buf;
    HX_TRY(buf.reserve(ctx, 8 * (size_t)n + 4 * (size_t)n * draws));
    uint32_t* d_seeds = buf.as<uint32_t>();
    uint32_t* d_out = d_seeds + 2 * (size_t)n;
    HX_CUDA(cudaMemcpyAsync(d_seeds, seeds, 8 * (size_t)n, cudaMemcpyHostToDevice, st));
    k_rng_streams<<<(n + 255) / 256, 256, 0, st>>>(kind, d_seeds, n, draws, d_out);
    HX_CUDA(cudaGetLastError());
    HX_CUDA(cudaMemcpyAsync(host_out, d_out, 4 * (size_t)n * draws, cudaMemcpyDeviceToHost, st));
    HX_CUDA(cudaStreamSynchronize(st));
    buf.release();
    return HX_OK;
}
