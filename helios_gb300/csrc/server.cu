// server.cu — resident render-serving loop (no counterpart in the reference;
// the nearest reference hook is the per-frame Renderer::render,
// src/engine/gfx/renderer.cpp:107, driven once per window frame by the
// application loop, src/engine/core/application.cpp:38-54).
//
// Scenes, BVHs and per-request accumulation images stay on the device.  A
// worker thread admits requests into a pre-allocated HBM arena (first fit,
// so a large request waiting for memory does not block smaller ones), and
// runs ticks: each tick of a scene batches chunks of several requests —
// different resolutions and sample counts — into one wavefront, shortest
// remaining work first, and replays a CUDA graph captured once per scene
// (every launch parameter lives in a device-side request table, so the same
// graph serves any batch).  Different scenes tick on their own streams and
// overlap on the device.  Per-pixel accumulation runs in sample order, so a
// request's image is identical whether it ran alone or in a mix.
#include "wavefront.cuh"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

namespace {

struct Chunk {              // device request-table entry: samples x pixels of one request
    uint32_t slot;          // request slot (index into the slot table)
    uint32_t sample_begin;  // first sample (progressive frame index)
    uint32_t nsamples;
    uint32_t pixel_begin;   // first pixel, row-major
    uint32_t npix;
    uint32_t path_begin;    // first path of the chunk in the wavefront (sample-major)
    uint32_t acc_begin;     // prefix of npix over chunks (accumulation threads)
    uint32_t pad;
};

struct SlotDev {            // per admitted request, device side
    hx_frame_desc frame;
    float4* acc;
    float4* aov_a;          // denoise requests: accumulated first-hit albedo + depth feature (else null)
    float4* aov_n;          // and shading normal
    uint32_t width, height, pad[2];
};

struct TableHeader {
    uint32_t num_chunks, total_paths, total_acc, pad;
};

constexpr uint32_t kMaxChunks = 1024;
constexpr uint32_t kMaxSlots = 4096;

__device__ __forceinline__ uint32_t find_chunk(const Chunk* c, uint32_t n, uint32_t key, bool by_acc) {
    uint32_t lo = 0, hi = n;  // last chunk with begin <= key
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        uint32_t b = by_acc ? c[mid].acc_begin : c[mid].path_begin;
        if (b <= key) lo = mid;
        else hi = mid;
    }
    return lo;
}

__global__ void k_raygen_multi(const TableHeader* hdr, const Chunk* chunks, const SlotDev* slots, uint32_t kind, Queues q) {
    const uint32_t total = hdr->total_paths, nc = hdr->num_chunks;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < total; p += gridDim.x * blockDim.x) {
        const Chunk c = chunks[find_chunk(chunks, nc, p, false)];
        const SlotDev& sd = slots[c.slot];
        uint32_t local = p - c.path_begin;
        uint32_t s = local / c.npix, pix = c.pixel_begin + (local - s * c.npix);
        uint32_t x = pix % sd.width, y = pix / sd.width;
        Rng rng = rng_init(kind, x, y, sd.width, c.sample_begin + s);
        V3 o, d;
        generate_ray(sd.frame, kind, x, y, sd.width, sd.height, rng, o, d);
        q.T[p] = make_float4(1.0f, 1.0f, 1.0f, __uint_as_float(0u));
        q.L[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        q.rng[p] = make_uint2(rng.s0, rng.s1);
        q.o[0][p] = make_float4(o.x, o.y, o.z, 0.001f);
        q.d[0][p] = make_float4(d.x, d.y, d.z, 10000.0f);
        float4 r0, r1;
        ray_record(d, 10000.0f, true, r0, r1);
        q.r0[0][p] = r0;
        q.r1[0][p] = r1;
        q.p[0][p] = p | kAnyHitFlag;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        q.counters[0] = total;
        q.counters[1] = 0;
        q.counters[2] = 0;
    }
}

// Running-mean accumulation (path_trace_rgen.glsl:217-248) per request pixel,
// samples of the chunk in order.
__global__ void k_accumulate_multi(const TableHeader* hdr, const Chunk* chunks, const SlotDev* slots, float clampv,
                                   uint32_t nan_red, const float4* __restrict__ L) {
    const uint32_t total = hdr->total_acc, nc = hdr->num_chunks;
    for (uint32_t a = blockIdx.x * blockDim.x + threadIdx.x; a < total; a += gridDim.x * blockDim.x) {
        const Chunk c = chunks[find_chunk(chunks, nc, a, true)];
        const SlotDev& sd = slots[c.slot];
        uint32_t i = a - c.acc_begin;
        float4* dst = sd.acc + c.pixel_begin + i;
        float4 v = *dst;
        for (uint32_t s = 0; s < c.nsamples; ++s) {
            float4 l = L[(size_t)c.path_begin + (size_t)s * c.npix + i];
            float cc[3] = {l.x, l.y, l.z};
            if (clampv > 0.0f)
                for (int k = 0; k < 3; ++k) cc[k] = gmin(cc[k], clampv);
            uint32_t frame = c.sample_begin + s;
            float* av = &v.x;
            for (int k = 0; k < 3; ++k) av[k] = frame == 0 ? cc[k] : av[k] + (cc[k] - av[k]) / (float)frame;
            if (nan_red && (isnan(l.x) || isnan(l.y) || isnan(l.z))) {
                v.x = 1.0f;
                v.y = 0.0f;
                v.z = 0.0f;
            }
            v.w = 1.0f;
        }
        *dst = v;
    }
}

// First-hit AOVs of denoise requests, accumulated per pixel in sample order
// right after the primary-ray trace (the integrator's k_aov_accumulate over
// the request table).
__global__ void k_aov_accumulate_multi(const TableHeader* hdr, const Chunk* chunks, const SlotDev* slots, DevScene s,
                                       const float4* __restrict__ hit) {
    const uint32_t total = hdr->total_acc, nc = hdr->num_chunks;
    for (uint32_t a = blockIdx.x * blockDim.x + threadIdx.x; a < total; a += gridDim.x * blockDim.x) {
        const Chunk c = chunks[find_chunk(chunks, nc, a, true)];
        const SlotDev& sd = slots[c.slot];
        if (!sd.aov_a) continue;
        const uint32_t i = a - c.acc_begin;
        float4 av = sd.aov_a[c.pixel_begin + i], nv = sd.aov_n[c.pixel_begin + i];
        for (uint32_t smp = 0; smp < c.nsamples; ++smp) {
            const float4 h = hit[(size_t)c.path_begin + (size_t)smp * c.npix + i];
            const uint32_t prim = __float_as_uint(h.y);
            V3 alb = v3(0.0f), nrm = v3(0.0f);
            float depth = 0.0f;
            if (prim != kNoHit) {
                Surface sf = populate(s, prim, h.z, h.w);
                alb = sf.albedo;
                nrm = normalize(sf.normal);
                depth = log1pf(h.x) * 0.125f;
            }
            const float w = 1.0f / (float)(c.sample_begin + smp + 1);
            av = make_float4(av.x + (alb.x - av.x) * w, av.y + (alb.y - av.y) * w, av.z + (alb.z - av.z) * w,
                             av.w + (depth - av.w) * w);
            nv = make_float4(nv.x + (nrm.x - nv.x) * w, nv.y + (nrm.y - nv.y) * w, nv.z + (nrm.z - nv.z) * w, 0.0f);
        }
        sd.aov_a[c.pixel_begin + i] = av;
        sd.aov_n[c.pixel_begin + i] = nv;
    }
}

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
struct ServerRequest {
    uint64_t id = 0;
    hx_request_desc desc{};
    double t_submit = 0, t_admit = 0, t_done = 0;
    int slot = -1;
    size_t arena_off = 0, arena_bytes = 0;
    size_t host_off = 0, host_bytes = 0;
    uint64_t work = 0;  // camera samples of the whole request
    float4* acc = nullptr;
    uchar4* ldr = nullptr;
    float* feat = nullptr;        // denoise: features (12 floats per pixel)
    float4* den = nullptr;        // denoise: denoised radiance
    float4* aov_a = nullptr;      // denoise: accumulated first-hit AOVs
    float4* aov_n = nullptr;
    uint8_t* host_ldr = nullptr;  // pinned
    uint32_t samples_done = 0, pixel_cursor = 0;
    bool in_flight = false, finishing = false, done = false;
    bool cancel = false;  // hx_server_cancel: ends with HX_ERR_CANCELLED once nothing of it is in flight
    hx_status status = HX_OK;
    uint64_t paths_traced = 0;
};

struct PendingChunk {
    ServerRequest* r;
    uint32_t nsamples, npix;
};

struct SceneBatch {
    const hx_scene* scene = nullptr;
    cudaStream_t stream = nullptr;
    Queues q{};
    std::vector<void*> allocs;
    TableHeader* d_hdr = nullptr;
    Chunk* d_chunks = nullptr;
    char* h_table = nullptr;  // pinned: header + chunks
    uint32_t* h_status = nullptr;  // pinned: the tick's device status word (traversal overflow, shading list)
    cudaGraphExec_t graph = nullptr;
    cudaEvent_t done = nullptr;
    bool busy = false;
    std::vector<PendingChunk> running;
    std::vector<ServerRequest*> finishing;
    cudaEvent_t finish_ev = nullptr;
    bool finish_busy = false;
    uint64_t ticks = 0;
    int grid_trace = 0, grid_gen = 0;
    cudaStream_t run = nullptr;  // stream of the tick in flight (and its finishing work)
    bool urgent = false;         // the short-request lane of its scene
};

struct hx_server {
    hx_context* ctx = nullptr;
    hx_server_desc desc{};
    std::vector<SceneBatch*> batches;
    // request slots (device table) and the HBM arena for per-request images
    SlotDev* d_slots = nullptr;
    std::vector<int> free_slots;
    char* arena = nullptr;
    size_t arena_bytes = 0;
    std::map<size_t, size_t> arena_free;  // offset -> size
    char* harena = nullptr;               // pinned host arena for finished images
    size_t harena_bytes = 0;
    std::map<size_t, size_t> harena_free;
    uint64_t admitted_work = 0;           // remaining camera samples of admitted requests
    // queues
    std::mutex mu;
    std::condition_variable cv;
    std::multimap<uint64_t, ServerRequest*> pending;  // by total work: smallest first
    std::vector<ServerRequest*> admitted;
    std::map<uint64_t, ServerRequest*> all;
    std::vector<hx_request_result> completed;
    uint64_t next_id = 1;
    std::thread worker;
    std::atomic<bool> running{false};
    std::atomic<int> worker_error{0};
    char worker_msg[512] = "";
    // stats
    uint64_t paths_total = 0, ticks_total = 0, requests_done = 0, denoised = 0;
    uint64_t active_peak = 0, arena_used_peak = 0;
    double t_start = 0, busy_first = 0, busy_last = 0;
    // learned denoiser for requests with denoise set (runs on the context stream)
    hx_denoiser* denoiser = nullptr;
    cudaEvent_t dn_ready = nullptr, dn_done = nullptr;
    // slot-table uploads of newly admitted requests: ticks wait on this event
    // instead of the worker thread waiting for the uploads
    cudaEvent_t slots_ev = nullptr;
};

static size_t round256(size_t b) { return (b + 255) & ~(size_t)255; }

// Arena bytes of a request: accumulation (16 B/px) + RGBA8 (4 B/px), and
// with denoise its features (48 B/px), denoised image (16 B/px) and
// accumulated AOVs (2 x 16 B/px).
static size_t request_bytes(const hx_request_desc& d) {
    size_t npix = (size_t)d.width * d.height;
    size_t b = round256(16 * npix) + round256(4 * npix);
    if (d.denoise) b += round256(48 * npix) + 3 * round256(16 * npix);
    return b;
}

// First-fit sub-allocation in an arena described by its free map (offset -> size).
static bool arena_alloc(std::map<size_t, size_t>& fm, size_t bytes, size_t* off) {
    for (auto it = fm.begin(); it != fm.end(); ++it) {
        if (it->second >= bytes) {
            *off = it->first;
            size_t rest = it->second - bytes;
            size_t noff = it->first + bytes;
            fm.erase(it);
            if (rest) fm[noff] = rest;
            return true;
        }
    }
    return false;
}

static void arena_release(std::map<size_t, size_t>& fm, size_t off, size_t bytes) {
    auto it = fm.emplace(off, bytes).first;
    auto next = std::next(it);
    if (next != fm.end() && it->first + it->second == next->first) {
        it->second += next->second;
        fm.erase(next);
    }
    if (it != fm.begin()) {
        auto prev = std::prev(it);
        if (prev->first + prev->second == it->first) {
            prev->second += it->second;
            fm.erase(it);
        }
    }
}

static uint64_t remaining_work(const ServerRequest* r) {
    return (uint64_t)(r->desc.spp - r->samples_done) * r->desc.width * r->desc.height - r->pixel_cursor;
}

static hx_status batch_init(hx_server* s, SceneBatch* b) {
    hx_context* ctx = s->ctx;
    const uint32_t cap = s->desc.max_paths_per_tick;
    auto A = [&](void** p, size_t bytes) -> hx_status {
        hx_status st = hx_alloc(ctx, p, bytes);
        if (st == HX_OK) b->allocs.push_back(*p);
        return st;
    };
    for (int k = 0; k < 2; ++k) {
        HX_TRY(A((void**)&b->q.o[k], 16ull * cap));
        HX_TRY(A((void**)&b->q.d[k], 16ull * cap));
        HX_TRY(A((void**)&b->q.r0[k], 16ull * cap));
        HX_TRY(A((void**)&b->q.r1[k], 16ull * cap));
        HX_TRY(A((void**)&b->q.p[k], 4ull * cap));
    }
    HX_TRY(A((void**)&b->q.hit, 16ull * cap));
    HX_TRY(A((void**)&b->q.so, 16ull * cap));
    HX_TRY(A((void**)&b->q.sr0, 16ull * cap));
    HX_TRY(A((void**)&b->q.sr1, 16ull * cap));
    HX_TRY(A((void**)&b->q.sc, 16ull * cap));
    HX_TRY(A((void**)&b->q.T, 16ull * cap));
    HX_TRY(A((void**)&b->q.L, 16ull * cap));
    HX_TRY(A((void**)&b->q.rng, 8ull * cap));
    HX_TRY(A((void**)&b->q.shade_list, 4ull * cap));
    b->q.shade_cap = cap;
    HX_TRY(A((void**)&b->q.part, 4ull * kPartBlocks));
    b->q.list_mode = shade_list_mode(cap, false);

    HX_TRY(A((void**)&b->q.counters, 64));
    HX_TRY(A((void**)&b->q.stats, 64));
    HX_TRY(A((void**)&b->q.status, 64));
    HX_TRY(A((void**)&b->d_hdr, sizeof(TableHeader) + sizeof(Chunk) * kMaxChunks));
    b->d_chunks = (Chunk*)(b->d_hdr + 1);
    HX_CUDA(cudaMallocHost(&b->h_table, sizeof(TableHeader) + sizeof(Chunk) * kMaxChunks));
    HX_CUDA(cudaMallocHost(&b->h_status, sizeof(uint32_t)));
    *b->h_status = 0;
    int lo_prio = 0, hi_prio = 0;
    HX_CUDA(cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio));
    HX_CUDA(cudaStreamCreateWithPriority(&b->stream, cudaStreamNonBlocking, b->urgent ? hi_prio : lo_prio));
    b->run = b->stream;
    HX_CUDA(cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming));
    HX_CUDA(cudaEventCreateWithFlags(&b->finish_ev, cudaEventDisableTiming));
    HX_CUDA(cudaMemsetAsync(b->q.stats, 0, 64, b->stream));
    HX_CUDA(cudaMemsetAsync(b->q.status, 0, 64, b->stream));
    // capture the tick: table upload, ray generation, bounces, accumulation
    const DevScene& sc = b->scene->d;
    Policy P = make_policy(s->desc.policy);
    int per_sm = 0;
    HX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_extend<false, false>, kTraceThreads, 0));
    const int grid_trace = std::max(1, per_sm) * ctx->num_sms;
    HX_CUDA(set_carveouts(k_extend_batched<false, false>, k_extend_batched<false, true>));
    HX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_extend_batched<false>, kTraceThreads, 0));
    const int grid_batched = std::max(1, per_sm) * ctx->num_sms;
    HX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_shade<false>, kShadeThreads, 0));
    const int grid_shade = std::max(1, per_sm) * ctx->num_sms;
    const int grid_gen = ctx->num_sms * 8;
    b->grid_trace = grid_trace;
    b->grid_gen = grid_gen;
    cudaStream_t st = b->stream;
    cudaGraph_t g;
    HX_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    cudaMemcpyAsync(b->d_hdr, b->h_table, sizeof(TableHeader) + sizeof(Chunk) * kMaxChunks, cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(b->q.status, 0, 4, st);
    k_raygen_multi<<<grid_gen, kGenThreads, 0, st>>>(b->d_hdr, b->d_chunks, s->d_slots, P.rng, b->q);
    // bounce bo: extension rays of bo + shadow rays of bo - 1 in one launch;
    // the last launch traces the final bounce's shadow rays
    for (uint32_t bo = 0; bo <= s->desc.max_ray_bounces; ++bo) {
        int cur = bo & 1;
        cudaMemsetAsync(b->q.counters + 4, 0, 24, st);  // fetch cursor, miss / hit counts
        launch_extend<false, false>(sc, b->q, grid_batched, grid_trace, st, b->q.o[cur], b->q.r0[cur], b->q.r1[cur],
                                    b->q.p[cur], b->q.counters + cur, b->q.counters + 4);
        if (bo == s->desc.max_ray_bounces) break;
        if (bo == 0)
            k_aov_accumulate_multi<<<grid_gen, kGenThreads, 0, st>>>(b->d_hdr, b->d_chunks, s->d_slots, sc, b->q.hit);
        cudaMemsetAsync(b->q.counters + (cur ^ 1), 0, 4, st);
        cudaMemsetAsync(b->q.counters + 2, 0, 4, st);
        launch_shade_partition<false>(b->q, cur, st);
        if (P.ray_offset) k_shade<false, false, true><<<grid_shade, kShadeThreads, 0, st>>>(sc, P, s->desc.max_ray_bounces, 0.0f, cur, b->q);
        else k_shade<false><<<grid_shade, kShadeThreads, 0, st>>>(sc, P, s->desc.max_ray_bounces, 0.0f, cur, b->q);
    }
    k_accumulate_multi<<<grid_gen, kGenThreads, 0, st>>>(b->d_hdr, b->d_chunks, s->d_slots, s->desc.policy.radiance_clamp,
                                                         s->desc.policy.visualize_nans ? 1u : 0u, b->q.L);
    cudaMemcpyAsync(b->h_status, b->q.status, 4, cudaMemcpyDeviceToHost, st);
    cudaError_t ce = cudaStreamEndCapture(st, &g);
    if (ce != cudaSuccess) {
        hx_set_error("server: graph capture failed: %s", cudaGetErrorString(ce));
        return HX_ERR_DEVICE;
    }
    HX_CUDA(cudaGraphInstantiate(&b->graph, g, 0));
    cudaGraphDestroy(g);
    return HX_OK;
}

static void batch_free(hx_server* s, SceneBatch* b) {
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    for (void* p : b->allocs) hx_free(s->ctx, p);
    if (b->h_table) cudaFreeHost(b->h_table);
    if (b->h_status) cudaFreeHost(b->h_status);
    if (b->done) cudaEventDestroy(b->done);
    if (b->finish_ev) cudaEventDestroy(b->finish_ev);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

// Admit pending requests, smallest total work first, while the admitted
// remaining work stays under the cap and both arenas (device image, pinned
// host result) have room; a request that does not fit is skipped, not
// blocking smaller ones behind it.
static void admit(hx_server* s) {
    for (auto it = s->pending.begin(); it != s->pending.end();) {
        ServerRequest* r = it->second;
        if (s->free_slots.empty()) break;
        // the admitted-work cap holds back long requests only: a request
        // that fits in one tick is always admitted (memory permitting), so a
        // long request admitted into an idle server cannot block short ones
        if (!s->admitted.empty() && r->work > s->desc.max_paths_per_tick &&
            s->admitted_work + r->work > s->desc.admitted_work_paths)
            break;
        size_t off, hoff;
        if (!arena_alloc(s->arena_free, r->arena_bytes, &off)) {
            ++it;
            continue;
        }
        if (!arena_alloc(s->harena_free, r->host_bytes, &hoff)) {
            arena_release(s->arena_free, off, r->arena_bytes);
            ++it;
            continue;
        }
        r->host_off = hoff;
        r->host_ldr = (uint8_t*)(s->harena + hoff);
        s->admitted_work += r->work;
        r->arena_off = off;
        r->slot = s->free_slots.back();
        s->free_slots.pop_back();
        size_t npix = (size_t)r->desc.width * r->desc.height;
        r->acc = (float4*)(s->arena + off);
        r->ldr = (uchar4*)(s->arena + off + round256(16 * npix));
        if (r->desc.denoise) {
            r->feat = (float*)(s->arena + off + round256(16 * npix) + round256(4 * npix));
            r->den = (float4*)((char*)r->feat + round256(48 * npix));
            r->aov_a = (float4*)((char*)r->den + round256(16 * npix));
            r->aov_n = (float4*)((char*)r->aov_a + round256(16 * npix));
        }
        r->t_admit = now_s();
        s->admitted.push_back(r);
        it = s->pending.erase(it);
        size_t free_b = 0;
        for (auto& kv : s->arena_free) free_b += kv.second;
        s->active_peak = std::max<uint64_t>(s->active_peak, s->admitted.size());
        s->arena_used_peak = std::max<uint64_t>(s->arena_used_peak, s->arena_bytes - free_b);
    }
}

// Result record of a request that ends now (finished or cancelled).
static void push_result(hx_server* s, ServerRequest* r) {
    r->done = true;
    r->t_done = now_s();
    hx_request_result res{};
    res.request_id = r->id;
    res.status = r->status;
    res.queue_ms = ((r->t_admit > 0 ? r->t_admit : r->t_done) - r->t_submit) * 1000.0;
    res.latency_ms = (r->t_done - r->t_submit) * 1000.0;
    res.paths = r->paths_traced;
    res.user_tag = r->desc.user_tag;
    s->completed.push_back(res);
    s->requests_done++;
}

static uint64_t remaining_work(const ServerRequest* r);

// Ends admitted requests marked for cancellation that have nothing in flight:
// their slot, device and host arena space are released at once.
static void retire_cancelled(hx_server* s) {
    for (size_t k = 0; k < s->admitted.size();) {
        ServerRequest* r = s->admitted[k];
        if (!r->cancel || r->in_flight || r->finishing) {
            ++k;
            continue;
        }
        r->status = HX_ERR_CANCELLED;
        s->admitted_work -= std::min<uint64_t>(s->admitted_work, remaining_work(r));
        s->free_slots.push_back(r->slot);
        r->slot = -1;
        arena_release(s->arena_free, r->arena_off, r->arena_bytes);
        arena_release(s->harena_free, r->host_off, r->host_bytes);
        r->host_bytes = 0;
        s->admitted.erase(s->admitted.begin() + k);
        push_result(s, r);
    }
}

static uint64_t remaining_work(const ServerRequest* r);

// Requests that fit in one tick go to their scene's short lane, the others
// to its long lane.
static bool is_short(const hx_server* s, const ServerRequest* r) {
    return remaining_work(r) <= (uint64_t)s->desc.max_paths_per_tick;
}

static hx_status launch_tick(hx_server* s, SceneBatch* b, uint32_t scene_id) {
    // requests of this scene and lane with work left and nothing in flight,
    // shortest remaining work first
    std::vector<ServerRequest*> cand;
    for (ServerRequest* r : s->admitted)
        if (r->desc.scene_id == scene_id && !r->in_flight && !r->finishing && !r->cancel && r->samples_done < r->desc.spp &&
            is_short(s, r) == b->urgent)
            cand.push_back(r);
    if (cand.empty()) return HX_OK;
    auto remaining = [](const ServerRequest* r) {
        return (uint64_t)(r->desc.spp - r->samples_done) * r->desc.width * r->desc.height - r->pixel_cursor;
    };
    std::stable_sort(cand.begin(), cand.end(), [&](ServerRequest* a, ServerRequest* c) { return remaining(a) < remaining(c); });
    TableHeader* hdr = (TableHeader*)b->h_table;
    Chunk* ch = (Chunk*)(hdr + 1);
    uint32_t nc = 0, paths = 0, accs = 0;
    const uint32_t cap = b->urgent ? s->desc.max_paths_per_tick : s->desc.max_paths_per_long_tick;
    b->running.clear();
    // slot table updates for newly admitted requests happen before the tick
    for (ServerRequest* r : cand) {
        if (nc >= kMaxChunks || paths >= cap) break;
        uint32_t npix_img = r->desc.width * r->desc.height;
        uint32_t left = cap - paths;
        Chunk c{};
        c.slot = (uint32_t)r->slot;
        c.sample_begin = r->samples_done;
        if (r->pixel_cursor == 0 && left >= npix_img) {
            c.nsamples = std::min<uint32_t>(r->desc.spp - r->samples_done, left / npix_img);
            c.pixel_begin = 0;
            c.npix = npix_img;
        } else {
            c.nsamples = 1;
            c.pixel_begin = r->pixel_cursor;
            c.npix = std::min<uint32_t>(npix_img - r->pixel_cursor, left);
        }
        c.path_begin = paths;
        c.acc_begin = accs;
        ch[nc++] = c;
        paths += c.nsamples * c.npix;
        accs += c.npix;
        r->in_flight = true;
        b->running.push_back({r, c.nsamples, c.npix});
    }
    hdr->num_chunks = nc;
    hdr->total_paths = paths;
    hdr->total_acc = accs;
    // the short lane's stream has the high priority: its kernels overtake
    // long ticks' kernels at kernel boundaries (a graph takes the priority of
    // its launch stream)
    HX_CUDA(cudaStreamWaitEvent(b->run, s->slots_ev, 0));
    HX_CUDA(cudaGraphLaunch(b->graph, b->run));
    HX_CUDA(cudaEventRecord(b->done, b->run));
    b->busy = true;
    b->ticks++;
    s->ticks_total++;
    s->paths_total += paths;
    return HX_OK;
}

// Denoise a finished request: its features are the accumulated image and
// the first-hit AOVs accumulated over the same samples (batch stream); the
// denoiser runs on the context stream and the batch stream waits for it
// before tone mapping.
static hx_status denoise_request(hx_server* s, SceneBatch* b, ServerRequest* r) {
    const uint32_t W = r->desc.width, H = r->desc.height;
    k_features_accumulated<<<b->grid_gen, kGenThreads, 0, b->run>>>(r->acc, r->aov_a, r->aov_n, W * H, nullptr,
                                                                    r->desc.spp, r->feat);
    HX_CUDA(cudaGetLastError());
    HX_CUDA(cudaEventRecord(s->dn_ready, b->run));
    HX_CUDA(cudaStreamWaitEvent(s->ctx->stream, s->dn_ready, 0));
    HX_TRY(hx_denoiser_infer(s->denoiser, r->feat, 1, H, W, reinterpret_cast<float*>(r->den)));
    HX_CUDA(cudaEventRecord(s->dn_done, s->ctx->stream));
    HX_CUDA(cudaStreamWaitEvent(b->run, s->dn_done, 0));
    s->denoised++;
    return HX_OK;
}

static hx_status retire_tick(hx_server* s, SceneBatch* b) {
    // a device-side problem in the tick (status word copied back by the graph)
    // fails the requests that had work in it
    const uint32_t dev_status = *b->h_status;
    *b->h_status = 0;
    for (const PendingChunk& pc : b->running) {
        ServerRequest* r = pc.r;
        if (dev_status) r->status = HX_ERR_DEVICE;
        r->in_flight = false;
        r->paths_traced += (uint64_t)pc.nsamples * pc.npix;
        s->admitted_work -= std::min<uint64_t>(s->admitted_work, (uint64_t)pc.nsamples * pc.npix);
        uint32_t npix_img = r->desc.width * r->desc.height;
        if (pc.npix == npix_img && r->pixel_cursor == 0) r->samples_done += pc.nsamples;
        else {
            r->pixel_cursor += pc.npix;
            if (r->pixel_cursor >= npix_img) {
                r->pixel_cursor = 0;
                r->samples_done += 1;
            }
        }
        if (r->samples_done >= r->desc.spp) {
            // (denoise, then) tone map to RGBA8 and copy to the request's pinned host buffer
            r->finishing = true;
            if (r->desc.denoise) HX_TRY(denoise_request(s, b, r));
            k_tonemap<<<s->ctx->num_sms * 4, kGenThreads, 0, b->run>>>(r->desc.denoise ? r->den : r->acc, nullptr,
                                                                           r->desc.width, r->desc.height,
                                                                           r->desc.tonemap_op, r->desc.exposure, r->ldr);
            HX_CUDA(cudaMemcpyAsync(r->host_ldr, r->ldr, 4ull * npix_img, cudaMemcpyDeviceToHost, b->run));
            b->finishing.push_back(r);
        }
    }
    b->running.clear();
    if (!b->finishing.empty()) {
        HX_CUDA(cudaEventRecord(b->finish_ev, b->run));
        b->finish_busy = true;
    }
    b->busy = false;
    return HX_OK;
}

static void complete_finished(hx_server* s, SceneBatch* b) {
    for (ServerRequest* r : b->finishing) {
        r->finishing = false;
        push_result(s, r);
        // release the device slot and arena space; the pinned LDR copy stays until fetch
        s->free_slots.push_back(r->slot);
        arena_release(s->arena_free, r->arena_off, r->arena_bytes);
        r->slot = -1;
        s->admitted.erase(std::find(s->admitted.begin(), s->admitted.end(), r));
    }
    b->finishing.clear();
    b->finish_busy = false;
}

static hx_status upload_new_slots(hx_server* s, cudaStream_t st, const std::vector<ServerRequest*>& fresh) {
    for (ServerRequest* r : fresh) {
        SlotDev sd;
        std::memset(&sd, 0, sizeof(sd));
        sd.frame = r->desc.frame;
        sd.acc = r->acc;
        sd.aov_a = r->aov_a;
        sd.aov_n = r->aov_n;
        sd.width = r->desc.width;
        sd.height = r->desc.height;
        HX_CUDA(cudaMemcpyAsync(s->d_slots + r->slot, &sd, sizeof(sd), cudaMemcpyHostToDevice, st));
        HX_CUDA(cudaMemsetAsync(r->acc, 0, 16ull * r->desc.width * r->desc.height, st));
        if (r->aov_a) {
            HX_CUDA(cudaMemsetAsync(r->aov_a, 0, 16ull * r->desc.width * r->desc.height, st));
            HX_CUDA(cudaMemsetAsync(r->aov_n, 0, 16ull * r->desc.width * r->desc.height, st));
        }
    }
    if (!fresh.empty()) HX_CUDA(cudaEventRecord(s->slots_ev, st));
    return HX_OK;
}

static void worker_main(hx_server* s) {
    cudaSetDevice(s->ctx->device);
    cudaStream_t setup;
    int lo_prio = 0, hi_prio = 0;
    cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio);
    cudaStreamCreateWithPriority(&setup, cudaStreamNonBlocking, hi_prio);
    while (s->running.load()) {
        std::vector<ServerRequest*> fresh;
        bool idle = true;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            size_t before = s->admitted.size();
            admit(s);
            fresh.assign(s->admitted.begin() + before, s->admitted.end());
        }
        hx_status st = upload_new_slots(s, setup, fresh);
        if (st == HX_OK) {
            std::unique_lock<std::mutex> lk(s->mu);
            uint32_t ticking = 0, urgent = 0;
            for (uint32_t k = 0; k < s->batches.size() && st == HX_OK; ++k) {
                SceneBatch* b = s->batches[k];
                if (b->finish_busy && cudaEventQuery(b->finish_ev) == cudaSuccess) complete_finished(s, b);
                if (b->busy && cudaEventQuery(b->done) == cudaSuccess) st = retire_tick(s, b);
                if (b->busy) {
                    ++ticking;
                    if (b->urgent) ++urgent;
                }
            }
            retire_cancelled(s);
            // start ticks up to the concurrency limit, the lane of the globally
            // smallest remaining request first (shortest remaining work); up to
            // two short-lane ticks may run beyond the limit, and no new long
            // tick starts while a short one runs (their kernels would interleave)
            while (st == HX_OK) {
                int best = -1;
                uint64_t best_work = ~0ull;
                for (ServerRequest* r : s->admitted) {
                    if (r->in_flight || r->finishing || r->cancel || r->samples_done >= r->desc.spp) continue;
                    const int lane = 2 * (int)r->desc.scene_id + (is_short(s, r) ? 1 : 0);
                    SceneBatch* b = s->batches[lane];
                    if (b->busy || b->finish_busy) continue;
                    uint64_t w = remaining_work(r);
                    if (w < best_work) { best_work = w; best = lane; }
                }
                if (best < 0) break;
                const bool short_req = (best & 1) != 0;
                if (!short_req && urgent > 0) break;
                if (ticking >= s->desc.max_concurrent_ticks && !(short_req && urgent < 2)) break;
                st = launch_tick(s, s->batches[best], (uint32_t)(best / 2));
                ++ticking;
                if (short_req) ++urgent;
            }
            for (SceneBatch* b : s->batches)
                if (b->busy || b->finish_busy) idle = false;
            if (!s->completed.empty()) s->cv.notify_all();
        }
        if (st != HX_OK) {
            std::snprintf(s->worker_msg, sizeof(s->worker_msg), "%s", hx_last_error_string());
            s->worker_error.store((int)st);
            s->cv.notify_all();
            break;
        }
        if (idle) {
            std::unique_lock<std::mutex> lk(s->mu);
            if (s->pending.empty()) s->cv.wait_for(lk, std::chrono::microseconds(500));
        } else {
            std::this_thread::sleep_for(std::chrono::microseconds(50));
        }
    }
    cudaStreamDestroy(setup);
}

extern "C" hx_status hx_server_create(hx_context* ctx, const hx_server_desc* desc, hx_server** out) {
    HX_CHECK_ARG(ctx && desc && out, "hx_server_create: null argument");
    HX_CHECK_ARG(desc->max_paths_per_tick >= 1024 && desc->max_ray_bounces >= 1 && desc->max_ray_bounces <= 64,
                 "hx_server_create: bad parameters");
    HX_CHECK_ARG(desc->request_arena_bytes >= (1u << 20), "hx_server_create: request arena too small");
    HX_CHECK_ARG(desc->policy.rng <= 1 && desc->policy.ray_offset <= 1, "hx_server_create: bad policy");
    HX_CUDA(cudaSetDevice(ctx->device));
    hx_server* s = new hx_server();
    s->ctx = ctx;
    s->desc = *desc;
    if (!s->desc.result_arena_bytes) s->desc.result_arena_bytes = std::max<uint64_t>(1u << 20, desc->request_arena_bytes / 4);
    if (!s->desc.admitted_work_paths) s->desc.admitted_work_paths = 4ull * desc->max_paths_per_tick;
    if (!s->desc.max_concurrent_ticks) s->desc.max_concurrent_ticks = 4;
    if (!s->desc.max_paths_per_long_tick || s->desc.max_paths_per_long_tick > desc->max_paths_per_tick)
        s->desc.max_paths_per_long_tick = desc->max_paths_per_tick;
    s->desc.max_paths_per_long_tick = std::max<uint32_t>(s->desc.max_paths_per_long_tick, 1024);
    hx_status st = hx_alloc(ctx, (void**)&s->arena, desc->request_arena_bytes);
    if (st != HX_OK) {
        delete s;
        return st;
    }
    s->arena_bytes = desc->request_arena_bytes;
    s->arena_free[0] = s->arena_bytes;
    if (cudaMallocHost(&s->harena, s->desc.result_arena_bytes) != cudaSuccess) {
        hx_free(ctx, s->arena);
        delete s;
        hx_set_error("hx_server_create: pinned result arena of %llu bytes", (unsigned long long)s->desc.result_arena_bytes);
        return HX_ERR_OOM_BUDGET;
    }
    s->harena_bytes = s->desc.result_arena_bytes;
    s->harena_free[0] = s->harena_bytes;
    st = hx_alloc(ctx, (void**)&s->d_slots, sizeof(SlotDev) * kMaxSlots);
    if (st != HX_OK) {
        hx_free(ctx, s->arena);
        delete s;
        return st;
    }
    for (int k = (int)kMaxSlots - 1; k >= 0; --k) s->free_slots.push_back(k);
    if (cudaEventCreateWithFlags(&s->dn_ready, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->dn_done, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->slots_ev, cudaEventDisableTiming) != cudaSuccess) {
        hx_free(ctx, s->arena);
        hx_free(ctx, s->d_slots);
        cudaFreeHost(s->harena);
        delete s;
        hx_set_error("hx_server_create: event creation failed");
        return HX_ERR_DEVICE;
    }
    s->t_start = now_s();
    *out = s;
    return HX_OK;
}

extern "C" hx_status hx_server_set_denoiser(hx_server* s, hx_denoiser* dn) {
    HX_CHECK_ARG(s, "hx_server_set_denoiser: null server");
    HX_CHECK_ARG(!s->running.load(), "hx_server_set_denoiser: attach the denoiser before hx_server_start");
    s->denoiser = dn;
    return HX_OK;
}

extern "C" hx_status hx_server_add_scene(hx_server* s, const hx_scene* scene, uint32_t* scene_id) {
    HX_CHECK_ARG(s && scene && scene_id, "hx_server_add_scene: null argument");
    HX_CHECK_ARG(!s->running.load(), "hx_server_add_scene: add scenes before hx_server_start");
    // two lanes per scene: long requests, and requests that fit in one tick
    SceneBatch* lanes[2] = {nullptr, nullptr};
    for (int k = 0; k < 2; ++k) {
        lanes[k] = new SceneBatch();
        lanes[k]->scene = scene;
        lanes[k]->urgent = k == 1;
        hx_status st = batch_init(s, lanes[k]);
        if (st != HX_OK) {
            for (int j = 0; j <= k; ++j) batch_free(s, lanes[j]);
            return st;
        }
    }
    *scene_id = (uint32_t)(s->batches.size() / 2);
    s->batches.push_back(lanes[0]);
    s->batches.push_back(lanes[1]);
    return HX_OK;
}

extern "C" hx_status hx_server_start(hx_server* s) {
    HX_CHECK_ARG(s && !s->running.load(), "hx_server_start: already running");
    s->running.store(true);
    s->worker = std::thread(worker_main, s);
    return HX_OK;
}

extern "C" hx_status hx_server_submit(hx_server* s, const hx_request_desc* d, uint64_t* request_id) {
    HX_CHECK_ARG(s && d && request_id, "hx_server_submit: null argument");
    HX_CHECK_ARG(d->scene_id < s->batches.size() / 2, "hx_server_submit: unknown scene %u", d->scene_id);
    HX_CHECK_ARG(d->width > 0 && d->height > 0 && (uint64_t)d->width * d->height <= 64ull << 20 && d->spp >= 1,
                 "hx_server_submit: bad request size");
    HX_CHECK_ARG(d->tonemap_op <= 2, "hx_server_submit: bad tone-map operator");
    HX_CHECK_ARG(!d->denoise || s->denoiser, "hx_server_submit: denoise requested but no denoiser is attached");
    if (s->worker_error.load()) {
        hx_set_error("server worker failed: %s", s->worker_msg);
        return (hx_status)s->worker_error.load();
    }
    ServerRequest* r = new ServerRequest();
    r->desc = *d;
    r->arena_bytes = request_bytes(*d);
    r->host_bytes = (4ull * d->width * d->height + 255) & ~(size_t)255;
    r->work = (uint64_t)d->width * d->height * d->spp;
    if (r->arena_bytes > s->arena_bytes || r->host_bytes > s->harena_bytes) {
        delete r;
        hx_set_error("hx_server_submit: request needs %zu device / %zu host bytes, the arenas hold %zu / %zu",
                     request_bytes(*d), (size_t)(4ull * d->width * d->height), s->arena_bytes, s->harena_bytes);
        return HX_ERR_OOM_BUDGET;
    }
    r->t_submit = now_s();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        r->id = s->next_id++;
        s->all[r->id] = r;
        s->pending.emplace(r->work, r);
    }
    s->cv.notify_all();
    *request_id = r->id;
    return HX_OK;
}

extern "C" hx_status hx_server_poll(hx_server* s, hx_request_result* out, uint32_t capacity, uint32_t* count,
                                    double wait_seconds) {
    HX_CHECK_ARG(s && count, "hx_server_poll: null argument");
    std::unique_lock<std::mutex> lk(s->mu);
    if (s->completed.empty() && wait_seconds > 0)
        s->cv.wait_for(lk, std::chrono::duration<double>(wait_seconds),
                       [&] { return !s->completed.empty() || s->worker_error.load() != 0; });
    if (s->worker_error.load()) {
        hx_set_error("server worker failed: %s", s->worker_msg);
        return (hx_status)s->worker_error.load();
    }
    uint32_t n = (uint32_t)std::min<size_t>(capacity, s->completed.size());
    if (out) std::copy(s->completed.begin(), s->completed.begin() + n, out);
    s->completed.erase(s->completed.begin(), s->completed.begin() + n);
    *count = n;
    return HX_OK;
}

extern "C" hx_status hx_server_cancel(hx_server* s, uint64_t request_id) {
    HX_CHECK_ARG(s, "hx_server_cancel: null server");
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->all.find(request_id);
        HX_CHECK_ARG(it != s->all.end(), "hx_server_cancel: unknown request %llu", (unsigned long long)request_id);
        ServerRequest* r = it->second;
        if (r->done || r->finishing) return HX_OK;  // its image is complete: nothing to cancel
        if (r->slot < 0) {  // still pending: never admitted, ends now
            for (auto p = s->pending.begin(); p != s->pending.end(); ++p)
                if (p->second == r) {
                    s->pending.erase(p);
                    break;
                }
            r->status = HX_ERR_CANCELLED;
            r->host_bytes = 0;
            push_result(s, r);
        } else {
            r->cancel = true;  // admitted: the worker ends it once nothing of it is in flight
        }
    }
    s->cv.notify_all();
    return HX_OK;
}

extern "C" hx_status hx_server_fetch(hx_server* s, uint64_t request_id, uint8_t* host_rgba8) {
    HX_CHECK_ARG(s, "hx_server_fetch: null server");
    ServerRequest* r = nullptr;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->all.find(request_id);
        HX_CHECK_ARG(it != s->all.end(), "hx_server_fetch: unknown request %llu", (unsigned long long)request_id);
        r = it->second;
        if (!r->done) {
            hx_set_error("hx_server_fetch: request %llu not finished", (unsigned long long)request_id);
            return HX_ERR_NOT_READY;
        }
        s->all.erase(it);
        if (r->status == HX_ERR_CANCELLED) {  // no image; its arenas were released when it ended
            delete r;
            hx_set_error("hx_server_fetch: request %llu was cancelled", (unsigned long long)request_id);
            return HX_ERR_CANCELLED;
        }
    }
    if (host_rgba8) std::memcpy(host_rgba8, r->host_ldr, 4ull * r->desc.width * r->desc.height);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        arena_release(s->harena_free, r->host_off, r->host_bytes);
    }
    s->cv.notify_all();
    delete r;
    return HX_OK;
}

extern "C" hx_status hx_server_stats_get(hx_server* s, hx_server_stats* out) {
    HX_CHECK_ARG(s && out, "hx_server_stats_get: null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    std::memset(out, 0, sizeof(*out));
    out->paths = s->paths_total;
    out->ticks = s->ticks_total;
    out->requests_done = s->requests_done;
    out->requests_pending = s->pending.size();
    out->requests_active = s->admitted.size();
    size_t free_b = 0;
    for (auto& kv : s->arena_free) free_b += kv.second;
    out->arena_bytes = s->arena_bytes;
    out->arena_used = s->arena_bytes - free_b;
    out->seconds = now_s() - s->t_start;
    out->requests_denoised = s->denoised;
    out->requests_active_peak = s->active_peak;
    out->arena_used_peak = s->arena_used_peak;
    return HX_OK;
}

extern "C" hx_status hx_server_destroy(hx_server* s) {
    if (!s) return HX_OK;
    if (s->running.load()) {
        s->running.store(false);
        s->cv.notify_all();
        if (s->worker.joinable()) s->worker.join();
    }
    for (SceneBatch* b : s->batches) batch_free(s, b);
    for (auto& kv : s->all) delete kv.second;
    if (s->harena) cudaFreeHost(s->harena);
    if (s->arena) hx_free(s->ctx, s->arena);
    if (s->d_slots) hx_free(s->ctx, s->d_slots);
    if (s->dn_ready) cudaEventDestroy(s->dn_ready);
    if (s->dn_done) cudaEventDestroy(s->dn_done);
    if (s->slots_ev) cudaEventDestroy(s->slots_ev);
    delete s;
    return HX_OK;
}
