// integrator.cu — the wavefront path integrator (replaces the ray-tracing
// pipeline of src/engine/gfx/path_integrator.cpp and the shaders
// path_trace_*.glsl) and the accumulate / tone-map passes
// (path_trace_rgen.glsl:217-248, tone_map.frag).
//
// One progressive frame = one sample per pixel of the current tile.  Several
// frames can share one wavefront (paths p = frame * npix + pixel); the
// accumulation then replays them in frame order, so the image is identical
// to frame-by-frame rendering.
//
// Per bounce:  k_trace (closest hit)  ->  k_shade (surface, NEE sample,
// BSDF sample, Russian roulette; appends shadow rays and next-bounce rays
// with warp-aggregated atomics)  ->  k_shadow (any-hit visibility, adds the
// NEE contribution).  Queue lengths live in device memory and every kernel
// is a grid-stride loop over them, so a frame is enqueued without host
// round trips.
#include "shade.cuh"

#include <algorithm>
#include <cstring>
#include <vector>

namespace {

constexpr uint32_t kAnyHitFlag = 0x80000000u;
constexpr int kTraceThreads = 128;
constexpr int kShadeThreads = 128;
constexpr int kGenThreads = 256;

struct Queues {
    float4* o[2];       // (origin, tmin)
    float4* d[2];       // (direction, tmax)
    uint32_t* p[2];     // path id | any-hit flag
    float4* hit;        // (t, prim bits, u, v)
    float4* so;         // shadow (origin, tmax)
    float4* sd;         // shadow (direction, any-hit flag bits)
    float4* sc;         // shadow (contribution, path id bits)
    float4* T;          // throughput + depth bits
    float4* L;          // radiance
    uint2* rng;
    uint32_t* counters; // [0],[1] ray queues, [2] shadow queue, [4],[5] trace / shadow fetch cursors
    unsigned long long* stats;  // [0] extension rays, [1] shadow rays
    uint32_t* status;   // bit 0: traversal stack overflow
};

struct Rect {
    uint32_t x0, y0, w, h;
};

// Warp-aggregated queue append: one atomic per warp, slots in lane order.
__device__ __forceinline__ uint32_t warp_append(uint32_t* counter, bool pred) {
    const uint32_t active = __activemask();
    const uint32_t mask = __ballot_sync(active, pred);
    if (mask == 0) return 0;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, __popc(mask));
    base = __shfl_sync(active, base, leader);
    return base + __popc(mask & ((1u << lane) - 1u));
}

__global__ void k_raygen(hx_frame_desc f, Rect rect, uint32_t W, uint32_t H, uint32_t frame0, uint32_t nframes,
                         uint32_t kind, Queues q) {
    uint32_t npix = rect.w * rect.h;
    uint32_t total = npix * nframes;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < total; p += gridDim.x * blockDim.x) {
        uint32_t fr = p / npix, pix = p - fr * npix;
        uint32_t x = rect.x0 + pix % rect.w, y = rect.y0 + pix / rect.w;
        Rng rng = rng_init(kind, x, y, W, frame0 + fr);
        V3 o, d;
        generate_ray(f, kind, x, y, W, H, rng, o, d);
        q.T[p] = make_float4(1.0f, 1.0f, 1.0f, __uint_as_float(0u));
        q.L[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        q.rng[p] = make_uint2(rng.s0, rng.s1);
        q.o[0][p] = make_float4(o.x, o.y, o.z, 0.001f);
        q.d[0][p] = make_float4(d.x, d.y, d.z, 10000.0f);
        q.p[0][p] = p | kAnyHitFlag;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        q.counters[0] = total;
        q.counters[1] = 0;
        q.counters[2] = 0;
    }
}

// Persistent-warp closest-hit kernel: lanes pull rays from the queue with
// warp-aggregated atomics (counter at fetch[0]) and refill as soon as their
// ray finishes.
template <bool COUNT>
__global__ void __launch_bounds__(kTraceThreads) k_trace(DevScene s, const float4* __restrict__ qo,
                                                         const float4* __restrict__ qd, const uint32_t* __restrict__ qp,
                                                         const uint32_t* __restrict__ count, float4* __restrict__ hits,
                                                         unsigned long long* stats, uint32_t* status, uint32_t* fetch) {
    const uint32_t n = *count;
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&stats[0], (unsigned long long)n);
    const uint32_t lane = threadIdx.x & 31u;
    bool overflow = false;
    TraverseCount cnt;
    uint2 stack[kStackSize];
    TravState st;
    uint32_t ray = kNoHit;  // kNoHit: lane needs a ray
    bool done = false;
    for (;;) {
        const uint32_t need = __ballot_sync(0xffffffffu, ray == kNoHit && !done);
        if (need) {
            const uint32_t leader = __ffs(need) - 1u;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(fetch, __popc(need));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (need & (1u << lane)) {
                const uint32_t i = base + __popc(need & ((1u << lane) - 1u));
                if (i < n) {
                    ray = i;
                    const float4 o = qo[i], d = qd[i];
                    trav_init(st, s, v3(o), v3(d), o.w, d.w, (qp[i] & kAnyHitFlag) != 0);
                } else {
                    done = true;
                }
            }
        }
        if (__ballot_sync(0xffffffffu, ray != kNoHit) == 0) break;
        if (ray != kNoHit) {
            if (trav_step<false, COUNT>(st, stack, s, overflow, &cnt)) {
                hits[ray] = st.best != kNoHit ? make_float4(st.best_t, __uint_as_float(st.best), st.bu, st.bv)
                                              : make_float4(0.0f, __uint_as_float(kNoHit), 0.0f, 0.0f);
                ray = kNoHit;
            }
        }
    }
    if (COUNT) {
        atomicAdd(&stats[2], (unsigned long long)cnt.nodes);
        atomicAdd(&stats[3], (unsigned long long)cnt.tris);
    }
    if (overflow) atomicOr(status, 1u);
}

__global__ void __launch_bounds__(kShadeThreads) k_shade(DevScene s, Policy P, uint32_t max_bounces, float bias, int cur,
                                                         Queues q) {
    const uint32_t n = q.counters[cur];
    const int nxt = cur ^ 1;
    const uint32_t num_lights = s.num_lights;
    // grid-stride with warp-uniform trip count so the append ballots see whole warps
    uint32_t stride = gridDim.x * blockDim.x;
    uint32_t start = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t iters = (n + stride - 1) / stride;
    for (uint32_t it = 0; it < iters; ++it) {
        uint32_t i = start + it * stride;
        bool active = i < n;
        bool emit_shadow = false, emit_ray = false;
        float4 so = make_float4(0, 0, 0, 0), sd = make_float4(0, 0, 0, 0), sc = make_float4(0, 0, 0, 0);
        float4 no = make_float4(0, 0, 0, 0), nd = make_float4(0, 0, 0, 0);
        uint32_t path = 0;
        if (active) {
            path = q.p[cur][i] & ~kAnyHitFlag;
            float4 Tw = q.T[path];
            float4 Lw = q.L[path];
            uint2 rs = q.rng[path];
            Rng rng{rs.x, rs.y};
            V3 T = v3(Tw), L = v3(Lw);
            uint32_t depth = __float_as_uint(Tw.w);
            float4 rd = q.d[cur][i];
            V3 d = v3(rd);
            float4 h = q.hit[i];
            uint32_t prim = __float_as_uint(h.y);
            if (prim == kNoHit) {
                V3 e = env_lookup(s.env, d);
                L = L + (depth == 0 ? e : T * e);
                q.L[path] = make_float4(L.x, L.y, L.z, 0.0f);
            } else {
                Surface p = populate(s, prim, h.z, h.w);
                if (depth == 0 && !is_black(p.emissive)) L = L + p.emissive;
                V3 Wo = -d;
                if (num_lights > 0) {
                    uint32_t li = next_uint(P.rng, rng, num_lights);
                    V3 Wi;
                    float pdf, stmax;
                    bool trace_it;
                    V3 Li = sample_light(s, P, p, li, rng, Wi, pdf, stmax, trace_it);
                    if (trace_it && !is_black(Li)) {
                        V3 Wh = normalize(Wo + Wi);
                        V3 brdf = evaluate_uber(p, Wo, Wh, Wi);
                        float cos_theta = gclamp(dot(p.normal, Wi), 0.0f, 1.0f);
                        V3 c = ((T * brdf) * cos_theta) * Li;
                        if (pdf != 0.0f) c = c / pdf;
                        c = c * (float)num_lights;
                        V3 o = p.position + p.normal * bias;
                        so = make_float4(o.x, o.y, o.z, stmax);
                        sd = make_float4(Wi.x, Wi.y, Wi.z, __uint_as_float(depth == 0 ? 1u : 0u));
                        sc = make_float4(c.x, c.y, c.z, __uint_as_float(path));
                        emit_shadow = true;
                    }
                }
                if ((depth + 1) < max_bounces) {
                    V3 Wi;
                    float pdf;
                    V3 brdf = sample_uber(P.rng, p, Wo, rng, Wi, pdf);
                    float cos_theta = gclamp(dot(p.normal, Wi), 0.0f, 1.0f);
                    V3 Tn = (T * (brdf * cos_theta)) / pdf;
                    bool alive = true;
                    if (depth >= P.rr_start) {
                        float prob = gmax(Tn.x, gmax(Tn.y, Tn.z));
                        if (P.rr_clamp) prob = gmin(prob, 1.0f);
                        if (next_float(P.rng, rng) > prob) alive = false;
                        else Tn = Tn * (1.0f / prob);
                    }
                    if (alive) {
                        q.T[path] = make_float4(Tn.x, Tn.y, Tn.z, __uint_as_float(depth + 1));
                        no = make_float4(p.position.x, p.position.y, p.position.z, 0.0001f);
                        nd = make_float4(Wi.x, Wi.y, Wi.z, 10000.0f);
                        emit_ray = true;
                    }
                }
                q.L[path] = make_float4(L.x, L.y, L.z, 0.0f);
                q.rng[path] = make_uint2(rng.s0, rng.s1);
            }
        }
        uint32_t sslot = warp_append(&q.counters[2], emit_shadow);
        if (emit_shadow) {
            q.so[sslot] = so;
            q.sd[sslot] = sd;
            q.sc[sslot] = sc;
        }
        uint32_t rslot = warp_append(&q.counters[nxt], emit_ray);
        if (emit_ray) {
            q.o[nxt][rslot] = no;
            q.d[nxt][rslot] = nd;
            q.p[nxt][rslot] = path;
        }
    }
}

// Persistent-warp any-hit kernel for the shadow queue (fetch counter at
// fetch[1]); an unoccluded entry adds its NEE contribution to its path.
__global__ void __launch_bounds__(kTraceThreads) k_shadow(DevScene s, Queues q, uint32_t* fetch) {
    const uint32_t n = q.counters[2];
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&q.stats[1], (unsigned long long)n);
    const uint32_t lane = threadIdx.x & 31u;
    bool overflow = false;
    uint2 stack[kStackSize];
    TravState st;
    uint32_t ray = kNoHit;
    bool done = false;
    for (;;) {
        const uint32_t need = __ballot_sync(0xffffffffu, ray == kNoHit && !done);
        if (need) {
            const uint32_t leader = __ffs(need) - 1u;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(fetch, __popc(need));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (need & (1u << lane)) {
                const uint32_t i = base + __popc(need & ((1u << lane) - 1u));
                if (i < n) {
                    ray = i;
                    const float4 o = q.so[i], d = q.sd[i];
                    trav_init(st, s, v3(o), v3(d), 0.0001f, o.w, __float_as_uint(d.w) != 0u);
                } else {
                    done = true;
                }
            }
        }
        if (__ballot_sync(0xffffffffu, ray != kNoHit) == 0) break;
        if (ray != kNoHit) {
            if (trav_step<true, false>(st, stack, s, overflow, nullptr)) {
                if (st.best == kNoHit) {
                    const float4 c = q.sc[ray];
                    const uint32_t path = __float_as_uint(c.w);
                    const float4 L = q.L[path];
                    q.L[path] = make_float4(L.x + c.x, L.y + c.y, L.z + c.z, 0.0f);
                }
                ray = kNoHit;
            }
        }
    }
    if (overflow) atomicOr(q.status, 1u);
}

// Accumulation (path_trace_rgen.glsl:217-248): clamp, then running mean
// prev + (c - prev) / num_frames with frame 0 stored raw; or Kahan sum.
__global__ void k_accumulate(Rect rect, uint32_t W, uint32_t frame0, uint32_t nframes, float clampv, uint32_t kahan,
                             const float4* __restrict__ L, float4* __restrict__ acc, float4* __restrict__ comp) {
    uint32_t npix = rect.w * rect.h;
    for (uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x; pix < npix; pix += gridDim.x * blockDim.x) {
        uint32_t x = rect.x0 + pix % rect.w, y = rect.y0 + pix / rect.w;
        size_t idx = (size_t)y * W + x;
        float4 a = acc[idx];
        float4 cp = kahan ? comp[idx] : make_float4(0, 0, 0, 0);
        for (uint32_t f = 0; f < nframes; ++f) {
            float4 l = L[(size_t)f * npix + pix];
            float c[3] = {l.x, l.y, l.z};
            if (clampv > 0.0f)
                for (int k = 0; k < 3; ++k) c[k] = gmin(c[k], clampv);
            uint32_t frame = frame0 + f;
            float* av = &a.x;
            float* cv = &cp.x;
            for (int k = 0; k < 3; ++k) {
                if (kahan) {
                    float yk = c[k] - cv[k];
                    float tk = av[k] + yk;
                    cv[k] = (tk - av[k]) - yk;
                    av[k] = tk;
                } else {
                    av[k] = frame == 0 ? c[k] : av[k] + (c[k] - av[k]) / (float)frame;
                }
            }
            a.w = 1.0f;
        }
        acc[idx] = a;
        if (kahan) comp[idx] = cp;
    }
}

// tone_map.frag:22-51, R8G8B8A8_UNORM, vertical flip.
__global__ void k_tonemap(const float4* __restrict__ acc, const float* __restrict__ inv_count, uint32_t W, uint32_t H,
                          uint32_t op, float exposure, uchar4* __restrict__ out) {
    uint32_t n = W * H;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t x = i % W, y = i / W;
        size_t src = (size_t)(H - 1 - y) * W + x;
        float4 c = acc[src];
        float sc = inv_count ? inv_count[src] : 1.0f;
        float v[3] = {c.x * sc, c.y * sc, c.z * sc};
        unsigned char o[3];
        for (int k = 0; k < 3; ++k) {
            float t = v[k] * exposure;
            if (op == HX_TONEMAP_ACES) {
                const float a = 2.51f, b = 0.03f, cc = 2.43f, d = 0.59f, e = 0.14f;
                t = gclamp((t * (a * t + b)) / (t * (cc * t + d) + e), 0.0f, 1.0f);
            } else if (op == HX_TONEMAP_REINHARD) {
                t = t / (1.0f + t);
            }
            t = powf(t, 1.0f / 2.2f);
            o[k] = (unsigned char)(gclamp(t, 0.0f, 1.0f) * 255.0f + 0.5f);
        }
        out[i] = make_uchar4(o[0], o[1], o[2], 255);
    }
}

// Resolved image: running mean as is; Kahan sum divided by the per-pixel
// sample count.
__global__ void k_resolve(const float4* __restrict__ acc, const uint32_t* __restrict__ count_map, uint32_t n, uint32_t kahan,
                          float4* __restrict__ out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 a = acc[i];
        if (kahan) {
            uint32_t c = count_map[i];
            float s = c ? 1.0f / (float)c : 0.0f;
            a = make_float4(a.x * s, a.y * s, a.z * s, 1.0f);
        }
        out[i] = a;
    }
}

__global__ void k_count_add(Rect rect, uint32_t W, uint32_t add, uint32_t* __restrict__ count_map) {
    uint32_t npix = rect.w * rect.h;
    for (uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x; pix < npix; pix += gridDim.x * blockDim.x) {
        uint32_t x = rect.x0 + pix % rect.w, y = rect.y0 + pix / rect.w;
        count_map[(size_t)y * W + x] += add;
    }
}

__global__ void k_trace_rays(DevScene s, const float* __restrict__ rays, uint32_t n, uint32_t any_hit, hx_hit* out,
                             uint32_t* status) {
    bool overflow = false;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float* r = rays + 8 * (size_t)i;
        HitRec h;
        bool hit = trace_bvh8(s, v3(r[0], r[1], r[2]), v3(r[4], r[5], r[6]), r[3], r[7], any_hit != 0, false, h, overflow);
        out[i].t = hit ? h.t : 0.0f;
        out[i].prim = hit ? h.prim : kNoHit;
        out[i].u = hit ? h.u : 0.0f;
        out[i].v = hit ? h.v : 0.0f;
    }
    if (overflow) atomicOr(status, 1u);
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

__global__ void k_hits_to_host_layout(const float4* __restrict__ hits, uint32_t n, hx_hit* out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 h = hits[i];
    out[i].t = h.x;
    out[i].prim = __float_as_uint(h.y);
    out[i].u = h.z;
    out[i].v = h.w;
}

__global__ void k_radiance_out(const float4* __restrict__ L, uint32_t n, float* out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 l = L[i];
    out[3 * (size_t)i] = l.x;
    out[3 * (size_t)i + 1] = l.y;
    out[3 * (size_t)i + 2] = l.z;
}

Policy make_policy(const hx_policy& p) {
    Policy P;
    P.rng = p.rng;
    P.rr_start = p.rr_start_depth;
    P.rr_clamp = p.rr_clamp;
    P.area_count_x = p.area_count_from_x;
    P.area_w_one = p.area_w_one;
    P.env_importance = p.env_sampling == HX_ENV_SAMPLE_IMPORTANCE;
    P.clampv = p.radiance_clamp;
    return P;
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
    // progressive state (path_integrator.h:46-53)
    uint32_t accumulated = 0, tile_idx = 0;
    std::vector<Rect> tiles;
    // timing / counting
    bool timing = false;
    bool counting = false;
    hx_stats stats{};
    int grid_trace = 0, grid_shadow = 0, grid_shade = 0, grid_gen = 0;
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
    HX_CHECK_ARG(desc->policy.rng <= 1 && desc->policy.accumulation <= 1, "hx_integrator_create: bad policy");
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
        HX_A(it->q.p[k], 4 * cap);
    }
    HX_A(it->q.hit, 16 * cap);
    HX_A(it->q.so, 16 * cap);
    HX_A(it->q.sd, 16 * cap);
    HX_A(it->q.sc, 16 * cap);
    HX_A(it->q.T, 16 * cap);
    HX_A(it->q.L, 16 * cap);
    HX_A(it->q.rng, 8 * cap);
    HX_A(it->q.counters, 64);
    HX_A(it->q.stats, 64);
    HX_A(it->q.status, 64);
    HX_A(it->acc, 16 * npix);
    HX_A(it->comp, 16 * npix);
    HX_A(it->count_map, 4 * npix);
    HX_A(it->resolved, 16 * npix);
    HX_A(it->ldr, 4 * npix);
    HX_A(it->hits_host_layout, sizeof(hx_hit) * npix);
    HX_A(it->rgb_tmp, 12 * npix);
#undef HX_A
    cudaStream_t st = ctx->stream;
    HX_CUDA(cudaMemsetAsync(it->acc, 0, 16 * npix, st));
    HX_CUDA(cudaMemsetAsync(it->comp, 0, 16 * npix, st));
    HX_CUDA(cudaMemsetAsync(it->count_map, 0, 4 * npix, st));
    HX_CUDA(cudaMemsetAsync(it->q.stats, 0, 64, st));
    HX_CUDA(cudaMemsetAsync(it->q.status, 0, 64, st));
    int per_sm = 0;
    HX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace<false>, kTraceThreads, 0));
    it->grid_trace = std::max(1, per_sm) * ctx->num_sms;
    HX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_shadow, kTraceThreads, 0));
    it->grid_shadow = std::max(1, per_sm) * ctx->num_sms;
    HX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_shade, kShadeThreads, 0));
    it->grid_shade = std::max(1, per_sm) * ctx->num_sms;
    it->grid_gen = ctx->num_sms * 8;
    compute_tiles(it);
    *out = it;
    return HX_OK;
}

extern "C" hx_status hx_integrator_destroy(hx_integrator* it) {
    if (!it) return HX_OK;
    if (it->ctx) cudaStreamSynchronize(it->ctx->stream);
    for (void* p : it->allocs) hx_free(it->ctx, p);
    delete it;
    return HX_OK;
}

static hx_status check_status(hx_integrator* it) {
    uint32_t st = 0;
    HX_CUDA(cudaMemcpyAsync(&st, it->q.status, 4, cudaMemcpyDeviceToHost, it->ctx->stream));
    HX_CUDA(cudaStreamSynchronize(it->ctx->stream));
    if (st & 1u) {
        hx_set_error("BVH traversal stack overflow (status word 0x%x)", st);
        cudaMemsetAsync(it->q.status, 0, 4, it->ctx->stream);
        return HX_ERR_DEVICE;
    }
    return HX_OK;
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
static hx_status run_wavefront(hx_integrator* it, const hx_frame_desc& f, Rect rect, uint32_t frame0, uint32_t nframes,
                               bool accumulate) {
    hx_context* ctx = it->ctx;
    cudaStream_t st = ctx->stream;
    const DevScene& s = it->scene->d;
    Policy P = make_policy(it->desc.policy);
    uint32_t npix = rect.w * rect.h;
    uint32_t total = npix * nframes;
    it->stats.paths += total;
    {
        StageTimer t(it, &it->stats.ms_raygen);
        k_raygen<<<it->grid_gen, kGenThreads, 0, st>>>(f, rect, it->desc.width, it->desc.height, frame0, nframes, P.rng, it->q);
        it->stats.kernel_launches++;
    }
    for (uint32_t b = 0; b < it->desc.max_ray_bounces; ++b) {
        int cur = b & 1;
        {
            StageTimer t(it, &it->stats.ms_trace);
            HX_CUDA(cudaMemsetAsync(it->q.counters + 4, 0, 8, st));
            if (it->counting)
                k_trace<true><<<it->grid_trace, kTraceThreads, 0, st>>>(s, it->q.o[cur], it->q.d[cur], it->q.p[cur],
                                                                       it->q.counters + cur, it->q.hit, it->q.stats, it->q.status,
                                                                       it->q.counters + 4);
            else
                k_trace<false><<<it->grid_trace, kTraceThreads, 0, st>>>(s, it->q.o[cur], it->q.d[cur], it->q.p[cur],
                                                                        it->q.counters + cur, it->q.hit, it->q.stats, it->q.status,
                                                                        it->q.counters + 4);
            it->stats.trace_launches++;
            it->stats.kernel_launches++;
        }
        HX_CUDA(cudaMemsetAsync(it->q.counters + (cur ^ 1), 0, 4, st));
        HX_CUDA(cudaMemsetAsync(it->q.counters + 2, 0, 4, st));
        {
            StageTimer t(it, &it->stats.ms_shade);
            k_shade<<<it->grid_shade, kShadeThreads, 0, st>>>(s, P, it->desc.max_ray_bounces, it->desc.shadow_ray_bias, cur, it->q);
            it->stats.kernel_launches++;
        }
        {
            StageTimer t(it, &it->stats.ms_shadow);
            k_shadow<<<it->grid_shadow, kTraceThreads, 0, st>>>(s, it->q, it->q.counters + 5);
            it->stats.kernel_launches++;
        }
    }
    if (accumulate) {
        StageTimer t(it, &it->stats.ms_accumulate);
        bool kahan = it->desc.policy.accumulation == HX_ACCUM_KAHAN;
        k_accumulate<<<it->grid_gen, kGenThreads, 0, st>>>(rect, it->desc.width, frame0, nframes, it->desc.policy.radiance_clamp,
                                                           kahan ? 1u : 0u, it->q.L, it->acc, it->comp);
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
    HX_CUDA(cudaMemsetAsync(it->q.stats, 0, 32, it->ctx->stream));
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
        unsigned long long h[4];
        HX_CUDA(cudaMemcpy(h, it->q.stats, 32, cudaMemcpyDeviceToHost));
        it->stats.extension_rays = h[0];
        it->stats.shadow_rays = h[1];
        it->stats.node_visits = h[2];
        it->stats.tri_tests = h[3];
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
    HX_CHECK_ARG(it && n >= 1 && n <= 64, "hx_integrator_set_max_ray_bounces: bad value");
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
    HX_CHECK_ARG(it && p && p->rng <= 1 && p->accumulation <= 1, "hx_integrator_set_policy: bad policy");
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
        HX_CUDA(cudaStreamSynchronize(st));
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
    HX_CUDA(cudaStreamSynchronize(st));
    return HX_OK;
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

extern "C" hx_status hx_integrator_primary_hits(hx_integrator* it, const hx_frame_desc* f, uint32_t frame_index,
                                                hx_hit* host) {
    HX_CHECK_ARG(it && f && host, "hx_integrator_primary_hits: null argument");
    cudaStream_t st = it->ctx->stream;
    uint32_t W = it->desc.width, H = it->desc.height;
    HX_CHECK_ARG((uint64_t)W * H <= it->capacity, "frame exceeds wavefront capacity");
    Rect r{0, 0, W, H};
    Policy P = make_policy(it->desc.policy);
    k_raygen<<<it->grid_gen, kGenThreads, 0, st>>>(*f, r, W, H, frame_index, 1, P.rng, it->q);
    HX_CUDA(cudaMemsetAsync(it->q.counters + 4, 0, 4, st));
    k_trace<false><<<it->grid_trace, kTraceThreads, 0, st>>>(it->scene->d, it->q.o[0], it->q.d[0], it->q.p[0], it->q.counters,
                                                             it->q.hit, it->q.stats, it->q.status, it->q.counters + 4);
    uint32_t n = W * H;
    k_hits_to_host_layout<<<(n + 255) / 256, 256, 0, st>>>(it->q.hit, n, it->hits_host_layout);
    HX_CUDA(cudaGetLastError());
    HX_CUDA(cudaMemcpyAsync(host, it->hits_host_layout, sizeof(hx_hit) * n, cudaMemcpyDeviceToHost, st));
    HX_TRY(check_status(it));
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
    k_radiance_out<<<(n + 255) / 256, 256, 0, st>>>(it->q.L, n, it->rgb_tmp);
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
    DevBuffer buf;
    HX_TRY(buf.reserve(ctx, 32 * (size_t)n + sizeof(hx_hit) * (size_t)n + 256));
    float* d_rays = buf.as<float>();
    hx_hit* d_hits = (hx_hit*)(buf.as<char>() + 32 * (size_t)n);
    uint32_t* d_status = (uint32_t*)(buf.as<char>() + 32 * (size_t)n + sizeof(hx_hit) * (size_t)n);
    HX_CUDA(cudaMemcpyAsync(d_rays, host_rays, 32 * (size_t)n, cudaMemcpyHostToDevice, st));
    HX_CUDA(cudaMemsetAsync(d_status, 0, 4, st));
    k_trace_rays<<<ctx->num_sms * 8, kTraceThreads, 0, st>>>(scene->d, d_rays, n, any_hit, d_hits, d_status);
    HX_CUDA(cudaGetLastError());
    uint32_t status = 0;
    HX_CUDA(cudaMemcpyAsync(host_hits, d_hits, sizeof(hx_hit) * (size_t)n, cudaMemcpyDeviceToHost, st));
    HX_CUDA(cudaMemcpyAsync(&status, d_status, 4, cudaMemcpyDeviceToHost, st));
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
