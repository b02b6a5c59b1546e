// wavefront.cuh — the wavefront stages shared by the progressive integrator
// (integrator.cu) and the serving loop (server.cu): path-state queues, ray
// generation, closest-hit / shade / shadow kernels, accumulation and tone
// map.  Kernels live in an anonymous namespace (one copy per translation
// unit).
#pragma once

#include "shade.cuh"

namespace {


constexpr uint32_t kAnyHitFlag = 0x80000000u;
constexpr int kTraceThreads = 128;
// 8 blocks of 128 threads per SM caps the traversal kernels at 64 registers:
// 32 resident warps instead of 28 (measured 4% faster than 72 registers;
// 9 and 10 blocks spill and measured 0.3-2.6% slower).  The shade kernel
// runs 7 blocks per SM (73 registers; shading-list order: 0.973 ms per frame
// vs 1.004 ms at 8 blocks and 0.998 ms at 6).
constexpr int kTraceMinBlocks = 8;
constexpr int kShadeMinBlocks = 7;
// Preferred shared-memory carve-out of the batched traversal, in percent of
// the SM's maximum: 10 % selects the 32 KB configuration (8 blocks of 3 KB +
// the driver's 1 KB each), the rest of the SM's memory is L1.  Without it
// the driver chose 100 KB.
constexpr int kBatchedCarveoutPct = 10;

// Applies the carve-out preferences to this translation unit's traversal
// and shading kernels (each unit has its own instances).
template <typename... F>
static inline cudaError_t set_carveouts(F... kernels) {
    cudaError_t e = cudaSuccess;
    for (const void* k : {reinterpret_cast<const void*>(kernels)...})
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, kBatchedCarveoutPct);
    return e;
}
constexpr int kShadeThreads = 128;
constexpr int kGenThreads = 256;

struct Queues {
    float4* o[2];       // (origin, tmin)
    float4* d[2];       // (direction, tmax)
    float4* r0[2];      // traversal record (ray_record; FP32 payloads only)
    float4* r1[2];
    uint32_t* p[2];     // path id | any-hit flag
    float4* hit;        // (t, prim bits, u, v)
    float4* so;         // shadow (origin, tmin)
    float4* sr0;        // shadow traversal record (ray_record: tmax, any-hit flag)
    float4* sr1;
    float4* sc;         // shadow (contribution, path id bits)
    float4* T;          // throughput + depth bits
    float4* L;          // radiance
    uint2* rng;
    uint32_t* counters; // [0],[1] ray queues, [2] shadow queue, [4] trace fetch cursor, [8] misses, [9] hits
    // Shading order (optional; nullptr: shade in queue order): the bounce's
    // extension-ray queue slots, misses at the front (counters[8] of them),
    // hits at the back (counters[9]), so shading runs misses and hits as two
    // contiguous ranges.  list_mode 1: the traversal appends each ray as it
    // finishes (one atomic per kind per warp step); 2: a partition after the
    // traversal — misses in ascending, hits in descending slot order — whose
    // per-slot shading reads are coalesced and which takes the hits last
    // traced first (their data is still in L2; the next bounce's queue,
    // appended in shading order, then runs the other way).  part: the
    // partition's per-block miss counts (kPartBlocks).
    uint32_t* shade_list = nullptr;
    uint32_t shade_cap = 0;
    uint32_t list_mode = 0;
    uint32_t* part = nullptr;
    unsigned long long* stats;  // [0] extension rays, [1] shadow rays, [2..8] counting mode (k_extend)
    uint32_t* status;   // bit 0: traversal stack overflow
    // ray-debug capture (k_raygen_debug, k_shade<_, true>): per-path segment
    // colour, recorded vertices (position, colour: two float4 each), their count
    float4* dbg_color = nullptr;
    float4* dbg_verts = nullptr;
    uint32_t* dbg_count = nullptr;
    uint32_t dbg_capacity = 0;  // vertices
};

struct Rect {
    uint32_t x0, y0, w, h;
};

// Appends a finished extension ray's queue slot to the shading list (misses
// at the front, hits at the back), aggregated over the lanes that finish in
// the same step: called only by those lanes, one atomic per kind.
__device__ __forceinline__ void shade_list_append(const Queues& q, bool miss, uint32_t slot) {
    const uint32_t active = __activemask();
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t same = __ballot_sync(active, miss) ^ (miss ? 0u : active);
    const uint32_t leader = __ffs(same) - 1u;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(q.counters + (miss ? 8 : 9), __popc(same));
    base = __shfl_sync(active, base, leader);
    const uint32_t k = base + __popc(same & ((1u << lane) - 1u));
    if (k < q.shade_cap) q.shade_list[miss ? k : q.shade_cap - 1u - k] = slot;
}

// Miss / hit partition of one bounce's extension-ray slots into the shading
// list (hit records: FP32 hit.y or FP16 hit.x = triangle id, kNoHit for a
// miss).  A fixed grid of kPartBlocks blocks, block b owning one contiguous
// range of slots: k_part_count counts each range's misses, k_part_write
// places each range's misses and hits after those of the ranges before it.
// n is read on the device (the host does not know it).
constexpr uint32_t kPartBlocks = 1024, kPartThreads = 256;

HXD void part_range(uint32_t n, uint32_t b, uint32_t& lo, uint32_t& hi) {
    const uint32_t per = ((n + kPartBlocks - 1u) / kPartBlocks + 31u) & ~31u;
    lo = min(n, b * per);
    hi = min(n, lo + per);
}

template <bool FP16>
HXD bool slot_is_miss(const float4* __restrict__ hit, uint32_t i) {
    const uint32_t* h = reinterpret_cast<const uint32_t*>(hit);
    return __ldg(FP16 ? h + 2 * (size_t)i : h + 4 * (size_t)i + 1) == kNoHit;
}

// Sum over the block (kPartThreads threads; every thread gets the total).
__device__ __forceinline__ uint32_t part_block_sum(uint32_t v, uint32_t* s_warp) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31u) == 0) s_warp[threadIdx.x >> 5] = v;
    __syncthreads();
    uint32_t t = 0;
#pragma unroll
    for (uint32_t w = 0; w < kPartThreads / 32; ++w) t += s_warp[w];
    return t;
}

template <bool FP16>
__global__ void __launch_bounds__(kPartThreads) k_part_count(const float4* __restrict__ hit, const uint32_t* __restrict__ count,
                                                             uint32_t* __restrict__ block_miss) {
    __shared__ uint32_t s_warp[kPartThreads / 32];
    uint32_t lo, hi;
    part_range(*count, blockIdx.x, lo, hi);
    uint32_t c = 0;
    for (uint32_t i = lo + threadIdx.x; i < hi; i += kPartThreads) c += slot_is_miss<FP16>(hit, i) ? 1u : 0u;
    c = part_block_sum(c, s_warp);
    if (threadIdx.x == 0) block_miss[blockIdx.x] = c;
}

template <bool FP16>
__global__ void __launch_bounds__(kPartThreads) k_part_write(const float4* __restrict__ hit, const uint32_t* __restrict__ count,
                                                             const uint32_t* __restrict__ block_miss, uint32_t* __restrict__ list,
                                                             uint32_t cap, uint32_t* __restrict__ counters) {
    __shared__ uint32_t s_warp[kPartThreads / 32], s_wm[kPartThreads / 32], s_wv[kPartThreads / 32];
    const uint32_t n = *count;
    uint32_t before = 0, total = 0;
    for (uint32_t b = threadIdx.x; b < kPartBlocks; b += kPartThreads) {
        const uint32_t c = block_miss[b];
        total += c;
        if (b < blockIdx.x) before += c;
    }
    before = part_block_sum(before, s_warp);
    total = part_block_sum(total, s_warp);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        counters[8] = total;
        counters[9] = n - total;
    }
    uint32_t lo, hi;
    part_range(n, blockIdx.x, lo, hi);
    uint32_t miss_base = before, hit_base = lo - before;  // hits k at list[cap - 1 - k]
    const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    const uint32_t below = (1u << lane) - 1u;
    for (uint32_t c0 = lo; c0 < hi; c0 += kPartThreads) {
        const uint32_t i = c0 + threadIdx.x;
        const bool valid = i < hi;
        const bool miss = valid && slot_is_miss<FP16>(hit, i);
        const uint32_t mm = __ballot_sync(0xffffffffu, miss), vm = __ballot_sync(0xffffffffu, valid);
        if (lane == 0) {
            s_wm[wid] = __popc(mm);
            s_wv[wid] = __popc(vm);
        }
        __syncthreads();
        uint32_t mb = 0, vb = 0, mt = 0, vt = 0;
#pragma unroll
        for (uint32_t w = 0; w < kPartThreads / 32; ++w) {
            const uint32_t a = s_wm[w], v = s_wv[w];
            if (w < wid) {
                mb += a;
                vb += v;
            }
            mt += a;
            vt += v;
        }
        const uint32_t lm = mb + __popc(mm & below), lv = vb + __popc(vm & below);
        if (miss) list[miss_base + lm] = i;
        else if (valid) list[cap - 1u - (hit_base + (lv - lm))] = i;
        miss_base += mt;
        hit_base += vt - mt;
        __syncthreads();
    }
}

// Shading-list mode of a wavefront of `paths` paths: the partition from 2^19
// paths up (on the benchmark scene at 1 spp: 512 x 512 117.2 vs 118.7
// Mpaths/s with the traversal's appends, 1024 x 1024 224.0 vs 220.0, 1080p
// 292.5 vs 284.6, eight 1080p frames 361.9 vs 346.1), the traversal's appends
// below it; 16-bit payloads shade small wavefronts in queue order (their
// lane-local traversal finishes rays too scattered for the appended list).
static inline uint32_t shade_list_mode(uint64_t paths, bool fp16) {
    return paths >= (1u << 19) ? 2u : (fp16 ? 0u : 1u);
}

// The partition of the extension rays of queue `cur` (after their traversal,
// before their shading) in list mode 2; returns the launches made.
template <bool FP16>
static inline int launch_shade_partition(const Queues& q, int cur, cudaStream_t st) {
    if (!q.shade_list || q.list_mode != 2u) return 0;
    k_part_count<FP16><<<kPartBlocks, kPartThreads, 0, st>>>(q.hit, q.counters + cur, q.part);
    k_part_write<FP16><<<kPartBlocks, kPartThreads, 0, st>>>(q.hit, q.counters + cur, q.part, q.shade_list, q.shade_cap,
                                                              q.counters);
    return 2;
}

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

// ---------------------------------------------------------------------------
// 16-bit payloads (precision form): an extension ray is 16 B — origin FP32
// and the direction as two 16-bit signed-normalised octahedral coordinates
// (FP16 coordinates spend their precision near zero and left 19% of the
// terrain's primary hits on a different triangle; snorm16 spacing is uniform,
// 2/65534).  tmin/tmax follow from the ray kind (primary 0.001 / secondary
// 0.0001, tmax 10000).  A hit record is 8 B — triangle id and FP16
// barycentrics.  Traversal stays FP32.
// ---------------------------------------------------------------------------
HXD uint32_t snorm16(float x) {
    float q = rintf(fminf(fmaxf(x, -1.0f), 1.0f) * 32767.0f);
    return (uint32_t)(int32_t)q & 0xffffu;
}
HXD float unsnorm16(uint32_t b) { return (float)(int32_t)(int16_t)(uint16_t)b / 32767.0f; }
HXD uint32_t oct_encode(V3 d) {
    float l1 = fabsf(d.x) + fabsf(d.y) + fabsf(d.z);
    float u = d.x / l1, v = d.y / l1;
    if (d.z < 0.0f) {
        float nu = (1.0f - fabsf(v)) * (u >= 0.0f ? 1.0f : -1.0f);
        float nv = (1.0f - fabsf(u)) * (v >= 0.0f ? 1.0f : -1.0f);
        u = nu;
        v = nv;
    }
    return snorm16(u) | (snorm16(v) << 16);
}
HXD V3 oct_decode(uint32_t bits) {
    float u = unsnorm16(bits & 0xffffu), v = unsnorm16(bits >> 16);
    float z = 1.0f - fabsf(u) - fabsf(v);
    if (z < 0.0f) {
        float nu = (1.0f - fabsf(v)) * (u >= 0.0f ? 1.0f : -1.0f);
        float nv = (1.0f - fabsf(u)) * (v >= 0.0f ? 1.0f : -1.0f);
        u = nu;
        v = nv;
    }
    return normalize(v3(u, v, z));
}
HXD uint32_t half2_bits(float a, float b) {
    __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&h);
}

// Path p of a wavefront over nframes frames of a rect: the frames interleave
// per pixel (p = pixel * nframes + frame), so the lanes of a warp carry the
// samples of a few neighbouring pixels (near-identical camera rays: coherent
// node fetches in the first bounce).  Results do not depend on the order.
HXD uint32_t path_index(uint32_t pix, uint32_t fr, uint32_t nframes) { return pix * nframes + fr; }

// Pixel order of a rect's paths (`pix`): 8 x 4-pixel tiles first — a warp's
// 32 single-frame paths cover one compact tile instead of a 32 x 1 strip —
// then the right remainder (rows of the tiled height), then the bottom
// remainder rows.  pix_xy and pix_of_xy are inverse bijections on the rect.
constexpr uint32_t kPixTileW = 8, kPixTileH = 4;
HXD void pix_xy(const Rect& r, uint32_t pix, uint32_t& x, uint32_t& y) {
    const uint32_t tw = r.w / kPixTileW, fx = tw * kPixTileW, fy = (r.h / kPixTileH) * kPixTileH;
    const uint32_t nfull = fx * fy;
    if (pix < nfull) {
        const uint32_t t = pix / (kPixTileW * kPixTileH), k = pix % (kPixTileW * kPixTileH);
        x = (t % tw) * kPixTileW + k % kPixTileW;
        y = (t / tw) * kPixTileH + k / kPixTileW;
    } else {
        uint32_t q = pix - nfull;
        const uint32_t rw = r.w - fx, rs = rw * fy;
        if (q < rs) {
            x = fx + q % rw;
            y = q / rw;
        } else {
            q -= rs;
            x = q % r.w;
            y = fy + q / r.w;
        }
    }
    x += r.x0;
    y += r.y0;
}
HXD uint32_t pix_of_xy(const Rect& r, uint32_t x, uint32_t y) {
    x -= r.x0;
    y -= r.y0;
    const uint32_t tw = r.w / kPixTileW, fx = tw * kPixTileW, fy = (r.h / kPixTileH) * kPixTileH;
    if (x < fx && y < fy)
        return ((y / kPixTileH) * tw + x / kPixTileW) * (kPixTileW * kPixTileH) + (y % kPixTileH) * kPixTileW +
               x % kPixTileW;
    const uint32_t nfull = fx * fy, rw = r.w - fx;
    if (y < fy) return nfull + y * rw + (x - fx);
    return nfull + rw * fy + (y - fy) * r.w + x;
}

// Camera rays of paths [path_base, path_base + path_count) of the rect's
// nframes frames (path_index); path p goes to ray-queue slot p - path_base,
// its state (T, L, rng) stays indexed by p.
template <bool FP16>
__global__ void k_raygen(hx_frame_desc f, Rect rect, uint32_t W, uint32_t H, uint32_t frame0, uint32_t nframes,
                         uint32_t path_base, uint32_t path_count, uint32_t kind, Queues q) {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < path_count; k += gridDim.x * blockDim.x) {
        const uint32_t p = path_base + k;
        const uint32_t pix = p / nframes, fr = p - pix * nframes;
        uint32_t x, y;
        pix_xy(rect, pix, x, y);
        Rng rng = rng_init(kind, x, y, W, frame0 + fr);
        V3 o, d;
        generate_ray(f, kind, x, y, W, H, rng, o, d);
        q.T[p] = make_float4(1.0f, 1.0f, 1.0f, __uint_as_float(0u));
        q.L[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        q.rng[p] = make_uint2(rng.s0, rng.s1);
        if (FP16) {
            q.o[0][k] = make_float4(o.x, o.y, o.z, __uint_as_float(oct_encode(d)));
        } else {
            q.o[0][k] = make_float4(o.x, o.y, o.z, 0.001f);
            q.d[0][k] = make_float4(d.x, d.y, d.z, 10000.0f);
            float4 r0, r1;
            ray_record(d, 10000.0f, true, r0, r1);
            q.r0[0][k] = r0;
            q.r1[0][k] = r1;
        }
        q.p[0][k] = p | kAnyHitFlag;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        q.counters[0] = path_count;
        q.counters[1] = 0;
        q.counters[2] = 0;
    }
}

// Camera rays of the ray-debug view (RAY_DEBUG_VIEW, path_trace_rgen.glsl:
// 136-147, 183-188; PathIntegrator::gather_debug_rays, path_integrator.cpp:
// 88-104): n paths all through pixel (px, py) of the W x H frame, path k
// seeded as launch (k, 0) of an n x 1 launch; three draws give the path's
// segment colour (each * 0.5 + 0.5) before the camera ray's own draws.  FP32
// payloads.
__global__ void k_raygen_debug(hx_frame_desc f, uint32_t px, uint32_t py, uint32_t W, uint32_t H, uint32_t n,
                               uint32_t frame, uint32_t kind, Queues q) {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        Rng rng = rng_init(kind, k, 0, n, frame);
        const float cr = next_float(kind, rng) * 0.5f + 0.5f;
        const float cg = next_float(kind, rng) * 0.5f + 0.5f;
        const float cb = next_float(kind, rng) * 0.5f + 0.5f;
        V3 o, d;
        generate_ray(f, kind, px, py, W, H, rng, o, d);
        q.T[k] = make_float4(1.0f, 1.0f, 1.0f, __uint_as_float(0u));
        q.L[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        q.rng[k] = make_uint2(rng.s0, rng.s1);
        q.o[0][k] = make_float4(o.x, o.y, o.z, 0.001f);
        q.d[0][k] = make_float4(d.x, d.y, d.z, 10000.0f);
        float4 r0, r1;
        ray_record(d, 10000.0f, true, r0, r1);
        q.r0[0][k] = r0;
        q.r1[0][k] = r1;
        q.p[0][k] = k | kAnyHitFlag;
        q.dbg_color[k] = make_float4(cr, cg, cb, 1.0f);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        q.counters[0] = n;
        q.counters[1] = 0;
        q.counters[2] = 0;
    }
}

// DEBUG: also records each hit of a ray after the camera ray as a segment
// (ray origin, hit point; the path's colour) in q.dbg_verts
// (path_trace_rchit.glsl:548-567); the order of segments is the order their
// hits are shaded.  OFFSET: the policy's HX_RAY_OFFSET_SCALED origins (an
// instantiation of its own, so the reference-origin kernel carries no code
// for them).
template <bool FP16, bool DEBUG = false, bool OFFSET = false>
__global__ void __launch_bounds__(kShadeThreads, kShadeMinBlocks) k_shade(DevScene s, Policy P, uint32_t max_bounces, float bias, int cur,
                                                         Queues q) {
    // with a shading list: misses [0, n_miss) then hits, else queue order
    const bool listed = q.shade_list != nullptr;
    const uint32_t n_miss = listed ? q.counters[8] : 0u;
    const uint32_t n = listed ? min(n_miss + q.counters[9], q.counters[cur]) : q.counters[cur];
    // every extension ray is listed exactly once as a miss or a hit; bit 1 of
    // the status word reports a disagreement (rays would go unshaded)
    if (listed && blockIdx.x == 0 && threadIdx.x == 0 && n_miss + q.counters[9] != q.counters[cur])
        atomicOr(q.status, 2u);
    const int nxt = cur ^ 1;
    const uint32_t num_lights = s.num_lights;
    // grid-stride with warp-uniform trip count so the append ballots see whole warps
    uint32_t stride = gridDim.x * blockDim.x;
    uint32_t start = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t iters = (n + stride - 1) / stride;
    for (uint32_t it = 0; it < iters; ++it) {
        uint32_t i = start + it * stride;
        bool active = i < n;
        if (active && listed) i = i < n_miss ? q.shade_list[i] : q.shade_list[q.shade_cap - 1u - (i - n_miss)];
        bool emit_shadow = false, emit_ray = false;
        float4 so = make_float4(0, 0, 0, 0), sr0 = make_float4(0, 0, 0, 0), sr1 = make_float4(0, 0, 0, 0),
               sc = make_float4(0, 0, 0, 0);
        float4 no = make_float4(0, 0, 0, 0), nd = make_float4(0, 0, 0, 0), nr0 = make_float4(0, 0, 0, 0),
               nr1 = make_float4(0, 0, 0, 0);
        uint32_t path = 0;
        if (active) {
            path = q.p[cur][i] & ~kAnyHitFlag;
            float4 Tw = q.T[path];
            float4 Lw = q.L[path];
            uint2 rs = q.rng[path];
            Rng rng{rs.x, rs.y};
            V3 T = v3(Tw), L = v3(Lw);
            uint32_t depth = __float_as_uint(Tw.w);
            V3 d;
            float4 h;
            uint32_t prim;
            if (FP16) {
                d = oct_decode(__float_as_uint(q.o[cur][i].w));
                const uint2 hh = reinterpret_cast<const uint2*>(q.hit)[i];
                prim = hh.x;
                __half2 uv = *reinterpret_cast<const __half2*>(&hh.y);
                h = make_float4(0.0f, 0.0f, __low2float(uv), __high2float(uv));
            } else {
                d = v3(q.d[cur][i]);
                h = q.hit[i];
                prim = __float_as_uint(h.y);
            }
            if (prim == kNoHit) {
                V3 e = env_lookup(s.env, d);
                L = L + (depth == 0 ? e : T * e);
                q.L[path] = make_float4(L.x, L.y, L.z, 0.0f);
            } else {
                if (DEBUG && depth > 0) {
                    const float4 o4 = q.o[cur][i];
                    const float t = h.x;
                    const float4 c = q.dbg_color[path];
                    const uint32_t v = atomicAdd(q.dbg_count, 2u);
                    if (v + 2u <= q.dbg_capacity) {
                        q.dbg_verts[2 * (size_t)v] = make_float4(o4.x, o4.y, o4.z, 1.0f);
                        q.dbg_verts[2 * (size_t)v + 1] = c;
                        q.dbg_verts[2 * (size_t)v + 2] = make_float4(o4.x + d.x * t, o4.y + d.y * t, o4.z + d.z * t, 1.0f);
                        q.dbg_verts[2 * (size_t)v + 3] = c;
                    }
                }
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
                        if (OFFSET) {
                            // the shadow ray starts closer to the light by at
                            // most the offset's length: shorten it by that
                            const V3 oo = offset_origin(o, geo_normal(s, prim), Wi);
                            stmax = stmax - (fabsf(oo.x - o.x) + fabsf(oo.y - o.y) + fabsf(oo.z - o.z));
                            o = oo;
                        }
                        so = make_float4(o.x, o.y, o.z, 0.0001f);
                        ray_record(Wi, stmax, depth == 0, sr0, sr1);
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
                        const V3 o = OFFSET ? offset_origin(p.position, geo_normal(s, prim), Wi) : p.position;
                        if (FP16) {
                            no = make_float4(o.x, o.y, o.z, __uint_as_float(oct_encode(Wi)));
                        } else {
                            no = make_float4(o.x, o.y, o.z, 0.0001f);
                            nd = make_float4(Wi.x, Wi.y, Wi.z, 10000.0f);
                            ray_record(Wi, 10000.0f, false, nr0, nr1);
                        }
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
            q.sr0[sslot] = sr0;
            q.sr1[sslot] = sr1;
            q.sc[sslot] = sc;
        }
        uint32_t rslot = warp_append(&q.counters[nxt], emit_ray);
        if (emit_ray) {
            q.o[nxt][rslot] = no;
            if (!FP16) {
                q.d[nxt][rslot] = nd;
                q.r0[nxt][rslot] = nr0;
                q.r1[nxt][rslot] = nr1;
            }
            q.p[nxt][rslot] = path;
        }
    }
}

// Persistent-warp traversal of one bounce's extension rays (origins qo,
// traversal records qr0/qr1 — FP16 payloads: qp and the encoded direction —,
// count, closest hit) followed by the previous bounce's shadow rays (any hit; an
// unoccluded entry adds its NEE contribution to its path) in one launch:
// lanes pull from the concatenated index space [extension | shadow], so the
// shadow rays fill the lanes that the extension rays' tail leaves idle and a
// bounce costs one traversal launch instead of two.  The radiance is the same
// as with separate launches: the shadow contribution of bounce b still lands
// in L after shade(b) and before shade(b + 1).  Fetch counter at fetch[0];
// stats [0] extension rays, [1] shadow rays, and in counting mode [2] node
// visits, [3] triangle tests, [4] warp node steps, [5] warp triangle steps,
// [6] warp loop iterations, [7] lane loop iterations with a ray, [8] alpha
// tests.
template <bool COUNT, bool FP16, bool WA = false>
__global__ void __launch_bounds__(kTraceThreads, kTraceMinBlocks) k_extend(DevScene s, Queues q, const float4* __restrict__ qo,
                                                                           const float4* __restrict__ qr0,
                                                                           const float4* __restrict__ qr1,
                                                                           const uint32_t* __restrict__ qp,
                                                                           const uint32_t* __restrict__ count,
                                                                           uint32_t* fetch) {
    const uint32_t n_ext = *count;
    const uint32_t n = n_ext + q.counters[2];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        atomicAdd(&q.stats[0], (unsigned long long)n_ext);
        atomicAdd(&q.stats[1], (unsigned long long)(n - n_ext));
    }
    const uint32_t lane = threadIdx.x & 31u;
    bool overflow = false;
    TraverseCount cnt;
    uint32_t loop_iters = 0, loop_busy = 0;
    uint2 stack[kStackSize];
    TravState st;
    uint32_t ray = kNoHit;  // kNoHit: lane needs a ray; else the queue index (shadow: minus n_ext)
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
                if (i < n_ext) {
                    ray = i;
                    const float4 o = qo[i];
                    if (FP16) {
                        const bool any = (qp[i] & kAnyHitFlag) != 0;
                        trav_init(st, s, v3(o), oct_decode(__float_as_uint(o.w)), any ? 0.001f : 0.0001f, 10000.0f, any);
                    } else {
                        trav_init_record(st, s, o, qr0[i], qr1[i]);
                    }
                } else if (i < n) {
                    ray = i - n_ext;
                    trav_init_record(st, s, q.so[ray], q.sr0[ray], q.sr1[ray]);
                    st.shadow = true;
                } else {
                    done = true;
                }
            }
        }
        const uint32_t busy = __ballot_sync(0xffffffffu, ray != kNoHit);
        if (busy == 0) break;
        if (COUNT) {
            if (lane == 0) loop_iters++;
            if (ray != kNoHit) loop_busy++;
        }
        if (ray != kNoHit) {
            if (trav_step<COUNT, WA>(st, stack, s, overflow, &cnt)) {
                if (st.shadow) {
                    if (st.best == kNoHit) {
                        const float4 c = q.sc[ray];
                        const uint32_t path = __float_as_uint(c.w);
                        const float4 L = q.L[path];
                        q.L[path] = make_float4(L.x + c.x, L.y + c.y, L.z + c.z, 0.0f);
                    }
                } else {
                    if (FP16) {
                        reinterpret_cast<uint2*>(q.hit)[ray] =
                            make_uint2(st.best, st.best != kNoHit ? half2_bits(st.bu, st.bv) : 0u);
                    } else {
                        q.hit[ray] = st.best != kNoHit ? make_float4(st.best_t, __uint_as_float(st.best), st.bu, st.bv)
                                                       : make_float4(0.0f, __uint_as_float(kNoHit), 0.0f, 0.0f);
                    }
                    if (q.list_mode == 1u) shade_list_append(q, st.best == kNoHit, ray);
                }
                ray = kNoHit;
            }
        }
    }
    if (COUNT) {
        atomicAdd(&q.stats[2], (unsigned long long)cnt.nodes);
        atomicAdd(&q.stats[3], (unsigned long long)cnt.tris);
        atomicAdd(&q.stats[4], (unsigned long long)cnt.warp_nodes);
        atomicAdd(&q.stats[5], (unsigned long long)cnt.warp_tris);
        atomicAdd(&q.stats[6], (unsigned long long)loop_iters);
        atomicAdd(&q.stats[7], (unsigned long long)loop_busy);
        atomicAdd(&q.stats[8], (unsigned long long)cnt.alpha);
    }
    if (overflow) atomicOr(q.status, 1u);
}

// Batched triangle tests run every bounce (with three node visits per
// iteration they also beat the lane-local k_extend on the small late
// launches: +0.7%), for both payload forms (16-bit payloads on the 34.5 M-
// triangle terrain: 845 Mpaths/s batched, 674 lane-local; FP32 885); k_extend
// serves scenes of 2^27 triangles or more.
// Flush after 24 queued triangles or 4 waiting lanes (measured on the
// 1.18 M-triangle scene at 1080p: 16-24 queued and 2-4 waiting lanes within
// 0.2 % of each other, 12 queued -0.8 %, 32 queued -1.5 %).
constexpr uint32_t kFlushTris = 24, kFlushParked = 4;
// Node visits per loop iteration for a lane whose nodes expose no triangle:
// spreads the warp's per-iteration queue bookkeeping over more visits
// (measured 1: 263.7, 2: 265.7, 3: 269.2, 4: 268.0, 6: 263.1 Mpaths/s; with
// the 32 KB shared-memory configuration 2: 269.7, 3: 279.2, 4: 277.0).
constexpr uint32_t kNodeSteps = 3;

// k_extend with batched triangle tests (trace.cuh, WarpTris), FP32 payloads:
// lanes visit nodes; the triangles their nodes expose queue up per warp and
// are tested by the whole warp together once flush_tris are queued, or
// flush_parked lanes whose rays have no node left wait on their triangles,
// or no lane has a node left.  A lane whose triangles do not fit the queue
// keeps them and visits no node until they do.  A ray is finished when it
// has no node left and no pending triangle (or, for a shadow ray, as soon as
// a flush accepted a hit).  Same queues, results and counters as k_extend.
// FP16: 16-bit payloads (qo = origin + octahedral direction, qp = path |
// any-hit flag, 8-byte hit records): a lane builds its ray's traversal record
// at refill, and the triangle testers take it from the owner's registers
// (warp_test_tris_shfl).
template <bool COUNT, bool WA = false, bool FP16 = false>
__global__ void __launch_bounds__(kTraceThreads, kTraceMinBlocks)
    k_extend_batched(DevScene s, Queues q, const float4* __restrict__ qo, const float4* __restrict__ qr0,
                     const float4* __restrict__ qr1, const uint32_t* __restrict__ count, uint32_t* fetch,
                     uint32_t flush_tris, uint32_t flush_parked, const uint32_t* __restrict__ qp) {
    __shared__ WarpTris warp_tris[kTraceThreads / 32];
    WarpTris& w = warp_tris[threadIdx.x >> 5];
    const uint32_t n_ext = *count;
    const uint32_t n = n_ext + q.counters[2];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        atomicAdd(&q.stats[0], (unsigned long long)n_ext);
        atomicAdd(&q.stats[1], (unsigned long long)(n - n_ext));
    }
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t lt_mask = (1u << lane) - 1u;
    bool overflow = false;
    TraverseCount cnt;
    uint32_t loop_iters = 0, loop_busy = 0;
    uint2 stack[kStackSize];
    TravState st;
    uint32_t ray = kNoHit;  // kNoHit: lane needs a ray; else the queue index (shadow: minus n_ext)
    bool done = false;
    bool queued = false;    // this lane's ray has triangles in the queue
    uint32_t tmask = 0, tbase = 0;  // exposed triangles not yet queued
    uint32_t qn = 0;        // queued triangles (warp-uniform)
    for (;;) {
        const uint32_t need = __ballot_sync(0xffffffffu, ray == kNoHit && !done);
        if (need) {
            const uint32_t leader = __ffs(need) - 1u;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(fetch, __popc(need));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (need & (1u << lane)) {
                const uint32_t i = base + __popc(need & lt_mask);
                float tmax = 0.0f;
                if (i < n_ext) {
                    ray = i;
                    if (FP16) {
                        // the record of trav_init(o, decoded d, tmin by ray kind, 10000, any)
                        const float4 o = qo[i];
                        const bool any = (qp[i] & kAnyHitFlag) != 0;
                        float4 r0, r1;
                        ray_record(oct_decode(__float_as_uint(o.w)), 10000.0f, any, r0, r1);
                        trav_init_record(st, s, make_float4(o.x, o.y, o.z, any ? 0.001f : 0.0001f), r0, r1);
                        tmax = r0.w;
                    } else {
                        const float4 r0 = qr0[i];
                        trav_init_record(st, s, qo[i], r0, qr1[i]);
                        tmax = r0.w;
                    }
                    w.rid[lane] = i;
                } else if (i < n) {
                    ray = i - n_ext;
                    const float4 r0 = q.sr0[ray];
                    trav_init_record(st, s, q.so[ray], r0, q.sr1[ray]);
                    st.shadow = true;
                    tmax = r0.w;
                    w.rid[lane] = ray | kShadowRid;
                } else {
                    done = true;
                }
                if (ray != kNoHit) w.key[lane] = ((unsigned long long)__float_as_uint(tmax) << 32) | kNoHit;
            }
        }
        __syncwarp();
        if (__ballot_sync(0xffffffffu, ray != kNoHit) == 0) break;
        if (COUNT) {
            if (lane == 0) loop_iters++;
            if (ray != kNoHit) loop_busy++;
        }
        // node phase (a lane holding unqueued triangles waits); a lane whose
        // node exposed no triangle takes the next node in the same iteration
#pragma unroll 1
        for (uint32_t k = 0; k < kNodeSteps; ++k) {
            if (ray != kNoHit && tmask == 0 && st.g_mask > 0x00ffffffu) {
                const float best_t = __uint_as_float((uint32_t)(w.key[lane] >> 32));
                tmask = node_step<COUNT>(st, stack, s, best_t, overflow, &cnt, tbase);
            }
        }
        // queue the exposed triangles that fit, in lane order
        const uint32_t c = __popc(tmask);
        uint32_t incl = c;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= (uint32_t)d) incl += y;
        }
        const bool fits = qn + incl <= kTriQueueCap;
        const uint32_t added = __reduce_max_sync(0xffffffffu, fits ? incl : 0u);
        if (c && fits) {
            uint32_t e = qn + incl - c;
            while (tmask) {
                const uint32_t b = __ffs(tmask) - 1u;
                tmask &= tmask - 1u;
                w.tri[e++] = (lane << 27) | (tbase + b);
            }
            queued = true;
        }
        qn += added;
        __syncwarp();
        const bool has_node = ray != kNoHit && st.g_mask > 0x00ffffffu;
        const bool pending = queued || tmask != 0;
        const uint32_t parked = __ballot_sync(0xffffffffu, ray != kNoHit && !has_node && pending);
        const uint32_t walking = __ballot_sync(0xffffffffu, has_node && tmask == 0);
        const uint32_t carried = __ballot_sync(0xffffffffu, tmask != 0);
        if (qn >= flush_tris || (uint32_t)__popc(parked) >= flush_parked || carried != 0 || (qn > 0 && walking == 0)) {
            if (FP16) warp_test_tris_shfl<COUNT, WA>(w, lane, qn, s, st, overflow, &cnt);
            else warp_test_tris<COUNT, WA>(w, lane, qn, s, qo, qr1, q.so, q.sr1, overflow, &cnt);
            qn = 0;
            queued = false;
        }
        // finish rays with no node and no pending triangle, and shadow rays with a hit
        if (ray != kNoHit && !queued && tmask == 0) {
            const unsigned long long key = w.key[lane];
            const uint32_t best = (uint32_t)key;
            if (!has_node || (st.shadow && best != kNoHit)) {
                if (st.shadow) {
                    if (best == kNoHit) {
                        const float4 cc = q.sc[ray];
                        const uint32_t path = __float_as_uint(cc.w);
                        const float4 L = q.L[path];
                        q.L[path] = make_float4(L.x + cc.x, L.y + cc.y, L.z + cc.z, 0.0f);
                    }
                } else {
                    const float2 uv = w.uv[lane];
                    if (FP16)
                        reinterpret_cast<uint2*>(q.hit)[ray] = make_uint2(best, best != kNoHit ? half2_bits(uv.x, uv.y) : 0u);
                    else
                        q.hit[ray] = best != kNoHit
                                         ? make_float4(__uint_as_float((uint32_t)(key >> 32)), __uint_as_float(best), uv.x, uv.y)
                                         : make_float4(0.0f, __uint_as_float(kNoHit), 0.0f, 0.0f);
                    if (q.list_mode == 1u) shade_list_append(q, best == kNoHit, ray);
                }
                ray = kNoHit;
            }
        }
        __syncwarp();
    }
    if (COUNT) {
        atomicAdd(&q.stats[2], (unsigned long long)cnt.nodes);
        atomicAdd(&q.stats[3], (unsigned long long)cnt.tris);
        atomicAdd(&q.stats[4], (unsigned long long)cnt.warp_nodes);
        atomicAdd(&q.stats[5], (unsigned long long)cnt.warp_tris);
        atomicAdd(&q.stats[6], (unsigned long long)loop_iters);
        atomicAdd(&q.stats[7], (unsigned long long)loop_busy);
        atomicAdd(&q.stats[8], (unsigned long long)cnt.alpha);
    }
    if (overflow) atomicOr(q.status, 1u);
}

// One traversal launch: the batched kernel for scenes under 2^27 triangles
// (the queue's triangle index field), else the per-lane one; the WA
// instantiations (wide-alpha any-hit path) only for scenes that need them.
template <bool COUNT, bool FP16>
static inline void launch_extend(const DevScene& s, const Queues& q, int grid_batched, int grid_trace, cudaStream_t st,
                                 const float4* qo, const float4* qr0, const float4* qr1, const uint32_t* qp,
                                 const uint32_t* count, uint32_t* fetch) {
    if (s.num_prims < (1u << 27)) {
        if (s.wide_alpha)
            k_extend_batched<COUNT, true, FP16><<<grid_batched, kTraceThreads, 0, st>>>(s, q, qo, qr0, qr1, count, fetch,
                                                                                        kFlushTris, kFlushParked, qp);
        else
            k_extend_batched<COUNT, false, FP16><<<grid_batched, kTraceThreads, 0, st>>>(s, q, qo, qr0, qr1, count, fetch,
                                                                                         kFlushTris, kFlushParked, qp);
    } else {
        if (s.wide_alpha)
            k_extend<COUNT, FP16, true><<<grid_trace, kTraceThreads, 0, st>>>(s, q, qo, qr0, qr1, qp, count, fetch);
        else
            k_extend<COUNT, FP16, false><<<grid_trace, kTraceThreads, 0, st>>>(s, q, qo, qr0, qr1, qp, count, fetch);
    }
}

// Accumulation (path_trace_rgen.glsl:217-248): clamp, then running mean
// prev + (c - prev) / num_frames with frame 0 stored raw; or Kahan sum.
// With nan_red, a sample whose radiance has a NaN stores (1, 0, 0) in its
// pixel in place of the running mean (VISUALIZE_NANS, path_trace_rgen.glsl:
// 225-244; running mean only).
__global__ void k_accumulate(Rect rect, uint32_t W, uint32_t frame0, uint32_t nframes, float clampv, uint32_t kahan,
                             uint32_t nan_red, const float4* __restrict__ L, float4* __restrict__ acc,
                             float4* __restrict__ comp) {
    uint32_t npix = rect.w * rect.h;
    for (uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x; pix < npix; pix += gridDim.x * blockDim.x) {
        uint32_t x, y;
        pix_xy(rect, pix, x, y);
        size_t idx = (size_t)y * W + x;
        float4 a = acc[idx];
        float4 cp = kahan ? comp[idx] : make_float4(0, 0, 0, 0);
        for (uint32_t f = 0; f < nframes; ++f) {
            float4 l = L[path_index(pix, f, nframes)];
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
            if (nan_red && (isnan(l.x) || isnan(l.y) || isnan(l.z))) {
                a.x = 1.0f;
                a.y = 0.0f;
                a.z = 0.0f;
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
        uint32_t x, y;
        pix_xy(rect, pix, x, y);
        count_map[(size_t)y * W + x] += add;
    }
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
    P.ray_offset = p.ray_offset == HX_RAY_OFFSET_SCALED ? 1u : 0u;
    return P;
}


// Denoiser features per pixel (12 floats): current image rgb, noise level,
// albedo rgb, depth feature log1p(t)/8, shading normal xyz, 0 — first-hit AOVs
// as the reference's debug views define them (debug_visualization.frag:
// 142-161: base colour, shading normal); zeros on a miss.  The noise level is
// 1 / sqrt(samples in the pixel) (the Monte Carlo standard error's scale), from
// the per-pixel count map, or `samples` for every pixel when it is null.
HXD float noise_level(const uint32_t* count_map, uint32_t samples, uint32_t i) {
    const uint32_t c = count_map ? count_map[i] : samples;
    return 1.0f / sqrtf((float)(c > 0u ? c : 1u));
}
__global__ void k_features(DevScene s, const float4* __restrict__ hit, const float4* __restrict__ img, uint32_t W,
                           uint32_t H, const uint32_t* __restrict__ count_map, float* __restrict__ feat) {
    const Rect rect{0, 0, W, H};
    const uint32_t n = W * H;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        // pixel i (row-major) was traced as path pix_of_xy (one frame)
        const float4 h = hit[pix_of_xy(rect, i % W, i / W)], r = img[i];
        const uint32_t prim = __float_as_uint(h.y);
        V3 alb = v3(0.0f), nrm = v3(0.0f);
        float depth = 0.0f;
        if (prim != kNoHit) {
            Surface sf = populate(s, prim, h.z, h.w);
            alb = sf.albedo;
            nrm = normalize(sf.normal);
            depth = log1pf(h.x) * 0.125f;
        }
        float4* o = reinterpret_cast<float4*>(feat + 12 * (size_t)i);
        o[0] = make_float4(r.x, r.y, r.z, noise_level(count_map, 1u, i));
        o[1] = make_float4(alb.x, alb.y, alb.z, depth);
        o[2] = make_float4(nrm.x, nrm.y, nrm.z, 0.0f);
    }
}

// First-hit AOVs accumulated per pixel over the frames of a wavefront, in
// frame order (exact running mean), right after the primary-ray trace:
// albedo rgb + depth feature log1p(t)/8 in aov_a, shading normal in aov_n;
// zeros on a miss.  These are the denoiser's auxiliary features averaged over
// the same jittered samples as the radiance.
template <bool FP16>
__global__ void k_aov_accumulate(DevScene s, Rect rect, uint32_t frame0, uint32_t nframes, const float4* __restrict__ hit,
                                 float4* __restrict__ aov_a, float4* __restrict__ aov_n, uint32_t W) {
    const uint32_t npix = rect.w * rect.h;
    for (uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x; pix < npix; pix += gridDim.x * blockDim.x) {
        uint32_t x, y;
        pix_xy(rect, pix, x, y);
        const size_t o = (size_t)y * W + x;
        float4 a = aov_a[o], nn = aov_n[o];
        for (uint32_t fr = 0; fr < nframes; ++fr) {
            const uint32_t p = path_index(pix, fr, nframes);
            uint32_t prim;
            float t, u, v;
            if (FP16) {
                const uint2 hh = reinterpret_cast<const uint2*>(hit)[p];
                prim = hh.x;
                __half2 uv = *reinterpret_cast<const __half2*>(&hh.y);
                u = __low2float(uv);
                v = __high2float(uv);
                t = 1.0f;  // the 8-byte hit record carries no distance
            } else {
                const float4 h = hit[p];
                prim = __float_as_uint(h.y);
                t = h.x;
                u = h.z;
                v = h.w;
            }
            V3 alb = v3(0.0f), nrm = v3(0.0f);
            float depth = 0.0f;
            if (prim != kNoHit) {
                Surface sf = populate(s, prim, u, v);
                alb = sf.albedo;
                nrm = normalize(sf.normal);
                depth = log1pf(t) * 0.125f;
            }
            const float w = 1.0f / (float)(frame0 + fr + 1);
            a = make_float4(a.x + (alb.x - a.x) * w, a.y + (alb.y - a.y) * w, a.z + (alb.z - a.z) * w,
                            a.w + (depth - a.w) * w);
            nn = make_float4(nn.x + (nrm.x - nn.x) * w, nn.y + (nrm.y - nn.y) * w, nn.z + (nrm.z - nn.z) * w, 0.0f);
        }
        aov_a[o] = a;
        aov_n[o] = nn;
    }
}

// Denoiser features from the accumulated image and accumulated AOVs (noise
// level from count_map, or `samples` for every pixel when it is null).
__global__ void k_features_accumulated(const float4* __restrict__ img, const float4* __restrict__ aov_a,
                                       const float4* __restrict__ aov_n, uint32_t n,
                                       const uint32_t* __restrict__ count_map, uint32_t samples,
                                       float* __restrict__ feat) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 r = img[i];
        float4* o = reinterpret_cast<float4*>(feat + 12 * (size_t)i);
        o[0] = make_float4(r.x, r.y, r.z, noise_level(count_map, samples, i));
        o[1] = aov_a[i];
        o[2] = aov_n[i];
    }
}

}  // namespace
