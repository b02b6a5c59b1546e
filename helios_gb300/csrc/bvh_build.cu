// bvh_build.cu — device LBVH -> BVH8 build (replaces the driver-built
// BLAS/TLAS of src/engine/resource/mesh.cpp:61-117, renderer.cpp:113-181).
//
// Pipeline (all on the context stream):
//   k_world_tris      instance transforms applied to every flattened triangle
//   k_centroid_bounds / k_bounds_final   scene bounds of triangle centroids
//   k_morton          30-bit Morton codes (10 bits per axis)
//   radix sort        stable (code, prim) sort
//   k_karras          binary radix tree (Karras 2012), duplicate codes
//                     resolved by the sorted index
//   k_fit             bottom-up boxes with one atomic arrival flag per node
//   k_collapse_plan / k_collapse_emit    breadth-first 8-wide collapse,
//                     one level per pair of launches; allocation offsets come
//                     from exclusive scans so the node order is deterministic
//   k_leaf_tris       leaf-ordered triangle records for traversal
// Built with --fmad=false: every float operation rounds exactly like the
// oracle's, so codes, topology, node order and quantised boxes are bit-exact.
#include "hx_internal.h"

#include <algorithm>

namespace {

constexpr int kThreads = 256;
constexpr uint32_t kLeafMax = 1;  // triangles per leaf slot
constexpr int kTreeletPasses = 3;
// meta bytes: the low 5 bits are the slot's bit in the traversal's hit mask
constexpr uint8_t kMetaEmpty = 0x10;     // bit 16: outside the triangle and child masks
constexpr uint8_t kMetaInternal = 0x98;  // | slot: bit 7 (internal) + bit 24 + slot
constexpr uint8_t kMetaLeaf = 0x20;      // | offset: one triangle

__device__ __forceinline__ uint32_t expand_bits(uint32_t v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

__global__ void k_world_tris(const uint4* __restrict__ prim_info, const uint32_t* __restrict__ indices,
                             const float4* __restrict__ vtx, const DevInstance* __restrict__ inst, uint32_t n,
                             float* __restrict__ world) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    uint4 pi = prim_info[p];
    const float* m = inst[pi.x].model;
    for (int c = 0; c < 3; ++c) {
        uint32_t vi = indices[3 * pi.y + c];
        float4 v = vtx[2 * vi];
        for (int r = 0; r < 3; ++r)
            world[9 * (size_t)p + 3 * c + r] = m[0 + r] * v.x + m[4 + r] * v.y + m[8 + r] * v.z + m[12 + r] * 1.0f;
    }
}

__device__ __forceinline__ void centroid(const float* __restrict__ world, uint32_t p, float c[3]) {
    const float* q = world + 9 * (size_t)p;
    for (int a = 0; a < 3; ++a) c[a] = (q[a] + q[3 + a] + q[6 + a]) / 3.0f;
}

__global__ void k_centroid_bounds(const float* __restrict__ world, uint32_t n, float* __restrict__ partial) {
    __shared__ float s[6][kThreads];
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        float c[3];
        centroid(world, p, c);
        for (int a = 0; a < 3; ++a) {
            lo[a] = c[a] < lo[a] ? c[a] : lo[a];
            hi[a] = c[a] > hi[a] ? c[a] : hi[a];
        }
    }
    for (int a = 0; a < 3; ++a) { s[a][threadIdx.x] = lo[a]; s[3 + a][threadIdx.x] = hi[a]; }
    __syncthreads();
    for (int o = kThreads / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            for (int a = 0; a < 3; ++a) {
                float x = s[a][threadIdx.x + o], y = s[3 + a][threadIdx.x + o];
                s[a][threadIdx.x] = x < s[a][threadIdx.x] ? x : s[a][threadIdx.x];
                s[3 + a][threadIdx.x] = y > s[3 + a][threadIdx.x] ? y : s[3 + a][threadIdx.x];
            }
        __syncthreads();
    }
    if (threadIdx.x < 6) partial[6 * blockIdx.x + threadIdx.x] = s[threadIdx.x][0];
}

__global__ void k_bounds_final(const float* __restrict__ partial, uint32_t nb, float* __restrict__ out) {
    if (threadIdx.x != 0) return;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t b = 0; b < nb; ++b)
        for (int a = 0; a < 3; ++a) {
            float x = partial[6 * b + a], y = partial[6 * b + 3 + a];
            lo[a] = x < lo[a] ? x : lo[a];
            hi[a] = y > hi[a] ? y : hi[a];
        }
    for (int a = 0; a < 3; ++a) { out[a] = lo[a]; out[3 + a] = hi[a]; }
}

__global__ void k_morton(const float* __restrict__ world, uint32_t n, const float* __restrict__ bounds,
                         uint32_t* __restrict__ morton, uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    float c[3];
    centroid(world, p, c);
    uint32_t q[3];
    for (int a = 0; a < 3; ++a) {
        float ext = bounds[3 + a] - bounds[a];
        float f = ext > 0.0f ? (c[a] - bounds[a]) / ext : 0.0f;
        float sc = f * 1024.0f;
        sc = sc < 0.0f ? 0.0f : (sc > 1023.0f ? 1023.0f : sc);
        q[a] = (uint32_t)sc;
    }
    uint32_t code = (expand_bits(q[0]) << 2) | (expand_bits(q[1]) << 1) | expand_bits(q[2]);
    morton[p] = code;
    keys[p] = code;
    vals[p] = p;
}

__device__ __forceinline__ int kdelta(const uint32_t* __restrict__ keys, int n, int i, int j) {
    if (j < 0 || j > n - 1) return -1;
    uint32_t a = keys[i], b = keys[j];
    if (a == b) return 32 + __clz((uint32_t)i ^ (uint32_t)j);
    return __clz(a ^ b);
}

__global__ void k_karras(const uint32_t* __restrict__ keys, int n, uint32_t* __restrict__ children,
                         uint32_t* __restrict__ first, uint32_t* __restrict__ count, int* __restrict__ parent_int,
                         int* __restrict__ parent_leaf) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    int d = kdelta(keys, n, i, i + 1) - kdelta(keys, n, i, i - 1) >= 0 ? 1 : -1;
    int dmin = kdelta(keys, n, i, i - d);
    int lmax = 2;
    while (kdelta(keys, n, i, i + lmax * d) > dmin) lmax *= 2;
    int l = 0;
    for (int t = lmax / 2; t >= 1; t /= 2)
        if (kdelta(keys, n, i, i + (l + t) * d) > dmin) l += t;
    int j = i + l * d;
    int dnode = kdelta(keys, n, i, j);
    int s = 0, t = l;
    do {
        t = (t + 1) >> 1;
        if (kdelta(keys, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    int gamma = i + s * d + (d < 0 ? d : 0);
    int lo = i < j ? i : j, hi = i < j ? j : i;
    uint32_t left, right;
    if (lo == gamma) { left = 0x80000000u | (uint32_t)gamma; parent_leaf[gamma] = i; }
    else { left = (uint32_t)gamma; parent_int[gamma] = i; }
    if (hi == gamma + 1) { right = 0x80000000u | (uint32_t)(gamma + 1); parent_leaf[gamma + 1] = i; }
    else { right = (uint32_t)(gamma + 1); parent_int[gamma + 1] = i; }
    children[2 * i] = left;
    children[2 * i + 1] = right;
    first[i] = lo;
    count[i] = hi - lo + 1;
}

__global__ void k_leaf_boxes(const float* __restrict__ world, const uint32_t* __restrict__ sorted, uint32_t n,
                             float* __restrict__ llo, float* __restrict__ lhi) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* p = world + 9 * (size_t)sorted[i];
    for (int a = 0; a < 3; ++a) {
        float lo = p[a], hi = p[a];
        lo = p[3 + a] < lo ? p[3 + a] : lo; hi = p[3 + a] > hi ? p[3 + a] : hi;
        lo = p[6 + a] < lo ? p[6 + a] : lo; hi = p[6 + a] > hi ? p[6 + a] : hi;
        llo[3 * (size_t)i + a] = lo;
        lhi[3 * (size_t)i + a] = hi;
    }
}

__device__ __forceinline__ void child_box(uint32_t c, const float* llo, const float* lhi, const float* blo,
                                          const float* bhi, const float*& lo, const float*& hi) {
    if (c & 0x80000000u) { lo = llo + 3 * (size_t)(c & 0x7fffffffu); hi = lhi + 3 * (size_t)(c & 0x7fffffffu); }
    else { lo = blo + 3 * (size_t)c; hi = bhi + 3 * (size_t)c; }
}

// Bottom-up fit: the second thread to reach a node computes its box.
__global__ void k_fit(uint32_t n, const uint32_t* __restrict__ children, const int* __restrict__ parent_int,
                      const int* __restrict__ parent_leaf, const float* __restrict__ llo, const float* __restrict__ lhi,
                      float* blo, float* bhi, uint32_t* flags, uint32_t* status) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int node = parent_leaf[i];
    // tree depth is at most n - 1; the cap turns a malformed hierarchy into
    // a reported error instead of an endless walk
    uint32_t steps = 0;
    while (node >= 0) {
        if (++steps > n + 1) {
            atomicOr(status, 1u);
            return;
        }
        __threadfence();
        if (atomicAdd(&flags[node], 1u) == 0) return;
        __threadfence();
        const float *al, *ah, *bl, *bh;
        child_box(children[2 * node], llo, lhi, blo, bhi, al, ah);
        child_box(children[2 * node + 1], llo, lhi, blo, bhi, bl, bh);
        for (int a = 0; a < 3; ++a) {
            float x = __ldcg(al + a), y = __ldcg(bl + a);
            float u = __ldcg(ah + a), v = __ldcg(bh + a);
            __stcg(blo + 3 * (size_t)node + a, x < y ? x : y);
            __stcg(bhi + 3 * (size_t)node + a, u > v ? u : v);
        }
        node = parent_int[node];
    }
}

__device__ __forceinline__ float half_area(const float* lo, const float* hi) {
    float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    return dx * dy + dy * dz + dz * dx;
}

// Treelet restructuring of the binary LBVH (Karras & Aila, "Fast Parallel
// Construction of High-Quality Bounding Volume Hierarchies", HPG 2013), one
// pass: threads climb from the leaves like k_fit, the second to arrive at a
// node processes it, so a node is handled after all its descendants.  A node
// R with >= 3 triangles grows a treelet of up to 7 leaves (open the leaf with
// the largest surface area, ties: the first), finds the binary topology over
// those leaves with the least surface-area cost by dynamic programming over
// leaf subsets (partitions enumerated downwards, ties: the first) and
// rebuilds the treelet with it when that is cheaper, reusing its internal
// nodes in pre-order and updating boxes, triangle counts, costs and parent
// links.  The oracle's builder runs the same steps in a topological order;
// the result depends only on each node's subtree, so the trees are equal.
constexpr int kTreeletLeaves = 7;
constexpr float kTreeletCi = 1.2f, kTreeletCt = 1.0f;

struct TreeletCtx {
    uint32_t* children;
    int* parent_int;
    int* parent_leaf;
    const float* llo;
    const float* lhi;
    float* blo;
    float* bhi;
    uint32_t* count;
    float* cost;
};

__device__ __forceinline__ void item_box(const TreeletCtx& t, uint32_t c, float lo[3], float hi[3]) {
    const float* l = (c & 0x80000000u) ? t.llo + 3 * (size_t)(c & 0x7fffffffu) : t.blo + 3 * (size_t)c;
    const float* h = (c & 0x80000000u) ? t.lhi + 3 * (size_t)(c & 0x7fffffffu) : t.bhi + 3 * (size_t)c;
    for (int a = 0; a < 3; ++a) {
        lo[a] = __ldcg(l + a);
        hi[a] = __ldcg(h + a);
    }
}
__device__ __forceinline__ float item_cost(const TreeletCtx& t, uint32_t c) {
    if (c & 0x80000000u) {
        float lo[3], hi[3];
        item_box(t, c, lo, hi);
        return kTreeletCt * half_area(lo, hi);
    }
    return __ldcg(t.cost + c);
}
__device__ __forceinline__ uint32_t item_count(const TreeletCtx& t, uint32_t c) {
    return (c & 0x80000000u) ? 1u : __ldcg(t.count + c);
}

__device__ void treelet_node(const TreeletCtx& t, uint32_t R) {
    const uint32_t l0 = __ldcg(t.children + 2 * (size_t)R), r0 = __ldcg(t.children + 2 * (size_t)R + 1);
    float lo[3], hi[3];
    item_box(t, R, lo, hi);
    const float cR = kTreeletCi * half_area(lo, hi) + (item_cost(t, l0) + item_cost(t, r0));
    __stcg(t.cost + R, cR);
    if (__ldcg(t.count + R) < 3u) return;
    uint32_t leaves[kTreeletLeaves], used[kTreeletLeaves - 1];
    int nl = 2, nu = 1;
    leaves[0] = l0;
    leaves[1] = r0;
    used[0] = R;
    while (nl < kTreeletLeaves) {
        int bi = -1;
        float ba = 0.0f;
        for (int k = 0; k < nl; ++k) {
            if (leaves[k] & 0x80000000u) continue;
            item_box(t, leaves[k], lo, hi);
            const float a = half_area(lo, hi);
            if (bi < 0 || a > ba) { bi = k; ba = a; }
        }
        if (bi < 0) break;
        const uint32_t x = leaves[bi];
        used[nu++] = x;
        leaves[bi] = __ldcg(t.children + 2 * (size_t)x);
        leaves[nl++] = __ldcg(t.children + 2 * (size_t)x + 1);
    }
    float llo_[kTreeletLeaves][3], lhi_[kTreeletLeaves][3];
    for (int k = 0; k < nl; ++k) item_box(t, leaves[k], llo_[k], lhi_[k]);
    const int full = (1 << nl) - 1;
    float sarea[1 << kTreeletLeaves], scost[1 << kTreeletLeaves];
    uint8_t spart[1 << kTreeletLeaves];
    for (int S = 1; S <= full; ++S) {
        float slo[3] = {INFINITY, INFINITY, INFINITY}, shi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int k = 0; k < nl; ++k) {
            if (!(S >> k & 1)) continue;
            for (int a = 0; a < 3; ++a) {
                slo[a] = llo_[k][a] < slo[a] ? llo_[k][a] : slo[a];
                shi[a] = lhi_[k][a] > shi[a] ? lhi_[k][a] : shi[a];
            }
        }
        sarea[S] = half_area(slo, shi);
    }
    for (int S = 1; S <= full; ++S) {
        if ((S & (S - 1)) == 0) {
            scost[S] = item_cost(t, leaves[__ffs(S) - 1]);
            spart[S] = 0;
            continue;
        }
        // partitions (P, S ^ P) with P holding the lowest leaf, P descending
        const int low = S & -S, rest = S ^ low;
        float best = INFINITY;
        int bp = 0;
        for (int Q = (rest - 1) & rest;; Q = (Q - 1) & rest) {
            const int P = Q | low;
            const float c = scost[P] + scost[S ^ P];
            if (c < best) { best = c; bp = P; }
            if (Q == 0) break;
        }
        scost[S] = kTreeletCi * sarea[S] + best;
        spart[S] = (uint8_t)bp;
    }
    if (!(scost[full] < cR * 0.99999f)) return;
    uint32_t node_of[1 << kTreeletLeaves];
    int seq[kTreeletLeaves - 1], ns = 0, stk[kTreeletLeaves], sp = 0, ui = 0;
    stk[sp++] = full;
    while (sp > 0) {
        const int S = stk[--sp];
        node_of[S] = used[ui++];
        seq[ns++] = S;
        const int P = spart[S], Q = S ^ P;
        if (Q & (Q - 1)) stk[sp++] = Q;
        if (P & (P - 1)) stk[sp++] = P;
    }
    for (int j = 0; j < ns; ++j) {
        const uint32_t node = node_of[seq[j]];
        const int P = spart[seq[j]], Q = seq[j] ^ P;
        const uint32_t l = (P & (P - 1)) == 0 ? leaves[__ffs(P) - 1] : node_of[P];
        const uint32_t r = (Q & (Q - 1)) == 0 ? leaves[__ffs(Q) - 1] : node_of[Q];
        __stcg(t.children + 2 * (size_t)node, l);
        __stcg(t.children + 2 * (size_t)node + 1, r);
        if (l & 0x80000000u) __stcg(t.parent_leaf + (l & 0x7fffffffu), (int)node);
        else __stcg(t.parent_int + l, (int)node);
        if (r & 0x80000000u) __stcg(t.parent_leaf + (r & 0x7fffffffu), (int)node);
        else __stcg(t.parent_int + r, (int)node);
    }
    for (int j = ns - 1; j >= 0; --j) {
        const uint32_t node = node_of[seq[j]];
        const uint32_t l = __ldcg(t.children + 2 * (size_t)node), r = __ldcg(t.children + 2 * (size_t)node + 1);
        float al[3], ah[3], bl[3], bh[3];
        item_box(t, l, al, ah);
        item_box(t, r, bl, bh);
        float nlo[3], nhi[3];
        for (int a = 0; a < 3; ++a) {
            nlo[a] = al[a] < bl[a] ? al[a] : bl[a];
            nhi[a] = ah[a] > bh[a] ? ah[a] : bh[a];
            __stcg(t.blo + 3 * (size_t)node + a, nlo[a]);
            __stcg(t.bhi + 3 * (size_t)node + a, nhi[a]);
        }
        __stcg(t.count + node, item_count(t, l) + item_count(t, r));
        __stcg(t.cost + node, kTreeletCi * half_area(nlo, nhi) + (item_cost(t, l) + item_cost(t, r)));
    }
}

__global__ void k_treelet(uint32_t n, TreeletCtx t, uint32_t* flags, uint32_t* status) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int node = __ldcg(t.parent_leaf + i);
    uint32_t steps = 0;
    while (node >= 0) {
        if (++steps > n + 1) {
            atomicOr(status, 1u);
            return;
        }
        __threadfence();
        if (atomicAdd(&flags[node], 1u) == 0) return;
        __threadfence();
        treelet_node(t, (uint32_t)node);
        __threadfence();
        node = __ldcg(t.parent_int + node);
    }
}

__device__ __forceinline__ float pow2f(int e) { return __uint_as_float((uint32_t)(e < -126 ? 1 : e + 127) << 23); }
__device__ __forceinline__ int ceil_log2f(float x) {
    uint32_t b = __float_as_uint(x);
    int ex = (int)((b >> 23) & 0xff);
    if (ex == 0) return -126;
    int e = ex - 127 + ((b & 0x7fffff) != 0 ? 1 : 0);
    return e < -126 ? -126 : e;
}
// Grid exponent of one node axis (see the oracle's grid_exponent): 254
// steps cover [lo, hi] (the snapped origin adds at most one) and 2^e >= 2 ulp(max |coordinate|), so every decoded
// plane is exactly representable.
__device__ __forceinline__ int grid_exponent(float lo, float hi) {
    float ext = hi - lo;
    int e = ext > 0.0f ? ceil_log2f(ext / 254.0f) : -126;
    float m = fabsf(lo) > fabsf(hi) ? fabsf(lo) : fabsf(hi);
    uint32_t mb = __float_as_uint(m);
    int mexp = (int)((mb >> 23) & 0xff);
    int e_min = mexp == 0 ? -126 : mexp - 127 - 23 + 1;
    e = e > e_min ? e : e_min;
    return e < -126 ? -126 : (e > 119 ? 119 : e);
}
struct Plan {
    uint32_t kids[8];
    uint32_t nk;
};

// Greedy collapse plan for each BVH8 node of the level: start from the two
// children of the binary node and repeatedly open the internal child with
// more than kLeafMax triangles and the largest surface area (ties: lower
// binary index) until 8 children or none left; children keep range order.
__global__ void k_collapse_plan(const uint32_t* __restrict__ queue, uint32_t level_begin, uint32_t level_count,
                                const uint32_t* __restrict__ children, const uint32_t* __restrict__ count,
                                const float* __restrict__ blo, const float* __restrict__ bhi, Plan* __restrict__ plans,
                                uint32_t* __restrict__ n_int, uint32_t* __restrict__ n_leaf) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= level_count) return;
    uint32_t src = queue[level_begin + k];
    Plan pl;
    uint32_t nk = 0;
    if (src & 0x80000000u) pl.kids[nk++] = src;
    else {
        pl.kids[nk++] = children[2 * src];
        pl.kids[nk++] = children[2 * src + 1];
        while (nk < 8) {
            int best = -1;
            float best_area = -1.0f;
            for (uint32_t c = 0; c < nk; ++c) {
                uint32_t it = pl.kids[c];
                if ((it & 0x80000000u) || count[it] <= kLeafMax) continue;
                float a = half_area(blo + 3 * (size_t)it, bhi + 3 * (size_t)it);
                if (best < 0 || a > best_area || (a == best_area && it < pl.kids[best])) { best = (int)c; best_area = a; }
            }
            if (best < 0) break;
            uint32_t it = pl.kids[best];
            for (int c = (int)nk; c > best + 1; --c) pl.kids[c] = pl.kids[c - 1];
            pl.kids[best] = children[2 * it];
            pl.kids[best + 1] = children[2 * it + 1];
            ++nk;
        }
    }
    pl.nk = nk;
    uint32_t ni = 0, nl = 0;
    for (uint32_t c = 0; c < nk; ++c) {
        uint32_t it = pl.kids[c];
        if (!(it & 0x80000000u) && count[it] > kLeafMax) ++ni;
        else nl += (it & 0x80000000u) ? 1u : count[it];
    }
    plans[k] = pl;
    n_int[k] = ni;
    n_leaf[k] = nl;
}

// Octant slot assignment (same rule as the oracle): slot bit k set = child
// centre on the positive side of the node centre along axis k; greedy over
// (child, slot) pairs by decreasing alignment score, ties to the lower child
// position then the lower slot.
__device__ void assign_octant_slots(uint32_t nk, const float (*klo)[3], const float (*khi)[3], uint32_t slot_kid[8]) {
    float nlo[3] = {INFINITY, INFINITY, INFINITY}, nhi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t c = 0; c < nk; ++c)
        for (int a = 0; a < 3; ++a) {
            nlo[a] = klo[c][a] < nlo[a] ? klo[c][a] : nlo[a];
            nhi[a] = khi[c][a] > nhi[a] ? khi[c][a] : nhi[a];
        }
    float score[8][8];
    for (uint32_t c = 0; c < nk; ++c) {
        float dv[3];
        for (int a = 0; a < 3; ++a) dv[a] = (klo[c][a] + khi[c][a]) * 0.5f - (nlo[a] + nhi[a]) * 0.5f;
        for (int sl = 0; sl < 8; ++sl) {
            float x = (sl & 1) ? dv[0] : -dv[0];
            float y = (sl & 2) ? dv[1] : -dv[1];
            float z = (sl & 4) ? dv[2] : -dv[2];
            score[c][sl] = x + y + z;
        }
    }
    for (int sl = 0; sl < 8; ++sl) slot_kid[sl] = 0xffffffffu;
    uint32_t done = 0;
    for (uint32_t round = 0; round < nk; ++round) {
        int bc = -1, bs = -1;
        float best = 0.0f;
        for (uint32_t c = 0; c < nk; ++c) {
            if (done & (1u << c)) continue;
            for (int sl = 0; sl < 8; ++sl) {
                if (slot_kid[sl] != 0xffffffffu) continue;
                if (bc < 0 || score[c][sl] > best) { bc = (int)c; bs = sl; best = score[c][sl]; }
            }
        }
        done |= 1u << bc;
        slot_kid[bs] = (uint32_t)bc;
    }
}

__global__ void k_collapse_emit(uint32_t* __restrict__ queue, uint32_t level_begin, uint32_t level_count,
                                uint32_t level_end, uint32_t leaf_base, const Plan* __restrict__ plans,
                                const uint32_t* __restrict__ scan_int, const uint32_t* __restrict__ scan_leaf,
                                const uint32_t* __restrict__ first, const uint32_t* __restrict__ count,
                                const uint32_t* __restrict__ sorted, const float* __restrict__ llo,
                                const float* __restrict__ lhi, const float* __restrict__ blo,
                                const float* __restrict__ bhi, hx_bvh8_node* __restrict__ nodes,
                                uint32_t* __restrict__ leaf_prims) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= level_count) return;
    const Plan pl = plans[k];
    float klo[8][3], khi[8][3];
    for (uint32_t c = 0; c < pl.nk; ++c) {
        const float *lo, *hi;
        child_box(pl.kids[c], llo, lhi, blo, bhi, lo, hi);
        for (int a = 0; a < 3; ++a) { klo[c][a] = lo[a]; khi[c][a] = hi[a]; }
    }
    uint32_t slot_kid[8];
    assign_octant_slots(pl.nk, klo, khi, slot_kid);
    hx_bvh8_node node;
    uint8_t* raw = (uint8_t*)&node;
    for (int b = 0; b < (int)sizeof(node); ++b) raw[b] = 0;
    node.child_base = level_end + scan_int[k];
    node.prim_base = leaf_base + scan_leaf[k];
    float clo[8][3], chi[8][3];
    uint32_t rank = 0, off = 0;
    for (uint32_t c = 0; c < 8; ++c) {
        if (slot_kid[c] == 0xffffffffu) {
            for (int a = 0; a < 3; ++a) { clo[c][a] = 0.0f; chi[c][a] = 0.0f; }
            node.meta[c] = kMetaEmpty;
            continue;
        }
        uint32_t it = pl.kids[slot_kid[c]];
        for (int a = 0; a < 3; ++a) { clo[c][a] = klo[slot_kid[c]][a]; chi[c][a] = khi[slot_kid[c]][a]; }
        if (!(it & 0x80000000u) && count[it] > kLeafMax) {
            node.meta[c] = (uint8_t)(kMetaInternal | c);
            node.internal_mask |= (uint8_t)(1u << c);
            queue[node.child_base + rank] = it;
            ++rank;
        } else {
            uint32_t cnt = (it & 0x80000000u) ? 1u : count[it];
            uint32_t f = (it & 0x80000000u) ? (it & 0x7fffffffu) : first[it];
            node.meta[c] = (uint8_t)(kMetaLeaf | off);
            for (uint32_t q = 0; q < cnt; ++q) leaf_prims[node.prim_base + off + q] = sorted[f + q];
            off += cnt;
        }
    }
    // quantise the occupied slots on the node grid (conservative, exact decode)
    float plo[3] = {INFINITY, INFINITY, INFINITY}, phi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t c = 0; c < 8; ++c) {
        if (node.meta[c] == kMetaEmpty) continue;
        for (int a = 0; a < 3; ++a) {
            plo[a] = clo[c][a] < plo[a] ? clo[c][a] : plo[a];
            phi[a] = chi[c][a] > phi[a] ? chi[c][a] : phi[a];
        }
    }
    for (int a = 0; a < 3; ++a) {
        int e = grid_exponent(plo[a], phi[a]);
        float scale = pow2f(e);
        float origin = floorf(plo[a] * pow2f(-e)) * scale;
        while (e < 119 && origin + 255.0f * scale < phi[a]) {
            ++e;
            scale = pow2f(e);
            origin = floorf(plo[a] * pow2f(-e)) * scale;
        }
        node.origin[a] = origin;
        node.exponent[a] = (int8_t)e;
        float inv = pow2f(-e);
        for (uint32_t c = 0; c < 8; ++c) {
            if (node.meta[c] == kMetaEmpty) continue;
            float fl = floorf((clo[c][a] - origin) * inv);
            int ql = fl < 0.0f ? 0 : (fl > 255.0f ? 255 : (int)fl);
            while (ql > 0 && origin + (float)ql * scale > clo[c][a]) --ql;
            float fh = ceilf((chi[c][a] - origin) * inv);
            int qh = fh < 0.0f ? 0 : (fh > 255.0f ? 255 : (int)fh);
            while (qh < 255 && origin + (float)qh * scale < chi[c][a]) ++qh;
            node.qlo[a][c] = (uint8_t)ql;
            node.qhi[a][c] = (uint8_t)qh;
        }
    }
    nodes[level_begin + k] = node;
}

__global__ void k_leaf_tris(const uint32_t* __restrict__ leaf_prims, uint32_t n, const float* __restrict__ world,
                            const uint4* __restrict__ prim_info, float4* __restrict__ tri) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    uint32_t p = leaf_prims[k];
    const float* q = world + 9 * (size_t)p;
    uint32_t flags = prim_info[p].w;
    tri[3 * (size_t)k + 0] = make_float4(q[0], q[1], q[2], __uint_as_float(p));
    tri[3 * (size_t)k + 1] = make_float4(q[3], q[4], q[5], __uint_as_float(flags));
    tri[3 * (size_t)k + 2] = make_float4(q[6], q[7], q[8], 0.0f);
}

__global__ void k_totals(const uint32_t* scan_a, const uint32_t* cnt_a, const uint32_t* scan_b, const uint32_t* cnt_b,
                         uint32_t m, uint32_t* out) {
    if (threadIdx.x == 0) {
        out[0] = scan_a[m - 1] + cnt_a[m - 1];
        out[1] = scan_b[m - 1] + cnt_b[m - 1];
    }
}

inline unsigned blocks_for(size_t n) { return (unsigned)((n + kThreads - 1) / kThreads); }

}  // namespace

// Builds the BVH8 for n world-space triangles (d_world, 9 floats each,
// flattened prim order) into s->d.nodes / s->d.tri and the parity exports.
hx_status hx_build_bvh(hx_context* ctx, hx_scene* s, const float* d_world, uint32_t n) {
    cudaStream_t st = ctx->stream;
    s->info.num_triangles = n;
    if (n == 0) {
        s->d.num_nodes = 0;
        return HX_OK;
    }
    cudaEvent_t e0, e1;
    HX_CUDA(cudaEventCreate(&e0));
    HX_CUDA(cudaEventCreate(&e1));
    HX_CUDA(cudaEventRecord(e0, st));

    auto own = [&](void* p) { s->allocs.push_back(p); };
    uint32_t *morton, *sorted, *children = nullptr, *leaf_prims;
    HX_TRY(hx_alloc_t(ctx, &morton, n)); own(morton);
    HX_TRY(hx_alloc_t(ctx, &sorted, n)); own(sorted);
    HX_TRY(hx_alloc_t(ctx, &leaf_prims, n)); own(leaf_prims);
    uint32_t ni = n - 1;
    if (ni > 0) { HX_TRY(hx_alloc_t(ctx, &children, 2 * (size_t)ni)); own(children); }
    uint32_t max_nodes = n;
    hx_bvh8_node* nodes;
    HX_TRY(hx_alloc_t(ctx, &nodes, max_nodes)); own(nodes);
    float4* tri;
    HX_TRY(hx_alloc_t(ctx, &tri, 3 * (size_t)n)); own(tri);

    // scratch
    size_t scratch_bytes = 0;
    auto carve = [&](size_t bytes) { size_t o = scratch_bytes; scratch_bytes += (bytes + 255) & ~(size_t)255; return o; };
    const uint32_t bnd_blocks = std::min<uint32_t>(1024, (n + kThreads - 1) / kThreads);
    size_t o_partial = carve(6 * sizeof(float) * bnd_blocks), o_bounds = carve(6 * sizeof(float));
    size_t o_keys = carve(4 * (size_t)n), o_vals = carve(4 * (size_t)n), o_keys2 = carve(4 * (size_t)n), o_vals2 = carve(4 * (size_t)n);
    size_t o_sort = carve(hx_radix_temp_bytes(n));
    size_t o_first = carve(4 * (size_t)std::max<uint32_t>(ni, 1)), o_count = carve(4 * (size_t)std::max<uint32_t>(ni, 1));
    size_t o_pint = carve(4 * (size_t)std::max<uint32_t>(ni, 1)), o_pleaf = carve(4 * (size_t)n);
    size_t o_llo = carve(12 * (size_t)n), o_lhi = carve(12 * (size_t)n);
    size_t o_blo = carve(12 * (size_t)std::max<uint32_t>(ni, 1)), o_bhi = carve(12 * (size_t)std::max<uint32_t>(ni, 1));
    size_t o_flags = carve(4 * (size_t)std::max<uint32_t>(ni, 1));
    size_t o_cost = carve(4 * (size_t)std::max<uint32_t>(ni, 1));
    size_t o_queue = carve(4 * (size_t)max_nodes);
    size_t o_plans = carve(sizeof(Plan) * (size_t)max_nodes);
    size_t o_nint = carve(4 * (size_t)max_nodes), o_nleaf = carve(4 * (size_t)max_nodes);
    size_t o_sint = carve(4 * (size_t)max_nodes), o_sleaf = carve(4 * (size_t)max_nodes);
    size_t o_scan = carve(hx_scan_temp_bytes(max_nodes));
    size_t o_tot = carve(16);
    DevBuffer scratch;
    HX_TRY(scratch.reserve(ctx, scratch_bytes));
    char* base = scratch.as<char>();
    float* partial = (float*)(base + o_partial);
    float* bounds = (float*)(base + o_bounds);
    uint32_t* keys = (uint32_t*)(base + o_keys);
    uint32_t* vals = (uint32_t*)(base + o_vals);
    uint32_t* first = (uint32_t*)(base + o_first);
    uint32_t* count = (uint32_t*)(base + o_count);
    int* pint = (int*)(base + o_pint);
    int* pleaf = (int*)(base + o_pleaf);
    float* llo = (float*)(base + o_llo);
    float* lhi = (float*)(base + o_lhi);
    float* blo = (float*)(base + o_blo);
    float* bhi = (float*)(base + o_bhi);
    uint32_t* flags = (uint32_t*)(base + o_flags);
    float* cost = (float*)(base + o_cost);
    uint32_t* queue = (uint32_t*)(base + o_queue);
    Plan* plans = (Plan*)(base + o_plans);
    uint32_t* nint = (uint32_t*)(base + o_nint);
    uint32_t* nleaf = (uint32_t*)(base + o_nleaf);
    uint32_t* sint = (uint32_t*)(base + o_sint);
    uint32_t* sleaf = (uint32_t*)(base + o_sleaf);
    uint32_t* tot = (uint32_t*)(base + o_tot);

    k_centroid_bounds<<<bnd_blocks, kThreads, 0, st>>>(d_world, n, partial);
    k_bounds_final<<<1, 32, 0, st>>>(partial, bnd_blocks, bounds);
    k_morton<<<blocks_for(n), kThreads, 0, st>>>(d_world, n, bounds, morton, keys, vals);
    HX_CUDA(hx_radix_sort_pairs(keys, vals, (uint32_t*)(base + o_keys2), (uint32_t*)(base + o_vals2), n, 30,
                                base + o_sort, st));
    HX_CUDA(cudaMemcpyAsync(sorted, vals, 4 * (size_t)n, cudaMemcpyDeviceToDevice, st));
    HX_CUDA(cudaMemsetAsync(pleaf, 0xff, 4 * (size_t)n, st));
    HX_CUDA(cudaMemsetAsync(tot, 0, 16, st));
    if (ni > 0) {
        HX_CUDA(cudaMemsetAsync(pint, 0xff, 4 * (size_t)ni, st));
        k_karras<<<blocks_for(ni), kThreads, 0, st>>>(keys, (int)n, children, first, count, pint, pleaf);
    }
    k_leaf_boxes<<<blocks_for(n), kThreads, 0, st>>>(d_world, sorted, n, llo, lhi);
    if (ni > 0) {
        HX_CUDA(cudaMemsetAsync(flags, 0, 4 * (size_t)ni, st));
        k_fit<<<blocks_for(n), kThreads, 0, st>>>(n, children, pint, pleaf, llo, lhi, blo, bhi, flags, tot + 2);
        TreeletCtx tc{children, pint, pleaf, llo, lhi, blo, bhi, count, cost};
        for (int pass = 0; pass < kTreeletPasses; ++pass) {
            HX_CUDA(cudaMemsetAsync(flags, 0, 4 * (size_t)ni, st));
            k_treelet<<<blocks_for(n), kThreads, 0, st>>>(n, tc, flags, tot + 2);
        }
    }
    // breadth-first collapse
    uint32_t root = ni > 0 ? 0u : 0x80000000u;
    HX_CUDA(cudaMemcpyAsync(queue, &root, 4, cudaMemcpyHostToDevice, st));
    uint32_t level_begin = 0, level_end = 1, leaf_base = 0;
    while (level_begin < level_end) {
        uint32_t m = level_end - level_begin;
        k_collapse_plan<<<blocks_for(m), kThreads, 0, st>>>(queue, level_begin, m, children, count, blo, bhi, plans, nint, nleaf);
        hx_scan_exclusive_u32(nint, sint, m, base + o_scan, st);
        hx_scan_exclusive_u32(nleaf, sleaf, m, base + o_scan, st);
        k_collapse_emit<<<blocks_for(m), kThreads, 0, st>>>(queue, level_begin, m, level_end, leaf_base, plans, sint, sleaf,
                                                            first, count, sorted, llo, lhi, blo, bhi, nodes, leaf_prims);
        k_totals<<<1, 32, 0, st>>>(sint, nint, sleaf, nleaf, m, tot);
        uint32_t h_tot[3];
        HX_CUDA(cudaMemcpyAsync(h_tot, tot, 12, cudaMemcpyDeviceToHost, st));
        HX_CUDA(cudaStreamSynchronize(st));
        if (h_tot[2]) {
            hx_set_error("BVH build: malformed hierarchy (bottom-up fit exceeded the depth bound)");
            return HX_ERR_DEVICE;
        }
        level_begin = level_end;
        level_end += h_tot[0];
        leaf_base += h_tot[1];
        if (level_end > max_nodes) {
            hx_set_error("BVH8 collapse exceeded node capacity");
            return HX_ERR_DEVICE;
        }
    }
    k_leaf_tris<<<blocks_for(n), kThreads, 0, st>>>(leaf_prims, n, d_world, s->d.prim_info, tri);
    HX_CUDA(cudaEventRecord(e1, st));
    HX_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    HX_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    HX_CUDA(cudaGetLastError());
    scratch.release();

    s->d.nodes = nodes;
    s->d.tri = tri;
    s->d.num_nodes = level_end;
    s->info.num_bvh8_nodes = level_end;
    s->info.num_binary_nodes = ni;
    s->info.build_ms = ms;
    s->morton = morton;
    s->sorted = sorted;
    s->children = children;
    s->leaf_prims = leaf_prims;
    return HX_OK;
}

// World-space triangles for the flattened prims (used before the build).
hx_status hx_world_tris(hx_context* ctx, const DevScene& d, float* world) {
    if (d.num_prims == 0) return HX_OK;
    k_world_tris<<<blocks_for(d.num_prims), kThreads, 0, ctx->stream>>>(d.prim_info, d.indices, d.vtx, d.inst, d.num_prims, world);
    HX_CUDA(cudaGetLastError());
    return HX_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free Morton sort (no counterpart in the reference).
//
// Some callers cannot allocate device memory: an engine or plugin host whose
// own allocator owns every device byte, a process that is not allowed to
// grow its CUDA memory footprint after start-up, or a caller in a
// latency-critical thread that must not take the allocator's locks and
// implicit synchronisation.  hx_lbvh_sort_noalloc gives them the Morton-code
// + stable-sort stage of the LBVH build without any cudaMalloc: inputs and
// outputs are the caller's device buffers, and every scratch byte lives in
// the fixed array below, which each GPU that loads this library holds until
// the process exits.
//
// The array is shared by all calls on a device and keeps the contents of the
// last call; nothing in it needs to start at zero (every pass writes the
// parts it reads).  Calls whose work overlaps on the GPU (different streams,
// or different host threads without ordering) race on it.
// ---------------------------------------------------------------------------
namespace {

constexpr uint32_t kNoAllocMaxTriangles = 1u << 18;
constexpr uint32_t kNoAllocBoundsBlocks = 1024;

constexpr size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// scratch layout: bound partials | bounds | keys | vals | keys2 | vals2 | radix temp
constexpr size_t kNoAllocOffPartial = 0;
constexpr size_t kNoAllocOffBounds = kNoAllocOffPartial + align256(6 * sizeof(float) * kNoAllocBoundsBlocks);
constexpr size_t kNoAllocOffKeys = kNoAllocOffBounds + align256(6 * sizeof(float));
constexpr size_t kNoAllocOffVals = kNoAllocOffKeys + align256(4 * (size_t)kNoAllocMaxTriangles);
constexpr size_t kNoAllocOffKeys2 = kNoAllocOffVals + align256(4 * (size_t)kNoAllocMaxTriangles);
constexpr size_t kNoAllocOffVals2 = kNoAllocOffKeys2 + align256(4 * (size_t)kNoAllocMaxTriangles);
constexpr size_t kNoAllocOffRadix = kNoAllocOffVals2 + align256(4 * (size_t)kNoAllocMaxTriangles);
// radix temp for 2^18 keys: 64 tiles -> 2 x 256 x 64 words + scan temp; 1 MiB covers it
constexpr size_t kNoAllocRadixBytes = 1u << 20;
constexpr size_t kNoAllocScratchBytes = kNoAllocOffRadix + kNoAllocRadixBytes;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

}  // namespace

extern "C" hx_status hx_lbvh_sort_noalloc(const float* d_world_tris, uint32_t n, uint32_t* d_morton,
                                          uint32_t* d_sorted, void* cuda_stream) {
    HX_CHECK_ARG(d_world_tris && d_morton && d_sorted, "hx_lbvh_sort_noalloc: null device pointer");
    HX_CHECK_ARG(n >= 1 && n <= kNoAllocMaxTriangles,
                 "hx_lbvh_sort_noalloc: %u triangles; this entry point handles 1..%u (its scratch is a fixed %zu-byte "
                 "device array)", n, kNoAllocMaxTriangles, (size_t)kNoAllocScratchBytes);
    HX_CHECK_ARG(hx_radix_temp_bytes(n) <= kNoAllocRadixBytes, "hx_lbvh_sort_noalloc: radix scratch too small");
    // the array's address on the current device, looked up on every call (a host-side table lookup, no
    // allocation) so that it stays right after a cudaDeviceReset reloads the module
    void* base = nullptr;
    {
        cudaError_t e = cudaGetSymbolAddress(&base, g_noalloc_scratch);
        if (e != cudaSuccess) {
            hx_set_error("hx_lbvh_sort_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
            return HX_ERR_DEVICE;
        }
    }
    cudaStream_t st = (cudaStream_t)cuda_stream;
    char* b = (char*)base;
    float* partial = (float*)(b + kNoAllocOffPartial);
    float* bounds = (float*)(b + kNoAllocOffBounds);
    uint32_t* keys = (uint32_t*)(b + kNoAllocOffKeys);
    uint32_t* vals = (uint32_t*)(b + kNoAllocOffVals);
    const uint32_t bnd_blocks = std::min<uint32_t>(kNoAllocBoundsBlocks, (n + kThreads - 1) / kThreads);
    k_centroid_bounds<<<bnd_blocks, kThreads, 0, st>>>(d_world_tris, n, partial);
    k_bounds_final<<<1, 32, 0, st>>>(partial, bnd_blocks, bounds);
    k_morton<<<blocks_for(n), kThreads, 0, st>>>(d_world_tris, n, bounds, d_morton, keys, vals);
    HX_CUDA(hx_radix_sort_pairs(keys, vals, (uint32_t*)(b + kNoAllocOffKeys2), (uint32_t*)(b + kNoAllocOffVals2), n,
                                30, b + kNoAllocOffRadix, st));
    HX_CUDA(cudaMemcpyAsync(d_sorted, vals, 4 * (size_t)n, cudaMemcpyDeviceToDevice, st));
    HX_CUDA(cudaGetLastError());
    return HX_OK;
}
