// sort.cu — device-wide exclusive scan and stable LSD radix sort (uint32
// key/value pairs).  Used by the LBVH build (Morton-code sort) and the
// BVH8 collapse (per-level allocation scans).
//
// Radix sort: 8-bit digits, one pass per digit.  Each pass: a per-tile
// digit histogram (tile = 256 threads x 16 keys), a device-wide exclusive
// scan of the digit-major histogram table (digit d of tile t lands at
// hist[d * tiles + t], so the scan yields global scatter offsets), and a
// stable scatter that ranks keys inside the tile with warp match masks.
#include "hx_internal.h"

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;  // 1024

constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortThreads * kSortItems;  // 4096

__device__ __forceinline__ uint32_t warp_exclusive_scan(uint32_t v, uint32_t& total) {
    const int lane = threadIdx.x & 31;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    total = __shfl_sync(0xffffffffu, x, 31);
    return x - v;
}

__global__ void k_scan_tiles(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, size_t n,
                             uint32_t* __restrict__ tile_sums) {
    __shared__ uint32_t s_warp[kScanThreads / 32];
    const size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t sum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = (base + k < n) ? in[base + k] : 0u;
        sum += v[k];
    }
    uint32_t wtotal;
    uint32_t excl = warp_exclusive_scan(sum, wtotal);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 31) s_warp[warp] = wtotal;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < kScanThreads / 32 ? s_warp[lane] : 0u;
        uint32_t t;
        uint32_t e = warp_exclusive_scan(w, t);
        if (lane < kScanThreads / 32) s_warp[lane] = e;
        if (lane == 0 && tile_sums) tile_sums[blockIdx.x] = t;
    }
    __syncthreads();
    uint32_t run = excl + s_warp[warp];
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
}

__global__ void k_scan_add(uint32_t* __restrict__ out, size_t n, const uint32_t* __restrict__ offsets) {
    const size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanItems;
    const uint32_t add = offsets[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; ++k)
        if (base + k < n) out[base + k] += add;
}

__global__ void k_radix_hist(const uint32_t* __restrict__ keys, size_t n, int shift, uint32_t* __restrict__ hist,
                             uint32_t tiles) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const size_t base = (size_t)blockIdx.x * kSortTile;
#pragma unroll 4
    for (int k = 0; k < kSortItems; ++k) {
        size_t i = base + (size_t)k * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 0xffu], 1u);
    }
    __syncthreads();
    hist[(size_t)threadIdx.x * tiles + blockIdx.x] = h[threadIdx.x];
}

__global__ void k_radix_scatter(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin,
                                uint32_t* __restrict__ kout, uint32_t* __restrict__ vout, size_t n, int shift,
                                const uint32_t* __restrict__ offsets, uint32_t tiles) {
    __shared__ uint32_t s_base[256];
    __shared__ uint32_t s_warp[kSortThreads / 32][256];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    s_base[tid] = offsets[(size_t)tid * tiles + blockIdx.x];
    const uint32_t lanemask_lt = (1u << lane) - 1u;
    const size_t base = (size_t)blockIdx.x * kSortTile;
    for (int r = 0; r < kSortItems; ++r) {
#pragma unroll
        for (int w = 0; w < kSortThreads / 32; ++w) s_warp[w][tid] = 0;
        __syncthreads();
        size_t i = base + (size_t)r * kSortThreads + tid;
        bool valid = i < n;
        uint32_t key = valid ? kin[i] : 0u;
        uint32_t digit = valid ? ((key >> shift) & 0xffu) : 256u;
        uint32_t peers = __match_any_sync(0xffffffffu, digit);
        uint32_t rank = __popc(peers & lanemask_lt);
        if (valid && rank == 0) s_warp[warp][digit] = __popc(peers);
        __syncthreads();
        uint32_t run = s_base[tid];
#pragma unroll
        for (int w = 0; w < kSortThreads / 32; ++w) {
            uint32_t c = s_warp[w][tid];
            s_warp[w][tid] = run;
            run += c;
        }
        s_base[tid] = run;
        __syncthreads();
        if (valid) {
            uint32_t pos = s_warp[warp][digit] + rank;
            kout[pos] = key;
            vout[pos] = vin[i];
        }
        __syncthreads();
    }
}

}  // namespace

size_t hx_scan_temp_bytes(size_t n) {
    size_t bytes = 0;
    size_t m = n;
    while (m > (size_t)kScanTile) {
        m = (m + kScanTile - 1) / kScanTile;
        bytes += 2 * m * sizeof(uint32_t);
    }
    return bytes + 256;
}

void hx_scan_exclusive_u32(const uint32_t* in, uint32_t* out, size_t n, void* temp, cudaStream_t st) {
    if (n == 0) return;
    size_t blocks = (n + kScanTile - 1) / kScanTile;
    if (blocks == 1) {
        k_scan_tiles<<<1, kScanThreads, 0, st>>>(in, out, n, nullptr);
        return;
    }
    uint32_t* sums = (uint32_t*)temp;
    uint32_t* scanned = sums + blocks;
    k_scan_tiles<<<(unsigned)blocks, kScanThreads, 0, st>>>(in, out, n, sums);
    hx_scan_exclusive_u32(sums, scanned, blocks, scanned + blocks, st);
    k_scan_add<<<(unsigned)blocks, kScanThreads, 0, st>>>(out, n, scanned);
}

size_t hx_radix_temp_bytes(size_t n) {
    size_t tiles = (n + kSortTile - 1) / kSortTile;
    size_t hist = 256 * tiles;
    return 2 * hist * sizeof(uint32_t) + hx_scan_temp_bytes(hist) + 256;
}

cudaError_t hx_radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t* keys_tmp, uint32_t* vals_tmp, size_t n,
                                int bits, void* temp, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    uint32_t tiles = (uint32_t)((n + kSortTile - 1) / kSortTile);
    size_t hist_n = (size_t)256 * tiles;
    uint32_t* hist = (uint32_t*)temp;
    uint32_t* offs = hist + hist_n;
    void* scan_tmp = offs + hist_n;
    uint32_t *ka = keys, *va = vals, *kb = keys_tmp, *vb = vals_tmp;
    int passes = (bits + 7) / 8;
    for (int p = 0; p < passes; ++p) {
        int shift = 8 * p;
        k_radix_hist<<<tiles, kSortThreads, 0, st>>>(ka, n, shift, hist, tiles);
        hx_scan_exclusive_u32(hist, offs, hist_n, scan_tmp, st);
        k_radix_scatter<<<tiles, kSortThreads, 0, st>>>(ka, va, kb, vb, n, shift, offs, tiles);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        std::swap(ka, kb);
        std::swap(va, vb);
    }
    if (ka != keys) {  // an odd number of passes ends in the temporary arrays
        cudaError_t e = cudaMemcpyAsync(keys, ka, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(vals, va, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st);
        return e;
    }
    return cudaSuccess;
}
