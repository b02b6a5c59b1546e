// hx_internal.h — internal types of the helios-gb300 core (host + device).
#pragma once

#include "../../include/hx.h"

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

// ---------------------------------------------------------------------------
// Errors: thread-local last error string, status codes across the ABI.
// ---------------------------------------------------------------------------
void hx_set_error(const char* fmt, ...);

#define HX_CHECK_ARG(cond, ...)                  \
    do {                                         \
        if (!(cond)) {                           \
            hx_set_error(__VA_ARGS__);           \
            return HX_ERR_INVALID_ARG;           \
        }                                        \
    } while (0)

#define HX_CUDA(call)                                                                                  \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess) {                                                                       \
            hx_set_error("%s:%d: %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_));          \
            return HX_ERR_DEVICE;                                                                      \
        }                                                                                              \
    } while (0)

#define HX_TRY(call)                      \
    do {                                  \
        hx_status s_ = (call);            \
        if (s_ != HX_OK) return s_;       \
    } while (0)

// ---------------------------------------------------------------------------
// Context: device, stream, HBM budget (the role of vk::Backend + VMA).
// ---------------------------------------------------------------------------
struct hx_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    uint64_t budget = 0;  // bytes
    uint64_t used = 0;
    std::mutex mu;
    std::unordered_map<void*, size_t> sizes;
    int num_sms = 0;
};

// Budgeted device allocation; returns HX_ERR_OOM_BUDGET when it would exceed
// the context budget.
hx_status hx_alloc(hx_context* ctx, void** ptr, size_t bytes);
void hx_free(hx_context* ctx, void* ptr);

template <typename T> static inline hx_status hx_alloc_t(hx_context* ctx, T** p, size_t count) {
    return hx_alloc(ctx, (void**)p, count * sizeof(T));
}

// Scratch region (device) reused by kernels of one call.
struct DevBuffer {
    hx_context* ctx = nullptr;
    void* ptr = nullptr;
    size_t bytes = 0;
    hx_status reserve(hx_context* c, size_t b) {
        if (b <= bytes) return HX_OK;
        release();
        ctx = c;
        hx_status s = hx_alloc(c, &ptr, b);
        if (s == HX_OK) bytes = b;
        return s;
    }
    void release() {
        if (ptr && ctx) hx_free(ctx, ptr);
        ptr = nullptr;
        bytes = 0;
    }
    template <typename T> T* as() const { return (T*)ptr; }
};

// ---------------------------------------------------------------------------
// Device scene layout.
// ---------------------------------------------------------------------------
struct DevInstance {       // 144 B: model, normal matrix (column-major), mesh info
    float model[16];
    float normal[16];
    uint32_t mesh_index;
    uint32_t mesh_tri_base;  // first triangle of the mesh in the global index buffer
    uint32_t pad[2];
};

struct DevEnv {
    uint32_t kind, width, height, pad;
    const __half* rgb;    // 4 halves per texel (rgb + 0)
    const float* marg;    // height + 1, normalised to [0, 1]
    const float* cond;    // height * (width + 1), each row normalised to [0, 1]
    const float* rowsum;  // height: row weight / total (for the pdf)
    const float* cellw;   // height * width: texel weight / row weight
    float total;
    // Guide tables of the two CDF searches: for bucket b of a power-of-two
    // count K, the search result at b / K, so a value in [b / K, (b + 1) / K)
    // is searched only between entries b and b + 1 (the same index as the
    // full search).  marg_guide: km + 1 entries; cond_guide: height rows of
    // kc + 1 entries.
    const uint32_t* marg_guide;
    const uint32_t* cond_guide;
    uint32_t km, kc;
};

// Entries of a ray's traversal stack (8-byte node groups, in local memory).
constexpr uint32_t kTraversalStackEntries = 32;

struct DevScene {
    uint32_t num_prims, num_nodes, num_lights, num_instances;
    uint32_t stack_limit;        // traversal stack entries a ray may use (<= kStackSize; a diagnostic knob)
    uint32_t wide_alpha;         // 1: some alpha-tested albedo texture is RGBA16F / SNORM (traversal's WA kernels)
    const float4* tri;           // 3 per leaf-ordered triangle: v0.xyz|prim, v1.xyz|flags, v2.xyz|0
    const hx_bvh8_node* nodes;
    const uint4* prim_info;      // per flattened prim: instance, global tri, material, flags
    const uint32_t* indices;     // global index buffer (absolute vertex ids)
    const float4* vtx;           // 2 per vertex: pos.xyz|u, normal.xyz|v
    const float4* vtx_tb;        // 2 per vertex: tangent.xyz|0, bitangent.xyz|0 (only with normal maps)
    const float* srgb_lut;       // 256 entries: sRGB byte -> linear (texture flag bit 0 of tex_desc.w)
    const float* vtx_w;          // position.w per vertex
    const DevInstance* inst;
    const hx_material* materials;
    const hx_light* lights;
    const uint4* tex_desc;       // per texture: texel offset, width, height, flags (bit 0: sRGB)
    const uint32_t* texels;      // RGBA8 packed
    const uint8_t* alpha8;       // alpha channel of every texture (same texel offsets): the any-hit test's working set
    const float4* alpha_uv;      // 2 per flattened prim: (u0,v0,u1,v1), (u2,v2,tex,0)
    DevEnv env;
};

#define HX_TRI_NONOPAQUE 1u

struct hx_scene {
    hx_context* ctx = nullptr;
    DevScene d{};
    hx_scene_info info{};
    std::vector<hx_light> lights_host;
    // owned allocations
    std::vector<void*> allocs;
    // parity exports (device)
    uint32_t* morton = nullptr;
    uint32_t* sorted = nullptr;
    uint32_t* children = nullptr;
    uint32_t* leaf_prims = nullptr;
};

// BVH build (bvh_build.cu)
hx_status hx_build_bvh(hx_context* ctx, hx_scene* s, const float* d_world /*9 per prim*/, uint32_t n);

// Environment bake (scene.cu)
hx_status hx_env_build(hx_context* ctx, hx_scene* s, const hx_environment_desc& e);

// Device-wide exclusive scan of uint32 (scan.cu); temp must hold
// hx_scan_temp_bytes(n) bytes.
size_t hx_scan_temp_bytes(size_t n);
void hx_scan_exclusive_u32(const uint32_t* in, uint32_t* out, size_t n, void* temp, cudaStream_t st);

// Stable LSD radix sort of (key, value) pairs on the low `bits` bits.
size_t hx_radix_temp_bytes(size_t n);
cudaError_t hx_radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t* keys_tmp, uint32_t* vals_tmp, size_t n, int bits,
                         void* temp, cudaStream_t st);
