// scene.cu — scene upload (replaces Scene::create_gpu_resources,
// src/engine/resource/scene.cpp:915-1311): flattened triangle list,
// device vertex/index/material/instance/light buffers, textures, the
// environment (Hosek-Wilkie bake or caller lat-long map) with its
// importance-sampling CDF, and the BVH build.
#include "devmath.cuh"
#include "hx_internal.h"

#include <algorithm>
#include <cmath>
#include <cstring>

hx_status hx_world_tris(hx_context* ctx, const DevScene& d, float* world);

namespace {

constexpr float kPi = 3.14159265358979323846f;

// Hosek-Wilkie RGB radiance (procedural_sky.frag:48-75) for direction v.
__device__ V3 hosek(const float* c, V3 v, V3 sun) {
    float cos_theta = gclamp(v.y, 0.0f, 1.0f);
    float cos_gamma = gclamp(dot(v, sun), 0.0f, 1.0f);
    float gamma = acosf(cos_gamma);
    float out[3];
    for (int k = 0; k < 3; ++k) {
        float A = c[0 + k], B = c[4 + k], C = c[8 + k], D = c[12 + k], E = c[16 + k], F = c[20 + k], G = c[24 + k],
              H = c[28 + k], I = c[32 + k], Z = c[36 + k];
        float chi = (1.0f + cos_gamma * cos_gamma) / powf(1.0f + H * H - 2.0f * cos_gamma * H, 1.5f);
        float hw = (1.0f + A * expf(B / (cos_theta + 0.01f))) *
                   (C + D * expf(E * gamma) + F * (cos_gamma * cos_gamma) + G * chi + I * sqrtf(cos_theta));
        out[k] = Z * hw;
    }
    return v3(out[0], out[1], out[2]);
}

struct SkyParams {
    float c[40];
    float sun[3];
};

// Bakes the sky into the lat-long map: texel centre (i+0.5, j+0.5),
// phi = 2 pi (u - 0.5), theta = pi v, d = (sin t sin p, cos t, -sin t cos p).
__global__ void k_sky_bake(SkyParams sp, uint32_t w, uint32_t h, __half* out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i >= w) return;
    float u = ((float)i + 0.5f) / (float)w, v = ((float)j + 0.5f) / (float)h;
    float phi = 2.0f * kPi * (u - 0.5f), theta = kPi * v;
    float st = sinf(theta);
    V3 d = v3(st * sinf(phi), cosf(theta), -st * cosf(phi));
    V3 r = hosek(sp.c, d, v3(sp.sun[0], sp.sun[1], sp.sun[2]));
    __half* o = out + 4 * ((size_t)j * w + i);
    o[0] = __float2half_rn(r.x);
    o[1] = __float2half_rn(r.y);
    o[2] = __float2half_rn(r.z);
    o[3] = __float2half_rn(0.0f);
}

__global__ void k_env_from_rgba32f(const float* in, size_t n, __half* out) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int c = 0; c < 3; ++c) out[4 * i + c] = __float2half_rn(in[4 * i + c]);
    out[4 * i + 3] = __float2half_rn(0.0f);
}

__device__ __forceinline__ float texel_lum(const __half* e, size_t k) {
    return 0.2126f * __half2float(e[4 * k]) + 0.7152f * __half2float(e[4 * k + 1]) + 0.0722f * __half2float(e[4 * k + 2]);
}

// Per-row luminance sums (one block per row).
__global__ void k_env_row_lum(const __half* env, uint32_t w, float* rowlum) {
    __shared__ float s[256];
    uint32_t j = blockIdx.x;
    float acc = 0.0f;
    for (uint32_t i = threadIdx.x; i < w; i += blockDim.x) acc += texel_lum(env, (size_t)j * w + i);
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) rowlum[j] = s[0];
}

// Conditional CDF per row: weights (lum + floor) * sin(theta_j), inclusive
// prefix normalised to 1; row total into rowsum (one block per row; each
// thread scans a contiguous chunk, then the chunk totals are scanned).
__global__ void k_env_rows(const __half* env, uint32_t w, uint32_t h, const float* rowlum, float* cond, float* rowsum) {
    __shared__ float s[256];
    __shared__ float s_floor;
    uint32_t j = blockIdx.x;
    if (threadIdx.x == 0) {
        float tot = 0.0f;
        for (uint32_t r = 0; r < h; ++r) tot += rowlum[r];
        s_floor = 1e-3f * tot / ((float)w * (float)h) + 1e-12f;
    }
    __syncthreads();
    float st = sinf(kPi * ((float)j + 0.5f) / (float)h);
    uint32_t chunk = (w + blockDim.x - 1) / blockDim.x;
    uint32_t i0 = threadIdx.x * chunk, i1 = min(w, i0 + chunk);
    float local = 0.0f;
    for (uint32_t i = i0; i < i1; ++i) local += (texel_lum(env, (size_t)j * w + i) + s_floor) * st;
    s[threadIdx.x] = local;
    __syncthreads();
    if (threadIdx.x == 0) {
        float run = 0.0f;
        for (uint32_t t = 0; t < blockDim.x; ++t) { float x = s[t]; s[t] = run; run += x; }
        rowsum[j] = run;
    }
    __syncthreads();
    float* row = cond + (size_t)j * (w + 1);
    float total = rowsum[j];
    float run = s[threadIdx.x];
    if (threadIdx.x == 0) row[0] = 0.0f;
    for (uint32_t i = i0; i < i1; ++i) {
        run += (texel_lum(env, (size_t)j * w + i) + s_floor) * st;
        row[i + 1] = total > 0.0f ? run / total : (float)(i + 1) / (float)w;
    }
    __syncthreads();
    if (threadIdx.x == 0) row[w] = 1.0f;
}

__global__ void k_env_marg(const float* rowsum, uint32_t h, float* marg, float* total_out) {
    if (threadIdx.x != 0) return;
    float tot = 0.0f;
    for (uint32_t j = 0; j < h; ++j) tot += rowsum[j];
    float run = 0.0f;
    marg[0] = 0.0f;
    for (uint32_t j = 0; j < h; ++j) {
        run += rowsum[j];
        marg[j + 1] = tot > 0.0f ? run / tot : (float)(j + 1) / (float)h;
    }
    marg[h] = 1.0f;
    *total_out = tot;
}

bool material_emissive(const hx_material& m) {  // Material::is_emissive, material.cpp:71-77
    if (m.texture_indices1[0] != -1) return true;
    return m.emissive[0] > 0.0f || m.emissive[1] > 0.0f || m.emissive[2] > 0.0f;
}

// Guide table of a search over n + 1 ascending CDF entries a[0..n] (search
// range [1, n + 1)): entry b in [0, k] is the search result at b / k (exact:
// k is a power of two).  rows > 1: one table per row of stride n + 1.
__global__ void k_env_guide(const float* __restrict__ a, uint32_t n, uint32_t rows, uint32_t k, uint32_t* __restrict__ g) {
    const size_t total = (size_t)rows * (k + 1);
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const uint32_t r = (uint32_t)(t / (k + 1)), b = (uint32_t)(t % (k + 1));
        const float x = (float)b * (1.0f / (float)k);
        g[t] = (uint32_t)upper_bound_f(a + (size_t)r * (n + 1), 1, (int)n + 1, x);
    }
}

}  // namespace

static uint32_t pow2_at_least(uint32_t v) {
    uint32_t k = 1;
    while (k < v) k <<= 1;
    return k;
}

hx_status hx_env_build(hx_context* ctx, hx_scene* s, const hx_environment_desc& e) {
    DevEnv& env = s->d.env;
    env.kind = e.kind;
    if (e.kind == HX_ENV_NONE) return HX_OK;
    HX_CHECK_ARG(e.width >= 2 && e.height >= 2 && e.width <= 16384 && e.height <= 16384, "environment: bad size %ux%u",
                 e.width, e.height);
    cudaStream_t st = ctx->stream;
    uint32_t w = e.width, h = e.height;
    env.width = w;
    env.height = h;
    __half* rgb;
    float *cond, *marg, *rowsum, *rowlum, *total;
    HX_TRY(hx_alloc_t(ctx, &rgb, 4 * (size_t)w * h)); s->allocs.push_back(rgb);
    HX_TRY(hx_alloc_t(ctx, &cond, (size_t)h * (w + 1))); s->allocs.push_back(cond);
    HX_TRY(hx_alloc_t(ctx, &marg, (size_t)h + 1)); s->allocs.push_back(marg);
    HX_TRY(hx_alloc_t(ctx, &rowsum, (size_t)h)); s->allocs.push_back(rowsum);
    HX_TRY(hx_alloc_t(ctx, &rowlum, (size_t)h)); s->allocs.push_back(rowlum);
    HX_TRY(hx_alloc_t(ctx, &total, 4)); s->allocs.push_back(total);
    if (e.kind == HX_ENV_HOSEK_WILKIE) {
        SkyParams sp;
        std::memcpy(sp.c, e.coeffs, sizeof(sp.c));
        for (int a = 0; a < 3; ++a) sp.sun[a] = e.sun_direction[a];
        dim3 grid((w + 255) / 256, h);
        k_sky_bake<<<grid, 256, 0, st>>>(sp, w, h, rgb);
    } else if (e.kind == HX_ENV_EQUIRECT) {
        HX_CHECK_ARG(e.rgba32f != nullptr, "environment: null lat-long data");
        DevBuffer tmp;
        size_t n = (size_t)w * h;
        HX_TRY(tmp.reserve(ctx, 16 * n));
        HX_CUDA(cudaMemcpyAsync(tmp.ptr, e.rgba32f, 16 * n, cudaMemcpyHostToDevice, st));
        k_env_from_rgba32f<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(tmp.as<float>(), n, rgb);
        HX_CUDA(cudaStreamSynchronize(st));
        tmp.release();
    } else {
        hx_set_error("environment: unknown kind %u", e.kind);
        return HX_ERR_INVALID_ARG;
    }
    k_env_row_lum<<<h, 256, 0, st>>>(rgb, w, rowlum);
    k_env_rows<<<h, 256, 0, st>>>(rgb, w, h, rowlum, cond, rowsum);
    k_env_marg<<<1, 32, 0, st>>>(rowsum, h, marg, total);
    env.km = pow2_at_least(h);
    env.kc = pow2_at_least(w);
    uint32_t *mg, *cg;
    HX_TRY(hx_alloc_t(ctx, &mg, (size_t)env.km + 1)); s->allocs.push_back(mg);
    HX_TRY(hx_alloc_t(ctx, &cg, (size_t)h * (env.kc + 1))); s->allocs.push_back(cg);
    k_env_guide<<<(env.km + 256) / 256, 256, 0, st>>>(marg, h, 1, env.km, mg);
    k_env_guide<<<(unsigned)std::min<size_t>(((size_t)h * (env.kc + 1) + 255) / 256, 65535), 256, 0, st>>>(cond, w, h, env.kc, cg);
    env.marg_guide = mg;
    env.cond_guide = cg;
    HX_CUDA(cudaGetLastError());
    env.rgb = rgb;
    env.cond = cond;
    env.marg = marg;
    env.rowsum = rowsum;
    env.cellw = nullptr;
    env.total = 0.0f;
    return HX_OK;
}

// Alpha channel copy of the RGBA8 texels: the alpha test reads one byte per
// texel instead of four (a quarter of the cache footprint).
__global__ void k_alpha8(const uint32_t* __restrict__ texels, size_t n, uint8_t* __restrict__ alpha8) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        alpha8[i] = (uint8_t)(texels[i] >> 24);
}

static hx_status scene_fail(hx_scene* s, hx_status st) {
    hx_scene_destroy(s);
    return st;
}

extern "C" hx_status hx_scene_upload(hx_context* ctx, const hx_scene_desc* desc, hx_scene** out) {
    HX_CHECK_ARG(ctx && desc && out, "hx_scene_upload: null argument");
    HX_CUDA(cudaSetDevice(ctx->device));
    // ---- validation (the reference trusted its loaders; here bad input is an error)
    for (uint32_t m = 0; m < desc->num_meshes; ++m) {
        const hx_mesh_desc& md = desc->meshes[m];
        HX_CHECK_ARG(md.vertices || md.num_vertices == 0, "mesh %u: null vertices", m);
        HX_CHECK_ARG(md.indices || md.num_indices == 0, "mesh %u: null indices", m);
        HX_CHECK_ARG(md.num_indices % 3 == 0, "mesh %u: index count %u not a multiple of 3", m, md.num_indices);
        for (uint32_t i = 0; i < md.num_indices; ++i)
            HX_CHECK_ARG(md.indices[i] < md.num_vertices, "mesh %u: index %u out of range", m, md.indices[i]);
        for (uint32_t k = 0; k < md.num_submeshes; ++k) {
            const hx_submesh& sm = md.submeshes[k];
            HX_CHECK_ARG(sm.base_index % 3 == 0 && sm.index_count % 3 == 0 &&
                             (uint64_t)sm.base_index + sm.index_count <= md.num_indices,
                         "mesh %u submesh %u: bad index range", m, k);
            HX_CHECK_ARG(sm.material < desc->num_materials, "mesh %u submesh %u: material out of range", m, k);
        }
    }
    for (uint32_t i = 0; i < desc->num_instances; ++i) {
        HX_CHECK_ARG(desc->instances[i].mesh_index < desc->num_meshes, "instance %u: mesh out of range", i);
        HX_CHECK_ARG(desc->instances[i].material_override < (int32_t)desc->num_materials, "instance %u: material override out of range", i);
    }
    for (uint32_t k = 0; k < desc->num_materials; ++k) {
        const hx_material& mt = desc->materials[k];
        for (int a = 0; a < 4; ++a) {
            HX_CHECK_ARG(mt.texture_indices0[a] < (int32_t)desc->num_textures, "material %u: texture out of range", k);
        }
        HX_CHECK_ARG(mt.texture_indices1[0] < (int32_t)desc->num_textures, "material %u: texture out of range", k);
    }
    for (uint32_t t = 0; t < desc->num_textures; ++t) {
        HX_CHECK_ARG(desc->textures[t].rgba8 && desc->textures[t].width > 0 && desc->textures[t].height > 0,
                     "texture %u: empty", t);
        HX_CHECK_ARG(desc->textures[t].format <= HX_TEXTURE_RGBA8_SNORM, "texture %u: unknown format %u", t,
                     desc->textures[t].format);
        HX_CHECK_ARG((desc->textures[t].format < HX_TEXTURE_BC6H_SF16) || !desc->textures[t].srgb,
                     "texture %u: half-float and SNORM formats have no sRGB variant", t);
    }
    for (uint32_t l = 0; l < desc->num_punctual_lights; ++l) {
        uint32_t ty = (uint32_t)desc->punctual_lights[l].data0[0];
        HX_CHECK_ARG(ty == HX_LIGHT_DIRECTIONAL || ty == HX_LIGHT_POINT || ty == HX_LIGHT_SPOT,
                     "punctual light %u: type %u is not directional/point/spot", l, ty);
    }

    hx_scene* s = new hx_scene();
    s->ctx = ctx;
    s->d.stack_limit = kTraversalStackEntries;
    s->d.wide_alpha = 0;
    cudaStream_t st = ctx->stream;
    // ---- host packing
    std::vector<uint32_t> vbase(desc->num_meshes), tbase(desc->num_meshes);
    size_t nv = 0, ni = 0;
    for (uint32_t m = 0; m < desc->num_meshes; ++m) {
        vbase[m] = (uint32_t)nv;
        tbase[m] = (uint32_t)(ni / 3);
        nv += desc->meshes[m].num_vertices;
        ni += desc->meshes[m].num_indices;
    }
    bool normal_maps = false;
    for (uint32_t k = 0; k < desc->num_materials; ++k) normal_maps |= desc->materials[k].texture_indices0[1] != -1;
    std::vector<float4> hv(2 * nv);
    std::vector<float4> htb(normal_maps ? 2 * nv : 0);
    std::vector<float> hw(nv);
    std::vector<uint32_t> hidx(ni);
    for (uint32_t m = 0; m < desc->num_meshes; ++m) {
        const hx_mesh_desc& md = desc->meshes[m];
        for (uint32_t v = 0; v < md.num_vertices; ++v) {
            const hx_vertex& x = md.vertices[v];
            hv[2 * (vbase[m] + v)] = make_float4(x.position[0], x.position[1], x.position[2], x.tex_coord[0]);
            hv[2 * (vbase[m] + v) + 1] = make_float4(x.normal[0], x.normal[1], x.normal[2], x.tex_coord[1]);
            hw[vbase[m] + v] = x.position[3];
            if (normal_maps) {
                htb[2 * (vbase[m] + v)] = make_float4(x.tangent[0], x.tangent[1], x.tangent[2], 0.0f);
                htb[2 * (vbase[m] + v) + 1] = make_float4(x.bitangent[0], x.bitangent[1], x.bitangent[2], 0.0f);
            }
        }
        for (uint32_t i = 0; i < md.num_indices; ++i) hidx[(size_t)tbase[m] * 3 + i] = vbase[m] + md.indices[i];
    }
    std::vector<DevInstance> hinst(desc->num_instances);
    size_t nprims = 0;
    for (uint32_t i = 0; i < desc->num_instances; ++i) {
        const hx_instance& in = desc->instances[i];
        std::memcpy(hinst[i].model, in.model_matrix, 64);
        std::memcpy(hinst[i].normal, in.normal_matrix, 64);
        hinst[i].mesh_index = in.mesh_index;
        hinst[i].mesh_tri_base = tbase[in.mesh_index];
        for (uint32_t k = 0; k < desc->meshes[in.mesh_index].num_submeshes; ++k)
            nprims += desc->meshes[in.mesh_index].submeshes[k].index_count / 3;
    }
    if (nprims >= 0x7fffffffull) { delete s; hx_set_error("too many triangles"); return HX_ERR_INVALID_ARG; }
    std::vector<uint4> hpi(nprims);
    std::vector<float4> hauv(2 * nprims);
    size_t p = 0;
    for (uint32_t ii = 0; ii < desc->num_instances; ++ii) {
        const hx_instance& in = desc->instances[ii];
        const hx_mesh_desc& md = desc->meshes[in.mesh_index];
        for (uint32_t k = 0; k < md.num_submeshes; ++k) {
            const hx_submesh& sm = md.submeshes[k];
            uint32_t mat = in.material_override >= 0 ? (uint32_t)in.material_override : sm.material;
            const hx_material& mt = desc->materials[mat];
            uint32_t flags = (sm.flags & HX_SUBMESH_NON_OPAQUE) ? HX_TRI_NONOPAQUE : 0u;
            for (uint32_t t = 0; t < sm.index_count / 3; ++t, ++p) {
                uint32_t mp = sm.base_index / 3 + t;
                hpi[p] = make_uint4(ii, tbase[in.mesh_index] + mp, mat, flags);
                const hx_vertex& a = md.vertices[md.indices[3 * mp]];
                const hx_vertex& b = md.vertices[md.indices[3 * mp + 1]];
                const hx_vertex& c = md.vertices[md.indices[3 * mp + 2]];
                // albedo texture index for the any-hit test; bit 31 marks an
                // RGBA16F / SNORM texture (alpha read without the A8 copy)
                uint32_t tex = 0xffffffffu;
                if (mt.texture_indices0[0] >= 0) {
                    const uint32_t f = desc->textures[mt.texture_indices0[0]].format;
                    const bool wide = f >= HX_TEXTURE_BC6H_SF16;
                    tex = (uint32_t)mt.texture_indices0[0] | (wide ? 0x80000000u : 0u);
                    if (wide && flags) s->d.wide_alpha = 1u;  // an alpha-tested triangle reads it
                }
                float tex_f;
                std::memcpy(&tex_f, &tex, 4);
                hauv[2 * p] = make_float4(a.tex_coord[0], a.tex_coord[1], b.tex_coord[0], b.tex_coord[1]);
                hauv[2 * p + 1] = make_float4(c.tex_coord[0], c.tex_coord[1], tex_f, mt.albedo[3]);
            }
        }
    }
    // light list in reference order (scene.cpp:1111-1119, 1269-1309)
    {
        std::vector<uint8_t> seen(desc->num_meshes, 0);
        for (uint32_t ii = 0; ii < desc->num_instances; ++ii) {
            const hx_instance& in = desc->instances[ii];
            if (seen[in.mesh_index]) continue;
            seen[in.mesh_index] = 1;
            const hx_mesh_desc& md = desc->meshes[in.mesh_index];
            for (uint32_t k = 0; k < md.num_submeshes; ++k) {
                const hx_submesh& sm = md.submeshes[k];
                uint32_t mat = in.material_override >= 0 ? (uint32_t)in.material_override : sm.material;
                if (!material_emissive(desc->materials[mat])) continue;
                hx_light l;
                std::memset(&l, 0, sizeof(l));
                l.data0[0] = (float)HX_LIGHT_AREA;
                l.data0[1] = (float)ii;
                l.data0[2] = (float)mat;
                l.data0[3] = (float)(sm.base_index / 3);
                l.data1[0] = (float)(sm.index_count / 3);
                s->lights_host.push_back(l);
            }
        }
        bool has_dir = false;
        for (uint32_t l = 0; l < desc->num_punctual_lights; ++l)
            has_dir |= (uint32_t)desc->punctual_lights[l].data0[0] == HX_LIGHT_DIRECTIONAL;
        if (desc->environment.kind != HX_ENV_NONE || has_dir) {
            hx_light l;
            std::memset(&l, 0, sizeof(l));
            l.data0[0] = (float)HX_LIGHT_ENVIRONMENT;
            s->lights_host.push_back(l);
        }
        for (uint32_t type : {HX_LIGHT_DIRECTIONAL, HX_LIGHT_POINT, HX_LIGHT_SPOT})
            for (uint32_t l = 0; l < desc->num_punctual_lights; ++l)
                if ((uint32_t)desc->punctual_lights[l].data0[0] == type) s->lights_host.push_back(desc->punctual_lights[l]);
    }
    // textures: one 32-bit word per RGBA8 texel, two per RGBA16F texel (at an
    // even word offset); flags in tex_desc.w (bit 0 sRGB, bit 1 half-float)
    std::vector<uint4> htd(desc->num_textures);
    size_t nwords = 0;
    for (uint32_t t = 0; t < desc->num_textures; ++t) {
        const uint32_t fmt = desc->textures[t].format;
        const bool half = fmt >= HX_TEXTURE_BC6H_SF16 && fmt <= HX_TEXTURE_RGBA16F;
        if (half) nwords = (nwords + 1) & ~(size_t)1;
        htd[t] = make_uint4((uint32_t)nwords, desc->textures[t].width, desc->textures[t].height,
                            (desc->textures[t].srgb ? 1u : 0u) | (half ? 2u : 0u) |
                                (fmt == HX_TEXTURE_RGBA8_SNORM ? 4u : 0u));
        nwords += (size_t)desc->textures[t].width * desc->textures[t].height * (half ? 2 : 1);
    }
    HX_CHECK_ARG(nwords < 0xffffffffull, "textures too large");

    // ---- device upload
    auto up = [&](void** dptr, const void* src, size_t bytes) -> hx_status {
        if (bytes == 0) { *dptr = nullptr; return HX_OK; }
        HX_TRY(hx_alloc(ctx, dptr, bytes));
        s->allocs.push_back(*dptr);
        HX_CUDA(cudaMemcpyAsync(*dptr, src, bytes, cudaMemcpyHostToDevice, st));
        return HX_OK;
    };
    hx_status rc;
#define UP(field, vec) \
    if ((rc = up((void**)&(field), (vec).data(), (vec).size() * sizeof((vec)[0]))) != HX_OK) return scene_fail(s, rc)
    // sRGB transfer function per byte (IEC 61966-2-1, as the Vulkan spec
    // decodes *_SRGB texels): c <= 0.04045 ? c / 12.92 : ((c + 0.055) / 1.055)^2.4
    std::vector<float> hlut(256);
    for (uint32_t q = 0; q < 256; ++q) {
        const double c = q / 255.0;
        hlut[q] = (float)(c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4));
    }
    UP(s->d.vtx, hv);
    UP(s->d.vtx_tb, htb);
    UP(s->d.srgb_lut, hlut);
    UP(s->d.vtx_w, hw);
    UP(s->d.indices, hidx);
    UP(s->d.inst, hinst);
    UP(s->d.prim_info, hpi);
    UP(s->d.alpha_uv, hauv);
    UP(s->d.lights, s->lights_host);
    UP(s->d.tex_desc, htd);
#undef UP
    {
        std::vector<hx_material> mats(desc->materials, desc->materials + desc->num_materials);
        if ((rc = up((void**)&s->d.materials, mats.data(), mats.size() * sizeof(hx_material))) != HX_OK) return scene_fail(s, rc);
    }
    if (nwords) {
        uint32_t* texels;
        if ((rc = hx_alloc_t(ctx, &texels, nwords)) != HX_OK) return scene_fail(s, rc);
        s->allocs.push_back(texels);
        // block-compressed textures are decoded on the host first (8-bit
        // formats to RGBA8, half-float formats to RGBA16F)
        std::vector<std::vector<uint8_t>> decoded;
        for (uint32_t t = 0; t < desc->num_textures; ++t) {
            const hx_texture_desc& td = desc->textures[t];
            size_t cnt = (size_t)td.width * td.height;
            const uint8_t* src = td.rgba8;
            const bool half = td.format >= HX_TEXTURE_BC6H_SF16 && td.format <= HX_TEXTURE_RGBA16F;
            if (half) {
                decoded.emplace_back(8 * cnt);
                if ((rc = hx_texture_decode_hdr(&td, reinterpret_cast<uint16_t*>(decoded.back().data()))) != HX_OK)
                    return scene_fail(s, rc);
                src = decoded.back().data();
            } else if (td.format != HX_TEXTURE_RGBA8 && td.format != HX_TEXTURE_RGBA8_SNORM) {
                decoded.emplace_back(4 * cnt);
                if ((rc = hx_texture_decode(&td, decoded.back().data())) != HX_OK) return scene_fail(s, rc);
                src = decoded.back().data();
            }
            HX_CUDA(cudaMemcpyAsync(texels + htd[t].x, src, (half ? 8 : 4) * cnt, cudaMemcpyHostToDevice, st));
        }
        if (!decoded.empty()) HX_CUDA(cudaStreamSynchronize(st));
        // the A8 copy shares the word offsets (the entries of half-float and
        // SNORM textures are unused: their alpha test goes through tex_bilinear)
        uint8_t* alpha8;
        if ((rc = hx_alloc_t(ctx, &alpha8, nwords)) != HX_OK) return scene_fail(s, rc);
        s->allocs.push_back(alpha8);
        k_alpha8<<<ctx->num_sms * 4, 256, 0, st>>>(texels, nwords, alpha8);
        HX_CUDA(cudaGetLastError());
        s->d.texels = texels;
        s->d.alpha8 = alpha8;
    }
    s->d.num_prims = (uint32_t)nprims;
    s->d.num_instances = desc->num_instances;
    s->d.num_lights = (uint32_t)s->lights_host.size();
    // ---- BVH
    if (nprims > 0) {
        DevBuffer world;
        if ((rc = world.reserve(ctx, 36 * nprims)) != HX_OK) return scene_fail(s, rc);
        if ((rc = hx_world_tris(ctx, s->d, world.as<float>())) != HX_OK) return scene_fail(s, rc);
        if ((rc = hx_build_bvh(ctx, s, world.as<float>(), (uint32_t)nprims)) != HX_OK) return scene_fail(s, rc);
        // scene bounds for info
        std::vector<float> hworld;
        world.release();
    }
    if ((rc = hx_env_build(ctx, s, desc->environment)) != HX_OK) return scene_fail(s, rc);
    HX_CUDA(cudaStreamSynchronize(st));
    s->info.num_lights = s->d.num_lights;
    {
        std::lock_guard<std::mutex> lk(ctx->mu);
        uint64_t bytes = 0;
        for (void* a : s->allocs) {
            auto itr = ctx->sizes.find(a);
            if (itr != ctx->sizes.end()) bytes += itr->second;
        }
        s->info.device_bytes = bytes;
    }
    *out = s;
    return HX_OK;
}

extern "C" hx_status hx_scene_destroy(hx_scene* s) {
    if (!s) return HX_OK;
    if (s->ctx) {
        cudaStreamSynchronize(s->ctx->stream);
        for (void* p : s->allocs) hx_free(s->ctx, p);
    }
    delete s;
    return HX_OK;
}

extern "C" hx_status hx_scene_set_traversal_stack_limit(hx_scene* s, uint32_t entries) {
    HX_CHECK_ARG(s && entries >= 1 && entries <= kTraversalStackEntries,
                 "hx_scene_set_traversal_stack_limit: entries must be in [1, %u]", kTraversalStackEntries);
    s->d.stack_limit = entries;
    return HX_OK;
}

extern "C" hx_status hx_scene_info_get(const hx_scene* s, hx_scene_info* out) {
    HX_CHECK_ARG(s && out, "hx_scene_info_get: null argument");
    *out = s->info;
    return HX_OK;
}

extern "C" hx_status hx_scene_lights(const hx_scene* s, hx_light* out, uint32_t capacity, uint32_t* count) {
    HX_CHECK_ARG(s && count, "hx_scene_lights: null argument");
    *count = (uint32_t)s->lights_host.size();
    if (out) std::memcpy(out, s->lights_host.data(), std::min<size_t>(capacity, s->lights_host.size()) * sizeof(hx_light));
    return HX_OK;
}

extern "C" hx_status hx_scene_export_bvh(const hx_scene* s, uint32_t* morton, uint32_t* sorted, uint32_t* children,
                                         void* nodes, uint32_t* leaf_prims) {
    HX_CHECK_ARG(s, "hx_scene_export_bvh: null scene");
    uint32_t n = s->d.num_prims;
    if (n == 0) return HX_OK;
    cudaStream_t st = s->ctx->stream;
    if (morton) HX_CUDA(cudaMemcpyAsync(morton, s->morton, 4 * (size_t)n, cudaMemcpyDeviceToHost, st));
    if (sorted) HX_CUDA(cudaMemcpyAsync(sorted, s->sorted, 4 * (size_t)n, cudaMemcpyDeviceToHost, st));
    if (children && n > 1) HX_CUDA(cudaMemcpyAsync(children, s->children, 8 * (size_t)(n - 1), cudaMemcpyDeviceToHost, st));
    if (nodes) HX_CUDA(cudaMemcpyAsync(nodes, s->d.nodes, sizeof(hx_bvh8_node) * (size_t)s->d.num_nodes, cudaMemcpyDeviceToHost, st));
    if (leaf_prims) HX_CUDA(cudaMemcpyAsync(leaf_prims, s->leaf_prims, 4 * (size_t)n, cudaMemcpyDeviceToHost, st));
    HX_CUDA(cudaStreamSynchronize(st));
    return HX_OK;
}

// Read back the baked environment (RGB float per texel) for parity tests.
extern "C" HX_API hx_status hx_scene_export_env(const hx_scene* s, float* out_rgb) {
    HX_CHECK_ARG(s && out_rgb, "hx_scene_export_env: null argument");
    const DevEnv& e = s->d.env;
    if (e.kind == HX_ENV_NONE) return HX_OK;
    size_t n = (size_t)e.width * e.height;
    std::vector<__half> h(4 * n);
    HX_CUDA(cudaMemcpy(h.data(), e.rgb, 8 * n, cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < n; ++i)
        for (int c = 0; c < 3; ++c) out_rgb[3 * i + c] = __half2float(h[4 * i + c]);
    return HX_OK;
}
