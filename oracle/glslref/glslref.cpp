// glslref.cpp — the reference's shader code, compiled as C++, beside the
// oracle's restatement (TEST INFRASTRUCTURE; built into oracle/_ref/ by
// oracle/glslref/build.py, loaded only by tests/test_reference_pin.py).
//
// The generated *_gen.inc files hold the reference's own GLSL functions
// (common.glsl, random.glsl, sampling.glsl, brdf.glsl, path_trace_rgen.glsl,
// path_trace_rchit.glsl, path_trace_rahit.glsl, path_trace_rmiss.glsl,
// path_trace_shadow.rchit/.rmiss, tone_map.frag) after the recipe's text
// rewrites.  This file supplies what the Vulkan pipeline supplies around
// them, written from the Vulkan / GL_EXT_ray_tracing specifications:
//   * each shader stage is a struct whose members are the stage's resources,
//     built-ins and payload variables; traceRayEXT binds the callee's
//     rayPayloadInEXT to the caller's payload at the given location, so the
//     closest-hit recursion of path_trace_rchit.glsl:487-536 runs as written;
//   * ray/triangle intersection, which the reference leaves to the driver and
//     RT cores, is the same watertight FP32 test and the same closest-hit rule
//     (lower t, then lower flattened triangle index) as the oracle, over all
//     world-space triangles (brute force), so both sides see the same hits
//     and the comparison isolates the shading code; non-opaque geometry runs
//     the reference's any-hit shader unless the ray is opaque, and
//     TerminateOnFirstHit ends a ray at its first accepted candidate;
//   * textures: bilinear filtering at level 0 with REPEAT addressing and
//     texel centres at +0.5 (Vulkan "Texel Filtering"), the weighted-sum form
//     of the specification, sRGB texels decoded before filtering;
//   * the environment "cubemap" is the library's lat-long map (the oracle's
//     map values), looked up bilinearly at the direction.
#include "../oracle.cpp"  // the restatement under test (its static functions)
#include "glsl_shim.h"

#include <vector>

namespace glsl {
namespace ref {

#define nonuniformEXT(x) (x)
#include "common_gen.inc"
#include "consts_gen.inc"

enum : uint {
    gl_RayFlagsNoneEXT = 0u,
    gl_RayFlagsOpaqueEXT = 1u,
    gl_RayFlagsNoOpaqueEXT = 2u,
    gl_RayFlagsTerminateOnFirstHitEXT = 4u,
    gl_RayFlagsSkipClosestHitShaderEXT = 8u,
};

struct samplerCube {};
struct Image {
    int w = 0, h = 0;
    std::vector<vec4> px;
};
struct Tex2D {
    int w = 0, h = 0;
    bool srgb = false;
    std::vector<uint8_t> rgba;
};

struct World {
    std::vector<std::vector<Vertex>> vertices;
    std::vector<std::vector<uint>> indices;
    std::vector<std::vector<uvec2>> submesh_info;  // per instance: uvec2(base_index / 3, material)
    std::vector<Material> materials;
    std::vector<Instance> instances;
    std::vector<Light> lights;
    std::vector<Tex2D> textures;
    int env_w = 0, env_h = 0;
    std::vector<float> env;  // rgb per texel
    struct Tri {
        oracle::V3<float> v0, v1, v2;
        uint instance, geometry, primitive;
        bool nonopaque;
    };
    std::vector<Tri> tris;
};

struct VertexBuf { const Vertex* data; };
struct IndexBuf { const uint* data; };
struct SubmeshBuf { const uvec2* data; };
struct MaterialBuf { const Material* data; };
struct InstanceBuf { const Instance* data; };
struct LightBuf { const Light* data; };
struct TexArray {
    int operator[](int i) const { return i; }
};

// sRGB EOTF (IEC 61966-2-1), evaluated in double and rounded once.
static float srgb_decode(uint8_t q) {
    double c = q / 255.0;
    return (float)(c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4));
}

// Recorded shadow query of probe mode (sample_light cases).
struct ShadowProbe {
    bool active = false, traced = false;
    uint flags = 0;
    vec3 origin, dir;
    float tmin = 0, tmax = 0;
};

struct Base {
    World& W;
    const PathTraceConsts& u_PathTraceConsts;
    ShadowProbe* probe;
    MaterialBuf Materials;
    InstanceBuf Instances;
    LightBuf Lights;
    std::vector<VertexBuf> Vertices;
    std::vector<IndexBuf> Indices;
    std::vector<SubmeshBuf> SubmeshInfo;
    TexArray s_Textures;
    samplerCube s_EnvironmentMap;
    int u_TopLevelAS = 0;

    Base(World& w, const PathTraceConsts& c, ShadowProbe* p = nullptr) : W(w), u_PathTraceConsts(c), probe(p) {
        Materials.data = w.materials.data();
        Instances.data = w.instances.data();
        Lights.data = w.lights.data();
        for (auto& v : w.vertices) Vertices.push_back({v.data()});
        for (auto& i : w.indices) Indices.push_back({i.data()});
        for (auto& s : w.submesh_info) SubmeshInfo.push_back({s.data()});
    }
    virtual ~Base() {}
    virtual void* payload(int loc) = 0;

    vec4 textureLod(int t, vec2 uv, float) const {
        const Tex2D& tx = W.textures[t];
        float x = uv.x * float(tx.w) - 0.5f, y = uv.y * float(tx.h) - 0.5f;
        float fx0 = std::floor(x), fy0 = std::floor(y);
        float a = x - fx0, b = y - fy0;
        long i0 = (long)fx0, j0 = (long)fy0;
        long W_ = tx.w, H_ = tx.h;
        long i0w = ((i0 % W_) + W_) % W_, j0w = ((j0 % H_) + H_) % H_;
        long i1w = (i0w + 1) % W_, j1w = (j0w + 1) % H_;
        vec4 r;
        for (int c = 0; c < 4; ++c) {
            auto tex = [&](long i, long j) {
                uint8_t q = tx.rgba[((size_t)j * tx.w + i) * 4 + c];
                return (tx.srgb && c < 3) ? srgb_decode(q) : float(q) / 255.0f;
            };
            r[c] = (1.0f - a) * (1.0f - b) * tex(i0w, j0w) + a * (1.0f - b) * tex(i1w, j0w) +
                   (1.0f - a) * b * tex(i0w, j1w) + a * b * tex(i1w, j1w);
        }
        return r;
    }
    vec4 texture(samplerCube, vec3 d) const {
        if (W.env_w == 0) return vec4(0.0f, 0.0f, 0.0f, 1.0f);
        float theta = std::acos(glsl::clamp(d.y, -1.0f, 1.0f));
        float phi = std::atan2(d.x, -d.z);
        float u = phi / (2.0f * 3.14159265358979323846f) + 0.5f;
        float v = theta / 3.14159265358979323846f;
        float x = u * float(W.env_w) - 0.5f, y = v * float(W.env_h) - 0.5f;
        float x0 = std::floor(x), y0 = std::floor(y);
        float fx = x - x0, fy = y - y0;
        long ix = (long)x0, iy = (long)y0, Wd = W.env_w, Hd = W.env_h;
        long ix0 = ((ix % Wd) + Wd) % Wd, ix1 = (ix0 + 1) % Wd;
        long iy0 = iy < 0 ? 0 : (iy >= Hd ? Hd - 1 : iy);
        long iy1 = iy + 1 < 0 ? 0 : (iy + 1 >= Hd ? Hd - 1 : iy + 1);
        vec4 out(0.0f, 0.0f, 0.0f, 1.0f);
        for (int c = 0; c < 3; ++c) {
            float a00 = W.env[((size_t)iy0 * Wd + ix0) * 3 + c], a10 = W.env[((size_t)iy0 * Wd + ix1) * 3 + c];
            float a01 = W.env[((size_t)iy1 * Wd + ix0) * 3 + c], a11 = W.env[((size_t)iy1 * Wd + ix1) * 3 + c];
            float top = a00 + (a10 - a00) * fx;
            float bot = a01 + (a11 - a01) * fx;
            out[c] = top + (bot - top) * fy;
        }
        return out;
    }

    void traceRayEXT(int, uint flags, uint, uint sbt_offset, uint, uint miss_index, vec3 origin, float tmin, vec3 dir,
                     float tmax, int location);
};

struct RAhit : Base {
    PathTracePayload dummy_payload;
    PathTracePayload& p_PathTracePayload = dummy_payload;
    bool ignored_ = false;
    vec2 b_HitAttribs;
    uint gl_InstanceCustomIndexEXT = 0, gl_GeometryIndexEXT = 0, gl_PrimitiveID = 0;
    using Base::Base;
    void* payload(int) override { return nullptr; }
#define ignoreIntersectionEXT \
    do {                      \
        ignored_ = true;      \
        return;               \
    } while (0)
#include "rahit_gen.inc"
#undef ignoreIntersectionEXT
};

struct RChit : Base {
    PathTracePayload& p_PathTracePayload;
    PathTracePayload p_IndirectPayload;
    bool p_Visibility = false;
    vec2 b_HitAttribs;
    uint gl_InstanceCustomIndexEXT = 0, gl_GeometryIndexEXT = 0, gl_PrimitiveID = 0;
    vec3 gl_WorldRayOriginEXT, gl_WorldRayDirectionEXT;
    float gl_HitTEXT = 0;
    RChit(World& w, const PathTraceConsts& c, PathTracePayload& pl, ShadowProbe* p = nullptr)
        : Base(w, c, p), p_PathTracePayload(pl) {}
    void* payload(int loc) override { return loc == 1 ? (void*)&p_IndirectPayload : (void*)&p_Visibility; }
#include "rchit_gen.inc"
};

struct RMiss : Base {
    PathTracePayload& p_PathTracePayload;
    vec3 gl_WorldRayOriginEXT, gl_WorldRayDirectionEXT;
    float gl_RayTmaxEXT = 0;
    RMiss(World& w, const PathTraceConsts& c, PathTracePayload& pl) : Base(w, c), p_PathTracePayload(pl) {}
    void* payload(int) override { return nullptr; }
#include "rmiss_gen.inc"
};

struct ShadowRChit {
    bool& p_Visibility;
#include "shadow_rchit_gen.inc"
};
struct ShadowRMiss {
    bool& p_Visibility;
#include "shadow_rmiss_gen.inc"
};

struct RGen : Base {
    PathTracePayload p_PathTracePayload;
    uvec3 gl_LaunchIDEXT;
    Image* i_PreviousColor = nullptr;
    Image* i_CurrentColor = nullptr;
    using Base::Base;
    void* payload(int) override { return &p_PathTracePayload; }
    vec4 imageLoad(Image* im, ivec2 p) const { return im->px[(size_t)p.y * im->w + p.x]; }
    void imageStore(Image* im, ivec2 p, vec4 v) const { im->px[(size_t)p.y * im->w + p.x] = v; }
#include "rgen_gen.inc"
};

struct ToneMapFrag {
    PushConstants u_PushConstants;
    const Image* src = nullptr;
    int samplerColor = 0;
    vec2 inUV;
    vec4 outFragColor;
    // inUV lies on a texel centre, where the linear filter returns that texel.
    vec4 texture(int, vec2 uv) const {
        int x = (int)std::floor(uv.x * float(src->w)), y = (int)std::floor(uv.y * float(src->h));
        return src->px[(size_t)y * src->w + x];
    }
#include "tonemap_gen.inc"
};

// Closest hit (or first accepted hit) over all triangles; runs the any-hit
// shader on non-opaque geometry unless the ray is opaque.
struct HitRec {
    bool found = false;
    float t = 0, u = 0, v = 0;
    uint tri = 0;
};
static HitRec intersect(World& W, const PathTraceConsts& c, vec3 o, vec3 d, float tmin, float tmax, uint flags) {
    oracle::RayPre<float> rp = oracle::ray_prepare(oracle::V3<float>(o.x, o.y, o.z), oracle::V3<float>(d.x, d.y, d.z));
    HitRec best;
    for (uint i = 0; i < W.tris.size(); ++i) {
        const World::Tri& tr = W.tris[i];
        float t, u, v;
        if (!oracle::intersect_triangle(rp, tr.v0, tr.v1, tr.v2, tmin, tmax, t, u, v)) continue;
        if (tr.nonopaque && !(flags & gl_RayFlagsOpaqueEXT)) {
            RAhit a(W, c);
            a.gl_InstanceCustomIndexEXT = tr.instance;
            a.gl_GeometryIndexEXT = tr.geometry;
            a.gl_PrimitiveID = tr.primitive;
            a.b_HitAttribs = vec2(u, v);
            a.main();
            if (a.ignored_) continue;
        }
        if (!best.found || t < best.t || (t == best.t && i < best.tri)) {
            best.found = true;
            best.t = t; best.u = u; best.v = v; best.tri = i;
        }
        if (flags & gl_RayFlagsTerminateOnFirstHitEXT) break;
    }
    return best;
}

// Primary-hit record of the current camera sample (first closest-hit query).
thread_local HitRec* g_primary = nullptr;

void Base::traceRayEXT(int, uint flags, uint, uint sbt_offset, uint, uint miss_index, vec3 origin, float tmin,
                       vec3 dir, float tmax, int location) {
    void* pl = payload(location);
    if (probe && probe->active && sbt_offset == VISIBILITY_CLOSEST_HIT_SHADER_IDX) {
        probe->traced = true;
        probe->flags = flags;
        probe->origin = origin; probe->dir = dir;
        probe->tmin = tmin; probe->tmax = tmax;
        *(bool*)pl = true;
        return;
    }
    HitRec h = intersect(W, u_PathTraceConsts, origin, dir, tmin, tmax, flags);
    if (sbt_offset == PATH_TRACE_CLOSEST_HIT_SHADER_IDX && g_primary) {
        *g_primary = h;
        g_primary = nullptr;
    }
    if (h.found) {
        if (sbt_offset == PATH_TRACE_CLOSEST_HIT_SHADER_IDX) {
            const World::Tri& tr = W.tris[h.tri];
            RChit c(W, u_PathTraceConsts, *(PathTracePayload*)pl);
            c.gl_InstanceCustomIndexEXT = tr.instance;
            c.gl_GeometryIndexEXT = tr.geometry;
            c.gl_PrimitiveID = tr.primitive;
            c.b_HitAttribs = vec2(h.u, h.v);
            c.gl_WorldRayOriginEXT = origin;
            c.gl_WorldRayDirectionEXT = dir;
            c.gl_HitTEXT = h.t;
            c.main();
        } else {
            ShadowRChit s{*(bool*)pl};
            s.main();
        }
    } else {
        if (miss_index == PATH_TRACE_MISS_SHADER_IDX) {
            RMiss m(W, u_PathTraceConsts, *(PathTracePayload*)pl);
            m.gl_WorldRayOriginEXT = origin;
            m.gl_WorldRayDirectionEXT = dir;
            m.gl_RayTmaxEXT = tmax;
            m.main();
        } else {
            ShadowRMiss s{*(bool*)pl};
            s.main();
        }
    }
}

static mat4 to_mat4(const float* m) {
    mat4 r;
    for (int c = 0; c < 4; ++c) r.c[c] = vec4(m[4 * c], m[4 * c + 1], m[4 * c + 2], m[4 * c + 3]);
    return r;
}
static vec4 to_vec4(const float* v) { return vec4(v[0], v[1], v[2], v[3]); }

static World* make_world(const hx_scene_desc* d, const hx_light* lights, uint32_t n_lights, const float* env_rgb,
                         uint32_t env_w, uint32_t env_h) {
    World* w = new World();
    for (uint32_t m = 0; m < d->num_meshes; ++m) {
        const hx_mesh_desc& md = d->meshes[m];
        std::vector<Vertex> vs(md.num_vertices);
        for (uint32_t i = 0; i < md.num_vertices; ++i) {
            const hx_vertex& v = md.vertices[i];
            vs[i].position = to_vec4(v.position);
            vs[i].tex_coord = to_vec4(v.tex_coord);
            vs[i].normal = to_vec4(v.normal);
            vs[i].tangent = to_vec4(v.tangent);
            vs[i].bitangent = to_vec4(v.bitangent);
        }
        w->vertices.push_back(vs);
        w->indices.push_back(std::vector<uint>(md.indices, md.indices + md.num_indices));
    }
    for (uint32_t k = 0; k < d->num_materials; ++k) {
        const hx_material& hm = d->materials[k];
        Material m;
        m.texture_indices0 = ivec4(hm.texture_indices0[0], hm.texture_indices0[1], hm.texture_indices0[2], hm.texture_indices0[3]);
        m.texture_indices1 = ivec4(hm.texture_indices1[0], hm.texture_indices1[1], hm.texture_indices1[2], hm.texture_indices1[3]);
        m.albedo = to_vec4(hm.albedo);
        m.emissive = to_vec4(hm.emissive);
        m.roughness_metallic = to_vec4(hm.roughness_metallic);
        w->materials.push_back(m);
    }
    for (uint32_t ii = 0; ii < d->num_instances; ++ii) {
        const hx_instance& hi = d->instances[ii];
        Instance inst;
        inst.model_matrix = to_mat4(hi.model_matrix);
        inst.normal_matrix = to_mat4(hi.normal_matrix);
        inst.mesh_idx = hi.mesh_index;
        w->instances.push_back(inst);
        const hx_mesh_desc& md = d->meshes[hi.mesh_index];
        std::vector<uvec2> info;
        for (uint32_t si = 0; si < md.num_submeshes; ++si) {
            const hx_submesh& sm = md.submeshes[si];
            uint mat = hi.material_override >= 0 ? (uint)hi.material_override : sm.material;
            info.push_back(uvec2(sm.base_index / 3, mat));
            for (uint p = 0; p < sm.index_count / 3; ++p) {
                World::Tri tr;
                oracle::V3<float>* dst[3] = {&tr.v0, &tr.v1, &tr.v2};
                for (int c = 0; c < 3; ++c) {
                    const hx_vertex& v = md.vertices[md.indices[sm.base_index + 3 * p + c]];
                    vec4 o = inst.model_matrix * vec4(v.position[0], v.position[1], v.position[2], 1.0f);
                    *dst[c] = oracle::V3<float>(o.x, o.y, o.z);
                }
                tr.instance = ii;
                tr.geometry = si;
                tr.primitive = p;
                tr.nonopaque = (sm.flags & HX_SUBMESH_NON_OPAQUE) != 0;
                w->tris.push_back(tr);
            }
        }
        w->submesh_info.push_back(info);
    }
    for (uint32_t k = 0; k < n_lights; ++k) {
        Light l;
        l.light_data0 = to_vec4(lights[k].data0);
        l.light_data1 = to_vec4(lights[k].data1);
        l.light_data2 = to_vec4(lights[k].data2);
        l.light_data3 = to_vec4(lights[k].data3);
        w->lights.push_back(l);
    }
    for (uint32_t t = 0; t < d->num_textures; ++t) {
        const hx_texture_desc& td = d->textures[t];
        Tex2D tx;
        tx.w = td.width;
        tx.h = td.height;
        tx.srgb = td.srgb != 0;
        tx.rgba.assign(td.rgba8, td.rgba8 + (size_t)td.width * td.height * 4);
        w->textures.push_back(tx);
    }
    if (env_rgb && env_w && env_h) {
        w->env_w = env_w;
        w->env_h = env_h;
        w->env.assign(env_rgb, env_rgb + (size_t)env_w * env_h * 3);
    }
    return w;
}

static PathTraceConsts make_consts(const World& w, const hx_integrator_desc* d, const hx_frame_desc* f, uint32_t frame) {
    PathTraceConsts c{};
    c.view_proj_inverse = to_mat4(f->view_proj_inverse);
    c.camera_pos = to_vec4(f->camera_pos);
    c.up_direction = to_vec4(f->up_direction);
    c.right_direction = to_vec4(f->right_direction);
    c.focal_plane = to_vec4(f->focal_plane);
    c.launch_id_size.x = 0;
    c.launch_id_size.y = 0;
    c.launch_id_size.z = d->width;
    c.launch_id_size.w = d->height;
    c.num_lights = (uint)w.lights.size();
    c.num_frames = frame;
    c.max_ray_bounces = d->max_ray_bounces;
    c.shadow_ray_bias = d->shadow_ray_bias;
    c.focal_length = f->focal_length;
    c.aperture_radius = f->aperture_radius;
    return c;
}

}  // namespace ref
}  // namespace glsl

namespace G = glsl;
namespace GR = glsl::ref;

static inline float bits_to_float(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }

extern "C" {

void* glslref_world_create(const hx_scene_desc* d, const hx_light* lights, uint32_t n_lights, const float* env_rgb,
                           uint32_t env_w, uint32_t env_h) {
    for (uint32_t t = 0; t < d->num_textures; ++t)
        if (d->textures[t].format != HX_TEXTURE_RGBA8) return nullptr;
    return GR::make_world(d, lights, n_lights, env_rgb, env_w, env_h);
}
void glslref_world_destroy(void* w) { delete (GR::World*)w; }

// Per-sample radiance of frame `frame`: the payload L after the reference's
// ray-gen shader has traced its camera ray (before clamping and
// accumulation), and the camera ray's closest hit (flattened triangle index,
// 0xffffffff on a miss; t).
void glslref_sample_radiance(void* hw, const hx_integrator_desc* d, const hx_frame_desc* f, uint32_t frame,
                             const uint32_t* pixels, uint32_t n, float* out_rgb, uint32_t* out_prim, float* out_t) {
    GR::World& w = *(GR::World*)hw;
    GR::PathTraceConsts c = GR::make_consts(w, d, f, frame);
#pragma omp parallel for schedule(dynamic, 16)
    for (long i = 0; i < (long)n; ++i) {
        uint32_t pix = pixels ? pixels[i] : (uint32_t)i;
        GR::RGen g(w, c);
        GR::HitRec prim;
        GR::g_primary = &prim;
        // The prologue of the ray-gen main() (path_trace_rgen.glsl:180-215):
        // payload init, rng_init, the reference's generate_ray and the camera
        // ray's trace; the payload is read before main()'s clamp and store.
        const G::uvec2 launch_id(pix % d->width, pix / d->width);
        const G::uvec2 launch_size(d->width, d->height);
        g.p_PathTracePayload.L = G::vec3(0.0f);
        g.p_PathTracePayload.T = G::vec3(1.0f);
        g.p_PathTracePayload.depth = 0;
        g.p_PathTracePayload.rng = GR::rng_init(launch_id, c.num_frames);
        GR::RGen::Ray ray = g.generate_ray(launch_id, launch_size);
        g.traceRayEXT(0, 0u, 0xFFu, PATH_TRACE_CLOSEST_HIT_SHADER_IDX, 0, PATH_TRACE_MISS_SHADER_IDX, ray.origin,
                      0.001f, ray.direction, 10000.0f, 0);
        GR::g_primary = nullptr;
        out_rgb[3 * i] = g.p_PathTracePayload.L.x;
        out_rgb[3 * i + 1] = g.p_PathTracePayload.L.y;
        out_rgb[3 * i + 2] = g.p_PathTracePayload.L.z;
        if (out_prim) out_prim[i] = prim.found ? prim.tri : 0xffffffffu;
        if (out_t) out_t[i] = prim.found ? prim.t : 0.0f;
    }
}

// Frames 0 .. num_frames-1 through the reference's ray-gen main(), which
// blends each sample into the ping-pong images (path_trace_rgen.glsl:217-248;
// num_frames = the frame index, path_integrator.cpp:154).  out: RGBA32F.
void glslref_render(void* hw, const hx_integrator_desc* d, const hx_frame_desc* f, uint32_t num_frames,
                    float* out_rgba) {
    GR::World& w = *(GR::World*)hw;
    GR::Image a, b;
    a.w = b.w = d->width;
    a.h = b.h = d->height;
    a.px.assign((size_t)d->width * d->height, G::vec4(0.0f));
    b.px.assign((size_t)d->width * d->height, G::vec4(0.0f));
    GR::Image *prev = &a, *cur = &b;
    for (uint32_t fr = 0; fr < num_frames; ++fr) {
        GR::PathTraceConsts c = GR::make_consts(w, d, f, fr);
#pragma omp parallel for schedule(dynamic, 16)
        for (long p = 0; p < (long)d->width * d->height; ++p) {
            GR::RGen g(w, c);
            g.gl_LaunchIDEXT = G::uvec3((uint)(p % d->width), (uint)(p / d->width), 0u);
            g.i_PreviousColor = prev;
            g.i_CurrentColor = cur;
            g.main();
        }
        std::swap(prev, cur);
    }
    for (size_t p = 0; p < prev->px.size(); ++p)
        for (int k = 0; k < 4; ++k) out_rgba[4 * p + k] = prev->px[p][k];
}

// tone_map.frag main() per pixel, then the R8G8B8A8_UNORM store (round to
// nearest), rows flipped like the renderer's negative-height viewport
// (renderer.cpp:394-399).
void glslref_tonemap(const float* accum_rgba, uint32_t w, uint32_t h, uint32_t op, float exposure, uint8_t* out) {
    GR::Image src;
    src.w = w;
    src.h = h;
    src.px.resize((size_t)w * h);
    for (size_t p = 0; p < src.px.size(); ++p)
        src.px[p] = G::vec4(accum_rgba[4 * p], accum_rgba[4 * p + 1], accum_rgba[4 * p + 2], accum_rgba[4 * p + 3]);
    for (uint32_t y = 0; y < h; ++y)
        for (uint32_t x = 0; x < w; ++x) {
            GR::ToneMapFrag fr;
            fr.u_PushConstants.exposure = exposure;
            fr.u_PushConstants.tone_map_operator = op;
            fr.src = &src;
            fr.inUV = G::vec2((x + 0.5f) / float(w), ((h - 1 - y) + 0.5f) / float(h));
            fr.main();
            uint8_t* o = &out[4 * ((size_t)y * w + x)];
            for (int c = 0; c < 4; ++c) {
                float v = glsl::clamp(fr.outFragColor[c], 0.0f, 1.0f);
                o[c] = (uint8_t)std::lrint(v * 255.0f);
            }
        }
}

// GR::RNG: n (x, y, frame) seeds -> `draws` xoroshiro64* outputs after
// rng_init, from the reference (out_ref) and the oracle (out_ora); plus
// next_float bits and next_uint for nmax = 1 + (k * 7919) % 100000.
void glslref_rng_cases(const uint32_t* seeds, uint32_t n, uint32_t draws, uint32_t* out_ref, uint32_t* out_ora) {
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t x = seeds[3 * i], y = seeds[3 * i + 1], fr = seeds[3 * i + 2];
        GR::RNG r = GR::rng_init(G::uvec2(x, y), fr);
        oracle::RNG o = oracle::rng_init(0, x, y, 0, fr);
        uint32_t* a = &out_ref[(size_t)i * draws * 3];
        uint32_t* b = &out_ora[(size_t)i * draws * 3];
        for (uint32_t k = 0; k < draws; ++k) {
            GR::RNG r2 = r;
            oracle::RNG o2 = o;
            a[3 * k] = GR::rng_next(r);
            b[3 * k] = oracle::rng_next(o);
            float fa = GR::next_float(r2), fb = oracle::next_float(o2);
            std::memcpy(&a[3 * k + 1], &fa, 4);
            std::memcpy(&b[3 * k + 1], &fb, 4);
            uint32_t nmax = 1 + (k * 7919u + i) % 100000u;
            a[3 * k + 2] = GR::next_uint(r2, nmax);
            b[3 * k + 2] = oracle::next_uint(o2, nmax);
        }
    }
}

// BSDF cases.  in: 16 floats per case — normal xyz, Wo xyz, Wi xyz,
// albedo rgb, roughness, metallic, two uniforms; rng: 2 words per case.
// out (both sides): 18 floats — GR::D_ggx(NdotH), G1(NdotL), evaluate_uber rgb,
// pdf_uber, sample_uber Wi xyz / pdf / value rgb, sample_cosine_lobe xyz,
// uniform_sample_triangle xy.
void glslref_brdf_cases(const float* in, const uint32_t* rng, uint32_t n, float* out_ref, float* out_ora) {
    for (uint32_t i = 0; i < n; ++i) {
        const float* q = &in[16 * i];
        G::vec3 N(q[0], q[1], q[2]), Wo(q[3], q[4], q[5]), Wi(q[6], q[7], q[8]);
        G::vec3 alb(q[9], q[10], q[11]);
        float rough = q[12], metal = q[13];
        GR::SurfaceProperties p{};
        p.normal = N;
        p.albedo = G::vec4(alb, 1.0f);
        p.roughness = rough;
        p.metallic = metal;
        p.F0 = G::mix(G::vec3(0.03f), alb, metal);
        p.alpha = rough * rough;
        p.alpha2 = p.alpha * p.alpha;
        G::vec3 Wh = G::normalize(Wo + Wi);
        float* a = &out_ref[18 * i];
        a[0] = GR::D_ggx(glsl::max(G::dot(N, Wh), 0.0f), rough * rough);
        a[1] = GR::G1_schlick_ggx(rough, glsl::max(G::dot(N, Wi), 0.0f));
        G::vec3 ev = GR::evaluate_uber(p, Wo, Wh, Wi);
        a[2] = ev.x; a[3] = ev.y; a[4] = ev.z;
        a[5] = GR::pdf_uber(p, Wo, Wh, Wi);
        GR::RNG r;
        r.s = G::uvec2(rng[2 * i], rng[2 * i + 1]);
        G::vec3 sWi;
        float spdf;
        G::vec3 sv = GR::sample_uber(p, Wo, r, sWi, spdf);
        a[6] = sWi.x; a[7] = sWi.y; a[8] = sWi.z; a[9] = spdf;
        a[10] = sv.x; a[11] = sv.y; a[12] = sv.z;
        G::vec3 cl = GR::sample_cosine_lobe(N, G::vec2(q[14], q[15]));
        a[13] = cl.x; a[14] = cl.y; a[15] = cl.z;
        G::vec2 ts = GR::uniform_sample_triangle(G::vec2(q[14], q[15]));
        a[16] = ts.x; a[17] = ts.y;

        using oracle::V3;
        oracle::Surface<float> s{};
        s.normal = V3<float>(q[0], q[1], q[2]);
        s.albedo = V3<float>(q[9], q[10], q[11]);
        s.albedo_a = 1.0f;
        s.roughness = rough;
        s.metallic = metal;
        s.F0 = V3<float>(0.03f) * (1.0f - metal) + s.albedo * metal;
        s.alpha = rough * rough;
        s.alpha2 = s.alpha * s.alpha;
        V3<float> oN(q[0], q[1], q[2]), oWo(q[3], q[4], q[5]), oWi(q[6], q[7], q[8]);
        V3<float> oWh = oracle::normalize(oWo + oWi);
        float* b = &out_ora[18 * i];
        b[0] = oracle::D_ggx(oracle::gmax(oracle::dot(oN, oWh), 0.0f), rough * rough);
        b[1] = oracle::G1_schlick_ggx(rough, oracle::gmax(oracle::dot(oN, oWi), 0.0f));
        V3<float> oev = oracle::evaluate_uber(s, oWo, oWh, oWi);
        b[2] = oev.x; b[3] = oev.y; b[4] = oev.z;
        b[5] = oracle::pdf_uber(s, oWo, oWh, oWi);
        oracle::RNG orng;
        orng.kind = 0;
        orng.s0 = rng[2 * i];
        orng.s1 = rng[2 * i + 1];
        V3<float> osWi;
        float ospdf;
        V3<float> osv = oracle::sample_uber(s, oWo, orng, osWi, ospdf);
        b[6] = osWi.x; b[7] = osWi.y; b[8] = osWi.z; b[9] = ospdf;
        b[10] = osv.x; b[11] = osv.y; b[12] = osv.z;
        V3<float> ocl = oracle::sample_cosine_lobe(oN, q[14], q[15]);
        b[13] = ocl.x; b[14] = ocl.y; b[15] = ocl.z;
        float su0 = std::sqrt(q[14]);  // the oracle inlines uniform_sample_triangle in sample_light
        b[16] = 1.0f - su0; b[17] = q[15] * su0;
    }
}

// sample_light cases on a world and the oracle's copy of the same scene.
// in: 8 floats per case — position xyz, normal xyz, depth, light index;
// rng: 2 words.  out (both sides): 16 floats — Wi xyz, Li rgb, pdf, shadow
// tmax, traced (0/1), any-hit enabled (0/1), shadow origin xyz, rng s0 s1
// (bit patterns).  Li is the light's radiance before visibility (the probe
// answers every shadow query with "visible").
void glslref_sample_light_cases(void* hw, void* oracle_scene, const hx_integrator_desc* d, const float* in,
                                const uint32_t* rng, uint32_t n, float* out_ref, float* out_ora) {
    GR::World& w = *(GR::World*)hw;
    const oracle::Scene& os = *(const oracle::Scene*)oracle_scene;
    hx_frame_desc fd{};
    GR::PathTraceConsts c = GR::make_consts(w, d, &fd, 0);
    oracle::Params P = oracle::make_params(*d, (uint32_t)os.lights.size());
    for (uint32_t i = 0; i < n; ++i) {
        const float* q = &in[8 * i];
        uint32_t depth = (uint32_t)q[6], li = (uint32_t)q[7];
        GR::ShadowProbe probe;
        probe.active = true;
        GR::PathTracePayload pl{};
        pl.depth = depth;
        pl.rng.s = G::uvec2(rng[2 * i], rng[2 * i + 1]);
        GR::RChit ch(w, c, pl, &probe);
        GR::SurfaceProperties p{};
        p.vertex.position = G::vec4(q[0], q[1], q[2], 1.0f);
        p.normal = G::vec3(q[3], q[4], q[5]);
        G::vec3 Wi;
        float pdf = 0;
        G::vec3 Li = ch.sample_light(p, w.lights[li], Wi, pdf);
        float* a = &out_ref[16 * i];
        a[0] = Wi.x; a[1] = Wi.y; a[2] = Wi.z;
        a[3] = Li.x; a[4] = Li.y; a[5] = Li.z;
        a[6] = pdf;
        a[7] = probe.tmax;
        a[8] = probe.traced ? 1.0f : 0.0f;
        a[9] = (probe.traced && !(probe.flags & GR::gl_RayFlagsOpaqueEXT)) ? 1.0f : 0.0f;
        a[10] = probe.origin.x; a[11] = probe.origin.y; a[12] = probe.origin.z;
        std::memcpy(&a[13], &pl.rng.s.x, 4);
        std::memcpy(&a[14], &pl.rng.s.y, 4);
        a[15] = 0;

        using oracle::V3;
        oracle::Surface<float> s{};
        s.position = V3<float>(q[0], q[1], q[2]);
        s.normal = V3<float>(q[3], q[4], q[5]);
        oracle::RNG orng;
        orng.kind = 0;
        orng.s0 = rng[2 * i];
        orng.s1 = rng[2 * i + 1];
        V3<float> oWi;
        float opdf = 0, otmax = 0;
        bool trace_it = false;
        V3<float> oLi = oracle::sample_light<float>(os, P, s, os.lights[li], orng, oWi, opdf, otmax, trace_it);
        float* b = &out_ora[16 * i];
        b[0] = oWi.x; b[1] = oWi.y; b[2] = oWi.z;
        b[3] = oLi.x; b[4] = oLi.y; b[5] = oLi.z;
        b[6] = opdf;
        b[7] = trace_it ? otmax : 0.0f;
        b[8] = trace_it ? 1.0f : 0.0f;
        b[9] = (trace_it && depth == 0) ? 1.0f : 0.0f;
        V3<float> so = s.position + s.normal * d->shadow_ray_bias;
        b[10] = trace_it ? so.x : 0.0f; b[11] = trace_it ? so.y : 0.0f; b[12] = trace_it ? so.z : 0.0f;
        std::memcpy(&b[13], &orng.s0, 4);
        std::memcpy(&b[14], &orng.s1, 4);
        b[15] = 0;
    }
}

// Camera rays: generate_ray of the reference (after rng_init of the pixel)
// and of the oracle.  out: 8 floats per pixel — origin xyz, direction xyz,
// rng s0 s1 (bit patterns).
void glslref_camera_cases(const hx_integrator_desc* d, const hx_frame_desc* f, uint32_t frame, const uint32_t* pixels,
                          uint32_t n, float* out_ref, float* out_ora) {
    GR::World w;
    GR::PathTraceConsts c = GR::make_consts(w, d, f, frame);
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t x = pixels[i] % d->width, y = pixels[i] / d->width;
        GR::RGen g(w, c);
        g.p_PathTracePayload.rng = GR::rng_init(G::uvec2(x, y), frame);
        GR::RGen::Ray r = g.generate_ray(G::uvec2(x, y), G::uvec2(d->width, d->height));
        float* a = &out_ref[8 * i];
        a[0] = r.origin.x; a[1] = r.origin.y; a[2] = r.origin.z;
        a[3] = r.direction.x; a[4] = r.direction.y; a[5] = r.direction.z;
        std::memcpy(&a[6], &g.p_PathTracePayload.rng.s.x, 4);
        std::memcpy(&a[7], &g.p_PathTracePayload.rng.s.y, 4);

        oracle::RNG orng = oracle::rng_init(0, x, y, d->width, frame);
        oracle::V3<float> o, dir;
        oracle::generate_ray<float>(*f, x, y, d->width, d->height, orng, o, dir);
        float* b = &out_ora[8 * i];
        b[0] = o.x; b[1] = o.y; b[2] = o.z;
        b[3] = dir.x; b[4] = dir.y; b[5] = dir.z;
        std::memcpy(&b[6], &orng.s0, 4);
        std::memcpy(&b[7], &orng.s1, 4);
    }
}

}  // extern "C"
