// oracle.cpp — CPU oracle for the helios-gb300 path-tracing core
// (TEST INFRASTRUCTURE ONLY: loaded by tests/, __graft_entry__.smoke() and
// bench.py's CPU-baseline leg; never linked into the product library).
//
// A scalar restatement of the reference's path-tracing shaders, templated on
// FP32 (bit-exact integer parity, CPU baseline) and FP64 (radiance oracle):
//   random.glsl, sampling.glsl (RNG)               -> oracle_core.h
//   brdf.glsl :6-167                               -> evaluate_uber / pdf_uber / sample_uber
//   path_trace_rgen.glsl generate_ray :132-174     -> generate_ray
//   path_trace_rgen.glsl main :180-250             -> trace_path + accumulate
//   path_trace_rchit.glsl :143-280                 -> populate
//   path_trace_rchit.glsl sample_light :284-451    -> sample_light
//   path_trace_rchit.glsl direct :455-483, indirect :487-536, main :542-580 -> trace_path
//   path_trace_rahit.glsl :162-188                 -> alpha_pass
//   path_trace_rmiss.glsl :38-67, path_trace_shadow.rchit/.rmiss -> env_lookup, any-hit visibility
//   tone_map.frag :8-51                            -> oracle_tonemap
//   procedural_sky.frag :48-75                     -> sky_radiance
//   scene.cpp :915-1311 (flattening, light order)  -> flatten / build_lights
// plus an independent LBVH -> BVH8 builder (Karras 2012 hierarchy, greedy
// 8-wide collapse, 8-bit conservative child boxes) whose integer outputs are
// compared bit for bit with the device builder.
//
// Parity status: unpinned against reference outputs (the reference has no
// tests and its Vulkan ray-tracing path cannot run without a graphics
// stack); see oracle_core.h for the floating-point contract.
#include "oracle_core.h"
#include "../include/hx.h"

#include <omp.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <numeric>
#include <vector>

namespace oracle {

template <typename R> static inline R kpi() { return R(3.14159265359); }  // M_PI, common.glsl:18
static const float kEpsilon = 0.0001f;                                    // EPSILON, common.glsl:19
static const float kMinRoughness = 0.1f;                                  // MIN_ROUGHNESS, common.glsl:21
static const uint32_t kNoHit = 0xffffffffu;

struct PrimInfo {
    uint32_t instance, mesh_prim, material, submesh;
};
struct Tex {
    std::vector<uint8_t> rgba;
    std::vector<float> hdr;  // RGBA16F textures: the half values as floats (then rgba is empty)
    uint32_t w = 0, h = 0;
    bool srgb = false;   // RGB sRGB-encoded (resource_manager.cpp:48-67)
    bool snorm = false;  // *_SNORM bytes (kNonSRGBFormats, resource_manager.cpp:32-36, 64)
};

struct Bvh {
    std::vector<uint32_t> morton, sorted;            // per input prim / sorted order
    std::vector<uint32_t> children;                  // 2*(n-1), bit31 = leaf
    std::vector<float> lo, hi;                       // internal boxes 3*(n-1)
    std::vector<uint32_t> first, count;              // internal node ranges
    std::vector<hx_bvh8_node> nodes;
    std::vector<uint32_t> leaf_prims;                // flattened prim ids in leaf order
};

struct Scene {
    std::vector<std::vector<hx_vertex>> vertices;
    std::vector<std::vector<uint32_t>> indices;
    std::vector<std::vector<hx_submesh>> submeshes;
    std::vector<hx_instance> instances;
    std::vector<hx_material> materials;
    std::vector<Tex> textures;
    std::vector<hx_light> punctual;
    std::vector<hx_light> lights;
    std::vector<PrimInfo> prims;
    std::vector<float> wpos;     // 9 floats per prim, world space, FP32
    std::vector<double> wpos64;  // same, FP64
    std::vector<uint8_t> nonopaque;
    Bvh bvh;
    uint32_t env_kind = HX_ENV_NONE, env_w = 0, env_h = 0;
    std::vector<float> env;  // rgb per texel, FP16-rounded
    std::vector<float> env_margf, env_condf;
    float sun[3] = {0, 1, 0};
    float coeffs[40] = {0};
};

// ---------------------------------------------------------------------------
// Hosek-Wilkie sky radiance, procedural_sky.frag:48-75.
// ---------------------------------------------------------------------------
template <typename R> static V3<R> sky_radiance(const float* c, V3<R> v, V3<R> sun) {
    R cos_theta = gclamp(v.y, R(0), R(1));
    R cos_gamma = gclamp(dot(v, sun), R(0), R(1));
    R gamma = std::acos(cos_gamma);
    V3<R> out;
    for (int k = 0; k < 3; ++k) {
        R A = c[0 + k], B = c[4 + k], C = c[8 + k], D = c[12 + k], E = c[16 + k], F = c[20 + k], G = c[24 + k],
          H = c[28 + k], I = c[32 + k], Z = c[36 + k];
        R chi = (R(1) + cos_gamma * cos_gamma) / std::pow(R(1) + H * H - R(2) * cos_gamma * H, R(1.5));
        R hw = (R(1) + A * std::exp(B / (cos_theta + R(0.01)))) *
               (C + D * std::exp(E * gamma) + F * (cos_gamma * cos_gamma) + G * chi + I * std::sqrt(cos_theta));
        out[k] = Z * hw;
    }
    return out;
}

// Lat-long mapping (texel centre): phi = 2pi(u - 0.5), theta = pi v,
// d = (sin(theta) sin(phi), cos(theta), -sin(theta) cos(phi)).
static V3<double> latlong_dir(double u, double v) {
    double phi = 2.0 * 3.14159265358979323846 * (u - 0.5);
    double theta = 3.14159265358979323846 * v;
    double st = std::sin(theta);
    return V3<double>(st * std::sin(phi), std::cos(theta), -st * std::cos(phi));
}


// Importance-sampling table (the device construction, restated in FP32
// with the same summation order): weight(i,j) = (lum + floor) * sin(theta_j),
// floor = 1e-3 * mean luminance; rows prefix-summed in 256 contiguous chunks,
// each row normalised to 1, then a normalised marginal over the row totals.
static float texel_lum(const float* e) { return 0.2126f * e[0] + 0.7152f * e[1] + 0.0722f * e[2]; }

static void build_env_cdf(Scene& s) {
    const uint32_t w = s.env_w, h = s.env_h, T = 256;
    std::vector<float> rowlum(h), rowsum(h);
    for (uint32_t j = 0; j < h; ++j) {
        float part[256];
        for (uint32_t t = 0; t < T; ++t) {
            float acc = 0.0f;
            for (uint32_t i = t; i < w; i += T) acc += texel_lum(&s.env[((size_t)j * w + i) * 3]);
            part[t] = acc;
        }
        for (uint32_t o = T / 2; o > 0; o >>= 1)
            for (uint32_t t = 0; t < o; ++t) part[t] += part[t + o];
        rowlum[j] = part[0];
    }
    float tot = 0.0f;
    for (uint32_t j = 0; j < h; ++j) tot += rowlum[j];
    const float floor_w = 1e-3f * tot / ((float)w * (float)h) + 1e-12f;
    const float kPiF32 = 3.14159265358979323846f;
    s.env_condf.assign((size_t)h * (w + 1), 0.0f);
    s.env_margf.assign(h + 1, 0.0f);
    const uint32_t chunk = (w + T - 1) / T;
    for (uint32_t j = 0; j < h; ++j) {
        float st = std::sin(kPiF32 * ((float)j + 0.5f) / (float)h);
        float part[256];
        for (uint32_t t = 0; t < T; ++t) {
            uint32_t i0 = t * chunk, i1 = std::min(w, i0 + chunk);
            float local = 0.0f;
            for (uint32_t i = i0; i < i1; ++i) local += (texel_lum(&s.env[((size_t)j * w + i) * 3]) + floor_w) * st;
            part[t] = local;
        }
        float run = 0.0f;
        for (uint32_t t = 0; t < T; ++t) { float x = part[t]; part[t] = run; run += x; }
        rowsum[j] = run;
        float* row = &s.env_condf[(size_t)j * (w + 1)];
        row[0] = 0.0f;
        for (uint32_t t = 0; t < T; ++t) {
            uint32_t i0 = t * chunk, i1 = std::min(w, i0 + chunk);
            float r = part[t];
            for (uint32_t i = i0; i < i1; ++i) {
                r += (texel_lum(&s.env[((size_t)j * w + i) * 3]) + floor_w) * st;
                row[i + 1] = run > 0.0f ? r / run : (float)(i + 1) / (float)w;
            }
        }
        row[w] = 1.0f;
    }
    float mt = 0.0f;
    for (uint32_t j = 0; j < h; ++j) mt += rowsum[j];
    float run = 0.0f;
    s.env_margf[0] = 0.0f;
    for (uint32_t j = 0; j < h; ++j) {
        run += rowsum[j];
        s.env_margf[j + 1] = mt > 0.0f ? run / mt : (float)(j + 1) / (float)h;
    }
    s.env_margf[h] = 1.0f;
}

template <typename R> static V3<R> env_lookup(const Scene& s, V3<R> d) {
    if (s.env_kind == HX_ENV_NONE) return V3<R>(R(0));
    R theta = std::acos(gclamp(d.y, R(-1), R(1)));
    R phi = std::atan2(d.x, -d.z);
    R u = phi / (R(2) * R(3.14159265358979323846)) + R(0.5);
    R v = theta / R(3.14159265358979323846);
    R x = u * R(s.env_w) - R(0.5), y = v * R(s.env_h) - R(0.5);
    R x0 = std::floor(x), y0 = std::floor(y);
    R fx = x - x0, fy = y - y0;
    long ix = (long)x0, iy = (long)y0;
    long W = s.env_w, H = s.env_h;
    long ix0 = ((ix % W) + W) % W, ix1 = (ix0 + 1) % W;
    long iy0 = iy < 0 ? 0 : (iy >= H ? H - 1 : iy);
    long iy1 = iy + 1 < 0 ? 0 : (iy + 1 >= H ? H - 1 : iy + 1);
    V3<R> out;
    for (int c = 0; c < 3; ++c) {
        R a00 = s.env[((size_t)iy0 * W + ix0) * 3 + c], a10 = s.env[((size_t)iy0 * W + ix1) * 3 + c];
        R a01 = s.env[((size_t)iy1 * W + ix0) * 3 + c], a11 = s.env[((size_t)iy1 * W + ix1) * 3 + c];
        R top = a00 + (a10 - a00) * fx;
        R bot = a01 + (a11 - a01) * fx;
        out[c] = top + (bot - top) * fy;
    }
    return out;
}

// Samples a direction from the lat-long CDF with two uniforms (binary
// searches over the normalised FP32 tables, continuous within the texel);
// returns the solid-angle pdf.
static int upper_bound_f(const float* a, int lo, int hi, float x) {
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (a[mid] > x) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}

template <typename R> static V3<R> env_sample(const Scene& s, float r0, float r1, R& pdf) {
    int W = (int)s.env_w, H = (int)s.env_h;
    int j = upper_bound_f(s.env_margf.data(), 1, H + 1, r1) - 1;
    j = j < 0 ? 0 : (j >= H ? H - 1 : j);
    const float* row = &s.env_condf[(size_t)j * (W + 1)];
    int i = upper_bound_f(row, 1, W + 1, r0) - 1;
    i = i < 0 ? 0 : (i >= W ? W - 1 : i);
    float m0 = s.env_margf[j], m1 = s.env_margf[j + 1], c0 = row[i], c1 = row[i + 1];
    R fv = m1 > m0 ? (R(r1) - R(m0)) / (R(m1) - R(m0)) : R(0.5);
    R fu = c1 > c0 ? (R(r0) - R(c0)) / (R(c1) - R(c0)) : R(0.5);
    fv = gclamp(fv, R(0), R(1));
    fu = gclamp(fu, R(0), R(1));
    R u = (R(i) + fu) / R(W), v = (R(j) + fv) / R(H);
    const R pi = R(3.14159265358979323846);
    R phi = R(2) * pi * (u - R(0.5));
    R theta = pi * v;
    R st = std::sin(theta);
    V3<R> d(st * std::sin(phi), std::cos(theta), -st * std::cos(phi));
    R pmf = (R(c1) - R(c0)) * (R(m1) - R(m0));
    pdf = st > R(0) ? pmf * R(W) * R(H) / (R(2) * pi * pi * st) : R(0);
    return d;
}

// ---------------------------------------------------------------------------
// Scene construction.
// ---------------------------------------------------------------------------
static void flatten(Scene& s) {
    for (uint32_t ii = 0; ii < s.instances.size(); ++ii) {
        const hx_instance& inst = s.instances[ii];
        uint32_t m = inst.mesh_index;
        const auto& vs = s.vertices[m];
        const auto& ix = s.indices[m];
        double md[16];
        for (int k = 0; k < 16; ++k) md[k] = inst.model_matrix[k];
        for (uint32_t si = 0; si < s.submeshes[m].size(); ++si) {
            const hx_submesh& sm = s.submeshes[m][si];
            uint32_t mat = inst.material_override >= 0 ? (uint32_t)inst.material_override : sm.material;
            for (uint32_t p = 0; p < sm.index_count / 3; ++p) {
                uint32_t mp = sm.base_index / 3 + p;
                s.prims.push_back({ii, mp, mat, si});
                s.nonopaque.push_back((sm.flags & HX_SUBMESH_NON_OPAQUE) ? 1 : 0);
                for (int c = 0; c < 3; ++c) {
                    const hx_vertex& v = vs[ix[3 * mp + c]];
                    float o[4];
                    mat4_mul(inst.model_matrix, v.position[0], v.position[1], v.position[2], 1.0f, o);
                    double od[4];
                    mat4_mul(md, (double)v.position[0], (double)v.position[1], (double)v.position[2], 1.0, od);
                    for (int a = 0; a < 3; ++a) {
                        s.wpos.push_back(o[a]);
                        s.wpos64.push_back(od[a]);
                    }
                }
            }
        }
    }
}

static bool material_emissive(const hx_material& m) {  // Material::is_emissive, material.cpp:71-77
    if (m.texture_indices1[0] != -1) return true;
    return m.emissive[0] > 0.0f || m.emissive[1] > 0.0f || m.emissive[2] > 0.0f;
}

static void build_lights(Scene& s) {
    std::vector<uint8_t> seen(s.vertices.size(), 0);
    for (uint32_t ii = 0; ii < s.instances.size(); ++ii) {
        uint32_t m = s.instances[ii].mesh_index;
        if (seen[m]) continue;
        seen[m] = 1;
        for (const hx_submesh& sm : s.submeshes[m]) {
            uint32_t mat = s.instances[ii].material_override >= 0 ? (uint32_t)s.instances[ii].material_override : sm.material;
            if (!material_emissive(s.materials[mat])) continue;
            hx_light l{};
            l.data0[0] = (float)HX_LIGHT_AREA;
            l.data0[1] = (float)ii;
            l.data0[2] = (float)mat;
            l.data0[3] = (float)(sm.base_index / 3);
            l.data1[0] = (float)(sm.index_count / 3);
            s.lights.push_back(l);
        }
    }
    bool has_dir = false;
    for (const hx_light& l : s.punctual) has_dir |= (uint32_t)l.data0[0] == HX_LIGHT_DIRECTIONAL;
    if (s.env_kind != HX_ENV_NONE || has_dir) {
        hx_light l{};
        l.data0[0] = (float)HX_LIGHT_ENVIRONMENT;
        s.lights.push_back(l);
    }
    for (uint32_t type : {HX_LIGHT_DIRECTIONAL, HX_LIGHT_POINT, HX_LIGHT_SPOT})
        for (const hx_light& l : s.punctual)
            if ((uint32_t)l.data0[0] == type) s.lights.push_back(l);
}

// ---------------------------------------------------------------------------
// LBVH: Morton codes, stable sort, Karras hierarchy, boxes, BVH8 collapse.
// ---------------------------------------------------------------------------
static uint32_t expand_bits(uint32_t v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

static int clz32(uint32_t x) { return x == 0 ? 32 : __builtin_clz(x); }

static int karras_delta(const std::vector<uint32_t>& keys, int n, int i, int j) {
    if (j < 0 || j > n - 1) return -1;
    uint32_t a = keys[i], b = keys[j];
    if (a == b) return 32 + clz32((uint32_t)i ^ (uint32_t)j);
    return clz32(a ^ b);
}

static float f32_bits(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
static uint32_t bits_f32(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }

// Smallest e with 2^e >= x (x > 0), e >= -126.
static int ceil_log2f(float x) {
    uint32_t b = bits_f32(x);
    int ex = (int)((b >> 23) & 0xff);
    if (ex == 0) return -126;
    int e = ex - 127 + ((b & 0x7fffff) != 0 ? 1 : 0);
    return e < -126 ? -126 : e;
}
static float pow2f(int e) { return f32_bits((uint32_t)(e < -126 ? 1 : e + 127) << 23); }

// Grid exponent of one node axis: 254 steps of 2^e cover [lo, hi] (the
// snapped origin takes at most one more step of the 255), and 2^e is at
// least twice the ulp of the largest coordinate, so with the origin snapped
// to a multiple of 2^e, |origin| < 2^23 2^e and every decoded plane
// origin + q 2^e (and origin - 2^23 2^e) is exactly representable: any
// decode formula that rounds once gives the same plane.
static int grid_exponent(float lo, float hi) {
    float ext = hi - lo;
    int e = ext > 0.0f ? ceil_log2f(ext / 254.0f) : -126;
    float m = std::fabs(lo) > std::fabs(hi) ? std::fabs(lo) : std::fabs(hi);
    uint32_t mb = bits_f32(m);
    int mexp = (int)((mb >> 23) & 0xff);
    int e_min = mexp == 0 ? -126 : mexp - 127 - 23 + 1;
    e = e > e_min ? e : e_min;
    return e < -126 ? -126 : (e > 119 ? 119 : e);
}

static float half_area(const float* lo, const float* hi) {
    float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    return dx * dy + dy * dz + dz * dx;
}

// meta bytes (hx_bvh8_node): the low 5 bits are the slot's bit in the
// traversal's hit mask.
constexpr uint8_t kMetaEmpty = 0x10, kMetaInternal = 0x98, kMetaLeaf = 0x20;

// Quantises the occupied slots (meta != empty) of a node on its own grid.
static void quantise_node(hx_bvh8_node& node, const float (*clo)[3], const float (*chi)[3]) {
    float plo[3] = {INFINITY, INFINITY, INFINITY}, phi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int k = 0; k < 8; ++k) {
        if (node.meta[k] == kMetaEmpty) continue;
        for (int a = 0; a < 3; ++a) {
            plo[a] = clo[k][a] < plo[a] ? clo[k][a] : plo[a];
            phi[a] = chi[k][a] > phi[a] ? chi[k][a] : phi[a];
        }
    }
    for (int a = 0; a < 3; ++a) {
        int e = grid_exponent(plo[a], phi[a]);
        float scale = pow2f(e);
        float origin = std::floor(plo[a] * pow2f(-e)) * scale;
        while (e < 119 && origin + 255.0f * scale < phi[a]) {
            ++e;
            scale = pow2f(e);
            origin = std::floor(plo[a] * pow2f(-e)) * scale;
        }
        node.origin[a] = origin;
        node.exponent[a] = (int8_t)e;
        float inv = pow2f(-e);
        for (int k = 0; k < 8; ++k) {
            if (node.meta[k] == kMetaEmpty) { node.qlo[a][k] = 0; node.qhi[a][k] = 0; continue; }
            float fl = std::floor((clo[k][a] - origin) * inv);
            int ql = fl < 0.0f ? 0 : (fl > 255.0f ? 255 : (int)fl);
            while (ql > 0 && origin + (float)ql * scale > clo[k][a]) --ql;
            float fh = std::ceil((chi[k][a] - origin) * inv);
            int qh = fh < 0.0f ? 0 : (fh > 255.0f ? 255 : (int)fh);
            while (qh < 255 && origin + (float)qh * scale < chi[k][a]) ++qh;
            node.qlo[a][k] = (uint8_t)ql;
            node.qhi[a][k] = (uint8_t)qh;
        }
    }
}

// Octant slot assignment of up to 8 children (boxes klo/khi): the score of
// child i in slot s is the sum over axes of +-(c_i - c_node), + where bit k
// of s is set; greedy over (child, slot) pairs by decreasing score, ties to
// the lower child position then the lower slot.  slot_kid[s] = child or ~0.
static void assign_octant_slots(int nk, const float (*klo)[3], const float (*khi)[3], uint32_t slot_kid[8]) {
    float nlo[3] = {INFINITY, INFINITY, INFINITY}, nhi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int c = 0; c < nk; ++c)
        for (int a = 0; a < 3; ++a) {
            nlo[a] = klo[c][a] < nlo[a] ? klo[c][a] : nlo[a];
            nhi[a] = khi[c][a] > nhi[a] ? khi[c][a] : nhi[a];
        }
    float score[8][8];
    for (int c = 0; c < nk; ++c) {
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
    bool kid_done[8] = {false, false, false, false, false, false, false, false};
    for (int round = 0; round < nk; ++round) {
        int bc = -1, bs = -1;
        float best = 0.0f;
        for (int c = 0; c < nk; ++c) {
            if (kid_done[c]) continue;
            for (int sl = 0; sl < 8; ++sl) {
                if (slot_kid[sl] != 0xffffffffu) continue;
                if (bc < 0 || score[c][sl] > best) { bc = c; bs = sl; best = score[c][sl]; }
            }
        }
        kid_done[bc] = true;
        slot_kid[bs] = (uint32_t)bc;
    }
}

// Triangles per BVH8 leaf slot (the device builder's kLeafMax): one — a
// triangle's own 8-bit box culls it before the triangle test.
constexpr uint32_t kLeafMax = 1;

// Treelet restructuring of the binary LBVH (Karras & Aila, "Fast Parallel
// Construction of High-Quality Bounding Volume Hierarchies", HPG 2013), the
// same steps as the device builder (bvh_build.cu, k_treelet): in each pass,
// every internal node R with >= 3 triangles, after all its descendants,
// grows a treelet of up to 7 leaves by opening the leaf with the largest
// surface area (ties: the first), finds the binary topology over those
// leaves with the least surface-area cost by dynamic programming over leaf
// subsets (partitions enumerated downwards, ties: the first), and rebuilds
// the treelet with it when that is cheaper, reusing its internal nodes in
// pre-order.  Cost: internal node Ci * area + children, leaf Ct * area.
// The result depends only on each node's subtree, so any bottom-up order
// (the device's arrival order, this topological order) gives the same tree.
constexpr int kTreeletLeaves = 7, kTreeletPasses = 3;
constexpr float kTreeletCi = 1.2f, kTreeletCt = 1.0f;

static void restructure_treelets(Bvh& b, int n, const std::vector<float>& llo, const std::vector<float>& lhi) {
    const int ni = n - 1;
    if (ni < 2) return;
    auto box = [&](uint32_t c, const float*& lo, const float*& hi) {
        if (c & 0x80000000u) { lo = &llo[3 * (size_t)(c & 0x7fffffffu)]; hi = &lhi[3 * (size_t)(c & 0x7fffffffu)]; }
        else { lo = &b.lo[3 * (size_t)c]; hi = &b.hi[3 * (size_t)c]; }
    };
    std::vector<float> cost(ni, 0.0f);
    auto area_of = [&](uint32_t c) { const float *lo, *hi; box(c, lo, hi); return half_area(lo, hi); };
    auto cost_of = [&](uint32_t c) { return (c & 0x80000000u) ? kTreeletCt * area_of(c) : cost[c]; };
    auto cnt_of = [&](uint32_t c) { return (c & 0x80000000u) ? 1u : b.count[c]; };
    std::vector<int> order(ni);
    for (int pass = 0; pass < kTreeletPasses; ++pass) {
        std::iota(order.begin(), order.end(), 0);
        std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return b.count[x] < b.count[y]; });
        for (int R : order) {
            cost[R] = kTreeletCi * area_of((uint32_t)R) + (cost_of(b.children[2 * (size_t)R]) + cost_of(b.children[2 * (size_t)R + 1]));
            if (b.count[R] < 3) continue;
            uint32_t leaves[kTreeletLeaves], used[kTreeletLeaves - 1];
            int nl = 2, nu = 1;
            leaves[0] = b.children[2 * (size_t)R];
            leaves[1] = b.children[2 * (size_t)R + 1];
            used[0] = (uint32_t)R;
            while (nl < kTreeletLeaves) {
                int bi = -1;
                float ba = 0.0f;
                for (int k = 0; k < nl; ++k) {
                    if (leaves[k] & 0x80000000u) continue;
                    float a = area_of(leaves[k]);
                    if (bi < 0 || a > ba) { bi = k; ba = a; }
                }
                if (bi < 0) break;
                const uint32_t x = leaves[bi];
                used[nu++] = x;
                leaves[bi] = b.children[2 * (size_t)x];
                leaves[nl++] = b.children[2 * (size_t)x + 1];
            }
            const int full = (1 << nl) - 1;
            float sarea[1 << kTreeletLeaves], scost[1 << kTreeletLeaves];
            uint8_t spart[1 << kTreeletLeaves];
            for (int S = 1; S <= full; ++S) {
                float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
                for (int k = 0; k < nl; ++k) {
                    if (!(S >> k & 1)) continue;
                    const float *l, *h;
                    box(leaves[k], l, h);
                    for (int a = 0; a < 3; ++a) {
                        lo[a] = l[a] < lo[a] ? l[a] : lo[a];
                        hi[a] = h[a] > hi[a] ? h[a] : hi[a];
                    }
                }
                sarea[S] = half_area(lo, hi);
            }
            for (int S = 1; S <= full; ++S) {
                if ((S & (S - 1)) == 0) {
                    scost[S] = cost_of(leaves[__builtin_ctz((unsigned)S)]);
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
            if (!(scost[full] < cost[R] * 0.99999f)) continue;
            // internal nodes to subsets in pre-order (left part first)
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
            auto item = [&](int C) { return (C & (C - 1)) == 0 ? leaves[__builtin_ctz((unsigned)C)] : node_of[C]; };
            for (int j = 0; j < ns; ++j) {
                const uint32_t node = node_of[seq[j]];
                b.children[2 * (size_t)node] = item(spart[seq[j]]);
                b.children[2 * (size_t)node + 1] = item(seq[j] ^ spart[seq[j]]);
            }
            for (int j = ns - 1; j >= 0; --j) {
                const uint32_t node = node_of[seq[j]];
                const uint32_t l = b.children[2 * (size_t)node], r = b.children[2 * (size_t)node + 1];
                const float *al, *ah, *bl, *bh;
                box(l, al, ah);
                box(r, bl, bh);
                for (int a = 0; a < 3; ++a) {
                    b.lo[3 * (size_t)node + a] = al[a] < bl[a] ? al[a] : bl[a];
                    b.hi[3 * (size_t)node + a] = ah[a] > bh[a] ? ah[a] : bh[a];
                }
                b.count[node] = cnt_of(l) + cnt_of(r);
                cost[node] = kTreeletCi * half_area(&b.lo[3 * (size_t)node], &b.hi[3 * (size_t)node]) + (cost_of(l) + cost_of(r));
            }
        }
    }
}

static void build_bvh(Scene& s) {
    Bvh& b = s.bvh;
    int n = (int)s.prims.size();
    b.morton.assign(n, 0);
    b.sorted.resize(n);
    if (n == 0) return;
    // centroids and their bounds
    std::vector<float> cen(3 * (size_t)n);
    float cmin[3] = {INFINITY, INFINITY, INFINITY}, cmax[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int i = 0; i < n; ++i) {
        const float* p = &s.wpos[9 * (size_t)i];
        for (int a = 0; a < 3; ++a) {
            float c = (p[a] + p[3 + a] + p[6 + a]) / 3.0f;
            cen[3 * (size_t)i + a] = c;
            cmin[a] = c < cmin[a] ? c : cmin[a];
            cmax[a] = c > cmax[a] ? c : cmax[a];
        }
    }
    for (int i = 0; i < n; ++i) {
        uint32_t q[3];
        for (int a = 0; a < 3; ++a) {
            float ext = cmax[a] - cmin[a];
            float f = ext > 0.0f ? (cen[3 * (size_t)i + a] - cmin[a]) / ext : 0.0f;
            float sc = f * 1024.0f;
            sc = sc < 0.0f ? 0.0f : (sc > 1023.0f ? 1023.0f : sc);
            q[a] = (uint32_t)sc;
        }
        b.morton[i] = (expand_bits(q[0]) << 2) | (expand_bits(q[1]) << 1) | expand_bits(q[2]);
    }
    std::iota(b.sorted.begin(), b.sorted.end(), 0u);
    std::stable_sort(b.sorted.begin(), b.sorted.end(), [&](uint32_t x, uint32_t y) { return b.morton[x] < b.morton[y]; });
    std::vector<uint32_t> keys(n);
    for (int i = 0; i < n; ++i) keys[i] = b.morton[b.sorted[i]];

    // leaf boxes in sorted order
    std::vector<float> llo(3 * (size_t)n), lhi(3 * (size_t)n);
    for (int i = 0; i < n; ++i) {
        const float* p = &s.wpos[9 * (size_t)b.sorted[i]];
        for (int a = 0; a < 3; ++a) {
            float lo = p[a], hi = p[a];
            lo = p[3 + a] < lo ? p[3 + a] : lo; hi = p[3 + a] > hi ? p[3 + a] : hi;
            lo = p[6 + a] < lo ? p[6 + a] : lo; hi = p[6 + a] > hi ? p[6 + a] : hi;
            llo[3 * (size_t)i + a] = lo;
            lhi[3 * (size_t)i + a] = hi;
        }
    }

    int ni = n - 1;
    b.children.assign(2 * (size_t)ni, 0);
    b.first.assign(ni, 0);
    b.count.assign(ni, 0);
    b.lo.assign(3 * (size_t)ni, 0.0f);
    b.hi.assign(3 * (size_t)ni, 0.0f);
    std::vector<int> parent_int(ni, -1), parent_leaf(n, -1);
    for (int i = 0; i < ni; ++i) {
        int d = karras_delta(keys, n, i, i + 1) - karras_delta(keys, n, i, i - 1) >= 0 ? 1 : -1;
        int dmin = karras_delta(keys, n, i, i - d);
        int lmax = 2;
        while (karras_delta(keys, n, i, i + lmax * d) > dmin) lmax *= 2;
        int l = 0;
        for (int t = lmax / 2; t >= 1; t /= 2)
            if (karras_delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
        int j = i + l * d;
        int dnode = karras_delta(keys, n, i, j);
        int sidx = 0;
        int t = l;
        do {
            t = (t + 1) >> 1;
            if (karras_delta(keys, n, i, i + (sidx + t) * d) > dnode) sidx += t;
        } while (t > 1);
        int gamma = i + sidx * d + (d < 0 ? d : 0);
        int lo = i < j ? i : j, hi = i < j ? j : i;
        uint32_t left = (lo == gamma) ? (0x80000000u | (uint32_t)gamma) : (uint32_t)gamma;
        uint32_t right = (hi == gamma + 1) ? (0x80000000u | (uint32_t)(gamma + 1)) : (uint32_t)(gamma + 1);
        b.children[2 * (size_t)i] = left;
        b.children[2 * (size_t)i + 1] = right;
        b.first[i] = lo;
        b.count[i] = hi - lo + 1;
    }
    // boxes bottom-up: children of an internal node always cover a sub-range,
    // so processing nodes by increasing range size is a valid topological order.
    std::vector<int> order(ni);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return b.count[x] < b.count[y]; });
    auto child_box = [&](uint32_t c, const float*& lo, const float*& hi) {
        if (c & 0x80000000u) { lo = &llo[3 * (size_t)(c & 0x7fffffffu)]; hi = &lhi[3 * (size_t)(c & 0x7fffffffu)]; }
        else { lo = &b.lo[3 * (size_t)c]; hi = &b.hi[3 * (size_t)c]; }
    };
    for (int i : order) {
        const float *al, *ah, *bl, *bh;
        child_box(b.children[2 * (size_t)i], al, ah);
        child_box(b.children[2 * (size_t)i + 1], bl, bh);
        for (int a = 0; a < 3; ++a) {
            b.lo[3 * (size_t)i + a] = al[a] < bl[a] ? al[a] : bl[a];
            b.hi[3 * (size_t)i + a] = ah[a] > bh[a] ? ah[a] : bh[a];
        }
    }

    restructure_treelets(b, n, llo, lhi);

    // BVH8 collapse, breadth-first.
    b.nodes.clear();
    b.leaf_prims.clear();
    auto item_count = [&](uint32_t c) -> uint32_t { return (c & 0x80000000u) ? 1u : b.count[c]; };
    auto item_first = [&](uint32_t c) -> uint32_t { return (c & 0x80000000u) ? (c & 0x7fffffffu) : b.first[c]; };
    std::vector<uint32_t> queue;
    if (n == 1) queue.push_back(0x80000000u);  // single leaf root
    else queue.push_back(0u);
    for (size_t k = 0; k < queue.size(); ++k) {
        uint32_t src = queue[k];
        uint32_t kids[8];
        int nk = 0;
        if (src & 0x80000000u) kids[nk++] = src;
        else {
            kids[nk++] = b.children[2 * (size_t)src];
            kids[nk++] = b.children[2 * (size_t)src + 1];
            while (nk < 8) {
                int best = -1;
                float best_area = -1.0f;
                for (int c = 0; c < nk; ++c) {
                    uint32_t it = kids[c];
                    if ((it & 0x80000000u) || b.count[it] <= kLeafMax) continue;
                    float a = half_area(&b.lo[3 * (size_t)it], &b.hi[3 * (size_t)it]);
                    if (best < 0 || a > best_area || (a == best_area && it < kids[best])) { best = c; best_area = a; }
                }
                if (best < 0) break;
                uint32_t it = kids[best];
                for (int c = nk; c > best + 1; --c) kids[c] = kids[c - 1];
                kids[best] = b.children[2 * (size_t)it];
                kids[best + 1] = b.children[2 * (size_t)it + 1];
                ++nk;
            }
        }
        // octant slot assignment: slot bit k set = child centre on the
        // positive side of the node centre along axis k; greedy on the
        // alignment score (ties: lower child position, then lower slot)
        float klo[8][3], khi[8][3];
        for (int c = 0; c < nk; ++c) {
            const float *lo, *hi;
            child_box(kids[c], lo, hi);
            for (int a = 0; a < 3; ++a) { klo[c][a] = lo[a]; khi[c][a] = hi[a]; }
        }
        uint32_t slot_kid[8];
        assign_octant_slots(nk, klo, khi, slot_kid);
        hx_bvh8_node node;
        std::memset(&node, 0, sizeof(node));
        node.child_base = (uint32_t)queue.size();
        node.prim_base = (uint32_t)b.leaf_prims.size();
        float clo[8][3], chi[8][3];
        int rank = 0;
        for (int c = 0; c < 8; ++c) {
            if (slot_kid[c] == 0xffffffffu) {
                for (int a = 0; a < 3; ++a) { clo[c][a] = 0.0f; chi[c][a] = 0.0f; }
                node.meta[c] = kMetaEmpty;
                continue;
            }
            uint32_t it = kids[slot_kid[c]];
            for (int a = 0; a < 3; ++a) { clo[c][a] = klo[slot_kid[c]][a]; chi[c][a] = khi[slot_kid[c]][a]; }
            if (!(it & 0x80000000u) && b.count[it] > kLeafMax) {
                node.meta[c] = (uint8_t)(kMetaInternal | c);
                node.internal_mask |= (uint8_t)(1u << c);
                ++rank;
                queue.push_back(it);
            } else {
                uint32_t cnt = item_count(it), f = item_first(it);
                uint32_t off = (uint32_t)b.leaf_prims.size() - node.prim_base;
                node.meta[c] = (uint8_t)(kMetaLeaf | off);
                for (uint32_t q = 0; q < cnt; ++q) b.leaf_prims.push_back(b.sorted[f + q]);
            }
        }
        quantise_node(node, clo, chi);
        b.nodes.push_back(node);
    }
}

// ---------------------------------------------------------------------------
// Traversal over the binary tree (independent of the BVH8 the device walks).
// ---------------------------------------------------------------------------
static inline uint8_t tex_fetch(const Tex& t, long x, long y, int c) { return t.rgba[((size_t)y * t.w + x) * 4 + c]; }

// A texel channel as a value in [0, 1]: q / 255, or for the RGB of an sRGB
// texture the sRGB transfer function (IEC 61966-2-1, the decode of *_SRGB
// formats), applied before filtering; in FP32 the exact value rounded once.
template <typename R> static R texel_value(uint8_t q, bool srgb, bool snorm = false) {
    if (snorm) return R(std::max((int)(int8_t)q / 127.0, -1.0));  // Vulkan SNORM: max(c / 127, -1)
    if (!srgb) return R(q) / R(255);
    const double c = q / 255.0;
    return R(c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4));
}

// Software bilinear filter, REPEAT addressing, level 0.
template <typename R> static R tex_bilinear(const Tex& t, R u, R v, int c) {
    R x = u * R(t.w) - R(0.5), y = v * R(t.h) - R(0.5);
    R x0 = std::floor(x), y0 = std::floor(y);
    R fx = x - x0, fy = y - y0;
    long W = t.w, H = t.h;
    long ix0 = (((long)x0 % W) + W) % W, iy0 = (((long)y0 % H) + H) % H;
    long ix1 = (ix0 + 1) % W, iy1 = (iy0 + 1) % H;
    const bool srgb = t.srgb && c < 3;
    R a00, a10, a01, a11;
    if (!t.hdr.empty()) {  // half-float texels: their values (the formats have no sRGB variant)
        auto hv = [&](long x, long y) { return R(t.hdr[((size_t)y * t.w + x) * 4 + c]); };
        a00 = hv(ix0, iy0), a10 = hv(ix1, iy0), a01 = hv(ix0, iy1), a11 = hv(ix1, iy1);
    } else {
        const bool sn = t.snorm;
        a00 = texel_value<R>(tex_fetch(t, ix0, iy0, c), srgb, sn), a10 = texel_value<R>(tex_fetch(t, ix1, iy0, c), srgb, sn);
        a01 = texel_value<R>(tex_fetch(t, ix0, iy1, c), srgb, sn), a11 = texel_value<R>(tex_fetch(t, ix1, iy1, c), srgb, sn);
    }
    R top = a00 + (a10 - a00) * fx;
    R bot = a01 + (a11 - a01) * fx;
    return top + (bot - top) * fy;
}

// Any-hit alpha test (path_trace_rahit.glsl:174-188): interpolated UV,
// albedo alpha, reject below 0.1.  Always evaluated in FP32.
static bool alpha_pass(const Scene& s, uint32_t prim, float u, float v) {
    const PrimInfo& pi = s.prims[prim];
    const hx_material& m = s.materials[pi.material];
    float alpha;
    if (m.texture_indices0[0] == -1) alpha = m.albedo[3];
    else {
        uint32_t mesh = s.instances[pi.instance].mesh_index;
        const auto& ix = s.indices[mesh];
        const hx_vertex& a = s.vertices[mesh][ix[3 * pi.mesh_prim]];
        const hx_vertex& b = s.vertices[mesh][ix[3 * pi.mesh_prim + 1]];
        const hx_vertex& c = s.vertices[mesh][ix[3 * pi.mesh_prim + 2]];
        float b0 = 1.0f - u - v;
        float tu = a.tex_coord[0] * b0 + b.tex_coord[0] * u + c.tex_coord[0] * v;
        float tv = a.tex_coord[1] * b0 + b.tex_coord[1] * u + c.tex_coord[1] * v;
        alpha = tex_bilinear<float>(s.textures[m.texture_indices0[0]], tu, tv, 3);
    }
    return !(alpha < 0.1f);
}

template <typename R> static V3<R> prim_vertex(const Scene& s, uint32_t p, int c);
template <> V3<float> prim_vertex<float>(const Scene& s, uint32_t p, int c) {
    const float* q = &s.wpos[9 * (size_t)p + 3 * c];
    return V3<float>(q[0], q[1], q[2]);
}
template <> V3<double> prim_vertex<double>(const Scene& s, uint32_t p, int c) {
    const double* q = &s.wpos64[9 * (size_t)p + 3 * c];
    return V3<double>(q[0], q[1], q[2]);
}

struct HitF {
    float t, u, v;
    uint32_t prim;
};

// Closest hit (any_hit = run the alpha test on non-opaque triangles) or, with
// shadow = true, first accepted hit.  Triangle test in Real, boxes in FP32.
template <typename R>
static bool trace(const Scene& s, V3<R> o, V3<R> d, R tmin, R tmax, bool any_hit, bool shadow, bool brute, R& t_out,
                  R& u_out, R& v_out, uint32_t& prim_out) {
    const Bvh& b = s.bvh;
    uint32_t n = (uint32_t)s.prims.size();
    prim_out = kNoHit;
    if (n == 0) return false;
    RayPre<R> rp = ray_prepare(o, d);
    R best_t = tmax, bu = 0, bv = 0;
    uint32_t best = kNoHit;
    float org[3] = {(float)o.x, (float)o.y, (float)o.z};
    float inv[3] = {safe_inv((float)d.x), safe_inv((float)d.y), safe_inv((float)d.z)};
    auto test = [&](uint32_t p) -> bool {
        R t, u, v;
        if (!intersect_triangle(rp, prim_vertex<R>(s, p, 0), prim_vertex<R>(s, p, 1), prim_vertex<R>(s, p, 2), tmin, best_t, t, u, v))
            return false;
        if (!(t < best_t || (t == best_t && p < best))) return false;
        if (any_hit && s.nonopaque[p] && !alpha_pass(s, p, (float)u, (float)v)) return false;
        best_t = t; bu = u; bv = v; best = p;
        return true;
    };
    if (brute) {
        for (uint32_t p = 0; p < n; ++p)
            if (test(p) && shadow) break;
    } else if (n == 1) {
        test(b.sorted[0]);
    } else {
        uint32_t stack[128];
        int sp = 0;
        stack[sp++] = 0;
        while (sp > 0) {
            uint32_t c = stack[--sp];
            if (c & 0x80000000u) {
                if (test(b.sorted[c & 0x7fffffffu]) && shadow) break;
                continue;
            }
            float tn;
            float lim = (float)best_t * 1.000001f;
            if (!slab_test(inv, org, &b.lo[3 * (size_t)c], &b.hi[3 * (size_t)c], (float)tmin, lim, tn)) continue;
            stack[sp++] = b.children[2 * (size_t)c + 1];
            stack[sp++] = b.children[2 * (size_t)c];
        }
    }
    if (best == kNoHit) return false;
    t_out = best_t; u_out = bu; v_out = bv; prim_out = best;
    return true;
}

// ---------------------------------------------------------------------------
// BVH8 traversal in the device's arithmetic (one FMA per child plane on
// per-node constants widened outward by 2^-21 of their magnitude,
// octant-ordered node groups; trace.cuh axis_slab).  Checks on the CPU that
// the quantised 8-wide tree never loses a hit; not used by the radiance path.
// ---------------------------------------------------------------------------
static bool trace_bvh8_cpu(const Scene& s, V3<float> o, V3<float> d, float tmin, float tmax, bool any_hit, float& t_out,
                           uint32_t& prim_out, uint32_t* node_visits) {
    const Bvh& b = s.bvh;
    prim_out = kNoHit;
    if (b.nodes.empty()) return false;
    RayPre<float> r = ray_prepare(o, d);
    float ix = safe_inv(d.x), iy = safe_inv(d.y), iz = safe_inv(d.z);
    uint32_t oct = (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u);
    uint32_t oct_inv = 7u - oct;
    float best_t = tmax;
    uint32_t best = kNoHit;
    std::vector<std::pair<uint32_t, uint32_t>> stack;
    uint32_t g_base = 0, g_mask = (1u << (24 + oct_inv)) | 1u;
    for (;;) {
        uint32_t t_base = 0, t_mask = 0;
        if (g_mask > 0x00ffffffu) {
            uint32_t bit = 31u - (uint32_t)__builtin_clz(g_mask);
            g_mask &= ~(1u << bit);
            uint32_t slot = (bit - 24u) ^ oct_inv;
            uint32_t child = g_base + (uint32_t)__builtin_popcount(g_mask & 0xffu & ((1u << slot) - 1u));
            if (g_mask > 0x00ffffffu) stack.push_back({g_base, g_mask});
            const hx_bvh8_node& n = b.nodes[child];
            if (node_visits) ++*node_visits;
            uint32_t hits = 0;
            // per axis t = f A + C with f = 1 + q 2^-15 (trace.cuh axis_slab):
            // A = 2^(e+15) inv, b = (g - o) inv, C = b - A -/+ 2^-21 (|b| + |A|)
            const float inv[3] = {ix, iy, iz}, org[3] = {o.x, o.y, o.z};
            float A[3], Cn[3], Cf[3];
            for (int a = 0; a < 3; ++a) {
                A[a] = pow2f(n.exponent[a] + 15) * inv[a];
                const float bb = (n.origin[a] - org[a]) * inv[a];
                const float C = bb - A[a];
                const float delta = (std::fabs(bb) + std::fabs(A[a])) * 4.76837158203125e-7f;
                Cn[a] = C - delta;
                Cf[a] = C + delta;
            }
            float lim = best_t * 1.000001f;
            for (int c = 0; c < 8; ++c) {
                uint32_t m = n.meta[c];
                float tn = tmin, tf = lim;
                float tna[3], tfa[3];
                for (int a = 0; a < 3; ++a) {
                    bool neg = inv[a] < 0.0f;
                    uint32_t qn = neg ? n.qhi[a][c] : n.qlo[a][c], qf = neg ? n.qlo[a][c] : n.qhi[a][c];
                    float un = f32_bits(0x3F800000u | (qn << 8)), uf = f32_bits(0x3F800000u | (qf << 8));
                    tna[a] = std::fma(un, A[a], Cn[a]);
                    tfa[a] = std::fma(uf, A[a], Cf[a]);
                }
                tn = std::fmax(std::fmax(tna[0], tna[1]), std::fmax(tna[2], tmin));
                tf = std::fmin(std::fmin(tfa[0], tfa[1]), std::fmin(tfa[2], lim));
                // hit bit: internal 24 + (slot ^ oct_inv), leaf its offset, empty 16
                uint32_t pos = (m & 0x80u) ? ((m & 31u) ^ oct_inv) : (m & 31u);
                if (tn <= tf) hits |= 1u << pos;
            }
            g_base = n.child_base;
            g_mask = (hits & 0xff000000u) | n.internal_mask;
            t_base = n.prim_base;
            t_mask = hits & 0xffu;
        }
        while (t_mask) {
            uint32_t bt = (uint32_t)__builtin_ctz(t_mask);
            t_mask &= t_mask - 1u;
            uint32_t p = b.leaf_prims[t_base + bt];
            float t, u, v;
            if (!intersect_triangle(r, prim_vertex<float>(s, p, 0), prim_vertex<float>(s, p, 1), prim_vertex<float>(s, p, 2),
                                    tmin, best_t, t, u, v))
                continue;
            if (!(t < best_t || (t == best_t && p < best))) continue;
            if (any_hit && s.nonopaque[p] && !alpha_pass(s, p, u, v)) continue;
            best_t = t;
            best = p;
        }
        if (g_mask <= 0x00ffffffu) {
            if (stack.empty()) break;
            g_base = stack.back().first;
            g_mask = stack.back().second;
            stack.pop_back();
        }
    }
    if (best == kNoHit) return false;
    t_out = best_t;
    prim_out = best;
    return true;
}

// ---------------------------------------------------------------------------
// Shading (brdf.glsl, path_trace_rchit.glsl) in Real precision.
// ---------------------------------------------------------------------------
template <typename R> struct Surface {
    V3<R> position, normal, F0, albedo, emissive;
    R albedo_a, metallic, roughness, alpha, alpha2;
};

template <typename R> static V3<R> rot_mul(V3<R> z, V3<R> t) {  // make_rotation_matrix(z) * t, sampling.glsl:28-36
    V3<R> ref = std::fabs(z.x * R(0) + z.y * R(1) + z.z * R(0)) > R(0.99f) ? V3<R>(0, 0, 1) : V3<R>(0, 1, 0);
    V3<R> x = normalize(cross(ref, z));
    V3<R> y = cross(z, x);
    return x * t.x + y * t.y + z * t.z;
}
template <typename R> static V3<R> sample_cosine_lobe(V3<R> n, R r0, R r1) {  // brdf.glsl:6-18
    R rx = gmax(R(0.00001f), r0), ry = gmax(R(0.00001f), r1);
    R phi = R(2) * kpi<R>() * ry;
    R cos_theta = std::sqrt(rx);
    R sin_theta = std::sqrt(R(1) - rx);
    V3<R> t(sin_theta * std::cos(phi), sin_theta * std::sin(phi), cos_theta);
    return normalize(rot_mul(n, t));
}
template <typename R> static R D_ggx(R ndoth, R alpha) {  // brdf.glsl:58-64
    R a2 = alpha * alpha;
    R denom = (ndoth * ndoth) * (a2 - R(1)) + R(1);
    return a2 / gmax(R(kEpsilon), (kpi<R>() * denom * denom));
}
template <typename R> static R G1_schlick_ggx(R roughness, R ndotv) {  // brdf.glsl:66-71
    R k = ((roughness + R(1)) * (roughness + R(1))) / R(8);
    return ndotv / gmax(R(kEpsilon), (ndotv * (R(1) - k) + k));
}
template <typename R> static V3<R> evaluate_uber(const Surface<R>& p, V3<R> Wo, V3<R> Wh, V3<R> Wi) {  // brdf.glsl:109-121
    R NdotL = gmax(dot(p.normal, Wi), R(0));
    R NdotV = gmax(dot(p.normal, Wo), R(0));
    R NdotH = gmax(dot(p.normal, Wh), R(0));
    R VdotH = gmax(dot(Wi, Wh), R(0));
    const R x = R(1) - VdotH, x2 = x * x;
    R f5 = x2 * x2 * x;  // pow(1 - VdotH, 5.0) as products (the device's order)
    V3<R> F = p.F0 + (V3<R>(R(1)) - p.F0) * f5;
    R D = D_ggx(NdotH, p.roughness * p.roughness);
    R G = G1_schlick_ggx(p.roughness, NdotL) * G1_schlick_ggx(p.roughness, NdotV);
    V3<R> specular = ((F * D) * G) / gmax(R(kEpsilon), (R(4) * NdotL * NdotV));
    V3<R> diffuse = p.albedo / kpi<R>();
    return (V3<R>(R(1)) - F) * diffuse + specular;
}
template <typename R> static R pdf_uber(const Surface<R>& p, V3<R> Wo, V3<R> Wh, V3<R> Wi) {  // brdf.glsl:123-134
    R NdotL = gmax(dot(p.normal, Wi), R(0));
    R NdotH = gmax(dot(p.normal, Wh), R(0));
    R VdotH = gmax(dot(Wi, Wh), R(0));
    (void)Wo;
    R pd = NdotL / kpi<R>();
    R ps = D_ggx(NdotH, p.roughness * p.roughness) * NdotH / gmax(R(kEpsilon), (R(4) * VdotH));
    return pd * (R(1) - R(0.5)) + ps * R(0.5);
}
template <typename R> static V3<R> sample_uber(const Surface<R>& p, V3<R> Wo, RNG rng, V3<R>& Wi, R& pdf) {  // brdf.glsl:136-167
    R alpha = p.roughness * p.roughness;
    R rx = next_float(rng), ry = next_float(rng), rz = next_float(rng);
    V3<R> Wh;
    bool is_specular = false;
    if (rx < R(0.5)) {
        R phi = R(2) * kpi<R>() * ry;  // sample_ggx, brdf.glsl:83-96
        R cos_theta = std::sqrt((R(1) - rz) / (R(1) + (alpha * alpha - R(1)) * rz));
        R sin_theta = std::sqrt(R(1) - cos_theta * cos_theta);
        V3<R> dl(sin_theta * std::cos(phi), sin_theta * std::sin(phi), cos_theta);
        Wh = normalize(rot_mul(p.normal, dl));
        Wi = reflect(-Wo, Wh);
        R NdotL = gmax(dot(p.normal, Wi), R(0));
        R NdotV = gmax(dot(p.normal, Wo), R(0));
        if (NdotL > R(0) && NdotV > R(0)) is_specular = true;
    }
    if (!is_specular) {
        Wi = sample_cosine_lobe(p.normal, ry, rz);
        Wh = normalize(Wo + Wi);
    }
    pdf = pdf_uber(p, Wo, Wh, Wi);
    return evaluate_uber(p, Wo, Wh, Wi);
}

template <typename R> static const hx_vertex& mesh_vertex(const Scene& s, uint32_t mesh, uint32_t mp, int c) {
    return s.vertices[mesh][s.indices[mesh][3 * mp + c]];
}

template <typename R> static Surface<R> populate(const Scene& s, uint32_t prim, float hu, float hv) {  // rchit.glsl:256-280
    const PrimInfo& pi = s.prims[prim];
    const hx_instance& inst = s.instances[pi.instance];
    uint32_t mesh = inst.mesh_index;
    const hx_vertex& a = mesh_vertex<R>(s, mesh, pi.mesh_prim, 0);
    const hx_vertex& b = mesh_vertex<R>(s, mesh, pi.mesh_prim, 1);
    const hx_vertex& c = mesh_vertex<R>(s, mesh, pi.mesh_prim, 2);
    R u = hu, v = hv;
    R b0 = R(1) - u - v, b1 = u, b2 = v;
    auto lerp3 = [&](const float* x, const float* y, const float* z) {
        return V3<R>(R(x[0]) * b0 + R(y[0]) * b1 + R(z[0]) * b2, R(x[1]) * b0 + R(y[1]) * b1 + R(z[1]) * b2,
                     R(x[2]) * b0 + R(y[2]) * b1 + R(z[2]) * b2);
    };
    V3<R> pos = lerp3(a.position, b.position, c.position);
    R tu = R(a.tex_coord[0]) * b0 + R(b.tex_coord[0]) * b1 + R(c.tex_coord[0]) * b2;
    R tv = R(a.tex_coord[1]) * b0 + R(b.tex_coord[1]) * b1 + R(c.tex_coord[1]) * b2;
    V3<R> nrm = normalize(lerp3(a.normal, b.normal, c.normal));
    R M[16], N[16];
    for (int k = 0; k < 16; ++k) { M[k] = inst.model_matrix[k]; N[k] = inst.normal_matrix[k]; }
    R wp[4];
    mat4_mul(M, pos.x, pos.y, pos.z, R(1), wp);
    Surface<R> p;
    p.position = V3<R>(wp[0], wp[1], wp[2]);
    p.normal = mat3_mul(N, nrm);
    const hx_material& m = s.materials[pi.material];
    if (m.texture_indices0[1] != -1) {  // fetch_normal / get_normal_from_map, rchit.glsl:190-219
        V3<R> tan = normalize(lerp3(a.tangent, b.tangent, c.tangent));
        V3<R> bit = normalize(lerp3(a.bitangent, b.bitangent, c.bitangent));
        V3<R> Tm = normalize(mat3_mul(N, tan)), Bm = normalize(mat3_mul(N, bit)), Nm = normalize(p.normal);
        const Tex& nt = s.textures[m.texture_indices0[1]];
        V3<R> mp(tex_bilinear<R>(nt, tu, tv, 0), tex_bilinear<R>(nt, tu, tv, 1), tex_bilinear<R>(nt, tu, tv, 2));
        V3<R> nm = normalize(mp * R(2) - V3<R>(R(1)));
        p.normal = normalize(V3<R>(Tm.x * nm.x + Bm.x * nm.y + Nm.x * nm.z, Tm.y * nm.x + Bm.y * nm.y + Nm.y * nm.z,
                                   Tm.z * nm.x + Bm.z * nm.y + Nm.z * nm.z));
    }
    if (m.texture_indices0[0] == -1) {
        p.albedo = V3<R>(R(m.albedo[0]), R(m.albedo[1]), R(m.albedo[2]));
        p.albedo_a = R(m.albedo[3]);
    } else {
        const Tex& t = s.textures[m.texture_indices0[0]];
        p.albedo = V3<R>(tex_bilinear<R>(t, tu, tv, 0), tex_bilinear<R>(t, tu, tv, 1), tex_bilinear<R>(t, tu, tv, 2));
        p.albedo_a = tex_bilinear<R>(t, tu, tv, 3);
    }
    p.roughness = m.texture_indices0[2] == -1 ? R(m.roughness_metallic[0])
                                               : tex_bilinear<R>(s.textures[m.texture_indices0[2]], tu, tv, m.texture_indices1[2]);
    p.metallic = m.texture_indices0[3] == -1 ? R(m.roughness_metallic[1])
                                              : tex_bilinear<R>(s.textures[m.texture_indices0[3]], tu, tv, m.texture_indices1[3]);
    if (m.texture_indices1[0] == -1) p.emissive = V3<R>(R(m.emissive[0]), R(m.emissive[1]), R(m.emissive[2]));
    else {
        const Tex& t = s.textures[m.texture_indices1[0]];
        p.emissive = V3<R>(tex_bilinear<R>(t, tu, tv, 0), tex_bilinear<R>(t, tu, tv, 1), tex_bilinear<R>(t, tu, tv, 2));
    }
    p.roughness = gmax(p.roughness, R(kMinRoughness));
    p.F0 = V3<R>(R(0.03f)) * (R(1) - p.metallic) + p.albedo * p.metallic;  // mix(x, y, a) = x(1-a) + ya
    p.alpha = p.roughness * p.roughness;
    p.alpha2 = p.alpha * p.alpha;
    return p;
}

// HX_RAY_OFFSET_SCALED (the library's own policy, not the reference's): the
// world-space geometric normal of a hit triangle (object-space edge cross
// product through the normal matrix) and the ray origin moved off the surface
// along it, to the side of the outgoing direction, by n_i (2^-15 |p_i| + 2^-16)
// per coordinate — a continuous form of Waechter and Binder's self-intersection
// offset (Ray Tracing Gems, 2019, ch. 6).  Same operation order as the device.
template <typename R> static V3<R> geo_normal(const Scene& s, uint32_t prim) {
    const PrimInfo& pi = s.prims[prim];
    const hx_instance& inst = s.instances[pi.instance];
    const hx_vertex& a = mesh_vertex<R>(s, inst.mesh_index, pi.mesh_prim, 0);
    const hx_vertex& b = mesh_vertex<R>(s, inst.mesh_index, pi.mesh_prim, 1);
    const hx_vertex& c = mesh_vertex<R>(s, inst.mesh_index, pi.mesh_prim, 2);
    V3<R> e1(R(b.position[0]) - R(a.position[0]), R(b.position[1]) - R(a.position[1]), R(b.position[2]) - R(a.position[2]));
    V3<R> e2(R(c.position[0]) - R(a.position[0]), R(c.position[1]) - R(a.position[1]), R(c.position[2]) - R(a.position[2]));
    R N[16];
    for (int k = 0; k < 16; ++k) N[k] = inst.normal_matrix[k];
    return normalize(mat3_mul(N, cross(e1, e2)));
}
template <typename R> static V3<R> offset_origin(V3<R> p, V3<R> ng, V3<R> dir) {
    const V3<R> n = dot(ng, dir) < R(0) ? -ng : ng;
    const R rel = R(3.0517578125e-5f), ab = R(1.52587890625e-5f);  // 2^-15, 2^-16
    return V3<R>(p.x + n.x * (std::fabs(p.x) * rel + ab), p.y + n.y * (std::fabs(p.y) * rel + ab),
                 p.z + n.z * (std::fabs(p.z) * rel + ab));
}

struct Params {
    uint32_t width, height, max_bounces;
    float shadow_bias;
    hx_policy pol;
};

struct Counters {
    uint64_t paths = 0, ext = 0, shadow = 0;
};

template <typename R> static V3<R> fv3(const float* f) { return V3<R>(R(f[0]), R(f[1]), R(f[2])); }

// sample_light (path_trace_rchit.glsl:284-451).  Returns Li (before
// visibility); sets Wi, pdf, the shadow-ray tmax and whether to trace.
template <typename R>
static V3<R> sample_light(const Scene& s, const Params& P, const Surface<R>& p, const hx_light& light, RNG& rng, V3<R>& Wi,
                          R& pdf, R& tmax, bool& trace_it) {
    tmax = R(10000.0f);
    trace_it = true;
    uint32_t type = (uint32_t)light.data0[0];
    V3<R> Li(R(0));
    Wi = V3<R>(R(0));
    pdf = R(0);
    if (type == HX_LIGHT_DIRECTIONAL || type == HX_LIGHT_SPOT || type == HX_LIGHT_POINT) {
        R r0 = next_float(rng), r1 = next_float(rng);
        V3<R> light_dir, to_light;
        R light_distance = 0, light_radius;
        if (type == HX_LIGHT_DIRECTIONAL) {
            light_dir = -fv3<R>(light.data1);
            light_radius = R(light.data2[3]);
        } else {
            to_light = fv3<R>(light.data2) - p.position;
            light_dir = normalize(to_light);
            light_distance = length(to_light);
            light_radius = R(light.data2[3]) / light_distance;
        }
        V3<R> lt = normalize(cross(light_dir, V3<R>(0, 1, 0)));
        V3<R> lb = normalize(cross(lt, light_dir));
        R point_radius = light_radius * std::sqrt(r0);
        R point_angle = r1 * R(2) * kpi<R>();
        R dx = point_radius * std::cos(point_angle), dy = point_radius * std::sin(point_angle);
        Wi = normalize(light_dir + lt * dx + lb * dy);
        V3<R> col = V3<R>(R(light.data0[1]), R(light.data0[2]), R(light.data0[3]));
        R intensity = R(light.data1[3]);
        if (type == HX_LIGHT_DIRECTIONAL) Li = col * intensity;
        else if (type == HX_LIGHT_POINT) Li = col * intensity / (light_distance * light_distance);
        else {
            R att = dot(light_dir, -fv3<R>(light.data1));
            R e0 = R(light.data3[1]), e1 = R(light.data3[0]);
            // smoothstep(outer, inner, x); equal edges (resource_manager.cpp:592) act as a step
            if (e1 == e0) att = att < e0 ? R(0) : R(1);
            else {
                R tt = gclamp((att - e0) / (e1 - e0), R(0), R(1));
                att = tt * tt * (R(3) - R(2) * tt);
            }
            Li = col * intensity * att / (light_distance * light_distance);
        }
        pdf = R(0);
        if (type != HX_LIGHT_DIRECTIONAL) tmax = light_distance;
    } else if (type == HX_LIGHT_ENVIRONMENT) {
        R r0 = next_float(rng), r1 = next_float(rng);
        if (P.pol.env_sampling == HX_ENV_SAMPLE_IMPORTANCE && s.env_kind != HX_ENV_NONE) {
            Wi = env_sample<R>(s, (float)r0, (float)r1, pdf);
            Li = env_lookup(s, Wi);
            if (!(pdf > R(0))) { Li = V3<R>(R(0)); trace_it = false; }
        } else {
            Wi = sample_cosine_lobe(p.normal, r0, r1);
            Li = env_lookup(s, Wi);
            pdf = dot(p.normal, Wi) / kpi<R>();
        }
    } else if (type == HX_LIGHT_AREA) {
        uint32_t inst_id = (uint32_t)light.data0[1];
        uint32_t num_tris = P.pol.area_count_from_x ? (uint32_t)light.data1[0] : (uint32_t)light.data1[2];
        uint32_t prim_id = next_uint(rng, num_tris);
        uint32_t mat = (uint32_t)light.data0[2];
        uint32_t mp = prim_id + (uint32_t)light.data0[3];
        const hx_instance& inst = s.instances[inst_id];
        uint32_t mesh = inst.mesh_index;
        R r0 = next_float(rng), r1 = next_float(rng);
        R su0 = std::sqrt(r0);  // uniform_sample_triangle, brdf.glsl:40-44
        R bx = R(1) - su0, by = r1 * su0;
        R M[16], N[16];
        for (int k = 0; k < 16; ++k) { M[k] = inst.model_matrix[k]; N[k] = inst.normal_matrix[k]; }
        V3<R> P3[3], N3[3];
        for (int c = 0; c < 3; ++c) {
            const hx_vertex& v = mesh_vertex<R>(s, mesh, mp, c);
            R w = P.pol.area_w_one ? R(1) : R(v.position[3]);
            R o[4];
            mat4_mul(M, R(v.position[0]), R(v.position[1]), R(v.position[2]), w, o);
            P3[c] = V3<R>(o[0], o[1], o[2]);
            N3[c] = fv3<R>(v.normal);
        }
        R c0 = R(1) - bx - by;  // barycentric_interpolate, brdf.glsl:46-51
        V3<R> light_pos = P3[0] * c0 + P3[1] * bx + P3[2] * by;
        V3<R> light_normal = normalize(mat3_mul(N, N3[0] * c0 + N3[1] * bx + N3[2] * by));
        V3<R> light_dir = p.position - light_pos;
        R dist_sqr = dot(light_dir, light_dir);
        R area = R(0.5) * length(cross(P3[1] - P3[0], P3[2] - P3[0]));
        if (area == R(0) || dist_sqr == R(0)) { trace_it = false; return V3<R>(R(0)); }
        R dist = std::sqrt(dist_sqr);
        light_dir = light_dir / dist;
        tmax = gmax(R(0), dist - R(kEpsilon));
        R cos_theta = dot(light_normal, light_dir);
        if (cos_theta == R(0)) { trace_it = false; return V3<R>(R(0)); }
        const hx_material& m = s.materials[mat];
        Li = V3<R>(R(m.emissive[0]), R(m.emissive[1]), R(m.emissive[2]));
        Wi = -light_dir;
        pdf = dist_sqr / gmax(R(kEpsilon), cos_theta * area);  // pdf_triangle
    }
    return Li;
}

template <typename R>
static void generate_ray(const hx_frame_desc& f, uint32_t x, uint32_t y, uint32_t W, uint32_t H, RNG& rng, V3<R>& org,
                         V3<R>& dir) {  // path_trace_rgen.glsl:132-174
    R px = R((float)x) + R(0.5), py = R((float)y) + R(0.5);
    R jx = next_float(rng), jy = next_float(rng);
    R tx = (px + jx) / R((float)W), ty = (py + jy) / R((float)H);
    R nx = tx * R(2) - R(1), ny = ty * R(2) - R(1);
    R m[16];
    for (int k = 0; k < 16; ++k) m[k] = f.view_proj_inverse[k];
    R tg[4];
    mat4_mul(m, nx, ny, R(0), R(1), tg);
    R tw = tg[3];
    V3<R> target(tg[0] / tw, tg[1] / tw, tg[2] / tw);
    V3<R> cam = fv3<R>(f.camera_pos);
    R angle = R(next_float(rng)) * R(2) * kpi<R>();
    R radius = std::sqrt(R(next_float(rng)));
    R ap = R(f.aperture_radius);
    R ox = std::cos(angle) * radius * ap, oy = std::sin(angle) * radius * ap;
    V3<R> aperture_pos = cam + fv3<R>(f.right_direction) * ox + fv3<R>(f.up_direction) * oy;
    V3<R> rdir = -normalize(target - cam);
    V3<R> fp = fv3<R>(f.focal_plane);
    R t = -(dot(cam, fp) + R(f.focal_plane[3])) / dot(rdir, fp);
    V3<R> focus = cam + rdir * t;
    org = aperture_pos;
    dir = normalize(focus - aperture_pos);
}

// 16-bit payload emulation (precision form): ray directions travel as two
// 16-bit snorm octahedral coordinates and hit barycentrics as FP16, exactly
// like the device queues; the arithmetic below matches the device codec.
static uint32_t snorm16_f(float x) {
    float q = std::rint(std::fmin(std::fmax(x, -1.0f), 1.0f) * 32767.0f);
    return (uint32_t)(int32_t)q & 0xffffu;
}
static float unsnorm16_f(uint32_t b) { return (float)(int32_t)(int16_t)(uint16_t)b / 32767.0f; }
static uint32_t oct_encode_f(V3<float> d) {
    float l1 = std::fabs(d.x) + std::fabs(d.y) + std::fabs(d.z);
    float u = d.x / l1, v = d.y / l1;
    if (d.z < 0.0f) {
        float nu = (1.0f - std::fabs(v)) * (u >= 0.0f ? 1.0f : -1.0f);
        float nv = (1.0f - std::fabs(u)) * (v >= 0.0f ? 1.0f : -1.0f);
        u = nu;
        v = nv;
    }
    return snorm16_f(u) | (snorm16_f(v) << 16);
}
static V3<float> oct_decode_f(uint32_t b) {
    float u = unsnorm16_f(b & 0xffffu), v = unsnorm16_f(b >> 16);
    float z = 1.0f - std::fabs(u) - std::fabs(v);
    if (z < 0.0f) {
        float nu = (1.0f - std::fabs(v)) * (u >= 0.0f ? 1.0f : -1.0f);
        float nv = (1.0f - std::fabs(u)) * (v >= 0.0f ? 1.0f : -1.0f);
        u = nu;
        v = nv;
    }
    return normalize(V3<float>(u, v, z));
}
template <typename R> static V3<R> payload_dir(V3<R> d) {
    V3<float> f = oct_decode_f(oct_encode_f(V3<float>((float)d.x, (float)d.y, (float)d.z)));
    return V3<R>(R(f.x), R(f.y), R(f.z));
}
static float payload_bary(float x) { return half_to_float(float_to_half(x)); }

// One camera sample: ray-gen + the closest-hit recursion unrolled into a
// loop (the payload recursion of path_trace_rchit.glsl:487-536 sums L in the
// same order: emission, direct light, then the deeper bounces).
// Ray-debug launch (RAY_DEBUG_VIEW): the path is launch (ray, 0) of a
// num_rays x 1 launch through pixel (x, y); its colour takes three draws
// first (path_trace_rgen.glsl:183-188) and every hit after the camera ray
// appends a segment (origin, hit point) with that colour
// (path_trace_rchit.glsl:548-567).
struct DebugPath {
    uint32_t ray, num_rays;
    std::vector<float>* verts;  // 8 floats per vertex: position xyz1, colour rgb1
};

template <typename R>
static V3<R> trace_path(const Scene& s, const Params& P, const hx_frame_desc& f, uint32_t x, uint32_t y, uint32_t frame,
                        Counters& cnt, hx_hit* primary, const DebugPath* dbg = nullptr) {
    RNG rng = dbg ? rng_init(P.pol.rng, dbg->ray, 0, dbg->num_rays, frame) : rng_init(P.pol.rng, x, y, P.width, frame);
    float dcol[3] = {0.0f, 0.0f, 0.0f};
    if (dbg)
        for (int k = 0; k < 3; ++k) dcol[k] = next_float(rng) * 0.5f + 0.5f;
    V3<R> L(R(0)), T(R(1));
    uint32_t depth = 0;
    V3<R> o, d;
    generate_ray<R>(f, x, y, P.width, P.height, rng, o, d);
    const bool fp16 = P.pol.payload == HX_PAYLOAD_FP16;
    if (fp16) d = payload_dir(d);
    R tmin = R(0.001f), tmax = R(10000.0f);
    bool any_hit = true;
    uint32_t num_lights = (uint32_t)s.lights.size();
    cnt.paths++;
    for (;;) {
        R t, hu, hv;
        uint32_t prim;
        cnt.ext++;
        bool hit = trace<R>(s, o, d, tmin, tmax, any_hit, false, false, t, hu, hv, prim);
        if (depth == 0 && primary) {
            primary->t = hit ? (float)t : 0.0f;
            primary->prim = hit ? prim : kNoHit;
            primary->u = hit ? (float)hu : 0.0f;
            primary->v = hit ? (float)hv : 0.0f;
        }
        if (!hit) {  // path_trace_rmiss.glsl:60-65
            V3<R> e = env_lookup(s, d);
            L = L + (depth == 0 ? e : T * e);
            break;
        }
        if (dbg && depth > 0) {
            const float seg[16] = {(float)o.x, (float)o.y, (float)o.z, 1.0f, dcol[0], dcol[1], dcol[2], 1.0f,
                                   (float)(o.x + d.x * t), (float)(o.y + d.y * t), (float)(o.z + d.z * t), 1.0f,
                                   dcol[0], dcol[1], dcol[2], 1.0f};
            dbg->verts->insert(dbg->verts->end(), seg, seg + 16);
        }
        float su = (float)hu, sv = (float)hv;
        if (fp16) {
            su = payload_bary(su);
            sv = payload_bary(sv);
        }
        Surface<R> p = populate<R>(s, prim, su, sv);
        if (depth == 0 && !is_black(p.emissive)) L = L + p.emissive;
        V3<R> Wo = -d;
        if (num_lights > 0) {  // direct_lighting, rchit.glsl:455-483
            uint32_t li = next_uint(rng, num_lights);
            V3<R> Wi;
            R pdf, stmax;
            bool trace_it;
            V3<R> Li = sample_light<R>(s, P, p, s.lights[li], rng, Wi, pdf, stmax, trace_it);
            if (trace_it && !is_black(Li)) {
                V3<R> Wh = normalize(Wo + Wi);
                V3<R> brdf = evaluate_uber(p, Wo, Wh, Wi);
                R cos_theta = gclamp(dot(p.normal, Wi), R(0), R(1));
                V3<R> so = p.position + p.normal * R(P.shadow_bias);
                if (P.pol.ray_offset == HX_RAY_OFFSET_SCALED) {
                    const V3<R> oo = offset_origin(so, geo_normal<R>(s, prim), Wi);
                    stmax = stmax - (std::fabs(oo.x - so.x) + std::fabs(oo.y - so.y) + std::fabs(oo.z - so.z));
                    so = oo;
                }
                R st, su, sv;
                uint32_t sp;
                cnt.shadow++;
                bool occluded = trace<R>(s, so, Wi, R(0.0001f), stmax, depth == 0, true, false, st, su, sv, sp);
                if (!occluded) {
                    V3<R> c = ((T * brdf) * cos_theta) * Li;
                    if (pdf != R(0)) c = c / pdf;
                    L = L + c * R((float)num_lights);
                }
            }
        }
        if (!((depth + 1) < P.max_bounces)) break;
        // indirect_lighting, rchit.glsl:487-536
        V3<R> Wi;
        R pdf;
        V3<R> brdf = sample_uber(p, Wo, rng, Wi, pdf);
        R cos_theta = gclamp(dot(p.normal, Wi), R(0), R(1));
        V3<R> Tn = (T * (brdf * cos_theta)) / pdf;
        if (depth >= P.pol.rr_start_depth) {
            R prob = gmax(Tn.x, gmax(Tn.y, Tn.z));
            if (P.pol.rr_clamp) prob = gmin(prob, R(1));
            if (R(next_float(rng)) > prob) break;
            Tn = Tn * (R(1) / prob);
        }
        T = Tn;
        depth++;
        o = P.pol.ray_offset == HX_RAY_OFFSET_SCALED ? offset_origin(p.position, geo_normal<R>(s, prim), Wi) : p.position;
        d = fp16 ? payload_dir(Wi) : Wi;
        tmin = R(0.0001f);
        tmax = R(10000.0f);
        any_hit = false;
    }
    return L;
}

static Params make_params(const hx_integrator_desc& d, uint32_t num_lights) {
    (void)num_lights;
    Params P;
    P.width = d.width;
    P.height = d.height;
    P.max_bounces = d.max_ray_bounces;
    P.shadow_bias = d.shadow_ray_bias;
    P.pol = d.policy;
    return P;
}

}  // namespace oracle

using namespace oracle;

// ---------------------------------------------------------------------------
// C ABI for the tests (ctypes).
// ---------------------------------------------------------------------------
extern "C" {

struct oracle_counters {
    uint64_t paths, extension_rays, shadow_rays;
    double seconds;
    int threads;
};

// Textures must be RGBA8 (UNORM, sRGB or SNORM) or RGBA16F (the oracle does
// not restate the block decoders; those are pinned by oracle/texture_ref.py):
// NULL otherwise.
void* oracle_scene_create(const hx_scene_desc* d) {
    for (uint32_t t = 0; t < d->num_textures; ++t)
        if (d->textures[t].format != HX_TEXTURE_RGBA8 && d->textures[t].format != HX_TEXTURE_RGBA16F &&
            d->textures[t].format != HX_TEXTURE_RGBA8_SNORM)
            return nullptr;
    Scene* s = new Scene();
    for (uint32_t m = 0; m < d->num_meshes; ++m) {
        const hx_mesh_desc& md = d->meshes[m];
        s->vertices.emplace_back(md.vertices, md.vertices + md.num_vertices);
        s->indices.emplace_back(md.indices, md.indices + md.num_indices);
        s->submeshes.emplace_back(md.submeshes, md.submeshes + md.num_submeshes);
    }
    s->instances.assign(d->instances, d->instances + d->num_instances);
    s->materials.assign(d->materials, d->materials + d->num_materials);
    for (uint32_t t = 0; t < d->num_textures; ++t) {
        Tex tx;
        tx.w = d->textures[t].width;
        tx.h = d->textures[t].height;
        if (d->textures[t].format == HX_TEXTURE_RGBA16F) {
            const uint8_t* b = d->textures[t].rgba8;
            tx.hdr.resize((size_t)tx.w * tx.h * 4);
            for (size_t i = 0; i < tx.hdr.size(); ++i) tx.hdr[i] = half_to_float((uint16_t)(b[2 * i] | (b[2 * i + 1] << 8)));
        } else {
            tx.rgba.assign(d->textures[t].rgba8, d->textures[t].rgba8 + (size_t)tx.w * tx.h * 4);
        }
        tx.srgb = d->textures[t].srgb != 0;
        tx.snorm = d->textures[t].format == HX_TEXTURE_RGBA8_SNORM;
        s->textures.push_back(std::move(tx));
    }
    s->punctual.assign(d->punctual_lights, d->punctual_lights + d->num_punctual_lights);
    const hx_environment_desc& e = d->environment;
    s->env_kind = e.kind;
    if (e.kind != HX_ENV_NONE) {
        s->env_w = e.width;
        s->env_h = e.height;
        s->env.resize((size_t)e.width * e.height * 3);
        std::memcpy(s->coeffs, e.coeffs, sizeof(s->coeffs));
        for (int a = 0; a < 3; ++a) s->sun[a] = e.sun_direction[a];
        for (uint32_t j = 0; j < e.height; ++j)
            for (uint32_t i = 0; i < e.width; ++i) {
                size_t k = (size_t)j * e.width + i;
                float rgb[3];
                if (e.kind == HX_ENV_EQUIRECT) {
                    for (int c = 0; c < 3; ++c) rgb[c] = e.rgba32f[k * 4 + c];
                } else {
                    V3<double> dir = latlong_dir((i + 0.5) / e.width, (j + 0.5) / e.height);
                    V3<double> sun((double)e.sun_direction[0], (double)e.sun_direction[1], (double)e.sun_direction[2]);
                    V3<double> r = sky_radiance<double>(e.coeffs, dir, sun);
                    for (int c = 0; c < 3; ++c) rgb[c] = (float)r[c];
                }
                for (int c = 0; c < 3; ++c) s->env[k * 3 + c] = half_to_float(float_to_half(rgb[c]));
            }
        build_env_cdf(*s);
    }
    flatten(*s);
    build_lights(*s);
    build_bvh(*s);
    return s;
}

void oracle_scene_destroy(void* h) { delete (Scene*)h; }

uint32_t oracle_scene_num_prims(void* h) { return (uint32_t)((Scene*)h)->prims.size(); }
uint32_t oracle_scene_num_bvh8_nodes(void* h) { return (uint32_t)((Scene*)h)->bvh.nodes.size(); }
uint32_t oracle_scene_num_lights(void* h) { return (uint32_t)((Scene*)h)->lights.size(); }

void oracle_scene_lights(void* h, hx_light* out) {
    Scene* s = (Scene*)h;
    std::memcpy(out, s->lights.data(), s->lights.size() * sizeof(hx_light));
}

void oracle_scene_env(void* h, float* out_rgb) {
    Scene* s = (Scene*)h;
    std::memcpy(out_rgb, s->env.data(), s->env.size() * sizeof(float));
}

void oracle_bvh_export(void* h, uint32_t* morton, uint32_t* sorted, uint32_t* children, void* nodes, uint32_t* leaf_prims) {
    Scene* s = (Scene*)h;
    const Bvh& b = s->bvh;
    if (morton) std::memcpy(morton, b.morton.data(), b.morton.size() * 4);
    if (sorted) std::memcpy(sorted, b.sorted.data(), b.sorted.size() * 4);
    if (children) std::memcpy(children, b.children.data(), b.children.size() * 4);
    if (nodes) std::memcpy(nodes, b.nodes.data(), b.nodes.size() * sizeof(hx_bvh8_node));
    if (leaf_prims) std::memcpy(leaf_prims, b.leaf_prims.data(), b.leaf_prims.size() * 4);
}

void oracle_trace(void* h, const float* rays, uint32_t n, uint32_t any_hit, uint32_t brute, hx_hit* out) {
    Scene* s = (Scene*)h;
#pragma omp parallel for schedule(dynamic, 64)
    for (long i = 0; i < (long)n; ++i) {
        const float* r = &rays[8 * (size_t)i];
        float t, u, v;
        uint32_t p;
        bool hit = trace<float>(*s, V3<float>(r[0], r[1], r[2]), V3<float>(r[4], r[5], r[6]), r[3], r[7], any_hit != 0, false,
                                brute != 0, t, u, v, p);
        out[i].t = hit ? t : 0.0f;
        out[i].prim = hit ? p : kNoHit;
        out[i].u = hit ? u : 0.0f;
        out[i].v = hit ? v : 0.0f;
    }
}

// Closest hits through the BVH8 in the device arithmetic (CPU check of the
// quantised tree); node_visits (optional) accumulates node fetches.
void oracle_trace_bvh8(void* h, const float* rays, uint32_t n, uint32_t any_hit, hx_hit* out, uint64_t* node_visits) {
    Scene* s = (Scene*)h;
    uint64_t total = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : total)
    for (long i = 0; i < (long)n; ++i) {
        const float* r = &rays[8 * (size_t)i];
        float t = 0.0f;
        uint32_t p, nv = 0;
        bool hit = trace_bvh8_cpu(*s, V3<float>(r[0], r[1], r[2]), V3<float>(r[4], r[5], r[6]), r[3], r[7], any_hit != 0, t, p, &nv);
        out[i].t = hit ? t : 0.0f;
        out[i].prim = hit ? p : kNoHit;
        out[i].u = 0.0f;
        out[i].v = 0.0f;
        total += nv;
    }
    if (node_visits) *node_visits = total;
}

void oracle_primary_rays(const hx_integrator_desc* d, const hx_frame_desc* f, uint32_t frame, float* out) {
    Params P = make_params(*d, 0);
    for (uint32_t y = 0; y < d->height; ++y)
        for (uint32_t x = 0; x < d->width; ++x) {
            RNG rng = rng_init(P.pol.rng, x, y, P.width, frame);
            V3<float> o, dir;
            generate_ray<float>(*f, x, y, P.width, P.height, rng, o, dir);
            float* r = &out[8 * ((size_t)y * d->width + x)];
            r[0] = o.x; r[1] = o.y; r[2] = o.z; r[3] = 0.001f;
            r[4] = dir.x; r[5] = dir.y; r[6] = dir.z; r[7] = 10000.0f;
        }
}

// Output-buffer views (renderer.cpp:491-545, debug_visualization.vert:54-64,
// debug_visualization.frag:71-161): a camera ray through each pixel centre,
// the closest triangle without alpha test, the fragment shader's value;
// misses (0, 0, 0, 1); display row r = camera row H - 1 - r.  FP32, the
// device's operation order.  which: 0 albedo, 1 normals, 2 roughness,
// 3 metallic, 4 emissive.
void oracle_output_view(void* h, const hx_frame_desc* f, uint32_t W, uint32_t H, uint32_t which, float* out) {
    Scene* s = (Scene*)h;
#pragma omp parallel for schedule(dynamic, 4)
    for (long row = 0; row < (long)H; ++row) {
        const uint32_t y = H - 1 - (uint32_t)row;
        for (uint32_t x = 0; x < W; ++x) {
            float* o = &out[4 * ((size_t)row * W + x)];
            const float tx = ((float)x + 0.5f) / (float)W, ty = ((float)y + 0.5f) / (float)H;
            const float nx = tx * 2.0f - 1.0f, ny = ty * 2.0f - 1.0f;
            float tg[4];
            mat4_mul(f->view_proj_inverse, nx, ny, 0.0f, 1.0f, tg);
            const V3<float> target(tg[0] / tg[3], tg[1] / tg[3], tg[2] / tg[3]);
            const V3<float> cam = fv3<float>(f->camera_pos);
            const V3<float> d = normalize(target - cam);
            float t, u, v;
            uint32_t prim;
            o[0] = o[1] = o[2] = 0.0f;
            o[3] = 1.0f;
            if (!trace<float>(*s, cam, d, 0.001f, 10000.0f, false, false, false, t, u, v, prim)) continue;
            const PrimInfo& pi = s->prims[prim];
            const hx_instance& inst = s->instances[pi.instance];
            const uint32_t mesh = inst.mesh_index;
            const hx_vertex& a = mesh_vertex<float>(*s, mesh, pi.mesh_prim, 0);
            const hx_vertex& b = mesh_vertex<float>(*s, mesh, pi.mesh_prim, 1);
            const hx_vertex& c = mesh_vertex<float>(*s, mesh, pi.mesh_prim, 2);
            const float b0 = 1.0f - u - v, b1 = u, b2 = v;
            const float tu = a.tex_coord[0] * b0 + b.tex_coord[0] * b1 + c.tex_coord[0] * b2;
            const float tv = a.tex_coord[1] * b0 + b.tex_coord[1] * b1 + c.tex_coord[1] * b2;
            const hx_material& m = s->materials[pi.material];
            V3<float> r(0.0f, 0.0f, 0.0f);
            auto rgb = [&](int tex) {
                const Tex& tt = s->textures[tex];
                return V3<float>(tex_bilinear<float>(tt, tu, tv, 0), tex_bilinear<float>(tt, tu, tv, 1),
                                 tex_bilinear<float>(tt, tu, tv, 2));
            };
            if (which == 0) {
                r = m.texture_indices0[0] == -1 ? V3<float>(m.albedo[0], m.albedo[1], m.albedo[2]) : rgb(m.texture_indices0[0]);
            } else if (which == 1) {
                const float* N = inst.normal_matrix;
                // FS_IN_* = interpolated normalize(mat3(normal_matrix) x) per vertex
                auto lerp_n = [&](const float* x0, const float* x1, const float* x2) {
                    const V3<float> na = normalize(mat3_mul(N, V3<float>(x0[0], x0[1], x0[2])));
                    const V3<float> nb = normalize(mat3_mul(N, V3<float>(x1[0], x1[1], x1[2])));
                    const V3<float> nc = normalize(mat3_mul(N, V3<float>(x2[0], x2[1], x2[2])));
                    return V3<float>(na.x * b0 + nb.x * b1 + nc.x * b2, na.y * b0 + nb.y * b1 + nc.y * b2,
                                     na.z * b0 + nb.z * b1 + nc.z * b2);
                };
                V3<float> nn = lerp_n(a.normal, b.normal, c.normal);
                if (m.texture_indices0[1] != -1) {  // debug_visualization.frag:77-90
                    const V3<float> T = normalize(lerp_n(a.tangent, b.tangent, c.tangent));
                    const V3<float> B = normalize(lerp_n(a.bitangent, b.bitangent, c.bitangent));
                    const V3<float> Nn = normalize(nn);
                    const V3<float> mp = rgb(m.texture_indices0[1]);
                    const V3<float> nm = normalize(mp * 2.0f - V3<float>(1.0f));
                    nn = normalize(V3<float>(T.x * nm.x + B.x * nm.y + Nn.x * nm.z, T.y * nm.x + B.y * nm.y + Nn.y * nm.z,
                                             T.z * nm.x + B.z * nm.y + Nn.z * nm.z));
                }
                r = nn * 0.5f + V3<float>(0.5f);
            } else if (which == 2) {
                r = V3<float>(m.texture_indices0[2] == -1
                                  ? m.roughness_metallic[0]
                                  : tex_bilinear<float>(s->textures[m.texture_indices0[2]], tu, tv, m.texture_indices1[2]));
            } else if (which == 3) {
                r = V3<float>(m.texture_indices0[3] == -1
                                  ? m.roughness_metallic[1]
                                  : tex_bilinear<float>(s->textures[m.texture_indices0[3]], tu, tv, m.texture_indices1[3]));
            } else {
                r = m.texture_indices1[0] == -1 ? V3<float>(m.emissive[0], m.emissive[1], m.emissive[2]) : rgb(m.texture_indices1[0]);
            }
            o[0] = r.x;
            o[1] = r.y;
            o[2] = r.z;
        }
    }
}

// Ray-debug capture (gather_debug_rays, path_integrator.cpp:88-104): the
// segments of num_rays FP32 paths through display pixel (px, py) (launch row
// height - py), seeded with sample index `frame`; out gets 8 floats per
// vertex, paths in order; returns the vertex count (at most capacity copied).
uint32_t oracle_debug_rays(void* h, const hx_integrator_desc* d, const hx_frame_desc* f, uint32_t px, uint32_t py,
                           uint32_t num_rays, uint32_t frame, float* out, uint32_t capacity) {
    Scene* s = (Scene*)h;
    Params P = make_params(*d, (uint32_t)s->lights.size());
    std::vector<float> verts;
    Counters c;
    for (uint32_t k = 0; k < num_rays; ++k) {
        DebugPath dp{k, num_rays, &verts};
        trace_path<float>(*s, P, *f, px, d->height - py, frame, c, nullptr, &dp);
    }
    const uint32_t n = (uint32_t)(verts.size() / 8);
    std::memcpy(out, verts.data(), 32 * (size_t)std::min(n, capacity));
    return n;
}

// Per-sample radiance L (before the clamp) of frame `frame` for the listed
// pixels (pixel = y*width + x; NULL = all), precision 32 or 64.
void oracle_sample_radiance(void* h, const hx_integrator_desc* d, const hx_frame_desc* f, uint32_t frame, uint32_t precision,
                            const uint32_t* pixels, uint32_t n_pixels, float* out_rgb, hx_hit* primary) {
    Scene* s = (Scene*)h;
    Params P = make_params(*d, (uint32_t)s->lights.size());
    uint32_t n = pixels ? n_pixels : d->width * d->height;
#pragma omp parallel for schedule(dynamic, 64)
    for (long i = 0; i < (long)n; ++i) {
        uint32_t pix = pixels ? pixels[i] : (uint32_t)i;
        uint32_t x = pix % d->width, y = pix / d->width;
        Counters c;
        hx_hit* ph = primary ? &primary[i] : nullptr;
        if (precision == 64) {
            V3<double> L = trace_path<double>(*s, P, *f, x, y, frame, c, ph);
            out_rgb[3 * i] = (float)L.x; out_rgb[3 * i + 1] = (float)L.y; out_rgb[3 * i + 2] = (float)L.z;
        } else {
            V3<float> L = trace_path<float>(*s, P, *f, x, y, frame, c, ph);
            out_rgb[3 * i] = L.x; out_rgb[3 * i + 1] = L.y; out_rgb[3 * i + 2] = L.z;
        }
    }
}

// Progressive accumulation of frames [0, num_frames) for the listed pixels
// (NULL = all, in 16x16 tiles; listed pixels in chunks sized to keep every
// thread busy), with the policy's accumulation rule
// (running mean of path_trace_rgen.glsl:217-248, or Kahan sum / n).
// out_rgb holds 3 doubles per listed pixel.  threads <= 0: all cores.
void oracle_render(void* h, const hx_integrator_desc* d, const hx_frame_desc* f, uint32_t num_frames, uint32_t precision,
                   const uint32_t* pixels, uint32_t n_pixels, double* out_rgb, int threads, oracle_counters* counters) {
    Scene* s = (Scene*)h;
    Params P = make_params(*d, (uint32_t)s->lights.size());
    uint32_t n = pixels ? n_pixels : d->width * d->height;
    int nt = threads > 0 ? threads : omp_get_max_threads();
    uint64_t tp = 0, te = 0, ts = 0;
    float clampv = d->policy.radiance_clamp;
    auto t0 = std::chrono::steady_clock::now();
    // work items: 16x16 pixel tiles for full frames, chunks of 256 listed pixels otherwise
    uint32_t tiles_x = (d->width + 15) / 16, tiles_y = (d->height + 15) / 16;
    uint32_t chunk = pixels ? std::max<uint32_t>(1, std::min<uint32_t>(256, n / (4u * (uint32_t)nt))) : 0;
    long items = pixels ? (long)((n + chunk - 1) / chunk) : (long)tiles_x * tiles_y;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt) reduction(+ : tp, te, ts)
    for (long it = 0; it < items; ++it) {
        std::vector<uint32_t> list;
        if (pixels) {
            for (uint32_t k = (uint32_t)it * chunk; k < n && k < (uint32_t)it * chunk + chunk; ++k) list.push_back(k);
        } else {
            uint32_t tx = (uint32_t)(it % tiles_x), ty = (uint32_t)(it / tiles_x);
            for (uint32_t y = ty * 16; y < ty * 16 + 16 && y < d->height; ++y)
                for (uint32_t x = tx * 16; x < tx * 16 + 16 && x < d->width; ++x) list.push_back(y * d->width + x);
        }
        Counters c;
        for (uint32_t k : list) {
            uint32_t pix = pixels ? pixels[k] : k;
            uint32_t x = pix % d->width, y = pix / d->width;
            double acc[3] = {0, 0, 0}, comp[3] = {0, 0, 0};
            float accf[3] = {0, 0, 0}, compf[3] = {0, 0, 0};
            for (uint32_t fr = 0; fr < num_frames; ++fr) {
                if (precision == 64) {
                    V3<double> L = trace_path<double>(*s, P, *f, x, y, fr, c, nullptr);
                    for (int ch = 0; ch < 3; ++ch) {
                        double v = clampv > 0 ? gmin(L[ch], (double)clampv) : L[ch];
                        if (d->policy.accumulation == HX_ACCUM_KAHAN) {
                            double yk = v - comp[ch];
                            double tk = acc[ch] + yk;
                            comp[ch] = (tk - acc[ch]) - yk;
                            acc[ch] = tk;
                        } else acc[ch] = fr == 0 ? v : acc[ch] + (v - acc[ch]) / (double)fr;
                    }
                    // VISUALIZE_NANS (path_trace_rgen.glsl:225-244)
                    if (d->policy.visualize_nans && (std::isnan(L.x) || std::isnan(L.y) || std::isnan(L.z))) {
                        acc[0] = 1.0;
                        acc[1] = acc[2] = 0.0;
                    }
                } else {
                    V3<float> L = trace_path<float>(*s, P, *f, x, y, fr, c, nullptr);
                    for (int ch = 0; ch < 3; ++ch) {
                        float v = clampv > 0 ? gmin(L[ch], clampv) : L[ch];
                        if (d->policy.accumulation == HX_ACCUM_KAHAN) {
                            float yk = v - compf[ch];
                            float tk = accf[ch] + yk;
                            compf[ch] = (tk - accf[ch]) - yk;
                            accf[ch] = tk;
                        } else accf[ch] = fr == 0 ? v : accf[ch] + (v - accf[ch]) / (float)fr;
                    }
                    if (d->policy.visualize_nans && (std::isnan(L.x) || std::isnan(L.y) || std::isnan(L.z))) {
                        accf[0] = 1.0f;
                        accf[1] = accf[2] = 0.0f;
                    }
                }
            }
            uint32_t slot = pixels ? k : pix;
            for (int ch = 0; ch < 3; ++ch) {
                double v = precision == 64 ? acc[ch] : (double)accf[ch];
                if (d->policy.accumulation == HX_ACCUM_KAHAN)
                    v = precision == 64 ? acc[ch] / (double)num_frames : (double)(accf[ch] / (float)num_frames);
                out_rgb[3 * (size_t)slot + ch] = v;
            }
        }
        tp += c.paths; te += c.ext; ts += c.shadow;
    }
    auto t1 = std::chrono::steady_clock::now();
    if (counters) {
        counters->paths = tp;
        counters->extension_rays = te;
        counters->shadow_rays = ts;
        counters->seconds = std::chrono::duration<double>(t1 - t0).count();
        counters->threads = nt;
    }
}

// tone_map.frag:22-51 + R8G8B8A8_UNORM store, vertically flipped
// (renderer.cpp:394-399 negative-height viewport).
void oracle_tonemap(const float* accum_rgba, uint32_t w, uint32_t h, uint32_t op, float exposure, uint8_t* out) {
    for (uint32_t y = 0; y < h; ++y)
        for (uint32_t x = 0; x < w; ++x) {
            const float* c = &accum_rgba[4 * ((size_t)(h - 1 - y) * w + x)];
            uint8_t* o = &out[4 * ((size_t)y * w + x)];
            for (int ch = 0; ch < 3; ++ch) {
                float v = c[ch] * exposure;
                if (op == HX_TONEMAP_ACES) {
                    float a = 2.51f, b = 0.03f, cc = 2.43f, dd = 0.59f, e = 0.14f;
                    v = gclamp((v * (a * v + b)) / (v * (cc * v + dd) + e), 0.0f, 1.0f);
                } else if (op == HX_TONEMAP_REINHARD) {
                    v = v / (1.0f + v);
                }
                v = std::pow(v, 1.0f / 2.2f);
                float q = gclamp(v, 0.0f, 1.0f) * 255.0f + 0.5f;
                o[ch] = (uint8_t)q;
            }
            o[3] = 255;
        }
}

void oracle_rng_streams(uint32_t kind, const uint32_t* seeds, uint32_t n, uint32_t draws, uint32_t* out) {
    for (uint32_t i = 0; i < n; ++i) {
        RNG r;
        r.kind = kind;
        if (kind == 0) {
            r.s0 = wang_hash(seeds[2 * i]);
            r.s1 = wang_hash(seeds[2 * i + 1]);
            rng_next(r);
        } else {
            r.s0 = pcg_hash(pcg_hash(seeds[2 * i]) + seeds[2 * i + 1]);
            r.s1 = 0;
        }
        for (uint32_t k = 0; k < draws; ++k) out[(size_t)i * draws + k] = rng_next(r);
    }
}

uint32_t oracle_wang_hash(uint32_t v) { return wang_hash(v); }
uint32_t oracle_pcg_hash(uint32_t v) { return pcg_hash(v); }
uint16_t oracle_float_to_half(float f) { return float_to_half(f); }
float oracle_half_to_float(uint16_t h) { return half_to_float(h); }
int oracle_max_threads(void) { return omp_get_max_threads(); }

// HX_RAY_OFFSET_SCALED origins in FP32 for n points (p, geometric normal ng,
// outgoing direction d; 3 floats each), for the property tests.
void oracle_offset_origins(const float* p, const float* ng, const float* d, uint32_t n, float* out) {
    for (uint32_t i = 0; i < n; ++i) {
        const float* a = p + 3 * (size_t)i;
        const float* b = ng + 3 * (size_t)i;
        const float* c = d + 3 * (size_t)i;
        V3<float> o = offset_origin(V3<float>(a[0], a[1], a[2]), V3<float>(b[0], b[1], b[2]), V3<float>(c[0], c[1], c[2]));
        out[3 * (size_t)i] = o.x;
        out[3 * (size_t)i + 1] = o.y;
        out[3 * (size_t)i + 2] = o.z;
    }
}

}  // extern "C"
