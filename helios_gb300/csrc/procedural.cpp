// procedural.cpp — seeded procedural scenes for the benchmark workloads
// (host side; no reference counterpart: the reference loads AssetCore
// scenes, src/engine/core/resource_manager.cpp:196-490, whose sample files
// are not part of its tree) and the Hosek-Wilkie coefficient lookup used by
// HosekWilkieSkyModel::update (src/engine/gfx/hosek_wilkie_sky_model.cpp:658-686).
//
// Scenes are returned as host arrays in the layouts of include/hx.h, so the
// same data feeds the device upload and the oracle.
#include "../../include/hx.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <random>
#include <vector>

#include "hosek_table.inc"

void hx_set_error(const char* fmt, ...);

struct hx_host_scene {
    std::vector<std::vector<hx_vertex>> vertices;
    std::vector<std::vector<uint32_t>> indices;
    std::vector<std::vector<hx_submesh>> submeshes;
    std::vector<hx_mesh_desc> meshes;
    std::vector<hx_instance> instances;
    std::vector<hx_material> materials;
    std::vector<std::vector<uint8_t>> texels;
    std::vector<hx_texture_desc> textures;
    std::vector<hx_light> lights;
    hx_scene_desc desc{};
    hx_camera camera{};
};

namespace {

struct Rng64 {  // splitmix64: portable, fixed output on every platform
    uint64_t s;
    explicit Rng64(uint64_t seed) : s(seed) {}
    uint64_t next() {
        uint64_t z = (s += 0x9e3779b97f4a7c15ull);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    double uniform(double a, double b) { return a + (b - a) * uniform(); }
};

void identity(float* m) {
    std::memset(m, 0, 64);
    m[0] = m[5] = m[10] = m[15] = 1.0f;
}

hx_vertex make_vertex(float px, float py, float pz, float w, float nx, float ny, float nz, float u, float v) {
    hx_vertex x;
    std::memset(&x, 0, sizeof(x));
    x.position[0] = px; x.position[1] = py; x.position[2] = pz; x.position[3] = w;
    x.tex_coord[0] = u; x.tex_coord[1] = v;
    x.normal[0] = nx; x.normal[1] = ny; x.normal[2] = nz;
    // tangent frame (unused without normal maps)
    float ax = std::fabs(ny) < 0.99f ? 0.0f : 1.0f, ay = std::fabs(ny) < 0.99f ? 1.0f : 0.0f;
    float tx = ay * nz, ty = -ax * nz, tz = ax * ny - ay * nx;
    float tl = std::sqrt(tx * tx + ty * ty + tz * tz);
    if (tl > 0) { tx /= tl; ty /= tl; tz /= tl; }
    x.tangent[0] = tx; x.tangent[1] = ty; x.tangent[2] = tz;
    x.bitangent[0] = ny * tz - nz * ty; x.bitangent[1] = nz * tx - nx * tz; x.bitangent[2] = nx * ty - ny * tx;
    return x;
}

hx_material make_material(float r, float g, float b, float roughness, float metallic) {
    hx_material m;
    std::memset(&m, 0, sizeof(m));
    for (int k = 0; k < 4; ++k) { m.texture_indices0[k] = -1; m.texture_indices1[k] = -1; }
    m.albedo[0] = r; m.albedo[1] = g; m.albedo[2] = b; m.albedo[3] = 1.0f;
    m.roughness_metallic[0] = roughness;
    m.roughness_metallic[1] = metallic;
    return m;
}

// Quad p0..p3 (counter-clockwise seen from the normal side), normal n,
// appended to a mesh; vertex position.w = submesh index.
void add_quad(std::vector<hx_vertex>& vs, std::vector<uint32_t>& ix, const float p[4][3], const float n[3], float w) {
    uint32_t b = (uint32_t)vs.size();
    const float uv[4][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};
    for (int k = 0; k < 4; ++k) vs.push_back(make_vertex(p[k][0], p[k][1], p[k][2], w, n[0], n[1], n[2], uv[k][0], uv[k][1]));
    const uint32_t t[6] = {0, 1, 2, 0, 2, 3};
    for (uint32_t k : t) ix.push_back(b + k);
}

// Axis-aligned box [lo, hi] with outward normals (12 triangles).
void add_box(std::vector<hx_vertex>& vs, std::vector<uint32_t>& ix, const float lo[3], const float hi[3], float w) {
    const float x0 = lo[0], y0 = lo[1], z0 = lo[2], x1 = hi[0], y1 = hi[1], z1 = hi[2];
    const float faces[6][4][3] = {
        {{x0, y0, z1}, {x1, y0, z1}, {x1, y1, z1}, {x0, y1, z1}},  // +z
        {{x1, y0, z0}, {x0, y0, z0}, {x0, y1, z0}, {x1, y1, z0}},  // -z
        {{x1, y0, z1}, {x1, y0, z0}, {x1, y1, z0}, {x1, y1, z1}},  // +x
        {{x0, y0, z0}, {x0, y0, z1}, {x0, y1, z1}, {x0, y1, z0}},  // -x
        {{x0, y1, z1}, {x1, y1, z1}, {x1, y1, z0}, {x0, y1, z0}},  // +y
        {{x0, y0, z0}, {x1, y0, z0}, {x1, y0, z1}, {x0, y0, z1}},  // -y
    };
    const float normals[6][3] = {{0, 0, 1}, {0, 0, -1}, {1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}};
    for (int f = 0; f < 6; ++f) add_quad(vs, ix, faces[f], normals[f], w);
}

void finish(hx_host_scene* s) {
    s->meshes.resize(s->vertices.size());
    for (size_t m = 0; m < s->vertices.size(); ++m) {
        s->meshes[m].vertices = s->vertices[m].data();
        s->meshes[m].num_vertices = (uint32_t)s->vertices[m].size();
        s->meshes[m].indices = s->indices[m].data();
        s->meshes[m].num_indices = (uint32_t)s->indices[m].size();
        s->meshes[m].submeshes = s->submeshes[m].data();
        s->meshes[m].num_submeshes = (uint32_t)s->submeshes[m].size();
    }
    s->textures.resize(s->texels.size());
    for (size_t t = 0; t < s->texels.size(); ++t) s->textures[t].rgba8 = s->texels[t].data();
    s->desc.meshes = s->meshes.data();
    s->desc.num_meshes = (uint32_t)s->meshes.size();
    s->desc.instances = s->instances.data();
    s->desc.num_instances = (uint32_t)s->instances.size();
    s->desc.materials = s->materials.data();
    s->desc.num_materials = (uint32_t)s->materials.size();
    s->desc.textures = s->textures.data();
    s->desc.num_textures = (uint32_t)s->textures.size();
    s->desc.punctual_lights = s->lights.data();
    s->desc.num_punctual_lights = (uint32_t)s->lights.size();
}

void add_instance(hx_host_scene* s, uint32_t mesh, const float* model, const float* normal, int32_t override_mat) {
    hx_instance in;
    std::memset(&in, 0, sizeof(in));
    std::memcpy(in.model_matrix, model, 64);
    std::memcpy(in.normal_matrix, normal, 64);
    in.mesh_index = mesh;
    in.material_override = override_mat;
    s->instances.push_back(in);
}

// Box scene: [0,1]^3 interior, front (z = 1) open; 5 walls (10 tris), two
// axis-aligned white boxes (24 tris), one quad light (2 tris).
void build_box(hx_host_scene* s) {
    s->materials.push_back(make_material(0.73f, 0.73f, 0.73f, 1.0f, 0.0f));  // 0 white
    s->materials.push_back(make_material(0.63f, 0.06f, 0.05f, 1.0f, 0.0f));  // 1 red
    s->materials.push_back(make_material(0.14f, 0.45f, 0.09f, 1.0f, 0.0f));  // 2 green
    hx_material light = make_material(0.78f, 0.78f, 0.78f, 1.0f, 0.0f);     // 3 light
    light.emissive[0] = 17.0f; light.emissive[1] = 12.0f; light.emissive[2] = 4.0f;
    s->materials.push_back(light);

    // mesh 0: walls; submesh 0 white (floor, ceiling, back), 1 red (left x=0), 2 green (right x=1)
    s->vertices.emplace_back(); s->indices.emplace_back(); s->submeshes.emplace_back();
    {
        auto& vs = s->vertices.back();
        auto& ix = s->indices.back();
        const float floor_[4][3] = {{0, 0, 1}, {1, 0, 1}, {1, 0, 0}, {0, 0, 0}};
        const float ceil_[4][3] = {{0, 1, 0}, {1, 1, 0}, {1, 1, 1}, {0, 1, 1}};
        const float back[4][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}};
        const float left[4][3] = {{0, 0, 1}, {0, 0, 0}, {0, 1, 0}, {0, 1, 1}};
        const float right[4][3] = {{1, 0, 0}, {1, 0, 1}, {1, 1, 1}, {1, 1, 0}};
        const float nu[3] = {0, 1, 0}, nd[3] = {0, -1, 0}, nb[3] = {0, 0, 1}, nl[3] = {1, 0, 0}, nr[3] = {-1, 0, 0};
        add_quad(vs, ix, floor_, nu, 0); add_quad(vs, ix, ceil_, nd, 0); add_quad(vs, ix, back, nb, 0);
        add_quad(vs, ix, left, nl, 1);
        add_quad(vs, ix, right, nr, 2);
        s->submeshes.back() = {{0, 18, 0, 0}, {18, 6, 1, 0}, {24, 6, 2, 0}};
    }
    const float boxes[2][2][3] = {{{0.13f, 0.0f, 0.37f}, {0.43f, 0.3f, 0.67f}}, {{0.53f, 0.0f, 0.12f}, {0.83f, 0.6f, 0.42f}}};
    for (int b = 0; b < 2; ++b) {
        s->vertices.emplace_back(); s->indices.emplace_back(); s->submeshes.emplace_back();
        add_box(s->vertices.back(), s->indices.back(), boxes[b][0], boxes[b][1], 0);
        s->submeshes.back() = {{0, 36, 0, 0}};
    }
    s->vertices.emplace_back(); s->indices.emplace_back(); s->submeshes.emplace_back();
    {
        const float q[4][3] = {{0.375f, 0.999f, 0.375f}, {0.625f, 0.999f, 0.375f}, {0.625f, 0.999f, 0.625f}, {0.375f, 0.999f, 0.625f}};
        const float n[3] = {0, -1, 0};
        add_quad(s->vertices.back(), s->indices.back(), q, n, 0);
        s->submeshes.back() = {{0, 6, 3, 0}};
    }
    float I[16];
    identity(I);
    for (uint32_t m = 0; m < 4; ++m) add_instance(s, m, I, I, -1);
    s->desc.environment.kind = HX_ENV_NONE;
    s->camera = hx_camera{{0.5f, 0.5f, 2.5f}, {0.5f, 0.5f, 0.0f}, {0.0f, 1.0f, 0.0f}, 40.0f, 1.0f, 1000.0f, 8.0f, 0.0f};
}

// Level-L icosphere (20 * 4^L triangles), unit radius, smooth normals.
void icosphere(uint32_t level, std::vector<hx_vertex>& vs, std::vector<uint32_t>& ix) {
    const double t = (1.0 + std::sqrt(5.0)) / 2.0;
    std::vector<std::array<double, 3>> p = {{-1, t, 0}, {1, t, 0}, {-1, -t, 0}, {1, -t, 0}, {0, -1, t}, {0, 1, t},
                                            {0, -1, -t}, {0, 1, -t}, {t, 0, -1}, {t, 0, 1}, {-t, 0, -1}, {-t, 0, 1}};
    for (auto& v : p) {
        double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        for (auto& c : v) c /= l;
    }
    std::vector<uint32_t> f = {0, 11, 5, 0, 5, 1, 0, 1, 7, 0, 7, 10, 0, 10, 11, 1, 5, 9, 5, 11, 4, 11, 10, 2, 10, 7, 6, 7, 1, 8,
                               3, 9, 4, 3, 4, 2, 3, 2, 6, 3, 6, 8, 3, 8, 9, 4, 9, 5, 2, 4, 11, 6, 2, 10, 8, 6, 7, 9, 8, 1};
    for (uint32_t l = 0; l < level; ++l) {
        std::map<uint64_t, uint32_t> mid;
        auto midpoint = [&](uint32_t a, uint32_t b) {
            uint64_t key = a < b ? ((uint64_t)a << 32 | b) : ((uint64_t)b << 32 | a);
            auto it = mid.find(key);
            if (it != mid.end()) return it->second;
            std::array<double, 3> m = {(p[a][0] + p[b][0]) * 0.5, (p[a][1] + p[b][1]) * 0.5, (p[a][2] + p[b][2]) * 0.5};
            double len = std::sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
            for (auto& c : m) c /= len;
            p.push_back(m);
            uint32_t idx = (uint32_t)p.size() - 1;
            mid[key] = idx;
            return idx;
        };
        std::vector<uint32_t> nf;
        nf.reserve(f.size() * 4);
        for (size_t k = 0; k < f.size(); k += 3) {
            uint32_t a = f[k], b = f[k + 1], c = f[k + 2];
            uint32_t ab = midpoint(a, b), bc = midpoint(b, c), ca = midpoint(c, a);
            uint32_t tri[12] = {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca};
            nf.insert(nf.end(), tri, tri + 12);
        }
        f.swap(nf);
    }
    vs.reserve(p.size());
    for (auto& v : p) {
        float u = (float)(0.5 + std::atan2(v[0], -v[2]) / (2.0 * 3.14159265358979323846));
        float w = (float)(std::acos(std::max(-1.0, std::min(1.0, v[1]))) / 3.14159265358979323846);
        vs.push_back(make_vertex((float)v[0], (float)v[1], (float)v[2], 0.0f, (float)v[0], (float)v[1], (float)v[2], u, w));
    }
    ix = f;
}

// Periodic value noise in [0, 1], three octaves.
void value_noise_mask(Rng64& rng, uint32_t size, std::vector<uint8_t>& out) {
    const uint32_t cells[3] = {8, 16, 32};
    const float wts[3] = {0.5f, 0.3f, 0.2f};
    std::vector<float> v((size_t)size * size, 0.0f);
    for (int o = 0; o < 3; ++o) {
        uint32_t g = cells[o];
        std::vector<float> lat((size_t)g * g);
        for (auto& x : lat) x = (float)rng.uniform();
        for (uint32_t y = 0; y < size; ++y)
            for (uint32_t x = 0; x < size; ++x) {
                float fx = (x + 0.5f) * g / size, fy = (y + 0.5f) * g / size;
                uint32_t x0 = (uint32_t)fx, y0 = (uint32_t)fy;
                float tx = fx - x0, ty = fy - y0;
                tx = tx * tx * (3 - 2 * tx);
                ty = ty * ty * (3 - 2 * ty);
                uint32_t x1 = (x0 + 1) % g, y1 = (y0 + 1) % g;
                x0 %= g; y0 %= g;
                float a = lat[y0 * g + x0], b = lat[y0 * g + x1], c = lat[y1 * g + x0], d = lat[y1 * g + x1];
                float top = a + (b - a) * tx, bot = c + (d - c) * tx;
                v[(size_t)y * size + x] += wts[o] * (top + (bot - top) * ty);
            }
    }
    std::vector<float> sorted(v);
    std::nth_element(sorted.begin(), sorted.begin() + sorted.size() / 2, sorted.end());
    float median = sorted[sorted.size() / 2];
    out.resize((size_t)size * size * 4);
    for (size_t k = 0; k < v.size(); ++k) {
        float n = v[k];
        out[4 * k + 0] = (uint8_t)std::min(255.0f, 40.0f + 60.0f * n);
        out[4 * k + 1] = (uint8_t)std::min(255.0f, 90.0f + 130.0f * n);
        out[4 * k + 2] = (uint8_t)std::min(255.0f, 30.0f + 40.0f * n);
        out[4 * k + 3] = n >= median ? 255 : 0;  // 50% cutout
    }
}

void trs(const double q[4], double scale, const double t[3], float* model, float* normal) {
    double x = q[0], y = q[1], z = q[2], w = q[3];
    double R[9] = {1 - 2 * (y * y + z * z), 2 * (x * y + z * w), 2 * (x * z - y * w),
                   2 * (x * y - z * w), 1 - 2 * (x * x + z * z), 2 * (y * z + x * w),
                   2 * (x * z + y * w), 2 * (y * z - x * w), 1 - 2 * (x * x + y * y)};  // column-major 3x3
    std::memset(model, 0, 64);
    std::memset(normal, 0, 64);
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) {
            model[c * 4 + r] = (float)(R[c * 3 + r] * scale);
            normal[c * 4 + r] = (float)R[c * 3 + r];
        }
    for (int r = 0; r < 3; ++r) { model[12 + r] = (float)t[r]; normal[12 + r] = (float)t[r]; }
    model[15] = normal[15] = 1.0f;
}

hx_status build_icospheres(hx_host_scene* s, const hx_procedural_params& P) {
    Rng64 rng(P.seed);
    // materials: 0 placeholder, 1..12 spheres, 13 ground, 14.. alpha quads
    s->materials.push_back(make_material(0.8f, 0.8f, 0.8f, 0.5f, 0.0f));
    for (int i = 0; i < 12; ++i) {
        float r = (float)rng.uniform(), g = (float)rng.uniform(), b = (float)rng.uniform();
        float rough = (float)rng.uniform(0.05, 1.0);
        float metal = rng.uniform() < 0.3 ? 1.0f : 0.0f;
        s->materials.push_back(make_material(r, g, b, rough, metal));
    }
    s->materials.push_back(make_material(0.5f, 0.5f, 0.5f, 0.9f, 0.0f));
    const uint32_t pool = std::max<uint32_t>(1, P.mask_pool);
    for (uint32_t k = 0; k < pool; ++k) {
        hx_material m = make_material(1.0f, 1.0f, 1.0f, 0.7f, 0.0f);
        m.texture_indices0[0] = (int32_t)k;
        s->materials.push_back(m);
    }
    // mesh 0: icosphere
    s->vertices.emplace_back(); s->indices.emplace_back(); s->submeshes.emplace_back();
    icosphere(P.icosphere_level, s->vertices.back(), s->indices.back());
    s->submeshes.back() = {{0, (uint32_t)s->indices.back().size(), 0, 0}};
    // mesh 1: ground plane (2 tris)
    s->vertices.emplace_back(); s->indices.emplace_back(); s->submeshes.emplace_back();
    {
        const float q[4][3] = {{-200, -20, 200}, {200, -20, 200}, {200, -20, -200}, {-200, -20, -200}};
        const float n[3] = {0, 1, 0};
        add_quad(s->vertices.back(), s->indices.back(), q, n, 0);
        s->submeshes.back() = {{0, 6, 13, 0}};
    }
    // mesh 2: alpha quads grouped by mask (submesh k uses mask k)
    s->vertices.emplace_back(); s->indices.emplace_back(); s->submeshes.emplace_back();
    {
        uint32_t nq = P.num_alpha_quads;
        struct Q { float p[4][3]; float n[3]; };
        std::vector<Q> quads(nq);
        for (uint32_t q = 0; q < nq; ++q) {
            double c[3] = {rng.uniform(-20, 20), rng.uniform(-20, 20), rng.uniform(-20, 20)};
            double z = rng.uniform(-1, 1), ph = rng.uniform(0, 2 * 3.14159265358979323846);
            double r = std::sqrt(std::max(0.0, 1 - z * z));
            double n[3] = {r * std::cos(ph), z, r * std::sin(ph)};
            double a[3] = {std::fabs(n[1]) < 0.9 ? 0.0 : 1.0, std::fabs(n[1]) < 0.9 ? 1.0 : 0.0, 0.0};
            double t1[3] = {a[1] * n[2] - a[2] * n[1], a[2] * n[0] - a[0] * n[2], a[0] * n[1] - a[1] * n[0]};
            double l = std::sqrt(t1[0] * t1[0] + t1[1] * t1[1] + t1[2] * t1[2]);
            for (auto& v : t1) v /= l;
            double t2[3] = {n[1] * t1[2] - n[2] * t1[1], n[2] * t1[0] - n[0] * t1[2], n[0] * t1[1] - n[1] * t1[0]};
            double rot = rng.uniform(0, 2 * 3.14159265358979323846);
            double cr = std::cos(rot), sr = std::sin(rot);
            double u[3], v[3];
            for (int k = 0; k < 3; ++k) { u[k] = cr * t1[k] + sr * t2[k]; v[k] = -sr * t1[k] + cr * t2[k]; }
            double h = 0.5 * rng.uniform(0.1, 0.4);
            const double sgn[4][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}};
            for (int k = 0; k < 4; ++k)
                for (int d = 0; d < 3; ++d) quads[q].p[k][d] = (float)(c[d] + h * (sgn[k][0] * u[d] + sgn[k][1] * v[d]));
            for (int d = 0; d < 3; ++d) quads[q].n[d] = (float)n[d];
        }
        auto& vs = s->vertices.back();
        auto& ix = s->indices.back();
        vs.reserve(4 * (size_t)nq);
        ix.reserve(6 * (size_t)nq);
        for (uint32_t k = 0; k < pool; ++k) {
            uint32_t base = (uint32_t)ix.size();
            for (uint32_t q = k; q < nq; q += pool) add_quad(vs, ix, quads[q].p, quads[q].n, (float)k);
            uint32_t cnt = (uint32_t)ix.size() - base;
            if (cnt) s->submeshes.back().push_back({base, cnt, 14 + k, HX_SUBMESH_NON_OPAQUE});
        }
    }
    // masks
    for (uint32_t k = 0; k < pool; ++k) {
        s->texels.emplace_back();
        value_noise_mask(rng, P.mask_size, s->texels.back());
        hx_texture_desc td{};
        td.rgba8 = nullptr;
        td.width = P.mask_size;
        td.height = P.mask_size;
        s->textures.push_back(td);
    }
    // instances: 12 icospheres, ground, quads
    for (int i = 0; i < 12; ++i) {
        double u1 = rng.uniform(), u2 = rng.uniform(), u3 = rng.uniform();
        double q[4] = {std::sqrt(1 - u1) * std::sin(2 * 3.14159265358979323846 * u2),
                       std::sqrt(1 - u1) * std::cos(2 * 3.14159265358979323846 * u2),
                       std::sqrt(u1) * std::sin(2 * 3.14159265358979323846 * u3),
                       std::sqrt(u1) * std::cos(2 * 3.14159265358979323846 * u3)};
        double scale = rng.uniform(0.5, 2.0);
        double t[3] = {rng.uniform(-20, 20), rng.uniform(-20, 20), rng.uniform(-20, 20)};
        float model[16], normal[16];
        trs(q, scale, t, model, normal);
        add_instance(s, 0, model, normal, 1 + i);
    }
    float I[16];
    identity(I);
    add_instance(s, 1, I, I, -1);
    add_instance(s, 2, I, I, -1);
    // 4 point lights
    for (int i = 0; i < 4; ++i) {
        hx_light l;
        std::memset(&l, 0, sizeof(l));
        l.data0[0] = (float)HX_LIGHT_POINT;
        l.data0[1] = 1.0f; l.data0[2] = 0.9f; l.data0[3] = 0.8f;
        l.data1[3] = 150.0f;
        l.data2[0] = (float)rng.uniform(-15, 15);
        l.data2[1] = (float)rng.uniform(0, 18);
        l.data2[2] = (float)rng.uniform(-15, 15);
        l.data2[3] = 0.3f;
        s->lights.push_back(l);
    }
    // Hosek-Wilkie sky
    hx_environment_desc& e = s->desc.environment;
    e.kind = HX_ENV_HOSEK_WILKIE;
    e.width = P.env_width;
    e.height = P.env_height;
    double el = P.sun_elevation_deg * 3.14159265358979323846 / 180.0, az = 40.0 * 3.14159265358979323846 / 180.0;
    e.sun_direction[0] = (float)(std::cos(el) * std::sin(az));
    e.sun_direction[1] = (float)std::sin(el);
    e.sun_direction[2] = (float)(std::cos(el) * std::cos(az));
    hx_status st = hx_hosek_wilkie_sky(e.sun_direction, P.turbidity, P.ground_albedo, 1.15f, e.coeffs);
    if (st != HX_OK) return st;
    s->camera = hx_camera{{8.0f, 6.0f, 26.0f}, {0.0f, -3.0f, 0.0f}, {0.0f, 1.0f, 0.0f}, 60.0f, 1.0f, 1000.0f, 8.0f, 0.0f};
    return HX_OK;
}

// Periodic value-noise fBm over [0,1)^2 (6 octaves), for terrain heights.
float fbm(const std::vector<float>& lat, uint32_t g, float x, float y) {
    float sum = 0.0f, amp = 0.5f, freq = 1.0f;
    for (int o = 0; o < 6; ++o) {
        float fx = x * g * freq, fy = y * g * freq;
        float x0f = std::floor(fx), y0f = std::floor(fy);
        float tx = fx - x0f, ty = fy - y0f;
        tx = tx * tx * (3 - 2 * tx);
        ty = ty * ty * (3 - 2 * ty);
        uint32_t gs = g * (1u << o);
        uint32_t x0 = (uint32_t)x0f % gs, y0 = (uint32_t)y0f % gs, x1 = (x0 + 1) % gs, y1 = (y0 + 1) % gs;
        // lattice values hashed from the base lattice (one table for every octave)
        auto L = [&](uint32_t i, uint32_t j) { return lat[((i * 73856093u) ^ (j * 19349663u) ^ (o * 83492791u)) % lat.size()]; };
        float a = L(x0, y0), b = L(x1, y0), c = L(x0, y1), d = L(x1, y1);
        float top = a + (b - a) * tx, bot = c + (d - c) * tx;
        sum += amp * (top + (bot - top) * ty);
        amp *= 0.5f;
        freq *= 2.0f;
    }
    return sum;
}

// Terrain scene (precision form at scale): num_spheres seeded subdivided
// spheres over an N x N-vertex fBm heightfield (2 (N-1)^2 triangles), sun and
// Hosek-Wilkie sky.
hx_status build_terrain(hx_host_scene* s, const hx_procedural_params& P) {
    Rng64 rng(P.seed ^ 0x7e77a1ull);
    const uint32_t N = std::max<uint32_t>(2, P.terrain_size);
    const float extent = 4096.0f, hmax = 300.0f;
    s->materials.push_back(make_material(0.35f, 0.30f, 0.22f, 0.9f, 0.0f));  // 0 terrain
    for (uint32_t i = 0; i < 16; ++i) {
        float r = (float)rng.uniform(), g = (float)rng.uniform(), b = (float)rng.uniform();
        s->materials.push_back(make_material(r, g, b, (float)rng.uniform(0.05, 1.0), rng.uniform() < 0.3 ? 1.0f : 0.0f));
    }
    std::vector<float> lat(1 << 16);
    for (auto& v : lat) v = (float)rng.uniform();
    // mesh 0: heightfield
    s->vertices.emplace_back(); s->indices.emplace_back(); s->submeshes.emplace_back();
    {
        auto& vs = s->vertices.back();
        auto& ix = s->indices.back();
        vs.resize((size_t)N * N);
        std::vector<float> h((size_t)N * N);
        for (uint32_t j = 0; j < N; ++j)
            for (uint32_t i = 0; i < N; ++i) h[(size_t)j * N + i] = hmax * fbm(lat, 4, (float)i / N, (float)j / N);
        const float step = extent / (float)(N - 1);
        for (uint32_t j = 0; j < N; ++j)
            for (uint32_t i = 0; i < N; ++i) {
                uint32_t il = i ? i - 1 : i, ir = i + 1 < N ? i + 1 : i, jd = j ? j - 1 : j, ju = j + 1 < N ? j + 1 : j;
                float dx = (h[(size_t)j * N + ir] - h[(size_t)j * N + il]) / ((ir - il) * step);
                float dz = (h[(size_t)ju * N + i] - h[(size_t)jd * N + i]) / ((ju - jd) * step);
                float nx = -dx, ny = 1.0f, nz = -dz;
                float nl = std::sqrt(nx * nx + ny * ny + nz * nz);
                vs[(size_t)j * N + i] = make_vertex(-extent * 0.5f + i * step, h[(size_t)j * N + i], -extent * 0.5f + j * step,
                                                    0.0f, nx / nl, ny / nl, nz / nl, (float)i / (N - 1), (float)j / (N - 1));
            }
        ix.reserve((size_t)6 * (N - 1) * (N - 1));
        for (uint32_t j = 0; j + 1 < N; ++j)
            for (uint32_t i = 0; i + 1 < N; ++i) {
                uint32_t a = j * N + i, b = a + 1, c = a + N, d = c + 1;
                const uint32_t t[6] = {a, c, b, b, c, d};
                ix.insert(ix.end(), t, t + 6);
            }
        s->submeshes.back() = {{0, (uint32_t)ix.size(), 0, 0}};
    }
    // mesh 1: sphere
    s->vertices.emplace_back(); s->indices.emplace_back(); s->submeshes.emplace_back();
    icosphere(P.icosphere_level, s->vertices.back(), s->indices.back());
    s->submeshes.back() = {{0, (uint32_t)s->indices.back().size(), 1, 0}};
    float I[16];
    identity(I);
    add_instance(s, 0, I, I, -1);
    for (uint32_t k = 0; k < P.num_spheres; ++k) {
        double u1 = rng.uniform(), u2 = rng.uniform(), u3 = rng.uniform();
        double q[4] = {std::sqrt(1 - u1) * std::sin(2 * 3.14159265358979323846 * u2),
                       std::sqrt(1 - u1) * std::cos(2 * 3.14159265358979323846 * u2),
                       std::sqrt(u1) * std::sin(2 * 3.14159265358979323846 * u3),
                       std::sqrt(u1) * std::cos(2 * 3.14159265358979323846 * u3)};
        double scale = rng.uniform(5.0, 40.0);
        double t[3] = {rng.uniform(-600, 600), rng.uniform(hmax, hmax + 200), rng.uniform(-600, 600)};
        float model[16], normal[16];
        trs(q, scale, t, model, normal);
        add_instance(s, 1, model, normal, 1 + (int32_t)(k % 16));
    }
    // sun (directional) + sky
    hx_environment_desc& e = s->desc.environment;
    e.kind = HX_ENV_HOSEK_WILKIE;
    e.width = P.env_width;
    e.height = P.env_height;
    double el = P.sun_elevation_deg * 3.14159265358979323846 / 180.0, az = 40.0 * 3.14159265358979323846 / 180.0;
    e.sun_direction[0] = (float)(std::cos(el) * std::sin(az));
    e.sun_direction[1] = (float)std::sin(el);
    e.sun_direction[2] = (float)(std::cos(el) * std::cos(az));
    hx_status st = hx_hosek_wilkie_sky(e.sun_direction, P.turbidity, P.ground_albedo, 1.15f, e.coeffs);
    if (st != HX_OK) return st;
    hx_light sun;
    std::memset(&sun, 0, sizeof(sun));
    sun.data0[0] = (float)HX_LIGHT_DIRECTIONAL;
    sun.data0[1] = 1.0f; sun.data0[2] = 0.95f; sun.data0[3] = 0.85f;
    for (int a = 0; a < 3; ++a) sun.data1[a] = -e.sun_direction[a];  // light forward: from the sun
    sun.data1[3] = 3.0f;
    sun.data2[3] = 0.01f;
    s->lights.push_back(sun);
    s->camera = hx_camera{{0.0f, hmax + 350.0f, 1100.0f}, {0.0f, hmax * 0.5f, 0.0f}, {0.0f, 1.0f, 0.0f}, 50.0f, 1.0f, 10000.0f, 8.0f, 0.0f};
    return HX_OK;
}

}  // namespace

extern "C" void hx_procedural_defaults(uint32_t kind, hx_procedural_params* p) {
    std::memset(p, 0, sizeof(*p));
    p->kind = kind;
    p->seed = 0x5eed1234ull;
    p->num_alpha_quads = 100000;
    p->mask_pool = 64;
    p->mask_size = 512;
    p->icosphere_level = 6;
    p->env_width = 2048;
    p->env_height = 1024;
    p->sun_elevation_deg = 30.0f;
    p->turbidity = 3.0f;
    p->ground_albedo = 0.1f;
    p->terrain_size = 4096;
    p->num_spheres = 200;
    if (kind == HX_SCENE_TERRAIN) p->icosphere_level = 4;
}

extern "C" hx_status hx_procedural_scene_create(const hx_procedural_params* params, hx_host_scene** out) {
    if (!params || !out) { hx_set_error("hx_procedural_scene_create: null argument"); return HX_ERR_INVALID_ARG; }
    if (params->kind > HX_SCENE_TERRAIN || params->icosphere_level > 8 || params->mask_size > 4096 ||
        params->mask_size == 0 || params->env_width < 2 || params->env_height < 2 || params->terrain_size > 8192) {
        hx_set_error("hx_procedural_scene_create: bad parameters");
        return HX_ERR_INVALID_ARG;
    }
    std::unique_ptr<hx_host_scene> s(new hx_host_scene());
    if (params->kind == HX_SCENE_BOX) build_box(s.get());
    else {
        hx_status st = params->kind == HX_SCENE_ICOSPHERES ? build_icospheres(s.get(), *params) : build_terrain(s.get(), *params);
        if (st != HX_OK) return st;
    }
    hx_environment_desc env = s->desc.environment;
    finish(s.get());
    s->desc.environment = env;
    *out = s.release();
    return HX_OK;
}

extern "C" const hx_scene_desc* hx_host_scene_desc(const hx_host_scene* s) { return s ? &s->desc : nullptr; }
extern "C" hx_status hx_host_scene_camera(const hx_host_scene* s, hx_camera* out) {
    if (!s || !out) return HX_ERR_INVALID_ARG;
    *out = s->camera;
    return HX_OK;
}
extern "C" hx_status hx_host_scene_destroy(hx_host_scene* s) {
    delete s;
    return HX_OK;
}

// Hosek-Wilkie RGB coefficients for any turbidity, ground albedo and sun
// angle, evaluated the way the reference's evaluate does
// (hosek_wilkie_sky_model.cpp:48-67): each raw coefficient is a quintic in
// e = (1 - theta / (pi / 2))^(1/3) per (albedo 0/1, integer turbidity), and
// the four splines around (turbidity, albedo) blend bilinearly.  The quintic
// comes from its six samples at e = j / 5 (kHosekNodes) by Lagrange
// interpolation in double — exact up to rounding, so the FP32 coefficients
// equal the reference's to an ulp.  Then the luminance normalisation of
// HosekWilkieSkyModel::update (hosek_wilkie_sky_model.cpp:681-686).
static double hosek_spline(int a, int t, int q, double e) {
    double v = 0.0;
    for (int j = 0; j < 6; ++j) {
        double l = 1.0;
        for (int m = 0; m < 6; ++m)
            if (m != j) l *= (e - m / 5.0) / ((j - m) / 5.0);
        v += kHosekNodes[a][t - 1][j][q] * l;
    }
    return v;
}

extern "C" hx_status hx_hosek_wilkie_sky(const float sun_direction[3], float turbidity, float albedo,
                                         float normalized_sun_y, float out[40]) {
    if (!sun_direction || !out) { hx_set_error("hx_hosek_wilkie_sky: null argument"); return HX_ERR_INVALID_ARG; }
    if (!std::isfinite(turbidity) || !std::isfinite(albedo) || !std::isfinite(normalized_sun_y)) {
        hx_set_error("hx_hosek_wilkie_sky: non-finite argument");
        return HX_ERR_INVALID_ARG;
    }
    const float theta = std::acos(std::min(std::max(sun_direction[1], 0.0f), 1.0f));
    const double kPi = 3.14159265358979323846;
    const double e = std::pow(std::max<float>(0.f, 1.f - theta / (kPi / 2.f)), 1.f / 3.0f);
    const int t0 = std::min(std::max(static_cast<int>(turbidity), 1), 10);
    const int t1 = std::min(t0 + 1, 10);
    const float tk = std::min(std::max(turbidity - t0, 0.f), 1.f);
    float c[30];
    for (int q = 0; q < 30; ++q) {
        const double a0t0 = hosek_spline(0, t0, q, e), a1t0 = hosek_spline(1, t0, q, e);
        const double a0t1 = hosek_spline(0, t1, q, e), a1t1 = hosek_spline(1, t1, q, e);
        c[q] = (float)(a0t0 * (1 - albedo) * (1 - tk) + a1t0 * albedo * (1 - tk) + a0t1 * (1 - albedo) * tk +
                       a1t1 * albedo * tk);
    }
    if (normalized_sun_y != 0.0f) {
        float S[3];
        for (int ch = 0; ch < 3; ++ch) {
            float A = c[0 + ch], B = c[3 + ch], C = c[6 + ch], D = c[9 + ch], E = c[12 + ch], F = c[15 + ch], G = c[18 + ch],
                  H = c[21 + ch], I = c[24 + ch];
            float cos_t = std::cos(theta), cos_g = 1.0f, gamma = 0.0f;
            float chi = (1.f + cos_g * cos_g) / std::pow(1.f + H * H - 2.f * cos_g * H, 1.5f);
            S[ch] = (1.f + A * std::exp(B / (cos_t + 0.01f))) * (C + D * std::exp(E * gamma) + F * (cos_g * cos_g) + G * chi +
                                                                 I * std::sqrt(std::max(0.f, cos_t))) * c[27 + ch];
        }
        float lum = S[0] * 0.2126f + S[1] * 0.7152f + S[2] * 0.0722f;
        for (int ch = 0; ch < 3; ++ch) { c[27 + ch] /= lum; c[27 + ch] *= normalized_sun_y; }
    }
    std::memset(out, 0, 40 * sizeof(float));
    for (int p = 0; p < 10; ++p)
        for (int ch = 0; ch < 3; ++ch) out[4 * p + ch] = c[3 * p + ch];
    return HX_OK;
}

// Ground albedo 0.1, the reference's default (hosek_wilkie_sky_model.h:33).
extern "C" hx_status hx_hosek_wilkie_coefficients(const float sun_direction[3], float turbidity, float normalized_sun_y,
                                                  float out[40]) {
    return hx_hosek_wilkie_sky(sun_direction, turbidity, 0.1f, normalized_sun_y, out);
}
