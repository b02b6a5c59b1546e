// shade.cuh — device restatement of the helios shading math:
//   brdf.glsl:6-167 (GGX/Lambert uber BSDF), path_trace_rchit.glsl:256-451
//   (surface properties, light sampling), path_trace_rmiss.glsl:38-67
//   (environment), path_trace_rgen.glsl:132-174 (camera ray).
// Same operation order as the oracle; FP32 throughout.
#pragma once

#include "trace.cuh"

struct Surface {
    V3 position, normal, F0, albedo, emissive;
    float metallic, roughness;
};

struct Policy {
    uint32_t rng, rr_start, rr_clamp, area_count_x, area_w_one, env_importance;
    float clampv;
    uint32_t ray_offset;  // 1: HX_RAY_OFFSET_SCALED
};

HXD V3 rot_mul(V3 z, V3 t) {  // make_rotation_matrix(z) * t, sampling.glsl:28-36
    V3 ref = fabsf(z.x * 0.0f + z.y * 1.0f + z.z * 0.0f) > 0.99f ? v3(0.0f, 0.0f, 1.0f) : v3(0.0f, 1.0f, 0.0f);
    V3 x = normalize(cross(ref, z));
    V3 y = cross(z, x);
    return x * t.x + y * t.y + z * t.z;
}
HXD V3 sample_cosine_lobe(V3 n, float r0, float r1) {  // brdf.glsl:6-18
    float rx = gmax(0.00001f, r0), ry = gmax(0.00001f, r1);
    float phi = 2.0f * kPiF * ry;
    float cos_theta = sqrtf(rx);
    float sin_theta = sqrtf(1.0f - rx);
    V3 t = v3(sin_theta * cosf(phi), sin_theta * sinf(phi), cos_theta);
    return normalize(rot_mul(n, t));
}
HXD float D_ggx(float ndoth, float alpha) {
    float a2 = alpha * alpha;
    float denom = (ndoth * ndoth) * (a2 - 1.0f) + 1.0f;
    return a2 / gmax(kEpsilonF, (kPiF * denom * denom));
}
HXD float G1_schlick_ggx(float roughness, float ndotv) {
    float k = ((roughness + 1.0f) * (roughness + 1.0f)) / 8.0f;
    return ndotv / gmax(kEpsilonF, (ndotv * (1.0f - k) + k));
}
HXD V3 evaluate_uber(const Surface& p, V3 Wo, V3 Wh, V3 Wi) {
    float NdotL = gmax(dot(p.normal, Wi), 0.0f);
    float NdotV = gmax(dot(p.normal, Wo), 0.0f);
    float NdotH = gmax(dot(p.normal, Wh), 0.0f);
    float VdotH = gmax(dot(Wi, Wh), 0.0f);
    const float x = 1.0f - VdotH, x2 = x * x;
    float f5 = x2 * x2 * x;  // pow(1 - VdotH, 5.0) as products
    V3 F = p.F0 + (v3(1.0f) - p.F0) * f5;
    float D = D_ggx(NdotH, p.roughness * p.roughness);
    float G = G1_schlick_ggx(p.roughness, NdotL) * G1_schlick_ggx(p.roughness, NdotV);
    V3 specular = ((F * D) * G) / gmax(kEpsilonF, (4.0f * NdotL * NdotV));
    V3 diffuse = p.albedo / kPiF;
    return (v3(1.0f) - F) * diffuse + specular;
}
HXD float pdf_uber(const Surface& p, V3 Wh, V3 Wi) {
    float NdotL = gmax(dot(p.normal, Wi), 0.0f);
    float NdotH = gmax(dot(p.normal, Wh), 0.0f);
    float VdotH = gmax(dot(Wi, Wh), 0.0f);
    float pd = NdotL / kPiF;
    float ps = D_ggx(NdotH, p.roughness * p.roughness) * NdotH / gmax(kEpsilonF, (4.0f * VdotH));
    return pd * (1.0f - 0.5f) + ps * 0.5f;
}
// sample_uber takes the RNG by value (brdf.glsl:136): the caller's state is
// not advanced.
HXD V3 sample_uber(uint32_t kind, const Surface& p, V3 Wo, Rng rng, V3& Wi, float& pdf) {
    float alpha = p.roughness * p.roughness;
    float rx = next_float(kind, rng), ry = next_float(kind, rng), rz = next_float(kind, rng);
    V3 Wh;
    bool is_specular = false;
    if (rx < 0.5f) {
        float phi = 2.0f * kPiF * ry;
        float cos_theta = sqrtf((1.0f - rz) / (1.0f + (alpha * alpha - 1.0f) * rz));
        float sin_theta = sqrtf(1.0f - cos_theta * cos_theta);
        V3 dl = v3(sin_theta * cosf(phi), sin_theta * sinf(phi), cos_theta);
        Wh = normalize(rot_mul(p.normal, dl));
        Wi = reflect(-Wo, Wh);
        float NdotL = gmax(dot(p.normal, Wi), 0.0f);
        float NdotV = gmax(dot(p.normal, Wo), 0.0f);
        if (NdotL > 0.0f && NdotV > 0.0f) is_specular = true;
    }
    if (!is_specular) {
        Wi = sample_cosine_lobe(p.normal, ry, rz);
        Wh = normalize(Wo + Wi);
    }
    pdf = pdf_uber(p, Wh, Wi);
    return evaluate_uber(p, Wo, Wh, Wi);
}

// Geometric normal of a hit triangle in world space: the object-space edge
// cross product through the instance's normal matrix, normalised.
HXD V3 geo_normal(const DevScene& s, uint32_t prim) {
    const uint4 pi = __ldg(&s.prim_info[prim]);
    const DevInstance& inst = s.inst[pi.x];
    const uint32_t i0 = __ldg(&s.indices[3 * pi.y]), i1 = __ldg(&s.indices[3 * pi.y + 1]),
                   i2 = __ldg(&s.indices[3 * pi.y + 2]);
    const float4 p0 = __ldg(&s.vtx[2 * (size_t)i0]), p1 = __ldg(&s.vtx[2 * (size_t)i1]), p2 = __ldg(&s.vtx[2 * (size_t)i2]);
    const V3 e1 = v3(p1.x - p0.x, p1.y - p0.y, p1.z - p0.z);
    const V3 e2 = v3(p2.x - p0.x, p2.y - p0.y, p2.z - p0.z);
    return normalize(mat3_mul(inst.normal, cross(e1, e2)));
}

// HX_RAY_OFFSET_SCALED: the origin p moved off the surface along the
// geometric normal ng, to the side of the outgoing direction, by
// n_i (2^-15 |p_i| + 2^-16) in each coordinate — a continuous form of the
// per-coordinate integer-ulp offset of Waechter and Binder ("A Fast and Robust
// Method for Avoiding Self-Intersection", Ray Tracing Gems, 2019): 2^-15 |p_i|
// is 128-256 ulps of p_i, well above the rounding of an interpolated,
// instance-transformed FP32 hit position.
HXD V3 offset_origin(V3 p, V3 ng, V3 dir) {
    const V3 n = dot(ng, dir) < 0.0f ? -ng : ng;
    return v3(p.x + n.x * (fabsf(p.x) * 3.0517578125e-5f + 1.52587890625e-5f),
              p.y + n.y * (fabsf(p.y) * 3.0517578125e-5f + 1.52587890625e-5f),
              p.z + n.z * (fabsf(p.z) * 3.0517578125e-5f + 1.52587890625e-5f));
}

// Surface properties at a hit (path_trace_rchit.glsl:256-280).
HXD Surface populate(const DevScene& s, uint32_t prim, float u, float v) {
    uint4 pi = __ldg(&s.prim_info[prim]);
    const DevInstance& inst = s.inst[pi.x];
    uint32_t i0 = __ldg(&s.indices[3 * pi.y]), i1 = __ldg(&s.indices[3 * pi.y + 1]), i2 = __ldg(&s.indices[3 * pi.y + 2]);
    float4 p0 = __ldg(&s.vtx[2 * (size_t)i0]), n0 = __ldg(&s.vtx[2 * (size_t)i0 + 1]);
    float4 p1 = __ldg(&s.vtx[2 * (size_t)i1]), n1 = __ldg(&s.vtx[2 * (size_t)i1 + 1]);
    float4 p2 = __ldg(&s.vtx[2 * (size_t)i2]), n2 = __ldg(&s.vtx[2 * (size_t)i2 + 1]);
    float b0 = 1.0f - u - v, b1 = u, b2 = v;
    V3 pos = v3(p0.x * b0 + p1.x * b1 + p2.x * b2, p0.y * b0 + p1.y * b1 + p2.y * b2, p0.z * b0 + p1.z * b1 + p2.z * b2);
    float tu = p0.w * b0 + p1.w * b1 + p2.w * b2;
    float tv = n0.w * b0 + n1.w * b1 + n2.w * b2;
    V3 nrm = normalize(v3(n0.x * b0 + n1.x * b1 + n2.x * b2, n0.y * b0 + n1.y * b1 + n2.y * b2, n0.z * b0 + n1.z * b1 + n2.z * b2));
    Surface p;
    p.position = mat4_mul3(inst.model, pos.x, pos.y, pos.z, 1.0f);
    p.normal = mat3_mul(inst.normal, nrm);
    const hx_material& m = s.materials[pi.z];
    if (m.texture_indices0[1] != -1) {  // get_normal_from_map, path_trace_rchit.glsl:190-219
        const float4 ta = __ldg(&s.vtx_tb[2 * (size_t)i0]), ba = __ldg(&s.vtx_tb[2 * (size_t)i0 + 1]);
        const float4 tb = __ldg(&s.vtx_tb[2 * (size_t)i1]), bb = __ldg(&s.vtx_tb[2 * (size_t)i1 + 1]);
        const float4 tc = __ldg(&s.vtx_tb[2 * (size_t)i2]), bc = __ldg(&s.vtx_tb[2 * (size_t)i2 + 1]);
        const V3 tan = normalize(v3(ta.x * b0 + tb.x * b1 + tc.x * b2, ta.y * b0 + tb.y * b1 + tc.y * b2,
                                    ta.z * b0 + tb.z * b1 + tc.z * b2));
        const V3 bit = normalize(v3(ba.x * b0 + bb.x * b1 + bc.x * b2, ba.y * b0 + bb.y * b1 + bc.y * b2,
                                    ba.z * b0 + bb.z * b1 + bc.z * b2));
        const V3 T = normalize(mat3_mul(inst.normal, tan)), B = normalize(mat3_mul(inst.normal, bit)), N = normalize(p.normal);
        const V3 mp = tex_bilinear_rgb(s, (uint32_t)m.texture_indices0[1], tu, tv);
        const V3 nm = normalize(mp * 2.0f - v3(1.0f));
        p.normal = normalize(v3(T.x * nm.x + B.x * nm.y + N.x * nm.z, T.y * nm.x + B.y * nm.y + N.y * nm.z,
                                T.z * nm.x + B.z * nm.y + N.z * nm.z));
    }
    if (m.texture_indices0[0] == -1) p.albedo = v3(m.albedo[0], m.albedo[1], m.albedo[2]);
    else {
        uint32_t t = (uint32_t)m.texture_indices0[0];
        p.albedo = tex_bilinear_rgb(s, t, tu, tv);
    }
    p.roughness = m.texture_indices0[2] == -1 ? m.roughness_metallic[0]
                                               : tex_bilinear(s, (uint32_t)m.texture_indices0[2], tu, tv, m.texture_indices1[2]);
    p.metallic = m.texture_indices0[3] == -1 ? m.roughness_metallic[1]
                                              : tex_bilinear(s, (uint32_t)m.texture_indices0[3], tu, tv, m.texture_indices1[3]);
    if (m.texture_indices1[0] == -1) p.emissive = v3(m.emissive[0], m.emissive[1], m.emissive[2]);
    else {
        uint32_t t = (uint32_t)m.texture_indices1[0];
        p.emissive = tex_bilinear_rgb(s, t, tu, tv);
    }
    p.roughness = gmax(p.roughness, kMinRoughnessF);
    p.F0 = v3(0.03f) * (1.0f - p.metallic) + p.albedo * p.metallic;
    return p;
}

// ---------------------------------------------------------------------------
// Environment: lat-long FP16 map, bilinear (wrap in u, clamp in v).
// ---------------------------------------------------------------------------
constexpr float kPiExact = 3.14159265358979323846f;

HXD V3 env_texel(const DevEnv& e, int i, int j) {
    const __half2* t = reinterpret_cast<const __half2*>(e.rgb) + 2 * ((size_t)j * e.width + i);
    __half2 a = t[0], b = t[1];
    return v3(__low2float(a), __high2float(a), __low2float(b));
}

HXD V3 env_lookup(const DevEnv& e, V3 d) {
    if (e.kind == HX_ENV_NONE) return v3(0.0f);
    float theta = acosf(gclamp(d.y, -1.0f, 1.0f));
    float phi = atan2f(d.x, -d.z);
    float u = phi / (2.0f * kPiExact) + 0.5f;
    float v = theta / kPiExact;
    float x = u * (float)e.width - 0.5f, y = v * (float)e.height - 0.5f;
    float x0 = floorf(x), y0 = floorf(y);
    float fx = x - x0, fy = y - y0;
    int W = (int)e.width, H = (int)e.height;
    int ix = (int)x0, iy = (int)y0;
    int ix0 = (W & (W - 1)) == 0 ? ix & (W - 1) : ((ix % W) + W) % W;
    int ix1 = ix0 + 1 == W ? 0 : ix0 + 1;
    int iy0 = iy < 0 ? 0 : (iy >= H ? H - 1 : iy);
    int iy1 = iy + 1 < 0 ? 0 : (iy + 1 >= H ? H - 1 : iy + 1);
    V3 a00 = env_texel(e, ix0, iy0), a10 = env_texel(e, ix1, iy0), a01 = env_texel(e, ix0, iy1), a11 = env_texel(e, ix1, iy1);
    V3 top = a00 + (a10 - a00) * fx;
    V3 bot = a01 + (a11 - a01) * fx;
    return top + (bot - top) * fy;
}


HXD V3 env_sample(const DevEnv& e, float r0, float r1, float& pdf) {
    int W = (int)e.width, H = (int)e.height;
    // r * k is exact (k a power of two) and r < 1, so b <= k - 1
    const uint32_t bm = (uint32_t)(r1 * (float)e.km);
    int j = upper_bound_f(e.marg, (int)__ldg(e.marg_guide + bm), (int)__ldg(e.marg_guide + bm + 1), r1) - 1;
    j = j < 0 ? 0 : (j >= H ? H - 1 : j);
    const float* row = e.cond + (size_t)j * (W + 1);
    const uint32_t* g = e.cond_guide + (size_t)j * (e.kc + 1);
    const uint32_t bc = (uint32_t)(r0 * (float)e.kc);
    int i = upper_bound_f(row, (int)__ldg(g + bc), (int)__ldg(g + bc + 1), r0) - 1;
    i = i < 0 ? 0 : (i >= W ? W - 1 : i);
    float m0 = __ldg(e.marg + j), m1 = __ldg(e.marg + j + 1);
    float c0 = __ldg(row + i), c1 = __ldg(row + i + 1);
    float fv = m1 > m0 ? (r1 - m0) / (m1 - m0) : 0.5f;
    float fu = c1 > c0 ? (r0 - c0) / (c1 - c0) : 0.5f;
    fv = gclamp(fv, 0.0f, 1.0f);
    fu = gclamp(fu, 0.0f, 1.0f);
    float u = ((float)i + fu) / (float)W, v = ((float)j + fv) / (float)H;
    float phi = 2.0f * kPiExact * (u - 0.5f);
    float theta = kPiExact * v;
    float st = sinf(theta);
    V3 d = v3(st * sinf(phi), cosf(theta), -st * cosf(phi));
    float pmf = (c1 - c0) * (m1 - m0);
    pdf = st > 0.0f ? pmf * (float)W * (float)H / (2.0f * kPiExact * kPiExact * st) : 0.0f;
    return d;
}

HXD V3 light_v3(const float* f) { return v3(f[0], f[1], f[2]); }

// sample_light (path_trace_rchit.glsl:284-451): Li before visibility.
HXD V3 sample_light(const DevScene& s, const Policy& P, const Surface& p, uint32_t li, Rng& rng, V3& Wi, float& pdf,
                    float& tmax, bool& trace_it) {
    const hx_light& light = s.lights[li];
    tmax = 10000.0f;
    trace_it = true;
    uint32_t type = (uint32_t)light.data0[0];
    V3 Li = v3(0.0f);
    Wi = v3(0.0f);
    pdf = 0.0f;
    if (type == HX_LIGHT_DIRECTIONAL || type == HX_LIGHT_SPOT || type == HX_LIGHT_POINT) {
        float r0 = next_float(P.rng, rng), r1 = next_float(P.rng, rng);
        V3 light_dir;
        float light_distance = 0.0f, light_radius;
        if (type == HX_LIGHT_DIRECTIONAL) {
            light_dir = -light_v3(light.data1);
            light_radius = light.data2[3];
        } else {
            V3 to_light = light_v3(light.data2) - p.position;
            light_dir = normalize(to_light);
            light_distance = length(to_light);
            light_radius = light.data2[3] / light_distance;
        }
        V3 lt = normalize(cross(light_dir, v3(0.0f, 1.0f, 0.0f)));
        V3 lb = normalize(cross(lt, light_dir));
        float point_radius = light_radius * sqrtf(r0);
        float point_angle = r1 * 2.0f * kPiF;
        float dx = point_radius * cosf(point_angle), dy = point_radius * sinf(point_angle);
        Wi = normalize(light_dir + lt * dx + lb * dy);
        V3 col = v3(light.data0[1], light.data0[2], light.data0[3]);
        float intensity = light.data1[3];
        if (type == HX_LIGHT_DIRECTIONAL) Li = col * intensity;
        else if (type == HX_LIGHT_POINT) Li = col * intensity / (light_distance * light_distance);
        else {
            float att = dot(light_dir, -light_v3(light.data1));
            float e0 = light.data3[1], e1 = light.data3[0];
            if (e1 == e0) att = att < e0 ? 0.0f : 1.0f;
            else {
                float tt = gclamp((att - e0) / (e1 - e0), 0.0f, 1.0f);
                att = tt * tt * (3.0f - 2.0f * tt);
            }
            Li = col * intensity * att / (light_distance * light_distance);
        }
        if (type != HX_LIGHT_DIRECTIONAL) tmax = light_distance;
    } else if (type == HX_LIGHT_ENVIRONMENT) {
        float r0 = next_float(P.rng, rng), r1 = next_float(P.rng, rng);
        if (P.env_importance && s.env.kind != HX_ENV_NONE) {
            Wi = env_sample(s.env, r0, r1, pdf);
            Li = env_lookup(s.env, Wi);
            if (!(pdf > 0.0f)) { Li = v3(0.0f); trace_it = false; }
        } else {
            Wi = sample_cosine_lobe(p.normal, r0, r1);
            Li = env_lookup(s.env, Wi);
            pdf = dot(p.normal, Wi) / kPiF;
        }
    } else if (type == HX_LIGHT_AREA) {
        uint32_t inst_id = (uint32_t)light.data0[1];
        uint32_t num_tris = P.area_count_x ? (uint32_t)light.data1[0] : (uint32_t)light.data1[2];
        uint32_t prim_id = next_uint(P.rng, rng, num_tris);
        uint32_t mat = (uint32_t)light.data0[2];
        uint32_t mp = prim_id + (uint32_t)light.data0[3];
        const DevInstance& inst = s.inst[inst_id];
        float r0 = next_float(P.rng, rng), r1 = next_float(P.rng, rng);
        float su0 = sqrtf(r0);
        float bx = 1.0f - su0, by = r1 * su0;
        uint32_t gt = inst.mesh_tri_base + mp;
        V3 P3[3], N3[3];
        for (int c = 0; c < 3; ++c) {
            uint32_t vi = __ldg(&s.indices[3 * gt + c]);
            float4 pv = __ldg(&s.vtx[2 * (size_t)vi]), nv = __ldg(&s.vtx[2 * (size_t)vi + 1]);
            float w = P.area_w_one ? 1.0f : __ldg(&s.vtx_w[vi]);
            P3[c] = mat4_mul3(inst.model, pv.x, pv.y, pv.z, w);
            N3[c] = v3(nv.x, nv.y, nv.z);
        }
        float c0 = 1.0f - bx - by;
        V3 light_pos = P3[0] * c0 + P3[1] * bx + P3[2] * by;
        V3 light_normal = normalize(mat3_mul(inst.normal, N3[0] * c0 + N3[1] * bx + N3[2] * by));
        V3 light_dir = p.position - light_pos;
        float dist_sqr = dot(light_dir, light_dir);
        float area = 0.5f * length(cross(P3[1] - P3[0], P3[2] - P3[0]));
        if (area == 0.0f || dist_sqr == 0.0f) { trace_it = false; return v3(0.0f); }
        float dist = sqrtf(dist_sqr);
        light_dir = light_dir / dist;
        tmax = gmax(0.0f, dist - kEpsilonF);
        float cos_theta = dot(light_normal, light_dir);
        if (cos_theta == 0.0f) { trace_it = false; return v3(0.0f); }
        const hx_material& m = s.materials[mat];
        Li = v3(m.emissive[0], m.emissive[1], m.emissive[2]);
        Wi = -light_dir;
        pdf = dist_sqr / gmax(kEpsilonF, cos_theta * area);
    }
    return Li;
}

// generate_ray (path_trace_rgen.glsl:132-174).
HXD void generate_ray(const hx_frame_desc& f, uint32_t kind, uint32_t x, uint32_t y, uint32_t W, uint32_t H, Rng& rng,
                      V3& org, V3& dir) {
    float px = (float)x + 0.5f, py = (float)y + 0.5f;
    float jx = next_float(kind, rng), jy = next_float(kind, rng);
    float tx = (px + jx) / (float)W, ty = (py + jy) / (float)H;
    float nx = tx * 2.0f - 1.0f, ny = ty * 2.0f - 1.0f;
    const float* m = f.view_proj_inverse;
    float tw = mat4_row(m, 3, nx, ny, 0.0f, 1.0f);
    V3 target = v3(mat4_row(m, 0, nx, ny, 0.0f, 1.0f) / tw, mat4_row(m, 1, nx, ny, 0.0f, 1.0f) / tw,
                   mat4_row(m, 2, nx, ny, 0.0f, 1.0f) / tw);
    V3 cam = light_v3(f.camera_pos);
    float angle = next_float(kind, rng) * 2.0f * kPiF;
    float radius = sqrtf(next_float(kind, rng));
    float ap = f.aperture_radius;
    float ox = cosf(angle) * radius * ap, oy = sinf(angle) * radius * ap;
    V3 aperture_pos = cam + light_v3(f.right_direction) * ox + light_v3(f.up_direction) * oy;
    V3 rdir = -normalize(target - cam);
    V3 fp = light_v3(f.focal_plane);
    float t = -(dot(cam, fp) + f.focal_plane[3]) / dot(rdir, fp);
    V3 focus = cam + rdir * t;
    org = aperture_pos;
    dir = normalize(focus - aperture_pos);
}
