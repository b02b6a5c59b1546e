// trace.cuh — BVH8 traversal, watertight ray/triangle test, any-hit alpha
// test.  Replaces traceRayEXT over the driver-built TLAS/BLAS and the any-hit
// shader path_trace_rahit.glsl:174-188.
//
// Closest-hit rule (deterministic, independent of traversal order): accept a
// triangle at t in [tmin, tmax] when t < best or (t == best and its
// flattened prim id is lower).  With the watertight test evaluated in the
// same operation order as the oracle (no FMA), the hit prim id of every ray
// is bit-exact with the oracle's independent binary-tree traversal.
#pragma once

#include "devmath.cuh"
#include "hx_internal.h"

struct RayPre {
    V3 o;
    int kx, ky, kz;
    float sx, sy, sz;
    float ix, iy, iz;  // safe reciprocal direction for the slab tests
};

HXD float safe_inv(float d) {
    float a = fabsf(d) < 1e-20f ? copysignf(1e-20f, d) : d;
    return 1.0f / a;
}

HXD RayPre ray_prepare(V3 o, V3 d) {
    RayPre p;
    p.o = o;
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    int kz = 0;
    if (ay > ax) kz = 1;
    if (az > (kz == 0 ? ax : ay)) kz = 2;
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    if (comp(d, kz) < 0.0f) { int t = kx; kx = ky; ky = t; }
    p.kx = kx; p.ky = ky; p.kz = kz;
    float dz = comp(d, kz);
    p.sx = comp(d, kx) / dz;
    p.sy = comp(d, ky) / dz;
    p.sz = 1.0f / dz;
    p.ix = safe_inv(d.x); p.iy = safe_inv(d.y); p.iz = safe_inv(d.z);
    return p;
}

// Woop/Benthin/Wald 2013 watertight test (no double-precision fallback).
HXD bool intersect_tri(const RayPre& r, V3 v0, V3 v1, V3 v2, float tmin, float tmax, float& t_out, float& u_out,
                       float& v_out) {
    V3 A = v0 - r.o, B = v1 - r.o, C = v2 - r.o;
    float Akz = comp(A, r.kz), Bkz = comp(B, r.kz), Ckz = comp(C, r.kz);
    float Ax = comp(A, r.kx) - r.sx * Akz;
    float Ay = comp(A, r.ky) - r.sy * Akz;
    float Bx = comp(B, r.kx) - r.sx * Bkz;
    float By = comp(B, r.ky) - r.sy * Bkz;
    float Cx = comp(C, r.kx) - r.sx * Ckz;
    float Cy = comp(C, r.ky) - r.sy * Ckz;
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    float det = U + V + W;
    if (det == 0.0f) return false;
    float Az = r.sz * Akz, Bz = r.sz * Bkz, Cz = r.sz * Ckz;
    float T = U * Az + V * Bz + W * Cz;
    float rcp = 1.0f / det;
    float t = T * rcp;
    if (!(t >= tmin && t <= tmax)) return false;
    t_out = t;
    u_out = V * rcp;
    v_out = W * rcp;
    return true;
}

// Software bilinear RGBA8 fetch, REPEAT addressing, level 0; channel c.
HXD float tex_bilinear(const DevScene& s, uint32_t tex, float u, float v, int c) {
    uint4 td = s.tex_desc[tex];
    int W = (int)td.y, H = (int)td.z;
    float x = u * (float)W - 0.5f, y = v * (float)H - 0.5f;
    float x0 = floorf(x), y0 = floorf(y);
    float fx = x - x0, fy = y - y0;
    int ix0 = (((int)x0 % W) + W) % W, iy0 = (((int)y0 % H) + H) % H;
    int ix1 = (ix0 + 1) % W, iy1 = (iy0 + 1) % H;
    const uint32_t* t = s.texels + td.x;
    int sh = 8 * c;
    float a00 = (float)((__ldg(t + iy0 * W + ix0) >> sh) & 0xffu) / 255.0f;
    float a10 = (float)((__ldg(t + iy0 * W + ix1) >> sh) & 0xffu) / 255.0f;
    float a01 = (float)((__ldg(t + iy1 * W + ix0) >> sh) & 0xffu) / 255.0f;
    float a11 = (float)((__ldg(t + iy1 * W + ix1) >> sh) & 0xffu) / 255.0f;
    float top = a00 + (a10 - a00) * fx;
    float bot = a01 + (a11 - a01) * fx;
    return top + (bot - top) * fy;
}

// Any-hit alpha test: interpolated UV, albedo alpha, reject below 0.1.
HXD bool alpha_pass(const DevScene& s, uint32_t prim, float u, float v) {
    float4 a = __ldg(&s.alpha_uv[2 * (size_t)prim]);
    float4 b = __ldg(&s.alpha_uv[2 * (size_t)prim + 1]);
    uint32_t tex = __float_as_uint(b.z);
    float alpha;
    if (tex == 0xffffffffu) alpha = b.w;
    else {
        float b0 = 1.0f - u - v;
        float tu = a.x * b0 + a.z * u + b.x * v;
        float tv = a.y * b0 + a.w * u + b.y * v;
        alpha = tex_bilinear(s, tex, tu, tv, 3);
    }
    return !(alpha < 0.1f);
}

struct HitRec {
    float t, u, v;
    uint32_t prim;
};

constexpr int kStackSize = 64;

// Node child-box decode + slab test for all 8 slots; returns a hit mask
// and the entry distances.
HXD uint32_t node_intersect(const hx_bvh8_node& n, const RayPre& r, float tmin, float lim, float* tn_out) {
    uint32_t mask = 0;
    float sx = __uint_as_float((uint32_t)((int)n.exponent[0] + 127) << 23);
    float sy = __uint_as_float((uint32_t)((int)n.exponent[1] + 127) << 23);
    float sz = __uint_as_float((uint32_t)((int)n.exponent[2] + 127) << 23);
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        if (n.meta[c] == 0) continue;
        float lx = n.origin[0] + (float)n.qlo[0][c] * sx, hx = n.origin[0] + (float)n.qhi[0][c] * sx;
        float ly = n.origin[1] + (float)n.qlo[1][c] * sy, hy = n.origin[1] + (float)n.qhi[1][c] * sy;
        float lz = n.origin[2] + (float)n.qlo[2][c] * sz, hz = n.origin[2] + (float)n.qhi[2][c] * sz;
        float t0x = (lx - r.o.x) * r.ix, t1x = (hx - r.o.x) * r.ix;
        float t0y = (ly - r.o.y) * r.iy, t1y = (hy - r.o.y) * r.iy;
        float t0z = (lz - r.o.z) * r.iz, t1z = (hz - r.o.z) * r.iz;
        float tn = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fmaxf(fminf(t0z, t1z), tmin));
        float tf = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fminf(fmaxf(t0z, t1z), lim));
        if (tn <= tf * 1.000000477f) {
            mask |= 1u << c;
            tn_out[c] = tn;
        }
    }
    return mask;
}

HXD void load_node(const hx_bvh8_node* nodes, uint32_t idx, hx_bvh8_node& n) {
    const uint4* src = reinterpret_cast<const uint4*>(nodes + idx);
    uint4* dst = reinterpret_cast<uint4*>(&n);
#pragma unroll
    for (int k = 0; k < 5; ++k) dst[k] = __ldg(src + k);
}

// Closest hit (shadow = false) or first accepted hit (shadow = true).
// Sets overflow when the traversal stack overflowed or the node-visit cap
// was hit (results then incomplete; the host reports HX_ERR_DEVICE).
struct TraverseCount {
    uint32_t nodes = 0, tris = 0;
};

template <bool COUNT = false>
HXD bool trace_bvh8(const DevScene& s, V3 o, V3 d, float tmin, float tmax, bool any_hit, bool shadow, HitRec& hit,
                    bool& overflow, TraverseCount* tc = nullptr) {
    if (s.num_nodes == 0) return false;
    RayPre r = ray_prepare(o, d);
    float best_t = tmax, bu = 0.0f, bv = 0.0f;
    uint32_t best = kNoHit;
    uint32_t stack[kStackSize];
    int sp = 0;
    uint32_t node_idx = 0;
    // A valid traversal visits each node at most once; the cap turns a
    // malformed tree into a reported error instead of an endless loop.
    uint32_t visits_left = s.num_nodes + 16;
    for (;;) {
        if (visits_left-- == 0 || node_idx >= s.num_nodes) {
            overflow = true;
            break;
        }
        hx_bvh8_node n;
        load_node(s.nodes, node_idx, n);
        if (COUNT) tc->nodes++;
        float tn[8];
        uint32_t mask = node_intersect(n, r, tmin, best_t * 1.000001f, tn);
        // leaves first (slot order), then push internal children far-to-near
        uint32_t leaf_mask = mask & ~(uint32_t)n.internal_mask;
        while (leaf_mask) {
            int c = __ffs(leaf_mask) - 1;
            leaf_mask &= leaf_mask - 1;
            uint32_t m = n.meta[c];
            uint32_t cnt = m >> 5, off = m & 31u;
            for (uint32_t q = 0; q < cnt; ++q) {
                uint32_t k = n.prim_base + off + q;
                if (k >= s.num_prims) {
                    overflow = true;
                    break;
                }
                if (COUNT) tc->tris++;
                float4 a = __ldg(&s.tri[3 * (size_t)k]);
                float4 b = __ldg(&s.tri[3 * (size_t)k + 1]);
                float4 cc = __ldg(&s.tri[3 * (size_t)k + 2]);
                float t, u, v;
                if (!intersect_tri(r, v3(a), v3(b), v3(cc), tmin, best_t, t, u, v)) continue;
                uint32_t prim = __float_as_uint(a.w);
                if (!(t < best_t || (t == best_t && prim < best))) continue;
                if (any_hit && (__float_as_uint(b.w) & HX_TRI_NONOPAQUE) && !alpha_pass(s, prim, u, v)) continue;
                best_t = t; bu = u; bv = v; best = prim;
                if (shadow) {
                    hit.t = t; hit.u = u; hit.v = v; hit.prim = prim;
                    return true;
                }
            }
        }
        uint32_t int_mask = mask & (uint32_t)n.internal_mask;
        // order internal hits by entry distance (insertion sort, <= 8)
        uint32_t ids[8];
        float ds[8];
        int nh = 0;
        while (int_mask) {
            int c = __ffs(int_mask) - 1;
            int_mask &= int_mask - 1;
            float dist = tn[c];
            uint32_t child = n.child_base + (n.meta[c] & 7u);
            int j = nh++;
            while (j > 0 && ds[j - 1] < dist) { ds[j] = ds[j - 1]; ids[j] = ids[j - 1]; --j; }
            ds[j] = dist;
            ids[j] = child;
        }
        // ds is sorted descending: push far first, the nearest is visited next
        if (nh > 0) {
            for (int j = 0; j < nh - 1; ++j) {
                if (sp < kStackSize) stack[sp++] = ids[j];
                else overflow = true;
            }
            node_idx = ids[nh - 1];
            continue;
        }
        if (sp == 0) break;
        node_idx = stack[--sp];
    }
    if (best == kNoHit) return false;
    hit.t = best_t; hit.u = bu; hit.v = bv; hit.prim = best;
    return true;
}
