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
    p.ix = safe_inv(d.x); p.iy = safe_inv(d.y); p.iz = safe_inv(d.z);
    // |d_kz| is the largest component, so safe_inv(d_kz) = 1 / d_kz: the
    // shear constants scale by it (one division per ray instead of three more)
    p.sz = kz == 0 ? p.ix : (kz == 1 ? p.iy : p.iz);
    p.sx = comp(d, kx) * p.sz;
    p.sy = comp(d, ky) * p.sz;
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

// q / 255 for a byte q, equal to the IEEE quotient (float)q / 255.0f for all
// 256 values (checked exhaustively in exact arithmetic): a product with the
// rounded reciprocal, corrected by one FMA residual step.
HXD float unorm8(uint32_t q) {
    const float c = 1.0f / 255.0f;
    const float x = (float)q;
    const float r = __fmul_rn(x, c);
    const float e = __fmaf_rn(-r, 255.0f, x);
    return __fmaf_rn(e, c, r);
}

// SNORM byte: max(int8(q) / 127, -1), the IEEE quotient (*_SNORM texels).
HXD float snorm8(uint32_t q) { return fmaxf(__fdiv_rn((float)(int8_t)(uint8_t)q, 127.0f), -1.0f); }

// Texel channel value of an 8-bit texel by encoding: 0 UNORM q / 255, 1 the
// sRGB-decoded linear value (an sRGB texture's RGB; alpha is never
// sRGB-encoded), 2 SNORM (every channel).
HXD float texel_value(const DevScene& s, uint32_t q, uint32_t enc) {
    return enc == 1u ? __ldg(s.srgb_lut + q) : (enc ? snorm8(q) : unorm8(q));
}

// Bilinear taps with REPEAT addressing at level 0: the four texel indices
// (row-major within the texture) and the fractional weights.  Power-of-two
// sizes wrap with a mask (the same integers as the modulo).
struct TexTaps {
    int i00, i10, i01, i11;
    float fx, fy;
};
HXD TexTaps tex_taps(uint4 td, float u, float v) {
    int W = (int)td.y, H = (int)td.z;
    float x = u * (float)W - 0.5f, y = v * (float)H - 0.5f;
    float x0 = floorf(x), y0 = floorf(y);
    TexTaps r;
    r.fx = x - x0;
    r.fy = y - y0;
    int ix0, iy0, ix1, iy1;
    if (((W & (W - 1)) | (H & (H - 1))) == 0) {
        ix0 = (int)x0 & (W - 1);
        iy0 = (int)y0 & (H - 1);
        ix1 = (ix0 + 1) & (W - 1);
        iy1 = (iy0 + 1) & (H - 1);
    } else {
        ix0 = (((int)x0 % W) + W) % W;
        iy0 = (((int)y0 % H) + H) % H;
        ix1 = ix0 + 1 == W ? 0 : ix0 + 1;
        iy1 = iy0 + 1 == H ? 0 : iy0 + 1;
    }
    r.i00 = iy0 * W + ix0;
    r.i10 = iy0 * W + ix1;
    r.i01 = iy1 * W + ix0;
    r.i11 = iy1 * W + ix1;
    return r;
}

HXD float bilerp(const TexTaps& k, float a00, float a10, float a01, float a11) {
    float top = a00 + (a10 - a00) * k.fx;
    float bot = a01 + (a11 - a01) * k.fx;
    return top + (bot - top) * k.fy;
}

// Channel c of an RGBA16F texel (two 32-bit words: R | G << 16, B | A << 16).
HXD float half_channel(uint2 q, int c) {
    const uint32_t w = c < 2 ? q.x : q.y;
    return __half2float(__ushort_as_half((unsigned short)((c & 1) ? (w >> 16) : (w & 0xffffu))));
}

// Texture flag bits (tex_desc.w): bit 0 sRGB-encoded RGB, bit 1 RGBA16F texels
// (half-float formats; two words per texel at an even word offset), bit 2
// SNORM RGBA8 texels.
constexpr uint32_t kTexSrgb = 1u, kTexHalf = 2u, kTexSnorm = 4u;

// Software bilinear fetch, REPEAT addressing, level 0; channel c.  RGBA8
// textures: q / 255 per texel, sRGB textures decode texels before filtering,
// as sampled *_SRGB images do, SNORM textures max(int8 / 127, -1); RGBA16F
// textures: the half values.
HXD float tex_bilinear(const DevScene& s, uint32_t tex, float u, float v, int c) {
    const uint4 td = s.tex_desc[tex];
    const TexTaps k = tex_taps(td, u, v);
    if (td.w & kTexHalf) {
        const uint2* t = reinterpret_cast<const uint2*>(s.texels + td.x);
        return bilerp(k, half_channel(__ldg(t + k.i00), c), half_channel(__ldg(t + k.i10), c),
                      half_channel(__ldg(t + k.i01), c), half_channel(__ldg(t + k.i11), c));
    }
    const uint32_t* t = s.texels + td.x;
    int sh = 8 * c;
    const uint32_t enc = (td.w & kTexSnorm) ? 2u : (((td.w & kTexSrgb) && c < 3) ? 1u : 0u);
    float a00 = texel_value(s, (__ldg(t + k.i00) >> sh) & 0xffu, enc);
    float a10 = texel_value(s, (__ldg(t + k.i10) >> sh) & 0xffu, enc);
    float a01 = texel_value(s, (__ldg(t + k.i01) >> sh) & 0xffu, enc);
    float a11 = texel_value(s, (__ldg(t + k.i11) >> sh) & 0xffu, enc);
    return bilerp(k, a00, a10, a01, a11);
}

// tex_bilinear for channels 0, 1, 2 at once: one address computation and one
// fetch of the four texels, the same per-channel arithmetic.
HXD V3 tex_bilinear_rgb(const DevScene& s, uint32_t tex, float u, float v) {
    const uint4 td = s.tex_desc[tex];
    const TexTaps k = tex_taps(td, u, v);
    float r[3];
    if (td.w & kTexHalf) {
        const uint2* t = reinterpret_cast<const uint2*>(s.texels + td.x);
        const uint2 t00 = __ldg(t + k.i00), t10 = __ldg(t + k.i10), t01 = __ldg(t + k.i01), t11 = __ldg(t + k.i11);
#pragma unroll
        for (int c = 0; c < 3; ++c)
            r[c] = bilerp(k, half_channel(t00, c), half_channel(t10, c), half_channel(t01, c), half_channel(t11, c));
        return v3(r[0], r[1], r[2]);
    }
    const uint32_t* t = s.texels + td.x;
    const uint32_t t00 = __ldg(t + k.i00), t10 = __ldg(t + k.i10);
    const uint32_t t01 = __ldg(t + k.i01), t11 = __ldg(t + k.i11);
    const uint32_t enc = (td.w & kTexSnorm) ? 2u : ((td.w & kTexSrgb) ? 1u : 0u);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const int sh = 8 * c;
        float a00 = texel_value(s, (t00 >> sh) & 0xffu, enc), a10 = texel_value(s, (t10 >> sh) & 0xffu, enc);
        float a01 = texel_value(s, (t01 >> sh) & 0xffu, enc), a11 = texel_value(s, (t11 >> sh) & 0xffu, enc);
        r[c] = bilerp(k, a00, a10, a01, a11);
    }
    return v3(r[0], r[1], r[2]);
}

// Bilinear alpha of an RGBA16F or SNORM texture, out of line: the any-hit test
// inside the traversal loop carries only the A8 path's code.
static __device__ __noinline__ float tex_alpha_wide(const uint32_t* __restrict__ texels, uint4 td, float u, float v) {
    const TexTaps k = tex_taps(td, u, v);
    if (td.w & kTexHalf) {
        const uint2* t = reinterpret_cast<const uint2*>(texels + td.x);
        return bilerp(k, half_channel(__ldg(t + k.i00), 3), half_channel(__ldg(t + k.i10), 3),
                      half_channel(__ldg(t + k.i01), 3), half_channel(__ldg(t + k.i11), 3));
    }
    const uint32_t* t = texels + td.x;  // SNORM
    return bilerp(k, snorm8(__ldg(t + k.i00) >> 24), snorm8(__ldg(t + k.i10) >> 24), snorm8(__ldg(t + k.i01) >> 24),
                  snorm8(__ldg(t + k.i11) >> 24));
}

// Bilinear alpha of a UNORM/sRGB RGBA8 texture from the scene's A8 copy (the
// same texel bytes and arithmetic as tex_bilinear(..., 3), a quarter of the
// cache footprint).
HXD float tex_alpha_bilinear(const DevScene& s, uint32_t tex, float u, float v) {
    uint4 td = s.tex_desc[tex];
    int W = (int)td.y, H = (int)td.z;
    float x = u * (float)W - 0.5f, y = v * (float)H - 0.5f;
    float x0 = floorf(x), y0 = floorf(y);
    float fx = x - x0, fy = y - y0;
    int ix0, iy0, ix1, iy1;
    if (((W & (W - 1)) | (H & (H - 1))) == 0) {
        ix0 = (int)x0 & (W - 1);
        iy0 = (int)y0 & (H - 1);
        ix1 = (ix0 + 1) & (W - 1);
        iy1 = (iy0 + 1) & (H - 1);
    } else {
        ix0 = (((int)x0 % W) + W) % W;
        iy0 = (((int)y0 % H) + H) % H;
        ix1 = ix0 + 1 == W ? 0 : ix0 + 1;
        iy1 = iy0 + 1 == H ? 0 : iy0 + 1;
    }
    const uint8_t* t = s.alpha8 + td.x;
    float a00 = unorm8(__ldg(t + iy0 * W + ix0));
    float a10 = unorm8(__ldg(t + iy0 * W + ix1));
    float a01 = unorm8(__ldg(t + iy1 * W + ix0));
    float a11 = unorm8(__ldg(t + iy1 * W + ix1));
    float top = a00 + (a10 - a00) * fx;
    float bot = a01 + (a11 - a01) * fx;
    return top + (bot - top) * fy;
}

// Any-hit alpha test: interpolated UV, albedo alpha, reject below 0.1.  The
// record's texture word is the albedo texture index, 0xffffffff for none, or
// the index | 0x80000000 for an RGBA16F / SNORM texture ("wide" alpha, read
// without the A8 copy).  Only scenes with such records (DevScene::wide_alpha)
// run the WA instantiation; the others carry no code for it.
template <bool WA>
HXD bool alpha_pass(const DevScene& s, uint32_t prim, float u, float v) {
    float4 a = __ldg(&s.alpha_uv[2 * (size_t)prim]);
    float4 b = __ldg(&s.alpha_uv[2 * (size_t)prim + 1]);
    uint32_t tex = __float_as_uint(b.z);
    float alpha;
    if (WA && (int32_t)tex < 0 && tex != 0xffffffffu) {
        float b0 = 1.0f - u - v;
        float tu = a.x * b0 + a.z * u + b.x * v;
        float tv = a.y * b0 + a.w * u + b.y * v;
        alpha = tex_alpha_wide(s.texels, s.tex_desc[tex & 0x7fffffffu], tu, tv);
    } else if (tex == 0xffffffffu) alpha = b.w;
    else {
        float b0 = 1.0f - u - v;
        float tu = a.x * b0 + a.z * u + b.x * v;
        float tv = a.y * b0 + a.w * u + b.y * v;
        alpha = tex_alpha_bilinear(s, tex, tu, tv);
    }
    return !(alpha < 0.1f);
}

constexpr int kStackSize = (int)kTraversalStackEntries;

HXD uint32_t byte_of(uint32_t w, int k) { return (w >> (8 * k)) & 0xffu; }

// 1 + q 2^-15 for byte k of w, built with one byte permute (bits
// 0x3F80 | q << 8 | 0x00: the byte fills mantissa bits 15..8 of 1.0).
HXD float byte_plane(uint32_t w, int k) { return __uint_as_float(__byte_perm(w, 0x3F800000u, 0x7604u | (k << 4))); }

// Slab distances of one node axis in the form t = f A + C, f = 1 + q 2^-15
// the byte-plane value of a child plane q: with the node grid origin g and
// step S = 2^e, the plane is L = g + q S, so
//   t = (L - o) inv = b + q S inv = f A + (b - A),  A = 2^(e+15) inv,
//   b = (g - o) inv
// (A is exact: a power-of-two multiple of inv).  Rounding of b, of b - A and
// of the final FMA is below 2^-22 (|b| + |A|) in total, and the reciprocal's
// own rounding below 2^-24 (|b| + |A|) of the true distance, so moving the
// near constant down and the far constant up by 2^-21 (|b| + |A|) keeps every
// child slab conservative: a box the ray meets is never culled.
struct AxisSlab {
    float2 A;   // (A, A)
    float2 C;   // (b - A - delta, b - A + delta)
};
HXD AxisSlab axis_slab(uint32_t origin_bits, uint32_t exp_byte, float o, float inv) {
    const int e = (int)(int8_t)exp_byte;
    const float A = __uint_as_float((uint32_t)(e + 142) << 23) * inv;
    const float b = (__uint_as_float(origin_bits) - o) * inv;
    const float C = b - A;
    const float delta = (fabsf(b) + fabsf(A)) * 4.76837158203125e-7f;  // 2^-21
    AxisSlab r;
    r.A = make_float2(A, A);
    r.C = make_float2(C - delta, C + delta);
    return r;
}

// Intersects the ray with the (up to) 8 children of a node held in five
// 16-byte words and returns the hit mask in node-group form: bit
// 24 + (slot ^ oct_inv) for a hit internal child, bit off for the triangle of
// a hit leaf slot (bit 16, outside both masks, for an empty slot).  The meta
// bytes carry these bit positions (internal slots: 24 + slot, flagged by bit
// 7, which selects the XOR with the ray octant), four slots per word.  Each
// child axis costs one packed FMA (near, far): t = f A + C (axis_slab).
HXD uint32_t intersect_children(const uint4 w0, const uint4 w1, const uint4 w2, const uint4 w3, const uint4 w4,
                                const RayPre& r, uint32_t oct_inv, float tmin, float lim) {
    const AxisSlab X = axis_slab(w0.x, w0.w & 0xffu, r.o.x, r.ix);
    const AxisSlab Y = axis_slab(w0.y, (w0.w >> 8) & 0xffu, r.o.y, r.iy);
    const AxisSlab Z = axis_slab(w0.z, (w0.w >> 16) & 0xffu, r.o.z, r.iz);
    // near/far byte planes per axis chosen by the direction sign
    const bool nx = r.ix < 0.0f, ny = r.iy < 0.0f, nz = r.iz < 0.0f;
    const uint32_t lox0 = w2.x, lox1 = w2.y, loy0 = w2.z, loy1 = w2.w, loz0 = w3.x, loz1 = w3.y;
    const uint32_t hix0 = w3.z, hix1 = w3.w, hiy0 = w4.x, hiy1 = w4.y, hiz0 = w4.z, hiz1 = w4.w;
    const uint32_t nx0 = nx ? hix0 : lox0, nx1 = nx ? hix1 : lox1, fx0 = nx ? lox0 : hix0, fx1 = nx ? lox1 : hix1;
    const uint32_t ny0 = ny ? hiy0 : loy0, ny1 = ny ? hiy1 : loy1, fy0 = ny ? loy0 : hiy0, fy1 = ny ? loy1 : hiy1;
    const uint32_t nz0 = nz ? hiz0 : loz0, nz1 = nz ? hiz1 : loz1, fz0 = nz ? loz0 : hiz0, fz1 = nz ? loz1 : hiz1;
    const uint32_t mw0 = (w1.z ^ (((w1.z & 0x80808080u) >> 7) * oct_inv)) & 0x1f1f1f1fu;
    const uint32_t mw1 = (w1.w ^ (((w1.w & 0x80808080u) >> 7) * oct_inv)) & 0x1f1f1f1fu;
    uint32_t hits = 0;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const uint32_t pos = byte_of(c < 4 ? mw0 : mw1, c & 3);
        const int k = c & 3;
        const float2 tx = fma2_rn(make_float2(byte_plane(c < 4 ? nx0 : nx1, k), byte_plane(c < 4 ? fx0 : fx1, k)), X.A, X.C);
        const float2 ty = fma2_rn(make_float2(byte_plane(c < 4 ? ny0 : ny1, k), byte_plane(c < 4 ? fy0 : fy1, k)), Y.A, Y.C);
        const float2 tz = fma2_rn(make_float2(byte_plane(c < 4 ? nz0 : nz1, k), byte_plane(c < 4 ? fz0 : fz1, k)), Z.A, Z.C);
        const float tn = fmaxf(max3f(tx.x, ty.x, tz.x), tmin);
        const float tf = fminf(min3f(tx.y, ty.y, tz.y), lim);
        if (tn <= tf) hits |= 1u << pos;
    }
    return hits;
}

// Counting mode: lane-level node visits and triangle tests, and the
// warp-level steps that executed them (lanes per warp step = SIMD
// utilisation of each phase).
struct TraverseCount {
    uint32_t nodes = 0, tris = 0;
    uint32_t warp_nodes = 0, warp_tris = 0;
    uint32_t alpha = 0;  // any-hit alpha tests
};

HXD bool lowest_active_lane() { return (threadIdx.x & 31u) == (uint32_t)(__ffs(__activemask()) - 1); }

// ---------------------------------------------------------------------------
// Persistent-warp traversal: per-lane state machine.  One call of step()
// intersects at most one node and then tests the triangles it exposed; a
// lane whose ray finished refills itself with the next ray of the queue, so
// long rays never hold their warp-mates idle.
// ---------------------------------------------------------------------------
struct TravState {
    RayPre r;
    uint32_t oct_inv;
    float tmin, best_t, bu, bv;
    uint32_t best;
    uint32_t g_base, g_mask, t_base, t_mask;
    int sp;
    uint32_t visits_left;
    bool any_hit;
    bool shadow;  // first accepted hit ends the ray
};

HXD void trav_init(TravState& st, const DevScene& s, V3 o, V3 d, float tmin, float tmax, bool any_hit) {
    st.r = ray_prepare(o, d);
    const uint32_t oct = (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u);
    st.oct_inv = 7u - oct;
    st.tmin = tmin;
    st.best_t = tmax;
    st.bu = st.bv = 0.0f;
    st.best = kNoHit;
    st.g_base = 0;
    st.g_mask = s.num_nodes ? ((1u << (24 + st.oct_inv)) | 1u) : 0u;
    st.t_base = 0;
    st.t_mask = 0;
    st.sp = 0;
    st.visits_left = s.num_nodes + 16;
    st.any_hit = any_hit;
    st.shadow = false;
}

// Traversal record of a ray, computed where the ray is made (ray generation
// and shading, which run convergent) so that the persistent traversal's
// refill only loads it:
//   r0 = (1/dx, 1/dy, 1/dz [safe_inv], tmax)
//   r1 = (Sx, Sy, Sz, bits)   the watertight test's shear; bits: kx | ky << 2 |
//        kz << 4 | octant << 6 | any-hit << 9 (octant from the signs of d, as
//        trav_init)
// The values are those ray_prepare computes, so traversal from a record is
// bit-identical to traversal from (o, d).
HXD void ray_record(V3 d, float tmax, bool any_hit, float4& r0, float4& r1) {
    const RayPre p = ray_prepare(v3(0.0f), d);
    const uint32_t oct = (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u);
    const uint32_t bits = (uint32_t)p.kx | ((uint32_t)p.ky << 2) | ((uint32_t)p.kz << 4) | (oct << 6) |
                          (any_hit ? 1u << 9 : 0u);
    r0 = make_float4(p.ix, p.iy, p.iz, tmax);
    r1 = make_float4(p.sx, p.sy, p.sz, __uint_as_float(bits));
}

HXD void trav_init_record(TravState& st, const DevScene& s, float4 o_tmin, float4 r0, float4 r1) {
    const uint32_t bits = __float_as_uint(r1.w);
    st.r.o = v3(o_tmin);
    st.r.kx = (int)(bits & 3u);
    st.r.ky = (int)((bits >> 2) & 3u);
    st.r.kz = (int)((bits >> 4) & 3u);
    st.r.sx = r1.x; st.r.sy = r1.y; st.r.sz = r1.z;
    st.r.ix = r0.x; st.r.iy = r0.y; st.r.iz = r0.z;
    st.oct_inv = 7u - ((bits >> 6) & 7u);
    st.tmin = o_tmin.w;
    st.best_t = r0.w;
    st.bu = st.bv = 0.0f;
    st.best = kNoHit;
    st.g_base = 0;
    st.g_mask = s.num_nodes ? ((1u << (24 + st.oct_inv)) | 1u) : 0u;
    st.t_base = 0;
    st.t_mask = 0;
    st.sp = 0;
    st.visits_left = s.num_nodes + 16;
    st.any_hit = (bits >> 9) & 1u;
    st.shadow = false;
}

// One step of a lane's traversal: visits one node and tests the triangles it
// exposed.  Returns true when the ray is finished (traversal exhausted, or
// the first accepted hit of a shadow ray, st.shadow).
template <bool COUNT, bool WA>
HXD bool trav_step(TravState& st, uint2* stack, const DevScene& s, bool& overflow, TraverseCount* tc) {
    if (st.g_mask > 0x00ffffffu) {
        const uint32_t bit = 31u - __clz(st.g_mask);
        st.g_mask &= ~(1u << bit);
        const uint32_t slot = (bit - 24u) ^ st.oct_inv;
        const uint32_t child = st.g_base + __popc(st.g_mask & 0xffu & ((1u << slot) - 1u));
        if (st.g_mask > 0x00ffffffu) {
            if (st.sp < s.stack_limit) stack[st.sp++] = make_uint2(st.g_base, st.g_mask);
            else overflow = true;
        }
        if (st.visits_left-- == 0 || child >= s.num_nodes) {
            overflow = true;
            return true;
        }
        const uint4* np = reinterpret_cast<const uint4*>(s.nodes + child);
        const uint4 w0 = __ldg(np), w1 = __ldg(np + 1), w2 = __ldg(np + 2), w3 = __ldg(np + 3), w4 = __ldg(np + 4);
        if (COUNT) {
            tc->nodes++;
            if (lowest_active_lane()) tc->warp_nodes++;
        }
        const uint32_t hm = intersect_children(w0, w1, w2, w3, w4, st.r, st.oct_inv, st.tmin,
                                               st.best_t * 1.000001f);
        st.g_base = w1.x;
        st.g_mask = (hm & 0xff000000u) | (w0.w >> 24);
        st.t_base = w1.y;
        st.t_mask = hm & 0xffu;
    } else {
        st.t_base = st.g_base;
        st.t_mask = st.g_mask;
        st.g_mask = 0;
    }
    while (st.t_mask) {
        const uint32_t b = __ffs(st.t_mask) - 1u;
        st.t_mask &= st.t_mask - 1u;
        const uint32_t k = st.t_base + b;
        if (k >= s.num_prims) {
            overflow = true;
            return true;
        }
        if (COUNT) {
            tc->tris++;
            if (lowest_active_lane()) tc->warp_tris++;
        }
        const float4 a = __ldg(&s.tri[3 * (size_t)k]);
        const float4 bb = __ldg(&s.tri[3 * (size_t)k + 1]);
        const float4 cc = __ldg(&s.tri[3 * (size_t)k + 2]);
        float t, u, v;
        if (!intersect_tri(st.r, v3(a), v3(bb), v3(cc), st.tmin, st.best_t, t, u, v)) continue;
        const uint32_t prim = __float_as_uint(a.w);
        if (!(t < st.best_t || (t == st.best_t && prim < st.best))) continue;
        if (st.any_hit && (__float_as_uint(bb.w) & HX_TRI_NONOPAQUE)) {
            if (COUNT) tc->alpha++;
            if (!alpha_pass<WA>(s, prim, u, v)) continue;
        }
        st.best_t = t; st.bu = u; st.bv = v; st.best = prim;
        if (st.shadow) return true;
    }
    if (st.g_mask <= 0x00ffffffu) {
        if (st.sp == 0) return true;
        const uint2 e = stack[--st.sp];
        st.g_base = e.x;
        st.g_mask = e.y;
    }
    return false;
}

// ---------------------------------------------------------------------------
// Batched traversal: lanes visit nodes on their own rays, but the triangles
// their nodes expose go to a per-warp queue that the whole warp tests
// together, one triangle per lane (a triangle test by one lane of a warp
// otherwise holds the other 31 idle).  The closest hit of a ray is the
// lexicographic minimum of (t, triangle id) over its accepted triangles —
// independent of the order they are tested in — kept as one 64-bit key per
// ray in shared memory (atomicMin).
// ---------------------------------------------------------------------------

// One node visit: pops the next internal child of the current group,
// intersects its children against [tmin, best_t] and returns the leaf
// triangles it hit (bits over t_base).  Afterwards g_mask holds the next
// group to visit (from the stack when the node hit no internal child) or is
// <= 0xffffff when the ray has no node left.
template <bool COUNT>
HXD uint32_t node_step(TravState& st, uint2* stack, const DevScene& s, float best_t, bool& overflow, TraverseCount* tc,
                       uint32_t& t_base) {
    const uint32_t bit = 31u - __clz(st.g_mask);
    st.g_mask &= ~(1u << bit);
    const uint32_t slot = (bit - 24u) ^ st.oct_inv;
    const uint32_t child = st.g_base + __popc(st.g_mask & 0xffu & ((1u << slot) - 1u));
    if (st.g_mask > 0x00ffffffu) {
        if (st.sp < s.stack_limit) stack[st.sp++] = make_uint2(st.g_base, st.g_mask);
        else overflow = true;
    }
    if (st.visits_left-- == 0 || child >= s.num_nodes) {
        overflow = true;
        st.g_mask = 0;
        st.sp = 0;
        return 0u;
    }
    const uint4* np = reinterpret_cast<const uint4*>(s.nodes + child);
    const uint4 w0 = __ldg(np), w1 = __ldg(np + 1), w2 = __ldg(np + 2), w3 = __ldg(np + 3), w4 = __ldg(np + 4);
    if (COUNT) {
        tc->nodes++;
        if (lowest_active_lane()) tc->warp_nodes++;
    }
    const uint32_t hm = intersect_children(w0, w1, w2, w3, w4, st.r, st.oct_inv, st.tmin,
                                           best_t * 1.000001f);
    st.g_base = w1.x;
    st.g_mask = (hm & 0xff000000u) | (w0.w >> 24);
    t_base = w1.y;
    if (st.g_mask <= 0x00ffffffu && st.sp > 0) {
        const uint2 e = stack[--st.sp];
        st.g_base = e.x;
        st.g_mask = e.y;
    }
    return hm & 0xffu;
}

// Per-warp shared state of the batched traversal: per lane the best key of
// its ray (t bits << 32 | triangle id), the barycentrics of that hit and the
// ray's queue index; the queue of triangles to test (owner lane << 27 |
// leaf-triangle index).  The testing lane reads the owner's origin and shear
// from the ray's traversal record in global memory.
// 32 entries (3 KB of shared memory per 4-warp block) let 8 blocks fit the
// 32 KB shared-memory configuration, which leaves 224 KB of the SM's 256 KB
// to L1 (a 64-entry queue got the 100 KB configuration: L1 hit rate 58.5 %
// vs 64.9 %, 273 vs 278 Mpaths/s; 24 entries overflow: -4 %).
constexpr uint32_t kTriQueueCap = 32;
constexpr uint32_t kShadowRid = 0x80000000u;
struct WarpTris {
    unsigned long long key[32];
    float2 uv[32];
    uint32_t rid[32];  // queue index | kShadowRid
    uint32_t tri[kTriQueueCap];
};

// Tests the first n queued triangles, one per lane and round (all 32 lanes
// call it together); accepted hits lower their ray's key.
template <bool COUNT, bool WA>
HXD void warp_test_tris(WarpTris& w, uint32_t lane, uint32_t n, const DevScene& s, const float4* __restrict__ qo,
                        const float4* __restrict__ qr1, const float4* __restrict__ so, const float4* __restrict__ sr1,
                        bool& overflow, TraverseCount* tc) {
    for (uint32_t b0 = 0; b0 < n; b0 += 32u) {
        const uint32_t e = b0 + lane;
        unsigned long long cand = ~0ull;
        uint32_t own = 0;
        float cu = 0.0f, cv = 0.0f;
        if (e < n) {
            const uint32_t ent = w.tri[e];
            const uint32_t k = ent & 0x07ffffffu;
            own = ent >> 27;
            if (COUNT) {
                tc->tris++;
                if (lowest_active_lane()) tc->warp_tris++;
            }
            if (k < s.num_prims) {
                const float4 a = __ldg(&s.tri[3 * (size_t)k]);
                const float4 bb = __ldg(&s.tri[3 * (size_t)k + 1]);
                const float4 cc = __ldg(&s.tri[3 * (size_t)k + 2]);
                const uint32_t rid = w.rid[own];
                const uint32_t ri = rid & ~kShadowRid;
                const float4 ra = (rid & kShadowRid) ? so[ri] : qo[ri];
                const float4 rb = (rid & kShadowRid) ? sr1[ri] : qr1[ri];
                const unsigned long long key = w.key[own];
                const uint32_t bits = __float_as_uint(rb.w);
                RayPre r;
                r.o = v3(ra);
                r.kx = (int)(bits & 3u);
                r.ky = (int)((bits >> 2) & 3u);
                r.kz = (int)((bits >> 4) & 3u);
                r.sx = rb.x; r.sy = rb.y; r.sz = rb.z;
                r.ix = r.iy = r.iz = 0.0f;
                const float best_t = __uint_as_float((uint32_t)(key >> 32));
                const uint32_t best = (uint32_t)key;
                float t, u, v;
                if (intersect_tri(r, v3(a), v3(bb), v3(cc), ra.w, best_t, t, u, v)) {
                    const uint32_t prim = __float_as_uint(a.w);
                    if (t < best_t || (t == best_t && prim < best)) {
                        bool pass = true;
                        if ((bits & (1u << 9)) && (__float_as_uint(bb.w) & HX_TRI_NONOPAQUE)) {
                            if (COUNT) tc->alpha++;
                            pass = alpha_pass<WA>(s, prim, u, v);
                        }
                        if (pass) {
                            cand = ((unsigned long long)__float_as_uint(t) << 32) | prim;
                            atomicMin(&w.key[own], cand);
                            cu = u;
                            cv = v;
                        }
                    }
                }
            } else {
                overflow = true;
            }
        }
        __syncwarp();
        if (cand != ~0ull && w.key[own] == cand) w.uv[own] = make_float2(cu, cv);
        __syncwarp();
    }
}

// The same tests for 16-bit payloads, whose extension rays carry no traversal
// record in memory: the testing lane takes the owner's origin, tmin, shear and
// flags from the owner's registers (warp shuffles of its TravState, which
// trav_init_record filled with exactly the record's values).
template <bool COUNT, bool WA>
HXD void warp_test_tris_shfl(WarpTris& w, uint32_t lane, uint32_t n, const DevScene& s, const TravState& st,
                             bool& overflow, TraverseCount* tc) {
    const uint32_t my_bits = (uint32_t)st.r.kx | ((uint32_t)st.r.ky << 2) | ((uint32_t)st.r.kz << 4) |
                             (st.any_hit ? 1u << 9 : 0u);
    for (uint32_t b0 = 0; b0 < n; b0 += 32u) {
        const uint32_t e = b0 + lane;
        const uint32_t ent = e < n ? w.tri[e] : 0u;
        const uint32_t own = ent >> 27;
        RayPre r;
        r.o = v3(__shfl_sync(0xffffffffu, st.r.o.x, own), __shfl_sync(0xffffffffu, st.r.o.y, own),
                 __shfl_sync(0xffffffffu, st.r.o.z, own));
        const float tmin = __shfl_sync(0xffffffffu, st.tmin, own);
        r.sx = __shfl_sync(0xffffffffu, st.r.sx, own);
        r.sy = __shfl_sync(0xffffffffu, st.r.sy, own);
        r.sz = __shfl_sync(0xffffffffu, st.r.sz, own);
        const uint32_t bits = __shfl_sync(0xffffffffu, my_bits, own);
        r.kx = (int)(bits & 3u);
        r.ky = (int)((bits >> 2) & 3u);
        r.kz = (int)((bits >> 4) & 3u);
        r.ix = r.iy = r.iz = 0.0f;
        unsigned long long cand = ~0ull;
        float cu = 0.0f, cv = 0.0f;
        if (e < n) {
            const uint32_t k = ent & 0x07ffffffu;
            if (COUNT) {
                tc->tris++;
                if (lowest_active_lane()) tc->warp_tris++;
            }
            if (k < s.num_prims) {
                const float4 a = __ldg(&s.tri[3 * (size_t)k]);
                const float4 bb = __ldg(&s.tri[3 * (size_t)k + 1]);
                const float4 cc = __ldg(&s.tri[3 * (size_t)k + 2]);
                const unsigned long long key = w.key[own];
                const float best_t = __uint_as_float((uint32_t)(key >> 32));
                const uint32_t best = (uint32_t)key;
                float t, u, v;
                if (intersect_tri(r, v3(a), v3(bb), v3(cc), tmin, best_t, t, u, v)) {
                    const uint32_t prim = __float_as_uint(a.w);
                    if (t < best_t || (t == best_t && prim < best)) {
                        bool pass = true;
                        if ((bits & (1u << 9)) && (__float_as_uint(bb.w) & HX_TRI_NONOPAQUE)) {
                            if (COUNT) tc->alpha++;
                            pass = alpha_pass<WA>(s, prim, u, v);
                        }
                        if (pass) {
                            cand = ((unsigned long long)__float_as_uint(t) << 32) | prim;
                            atomicMin(&w.key[own], cand);
                            cu = u;
                            cv = v;
                        }
                    }
                }
            } else {
                overflow = true;
            }
        }
        __syncwarp();
        if (cand != ~0ull && w.key[own] == cand) w.uv[own] = make_float2(cu, cv);
        __syncwarp();
    }
}
