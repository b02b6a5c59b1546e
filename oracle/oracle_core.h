// oracle_core.h — CPU restatement of the helios shader math (TEST INFRASTRUCTURE).
//
// This header is part of the oracle: a scalar C++ transcription of the
// reference's GLSL path-tracing shaders, used only by the tests, by the
// smoke check and as the timed CPU baseline.  It is never linked into the
// product library.
//
// Parity status: the reference has no tests, golden vectors or fixtures, and
// its ray-tracing pipeline cannot run without a Vulkan stack, so this
// restatement is pinned only where the reference's CPU code compiles here
// (the Hosek-Wilkie coefficient evaluation); everything else is
// "parity unpinned" against reference outputs and is checked against the
// published definitions it cites (xoroshiro64*, Wang hash, PCG, the
// Woop/Benthin/Wald watertight test, Karras 2012).
//
// Floating-point contract shared with the device code: no FMA contraction
// (built with -ffp-contract=off; the CUDA side uses --fmad=false), IEEE
// division and square root, and the same left-to-right operation order as
// the GLSL source.  With that, every integer output (RNG draws, Morton
// codes, BVH topology, hit triangle IDs) is bit-exact between the two.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <algorithm>

namespace oracle {

// ---------------------------------------------------------------------------
// Vector types with GLSL semantics (glm is absent in the reference tree too).
// ---------------------------------------------------------------------------
template <typename R> struct V3 {
    R x, y, z;
    V3() : x(0), y(0), z(0) {}
    V3(R a, R b, R c) : x(a), y(b), z(c) {}
    explicit V3(R a) : x(a), y(a), z(a) {}
    R& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    R operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template <typename R> inline V3<R> operator+(V3<R> a, V3<R> b) { return V3<R>(a.x + b.x, a.y + b.y, a.z + b.z); }
template <typename R> inline V3<R> operator-(V3<R> a, V3<R> b) { return V3<R>(a.x - b.x, a.y - b.y, a.z - b.z); }
template <typename R> inline V3<R> operator-(V3<R> a) { return V3<R>(-a.x, -a.y, -a.z); }
template <typename R> inline V3<R> operator*(V3<R> a, V3<R> b) { return V3<R>(a.x * b.x, a.y * b.y, a.z * b.z); }
template <typename R> inline V3<R> operator/(V3<R> a, V3<R> b) { return V3<R>(a.x / b.x, a.y / b.y, a.z / b.z); }
template <typename R> inline V3<R> operator*(V3<R> a, R s) { return V3<R>(a.x * s, a.y * s, a.z * s); }
template <typename R> inline V3<R> operator*(R s, V3<R> a) { return V3<R>(s * a.x, s * a.y, s * a.z); }
// vector / scalar as one division and three products, as the device
template <typename R> inline V3<R> operator/(V3<R> a, R s) {
    const R r = R(1) / s;
    return V3<R>(a.x * r, a.y * r, a.z * r);
}
template <typename R> inline R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename R> inline V3<R> cross(V3<R> a, V3<R> b) {
    return V3<R>(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
template <typename R> inline R length(V3<R> a) { return std::sqrt(dot(a, a)); }
// normalize(v) = v / length(v): three IEEE divisions by one IEEE sqrt.
// one division (the reciprocal length) and three products, as the device
template <typename R> inline V3<R> normalize(V3<R> a) {
    const R r = R(1) / std::sqrt(dot(a, a));
    return V3<R>(a.x * r, a.y * r, a.z * r);
}
// GLSL min/max: min(x, y) = y < x ? y : x (GLSL 4.60 spec 8.3).
template <typename R> inline R gmin(R a, R b) { return b < a ? b : a; }
template <typename R> inline R gmax(R a, R b) { return a < b ? b : a; }
template <typename R> inline R gclamp(R x, R lo, R hi) { return gmin(gmax(x, lo), hi); }
template <typename R> inline V3<R> vmin(V3<R> a, V3<R> b) { return V3<R>(gmin(a.x, b.x), gmin(a.y, b.y), gmin(a.z, b.z)); }
template <typename R> inline V3<R> vmax(V3<R> a, V3<R> b) { return V3<R>(gmax(a.x, b.x), gmax(a.y, b.y), gmax(a.z, b.z)); }
// reflect(I, N) = I - 2 * dot(N, I) * N (GLSL 4.60 spec 8.5).
template <typename R> inline V3<R> reflect(V3<R> i, V3<R> n) { R d = dot(n, i); return i - n * (R(2) * d); }
template <typename R> inline bool is_black(V3<R> c) { return c.x == R(0) && c.y == R(0) && c.z == R(0); }
template <typename R, typename S> inline V3<R> cvt(V3<S> a) { return V3<R>(R(a.x), R(a.y), R(a.z)); }

// mat4 (column-major, glm) times vec4, evaluated as
// col0*x + col1*y + col2*z + col3*w left to right per component.
template <typename R> inline void mat4_mul(const R m[16], R x, R y, R z, R w, R out[4]) {
    for (int r = 0; r < 4; ++r) out[r] = m[0 + r] * x + m[4 + r] * y + m[8 + r] * z + m[12 + r] * w;
}
// mat3(m4) * v3 (upper-left 3x3 of a column-major mat4).
template <typename R> inline V3<R> mat3_mul(const R m[16], V3<R> v) {
    return V3<R>(m[0] * v.x + m[4] * v.y + m[8] * v.z,
                 m[1] * v.x + m[5] * v.y + m[9] * v.z,
                 m[2] * v.x + m[6] * v.y + m[10] * v.z);
}

// ---------------------------------------------------------------------------
// RNG — random.glsl:4-50 and sampling.glsl:6-26
// ---------------------------------------------------------------------------
inline uint32_t rotl32(uint32_t x, uint32_t k) { return (x << k) | (x >> (32 - k)); }

// Thomas Wang 32-bit hash (random.glsl:30-38).
inline uint32_t wang_hash(uint32_t seed) {
    seed = (seed ^ 61u) ^ (seed >> 16);
    seed *= 9u;
    seed = seed ^ (seed >> 4);
    seed *= 0x27d4eb2du;
    seed = seed ^ (seed >> 15);
    return seed;
}

// PCG hash (RXS-M-XS output of one LCG step, O'Neill 2014; the GPU-hash form
// of Jarzynski & Olano 2020).  Used by the benchmark-spec RNG policy.
inline uint32_t pcg_hash(uint32_t v) {
    uint32_t state = v * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}

struct RNG {
    uint32_t s0, s1;
    uint32_t kind;  // 0 = xoroshiro64*, 1 = PCG
};

// xoroshiro64* step (random.glsl:17-26) or PCG step.
inline uint32_t rng_next(RNG& r) {
    if (r.kind == 0) {
        uint32_t result = r.s0 * 0x9e3779bbu;
        r.s1 ^= r.s0;
        r.s0 = rotl32(r.s0, 26) ^ r.s1 ^ (r.s1 << 9);
        r.s1 = rotl32(r.s1, 13);
        return result;
    }
    r.s0 = r.s0 * 747796405u + 2891336453u;
    uint32_t word = ((r.s0 >> ((r.s0 >> 28u) + 4u)) ^ r.s0) * 277803737u;
    return (word >> 22u) ^ word;
}

// rng_init (random.glsl:40-50): s = (hash((x<<16)|y), hash(frame)), one
// discarded draw.  PCG policy: state = pcg_hash(pcg_hash(pixel id) + sample).
inline RNG rng_init(uint32_t kind, uint32_t x, uint32_t y, uint32_t width, uint32_t frame) {
    RNG r;
    r.kind = kind;
    if (kind == 0) {
        r.s0 = wang_hash((x << 16) | y);
        r.s1 = wang_hash(frame);
        rng_next(r);
    } else {
        uint32_t pixel = y * width + x;
        r.s0 = pcg_hash(pcg_hash(pixel) + frame);
        r.s1 = 0;
    }
    return r;
}

// next_float (sampling.glsl:6-10): 23 random mantissa bits, [1,2) - 1.
inline float next_float(RNG& r) {
    uint32_t u = 0x3f800000u | (rng_next(r) >> 9);
    float f;
    std::memcpy(&f, &u, 4);
    return f - 1.0f;
}
// next_uint (sampling.glsl:12-16): uint(floor(f * nmax)), evaluated in FP32.
// A product that rounds up to nmax (impossible for nmax < 2^23 with these
// mantissas, kept as a guard) is clamped to nmax - 1.
inline uint32_t next_uint(RNG& r, uint32_t nmax) {
    float f = next_float(r);
    uint32_t i = (uint32_t)std::floor(f * (float)nmax);
    return (nmax > 0 && i >= nmax) ? nmax - 1 : i;
}

// ---------------------------------------------------------------------------
// IEEE half conversion (round to nearest even), for the FP16 environment map.
// ---------------------------------------------------------------------------
inline uint16_t float_to_half(float f) {
    uint32_t x;
    std::memcpy(&x, &f, 4);
    uint32_t sign = (x >> 16) & 0x8000u;
    uint32_t ax = x & 0x7fffffffu;
    if (ax >= 0x7f800000u) return (uint16_t)(sign | (ax > 0x7f800000u ? 0x7e00u : 0x7c00u));
    if (ax >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u);  // rounds to >= 65520 -> inf
    if (ax < 0x38800000u) {                                    // subnormal half
        if (ax < 0x33000000u) return (uint16_t)sign;           // < 2^-25 -> 0
        uint32_t e = ax >> 23;
        uint32_t m = (ax & 0x7fffffu) | 0x800000u;
        uint32_t shift = 126u - e;  // m >> shift gives half mantissa (units of 2^-24)
        uint32_t hm = m >> shift;
        uint32_t rem = m & ((1u << shift) - 1u);
        uint32_t half_ulp = 1u << (shift - 1);
        if (rem > half_ulp || (rem == half_ulp && (hm & 1u))) hm++;
        return (uint16_t)(sign | hm);
    }
    uint32_t e = (ax >> 23) - 112u;
    uint32_t m = ax & 0x7fffffu;
    uint32_t h = (e << 10) | (m >> 13);
    uint32_t rem = m & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h++;
    return (uint16_t)(sign | h);
}
inline float half_to_float(uint16_t h) {
    uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    uint32_t e = (h >> 10) & 0x1fu;
    uint32_t m = h & 0x3ffu;
    uint32_t x;
    if (e == 0) {
        if (m == 0) x = sign;
        else {  // subnormal: value = m * 2^-24
            float f = (float)m * 5.9604644775390625e-08f;
            std::memcpy(&x, &f, 4);
            x |= sign;
        }
    } else if (e == 31) x = sign | 0x7f800000u | (m << 13);
    else x = sign | ((e + 112u) << 23) | (m << 13);
    float f;
    std::memcpy(&f, &x, 4);
    return f;
}

// ---------------------------------------------------------------------------
// Watertight ray/triangle test (Woop, Benthin, Wald, JCGT 2(1) 2013), FP32
// or FP64, without the double-precision fallback for zero edge functions.
// Returns true with t, u (weight of v1), v (weight of v2) when
// tmin <= t <= tmax.
// ---------------------------------------------------------------------------
template <typename R> struct RayPre {
    V3<R> o, d;
    int kx, ky, kz;
    R sx, sy, sz;
};
template <typename R> inline RayPre<R> ray_prepare(V3<R> o, V3<R> d) {
    RayPre<R> p;
    p.o = o;
    p.d = d;
    R ax = std::fabs(d.x), ay = std::fabs(d.y), az = std::fabs(d.z);
    int kz = 0;
    if (ay > ax) kz = 1;
    if (az > (kz == 0 ? ax : ay)) kz = 2;
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    if (d[kz] < R(0)) std::swap(kx, ky);
    p.kx = kx; p.ky = ky; p.kz = kz;
    // one division: the shear constants scale by the reciprocal (the device
    // takes it from its per-axis reciprocals; consistent for all triangles
    // of the ray, which is what keeps the test watertight)
    p.sz = R(1) / d[kz];
    p.sx = d[kx] * p.sz;
    p.sy = d[ky] * p.sz;
    return p;
}
template <typename R>
inline bool intersect_triangle(const RayPre<R>& r, V3<R> v0, V3<R> v1, V3<R> v2, R tmin, R tmax,
                               R& t_out, R& u_out, R& v_out) {
    V3<R> A = v0 - r.o, B = v1 - r.o, C = v2 - r.o;
    R Ax = A[r.kx] - r.sx * A[r.kz];
    R Ay = A[r.ky] - r.sy * A[r.kz];
    R Bx = B[r.kx] - r.sx * B[r.kz];
    R By = B[r.ky] - r.sy * B[r.kz];
    R Cx = C[r.kx] - r.sx * C[r.kz];
    R Cy = C[r.ky] - r.sy * C[r.kz];
    R U = Cx * By - Cy * Bx;
    R V = Ax * Cy - Ay * Cx;
    R W = Bx * Ay - By * Ax;
    if ((U < R(0) || V < R(0) || W < R(0)) && (U > R(0) || V > R(0) || W > R(0))) return false;
    R det = U + V + W;
    if (det == R(0)) return false;
    R Az = r.sz * A[r.kz];
    R Bz = r.sz * B[r.kz];
    R Cz = r.sz * C[r.kz];
    R T = U * Az + V * Bz + W * Cz;
    R rcp = R(1) / det;
    R t = T * rcp;
    if (!(t >= tmin && t <= tmax)) return false;
    t_out = t;
    u_out = V * rcp;
    v_out = W * rcp;
    return true;
}

// Robust slab test (Ize 2013 style): the far distance is widened by
// 1 + 2^-21 and the near distance compared against a widened limit, so a
// box is never rejected for a ray that hits a triangle inside it.  Zero
// direction components are replaced by +-1e-20 before inversion.
inline float safe_inv(float d) {
    float a = std::fabs(d) < 1e-20f ? std::copysign(1e-20f, d) : d;
    return 1.0f / a;
}
inline bool slab_test(const float inv[3], const float org[3], const float lo[3], const float hi[3],
                      float tmin, float tmax, float& tnear_out) {
    float tn = tmin, tf = tmax;
    for (int a = 0; a < 3; ++a) {
        float t0 = (lo[a] - org[a]) * inv[a];
        float t1 = (hi[a] - org[a]) * inv[a];
        float n = t0 < t1 ? t0 : t1;
        float f = t0 < t1 ? t1 : t0;
        tn = n > tn ? n : tn;
        tf = f < tf ? f : tf;
    }
    tnear_out = tn;
    return tn <= tf * 1.000000477f;
}

}  // namespace oracle
