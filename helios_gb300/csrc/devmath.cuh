// devmath.cuh — device vector math with GLSL semantics, the RNGs of
// random.glsl/sampling.glsl and the PCG policy.  Every helper evaluates in
// the same order as the GLSL source (left to right, no FMA: the library is
// compiled with --fmad=false), so integer-valued results are bit-exact with
// the host oracle.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#define HXD __device__ __forceinline__

struct V3 {
    float x, y, z;
};
HXD V3 v3(float a, float b, float c) { return V3{a, b, c}; }
HXD V3 v3(float a) { return V3{a, a, a}; }
HXD V3 v3(float4 a) { return V3{a.x, a.y, a.z}; }
HXD V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
HXD V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
HXD V3 operator-(V3 a) { return v3(-a.x, -a.y, -a.z); }
HXD V3 operator*(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
HXD V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
// vector / scalar as one division and three products (the oracle's operator/ is the same)
HXD V3 operator/(V3 a, float s) {
    const float r = 1.0f / s;
    return v3(a.x * r, a.y * r, a.z * r);
}
HXD float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
HXD V3 cross(V3 a, V3 b) { return v3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y); }
HXD float length(V3 a) { return sqrtf(dot(a, a)); }
HXD V3 normalize(V3 a) {
    // one division (the reciprocal length) and three products; the oracle's
    // normalize is the same sequence
    const float r = 1.0f / sqrtf(dot(a, a));
    return v3(a.x * r, a.y * r, a.z * r);
}
// GLSL min/max/clamp (4.60 spec 8.3): min(x, y) = y < x ? y : x.
HXD float gmin(float a, float b) { return b < a ? b : a; }
HXD float gmax(float a, float b) { return a < b ? b : a; }
HXD float gclamp(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }
HXD V3 reflect(V3 i, V3 n) {
    float d = dot(n, i);
    return i - n * (2.0f * d);
}
HXD bool is_black(V3 c) { return c.x == 0.0f && c.y == 0.0f && c.z == 0.0f; }
HXD float comp(V3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

// first index k in [lo, hi) with a[k] > x (a sorted ascending), hi if none
HXD int upper_bound_f(const float* a, int lo, int hi, float x) {
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (__ldg(a + mid) > x) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}

// column-major mat4 * (x, y, z, w), left to right per component
HXD V3 mat4_mul3(const float* m, float x, float y, float z, float w) {
    return v3(m[0] * x + m[4] * y + m[8] * z + m[12] * w, m[1] * x + m[5] * y + m[9] * z + m[13] * w,
              m[2] * x + m[6] * y + m[10] * z + m[14] * w);
}
HXD float mat4_row(const float* m, int r, float x, float y, float z, float w) {
    return m[0 + r] * x + m[4 + r] * y + m[8 + r] * z + m[12 + r] * w;
}
HXD V3 mat3_mul(const float* m, V3 v) {
    return v3(m[0] * v.x + m[4] * v.y + m[8] * v.z, m[1] * v.x + m[5] * v.y + m[9] * v.z,
              m[2] * v.x + m[6] * v.y + m[10] * v.z);
}

// ---------------------------------------------------------------------------
// RNG: xoroshiro64* seeded by the Wang hash (random.glsl:11-50) or PCG.
// ---------------------------------------------------------------------------
HXD uint32_t rotl32(uint32_t x, uint32_t k) { return (x << k) | (x >> (32 - k)); }
HXD uint32_t wang_hash(uint32_t seed) {
    seed = (seed ^ 61u) ^ (seed >> 16);
    seed *= 9u;
    seed = seed ^ (seed >> 4);
    seed *= 0x27d4eb2du;
    seed = seed ^ (seed >> 15);
    return seed;
}
HXD uint32_t pcg_hash(uint32_t v) {
    uint32_t state = v * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}

struct Rng {
    uint32_t s0, s1;
};

template <uint32_t KIND> HXD uint32_t rng_next(Rng& r) {
    if (KIND == 0) {
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
HXD uint32_t rng_next_k(uint32_t kind, Rng& r) { return kind == 0 ? rng_next<0>(r) : rng_next<1>(r); }

HXD Rng rng_init(uint32_t kind, uint32_t x, uint32_t y, uint32_t width, uint32_t frame) {
    Rng r;
    if (kind == 0) {
        r.s0 = wang_hash((x << 16) | y);
        r.s1 = wang_hash(frame);
        rng_next<0>(r);
    } else {
        r.s0 = pcg_hash(pcg_hash(y * width + x) + frame);
        r.s1 = 0;
    }
    return r;
}
HXD float next_float(uint32_t kind, Rng& r) {
    uint32_t u = 0x3f800000u | (rng_next_k(kind, r) >> 9);
    return __uint_as_float(u) - 1.0f;
}
HXD uint32_t next_uint(uint32_t kind, Rng& r, uint32_t nmax) {
    float f = next_float(kind, r);
    uint32_t i = (uint32_t)floorf(f * (float)nmax);
    return (nmax > 0 && i >= nmax) ? nmax - 1 : i;
}

constexpr float kPiF = 3.14159265359f;  // M_PI of common.glsl:18 as a float literal
constexpr float kEpsilonF = 0.0001f;    // EPSILON, common.glsl:19
constexpr float kMinRoughnessF = 0.1f;  // MIN_ROUGHNESS, common.glsl:21
constexpr uint32_t kNoHit = 0xffffffffu;

// ---------------------------------------------------------------------------
// Packed FP32x2 arithmetic (sm_100+ f32x2 instructions): each lane rounds
// exactly like the scalar instruction, so results equal the scalar forms.
// ---------------------------------------------------------------------------
HXD unsigned long long f2_bits(float2 a) { return ((unsigned long long)__float_as_uint(a.y) << 32) | __float_as_uint(a.x); }
HXD float2 bits_f2(unsigned long long r) { return make_float2(__uint_as_float((uint32_t)r), __uint_as_float((uint32_t)(r >> 32))); }
HXD float2 fma2_rn(float2 a, float2 b, float2 c) {
    unsigned long long r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(f2_bits(a)), "l"(f2_bits(b)), "l"(f2_bits(c)));
    return bits_f2(r);
}
HXD float2 sub2_rn(float2 a, float2 b) {
    unsigned long long r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_bits(a)), "l"(f2_bits(b)));
    return bits_f2(r);
}
HXD float2 mul2_rn(float2 a, float2 b) {
    unsigned long long r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_bits(a)), "l"(f2_bits(b)));
    return bits_f2(r);
}
HXD float max3f(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
HXD float min3f(float a, float b, float c) {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
