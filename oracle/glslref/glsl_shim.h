// glsl_shim.h — GLSL types and built-ins in C++ (TEST INFRASTRUCTURE).
//
// Lets the reference's own shader functions (random.glsl, sampling.glsl,
// brdf.glsl, common.glsl, the path_trace_* stages and tone_map.frag, copied
// out of the reference tree at build time by oracle/glslref/build.py and
// never committed) compile as C++, so the oracle's restatement can be checked
// against the reference's code itself.
//
// Semantics follow the GLSL 4.60 specification:
//   * vector constructors take their arguments in order (the build script
//     turns every constructor call into brace initialisation, which C++
//     evaluates left to right, as GLSL does — sampling.glsl:18-26 draws two
//     or three random numbers inside one constructor);
//   * normalize(x) = x / length(x), length(x) = sqrt(dot(x, x)),
//     reflect(I, N) = I - 2 dot(N, I) N, mix(x, y, a) = x (1 - a) + y a,
//     smoothstep(e0, e1, x) = t t (3 - 2 t) with t = clamp((x - e0) / (e1 - e0), 0, 1),
//     min(x, y) = y < x ? y : x, max(x, y) = x < y ? y : x (8.3, 8.5);
//   * matrices are column-major; M * v sums the columns left to right;
//   * float operations are IEEE binary32 without contraction (the recipe
//     compiles with -ffp-contract=off).
// GLSL leaves the precision of these built-ins to the implementation; this
// shim evaluates them as written, so the reference's code and the oracle's
// restatement may differ by a few ulps where the oracle chose another
// evaluation order (reciprocal products for normalize and vector / scalar).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

namespace glsl {

typedef uint32_t uint;

inline float abs(float x) { return std::fabs(x); }
inline float sqrt(float x) { return std::sqrt(x); }
inline float cos(float x) { return std::cos(x); }
inline float sin(float x) { return std::sin(x); }
inline float floor(float x) { return std::floor(x); }
inline float pow(float x, float y) { return std::pow(x, y); }
inline float min(float x, float y) { return y < x ? y : x; }
inline float max(float x, float y) { return x < y ? y : x; }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline float mix(float x, float y, float a) { return x * (1.0f - a) + y * a; }
inline float smoothstep(float e0, float e1, float x) {
    float t = clamp((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}
inline bool isnan(float x) { return std::isnan(x); }
inline float uintBitsToFloat(uint u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

struct vec2;
struct vec3;
struct vec4;

struct uvec2 {
    uint x, y;
    uvec2() : x(0), y(0) {}
    template <class A, class B> uvec2(A a, B b) : x(uint(a)), y(uint(b)) {}
};
struct ivec2 {
    int x, y;
    ivec2() : x(0), y(0) {}
    template <class A, class B> ivec2(A a, B b) : x(int(a)), y(int(b)) {}
    explicit ivec2(uvec2 v) : x(int(v.x)), y(int(v.y)) {}
};
struct vec2 {
    float x, y;
    vec2() : x(0), y(0) {}
    vec2(float s) : x(s), y(s) {}
    template <class A, class B> vec2(A a, B b) : x(float(a)), y(float(b)) {}
    explicit vec2(uvec2 v) : x(float(v.x)), y(float(v.y)) {}
    explicit vec2(ivec2 v) : x(float(v.x)), y(float(v.y)) {}
    float& operator[](int i) { return i == 0 ? x : y; }
    float operator[](int i) const { return i == 0 ? x : y; }
};

struct vec3 {
    float x, y, z;
    vec3() : x(0), y(0), z(0) {}
    vec3(float s) : x(s), y(s), z(s) {}
    template <class A, class B, class C> vec3(A a, B b, C c) : x(float(a)), y(float(b)), z(float(c)) {}
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    vec2 yz() const { return vec2(y, z); }
    vec2 xy() const { return vec2(x, y); }
    vec3 rgb() const { return *this; }
    inline vec3& operator*=(float s);
    inline vec3& operator/=(float s);
    inline vec3& operator+=(const vec3& o);
};
struct uvec3 {
    uint x, y, z;
    uvec3() : x(0), y(0), z(0) {}
    template <class A, class B, class C> uvec3(A a, B b, C c) : x(uint(a)), y(uint(b)), z(uint(c)) {}
};

// Swizzle results: a value that also writes back on assignment
// (o.tex_coord.xy = ..., v.normal.xyz = ...).
struct Swz3 : vec3 {
    float *px, *py, *pz;
    Swz3(float* a, float* b, float* c) : vec3(*a, *b, *c), px(a), py(b), pz(c) {}
    Swz3& operator=(const vec3& v) {
        *px = v.x; *py = v.y; *pz = v.z;
        x = v.x; y = v.y; z = v.z;
        return *this;
    }
};
struct Swz2 : vec2 {
    float *px, *py;
    Swz2(float* a, float* b) : vec2(*a, *b), px(a), py(b) {}
    Swz2& operator=(const vec2& v) {
        *px = v.x; *py = v.y;
        x = v.x; y = v.y;
        return *this;
    }
};

struct vec4 {
    float x, y, z, w;
    vec4() : x(0), y(0), z(0), w(0) {}
    vec4(float s) : x(s), y(s), z(s), w(s) {}
    template <class A, class B, class C, class D>
    vec4(A a, B b, C c, D d) : x(float(a)), y(float(b)), z(float(c)), w(float(d)) {}
    template <class D> vec4(const vec3& v, D d) : x(v.x), y(v.y), z(v.z), w(float(d)) {}
    template <class C, class D> vec4(const vec2& v, C c, D d) : x(v.x), y(v.y), z(float(c)), w(float(d)) {}
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    Swz3 xyz() { return Swz3(&x, &y, &z); }
    vec3 xyz() const { return vec3(x, y, z); }
    Swz3 rgb() { return Swz3(&x, &y, &z); }
    vec3 rgb() const { return vec3(x, y, z); }
    Swz3 yzw() { return Swz3(&y, &z, &w); }
    vec3 yzw() const { return vec3(y, z, w); }
    Swz2 xy() { return Swz2(&x, &y); }
    vec2 xy() const { return vec2(x, y); }
    vec2 zw() const { return vec2(z, w); }
    inline vec4& operator/=(float s);
};
struct ivec4 {
    int x, y, z, w;
    ivec4() : x(0), y(0), z(0), w(0) {}
    template <class A, class B, class C, class D>
    ivec4(A a, B b, C c, D d) : x(int(a)), y(int(b)), z(int(c)), w(int(d)) {}
    vec2 xy() const { return vec2(float(x), float(y)); }
    vec2 zw() const { return vec2(float(z), float(w)); }
};
struct uvec4 {
    uint x, y, z, w;
    uvec4() : x(0), y(0), z(0), w(0) {}
    uvec2 zw() const { return uvec2(z, w); }
};

// ---- vec2 arithmetic
inline vec2 operator+(vec2 a, vec2 b) { return vec2(a.x + b.x, a.y + b.y); }
inline vec2 operator-(vec2 a, vec2 b) { return vec2(a.x - b.x, a.y - b.y); }
inline vec2 operator*(vec2 a, vec2 b) { return vec2(a.x * b.x, a.y * b.y); }
inline vec2 operator/(vec2 a, vec2 b) { return vec2(a.x / b.x, a.y / b.y); }
inline vec2 operator*(vec2 a, float s) { return vec2(a.x * s, a.y * s); }
inline vec2 operator-(vec2 a, float s) { return vec2(a.x - s, a.y - s); }
inline vec2 max(vec2 a, vec2 b) { return vec2(max(a.x, b.x), max(a.y, b.y)); }

// ---- vec3 arithmetic
inline vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator-(const vec3& a) { return vec3(-a.x, -a.y, -a.z); }
inline vec3 operator*(const vec3& a, const vec3& b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator/(const vec3& a, const vec3& b) { return vec3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline vec3 operator*(const vec3& a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator*(float s, const vec3& a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator/(const vec3& a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
inline vec3 operator+(const vec3& a, float s) { return vec3(a.x + s, a.y + s, a.z + s); }
inline vec3 operator-(const vec3& a, float s) { return vec3(a.x - s, a.y - s, a.z - s); }
inline vec3 operator/(float s, const vec3& a) { return vec3(s / a.x, s / a.y, s / a.z); }
inline vec3 operator+(float s, const vec3& a) { return vec3(s + a.x, s + a.y, s + a.z); }
inline vec3& vec3::operator*=(float s) { x *= s; y *= s; z *= s; return *this; }
inline vec3& vec3::operator/=(float s) { x /= s; y /= s; z /= s; return *this; }
inline vec3& vec3::operator+=(const vec3& o) { x += o.x; y += o.y; z += o.z; return *this; }
inline float dot(const vec3& a, const vec3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline vec3 cross(const vec3& a, const vec3& b) {
    return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
inline float length(const vec3& a) { return std::sqrt(dot(a, a)); }
inline vec3 normalize(const vec3& a) { return a / length(a); }
inline vec3 reflect(const vec3& i, const vec3& n) { return i - 2.0f * dot(n, i) * n; }
inline vec3 min(const vec3& a, const vec3& b) { return vec3(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
inline vec3 max(const vec3& a, const vec3& b) { return vec3(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
inline vec3 clamp(const vec3& x, float lo, float hi) { return vec3(clamp(x.x, lo, hi), clamp(x.y, lo, hi), clamp(x.z, lo, hi)); }
inline vec3 mix(const vec3& x, const vec3& y, float a) { return x * (1.0f - a) + y * a; }
inline vec3 pow(const vec3& x, const vec3& y) { return vec3(pow(x.x, y.x), pow(x.y, y.y), pow(x.z, y.z)); }

// ---- vec4 arithmetic
inline vec4& vec4::operator/=(float s) { x /= s; y /= s; z /= s; w /= s; return *this; }

// ---- matrices (column-major)
struct mat4 {
    vec4 c[4];
    vec4& operator[](int i) { return c[i]; }
    const vec4& operator[](int i) const { return c[i]; }
};
struct mat3 {
    vec3 c[3];
    mat3() {}
    mat3(const vec3& a, const vec3& b, const vec3& d) { c[0] = a; c[1] = b; c[2] = d; }
    explicit mat3(const mat4& m) {
        for (int i = 0; i < 3; ++i) c[i] = vec3(m.c[i].x, m.c[i].y, m.c[i].z);
    }
};
inline vec4 operator*(const mat4& m, const vec4& v) {
    vec4 r;
    for (int i = 0; i < 4; ++i) r[i] = m.c[0][i] * v.x + m.c[1][i] * v.y + m.c[2][i] * v.z + m.c[3][i] * v.w;
    return r;
}
inline vec3 operator*(const mat3& m, const vec3& v) {
    vec3 r;
    for (int i = 0; i < 3; ++i) r[i] = m.c[0][i] * v.x + m.c[1][i] * v.y + m.c[2][i] * v.z;
    return r;
}

}  // namespace glsl
