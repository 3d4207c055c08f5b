// ORACLE — test infrastructure only.  A small GLSL-compatibility layer that lets the reference's shader
// source (reina-vk shaders/raytrace/*.glsl, shaders/postprocessing/**/*.glsl), after the mechanical
// rewrites of oracle/glsl/build_ref.py, compile as C++20 and run on the host: the GLSL vector and matrix
// types, their operators, and the built-in functions the shaders call, each written from the GLSL 4.60
// specification's definition (section 8, "Built-in Functions").
//
// Every function here evaluates the specification's expression in the written order in IEEE binary32
// (the translation units are compiled with -ffp-contract=off), and the transcendental functions are the
// host C library's (sinf, cosf, expf, logf, powf, acosf through the compiler's builtins, so that no C++
// math header is included and no global overload can shadow the GLSL names).  Nothing of this file is
// linked into the product; it is the checker's.
#pragma once

#include <stdint.h>
#include <string.h>

#include <type_traits>

namespace glsl {

using uint = uint32_t;

inline float f_sqrt(float x) { return __builtin_sqrtf(x); }

// ---------------------------------------------------------------------------------------------------
// vectors (components also named r, g, b, a as GLSL allows)

struct vec2;
struct vec3;
struct vec4;
struct ivec2;
struct ivec3;
struct uvec3;

template <class T>
constexpr bool is_scalar_v = std::is_arithmetic_v<T>;

struct vec2 {
    union { float x; float r; };
    union { float y; float g; };
    vec2() : x(0.0f), y(0.0f) {}
    template <class S> explicit vec2(S s) requires is_scalar_v<S> : x(float(s)), y(float(s)) {}
    template <class A, class B> vec2(A a, B b) requires (is_scalar_v<A> && is_scalar_v<B>) : x(float(a)), y(float(b)) {}
    explicit vec2(const ivec2& v);
    vec2 xy() const { return *this; }
    vec2& operator+=(const vec2& o) { x = x + o.x; y = y + o.y; return *this; }
    vec2& operator-=(const vec2& o) { x = x - o.x; y = y - o.y; return *this; }
    vec2& operator*=(float s) { x = x * s; y = y * s; return *this; }
    vec2& operator/=(float s) { x = x / s; y = y / s; return *this; }
};

struct vec3 {
    union { float x; float r; };
    union { float y; float g; };
    union { float z; float b; };
    vec3() : x(0.0f), y(0.0f), z(0.0f) {}
    template <class S> explicit vec3(S s) requires is_scalar_v<S> : x(float(s)), y(float(s)), z(float(s)) {}
    template <class A, class B, class C>
    vec3(A a, B b, C c) requires (is_scalar_v<A> && is_scalar_v<B> && is_scalar_v<C>) : x(float(a)), y(float(b)), z(float(c)) {}
    template <class C> vec3(const vec2& v, C c) requires is_scalar_v<C> : x(v.x), y(v.y), z(float(c)) {}
    explicit vec3(const vec4& v);
    explicit vec3(const ivec3& v);
    vec2 xy() const { return vec2(x, y); }
    vec3 xyz() const { return *this; }
    vec3 rgb() const { return *this; }
    vec3& operator+=(const vec3& o) { x = x + o.x; y = y + o.y; z = z + o.z; return *this; }
    vec3& operator-=(const vec3& o) { x = x - o.x; y = y - o.y; z = z - o.z; return *this; }
    vec3& operator*=(const vec3& o) { x = x * o.x; y = y * o.y; z = z * o.z; return *this; }
    template <class S> vec3& operator*=(S s) requires is_scalar_v<S> { const float f = float(s); x = x * f; y = y * f; z = z * f; return *this; }
    vec3& operator/=(const vec3& o) { x = x / o.x; y = y / o.y; z = z / o.z; return *this; }
    template <class S> vec3& operator/=(S s) requires is_scalar_v<S> { const float f = float(s); x = x / f; y = y / f; z = z / f; return *this; }
};

struct vec4 {
    union { float x; float r; };
    union { float y; float g; };
    union { float z; float b; };
    union { float w; float a; };
    vec4() : x(0.0f), y(0.0f), z(0.0f), w(0.0f) {}
    template <class S> explicit vec4(S s) requires is_scalar_v<S> : x(float(s)), y(float(s)), z(float(s)), w(float(s)) {}
    template <class A, class B, class C, class D>
    vec4(A a, B b, C c, D d) requires (is_scalar_v<A> && is_scalar_v<B> && is_scalar_v<C> && is_scalar_v<D>)
        : x(float(a)), y(float(b)), z(float(c)), w(float(d)) {}
    template <class D> vec4(const vec3& v, D d) requires is_scalar_v<D> : x(v.x), y(v.y), z(v.z), w(float(d)) {}
    template <class C, class D> vec4(const vec2& v, C c, D d) requires (is_scalar_v<C> && is_scalar_v<D>)
        : x(v.x), y(v.y), z(float(c)), w(float(d)) {}
    vec2 xy() const { return vec2(x, y); }
    vec3 xyz() const { return vec3(x, y, z); }
    vec3 rgb() const { return vec3(x, y, z); }
    template <class S> vec4& operator/=(S s) requires is_scalar_v<S> { const float f = float(s); x = x / f; y = y / f; z = z / f; w = w / f; return *this; }
};

inline vec3::vec3(const vec4& v) : x(v.x), y(v.y), z(v.z) {}

struct uvec2 {
    uint x, y;
};

struct ivec2 {
    int x, y;
    ivec2() : x(0), y(0) {}
    template <class A, class B> ivec2(A a, B b) requires (is_scalar_v<A> && is_scalar_v<B>) : x(int(a)), y(int(b)) {}
    explicit ivec2(const vec2& v) : x(int(v.x)), y(int(v.y)) {}
    explicit ivec2(const uvec2& v) : x(int(v.x)), y(int(v.y)) {}
};
inline vec2::vec2(const ivec2& v) : x(float(v.x)), y(float(v.y)) {}
struct uvec3 {
    uint x, y, z;
    uvec2 xy() const { return uvec2{x, y}; }
};

struct ivec3 {
    int x, y, z;
    ivec3() : x(0), y(0), z(0) {}
    explicit ivec3(const vec3& v) : x(int(v.x)), y(int(v.y)), z(int(v.z)) {}   // float -> int truncates
};
inline vec3::vec3(const ivec3& v) : x(float(v.x)), y(float(v.y)), z(float(v.z)) {}

inline ivec2 to_ivec2(const uvec2& v) { return ivec2(int(v.x), int(v.y)); }

// ivec2 arithmetic (pixel coordinates)
inline ivec2 operator+(const ivec2& a, const ivec2& b) { return ivec2(a.x + b.x, a.y + b.y); }
inline ivec2 operator*(int s, const ivec2& a) { return ivec2(s * a.x, s * a.y); }

// vector arithmetic, component-wise in component order
#define GLSL_VEC_OPS(V, N)                                                                              \
    inline V operator+(const V& a, const V& b) { V r; for (int i = 0; i < N; ++i) (&r.x)[i] = (&a.x)[i] + (&b.x)[i]; return r; } \
    inline V operator-(const V& a, const V& b) { V r; for (int i = 0; i < N; ++i) (&r.x)[i] = (&a.x)[i] - (&b.x)[i]; return r; } \
    inline V operator*(const V& a, const V& b) { V r; for (int i = 0; i < N; ++i) (&r.x)[i] = (&a.x)[i] * (&b.x)[i]; return r; } \
    inline V operator/(const V& a, const V& b) { V r; for (int i = 0; i < N; ++i) (&r.x)[i] = (&a.x)[i] / (&b.x)[i]; return r; } \
    inline V operator-(const V& a) { V r; for (int i = 0; i < N; ++i) (&r.x)[i] = -(&a.x)[i]; return r; } \
    template <class S> inline V operator+(const V& a, S s) requires is_scalar_v<S> { V r; const float f = float(s); for (int i = 0; i < N; ++i) (&r.x)[i] = (&a.x)[i] + f; return r; } \
    template <class S> inline V operator-(const V& a, S s) requires is_scalar_v<S> { V r; const float f = float(s); for (int i = 0; i < N; ++i) (&r.x)[i] = (&a.x)[i] - f; return r; } \
    template <class S> inline V operator*(const V& a, S s) requires is_scalar_v<S> { V r; const float f = float(s); for (int i = 0; i < N; ++i) (&r.x)[i] = (&a.x)[i] * f; return r; } \
    template <class S> inline V operator/(const V& a, S s) requires is_scalar_v<S> { V r; const float f = float(s); for (int i = 0; i < N; ++i) (&r.x)[i] = (&a.x)[i] / f; return r; } \
    template <class S> inline V operator+(S s, const V& a) requires is_scalar_v<S> { V r; const float f = float(s); for (int i = 0; i < N; ++i) (&r.x)[i] = f + (&a.x)[i]; return r; } \
    template <class S> inline V operator-(S s, const V& a) requires is_scalar_v<S> { V r; const float f = float(s); for (int i = 0; i < N; ++i) (&r.x)[i] = f - (&a.x)[i]; return r; } \
    template <class S> inline V operator*(S s, const V& a) requires is_scalar_v<S> { V r; const float f = float(s); for (int i = 0; i < N; ++i) (&r.x)[i] = f * (&a.x)[i]; return r; } \
    template <class S> inline V operator/(S s, const V& a) requires is_scalar_v<S> { V r; const float f = float(s); for (int i = 0; i < N; ++i) (&r.x)[i] = f / (&a.x)[i]; return r; }
GLSL_VEC_OPS(vec2, 2)
GLSL_VEC_OPS(vec3, 3)
GLSL_VEC_OPS(vec4, 4)
#undef GLSL_VEC_OPS

static_assert(sizeof(vec2) == 8 && sizeof(vec3) == 12 && sizeof(vec4) == 16, "vector layout");

// ---------------------------------------------------------------------------------------------------
// matrices: column-major, m[c] is column c

struct mat4x3;
struct mat4;

struct mat3 {
    vec3 c[3];
    mat3() {}
    template <class S> explicit mat3(S s) requires is_scalar_v<S> {   // diagonal
        c[0] = vec3(float(s), 0.0f, 0.0f); c[1] = vec3(0.0f, float(s), 0.0f); c[2] = vec3(0.0f, 0.0f, float(s));
    }
    mat3(const vec3& a, const vec3& b, const vec3& d) { c[0] = a; c[1] = b; c[2] = d; }
    explicit mat3(const mat4x3& m);
    explicit mat3(const mat4& m);
    vec3& operator[](int i) { return c[i]; }
    const vec3& operator[](int i) const { return c[i]; }
};

struct mat4x3 {   // 4 columns of 3 rows (gl_ObjectToWorldEXT)
    vec3 c[4];
    vec3& operator[](int i) { return c[i]; }
    const vec3& operator[](int i) const { return c[i]; }
};

struct mat4 {
    vec4 c[4];
    vec4& operator[](int i) { return c[i]; }
    const vec4& operator[](int i) const { return c[i]; }
};
using mat4x4 = mat4;

inline mat3::mat3(const mat4x3& m) { c[0] = m.c[0]; c[1] = m.c[1]; c[2] = m.c[2]; }
inline mat3::mat3(const mat4& m) { c[0] = vec3(m.c[0]); c[1] = vec3(m.c[1]); c[2] = vec3(m.c[2]); }

static_assert(sizeof(mat3) == 36 && sizeof(mat4) == 64 && sizeof(mat4x3) == 48, "matrix layout");

// matrix * column vector: r_i = sum_c m[c][i] v_c, summed in column order
inline vec3 operator*(const mat3& m, const vec3& v) {
    return vec3(m.c[0].x * v.x + m.c[1].x * v.y + m.c[2].x * v.z, m.c[0].y * v.x + m.c[1].y * v.y + m.c[2].y * v.z,
                m.c[0].z * v.x + m.c[1].z * v.y + m.c[2].z * v.z);
}
inline vec3 operator*(const mat4x3& m, const vec4& v) {
    return vec3(m.c[0].x * v.x + m.c[1].x * v.y + m.c[2].x * v.z + m.c[3].x * v.w,
                m.c[0].y * v.x + m.c[1].y * v.y + m.c[2].y * v.z + m.c[3].y * v.w,
                m.c[0].z * v.x + m.c[1].z * v.y + m.c[2].z * v.z + m.c[3].z * v.w);
}
inline vec4 operator*(const mat4& m, const vec4& v) {
    vec4 r;
    for (int i = 0; i < 4; ++i)
        (&r.x)[i] = (&m.c[0].x)[i] * v.x + (&m.c[1].x)[i] * v.y + (&m.c[2].x)[i] * v.z + (&m.c[3].x)[i] * v.w;
    return r;
}
// row vector * matrix: r_c = dot(v, m[c])
inline float dot(const vec3& a, const vec3& b);
inline vec3 operator*(const vec3& v, const mat3& m) { return vec3(dot(v, m.c[0]), dot(v, m.c[1]), dot(v, m.c[2])); }

inline mat3 transpose(const mat3& m) {
    return mat3(vec3(m.c[0].x, m.c[1].x, m.c[2].x), vec3(m.c[0].y, m.c[1].y, m.c[2].y), vec3(m.c[0].z, m.c[1].z, m.c[2].z));
}
// inverse by the adjugate over the determinant (cofactor expansion along the first column)
inline mat3 inverse(const mat3& m) {
    const float a00 = m.c[0].x, a01 = m.c[0].y, a02 = m.c[0].z;   // a_cr: column c, row r
    const float a10 = m.c[1].x, a11 = m.c[1].y, a12 = m.c[1].z;
    const float a20 = m.c[2].x, a21 = m.c[2].y, a22 = m.c[2].z;
    const float b01 = a22 * a11 - a12 * a21;
    const float b11 = -a22 * a10 + a12 * a20;
    const float b21 = a21 * a10 - a11 * a20;
    const float det = a00 * b01 + a01 * b11 + a02 * b21;
    mat3 r;
    r.c[0] = vec3(b01 / det, (-a22 * a01 + a02 * a21) / det, (a12 * a01 - a02 * a11) / det);
    r.c[1] = vec3(b11 / det, (a22 * a00 - a02 * a20) / det, (-a12 * a00 + a02 * a10) / det);
    r.c[2] = vec3(b21 / det, (-a21 * a00 + a01 * a20) / det, (a11 * a00 - a01 * a10) / det);
    return r;
}

// ---------------------------------------------------------------------------------------------------
// built-in functions (GLSL 4.60 section 8)

// min(x, y) = y < x ? y : x; max(x, y) = x < y ? y : x (8.3)
inline float min(float x, float y) { return y < x ? y : x; }
inline float max(float x, float y) { return x < y ? y : x; }
inline int min(int x, int y) { return y < x ? y : x; }
inline int max(int x, int y) { return x < y ? y : x; }
template <class A, class B> inline float min(A x, B y) requires (is_scalar_v<A> && is_scalar_v<B>) { return min(float(x), float(y)); }
template <class A, class B> inline float max(A x, B y) requires (is_scalar_v<A> && is_scalar_v<B>) { return max(float(x), float(y)); }
inline vec3 max(const vec3& a, const vec3& b) { return vec3(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
inline vec3 min(const vec3& a, const vec3& b) { return vec3(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
// clamp(x, lo, hi) = min(max(x, lo), hi)
template <class A, class B, class C> inline float clamp(A x, B lo, C hi) requires (is_scalar_v<A> && is_scalar_v<B> && is_scalar_v<C>) {
    return min(max(float(x), float(lo)), float(hi));
}
inline vec3 clamp(const vec3& x, const vec3& lo, const vec3& hi) { return min(max(x, lo), hi); }
template <class B, class C> inline vec3 clamp(const vec3& x, B lo, C hi) requires (is_scalar_v<B> && is_scalar_v<C>) {
    return clamp(x, vec3(float(lo)), vec3(float(hi)));
}

inline float abs(float x) { return x >= 0.0f ? x : -x; }   // "x if x >= 0, otherwise -x"
inline int abs(int x) { return x < 0 ? -x : x; }
inline float sign(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
inline float floor(float x) { return __builtin_floorf(x); }
inline float fract(float x) { return x - floor(x); }
// mod(x, y) = x - y * floor(x / y)
inline float mod(float x, float y) { return x - y * floor(x / y); }
inline vec2 mod(const vec2& v, float y) { return vec2(mod(v.x, y), mod(v.y, y)); }

inline float sqrt(float x) { return __builtin_sqrtf(x); }
inline float inversesqrt(float x) { return 1.0f / __builtin_sqrtf(x); }
inline float exp(float x) { return __builtin_expf(x); }
inline float exp2(float x) { return __builtin_exp2f(x); }
inline float log(float x) { return __builtin_logf(x); }
inline float sin(float x) { return __builtin_sinf(x); }
inline float cos(float x) { return __builtin_cosf(x); }
inline float acos(float x) { return __builtin_acosf(x); }
template <class A, class B> inline float pow(A x, B y) requires (is_scalar_v<A> && is_scalar_v<B>) { return __builtin_powf(float(x), float(y)); }
inline vec3 pow(const vec3& x, const vec3& y) { return vec3(pow(x.x, y.x), pow(x.y, y.y), pow(x.z, y.z)); }
inline vec3 exp(const vec3& x) { return vec3(exp(x.x), exp(x.y), exp(x.z)); }

// mix(x, y, a) = x * (1 - a) + y * a; with a bool selector: a ? y : x
template <class A, class B, class C> inline float mix(A x, B y, C a) requires (is_scalar_v<A> && is_scalar_v<B> && is_scalar_v<C> && !std::is_same_v<C, bool>) {
    return float(x) * (1.0f - float(a)) + float(y) * float(a);
}
template <class A, class B> inline float mix(A x, B y, bool a) requires (is_scalar_v<A> && is_scalar_v<B>) { return a ? float(y) : float(x); }
inline vec3 mix(const vec3& x, const vec3& y, float a) { return x * (1.0f - a) + y * a; }
inline vec3 mix(const vec3& x, const vec3& y, const vec3& a) { return x * (1.0f - a) + y * a; }
inline vec2 mix(const vec2& x, const vec2& y, float a) { return x * (1.0f - a) + y * a; }

inline float dot(const vec2& a, const vec2& b) { return a.x * b.x + a.y * b.y; }
inline float dot(const vec3& a, const vec3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float length(const vec2& v) { return sqrt(dot(v, v)); }
inline float length(const vec3& v) { return sqrt(dot(v, v)); }
inline vec3 cross(const vec3& a, const vec3& b) {
    return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
// normalize(x) = x / length(x)
inline vec3 normalize(const vec3& v) { return v / length(v); }
// reflect(I, N) = I - 2 dot(N, I) N
inline vec3 reflect(const vec3& i, const vec3& n) { return i - 2.0f * dot(n, i) * n; }
// refract(I, N, eta): k = 1 - eta^2 (1 - dot(N, I)^2); k < 0 -> 0, else eta I - (eta dot(N, I) + sqrt(k)) N
inline vec3 refract(const vec3& i, const vec3& n, float eta) {
    const float d = dot(n, i);
    const float k = 1.0f - eta * eta * (1.0f - d * d);
    if (k < 0.0f) return vec3(0.0f);
    return eta * i - (eta * d + sqrt(k)) * n;
}
// faceforward(N, I, Nref) = dot(Nref, I) < 0 ? N : -N
inline vec3 faceforward(const vec3& n, const vec3& i, const vec3& nref) { return dot(nref, i) < 0.0f ? n : -n; }

struct bvec3 { bool x, y, z; };
inline bool isnan(float x) { return x != x; }
inline bvec3 isnan(const vec3& v) { return bvec3{isnan(v.x), isnan(v.y), isnan(v.z)}; }
inline bool any(const bvec3& b) { return b.x || b.y || b.z; }

inline int floatBitsToInt(float f) { int i; memcpy(&i, &f, 4); return i; }
inline float intBitsToFloat(int i) { float f; memcpy(&f, &i, 4); return f; }

}  // namespace glsl
