// ORACLE — test infrastructure only.  A CPU restatement of the reference's trace path used to check
// the CUDA kernels; it is never linked into, loaded by, or called from the product library.
//
// Parity status: the reference (AlexanderJCS/reina-vk) ships no tests, golden images or known-answer
// vectors, and it cannot be built or run here (Vulkan ray tracing + GLSL).  The oracle is therefore
// "parity unpinned" with respect to the reference itself; it is pinned to known-answer vectors derived
// from the formulas it restates (tests/golden/) and to analytic checks (watertightness, furnace tests).
//
// Shared helpers: the shader RNG, a small templated vector type, and the ray/hit records.
#pragma once

#include <cmath>
#include <cstdint>

namespace oracle {

template <class T>
struct Vec3 {
    T x, y, z;
    Vec3() : x(0), y(0), z(0) {}
    Vec3(T a, T b, T c) : x(a), y(b), z(c) {}
    template <class U>
    explicit Vec3(const Vec3<U>& o) : x((T)o.x), y((T)o.y), z((T)o.z) {}
    T operator[](int k) const { return k == 0 ? x : (k == 1 ? y : z); }
    T& operator[](int k) { return k == 0 ? x : (k == 1 ? y : z); }
};
template <class T> inline Vec3<T> operator+(Vec3<T> a, Vec3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> inline Vec3<T> operator-(Vec3<T> a, Vec3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> inline Vec3<T> operator-(Vec3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T> inline Vec3<T> operator*(Vec3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> inline Vec3<T> operator*(T s, Vec3<T> a) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> inline Vec3<T> operator*(Vec3<T> a, Vec3<T> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class T> inline Vec3<T> operator/(Vec3<T> a, T s) { return {a.x / s, a.y / s, a.z / s}; }
template <class T> inline T dot(Vec3<T> a, Vec3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> inline Vec3<T> cross(Vec3<T> a, Vec3<T> b) {
    return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
template <class T> inline T length(Vec3<T> a) { return std::sqrt(dot(a, a)); }
template <class T> inline Vec3<T> normalize(Vec3<T> a) { return a / length(a); }

// shaders/raytrace/shaderCommon.h.glsl:39-45 — PCG-style LCG step plus the RXS-M-XS output function,
// converted to [0, 1] by float(word) / 4294967295.0f (round to nearest; can give exactly 1.0).
inline uint32_t rng_step(uint32_t& state) {
    state = state * 747796405u + 1u;
    uint32_t word = ((state >> ((state >> 28) + 4u)) ^ state) * 277803737u;
    word = (word >> 22) ^ word;
    return word;
}
template <class T>
inline T rng_random(uint32_t& state) {
    const uint32_t w = rng_step(state);
    if (sizeof(T) == sizeof(float)) return (T)((float)w / 4294967295.0f);
    return (T)((double)w / 4294967295.0);
}

struct RayRec {
    float ox, oy, oz, tmin, dx, dy, dz, tmax;
};
struct HitRec {
    uint32_t prim;
    float t, u, v;
};
struct HitRec64 {
    uint32_t prim;
    uint32_t pad;
    double t, u, v;
};

constexpr uint32_t kMiss = 0xFFFFFFFFu;

}  // namespace oracle
