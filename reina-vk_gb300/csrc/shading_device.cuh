// Device shading math of the trace path, transcribed from the reference's GLSL:
//   shaders/raytrace/shaderCommon.h.glsl   random() (PCG-style LCG + RXS-M-XS output)
//   shaders/raytrace/closestHitCommon.h.glsl getObjectHitInfo, offsetPositionAlongNormal, randomUnitVec,
//                                            fuzzyReflection, diffuseReflection
//   shaders/raytrace/brdfDisney.h.glsl     the Disney BSDF (sampleDisney / evalDisney and helpers)
//   shaders/raytrace/pdf.h.glsl            power heuristic, Lambertian pdf
// GLSL built-ins follow the GLSL 4.60 definitions (reflect, refract with k < 0 -> 0, faceforward, mix,
// normalize = v / length(v)).  pow(x, n) with a literal integer n is repeated multiplication.
#pragma once

#include <stdint.h>

#include "device_scene.h"
#include "rt_common.h"

namespace rt {

constexpr float kPi = 3.14159265f;      // k_pi
constexpr float kInvPi = 0.31830989f;   // k_inv_pi

__device__ __forceinline__ float dot3(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 cross3(V3 a, V3 b) {
    return V3{a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
__device__ __forceinline__ float len3(V3 a) { return sqrtf(dot3(a, a)); }
__device__ __forceinline__ V3 norm3(V3 a) {
    const float l = len3(a);
    return V3{a.x / l, a.y / l, a.z / l};
}
__device__ __forceinline__ V3 div3(V3 a, float s) { return V3{a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ V3 reflect3(V3 I, V3 N) { return I - N * (2.0f * dot3(N, I)); }
__device__ __forceinline__ V3 refract3(V3 I, V3 N, float eta) {
    const float d = dot3(N, I);
    const float k = 1.0f - eta * eta * (1.0f - d * d);
    if (k < 0.0f) return V3{0.0f, 0.0f, 0.0f};
    return I * eta - N * (eta * d + sqrtf(k));
}
__device__ __forceinline__ V3 faceforward3(V3 N, V3 I, V3 Nref) { return dot3(Nref, I) < 0.0f ? N : -N; }
__device__ __forceinline__ float mixf(float x, float y, float a) { return x * (1.0f - a) + y * a; }
__device__ __forceinline__ V3 mix3(V3 x, V3 y, float a) { return x * (1.0f - a) + y * a; }
__device__ __forceinline__ V3 mix3v(V3 x, V3 y, V3 a) {
    return V3{mixf(x.x, y.x, a.x), mixf(x.y, y.y, a.y), mixf(x.z, y.z, a.z)};
}
__device__ __forceinline__ float pow5f(float x) { return x * x * x * x * x; }
__device__ __forceinline__ float sqf(float x) { return x * x; }
__device__ __forceinline__ V3 ld3(const float* p) { return V3{p[0], p[1], p[2]}; }
__device__ __forceinline__ bool has_nan3(V3 a) { return isnan(a.x) || isnan(a.y) || isnan(a.z); }

struct M3 {   // columns (GLSL mat3(c0, c1, c2))
    V3 c0, c1, c2;
};
__device__ __forceinline__ V3 mul(const M3& m, V3 v) { return m.c0 * v.x + m.c1 * v.y + m.c2 * v.z; }
__device__ __forceinline__ V3 mulT(const M3& m, V3 v) { return V3{dot3(m.c0, v), dot3(m.c1, v), dot3(m.c2, v)}; }

// shaderCommon.h.glsl:39-45
__device__ __forceinline__ float rng_next(uint32_t& s) {
    s = s * 747796405u + 1u;
    uint32_t w = ((s >> ((s >> 28) + 4u)) ^ s) * 277803737u;
    w = (w >> 22) ^ w;
    return __fdiv_rn(__uint2float_rn(w), 4294967295.0f);
}

// Per-path seed of the nee_mis mode: a murmur3-style finalizer over (pixel, sample, seed).
__host__ __device__ __forceinline__ uint32_t path_seed(uint32_t pixel, uint32_t sample, uint32_t seed) {
    uint32_t h = seed * 0x9E3779B1u ^ (pixel * 0x85EBCA77u + 0x165667B1u) ^ (sample * 0xC2B2AE3Du + 0x27D4EB2Fu);
    h ^= h >> 16;
    h *= 0x7FEB352Du;
    h ^= h >> 15;
    h *= 0x846CA68Bu;
    h ^= h >> 16;
    return h;
}

// ---- closestHitCommon.h.glsl ----------------------------------------------------------------------
__device__ __forceinline__ V3 random_unit_vec(uint32_t& rng) {   // :195-205
    for (int it = 0; it < 1 << 20; ++it) {
        const float a = rng_next(rng), b = rng_next(rng), c = rng_next(rng);
        const V3 v{a * 2.0f - 1.0f, b * 2.0f - 1.0f, c * 2.0f - 1.0f};
        const float l2 = dot3(v, v);
        if (0.0001f < l2 && l2 < 1.0f) return norm3(v);
    }
    return V3{0.0f, 0.0f, 1.0f};   // unreachable for a working generator; bounds the loop
}
__device__ __forceinline__ V3 fuzzy_reflection(V3 rayIn, V3 n, float fuzz, uint32_t& rng) {   // :211-213
    return reflect3(norm3(rayIn), norm3(n)) + random_unit_vec(rng) * fuzz;
}
__device__ __forceinline__ V3 diffuse_reflection(V3 n, uint32_t& rng) {   // :215-222
    const float theta = 2.0f * kPi * rng_next(rng);
    const float u = 2.0f * rng_next(rng) - 1.0f;
    const float r = sqrtf(1.0f - u * u);
    float s, c;
    sincosf(theta, &s, &c);
    return norm3(n + V3{r * c, r * s, u});
}

// Wächter & Binder offset (closestHitCommon.h.glsl:156-177).
__device__ __forceinline__ V3 offset_along_normal(V3 p, V3 n) {
    auto one = [](float pk, float nk) {
        const int of = (int)(256.0f * nk);
        const int bits = __float_as_int(pk) + (pk < 0.0f ? -of : of);
        return fabsf(pk) < (1.0f / 32.0f) ? pk + (1.0f / 65536.0f) * nk : __int_as_float(bits);
    };
    return V3{one(p.x, n.x), one(p.y, n.y), one(p.z, n.z)};
}
// dielectric.rchit.glsl:14-38 / disney.rchit.glsl:10-34
__device__ __forceinline__ V3 offset_for_dielectric(V3 p, V3 n, V3 dir) {
    return offset_along_normal(p, dot3(n, dir) < 0.0f ? -n : n);
}

__device__ __forceinline__ float pdf_lambertian(V3 n, V3 w) { return fmaxf(dot3(n, w), 0.0f) / kPi; }
__device__ __forceinline__ float power_heuristic(float a, float b) { return a * a / (a * a + b * b); }

struct HitInfo {
    V3 pos, n, ng;
    bool front;
    M3 tbn;
    uint32_t props;
    uint32_t inst;
    uint32_t lp;      // triangle index within its model
    float bu, bv;     // barycentric weights of vertices 1 and 2
};

// getObjectHitInfo (closestHitCommon.h.glsl:52-148).  The UV is reconstructed on demand by surface_uv()
// (only textured materials read it).  Models without TBN data use the tangent frame (1,0,0), (0,1,0) and
// the geometric normal at every vertex (the reference reads its TBN buffer unconditionally).
__device__ __forceinline__ HitInfo hit_info(const DeviceScene& s, uint32_t prim, float bu, float bv, V3 rayDir) {
    HitInfo h;
    uint32_t ii, pid;
    prim_lookup(s, prim, ii, pid);
    const InstanceGpu& inst = s.instances[ii];
    h.inst = ii;
    h.props = pid;
    const InstanceProperties& pr = s.props[h.props];
    const uint32_t lp = prim - inst.first_prim;
    h.lp = lp;
    h.bu = bu;
    h.bv = bv;
    const uint32_t i0 = s.indices[3 * lp + pr.indicesOffset + 0];
    const uint32_t i1 = s.indices[3 * lp + pr.indicesOffset + 1];
    const uint32_t i2 = s.indices[3 * lp + pr.indicesOffset + 2];
    const V3 v0 = ld3(s.vertices + 4ull * i0), v1 = ld3(s.vertices + 4ull * i1), v2 = ld3(s.vertices + 4ull * i2);
    const float b0 = 1.0f - bu - bv;
    const V3 op = v0 * b0 + v1 * bu + v2 * bv;
    const float* m = inst.m;
    h.pos = V3{m[0] * op.x + m[1] * op.y + m[2] * op.z + m[3], m[4] * op.x + m[5] * op.y + m[6] * op.z + m[7],
               m[8] * op.x + m[9] * op.y + m[10] * op.z + m[11]};
    auto m3 = [&](V3 v) {
        return V3{m[0] * v.x + m[1] * v.y + m[2] * v.z, m[4] * v.x + m[5] * v.y + m[6] * v.z,
                  m[8] * v.x + m[9] * v.y + m[10] * v.z};
    };
    const V3 ngo = norm3(cross3(v1 - v0, v2 - v0));
    V3 no = ngo;
    M3 t0, t1, t2;
    const bool have_tbn = s.tbn_indices != nullptr && s.has_tbn != nullptr && s.has_tbn[inst.object];
    if (have_tbn) {
        auto ldm = [&](uint32_t k) {
            const float* q = s.tbns + 9ull * s.tbn_indices[3 * lp + pr.tbnsIndicesOffset + k];
            return M3{ld3(q), ld3(q + 3), ld3(q + 6)};
        };
        t0 = ldm(0);
        t1 = ldm(1);
        t2 = ldm(2);
        if (pr.interpNormals) no = norm3(norm3(t0.c2) * b0 + norm3(t1.c2) * bu + norm3(t2.c2) * bv);
    } else {
        t0.c0 = t1.c0 = t2.c0 = V3{1.0f, 0.0f, 0.0f};
        t0.c1 = t1.c1 = t2.c1 = V3{0.0f, 1.0f, 0.0f};
        t0.c2 = t1.c2 = t2.c2 = ngo;
    }
    h.n = norm3(m3(no));
    h.ng = norm3(m3(ngo));
    h.front = dot3(rayDir, h.ng) < 0.0f;
    h.n = faceforward3(h.n, rayDir, h.ng);
    h.ng = faceforward3(h.ng, rayDir, h.ng);
    const V3 tangent = norm3(t0.c0 * b0 + t1.c0 * bu + t2.c0 * bv);
    const V3 bitangent = norm3(t0.c1 * b0 + t1.c1 * bu + t2.c1 * bv);
    const V3 normal = norm3(t0.c2 * b0 + t1.c2 * bu + t2.c2 * bv);
    const float* nm = inst.nrm;
    const V3 nN{nm[0] * normal.x + nm[1] * normal.y + nm[2] * normal.z, nm[3] * normal.x + nm[4] * normal.y + nm[5] * normal.z,
                nm[6] * normal.x + nm[7] * normal.y + nm[8] * normal.z};
    V3 wT = norm3(m3(tangent));
    V3 wB = norm3(m3(bitangent));
    V3 wN = norm3(nN);
    wT = norm3(wT - wN * dot3(wN, wT));
    wB = norm3(wB - wN * dot3(wN, wB));
    wB = wB * -1.0f;
    wN = wN * (h.front ? 1.0f : -1.0f);
    h.tbn = M3{wT, wB, wN};
    return h;
}

// ---- textures ---------------------------------------------------------------------------------------

// Hit UV (closestHitCommon.h.glsl:96-111): barycentric blend of the corner texture coordinates, (0, 0)
// for a model without texture coordinates; a corner whose texture index is 0xFFFFFFFF contributes (0, 0).
__device__ __forceinline__ float2 surface_uv(const DeviceScene& s, const InstanceProperties& pr, const HitInfo& h) {
    if (pr.texIndicesOffset == 0xFFFFFFFFu) return make_float2(0.0f, 0.0f);
    auto tc = [&](uint32_t k) {
        const uint32_t t = s.tex_indices[3 * h.lp + pr.texIndicesOffset + k];
        return t == 0xFFFFFFFFu ? make_float2(0.0f, 0.0f) : make_float2(s.tex_coords[2ull * t], s.tex_coords[2ull * t + 1]);
    };
    const float2 t0 = tc(0), t1 = tc(1), t2 = tc(2);
    const float b0 = 1.0f - h.bu - h.bv;
    return make_float2(t0.x * b0 + t1.x * h.bu + t2.x * h.bv, t0.y * b0 + t1.y * h.bu + t2.y * h.bv);
}

// One axis of bilinear addressing with REPEAT wrapping (the sampler of src/tools/vktools.cpp:765-780;
// Vulkan texel filtering: coordinate c * size - 0.5, texels floor() and floor() + 1 modulo the size,
// weight frac()).  Non-finite coordinates address texel 0 with weight 0.  Explicitly rounded FP32 so the
// host restatement matches bit for bit.
__device__ __forceinline__ void tex_axis(float c, uint32_t size, uint32_t& i0, uint32_t& i1, float& w) {
    const float fs = (float)size;
    float x = __fsub_rn(__fmul_rn(c, fs), 0.5f);
    if (!(fabsf(x) <= 3.0e38f)) x = 0.0f;
    const float fx = floorf(x);
    w = __fsub_rn(x, fx);
    float r = fmodf(fx, fs);
    if (r < 0.0f) r = __fadd_rn(r, fs);
    i0 = (uint32_t)r;
    i1 = i0 + 1u == size ? 0u : i0 + 1u;
}

// texture(sampler2D, uv) at level 0 on R8G8B8A8_UNORM texels (src/graphics/Image.cpp:56): the four texels'
// 8-bit values are blended with the bilinear weights, then scaled by 1/255 (one division per channel).
template <int CH>
__device__ __forceinline__ float4 tex_sample(const DeviceScene& s, int id, float u, float v) {
    const uint4 ti = s.tex_info[id];
    uint32_t x0, x1, y0, y1;
    float a, b;
    tex_axis(u, ti.y, x0, x1, a);
    tex_axis(v, ti.z, y0, y1, b);
    const uint32_t* t = s.tex_texels + ti.x;
    const uint32_t c00 = __ldg(t + (size_t)y0 * ti.y + x0), c10 = __ldg(t + (size_t)y0 * ti.y + x1);
    const uint32_t c01 = __ldg(t + (size_t)y1 * ti.y + x0), c11 = __ldg(t + (size_t)y1 * ti.y + x1);
    const float na = __fsub_rn(1.0f, a), nb = __fsub_rn(1.0f, b);
    const float w00 = __fmul_rn(na, nb), w10 = __fmul_rn(a, nb), w01 = __fmul_rn(na, b), w11 = __fmul_rn(a, b);
    float out[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int k = 0; k < CH; ++k) {
        const int sh = 8 * k;
        float acc = __fmul_rn(w00, (float)((c00 >> sh) & 255u));
        acc = __fadd_rn(acc, __fmul_rn(w10, (float)((c10 >> sh) & 255u)));
        acc = __fadd_rn(acc, __fmul_rn(w01, (float)((c01 >> sh) & 255u)));
        acc = __fadd_rn(acc, __fmul_rn(w11, (float)((c11 >> sh) & 255u)));
        out[k] = __fdiv_rn(acc, 255.0f);
    }
    return make_float4(out[0], out[1], out[2], out[3]);
}

// bumpMapping (texutils.h.glsl:4-45): layered parallax search of the height map's red channel along the
// tangent-space view direction.  The layer loop ends by itself within 0.2 * 512 + 1 steps for finite
// input; the bound only guards NaN input.
__device__ __forceinline__ float2 bump_mapping(const DeviceScene& s, int id, float2 uv, V3 rayIn, const M3& T) {
    constexpr float kHeightScale = 0.2f, kMinLayers = 64.0f, kMaxLayers = 512.0f;
    const V3 V = norm3(mulT(T, -rayIn));
    if (V.z <= 0.0f) return uv;
    const float numLayers = mixf(kMaxLayers, kMinLayers, fminf(fmaxf(V.z, 0.0f), 1.0f));
    const float layerDepth = 1.0f / numLayers;
    const float px = V.x / V.z * kHeightScale, py = V.y / V.z * kHeightScale;
    const float dx = px / numLayers, dy = py / numLayers;
    float cu = uv.x, cv = uv.y;
    float depthSum = 0.0f;
    float h = tex_sample<1>(s, id, cu, cv).x * kHeightScale;
    for (int it = 0; depthSum < h && it < 1024; ++it) {
        cu -= dx;
        cv -= dy;
        depthSum += layerDepth;
        h = tex_sample<1>(s, id, cu, cv).x * kHeightScale;
    }
    const float pu = cu + dx, pv = cv + dy;
    const float hPrev = tex_sample<1>(s, id, pu, pv).x * kHeightScale;
    const float sumPrev = depthSum - layerDepth;
    const float after = h - depthSum;
    const float before = hPrev - sumPrev;
    const float weight = after / (after - before);
    return make_float2(mixf(pu, cu, weight), mixf(pv, cv, weight));
}

// The texture stage of the closest-hit shaders (lambertian.rchit.glsl:20-58, metal.rchit.glsl:18-50,
// dielectric.rchit.glsl:54-73, disney.rchit.glsl:19-72): UV wrapped by mod(uv, 1), bump mapping, the
// out-of-[0,1] skip (UVCHECK: Lambertian, Disney), the normal map (tangent normal rgb * 2 - 1 with y
// negated, through the hit's TBN) and the albedo texture with its alpha test (ALPHA: a < 0.999 and a
// uniform draw above a skips the hit; dielectrics only tint).  Returns false when the hit is skipped;
// `n` and `albedo` receive the shading normal and the albedo.
template <bool UVCHECK, bool ALPHA>
__device__ __forceinline__ bool apply_textures(const DeviceScene& s, const HitInfo& h, const InstanceProperties& pr, V3 rd,
                                               uint32_t& rng, V3& n, V3& albedo) {
    n = h.n;
    albedo = ld3(pr.albedo);
    if ((pr.textureID & pr.normalMapTexID & pr.bumpMapTexID) < 0) return true;   // all three unset
    float2 uv = surface_uv(s, pr, h);
    uv.x = uv.x - floorf(uv.x);
    uv.y = uv.y - floorf(uv.y);
    if (pr.bumpMapTexID >= 0) uv = bump_mapping(s, pr.bumpMapTexID, uv, norm3(rd), h.tbn);
    if (UVCHECK && (uv.x < 0.0f || uv.x > 1.0f || uv.y < 0.0f || uv.y > 1.0f)) return false;
    if (pr.normalMapTexID >= 0) {
        const float4 t = tex_sample<3>(s, pr.normalMapTexID, uv.x, uv.y);
        const V3 tn{t.x * 2.0f - 1.0f, -(t.y * 2.0f - 1.0f), t.z * 2.0f - 1.0f};
        n = norm3(mul(h.tbn, tn));
    }
    if (pr.textureID >= 0) {
        const float4 t = tex_sample<4>(s, pr.textureID, uv.x, uv.y);
        if (ALPHA && t.w < 0.999f && rng_next(rng) > t.w) return false;
        albedo = albedo * V3{t.x, t.y, t.z};
    }
    return true;
}

// ---- brdfDisney.h.glsl ------------------------------------------------------------------------------
__device__ __forceinline__ V3 sample_ggx_vndf(V3 V, float ax, float ay, uint32_t& rng) {   // :9-40
    const bool flip = V.z < 0.0f;
    if (flip) V.z = -V.z;
    const float r1 = rng_next(rng), r2 = rng_next(rng);
    const V3 Vh = norm3(V3{ax * V.x, ay * V.y, V.z});
    const float lensq = Vh.x * Vh.x + Vh.y * Vh.y;
    const V3 T1 = lensq > 0.0f ? V3{-Vh.y, Vh.x, 0.0f} * (1.0f / sqrtf(lensq)) : V3{1.0f, 0.0f, 0.0f};
    const V3 T2 = cross3(Vh, T1);
    const float r = sqrtf(r1);
    const float phi = 2.0f * kPi * r2;
    float sp, cp;
    sincosf(phi, &sp, &cp);
    const float t1 = r * cp;
    float t2 = r * sp;
    const float s = 0.5f * (1.0f + Vh.z);
    t2 = (1.0f - s) * sqrtf(1.0f - t1 * t1) + s * t2;
    V3 Nh = T1 * t1 + T2 * t2 + Vh * sqrtf(fmaxf(0.0f, 1.0f - t1 * t1 - t2 * t2));
    if (flip) Nh.z = -Nh.z;
    return norm3(V3{ax * Nh.x, ay * Nh.y, fmaxf(0.0f, Nh.z)});
}

__device__ __forceinline__ float d_ggx_aniso(V3 m, float ax, float ay) {   // :42-48
    const float NoM = fmaxf(m.z, 0.0f);
    const float inv = 1.0f / ((m.x / ax) * (m.x / ax) + (m.y / ay) * (m.y / ay) + NoM * NoM);
    return inv * inv / (kPi * ax * ay);
}

__device__ __forceinline__ float pdf_ggx_reflection(V3 i, V3 o, float ax, float ay) {   // :55-73
    const V3 m = norm3(i + o);
    const float ndf = d_ggx_aniso(m, ax, ay);
    const float aix = ax * i.x, aiy = ay * i.y;
    const float len2 = aix * aix + aiy * aiy;
    const float t = sqrtf(len2 + i.z * i.z);
    if (i.z >= 0.0f) {
        const float a = fminf(fmaxf(fminf(ax, ay), 0.0f), 1.0f);
        const float s = 1.0f + sqrtf(i.x * i.x + i.y * i.y);
        const float a2 = a * a, s2 = s * s;
        const float k = (1.0f - a2) * s2 / (s2 + a2 * i.z * i.z);
        return ndf / (2.0f * (k * i.z + t));
    }
    return ndf * (t - i.z) / (2.0f * len2);
}

__device__ __forceinline__ V3 sample_gtr1(float alpha, uint32_t& rng) {   // sampleGTR1_attempt2, :96-111
    const float r1 = rng_next(rng), r2 = rng_next(rng);
    const float a = fmaxf(0.001f, alpha);
    const float ch = sqrtf((1.0f - expf(r1 * logf(a * a))) / (1.0f - a * a));
    const float he = acosf(ch);
    const float ha = 2.0f * kPi * r2;
    float sh, chh, sa, ca;
    sincosf(he, &sh, &chh);
    sincosf(ha, &sa, &ca);
    return V3{sh * ca, sh * sa, ch};
}

__device__ __forceinline__ float fd_term(V3 n, V3 w, float fd90) { return 1.0f + (fd90 - 1.0f) * pow5f(1.0f - fmaxf(dot3(n, w), 0.0f)); }

__device__ __forceinline__ V3 eval_diffuse(float rough, float subsurface, V3 base, V3 n, V3 wi, V3 wo, V3 h) {   // :124-168
    const float hwo = dot3(h, wo);
    const float fd90 = 0.5f + 2.0f * rough * fmaxf(hwo, 0.0f) * fmaxf(hwo, 0.0f);
    const V3 bd = div3(base, kPi) * fd_term(n, wi, fd90) * fd_term(n, wo, fd90);
    const V3 k = base * 1.25f * kInvPi;
    const float fss90 = rough * fmaxf(dot3(h, wo), 0.0f) * fmaxf(dot3(h, wo), 0.0f);
    const float fin = 1.0f + (fss90 - 1.0f) * pow5f(1.0f - fmaxf(dot3(n, wi), 0.0f));
    const float fout = 1.0f + (fss90 - 1.0f) * pow5f(1.0f - fmaxf(dot3(n, wo), 0.0f));
    const float third = 1.0f / (fmaxf(dot3(n, wi), 0.0f) + fmaxf(dot3(n, wo), 0.0f)) - 0.5f;
    const V3 fsub = k * (fin * fout * third + 0.5f);
    return mix3(bd, fsub, subsurface);
}

__device__ __forceinline__ float pdf_diffuse(V3 wo, V3 n) {   // :170-179
    const float c = dot3(n, wo);
    return c <= 0.0f ? 0.0f : c * kInvPi;
}

__device__ __forceinline__ V3 sample_diffuse(V3 n, uint32_t& rng) {   // :181-201
    const float xi1 = rng_next(rng), xi2 = rng_next(rng);
    const float r = sqrtf(xi1);
    const float phi = 2.0f * kPi * xi2;
    float sp, cp;
    sincosf(phi, &sp, &cp);
    const float x = r * cp, y = r * sp;
    const float z = sqrtf(fmaxf(0.0f, 1.0f - xi1));
    const V3 t = fabsf(n.x) < 0.5f ? norm3(cross3(n, V3{1.0f, 0.0f, 0.0f})) : norm3(cross3(n, V3{0.0f, 1.0f, 0.0f}));
    const V3 b = cross3(n, t);
    return norm3(t * x + b * y + n * z);
}

__device__ __forceinline__ float eval_r0(float ior) { return (ior - 1.0f) * (ior - 1.0f) / ((ior + 1.0f) * (ior + 1.0f)); }
__device__ __forceinline__ float luminance3(V3 c) { return dot3(c, V3{0.2126f, 0.7152f, 0.0722f}); }

__device__ __forceinline__ V3 eval_fm(V3 base, V3 h, V3 wo, float specular, V3 specTint, float metallic, float eta) {   // :215-222
    const float lum = luminance3(base);
    const V3 one{1.0f, 1.0f, 1.0f};
    const V3 ctint = lum > 0.0f ? div3(base, lum) : one;
    const V3 ks = (one - ctint) + specTint * ctint;
    const V3 c0 = ks * (specular * eval_r0(eta) * (1.0f - metallic)) + base * metallic;
    return c0 + (one - c0) * pow5f(1.0f - fabsf(dot3(h, wo)));
}

__device__ __forceinline__ float eval_dm(V3 hl, float ax, float ay) {   // :224-229
    const float c = kPi * ax * ay;
    const float o = sqf(sqf(hl.x) / sqf(ax) + sqf(hl.y) / sqf(ay) + sqf(hl.z));
    return 1.0f / (c * o);
}
__device__ __forceinline__ float smith_g(V3 wl, float ax, float ay) {   // :231-239
    const float s = sqrtf(1.0f + (sqf(wl.x * ax) + sqf(wl.y * ay)) / sqf(wl.z));
    return 1.0f / (1.0f + (s - 1.0f) / 2.0f);
}
__device__ __forceinline__ void alphas(float aniso, float rough, float& ax, float& ay) {
    const float aspect = sqrtf(1.0f - 0.9f * aniso);
    ax = fmaxf(0.0001f, rough * rough / aspect);
    ay = fmaxf(0.0001f, rough * rough * aspect);
}

__device__ __forceinline__ V3 eval_metal(const M3& tbn, V3 base, float aniso, float rough, V3 n, V3 wi, V3 wo, V3 h,
                                         float specular, V3 specTint, float metallic, float eta) {   // :247-267
    float ax, ay;
    alphas(aniso, rough, ax, ay);
    const V3 fm = eval_fm(base, h, wo, specular, specTint, metallic, eta);
    const V3 wiT = norm3(mulT(tbn, wi)), woT = norm3(mulT(tbn, wo)), hT = norm3(mulT(tbn, h));
    const float dm = eval_dm(hT, ax, ay);
    const float gm = smith_g(wiT, ax, ay) * smith_g(woT, ax, ay);
    const float ni = fabsf(dot3(n, wi)), no = fabsf(dot3(n, wo));
    return div3(fm * dm * gm, 4.0f * ni * no);
}

__device__ __forceinline__ V3 sample_metal(const M3& tbn, float aniso, float rough, V3 wi, uint32_t& rng) {   // :269-285
    float ax, ay;
    alphas(aniso, rough, ax, ay);
    V3 h = sample_ggx_vndf(mulT(tbn, wi), ax, ay, rng);
    h = norm3(mul(tbn, h));
    return reflect3(-wi, h);
}

__device__ __forceinline__ float pdf_metal(const M3& tbn, V3 wi, V3 wo, float aniso, float rough) {   // :287-299
    float ax, ay;
    alphas(aniso, rough, ax, ay);
    return pdf_ggx_reflection(mulT(tbn, wi), mulT(tbn, wo), ax, ay);
}

__device__ __forceinline__ float sep_smith_g1(V3 w, float a) {   // :313-319
    const float a2 = a * a;
    return 2.0f / (1.0f + sqrtf(a2 + (1.0f - a2) * w.z * w.z));
}
__device__ __forceinline__ float eval_dc(float ag, V3 hl) {   // :328-333
    return (ag * ag - 1.0f) / (kPi * logf(ag * ag) * (1.0f + (ag * ag - 1.0f) * (hl.z * hl.z)));
}
__device__ __forceinline__ float clearcoat_alpha(float g) { return (1.0f - g) * 0.1f + g * 0.001f; }

__device__ __forceinline__ V3 eval_clearcoat(const M3& tbn, V3 wi, V3 wo, float gloss, V3 h) {   // :341-354
    const float ag = clearcoat_alpha(gloss);
    const V3 hT = mulT(tbn, h), wiT = mulT(tbn, wi), woT = mulT(tbn, wo);
    const float r0 = eval_r0(1.5f);
    const float fc = r0 + (1.0f - r0) * pow5f(1.0f - dot3(h, wo));
    const float gc = sep_smith_g1(wiT, 0.25f) * sep_smith_g1(woT, 0.25f);
    const float v = 0.25f * fc * gc * eval_dc(ag, hT);
    return V3{v, v, v};
}

__device__ __forceinline__ V3 sample_clearcoat(const M3& tbn, float gloss, V3 wi, uint32_t& rng) {   // :356-366
    V3 h = norm3(sample_gtr1(clearcoat_alpha(gloss), rng));
    h = norm3(mul(tbn, h));
    return norm3(reflect3(-wi, h));
}

__device__ __forceinline__ float pdf_clearcoat(const M3& tbn, V3 wi, V3 wo, V3 h, float gloss) {   // :368-383
    const float ag = clearcoat_alpha(gloss);
    const V3 wiT = mulT(tbn, wi), woT = mulT(tbn, wo), hT = mulT(tbn, h);
    if (wiT.z <= 0.0f || woT.z <= 0.0f) return 0.0f;
    const float dc = eval_dc(ag, hT) * hT.z;
    return dc / (4.0f * fabsf(dot3(woT, hT)));
}

__device__ __forceinline__ float reflectance(float cosine, float ri) {   // :389-394
    float r0 = (1.0f - ri) / (1.0f + ri);
    r0 = r0 * r0;
    return r0 + (1.0f - r0) * pow5f(1.0f - cosine);
}

__device__ __forceinline__ V3 sample_glass(const M3& tbn, V3 wi, float rough, float aniso, float eta, uint32_t& rng,
                                           bool& refracted) {   // :396-431
    float ax, ay;
    alphas(aniso, rough, ax, ay);
    const V3 wiT = mulT(tbn, wi);
    const V3 hT = sample_ggx_vndf(wiT, ax, ay, rng);
    const float c = dot3(wiT, hT);
    const V3 hW = norm3(mul(tbn, hT));
    const float refl = reflectance(c, eta);
    const float s = sqrtf(1.0f - c * c);
    const bool cannot = eta * s > 1.0f;
    if (cannot || refl > rng_next(rng)) {
        refracted = false;
        return reflect3(-wi, hW);
    }
    refracted = true;
    return refract3(-wi, hW, eta);
}

__device__ __forceinline__ float smith_g_aniso(float NdV, float VdX, float VdY, float ax, float ay) {   // :433-439
    const float a = VdX * ax, b = VdY * ay, c = NdV;
    return (2.0f * NdV) / (NdV + sqrtf(a * a + b * b + c * c));
}

__device__ __forceinline__ V3 eval_microfacet_refraction(V3 base, float aniso, float rough, float eta, V3 V, V3 L, V3 H,
                                                         float& pdf) {   // :441-467
    float ax, ay;
    alphas(aniso, rough, ax, ay);
    pdf = 0.0f;
    if (L.z >= 0.0f) return V3{0.0f, 0.0f, 0.0f};
    const float LdH = dot3(L, H), VdH = dot3(V, H);
    const float D = eval_dm(H, ax, ay);
    const float G1 = smith_g_aniso(fabsf(V.z), V.x, V.y, ax, ay);
    const float G2 = G1 * smith_g_aniso(fabsf(L.z), L.x, L.y, ax, ay);
    float denom = LdH + VdH * eta;
    denom *= denom;
    const float jac = fabsf(LdH) * (eta * eta) / denom;
    pdf = G1 * fmaxf(0.0f, VdH) * D * jac / V.z;
    const float F = reflectance(dot3(V, H), eta);
    const V3 sb{sqrtf(base.x), sqrtf(base.y), sqrtf(base.z)};
    return sb * ((1.0f - F) * D * G2 * fabsf(VdH) * jac / fabsf(L.z * V.z));
}

__device__ __forceinline__ V3 eval_glass(const M3& tbn, V3 base, float aniso, float rough, float eta, V3 n, V3 wi, V3 wo,
                                         bool didRefract, float& pdf) {   // :539-581
    V3 h = didRefract ? norm3(wo + wi * eta) : norm3(wo + wi);
    if (dot3(h, n) < 0.0f) h = -h;
    float tpdf;
    const V3 gf = eval_microfacet_refraction(base, aniso, rough, eta, mulT(tbn, wi), mulT(tbn, wo), mulT(tbn, h), tpdf);
    const float mpdf = pdf_metal(tbn, wi, wo, aniso, rough);
    const V3 mf = eval_metal(tbn, base, aniso, rough, n, wi, wo, h, 0.0f, V3{1.0f, 1.0f, 1.0f}, 1.0f, eta);
    if (didRefract) {
        pdf = tpdf;
        return gf;
    }
    pdf = mpdf;
    return mf;
}

__device__ __forceinline__ V3 eval_sheen(V3 base, V3 wo, V3 h, V3 n, V3 sheenTint) {   // :587-594
    const float lum = luminance3(base);
    const V3 one{1.0f, 1.0f, 1.0f};
    const V3 ctint = lum > 0.0f ? div3(base, lum) : one;
    const V3 cs = mix3v(one, ctint, sheenTint);
    return cs * (pow5f(1.0f - fmaxf(dot3(h, wo), 0.0f)) * fmaxf(dot3(n, wo), 0.0f));
}

struct DisneyParams {
    V3 base, specTint, sheenTint;
    float aniso, rough, subsurface, ccGloss, metallic, clearcoat, specTrans, sheen;
};

__device__ __forceinline__ DisneyParams disney_params(const InstanceProperties& p, V3 albedo) {
    DisneyParams d;
    d.base = albedo;
    d.specTint = ld3(p.specularTint);
    d.sheenTint = ld3(p.sheenTint);
    d.aniso = p.anisotropic;
    d.rough = p.roughness;
    d.subsurface = p.subsurface;
    d.ccGloss = p.clearcoatGloss;
    d.metallic = p.metallic;
    d.clearcoat = p.clearcoat;
    d.specTrans = p.specularTransmission;
    d.sheen = p.sheen;
    return d;
}

__device__ __forceinline__ V3 sample_disney(const M3& tbn, const DisneyParams& p, float eta, V3 n, V3 wi, bool& didRefract,
                                            bool& choseGlass, uint32_t& rng) {   // :609-654
    const float dw = (1.0f - p.specTrans) * (1.0f - p.metallic);
    const float mw = p.metallic;
    const float cw = 0.25f * p.clearcoat;
    const float gw = (1.0f - p.metallic) * p.specTrans;
    const float c0 = dw, c1 = c0 + mw, c2 = c1 + cw, c3 = c2 + gw;
    didRefract = false;
    const float r = rng_next(rng) * c3;
    choseGlass = false;
    if (r < c0) return sample_diffuse(n, rng);
    if (r < c1) return sample_metal(tbn, p.aniso, p.rough, wi, rng);
    if (r < c2) return sample_clearcoat(tbn, p.ccGloss, wi, rng);
    choseGlass = true;
    return sample_glass(tbn, wi, p.rough, p.aniso, eta, rng, didRefract);
}

__device__ __forceinline__ V3 eval_disney(const M3& tbn, const DisneyParams& p, float eta, bool didRefract, V3 n, V3 wi,
                                          V3 wo, V3 h, float& pdf) {   // :656-711
    const float dw = (1.0f - p.specTrans) * (1.0f - p.metallic);
    const float mw = p.metallic;
    const float cw = 0.25f * p.clearcoat;
    const float gw = (1.0f - p.metallic) * p.specTrans;
    const float sum = dw + mw + gw;
    const V3 fd = eval_diffuse(p.rough, p.subsurface, p.base, n, wi, wo, h);
    const float dpdf = pdf_diffuse(wo, n);
    const V3 fs = eval_sheen(p.base, wo, h, n, p.sheenTint);
    // evalMetal's `specular` argument receives specularTransmission (:692)
    const V3 fm = eval_metal(tbn, p.base, p.aniso, p.rough, n, wi, wo, h, p.specTrans, p.specTint, p.metallic, eta);
    const float mpdf = pdf_metal(tbn, wi, wo, p.aniso, p.rough);
    const V3 fc = eval_clearcoat(tbn, wi, wo, p.ccGloss, h);
    const float cpdf = pdf_clearcoat(tbn, wi, wo, h, p.ccGloss);
    float gpdf;
    const V3 fg = eval_glass(tbn, p.base, p.aniso, p.rough, eta, n, wi, wo, didRefract, gpdf);
    pdf = dpdf * dw / sum + mpdf * mw / sum + cpdf * cw + gpdf * gw / sum;
    return (fd + fs * p.sheen) * (dw / sum) + fm * (mw / sum) + fc * cw + fg * (gw / sum);
}

}  // namespace rt
