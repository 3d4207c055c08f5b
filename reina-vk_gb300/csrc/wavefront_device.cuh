// Device pieces shared by the single-frame wavefront (render.cu) and the multi-job batch engine
// (batch.cu): warp-aggregated queue appends, NEE (shaders/raytrace/nee.h.glsl, raytrace.rgen.glsl:43-95),
// the emission MIS light pdf, and the four closest-hit shaders (lambertian, metal, dielectric, disney
// .rchit.glsl) returning the payload fields the raygen loop reads next.
#pragma once

#include <stdint.h>

#include <type_traits>

#include <cuda_runtime.h>

#include "device_scene.h"
#include "kernels.h"
#include "render.h"
#include "shading_device.cuh"

namespace rt {

// Resident-block floor of the shading kernels, i.e. a register cap: uncapped, the Disney kernel takes
// ~200 registers (two 128-thread blocks per SM); at four blocks (128 registers) the batched render of 48
// scenes ran 5 % faster and the single-scene frame was unchanged.
#ifndef RT_SHADE_MINB
#define RT_SHADE_MINB 4
#endif
constexpr int kShadeMinBlocks = RT_SHADE_MINB;


// Checked build (compiled with -DRT_CHECKED): every queue position and path index the wavefront kernels
// read or write is checked against the path capacity; an index outside it is recorded in the error
// word (bit kErrIndexBounds) and replaced by 0, so the access stays in bounds and the call fails with
// REINA_ERR_DEVICE.  The normal build compiles the checks away.
constexpr uint32_t kErrIndexBounds = 4u;
__device__ __forceinline__ uint32_t checked_index(uint32_t i, uint64_t n, uint32_t* err) {
#ifdef RT_CHECKED
    if (i >= n) {
        atomicOr(err, kErrIndexBounds);
        return 0u;
    }
#else
    (void)n;
    (void)err;
#endif
    return i;
}

constexpr int kBlock = 128;
constexpr uint32_t kFlagInside = 1u;
constexpr uint32_t kFlagPrevNee = 2u;

// Appends for every lane with `pred` set; all 32 lanes of the warp must call it together.
__device__ __forceinline__ uint32_t warp_append(uint32_t* counter, bool pred) {
    const unsigned mask = __ballot_sync(0xFFFFFFFFu, pred);
    const int lane = threadIdx.x & 31;
    uint32_t base = 0;
    if (lane == 0 && mask) base = atomicAdd(counter, (uint32_t)__popc(mask));
    base = __shfl_sync(0xFFFFFFFFu, base, 0);
    return base + (uint32_t)__popc(mask & ((1u << lane) - 1u));
}

__device__ __forceinline__ void warp_count64(unsigned long long* counter, bool pred) {
    const unsigned mask = __ballot_sync(0xFFFFFFFFu, pred);
    if ((threadIdx.x & 31) == 0 && mask) atomicAdd(counter, (unsigned long long)__popc(mask));
}

__device__ __forceinline__ V3 clamp_keep_nan(V3 c, float hi) {
    auto one = [&](float x) { return isnan(x) ? x : fminf(fmaxf(x, 0.0f), hi); };
    return V3{one(c.x), one(c.y), one(c.z)};
}

__device__ __forceinline__ V3 load_thr(const PathState& ps, uint32_t p) { return V3{ps.tr[p], ps.tg[p], ps.tb[p]}; }
__device__ __forceinline__ V3 load_rad(const PathState& ps, uint32_t p) { return V3{ps.rr[p], ps.rg[p], ps.rb[p]}; }
__device__ __forceinline__ void store_thr(const PathState& ps, uint32_t p, V3 v) { ps.tr[p] = v.x; ps.tg[p] = v.y; ps.tb[p] = v.z; }
__device__ __forceinline__ void store_rad(const PathState& ps, uint32_t p, V3 v) { ps.rr[p] = v.x; ps.rg[p] = v.y; ps.rb[p] = v.z; }
__device__ __forceinline__ void store_ray(const PathState& ps, uint32_t p, V3 o, V3 d) {
    ps.ox[p] = o.x; ps.oy[p] = o.y; ps.oz[p] = o.z;
    ps.dx[p] = d.x; ps.dy[p] = d.y; ps.dz[p] = d.z;
}


// ------------------------------------------------------------------------------------------------
// Shared pieces of the shade kernels.

// Light pdf (solid angle) of reaching `p` on emissive triangle `prim` from `from` (emission MIS).
__device__ __forceinline__ float light_pdf_sa(const DeviceScene& s, float total_w, uint32_t prim, V3 from, V3 p) {
    uint32_t ii, pid;
    prim_lookup(s, prim, ii, pid);
    const InstanceGpu& inst = s.instances[ii];
    if (!(inst.light_weight > 0.0f)) return 0.0f;
    const InstanceProperties& pr = s.props[pid];
    const uint32_t lp = prim - inst.first_prim;
    const float* m = inst.m;
    auto wpos = [&](uint32_t k) {
        const V3 v = ld3(s.vertices + 4ull * s.indices[3 * lp + pr.indicesOffset + k]);
        return V3{m[0] * v.x + m[1] * v.y + m[2] * v.z + m[3], m[4] * v.x + m[5] * v.y + m[6] * v.z + m[7],
                  m[8] * v.x + m[9] * v.y + m[10] * v.z + m[11]};
    };
    const V3 v0 = wpos(0), v1 = wpos(1), v2 = wpos(2);
    const V3 n = norm3(cross3(v1 - v0, v2 - v0));
    const V3 dv = p - from;
    const float dist = len3(dv);
    const V3 dir = div3(dv, dist);
    const float pdf_area = (inst.light_weight / total_w) * (1.0f / inst.light_area);
    return pdf_area * dist * dist / fmaxf(dot3(n, -dir), 0.0001f);
}

struct LightSample {
    V3 point, normal, emission;
    float pdf;
    bool cull, valid;
};

// nee.h.glsl:52-124; an out-of-model triangle index (see randomEmissivePoint's use of the global CDF
// index as a model-relative index) yields an invalid sample instead of an out-of-range read.
__device__ __forceinline__ LightSample random_emissive_point(const DeviceScene& s, float total_w, uint32_t& rng) {
    LightSample ls;
    ls.valid = false;
    const float u0 = rng_next(rng);
    int lo = 0, hi = (int)s.emissive_count - 1;
    while (lo < hi) {
        const int mid = (lo + hi) / 2;
        if (u0 <= s.cdf_instances[mid]) hi = mid;
        else lo = mid + 1;
    }
    const EmissiveInstanceData& ed = s.emissive[lo];
    const float u1 = rng_next(rng);
    lo = (int)ed.cdfRangeStart;
    hi = (int)ed.cdfRangeEnd;
    while (lo < hi) {
        const int mid = (lo + hi) / 2;
        if (u1 <= s.cdf_triangles[mid]) hi = mid;
        else lo = mid + 1;
    }
    const uint32_t tri = (uint32_t)lo;
    const float r1 = rng_next(rng), r2 = rng_next(rng);
    if (tri > ed.cdfRangeEnd - ed.cdfRangeStart) return ls;
    const float* T = ed.transform;
    auto wpos = [&](uint32_t k) {
        const V3 v = ld3(s.vertices + 4ull * s.indices[3 * tri + ed.indexOffset + k]);
        return V3{T[0] * v.x + T[4] * v.y + T[8] * v.z + T[12], T[1] * v.x + T[5] * v.y + T[9] * v.z + T[13],
                  T[2] * v.x + T[6] * v.y + T[10] * v.z + T[14]};
    };
    const V3 v0 = wpos(0), v1 = wpos(1), v2 = wpos(2);
    const float beta = 1.0f - sqrtf(r1);
    const float gamma = (1.0f - beta) * r2;
    const float alpha = 1.0f - beta - gamma;
    ls.point = v0 * alpha + v1 * beta + v2 * gamma;
    ls.normal = norm3(cross3(v1 - v0, v2 - v0));
    ls.emission = ld3(ed.emission);
    ls.pdf = (ed.weight / total_w) * (1.0f / ed.area);
    ls.cull = ed.cullBackface != 0;
    ls.valid = true;
    return ls;
}

struct ShadowRec {
    V3 o, d, contrib;
    float tmax;
};

// directLight (raytrace.rgen.glsl:43-95) weighted by the power heuristic against the BSDF pdf of the
// light direction; returns false when no shadow ray is needed.
__device__ __forceinline__ bool next_event(const DeviceScene& s, float total_w, uint32_t& rng, bool disney, V3 origin, V3 n, V3 albedo,
                                           const InstanceProperties& pr, const M3& tbn, V3 rayIn, V3 thr, ShadowRec& out) {
    const LightSample t = random_emissive_point(s, total_w, rng);
    if (!t.valid) return false;
    const V3 dv = t.point - origin;
    const V3 dir = norm3(dv);
    const float dist = len3(dv);
    const float pl = t.pdf * dist * dist / fmaxf(dot3(t.normal, -dir), 0.0001f);
    V3 brdf;
    float pb;
    if (!disney) {
        brdf = div3(albedo, kPi);
        pb = pdf_lambertian(n, dir);
    } else {
        const V3 h = norm3(dir + -rayIn);
        brdf = eval_disney(tbn, disney_params(pr, albedo), 0.0f, false, n, -rayIn, dir, h, pb);
    }
    float cosI = dot3(n, dir);
    cosI = t.cull ? fmaxf(cosI, 0.0f) : fabsf(cosI);
    float gn = dot3(t.normal, -dir);
    gn = t.cull ? fmaxf(gn, 0.0f) : fabsf(gn);
    const float G = gn / (dist * dist);
    const V3 light = t.emission * brdf * (cosI * G / t.pdf);
    if (!(pl > 0.0f)) return false;
    out.o = origin;
    out.d = dir;
    out.tmax = dist - 0.001f;
    out.contrib = light * power_heuristic(pl, pb) * thr;
    return true;
}

// ------------------------------------------------------------------------------------------------
// Closest-hit shaders.  Each returns the payload fields the raygen loop reads next; `n` is the shading
// normal (the payload's surfaceNormal, which NEE uses).
struct Vertex {
    V3 color, albedo, emission, newO, newD, n;
    float pdf;
    bool inside, skip;
};

// closestHitCommon.h.glsl:185-193 (offset along the unperturbed normal)
__device__ __forceinline__ void skip_vertex(const HitInfo& h, V3 rd, Vertex& v) {
    v.newO = offset_along_normal(h.pos, -h.n);
    v.newD = rd;
    v.skip = true;
}

// lambertian.rchit.glsl:11-78
__device__ __forceinline__ Vertex shade_lambert(const DeviceScene& s, const HitInfo& h, const InstanceProperties& pr,
                                                V3 rd, uint32_t& rng, bool inside, float& acc) {
    Vertex v;
    v.skip = false;
    v.inside = inside;
    if (pr.cullBackface != 0u && !h.front) { skip_vertex(h, rd, v); return v; }
    V3 n, albedo;
    if (!apply_textures<true, true>(s, h, pr, rd, rng, n, albedo)) { skip_vertex(h, rd, v); return v; }
    v.color = albedo;
    v.albedo = v.color;
    v.emission = ld3(pr.emission);
    v.newO = offset_along_normal(h.pos, h.ng);
    v.newD = diffuse_reflection(n, rng);
    v.inside = false;
    v.n = n;
    v.pdf = pdf_lambertian(n, v.newD);
    acc = 0.0f;
    return v;
}

// metal.rchit.glsl:7-70
__device__ __forceinline__ Vertex shade_metal(const DeviceScene& s, const HitInfo& h, const InstanceProperties& pr,
                                              V3 rd, uint32_t& rng, bool inside, float& acc) {
    Vertex v;
    v.skip = false;
    v.inside = inside;
    if (pr.cullBackface != 0u && !h.front) { skip_vertex(h, rd, v); return v; }
    V3 n, albedo;
    if (!apply_textures<false, true>(s, h, pr, rd, rng, n, albedo)) { skip_vertex(h, rd, v); return v; }
    v.color = albedo;
    v.albedo = v.color;
    v.emission = ld3(pr.emission);
    v.newO = offset_along_normal(h.pos, h.ng);
    v.newD = fuzzy_reflection(rd, n, pr.roughness, rng);
    v.inside = false;
    v.n = n;
    v.pdf = 0.0f;
    acc = 0.0f;
    return v;
}

// dielectric.rchit.glsl:40-113 (the Fresnel term uses the unperturbed normal; the normal map bends the
// reflected and refracted directions; the albedo texture tints without an alpha test)
__device__ __forceinline__ Vertex shade_dielectric(const DeviceScene& s, const HitInfo& h, const InstanceProperties& pr,
                                                   V3 ro, V3 rd, uint32_t& rng, bool inside, float& acc) {
    Vertex v;
    v.skip = false;
    const float ri = h.front ? 1.0f / pr.ior : pr.ior;
    const V3 unitDir = norm3(rd);
    const float cosT = fminf(dot3(-unitDir, h.n), 1.0f);
    const float sinT = sqrtf(1.0f - cosT * cosT);
    const bool cannot = ri * sinT > 1.0f;
    const float refl = reflectance(cosT, ri);
    const bool prevInside = inside;
    V3 n, albedo;
    apply_textures<false, false>(s, h, pr, rd, rng, n, albedo);
    v.inside = inside;
    if (cannot || refl > rng_next(rng)) {
        v.newD = fuzzy_reflection(unitDir, n, pr.roughness, rng);
        v.color = V3{1.0f, 1.0f, 1.0f};
        v.newO = offset_along_normal(h.pos, h.ng);
    } else {
        v.inside = h.front;
        v.newD = refract3(unitDir, n, ri) + random_unit_vec(rng) * pr.roughness;
        v.color = albedo;
        v.newO = offset_for_dielectric(h.pos, h.ng, unitDir);
    }
    acc += prevInside ? len3(h.pos - ro) : 0.0f;
    if (prevInside && !v.inside) {
        v.color = V3{1.0f, 1.0f, 1.0f} * expf(-pr.absorption * acc);
        v.color = v.color * albedo;
        acc = 0.0f;
    }
    v.albedo = v.color;
    v.emission = ld3(pr.emission);
    v.n = n;
    v.pdf = 0.0f;
    return v;
}

// disney.rchit.glsl:36-198
__device__ __forceinline__ Vertex shade_disney(const DeviceScene& s, const HitInfo& h, const InstanceProperties& pr,
                                               V3 ro, V3 rd, uint32_t& rng, bool inside, float& acc) {
    Vertex v;
    v.skip = false;
    v.inside = inside;
    if (pr.cullBackface != 0u && !h.front) { skip_vertex(h, rd, v); return v; }
    V3 n, albedo;
    if (!apply_textures<true, true>(s, h, pr, rd, rng, n, albedo)) { skip_vertex(h, rd, v); return v; }
    const float eta = h.front ? 1.0f / pr.ior : pr.ior;
    const DisneyParams dp = disney_params(pr, albedo);
    bool didRefract = false, choseGlass = false;
    const V3 wi = -rd;
    const V3 dir = sample_disney(h.tbn, dp, eta, n, wi, didRefract, choseGlass, rng);
    const V3 hv = norm3(dir + wi);
    float pdf;
    const V3 f = eval_disney(h.tbn, dp, eta, didRefract, n, wi, dir, hv, pdf);
    const float cosI = fmaxf(dot3(n, dir), 0.0f);
    v.color = div3(f * cosI, pdf);
    v.albedo = albedo;
    v.pdf = pdf;
    v.emission = ld3(pr.emission);
    v.newO = offset_for_dielectric(h.pos, h.ng, dir);
    v.newD = dir;
    v.n = n;
    v.inside = choseGlass;
    if (v.inside) acc += len3(h.pos - ro);
    else acc = 0.0f;
    return v;
}


// getStartingRay (raytrace.rgen.glsl:34-41, 194-247): Gaussian pixel jitter (2 draws), unprojection
// through invProjection / invView, hexagonal aperture on a by-value copy of the RNG state.
__device__ __forceinline__ void camera_ray(const RtPushConsts& pc, uint32_t W, uint32_t H, uint32_t x, uint32_t y,
                                           uint32_t& rng, V3& o, V3& d) {
    const float u1 = fmaxf(1e-5f, rng_next(rng));
    const float u2 = rng_next(rng);
    const float r = sqrtf(-2.0f * logf(u1));
    const float theta = 2.0f * kPi * u2;
    float st, ct;
    sincosf(theta, &st, &ct);
    const float cx = (float)x + 0.5f + 0.375f * (r * ct);
    const float cy = (float)y + 0.5f + 0.375f * (r * st);
    const float ndcx = (cx / (float)W) * 2.0f - 1.0f;
    const float ndcy = -((cy / (float)H) * 2.0f - 1.0f);
    const float* P = pc.invProjection;
    float vp[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) vp[k] = P[0 * 4 + k] * ndcx + P[1 * 4 + k] * ndcy + P[2 * 4 + k] * -1.0f + P[3 * 4 + k] * 1.0f;
    const float w = vp[3];
    const V3 viewDir = norm3(V3{vp[0] / w, vp[1] / w, vp[2] / w});
    const float* V = pc.invView;
    const V3 wd{V[0] * viewDir.x + V[4] * viewDir.y + V[8] * viewDir.z, V[1] * viewDir.x + V[5] * viewDir.y + V[9] * viewDir.z,
                V[2] * viewDir.x + V[6] * viewDir.y + V[10] * viewDir.z};
    const V3 rd = norm3(wd);
    const V3 origin{V[12], V[13], V[14]};
    const V3 focal = origin + rd * pc.focusDist;
    uint32_t hs = rng;
    const float sqrt3 = 1.73205080757f;
    float hx = 0.0f, hy = 0.0f;
    for (int it = 0; it < 1 << 16; ++it) {
        hx = 2.0f * rng_next(hs) - 1.0f;
        hy = (rng_next(hs) - 0.5f) * sqrt3;
        if (!(fabsf(hy) > sqrt3 * 0.5f || (sqrt3 * fabsf(hx) + fabsf(hy)) > sqrt3)) break;
    }
    const float lx = hx * pc.defocusMultiplier, ly = hy * pc.defocusMultiplier;
    const V3 right = norm3(V3{V[0], V[1], V[2]});
    const V3 up = norm3(V3{V[4], V[5], V[6]});
    o = origin + right * lx + up * ly;
    d = norm3(focal - o);
}

// Host: calls f(std::integral_constant<int, BLOCK>, std::integral_constant<int, STACK>) for the traversal
// kernels' configured block size (64, 128, 256) and shared-memory stack depth (8, 12, 16).
template <class F>
inline void with_trace_variant(const TraceConfig& c, F&& f) {
    auto by_stack = [&](auto blk) {
        if (c.stack == 8) f(blk, std::integral_constant<int, 8>{});
        else if (c.stack == 16) f(blk, std::integral_constant<int, 16>{});
        else f(blk, std::integral_constant<int, 12>{});
    };
    if (c.block == 64) by_stack(std::integral_constant<int, 64>{});
    else if (c.block == 256) by_stack(std::integral_constant<int, 256>{});
    else by_stack(std::integral_constant<int, 128>{});
}

// Host: resident blocks of `kernel` at `block` threads, times the SM count (grid of a grid-stride kernel).
inline int resident_grid(const void* kernel, int block, int sm_count) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0);
    return (per_sm > 0 ? per_sm : 1) * (sm_count > 0 ? sm_count : 1);
}

}  // namespace rt
