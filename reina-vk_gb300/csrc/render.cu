// Wavefront path tracer: the reference's per-pixel megakernel (shaders/raytrace/raytrace.rgen.glsl:97-285)
// split into kernels over queues of paths kept as SoA in HBM.  One wave = one sample of every pixel.
//   init      camera rays (getStartingRay, :206-247), per-pixel RNG / accumulatedDistance carry
//   extend    BVH8 closest hit of every active path + classification into per-material shade queues
//   shade_*   one kernel per material (miss, Lambertian, metal, dielectric, Disney): the closest-hit
//             shader followed by the raygen loop body (:124-180); surviving paths are appended to the
//             next active queue, NEE shadow rays to the shadow queue (nee_mis mode)
//   shadow    BVH8 any hit of the shadow queue (nee.h.glsl:126-144), unoccluded contributions added
//   finish    sample clamp / NaN drop / sum (:264-275)      resolve   mean and running mean (:277-284)
// Queue appends are warp-aggregated: one ballot, one atomicAdd per warp and queue, prefix by popcount.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>

#include "kernels.h"
#include "render.h"
#include "shading_device.cuh"
#include "trace_device.cuh"

namespace rt {

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
// init: getStartingRay (raytrace.rgen.glsl:34-41, 194-247) and per-path state
__global__ void __launch_bounds__(kBlock) k_init(RenderLaunch L) {
    const PathState& ps = L.ps;
    const uint32_t spp = L.pc.samplesPerPixel;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < L.P; i += gridDim.x * blockDim.x) {
        const uint32_t x = i % L.W, y = i / L.W;
        uint32_t rng;
        float acc;
        if (L.mode == kModeNeeMis) {
            rng = path_seed(i, L.pc.sampleBatch * spp + L.sample, L.seed);
            acc = 0.0f;
        } else if (L.sample == 0) {
            rng = (L.pc.sampleBatch * L.H + y) * L.W + x;
            acc = 0.0f;   // the payload's accumulatedDistance is uninitialized at launch start
        } else {
            rng = ps.pix_rng[i];
            acc = ps.pix_acc[i];
        }
        if (L.sample == 0) {
            ps.sr[i] = 0.0f; ps.sg[i] = 0.0f; ps.sb[i] = 0.0f;
            ps.cnt[i] = 0;
        }
        // randomGaussian
        const float u1 = fmaxf(1e-5f, rng_next(rng));
        const float u2 = rng_next(rng);
        const float r = sqrtf(-2.0f * logf(u1));
        const float theta = 2.0f * kPi * u2;
        float st, ct;
        sincosf(theta, &st, &ct);
        const float cx = (float)x + 0.5f + 0.375f * (r * ct);
        const float cy = (float)y + 0.5f + 0.375f * (r * st);
        const float ndcx = (cx / (float)L.W) * 2.0f - 1.0f;
        const float ndcy = -((cy / (float)L.H) * 2.0f - 1.0f);
        const float* P = L.pc.invProjection;
        float vp[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) vp[k] = P[0 * 4 + k] * ndcx + P[1 * 4 + k] * ndcy + P[2 * 4 + k] * -1.0f + P[3 * 4 + k] * 1.0f;
        const float w = vp[3];
        const V3 viewDir = norm3(V3{vp[0] / w, vp[1] / w, vp[2] / w});
        const float* V = L.pc.invView;
        const V3 wd{V[0] * viewDir.x + V[4] * viewDir.y + V[8] * viewDir.z, V[1] * viewDir.x + V[5] * viewDir.y + V[9] * viewDir.z,
                    V[2] * viewDir.x + V[6] * viewDir.y + V[10] * viewDir.z};
        const V3 rd = norm3(wd);
        const V3 origin{V[12], V[13], V[14]};
        const V3 focal = origin + rd * L.pc.focusDist;
        // randomInUnitHexagon takes the RNG state by value: it does not advance the path's stream
        uint32_t hs = rng;
        const float sqrt3 = 1.73205080757f;
        float hx = 0.0f, hy = 0.0f;
        for (int it = 0; it < 1 << 16; ++it) {
            hx = 2.0f * rng_next(hs) - 1.0f;
            hy = (rng_next(hs) - 0.5f) * sqrt3;
            if (!(fabsf(hy) > sqrt3 * 0.5f || (sqrt3 * fabsf(hx) + fabsf(hy)) > sqrt3)) break;
        }
        const float lx = hx * L.pc.defocusMultiplier, ly = hy * L.pc.defocusMultiplier;
        const V3 right = norm3(V3{V[0], V[1], V[2]});
        const V3 up = norm3(V3{V[4], V[5], V[6]});
        const V3 o = origin + right * lx + up * ly;
        const V3 d = norm3(focal - o);
        store_ray(ps, i, o, d);
        store_thr(ps, i, V3{1.0f, 1.0f, 1.0f});
        store_rad(ps, i, V3{0.0f, 0.0f, 0.0f});
        ps.rng[i] = rng;
        ps.acc[i] = acc;
        ps.flags[i] = 0u;
        ps.ppdf[i] = 0.0f;
        ps.q_active[0][i] = i;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) ps.counters[kCntActive] = L.P;
}

// ------------------------------------------------------------------------------------------------
// extend: closest hit + classification.  Grid form: each warp takes 32 consecutive queue entries.
__global__ void __launch_bounds__(kBlock) k_extend_grid(RenderLaunch L, int cur) {
    __shared__ uint2 stack[kSmemStack * kBlock];
    const PathState& ps = L.ps;
    const uint32_t n = ps.counters[kCntActive + cur];
    const uint32_t* q = ps.q_active[cur];
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const bool active = i < n;
        int m = -1;
        uint32_t p = 0;
        if (active) {
            p = q[i];
            const TraceRay r = make_trace_ray(ps.ox[p], ps.oy[p], ps.oz[p], ps.dx[p], ps.dy[p], ps.dz[p], 0.0f, 10000.0f);
            Hit h;
            TraceCounters c{0u, 0u};
            uint32_t e = 0;
            if (L.s.node_count) e = traverse<false, false, true>(L.s.nodes, L.s.tris, r, stack + threadIdx.x, kBlock, h, c);
            else h.prim = kMiss;
            if (e) atomicOr(ps.counters + kCntError, e);
            ps.hprim[p] = h.prim;
            ps.hu[p] = h.u;
            ps.hv[p] = h.v;
            m = h.prim == kMiss ? kQueueMiss : 1 + (int)L.s.props_material[L.s.prim_props[h.prim]];
        }
        warp_count64(reinterpret_cast<unsigned long long*>(ps.counters + kCntRays), active);
#pragma unroll
        for (int k = 0; k < kNumQueues; ++k) {
            const bool mine = active && m == k;
            const uint32_t pos = warp_append(ps.counters + kCntQueue + k, mine);
            if (mine) ps.q_shade[(size_t)k * L.P + pos] = p;
        }
    }
}

// Persistent form: warps refill idle lanes from the queue (dynamic ray fetch).
__global__ void __launch_bounds__(kBlock) k_extend(RenderLaunch L, int cur) {
    __shared__ uint2 stack[kSmemStack * kBlock];
    const PathState& ps = L.ps;
    const uint32_t n = ps.counters[kCntActive + cur];
    const uint32_t* q = ps.q_active[cur];
    TraceCounters c{0u, 0u};
    auto load = [&](uint32_t i, TraceRay& r) {
        const uint32_t p = q[i];
        r = make_trace_ray(ps.ox[p], ps.oy[p], ps.oz[p], ps.dx[p], ps.dy[p], ps.dz[p], 0.0f, 10000.0f);
        return true;
    };
    auto store = [&](uint32_t i, const Hit& h, bool valid) {   // called by all 32 lanes
        if (__ballot_sync(0xFFFFFFFFu, valid) == 0u) return;
        int m = -1;
        uint32_t p = 0;
        if (valid) {
            p = q[i];
            ps.hprim[p] = h.prim;
            ps.hu[p] = h.u;
            ps.hv[p] = h.v;
            m = h.prim == kMiss ? kQueueMiss : 1 + (int)L.s.props_material[L.s.prim_props[h.prim]];
        }
        warp_count64(reinterpret_cast<unsigned long long*>(ps.counters + kCntRays), valid);
#pragma unroll
        for (int k = 0; k < kNumQueues; ++k) {
            const bool mine = valid && m == k;
            const uint32_t pos = warp_append(ps.counters + kCntQueue + k, mine);
            if (mine) ps.q_shade[(size_t)k * L.P + pos] = p;
        }
    };
    const uint32_t e = persistent_trace<false, false, true>(L.s.nodes, L.s.tris, L.s.node_count, n,
                                                           ps.counters + kCntFetchExtend, stack + threadIdx.x, kBlock,
                                                           L.refill, load, store, c);
    if (e) atomicOr(ps.counters + kCntError, e);
}

// ------------------------------------------------------------------------------------------------
// Shared pieces of the shade kernels.

// Light pdf (solid angle) of reaching `p` on emissive triangle `prim` from `from` (emission MIS).
__device__ __forceinline__ float light_pdf_sa(const RenderLaunch& L, uint32_t prim, V3 from, V3 p) {
    const DeviceScene& s = L.s;
    const InstanceGpu& inst = s.instances[s.prim_instance[prim]];
    if (!(inst.light_weight > 0.0f)) return 0.0f;
    const InstanceProperties& pr = s.props[s.prim_props[prim]];
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
    const float pdf_area = (inst.light_weight / L.pc.totalEmissiveWeight) * (1.0f / inst.light_area);
    return pdf_area * dist * dist / fmaxf(dot3(n, -dir), 0.0001f);
}

struct LightSample {
    V3 point, normal, emission;
    float pdf;
    bool cull, valid;
};

// nee.h.glsl:52-124; an out-of-model triangle index (see randomEmissivePoint's use of the global CDF
// index as a model-relative index) yields an invalid sample instead of an out-of-range read.
__device__ __forceinline__ LightSample random_emissive_point(const RenderLaunch& L, uint32_t& rng) {
    const DeviceScene& s = L.s;
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
    ls.pdf = (ed.weight / L.pc.totalEmissiveWeight) * (1.0f / ed.area);
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
__device__ __forceinline__ bool next_event(const RenderLaunch& L, uint32_t& rng, bool disney, V3 origin, V3 n, V3 albedo,
                                           const InstanceProperties& pr, const M3& tbn, V3 rayIn, V3 thr, ShadowRec& out) {
    const LightSample t = random_emissive_point(L, rng);
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
// Closest-hit shaders.  Each returns the payload fields the raygen loop reads next.
struct Vertex {
    V3 color, albedo, emission, newO, newD;
    float pdf;
    bool inside, skip;
};

// closestHitCommon.h.glsl:185-193
__device__ __forceinline__ void skip_vertex(const HitInfo& h, V3 rd, Vertex& v) {
    v.newO = offset_along_normal(h.pos, -h.n);
    v.newD = rd;
    v.skip = true;
}

// lambertian.rchit.glsl:11-78
__device__ __forceinline__ Vertex shade_lambert(const HitInfo& h, const InstanceProperties& pr, V3 rd, uint32_t& rng,
                                                bool inside, float& acc) {
    Vertex v;
    v.skip = false;
    v.inside = inside;
    if (pr.cullBackface != 0u && !h.front) { skip_vertex(h, rd, v); return v; }
    v.color = ld3(pr.albedo);
    v.albedo = v.color;
    v.emission = ld3(pr.emission);
    v.newO = offset_along_normal(h.pos, h.ng);
    v.newD = diffuse_reflection(h.n, rng);
    v.inside = false;
    v.pdf = pdf_lambertian(h.n, v.newD);
    acc = 0.0f;
    return v;
}

// metal.rchit.glsl:7-70
__device__ __forceinline__ Vertex shade_metal(const HitInfo& h, const InstanceProperties& pr, V3 rd, uint32_t& rng,
                                              bool inside, float& acc) {
    Vertex v;
    v.skip = false;
    v.inside = inside;
    if (pr.cullBackface != 0u && !h.front) { skip_vertex(h, rd, v); return v; }
    v.color = ld3(pr.albedo);
    v.albedo = v.color;
    v.emission = ld3(pr.emission);
    v.newO = offset_along_normal(h.pos, h.ng);
    v.newD = fuzzy_reflection(rd, h.n, pr.roughness, rng);
    v.inside = false;
    v.pdf = 0.0f;
    acc = 0.0f;
    return v;
}

// dielectric.rchit.glsl:40-113
__device__ __forceinline__ Vertex shade_dielectric(const HitInfo& h, const InstanceProperties& pr, V3 ro, V3 rd,
                                                   uint32_t& rng, bool inside, float& acc) {
    Vertex v;
    v.skip = false;
    const float ri = h.front ? 1.0f / pr.ior : pr.ior;
    const V3 unitDir = norm3(rd);
    const float cosT = fminf(dot3(-unitDir, h.n), 1.0f);
    const float sinT = sqrtf(1.0f - cosT * cosT);
    const bool cannot = ri * sinT > 1.0f;
    const float refl = reflectance(cosT, ri);
    const bool prevInside = inside;
    const V3 albedo = ld3(pr.albedo);
    v.inside = inside;
    if (cannot || refl > rng_next(rng)) {
        v.newD = fuzzy_reflection(unitDir, h.n, pr.roughness, rng);
        v.color = V3{1.0f, 1.0f, 1.0f};
        v.newO = offset_along_normal(h.pos, h.ng);
    } else {
        v.inside = h.front;
        v.newD = refract3(unitDir, h.n, ri) + random_unit_vec(rng) * pr.roughness;
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
    v.pdf = 0.0f;
    return v;
}

// disney.rchit.glsl:36-198
__device__ __forceinline__ Vertex shade_disney(const HitInfo& h, const InstanceProperties& pr, V3 ro, V3 rd,
                                               uint32_t& rng, bool inside, float& acc) {
    Vertex v;
    v.skip = false;
    v.inside = inside;
    if (pr.cullBackface != 0u && !h.front) { skip_vertex(h, rd, v); return v; }
    const V3 albedo = ld3(pr.albedo);
    const float eta = h.front ? 1.0f / pr.ior : pr.ior;
    const DisneyParams dp = disney_params(pr, albedo);
    bool didRefract = false, choseGlass = false;
    const V3 wi = -rd;
    const V3 dir = sample_disney(h.tbn, dp, eta, h.n, wi, didRefract, choseGlass, rng);
    const V3 hv = norm3(dir + wi);
    float pdf;
    const V3 f = eval_disney(h.tbn, dp, eta, didRefract, h.n, wi, dir, hv, pdf);
    const float cosI = fmaxf(dot3(h.n, dir), 0.0f);
    v.color = div3(f * cosI, pdf);
    v.albedo = albedo;
    v.pdf = pdf;
    v.emission = ld3(pr.emission);
    v.newO = offset_for_dielectric(h.pos, h.ng, dir);
    v.newD = dir;
    v.inside = choseGlass;
    if (v.inside) acc += len3(h.pos - ro);
    else acc = 0.0f;
    return v;
}

// One kernel per material queue (MAT = 1 Lambertian, 2 metal, 3 dielectric, 4 Disney): the closest-hit
// shader, then the raygen loop body (raytrace.rgen.glsl:124-180).
template <int MAT>
__global__ void __launch_bounds__(kBlock) k_shade(RenderLaunch L, int cur) {
    const PathState& ps = L.ps;
    const uint32_t n = ps.counters[kCntQueue + MAT];
    const uint32_t* q = ps.q_shade + (size_t)MAT * L.P;
    const bool nee = L.mode == kModeNeeMis;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const bool active = i < n;
        bool emit = false;
        ShadowRec sh;
        uint32_t p = 0;
        if (active) {
            p = q[i];
            const V3 ro{ps.ox[p], ps.oy[p], ps.oz[p]};
            const V3 rd{ps.dx[p], ps.dy[p], ps.dz[p]};
            const uint32_t prim = ps.hprim[p];
            const HitInfo h = hit_info(L.s, prim, ps.hu[p], ps.hv[p], rd);
            const InstanceProperties& pr = L.s.props[h.props];
            uint32_t rng = ps.rng[p];
            uint32_t flags = ps.flags[p];
            float acc = ps.acc[p];
            const bool inside = (flags & kFlagInside) != 0;
            Vertex vx;
            if (MAT == 1) vx = shade_lambert(h, pr, rd, rng, inside, acc);
            else if (MAT == 2) vx = shade_metal(h, pr, rd, rng, inside, acc);
            else if (MAT == 3) vx = shade_dielectric(h, pr, ro, rd, rng, inside, acc);
            else vx = shade_disney(h, pr, ro, rd, rng, inside, acc);
            if (vx.skip) {
                flags &= ~kFlagPrevNee;
            } else {
                flags = vx.inside ? (flags | kFlagInside) : (flags & ~kFlagInside);
                if (!vx.inside) {
                    V3 thr = load_thr(ps, p), rad = load_rad(ps, p);
                    V3 contrib = vx.emission;
                    if (nee) {
                        if ((flags & kFlagPrevNee) && (vx.emission.x != 0.0f || vx.emission.y != 0.0f || vx.emission.z != 0.0f))
                            contrib = contrib * power_heuristic(ps.ppdf[p], light_pdf_sa(L, prim, ro, vx.newO));
                        const bool do_nee = (MAT == 1 || MAT == 4) && L.s.emissive_count > 0;
                        if (do_nee) emit = next_event(L, rng, MAT == 4, vx.newO, h.n, vx.albedo, pr, h.tbn, rd, thr, sh);
                        flags = do_nee ? (flags | kFlagPrevNee) : (flags & ~kFlagPrevNee);
                        ps.ppdf[p] = vx.pdf;
                    }
                    rad = rad + contrib * thr;
                    thr = thr * vx.color;
                    store_thr(ps, p, thr);
                    store_rad(ps, p, rad);
                } else {
                    flags &= ~kFlagPrevNee;
                }
            }
            store_ray(ps, p, vx.newO, vx.newD);
            ps.rng[p] = rng;
            ps.flags[p] = flags;
            ps.acc[p] = acc;
        }
        const uint32_t pos = warp_append(ps.counters + kCntActive + (cur ^ 1), active);
        if (active) ps.q_active[cur ^ 1][pos] = p;
        const uint32_t spos = warp_append(ps.counters + kCntShadow, emit);
        if (emit) {
            ps.q_shadow[spos] = p;
            ps.s_ox[spos] = sh.o.x; ps.s_oy[spos] = sh.o.y; ps.s_oz[spos] = sh.o.z;
            ps.s_dx[spos] = sh.d.x; ps.s_dy[spos] = sh.d.y; ps.s_dz[spos] = sh.d.z;
            ps.s_tmax[spos] = sh.tmax;
            ps.s_cr[spos] = sh.contrib.x; ps.s_cg[spos] = sh.contrib.y; ps.s_cb[spos] = sh.contrib.z;
        }
    }
}

// raytrace.rmiss.glsl:10-19: the path ends with sky (or constant environment) radiance.
__global__ void __launch_bounds__(kBlock) k_shade_miss(RenderLaunch L) {
    const PathState& ps = L.ps;
    const uint32_t n = ps.counters[kCntQueue + kQueueMiss];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t p = ps.q_shade[i];
        V3 sky;
        if (L.env_mode == 1) {
            sky = V3{L.env[0], L.env[1], L.env[2]};
        } else {
            const float y = norm3(V3{ps.dx[p], ps.dy[p], ps.dz[p]}).y;
            const float t = 0.5f * (y + 1.0f);
            sky = mix3(V3{0.1f, 0.1f, 0.1f}, V3{0.4f, 1.7f, 2.0f}, t) * 0.07f;
        }
        store_rad(ps, p, load_rad(ps, p) + sky * load_thr(ps, p));
    }
}

// nee.h.glsl:126-144: any hit in [0, dist - 0.001]; unoccluded contributions are added.  Grid form.
__global__ void __launch_bounds__(kBlock) k_shadow_grid(RenderLaunch L) {
    __shared__ uint2 stack[kSmemStack * kBlock];
    const PathState& ps = L.ps;
    const uint32_t n = ps.counters[kCntShadow];
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const bool active = i < n;
        if (active) {
            const TraceRay r = make_trace_ray(ps.s_ox[i], ps.s_oy[i], ps.s_oz[i], ps.s_dx[i], ps.s_dy[i], ps.s_dz[i], 0.0f,
                                              ps.s_tmax[i]);
            Hit h;
            TraceCounters c{0u, 0u};
            uint32_t e = 0;
            if (L.s.node_count) e = traverse<true, false, false>(L.s.nodes, L.s.tris, r, stack + threadIdx.x, kBlock, h, c);
            else h.prim = kMiss;
            if (e) atomicOr(ps.counters + kCntError, e);
            if (h.prim == kMiss) {
                const uint32_t p = ps.q_shadow[i];
                store_rad(ps, p, load_rad(ps, p) + V3{ps.s_cr[i], ps.s_cg[i], ps.s_cb[i]});
            }
        }
        warp_count64(reinterpret_cast<unsigned long long*>(ps.counters + kCntShadowRays), active);
    }
}

// Persistent form of the shadow kernel.
__global__ void __launch_bounds__(kBlock) k_shadow(RenderLaunch L) {
    __shared__ uint2 stack[kSmemStack * kBlock];
    const PathState& ps = L.ps;
    const uint32_t n = ps.counters[kCntShadow];
    TraceCounters c{0u, 0u};
    auto load = [&](uint32_t i, TraceRay& r) {
        r = make_trace_ray(ps.s_ox[i], ps.s_oy[i], ps.s_oz[i], ps.s_dx[i], ps.s_dy[i], ps.s_dz[i], 0.0f, ps.s_tmax[i]);
        return true;
    };
    auto store = [&](uint32_t i, const Hit& h, bool valid) {   // called by all 32 lanes
        if (valid && h.prim == kMiss) {
            const uint32_t p = ps.q_shadow[i];
            store_rad(ps, p, load_rad(ps, p) + V3{ps.s_cr[i], ps.s_cg[i], ps.s_cb[i]});
        }
        warp_count64(reinterpret_cast<unsigned long long*>(ps.counters + kCntShadowRays), valid);
    };
    const uint32_t e = persistent_trace<true, false, false>(L.s.nodes, L.s.tris, L.s.node_count, n,
                                                           ps.counters + kCntFetchShadow, stack + threadIdx.x, kBlock,
                                                           L.refill, load, store, c);
    if (e) atomicOr(ps.counters + kCntError, e);
}

// raytrace.rgen.glsl:264-275: clamp to [0, directClamp] (NaN kept), drop NaN samples, sum the rest.
__global__ void __launch_bounds__(kBlock) k_finish(RenderLaunch L) {
    const PathState& ps = L.ps;
    const uint32_t spp = L.pc.samplesPerPixel;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < L.P; i += gridDim.x * blockDim.x) {
        const V3 c = clamp_keep_nan(load_rad(ps, i), L.pc.directClamp);
        if (L.samples) {
            float* o = L.samples + 3ull * ((uint64_t)i * spp + L.sample);
            o[0] = c.x; o[1] = c.y; o[2] = c.z;
        }
        if (!has_nan3(c)) {
            ps.sr[i] += c.x;
            ps.sg[i] += c.y;
            ps.sb[i] += c.z;
            ps.cnt[i] += 1;
        }
        ps.pix_rng[i] = ps.rng[i];
        ps.pix_acc[i] = ps.acc[i];
    }
}

// raytrace.rgen.glsl:277-284: mean over kept samples, running mean with the previous image.
__global__ void __launch_bounds__(kBlock) k_resolve(RenderLaunch L) {
    const PathState& ps = L.ps;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < L.P; i += gridDim.x * blockDim.x) {
        const float k = (float)ps.cnt[i];
        V3 fin{ps.sr[i] / k, ps.sg[i] / k, ps.sb[i] / k};
        float4* a = reinterpret_cast<float4*>(L.accum) + i;
        if (L.pc.sampleBatch > 0) {
            const float4 prev = *a;
            const float b = (float)L.pc.sampleBatch;
            fin = div3(V3{prev.x, prev.y, prev.z} * b + fin, (float)(L.pc.sampleBatch + 1));
        }
        *a = make_float4(fin.x, fin.y, fin.z, 1.0f);
    }
}

// ------------------------------------------------------------------------------------------------
// Plain form: the reference's megakernel structure (raytrace.rgen.glsl:250-285) — one thread per pixel
// runs every sample and segment, with the closest-hit shading and NEE shadow rays inline.  Same device
// functions as the wavefront kernels; used as the single-kernel baseline the wavefront is compared with.
__global__ void __launch_bounds__(kBlock) k_megakernel(RenderLaunch L) {
    __shared__ uint2 stack[kSmemStack * kBlock];
    const PathState& ps = L.ps;
    const uint32_t spp = L.pc.samplesPerPixel;
    const bool nee = L.mode == kModeNeeMis;
    unsigned long long n_rays = 0, n_shadow = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < L.P; i += gridDim.x * blockDim.x) {
        const uint32_t x = i % L.W, y = i / L.W;
        uint32_t rng = (L.pc.sampleBatch * L.H + y) * L.W + x;
        float acc = 0.0f;
        V3 sum{0.0f, 0.0f, 0.0f};
        uint32_t kept = 0;
        for (uint32_t smp = 0; smp < spp; ++smp) {
            if (nee) {
                rng = path_seed(i, L.pc.sampleBatch * spp + smp, L.seed);
                acc = 0.0f;
            }
            // getStartingRay
            const float u1 = fmaxf(1e-5f, rng_next(rng));
            const float u2 = rng_next(rng);
            const float rr = sqrtf(-2.0f * logf(u1));
            float st, ct;
            sincosf(2.0f * kPi * u2, &st, &ct);
            const float cx = (float)x + 0.5f + 0.375f * (rr * ct);
            const float cy = (float)y + 0.5f + 0.375f * (rr * st);
            const float ndcx = (cx / (float)L.W) * 2.0f - 1.0f;
            const float ndcy = -((cy / (float)L.H) * 2.0f - 1.0f);
            const float* P = L.pc.invProjection;
            float vp[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) vp[k] = P[0 * 4 + k] * ndcx + P[1 * 4 + k] * ndcy + P[2 * 4 + k] * -1.0f + P[3 * 4 + k] * 1.0f;
            const V3 viewDir = norm3(V3{vp[0] / vp[3], vp[1] / vp[3], vp[2] / vp[3]});
            const float* V = L.pc.invView;
            const V3 rd0 = norm3(V3{V[0] * viewDir.x + V[4] * viewDir.y + V[8] * viewDir.z,
                                    V[1] * viewDir.x + V[5] * viewDir.y + V[9] * viewDir.z,
                                    V[2] * viewDir.x + V[6] * viewDir.y + V[10] * viewDir.z});
            const V3 origin{V[12], V[13], V[14]};
            const V3 focal = origin + rd0 * L.pc.focusDist;
            uint32_t hs = rng;
            const float sqrt3 = 1.73205080757f;
            float hx = 0.0f, hy = 0.0f;
            for (int it = 0; it < 1 << 16; ++it) {
                hx = 2.0f * rng_next(hs) - 1.0f;
                hy = (rng_next(hs) - 0.5f) * sqrt3;
                if (!(fabsf(hy) > sqrt3 * 0.5f || (sqrt3 * fabsf(hx) + fabsf(hy)) > sqrt3)) break;
            }
            V3 ro = origin + norm3(V3{V[0], V[1], V[2]}) * (hx * L.pc.defocusMultiplier) +
                    norm3(V3{V[4], V[5], V[6]}) * (hy * L.pc.defocusMultiplier);
            V3 rd = norm3(focal - ro);
            // traceSegments
            V3 thr{1.0f, 1.0f, 1.0f}, rad{0.0f, 0.0f, 0.0f};
            bool inside = false, prev_nee = false;
            float ppdf = 0.0f;
            for (uint32_t seg = 0; seg < L.pc.maxBounces; ++seg) {
                const TraceRay r = make_trace_ray(ro.x, ro.y, ro.z, rd.x, rd.y, rd.z, 0.0f, 10000.0f);
                Hit h;
                TraceCounters c{0u, 0u};
                uint32_t e = 0;
                if (L.s.node_count) e = traverse<false, false, true>(L.s.nodes, L.s.tris, r, stack + threadIdx.x, kBlock, h, c);
                else h.prim = kMiss;
                if (e) atomicOr(ps.counters + kCntError, e);
                ++n_rays;
                if (h.prim == kMiss) {
                    V3 sky;
                    if (L.env_mode == 1) {
                        sky = V3{L.env[0], L.env[1], L.env[2]};
                    } else {
                        const float t = 0.5f * (norm3(rd).y + 1.0f);
                        sky = mix3(V3{0.1f, 0.1f, 0.1f}, V3{0.4f, 1.7f, 2.0f}, t) * 0.07f;
                    }
                    rad = rad + sky * thr;
                    break;
                }
                const HitInfo hi = hit_info(L.s, h.prim, h.u, h.v, rd);
                const InstanceProperties& pr = L.s.props[hi.props];
                const uint32_t mat = L.s.props_material[hi.props];
                Vertex vx;
                if (mat == 0) vx = shade_lambert(hi, pr, rd, rng, inside, acc);
                else if (mat == 1) vx = shade_metal(hi, pr, rd, rng, inside, acc);
                else if (mat == 2) vx = shade_dielectric(hi, pr, ro, rd, rng, inside, acc);
                else vx = shade_disney(hi, pr, ro, rd, rng, inside, acc);
                const V3 ray_org = ro, ray_in = rd;
                ro = vx.newO;
                rd = vx.newD;
                if (vx.skip) {
                    prev_nee = false;
                    continue;
                }
                inside = vx.inside;
                if (!inside) {
                    V3 contrib = vx.emission;
                    if (nee) {
                        if (prev_nee && (vx.emission.x != 0.0f || vx.emission.y != 0.0f || vx.emission.z != 0.0f))
                            contrib = contrib * power_heuristic(ppdf, light_pdf_sa(L, h.prim, ray_org, vx.newO));
                        const bool do_nee = (mat == 0 || mat == 3) && L.s.emissive_count > 0;
                        if (do_nee) {
                            ShadowRec sh;
                            if (next_event(L, rng, mat == 3, vx.newO, hi.n, vx.albedo, pr, hi.tbn, ray_in, thr, sh)) {
                                const TraceRay sr = make_trace_ray(sh.o.x, sh.o.y, sh.o.z, sh.d.x, sh.d.y, sh.d.z, 0.0f, sh.tmax);
                                Hit sh_hit;
                                uint32_t e2 = 0;
                                e2 = traverse<true, false, false>(L.s.nodes, L.s.tris, sr, stack + threadIdx.x, kBlock, sh_hit, c);
                                if (e2) atomicOr(ps.counters + kCntError, e2);
                                ++n_shadow;
                                if (sh_hit.prim == kMiss) rad = rad + sh.contrib;
                            }
                        }
                        prev_nee = do_nee;
                        ppdf = vx.pdf;
                    }
                    rad = rad + contrib * thr;
                    thr = thr * vx.color;
                } else {
                    prev_nee = false;
                }
            }
            const V3 col = clamp_keep_nan(rad, L.pc.directClamp);
            if (L.samples) {
                float* o = L.samples + 3ull * ((uint64_t)i * spp + smp);
                o[0] = col.x; o[1] = col.y; o[2] = col.z;
            }
            if (!has_nan3(col)) {
                sum = sum + col;
                kept++;
            }
        }
        const float k = (float)kept;
        V3 fin{sum.x / k, sum.y / k, sum.z / k};
        float4* a = reinterpret_cast<float4*>(L.accum) + i;
        if (L.pc.sampleBatch > 0) {
            const float4 prev = *a;
            fin = div3(V3{prev.x, prev.y, prev.z} * (float)L.pc.sampleBatch + fin, (float)(L.pc.sampleBatch + 1));
        }
        *a = make_float4(fin.x, fin.y, fin.z, 1.0f);
    }
    // every lane of the warp reaches this point: reduce the per-thread ray counts
    for (int o = 16; o > 0; o >>= 1) {
        n_rays += __shfl_down_sync(0xFFFFFFFFu, n_rays, o);
        n_shadow += __shfl_down_sync(0xFFFFFFFFu, n_shadow, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(reinterpret_cast<unsigned long long*>(ps.counters + kCntRays), n_rays);
        atomicAdd(reinterpret_cast<unsigned long long*>(ps.counters + kCntShadowRays), n_shadow);
    }
}

// ------------------------------------------------------------------------------------------------
// Host side
// 4-byte words per path: ray 6, hit 3, throughput 3, radiance 3, rng, flags, acc, ppdf (19);
// per pixel: rng, acc, sum 3, count (6); queues: active 2, shade 5, shadow 1 (8); shadow rays 10.
constexpr size_t kWordsPerPath = 19 + 6 + 8 + 10;
constexpr size_t kHeaderWords = 64;   // counters, padded so that the arrays start 256-byte aligned

static size_t path_state_words(size_t paths) { return paths * kWordsPerPath + kHeaderWords; }

// Carves the SoA path state for `paths` slots out of `w` (path_state_words(paths) words).
static PathState layout_path_state(uint32_t* w, size_t P) {
    size_t off = 0;
    auto f = [&]() { float* r = reinterpret_cast<float*>(w + off); off += P; return r; };
    auto u = [&]() { uint32_t* r = w + off; off += P; return r; };
    PathState s;
    s.counters = w;
    off = kHeaderWords;
    s.ox = f(); s.oy = f(); s.oz = f(); s.dx = f(); s.dy = f(); s.dz = f();
    s.hprim = u(); s.hu = f(); s.hv = f();
    s.tr = f(); s.tg = f(); s.tb = f();
    s.rr = f(); s.rg = f(); s.rb = f();
    s.rng = u(); s.flags = u(); s.acc = f(); s.ppdf = f();
    s.pix_rng = u(); s.pix_acc = f(); s.sr = f(); s.sg = f(); s.sb = f(); s.cnt = u();
    s.q_active[0] = u(); s.q_active[1] = u();
    s.q_shade = w + off; off += P * kNumQueues;
    s.q_shadow = u();
    s.s_ox = f(); s.s_oy = f(); s.s_oz = f(); s.s_dx = f(); s.s_dy = f(); s.s_dz = f(); s.s_tmax = f();
    s.s_cr = f(); s.s_cg = f(); s.s_cb = f();
    return s;
}

void RenderWorkspace::ensure(uint32_t paths) {
    if (paths <= capacity_ && buf_.get()) return;
    buf_.alloc(path_state_words(paths) * 4);
    ps_ = layout_path_state(buf_.as<uint32_t>(), paths);
    capacity_ = paths;
}

static int occupancy_blocks(const void* fn, int sm_count) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kBlock, 0);
    return std::max(1, per_sm) * std::max(1, sm_count);
}

// The frame's launch sequence over path state `ps` (at least width*height slots).
static void launch_frame(const PathState& ps, const DeviceScene& s, const RtPushConsts& pc, const RenderOpts& opt,
                         float* d_accum, float* d_samples, int sm_count, cudaStream_t st, RenderStats* stats) {
    const uint32_t P = opt.width * opt.height;
    RenderLaunch L;
    L.s = s;
    L.pc = pc;
    L.ps = ps;
    L.W = opt.width;
    L.H = opt.height;
    L.P = P;
    L.mode = opt.mode;
    L.seed = opt.seed;
    L.env_mode = opt.env_mode;
    for (int k = 0; k < 3; ++k) L.env[k] = opt.env_color[k];
    L.accum = d_accum;
    L.samples = d_samples;
    L.refill = opt.refill;

    static int g_ext = 0, g_sh = 0, g_shade[5] = {0, 0, 0, 0, 0}, g_simple = 0;
    static int g_sm = -1;
    if (g_sm != sm_count) {
        g_ext = occupancy_blocks((const void*)k_extend, sm_count);
        g_sh = occupancy_blocks((const void*)k_shadow, sm_count);
        g_shade[1] = occupancy_blocks((const void*)k_shade<1>, sm_count);
        g_shade[2] = occupancy_blocks((const void*)k_shade<2>, sm_count);
        g_shade[3] = occupancy_blocks((const void*)k_shade<3>, sm_count);
        g_shade[4] = occupancy_blocks((const void*)k_shade<4>, sm_count);
        g_simple = occupancy_blocks((const void*)k_finish, sm_count);
        g_sm = sm_count;
    }
    const int simple_blocks = (int)std::min<uint64_t>((P + kBlock - 1) / kBlock, (uint64_t)g_simple);
    uint32_t* cnt = L.ps.counters;
    check_cuda(cudaMemsetAsync(cnt, 0, kNumCounters * sizeof(uint32_t), st), "cudaMemsetAsync counters");
    if (opt.megakernel) {
        static int g_mega = 0, g_mega_sm = -1;
        if (g_mega_sm != sm_count) {
            g_mega = occupancy_blocks((const void*)k_megakernel, sm_count);
            g_mega_sm = sm_count;
        }
        const int blocks = (int)std::min<uint64_t>((P + kBlock - 1) / kBlock, (uint64_t)g_mega);
        k_megakernel<<<blocks, kBlock, 0, st>>>(L);
    }
    for (uint32_t smp = 0; smp < (opt.megakernel ? 0u : pc.samplesPerPixel); ++smp) {
        L.sample = smp;
        k_init<<<simple_blocks, kBlock, 0, st>>>(L);
        int cur = 0;
        for (uint32_t seg = 0; seg < pc.maxBounces; ++seg) {
            // next active queue and the shade / shadow queues start empty
            check_cuda(cudaMemsetAsync(cnt + kCntActive + (cur ^ 1), 0, sizeof(uint32_t), st), "cudaMemsetAsync");
            check_cuda(cudaMemsetAsync(cnt + kCntQueue, 0, 6 * sizeof(uint32_t), st), "cudaMemsetAsync");
            check_cuda(cudaMemsetAsync(cnt + kCntFetchExtend, 0, 2 * sizeof(uint32_t), st), "cudaMemsetAsync");
            if (opt.refill > 0) k_extend<<<g_ext, kBlock, 0, st>>>(L, cur);
            else k_extend_grid<<<g_ext, kBlock, 0, st>>>(L, cur);
            k_shade_miss<<<simple_blocks, kBlock, 0, st>>>(L);
            k_shade<1><<<g_shade[1], kBlock, 0, st>>>(L, cur);
            k_shade<2><<<g_shade[2], kBlock, 0, st>>>(L, cur);
            k_shade<3><<<g_shade[3], kBlock, 0, st>>>(L, cur);
            k_shade<4><<<g_shade[4], kBlock, 0, st>>>(L, cur);
            if (opt.mode == kModeNeeMis) {
                if (opt.refill > 0) k_shadow<<<g_sh, kBlock, 0, st>>>(L);
                else k_shadow_grid<<<g_sh, kBlock, 0, st>>>(L);
            }
            cur ^= 1;
        }
        k_finish<<<simple_blocks, kBlock, 0, st>>>(L);
    }
    if (!opt.megakernel) k_resolve<<<simple_blocks, kBlock, 0, st>>>(L);
    check_cuda(cudaGetLastError(), "render launch");
    if (stats) {
        uint32_t c[kNumCounters];
        check_cuda(cudaMemcpyAsync(c, cnt, sizeof(c), cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync counters");
        check_cuda(cudaStreamSynchronize(st), "cudaStreamSynchronize");
        uint64_t rays, srays;
        std::memcpy(&rays, c + kCntRays, 8);
        std::memcpy(&srays, c + kCntShadowRays, 8);
        stats->rays = rays;
        stats->shadow_rays = srays;
        stats->error = c[kCntError];
    }
}

void render_frame(RenderWorkspace& ws, const DeviceScene& s, const RtPushConsts& pc, const RenderOpts& opt,
                  float* d_accum, float* d_samples, int sm_count, cudaStream_t st, RenderStats* stats) {
    const uint32_t P = opt.width * opt.height;
    if (P == 0) return;
    ws.ensure(P);
    launch_frame(ws.view(), s, pc, opt, d_accum, d_samples, sm_count, st, stats);
}

// ------------------------------------------------------------------------------------------------
// Allocation-free variant (reina_render_device_noalloc): the path state and queues live in this
// file-scope device array instead of a cudaMalloc'd workspace.  Every GPU that loads the library holds
// it (path_state_words(kNoAllocMaxPixels) words = 11.3 MB) until the process exits.  All calls share
// it: the launch sequence clears what must start at zero (the queue counters, the per-pixel sums at
// sample 0), and calls whose work overlaps on the GPU race on it.
static __device__ __align__(256) uint32_t g_noalloc_scratch[kNoAllocMaxPixels * kWordsPerPath + kHeaderWords];

static std::mutex g_noalloc_mutex;
static uint32_t* g_noalloc_addr[kNoAllocMaxDevices] = {};

// Device address of the array on `device` (which must be current).  Host code only sees a host-side
// stand-in under the array's name, so the address is looked up once per device, on that device's first
// call, and cached.
static uint32_t* noalloc_scratch(int device) {
    if (device < 0 || device >= kNoAllocMaxDevices) fail(REINA_ERR_INVALID, "device ordinal out of range for the allocation-free render");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_addr[device]) {
        void* p = nullptr;
        check_cuda(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress(allocation-free render scratch)");
        g_noalloc_addr[device] = static_cast<uint32_t*>(p);
    }
    return g_noalloc_addr[device];
}

void render_frame_noalloc(int device, const DeviceScene& s, const RtPushConsts& pc, const RenderOpts& opt,
                          float* d_accum, float* d_samples, int sm_count, cudaStream_t st) {
    const uint64_t P = (uint64_t)opt.width * opt.height;
    if (P > kNoAllocMaxPixels)
        fail(REINA_ERR_INVALID, "allocation-free render is limited to " + std::to_string(kNoAllocMaxPixels) +
                                    " pixels (e.g. 256x256); got " + std::to_string(opt.width) + "x" + std::to_string(opt.height));
    if (P == 0) return;
    uint32_t* base = noalloc_scratch(device);
    launch_frame(layout_path_state(base, P), s, pc, opt, d_accum, d_samples, sm_count, st, nullptr);
}

}  // namespace rt
