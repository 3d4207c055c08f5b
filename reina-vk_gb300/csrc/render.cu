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
#include <map>
#include <mutex>
#include <tuple>
#include <string>

#include "kernels.h"
#include "render.h"
#include "coop_trace.cuh"
#include "shading_device.cuh"
#include "trace_device.cuh"
#include "wavefront_device.cuh"

namespace rt {

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
        V3 o, d;
        camera_ray(L.pc, L.W, L.H, x, y, rng, o, d);
        store_ray(ps, i, o, d);
        store_thr(ps, i, V3{1.0f, 1.0f, 1.0f});
        store_rad(ps, i, V3{0.0f, 0.0f, 0.0f});
        ps.rng[i] = rng;
        ps.acc[i] = acc;
        ps.flags[i] = 0u;
        ps.ppdf[i] = 0.0f;
        ps.q_active[0][checked_index(i, L.P, ps.counters + kCntError)] = i;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) ps.counters[kCntActive] = L.P;
}

// ------------------------------------------------------------------------------------------------
// extend: closest hit + classification.  Grid form: each warp takes 32 consecutive queue entries.
template <int BLOCK, int SS, bool TWO>
__global__ void __launch_bounds__(BLOCK) k_extend_grid(RenderLaunch L, int cur) {
    __shared__ uint2 stack[SS * BLOCK];
    const PathState& ps = L.ps;
    const uint32_t n = ps.counters[kCntActive + cur];
    const uint32_t* q = ps.q_active[cur];
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const bool active = i < n;
        int m = -1;
        uint32_t p = 0;
        if (active) {
            p = checked_index(q[i], L.P, ps.counters + kCntError);
            const TraceRay r = make_trace_ray(ps.ox[p], ps.oy[p], ps.oz[p], ps.dx[p], ps.dy[p], ps.dz[p], 0.0f, 10000.0f);
            Hit h;
            TraceCounters c{0u, 0u};
            uint32_t e = 0;
            if (L.s.node_count)
                e = trace_scene<false, false, true, SS, TWO>(L.s, r, stack + threadIdx.x, BLOCK, h, c);
            else h.prim = kMiss;
            if (e) atomicOr(ps.counters + kCntError, e);
            ps.hprim[p] = h.prim;
            ps.hu[p] = h.u;
            ps.hv[p] = h.v;
            m = h.prim == kMiss ? kQueueMiss : 1 + (int)L.s.props_material[prim_props_of(L.s, h.prim)];
        }
        warp_count64(reinterpret_cast<unsigned long long*>(ps.counters + kCntRays), active);
#pragma unroll
        for (int k = 0; k < kNumQueues; ++k) {
            const bool mine = active && m == k;
            const uint32_t pos = warp_append(ps.counters + kCntQueue + k, mine);
            if (mine) ps.q_shade[(size_t)k * L.P + checked_index(pos, L.P, ps.counters + kCntError)] = p;
        }
    }
}

// Cooperative persistent form (coop_trace.cuh): warps refill idle lanes from the queue; triangle tests
// and hit refinement are spread over the warp.  Flat scenes.
__global__ void __launch_bounds__(kBlock, kCoopMinBlocks) k_extend(RenderLaunch L, int cur) {
    __shared__ CoopWarp warps[kBlock / 32];
    __shared__ uint2 stack[kSmemStack * kBlock];
    const PathState& ps = L.ps;
    const uint32_t n = ps.counters[kCntActive + cur];
    const uint32_t* q = ps.q_active[cur];
    TraceCounters c{0u, 0u};
    auto load = [&](uint32_t i, TraceRay& r, CoopScene& sc) {
        const uint32_t p = checked_index(q[i], L.P, ps.counters + kCntError);
        r = make_trace_ray(ps.ox[p], ps.oy[p], ps.oz[p], ps.dx[p], ps.dy[p], ps.dz[p], 0.0f, 10000.0f);
        (void)sc;
        return true;
    };
    auto store = [&](uint32_t i, const Hit& h, bool valid) {   // called by all 32 lanes
        int m = -1;
        uint32_t p = 0;
        if (valid) {
            p = checked_index(q[i], L.P, ps.counters + kCntError);
            ps.hprim[p] = h.prim;
            ps.hu[p] = h.u;
            ps.hv[p] = h.v;
            m = h.prim == kMiss ? kQueueMiss : 1 + (int)L.s.props_material[prim_props_of(L.s, h.prim)];
        }
        warp_count64(reinterpret_cast<unsigned long long*>(ps.counters + kCntRays), valid);
        warp_count64(reinterpret_cast<unsigned long long*>(ps.counters + kCntShaded), valid && m != kQueueMiss);
#pragma unroll
        for (int k = 0; k < kNumQueues; ++k) {
            const bool mine = valid && m == k;
            const uint32_t pos = warp_append(ps.counters + kCntQueue + k, mine);
            if (mine) ps.q_shade[(size_t)k * L.P + checked_index(pos, L.P, ps.counters + kCntError)] = p;
        }
    };
    const uint32_t e = coop_trace<false, true, true, false, kSmemStack>(CoopScene{L.s.nodes, L.s.tris, L.s.node_count}, n,
                                                                        ps.counters + kCntFetchExtend, (uint32_t)(32 - L.refill),
                                                                 warps[threadIdx.x >> 5], stack + threadIdx.x, kBlock,
                                                                 load, store, c);
    if (e) atomicOr(ps.counters + kCntError, e);
    coop_add_counts(c, ps.counters, kCntNodes, kCntTris);
}

// One kernel per material queue (MAT = 1 Lambertian, 2 metal, 3 dielectric, 4 Disney): the closest-hit
// shader, then the raygen loop body (raytrace.rgen.glsl:124-180).
template <int MAT>
__global__ void __launch_bounds__(kBlock, kShadeMinBlocks) k_shade(RenderLaunch L, int cur) {
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
            p = checked_index(q[i], L.P, ps.counters + kCntError);
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
            if (MAT == 1) vx = shade_lambert(L.s, h, pr, rd, rng, inside, acc);
            else if (MAT == 2) vx = shade_metal(L.s, h, pr, rd, rng, inside, acc);
            else if (MAT == 3) vx = shade_dielectric(L.s, h, pr, ro, rd, rng, inside, acc);
            else vx = shade_disney(L.s, h, pr, ro, rd, rng, inside, acc);
            if (vx.skip) {
                flags &= ~kFlagPrevNee;
            } else {
                flags = vx.inside ? (flags | kFlagInside) : (flags & ~kFlagInside);
                if (!vx.inside) {
                    V3 thr = load_thr(ps, p), rad = load_rad(ps, p);
                    V3 contrib = vx.emission;
                    if (nee) {
                        if ((flags & kFlagPrevNee) && (vx.emission.x != 0.0f || vx.emission.y != 0.0f || vx.emission.z != 0.0f))
                            contrib = contrib * power_heuristic(ps.ppdf[p], light_pdf_sa(L.s, L.pc.totalEmissiveWeight, prim, ro, vx.newO));
                        const bool do_nee = (MAT == 1 || MAT == 4) && L.s.emissive_count > 0;
                        if (do_nee) emit = next_event(L.s, L.pc.totalEmissiveWeight, rng, MAT == 4, vx.newO, vx.n, vx.albedo, pr, h.tbn, rd, thr, sh);
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
        if (active) ps.q_active[cur ^ 1][checked_index(pos, L.P, ps.counters + kCntError)] = p;
        const uint32_t spos = warp_append(ps.counters + kCntShadow, emit);
        if (emit) {
            const uint32_t sp_ = checked_index(spos, L.P, ps.counters + kCntError);
            ps.q_shadow[sp_] = p;
            ps.s_ox[sp_] = sh.o.x; ps.s_oy[sp_] = sh.o.y; ps.s_oz[sp_] = sh.o.z;
            ps.s_dx[sp_] = sh.d.x; ps.s_dy[sp_] = sh.d.y; ps.s_dz[sp_] = sh.d.z;
            ps.s_tmax[sp_] = sh.tmax;
            ps.s_cr[sp_] = sh.contrib.x; ps.s_cg[sp_] = sh.contrib.y; ps.s_cb[sp_] = sh.contrib.z;
        }
    }
}

// raytrace.rmiss.glsl:10-19: the path ends with sky (or constant environment) radiance.
__global__ void __launch_bounds__(kBlock) k_shade_miss(RenderLaunch L) {
    const PathState& ps = L.ps;
    const uint32_t n = ps.counters[kCntQueue + kQueueMiss];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t p = checked_index(ps.q_shade[i], L.P, ps.counters + kCntError);
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
template <int BLOCK, int SS, bool TWO>
__global__ void __launch_bounds__(BLOCK) k_shadow_grid(RenderLaunch L) {
    __shared__ uint2 stack[SS * BLOCK];
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
            if (L.s.node_count)
                e = trace_scene<true, false, false, SS, TWO>(L.s, r, stack + threadIdx.x, BLOCK, h, c);
            else h.prim = kMiss;
            if (e) atomicOr(ps.counters + kCntError, e);
            if (h.prim == kMiss) {
                const uint32_t p = checked_index(ps.q_shadow[i], L.P, ps.counters + kCntError);
                store_rad(ps, p, load_rad(ps, p) + V3{ps.s_cr[i], ps.s_cg[i], ps.s_cb[i]});
            }
        }
        warp_count64(reinterpret_cast<unsigned long long*>(ps.counters + kCntShadowRays), active);
    }
}

// Cooperative persistent form of the shadow kernel (flat scenes).
__global__ void __launch_bounds__(kBlock, kCoopMinBlocks) k_shadow(RenderLaunch L) {
    __shared__ CoopWarp warps[kBlock / 32];
    __shared__ uint2 stack[kSmemStack * kBlock];
    const PathState& ps = L.ps;
    const uint32_t n = ps.counters[kCntShadow];
    TraceCounters c{0u, 0u};
    auto load = [&](uint32_t i, TraceRay& r, CoopScene& sc) {
        r = make_trace_ray(ps.s_ox[i], ps.s_oy[i], ps.s_oz[i], ps.s_dx[i], ps.s_dy[i], ps.s_dz[i], 0.0f, ps.s_tmax[i]);
        (void)sc;
        return true;
    };
    auto store = [&](uint32_t i, const Hit& h, bool valid) {   // called by all 32 lanes
        if (valid && h.prim == kMiss) {
            const uint32_t p = checked_index(ps.q_shadow[i], L.P, ps.counters + kCntError);
            store_rad(ps, p, load_rad(ps, p) + V3{ps.s_cr[i], ps.s_cg[i], ps.s_cb[i]});
        }
        warp_count64(reinterpret_cast<unsigned long long*>(ps.counters + kCntShadowRays), valid);
    };
    const uint32_t e = coop_trace<true, true, false, false, kSmemStack>(CoopScene{L.s.nodes, L.s.tris, L.s.node_count}, n,
                                                                        ps.counters + kCntFetchShadow, (uint32_t)(32 - L.refill),
                                                                 warps[threadIdx.x >> 5], stack + threadIdx.x, kBlock,
                                                                 load, store, c);
    if (e) atomicOr(ps.counters + kCntError, e);
    coop_add_counts(c, ps.counters, kCntShadowNodes, kCntShadowTris);
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
template <bool TWO>
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
            V3 ro, rd;
            camera_ray(L.pc, L.W, L.H, x, y, rng, ro, rd);
            // traceSegments
            V3 thr{1.0f, 1.0f, 1.0f}, rad{0.0f, 0.0f, 0.0f};
            bool inside = false, prev_nee = false;
            float ppdf = 0.0f;
            for (uint32_t seg = 0; seg < L.pc.maxBounces; ++seg) {
                const TraceRay r = make_trace_ray(ro.x, ro.y, ro.z, rd.x, rd.y, rd.z, 0.0f, 10000.0f);
                Hit h;
                TraceCounters c{0u, 0u};
                uint32_t e = 0;
                if (L.s.node_count) e = trace_scene<false, false, true, kSmemStack, TWO>(L.s, r, stack + threadIdx.x, kBlock, h, c);
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
                if (mat == 0) vx = shade_lambert(L.s, hi, pr, rd, rng, inside, acc);
                else if (mat == 1) vx = shade_metal(L.s, hi, pr, rd, rng, inside, acc);
                else if (mat == 2) vx = shade_dielectric(L.s, hi, pr, ro, rd, rng, inside, acc);
                else vx = shade_disney(L.s, hi, pr, ro, rd, rng, inside, acc);
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
                            contrib = contrib * power_heuristic(ppdf, light_pdf_sa(L.s, L.pc.totalEmissiveWeight, h.prim, ray_org, vx.newO));
                        const bool do_nee = (mat == 0 || mat == 3) && L.s.emissive_count > 0;
                        if (do_nee) {
                            ShadowRec sh;
                            if (next_event(L.s, L.pc.totalEmissiveWeight, rng, mat == 3, vx.newO, vx.n, vx.albedo, pr, hi.tbn, ray_in, thr, sh)) {
                                const TraceRay sr = make_trace_ray(sh.o.x, sh.o.y, sh.o.z, sh.d.x, sh.d.y, sh.d.z, 0.0f, sh.tmax);
                                Hit sh_hit;
                                uint32_t e2 = 0;
                                e2 = trace_scene<true, false, false, kSmemStack, TWO>(L.s, sr, stack + threadIdx.x, kBlock, sh_hit, c);
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

// Resident grid (blocks per SM x SMs) of a kernel at a block size, computed once per (kernel, block size,
// SM count) and kept in a table that any thread rendering may read or fill (under a lock).
static int cached_grid(const void* fn, int block, int sm_count) {
    static std::mutex mu;
    static std::map<std::tuple<const void*, int, int>, int> table;
    const auto key = std::make_tuple(fn, block, sm_count);
    {
        std::lock_guard<std::mutex> lock(mu);
        const auto it = table.find(key);
        if (it != table.end()) return it->second;
    }
    const int g = resident_grid(fn, block, sm_count);
    std::lock_guard<std::mutex> lock(mu);
    table[key] = g;
    return g;
}

static int occupancy_blocks(const void* fn, int sm_count) { return cached_grid(fn, kBlock, sm_count); }

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
    L.refill = opt.trace.refill;

    const int g_ext = occupancy_blocks((const void*)k_extend, sm_count);
    const int g_sh = occupancy_blocks((const void*)k_shadow, sm_count);
    const int g_shade[5] = {0, occupancy_blocks((const void*)k_shade<1>, sm_count),
                            occupancy_blocks((const void*)k_shade<2>, sm_count),
                            occupancy_blocks((const void*)k_shade<3>, sm_count),
                            occupancy_blocks((const void*)k_shade<4>, sm_count)};
    const int g_simple = occupancy_blocks((const void*)k_finish, sm_count);
    const int simple_blocks = (int)std::min<uint64_t>((P + kBlock - 1) / kBlock, (uint64_t)g_simple);
    uint32_t* cnt = L.ps.counters;
    check_cuda(cudaMemsetAsync(cnt, 0, kNumCounters * sizeof(uint32_t), st), "cudaMemsetAsync counters");
    const bool two = L.s.inst_trav != nullptr;
    if (opt.megakernel) {
        const int g_mega[2] = {occupancy_blocks((const void*)k_megakernel<false>, sm_count),
                               occupancy_blocks((const void*)k_megakernel<true>, sm_count)};
        const int blocks = (int)std::min<uint64_t>((P + kBlock - 1) / kBlock, (uint64_t)g_mega[two ? 1 : 0]);
        if (two) k_megakernel<true><<<blocks, kBlock, 0, st>>>(L);
        else k_megakernel<false><<<blocks, kBlock, 0, st>>>(L);
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
            if (two) {   // two-level scenes: the default traversal variant
                const int grid = cached_grid((const void*)k_extend_grid<kTraceBlock, kDefaultTraceStack, true>, kTraceBlock, sm_count);
                k_extend_grid<kTraceBlock, kDefaultTraceStack, true><<<grid, kTraceBlock, 0, st>>>(L, cur);
            } else if (opt.trace.refill > 0) {
                k_extend<<<g_ext, kBlock, 0, st>>>(L, cur);
            } else {
                with_trace_variant(opt.trace, [&](auto B, auto S) {
                    const int grid = cached_grid((const void*)k_extend_grid<B.value, S.value, false>, B.value, sm_count);
                    k_extend_grid<B.value, S.value, false><<<grid, B.value, 0, st>>>(L, cur);
                });
            }
            k_shade_miss<<<simple_blocks, kBlock, 0, st>>>(L);
            k_shade<1><<<g_shade[1], kBlock, 0, st>>>(L, cur);
            k_shade<2><<<g_shade[2], kBlock, 0, st>>>(L, cur);
            k_shade<3><<<g_shade[3], kBlock, 0, st>>>(L, cur);
            k_shade<4><<<g_shade[4], kBlock, 0, st>>>(L, cur);
            if (opt.mode == kModeNeeMis) {
                if (two) {
                    const int grid = cached_grid((const void*)k_shadow_grid<kTraceBlock, kDefaultTraceStack, true>, kTraceBlock, sm_count);
                    k_shadow_grid<kTraceBlock, kDefaultTraceStack, true><<<grid, kTraceBlock, 0, st>>>(L);
                } else if (opt.trace.refill > 0) {
                    k_shadow<<<g_sh, kBlock, 0, st>>>(L);
                } else {
                    with_trace_variant(opt.trace, [&](auto B, auto S) {
                        const int grid = cached_grid((const void*)k_shadow_grid<B.value, S.value, false>, B.value, sm_count);
                        k_shadow_grid<B.value, S.value, false><<<grid, B.value, 0, st>>>(L);
                    });
                }
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
        auto u64 = [&](int at) { uint64_t v; std::memcpy(&v, c + at, 8); return v; };
        stats->rays = u64(kCntRays);
        stats->shadow_rays = u64(kCntShadowRays);
        stats->nodes = u64(kCntNodes);
        stats->tris = u64(kCntTris);
        stats->shadow_nodes = u64(kCntShadowNodes);
        stats->shadow_tris = u64(kCntShadowTris);
        stats->shaded = u64(kCntShaded);
        stats->error = c[kCntError];
    }
}

// ORs a frame's error word into the caller's error word (one thread; enqueued after the frame).
__global__ void k_or_error(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst) {
    if (threadIdx.x == 0 && *src) atomicOr(dst, *src);
}

void render_frame(RenderWorkspace& ws, const DeviceScene& s, const RtPushConsts& pc, const RenderOpts& opt,
                  float* d_accum, float* d_samples, int sm_count, cudaStream_t st, RenderStats* stats,
                  uint32_t* err_accum) {
    const uint32_t P = opt.width * opt.height;
    if (P == 0) return;
    ws.ensure(P);
    launch_frame(ws.view(), s, pc, opt, d_accum, d_samples, sm_count, st, stats);
    if (err_accum) {
        k_or_error<<<1, 32, 0, st>>>(ws.view().counters + kCntError, err_accum);
        check_cuda(cudaGetLastError(), "error word launch");
    }
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
                          float* d_accum, float* d_samples, int sm_count, cudaStream_t st, uint32_t* err_accum) {
    const uint64_t P = (uint64_t)opt.width * opt.height;
    if (P > kNoAllocMaxPixels)
        fail(REINA_ERR_INVALID, "allocation-free render is limited to " + std::to_string(kNoAllocMaxPixels) +
                                    " pixels (e.g. 256x256); got " + std::to_string(opt.width) + "x" + std::to_string(opt.height));
    if (P == 0) return;
    uint32_t* base = noalloc_scratch(device);
    const PathState ps = layout_path_state(base, P);
    launch_frame(ps, s, pc, opt, d_accum, d_samples, sm_count, st, nullptr);
    if (err_accum) {
        k_or_error<<<1, 32, 0, st>>>(ps.counters + kCntError, err_accum);
        check_cuda(cudaGetLastError(), "error word launch");
    }
}

}  // namespace rt
