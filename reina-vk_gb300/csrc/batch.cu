// Multi-job wavefront engine.  A wave is a set of path slots, each one (job, pixel, sample); it runs the
// same kernel sequence as the single-frame wavefront (init, extend, per-material shade, shadow, finish),
// with every kernel reading its path's job record for the scene, camera and integrator options.  A job
// contributes at most one sample per pixel to a wave and its samples are scheduled in order, so each
// pixel's samples are summed in sample order: a job's image does not depend on the jobs it shares waves
// with.  The per-wave launch sequence is captured once per (bounces, NEE) into a CUDA
// graph and replayed; only the wave descriptor (segments + job table) is copied in before each wave.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "batch.h"
#include "coop_trace.cuh"
#include "trace_device.cuh"
#include "wavefront_device.cuh"

namespace rt {

struct BatchPaths {
    PathState ps;      // per-slot path state and queues (its per-pixel arrays are unused here)
    uint32_t* job;     // per slot: index into the wave's job table
    uint32_t* pix;     // per slot: pixel within its job
    uint32_t* smp;     // per slot: sample index
    uint32_t* depth;   // per slot: segments traced
};

struct BatchLaunch {
    BatchPaths bp;
    const WaveHeader* hdr;
    const WaveSeg* segs;
    const JobGpu* jobs;
    uint32_t P;
};

// Sets up slot i (job, pixel, sample, camera ray — raytrace.rgen.glsl:250-263); returns whether its job
// traces any segment (paths of jobs with maxBounces = 0 finish with zero radiance).
__device__ __forceinline__ bool init_slot(const BatchLaunch& B, const JobGpu* __restrict__ jobs, uint32_t i) {
    const PathState& ps = B.bp.ps;
    int lo = 0, hi = (int)B.hdr->nseg - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) / 2;
        if (B.segs[mid].wave_start <= i) lo = mid;
        else hi = mid - 1;
    }
    const WaveSeg sg = B.segs[lo];
    const JobGpu& J = jobs[sg.job];
    const uint32_t pixel = sg.pixel_start + (i - sg.wave_start);
    const uint32_t k = sg.sample;
    const uint32_t x = pixel % J.W, y = pixel / J.W;
    uint32_t rng;
    float acc;
    if (J.mode == kModeNeeMis) {
        rng = path_seed(pixel, J.pc.sampleBatch * J.spp + k, J.seed);
        acc = 0.0f;
    } else if (k == 0) {
        rng = (J.pc.sampleBatch * J.H + y) * J.W + x;
        acc = 0.0f;
    } else {
        rng = J.pix_rng[pixel];
        acc = J.pix_acc[pixel];
    }
    if (k == 0) {
        J.sr[pixel] = 0.0f; J.sg[pixel] = 0.0f; J.sb[pixel] = 0.0f;
        J.cnt[pixel] = 0;
    }
    V3 o, d;
    camera_ray(J.pc, J.W, J.H, x, y, rng, o, d);
    store_ray(ps, i, o, d);
    store_thr(ps, i, V3{1.0f, 1.0f, 1.0f});
    store_rad(ps, i, V3{0.0f, 0.0f, 0.0f});
    ps.rng[i] = rng;
    ps.acc[i] = acc;
    ps.flags[i] = 0u;
    ps.ppdf[i] = 0.0f;
    B.bp.job[i] = sg.job;
    B.bp.pix[i] = pixel;
    B.bp.smp[i] = k;
    B.bp.depth[i] = 0;
    return J.max_bounces > 0;
}

// The active-path counter is zero at launch (cleared with the other counters before the wave).
__global__ void __launch_bounds__(kBlock) kb_init(BatchLaunch B, const JobGpu* __restrict__ jobs) {
    const PathState& ps = B.bp.ps;
    const uint32_t n = B.hdr->count;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const bool live = i < n && init_slot(B, jobs, i);
        const uint32_t pos = warp_append(ps.counters + kCntActive, live);
        if (live) ps.q_active[0][checked_index(pos, B.P, ps.counters + kCntError)] = i;
    }
}

// COUNT: the traversal work (nodes visited, triangles tested) is added to the wave's counters.
template <int BLOCK, int SS, bool TWO, bool COUNT = false>
__global__ void __launch_bounds__(BLOCK, 1024 / BLOCK) kb_extend(BatchLaunch B, const JobGpu* __restrict__ jobs, int cur) {
    __shared__ uint2 stack[SS * BLOCK];
    const PathState& ps = B.bp.ps;
    const uint32_t n = ps.counters[kCntActive + cur];
    const uint32_t* q = ps.q_active[cur];
    TraceCounters c{0u, 0u};
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const bool active = i < n;
        int m = -1;
        uint32_t p = 0;
        if (active) {
            p = checked_index(q[i], B.P, ps.counters + kCntError);
            const DeviceScene& s = jobs[B.bp.job[p]].s;
            const TraceRay r = make_trace_ray(ps.ox[p], ps.oy[p], ps.oz[p], ps.dx[p], ps.dy[p], ps.dz[p], 0.0f, 10000.0f);
            Hit h;
            uint32_t e = 0;
            if (s.node_count) e = trace_scene<false, COUNT, true, SS, TWO>(s, r, stack + threadIdx.x, BLOCK, h, c);
            else h.prim = kMiss;
            if (e) atomicOr(ps.counters + kCntError, e);
            ps.hprim[p] = h.prim;
            ps.hu[p] = h.u;
            ps.hv[p] = h.v;
            m = h.prim == kMiss ? kQueueMiss : 1 + (int)s.props_material[prim_props_of(s, h.prim)];
        }
        warp_count64(reinterpret_cast<unsigned long long*>(ps.counters + kCntRays), active);
        if (COUNT) warp_count64(reinterpret_cast<unsigned long long*>(ps.counters + kCntShaded), active && m != kQueueMiss);
#pragma unroll
        for (int k = 0; k < kNumQueues; ++k) {
            const bool mine = active && m == k;
            const uint32_t pos = warp_append(ps.counters + kCntQueue + k, mine);
            if (mine) ps.q_shade[(size_t)k * B.P + checked_index(pos, B.P, ps.counters + kCntError)] = p;
        }
    }
    if (COUNT) coop_add_counts(c, ps.counters, kCntNodes, kCntTris);
}

// Cooperative persistent form of the extension kernel (coop_trace.cuh; waves of flat scenes): warps
// refill idle lanes from the active queue once at most `refill_at` lanes still trace; each lane's ray
// uses its own job's scene.
__global__ void __launch_bounds__(kTraceBlock, kCoopMinBlocks) kb_extend_coop(BatchLaunch B, const JobGpu* __restrict__ jobs, int cur,
                                                             uint32_t refill_at) {
    __shared__ CoopWarp warps[kTraceBlock / 32];
    __shared__ uint2 stack[kSmemStack * kTraceBlock];
    const PathState& ps = B.bp.ps;
    const uint32_t n = ps.counters[kCntActive + cur];
    const uint32_t* q = ps.q_active[cur];
    TraceCounters c{0u, 0u};
    auto load = [&](uint32_t i, TraceRay& r, CoopScene& sc) {
        const uint32_t p = checked_index(q[i], B.P, ps.counters + kCntError);
        const DeviceScene& s = jobs[B.bp.job[p]].s;
        r = make_trace_ray(ps.ox[p], ps.oy[p], ps.oz[p], ps.dx[p], ps.dy[p], ps.dz[p], 0.0f, 10000.0f);
        sc = CoopScene{s.nodes, s.tris, s.node_count};
        return true;
    };
    auto store = [&](uint32_t i, const Hit& h, bool valid) {   // called by all 32 lanes
        int m = -1;
        uint32_t p = 0;
        if (valid) {
            p = checked_index(q[i], B.P, ps.counters + kCntError);
            const DeviceScene& s = jobs[B.bp.job[p]].s;
            ps.hprim[p] = h.prim;
            ps.hu[p] = h.u;
            ps.hv[p] = h.v;
            m = h.prim == kMiss ? kQueueMiss : 1 + (int)s.props_material[prim_props_of(s, h.prim)];
        }
        warp_count64(reinterpret_cast<unsigned long long*>(ps.counters + kCntRays), valid);
        warp_count64(reinterpret_cast<unsigned long long*>(ps.counters + kCntShaded), valid && m != kQueueMiss);
#pragma unroll
        for (int k = 0; k < kNumQueues; ++k) {
            const bool mine = valid && m == k;
            const uint32_t pos = warp_append(ps.counters + kCntQueue + k, mine);
            if (mine) ps.q_shade[(size_t)k * B.P + checked_index(pos, B.P, ps.counters + kCntError)] = p;
        }
    };
    const uint32_t e = coop_trace<false, true, true, true, kSmemStack>(CoopScene{nullptr, nullptr, 0u}, n,
                                                                       ps.counters + kCntFetchExtend, refill_at,
                                                                 warps[threadIdx.x >> 5], stack + threadIdx.x,
                                                                 kTraceBlock, load, store, c);
    if (e) atomicOr(ps.counters + kCntError, e);
    coop_add_counts(c, ps.counters, kCntNodes, kCntTris);
}

template <int MAT>
__global__ void __launch_bounds__(kBlock, kShadeMinBlocks) kb_shade(BatchLaunch B, const JobGpu* __restrict__ jobs, int cur) {
    const PathState& ps = B.bp.ps;
    const uint32_t n = ps.counters[kCntQueue + MAT];
    const uint32_t* q = ps.q_shade + (size_t)MAT * B.P;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const bool active = i < n;
        bool emit = false, cont = false;
        ShadowRec sh;
        uint32_t p = 0;
        if (active) {
            p = checked_index(q[i], B.P, ps.counters + kCntError);
            const JobGpu& J = jobs[B.bp.job[p]];
            const bool nee = J.mode == kModeNeeMis;
            const V3 ro{ps.ox[p], ps.oy[p], ps.oz[p]};
            const V3 rd{ps.dx[p], ps.dy[p], ps.dz[p]};
            const uint32_t prim = ps.hprim[p];
            const HitInfo h = hit_info(J.s, prim, ps.hu[p], ps.hv[p], rd);
            const InstanceProperties& pr = J.s.props[h.props];
            uint32_t rng = ps.rng[p];
            uint32_t flags = ps.flags[p];
            float acc = ps.acc[p];
            const bool inside = (flags & kFlagInside) != 0;
            Vertex vx;
            if (MAT == 1) vx = shade_lambert(J.s, h, pr, rd, rng, inside, acc);
            else if (MAT == 2) vx = shade_metal(J.s, h, pr, rd, rng, inside, acc);
            else if (MAT == 3) vx = shade_dielectric(J.s, h, pr, ro, rd, rng, inside, acc);
            else vx = shade_disney(J.s, h, pr, ro, rd, rng, inside, acc);
            if (vx.skip) {
                flags &= ~kFlagPrevNee;
            } else {
                flags = vx.inside ? (flags | kFlagInside) : (flags & ~kFlagInside);
                if (!vx.inside) {
                    V3 thr = load_thr(ps, p), rad = load_rad(ps, p);
                    V3 contrib = vx.emission;
                    if (nee) {
                        const float tw = J.pc.totalEmissiveWeight;
                        if ((flags & kFlagPrevNee) && (vx.emission.x != 0.0f || vx.emission.y != 0.0f || vx.emission.z != 0.0f))
                            contrib = contrib * power_heuristic(ps.ppdf[p], light_pdf_sa(J.s, tw, prim, ro, vx.newO));
                        const bool do_nee = (MAT == 1 || MAT == 4) && J.s.emissive_count > 0;
                        if (do_nee) emit = next_event(J.s, tw, rng, MAT == 4, vx.newO, vx.n, vx.albedo, pr, h.tbn, rd, thr, sh);
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
            const uint32_t dep = B.bp.depth[p] + 1;
            B.bp.depth[p] = dep;
            cont = dep < J.max_bounces;
        }
        const uint32_t pos = warp_append(ps.counters + kCntActive + (cur ^ 1), cont);
        if (cont) ps.q_active[cur ^ 1][checked_index(pos, B.P, ps.counters + kCntError)] = p;
        const uint32_t spos = warp_append(ps.counters + kCntShadow, emit);
        if (emit) {
            const uint32_t sp_ = checked_index(spos, B.P, ps.counters + kCntError);
            ps.q_shadow[sp_] = p;
            ps.s_ox[sp_] = sh.o.x; ps.s_oy[sp_] = sh.o.y; ps.s_oz[sp_] = sh.o.z;
            ps.s_dx[sp_] = sh.d.x; ps.s_dy[sp_] = sh.d.y; ps.s_dz[sp_] = sh.d.z;
            ps.s_tmax[sp_] = sh.tmax;
            ps.s_cr[sp_] = sh.contrib.x; ps.s_cg[sp_] = sh.contrib.y; ps.s_cb[sp_] = sh.contrib.z;
        }
    }
}

__global__ void __launch_bounds__(kBlock) kb_shade_miss(BatchLaunch B, const JobGpu* __restrict__ jobs) {
    const PathState& ps = B.bp.ps;
    const uint32_t n = ps.counters[kCntQueue + kQueueMiss];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t p = checked_index(ps.q_shade[i], B.P, ps.counters + kCntError);
        const JobGpu& J = jobs[B.bp.job[p]];
        V3 sky;
        if (J.env_mode == 1) {
            sky = V3{J.env[0], J.env[1], J.env[2]};
        } else {
            const float y = norm3(V3{ps.dx[p], ps.dy[p], ps.dz[p]}).y;
            const float t = 0.5f * (y + 1.0f);
            sky = mix3(V3{0.1f, 0.1f, 0.1f}, V3{0.4f, 1.7f, 2.0f}, t) * 0.07f;
        }
        store_rad(ps, p, load_rad(ps, p) + sky * load_thr(ps, p));
    }
}

template <int BLOCK, int SS, bool TWO, bool COUNT = false>
__global__ void __launch_bounds__(BLOCK) kb_shadow(BatchLaunch B, const JobGpu* __restrict__ jobs) {
    __shared__ uint2 stack[SS * BLOCK];
    const PathState& ps = B.bp.ps;
    const uint32_t n = ps.counters[kCntShadow];
    TraceCounters c{0u, 0u};
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const bool active = i < n;
        if (active) {
            const uint32_t p = checked_index(ps.q_shadow[i], B.P, ps.counters + kCntError);
            const DeviceScene& s = jobs[B.bp.job[p]].s;
            const TraceRay r = make_trace_ray(ps.s_ox[i], ps.s_oy[i], ps.s_oz[i], ps.s_dx[i], ps.s_dy[i], ps.s_dz[i], 0.0f,
                                              ps.s_tmax[i]);
            Hit h;
            uint32_t e = 0;
            if (s.node_count) e = trace_scene<true, COUNT, false, SS, TWO>(s, r, stack + threadIdx.x, BLOCK, h, c);
            else h.prim = kMiss;
            if (e) atomicOr(ps.counters + kCntError, e);
            if (h.prim == kMiss) store_rad(ps, p, load_rad(ps, p) + V3{ps.s_cr[i], ps.s_cg[i], ps.s_cb[i]});
        }
        warp_count64(reinterpret_cast<unsigned long long*>(ps.counters + kCntShadowRays), active);
    }
    if (COUNT) coop_add_counts(c, ps.counters, kCntShadowNodes, kCntShadowTris);
}

// Cooperative persistent form of the shadow kernel (waves of flat scenes).
__global__ void __launch_bounds__(kTraceBlock, kCoopMinBlocks) kb_shadow_coop(BatchLaunch B, const JobGpu* __restrict__ jobs,
                                                             uint32_t refill_at) {
    __shared__ CoopWarp warps[kTraceBlock / 32];
    __shared__ uint2 stack[kSmemStack * kTraceBlock];
    const PathState& ps = B.bp.ps;
    const uint32_t n = ps.counters[kCntShadow];
    TraceCounters c{0u, 0u};
    auto load = [&](uint32_t i, TraceRay& r, CoopScene& sc) {
        const uint32_t p = checked_index(ps.q_shadow[i], B.P, ps.counters + kCntError);
        const DeviceScene& s = jobs[B.bp.job[p]].s;
        r = make_trace_ray(ps.s_ox[i], ps.s_oy[i], ps.s_oz[i], ps.s_dx[i], ps.s_dy[i], ps.s_dz[i], 0.0f, ps.s_tmax[i]);
        sc = CoopScene{s.nodes, s.tris, s.node_count};
        return true;
    };
    auto store = [&](uint32_t i, const Hit& h, bool valid) {   // called by all 32 lanes
        if (valid && h.prim == kMiss) {
            const uint32_t p = checked_index(ps.q_shadow[i], B.P, ps.counters + kCntError);
            store_rad(ps, p, load_rad(ps, p) + V3{ps.s_cr[i], ps.s_cg[i], ps.s_cb[i]});
        }
        warp_count64(reinterpret_cast<unsigned long long*>(ps.counters + kCntShadowRays), valid);
    };
    const uint32_t e = coop_trace<true, true, false, true, kSmemStack>(CoopScene{nullptr, nullptr, 0u}, n,
                                                                       ps.counters + kCntFetchShadow, refill_at,
                                                                 warps[threadIdx.x >> 5], stack + threadIdx.x,
                                                                 kTraceBlock, load, store, c);
    if (e) atomicOr(ps.counters + kCntError, e);
    coop_add_counts(c, ps.counters, kCntShadowNodes, kCntShadowTris);
}

// raytrace.rgen.glsl:264-275 per pixel of each job in the wave: clamp (NaN kept), sample output, NaN
// drop, sum — over the pixel's samples in this wave in sample order (a job whose samples are independent
// may have several samples of a pixel in one wave) — and carry the RNG state and accumulatedDistance of
// the last one to the pixel's next sample.
__global__ void __launch_bounds__(kBlock) kb_finish(BatchLaunch B, const JobGpu* __restrict__ jobs) {
    const PathState& ps = B.bp.ps;
    const uint32_t n = B.hdr->finish_total;
    const int nj = (int)B.hdr->njobs;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int lo = 0, hi = nj - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) / 2;
            if (jobs[mid].finish_start <= i) lo = mid;
            else hi = mid - 1;
        }
        const JobGpu& J = jobs[lo];
        const uint64_t px = (uint64_t)J.W * J.H;
        const uint64_t first = J.cursor0 + (i - J.finish_start), end = J.cursor0 + J.take;
        const uint32_t pixel = (uint32_t)(first % px);
        float sr = J.sr[pixel], sg = J.sg[pixel], sb = J.sb[pixel];
        uint32_t cnt = J.cnt[pixel];
        uint32_t slot = 0;
        for (uint64_t idx = first; idx < end; idx += px) {
            slot = J.wave_start + (uint32_t)(idx - J.cursor0);
            const V3 c = clamp_keep_nan(load_rad(ps, slot), J.pc.directClamp);
            if (J.samples) {
                float* o = J.samples + 3ull * ((uint64_t)pixel * J.spp + idx / px);
                o[0] = c.x; o[1] = c.y; o[2] = c.z;
            }
            if (!has_nan3(c)) {
                sr += c.x;
                sg += c.y;
                sb += c.z;
                cnt += 1;
            }
        }
        J.sr[pixel] = sr; J.sg[pixel] = sg; J.sb[pixel] = sb;
        J.cnt[pixel] = cnt;
        J.pix_rng[pixel] = ps.rng[slot];
        J.pix_acc[pixel] = ps.acc[slot];
    }
}

// raytrace.rgen.glsl:277-284 for one finished job.
__global__ void __launch_bounds__(kBlock) kb_resolve(JobGpu J) {
    const uint32_t n = J.W * J.H;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float k = (float)J.cnt[i];
        V3 fin{J.sr[i] / k, J.sg[i] / k, J.sb[i] / k};
        float4* a = reinterpret_cast<float4*>(J.accum) + i;
        if (J.pc.sampleBatch > 0) {
            const float4 prev = *a;
            fin = div3(V3{prev.x, prev.y, prev.z} * (float)J.pc.sampleBatch + fin, (float)(J.pc.sampleBatch + 1));
        }
        *a = make_float4(fin.x, fin.y, fin.z, 1.0f);
    }
}

// ------------------------------------------------------------------------------------------------
// Host side
constexpr size_t kBatchWordsPerPath = 19 + 8 + 10 + 4;   // path state, queues, shadow records, job/pix/smp/depth
constexpr uint32_t kMaxWaveJobs = kMaxWaveSegments / 2;

static BatchPaths layout_batch(uint32_t* w, size_t P) {
    size_t off = 64;   // 16 counters, padded to 256 bytes
    auto f = [&]() { float* r = reinterpret_cast<float*>(w + off); off += P; return r; };
    auto u = [&]() { uint32_t* r = w + off; off += P; return r; };
    BatchPaths b;
    PathState& s = b.ps;
    std::memset(&s, 0, sizeof(s));
    s.counters = w;
    s.ox = f(); s.oy = f(); s.oz = f(); s.dx = f(); s.dy = f(); s.dz = f();
    s.hprim = u(); s.hu = f(); s.hv = f();
    s.tr = f(); s.tg = f(); s.tb = f();
    s.rr = f(); s.rg = f(); s.rb = f();
    s.rng = u(); s.flags = u(); s.acc = f(); s.ppdf = f();
    s.q_active[0] = u(); s.q_active[1] = u();
    s.q_shade = w + off; off += P * kNumQueues;
    s.q_shadow = u();
    s.s_ox = f(); s.s_oy = f(); s.s_oz = f(); s.s_dx = f(); s.s_dy = f(); s.s_dz = f(); s.s_tmax = f();
    s.s_cr = f(); s.s_cg = f(); s.s_cb = f();
    b.job = u(); b.pix = u(); b.smp = u(); b.depth = u();
    return b;
}

static int occupancy(const void* fn, int sm_count) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kBlock, 0);
    return std::max(1, per_sm) * std::max(1, sm_count);
}

BatchEngine::BatchEngine(int device, int sm_count, uint32_t wave_capacity, bool use_graphs, const TraceConfig& trace,
                         int lanes)
    : device_(device), sm_count_(sm_count), capacity_(wave_capacity), use_graphs_(use_graphs), trace_(trace) {
    if (wave_capacity == 0) fail(REINA_ERR_INVALID, "wave capacity must be positive");
    if (lanes < 1 || lanes > 16) fail(REINA_ERR_INVALID, "a batch engine has 1 to 16 lanes");
    desc_bytes_ = sizeof(WaveHeader) + kMaxWaveSegments * sizeof(WaveSeg) + kMaxWaveJobs * sizeof(JobGpu);
    lanes_.resize((size_t)lanes);
    try {
        for (Lane& L : lanes_) {
            L.paths.alloc((64 + kBatchWordsPerPath * (size_t)capacity_) * 4);
            L.desc.alloc(desc_bytes_);
            check_cuda(cudaMallocHost(&L.host_desc, desc_bytes_), "cudaMallocHost");
            check_cuda(cudaMallocHost(reinterpret_cast<void**>(&L.host_counters), kNumCounters * sizeof(uint32_t)),
                       "cudaMallocHost");
            check_cuda(cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking), "cudaStreamCreate");
            check_cuda(cudaEventCreateWithFlags(&L.finished, cudaEventDisableTiming), "cudaEventCreate");
            check_cuda(cudaEventCreateWithFlags(&L.done, cudaEventDisableTiming), "cudaEventCreate");
        }
    } catch (...) {   // the destructor does not run for a constructor that throws
        release_lanes();
        throw;
    }
    if (trace_.refill > 0) {
        blocks_ext_ = resident_grid((const void*)kb_extend_coop, kTraceBlock, sm_count);
        blocks_sh_ = resident_grid((const void*)kb_shadow_coop, kTraceBlock, sm_count);
    } else {
        with_trace_variant(trace_, [&](auto B, auto S) {
            blocks_ext_ = resident_grid((const void*)kb_extend<B.value, S.value, false>, B.value, sm_count);
            blocks_sh_ = resident_grid((const void*)kb_shadow<B.value, S.value, false>, B.value, sm_count);
        });
    }
    blocks_ext_two_ = resident_grid((const void*)kb_extend<kTraceBlock, kDefaultTraceStack, true>, kTraceBlock, sm_count);
    blocks_sh_two_ = resident_grid((const void*)kb_shadow<kTraceBlock, kDefaultTraceStack, true>, kTraceBlock, sm_count);
    blocks_shade_[1] = occupancy((const void*)kb_shade<1>, sm_count);
    blocks_shade_[2] = occupancy((const void*)kb_shade<2>, sm_count);
    blocks_shade_[3] = occupancy((const void*)kb_shade<3>, sm_count);
    blocks_shade_[4] = occupancy((const void*)kb_shade<4>, sm_count);
    blocks_simple_ = occupancy((const void*)kb_finish, sm_count);
}

BatchEngine::~BatchEngine() { release_lanes(); }

void BatchEngine::release_lanes() {
    for (Lane& L : lanes_) {
        if (L.stream) cudaStreamSynchronize(L.stream);
        for (auto& g : L.graphs)
            if (g.exec) cudaGraphExecDestroy(g.exec);
        if (L.finished) cudaEventDestroy(L.finished);
        if (L.done) cudaEventDestroy(L.done);
        if (L.stream) cudaStreamDestroy(L.stream);
        if (L.host_desc) cudaFreeHost(L.host_desc);
        if (L.host_counters) cudaFreeHost(L.host_counters);
    }
    lanes_.clear();
}

void BatchEngine::prepare(BatchJob& job, cudaMemPool_t pool, cudaStream_t st) {
    const size_t px = (size_t)job.opt.width * job.opt.height;
    job.total = (uint64_t)job.pc.samplesPerPixel * px;
    job.cursor = 0;
    job.resolved = false;
    if (pool) job.pixel_state.alloc_async(px * 6 * sizeof(uint32_t), pool, st);
    else job.pixel_state.alloc(px * 6 * sizeof(uint32_t));
}

static JobGpu job_record(const BatchJob& j) {
    JobGpu g;
    std::memset(&g, 0, sizeof(g));
    g.s = j.scene;
    g.pc = j.pc;
    g.W = j.opt.width;
    g.H = j.opt.height;
    g.mode = j.opt.mode;
    g.seed = j.opt.seed;
    g.env_mode = j.opt.env_mode;
    for (int k = 0; k < 3; ++k) g.env[k] = j.opt.env_color[k];
    g.spp = j.pc.samplesPerPixel;
    g.max_bounces = j.pc.maxBounces;
    g.accum = j.d_accum;
    g.samples = j.d_samples;
    const size_t px = (size_t)g.W * g.H;
    uint32_t* w = j.pixel_state.as<uint32_t>();
    g.pix_rng = w;
    g.pix_acc = reinterpret_cast<float*>(w + px);
    g.sr = reinterpret_cast<float*>(w + 2 * px);
    g.sg = reinterpret_cast<float*>(w + 3 * px);
    g.sb = reinterpret_cast<float*>(w + 4 * px);
    g.cnt = w + 5 * px;
    return g;
}

void BatchEngine::launch_body(Lane& L, const Packed& pk, cudaStream_t st) {
    const WaveHeader& h = pk.hdr;
    uint8_t* d = L.desc.as<uint8_t>();
    const uint8_t* hd = static_cast<const uint8_t*>(L.host_desc);
    check_cuda(cudaMemcpyAsync(d, hd, sizeof(WaveHeader) + h.nseg * sizeof(WaveSeg), cudaMemcpyHostToDevice, st),
               "H2D wave");
    const size_t job_off = sizeof(WaveHeader) + kMaxWaveSegments * sizeof(WaveSeg);
    check_cuda(cudaMemcpyAsync(d + job_off, hd + job_off, h.njobs * sizeof(JobGpu), cudaMemcpyHostToDevice, st),
               "H2D jobs");
    BatchLaunch B;
    B.bp = layout_batch(L.paths.as<uint32_t>(), capacity_);
    B.hdr = reinterpret_cast<const WaveHeader*>(d);
    B.segs = reinterpret_cast<const WaveSeg*>(d + sizeof(WaveHeader));
    B.jobs = reinterpret_cast<const JobGpu*>(d + job_off);
    B.P = capacity_;
    uint32_t* cnt = B.bp.ps.counters;
    const int simple = std::min<int>(blocks_simple_, (int)((capacity_ + kBlock - 1) / kBlock));
    const bool any_nee = pk.any_nee, two = pk.two, count = count_;
    if (count && blocks_ext_cnt_ == 0) {   // grids of the counting kernels (default block and stack)
        blocks_ext_cnt_ = resident_grid((const void*)kb_extend<kTraceBlock, kDefaultTraceStack, false, true>, kTraceBlock, sm_count_);
        blocks_sh_cnt_ = resident_grid((const void*)kb_shadow<kTraceBlock, kDefaultTraceStack, false, true>, kTraceBlock, sm_count_);
        blocks_ext_two_cnt_ = resident_grid((const void*)kb_extend<kTraceBlock, kDefaultTraceStack, true, true>, kTraceBlock, sm_count_);
        blocks_sh_two_cnt_ = resident_grid((const void*)kb_shadow<kTraceBlock, kDefaultTraceStack, true, true>, kTraceBlock, sm_count_);
    }
    auto sequence = [&](cudaStream_t s) {
        check_cuda(cudaMemsetAsync(cnt, 0, kNumCounters * sizeof(uint32_t), s), "cudaMemsetAsync");
        kb_init<<<simple, kBlock, 0, s>>>(B, B.jobs);
        int cur = 0;
        for (uint32_t seg = 0; seg < h.max_bounces; ++seg) {
            check_cuda(cudaMemsetAsync(cnt + kCntActive + (cur ^ 1), 0, sizeof(uint32_t), s), "cudaMemsetAsync");
            check_cuda(cudaMemsetAsync(cnt + kCntQueue, 0, 6 * sizeof(uint32_t), s), "cudaMemsetAsync");
            if (!two && trace_.refill > 0)
                check_cuda(cudaMemsetAsync(cnt + kCntFetchExtend, 0, 2 * sizeof(uint32_t), s), "cudaMemsetAsync");
            if (two && count)
                kb_extend<kTraceBlock, kDefaultTraceStack, true, true><<<blocks_ext_two_cnt_, kTraceBlock, 0, s>>>(B, B.jobs, cur);
            else if (two)   // a two-level scene in the wave: the default grid variant, both traversals
                kb_extend<kTraceBlock, kDefaultTraceStack, true><<<blocks_ext_two_, kTraceBlock, 0, s>>>(B, B.jobs, cur);
            else if (trace_.refill > 0)
                kb_extend_coop<<<blocks_ext_, kTraceBlock, 0, s>>>(B, B.jobs, cur, (uint32_t)(32 - trace_.refill));
            else if (count)
                kb_extend<kTraceBlock, kDefaultTraceStack, false, true><<<blocks_ext_cnt_, kTraceBlock, 0, s>>>(B, B.jobs, cur);
            else
                with_trace_variant(trace_, [&](auto BS, auto SS) {
                    kb_extend<BS.value, SS.value, false><<<blocks_ext_, BS.value, 0, s>>>(B, B.jobs, cur);
                });
            kb_shade_miss<<<simple, kBlock, 0, s>>>(B, B.jobs);
            kb_shade<1><<<blocks_shade_[1], kBlock, 0, s>>>(B, B.jobs, cur);
            kb_shade<2><<<blocks_shade_[2], kBlock, 0, s>>>(B, B.jobs, cur);
            kb_shade<3><<<blocks_shade_[3], kBlock, 0, s>>>(B, B.jobs, cur);
            kb_shade<4><<<blocks_shade_[4], kBlock, 0, s>>>(B, B.jobs, cur);
            if (any_nee && two && count)
                kb_shadow<kTraceBlock, kDefaultTraceStack, true, true><<<blocks_sh_two_cnt_, kTraceBlock, 0, s>>>(B, B.jobs);
            else if (any_nee && two)
                kb_shadow<kTraceBlock, kDefaultTraceStack, true><<<blocks_sh_two_, kTraceBlock, 0, s>>>(B, B.jobs);
            else if (any_nee && trace_.refill > 0)
                kb_shadow_coop<<<blocks_sh_, kTraceBlock, 0, s>>>(B, B.jobs, (uint32_t)(32 - trace_.refill));
            else if (any_nee && count)
                kb_shadow<kTraceBlock, kDefaultTraceStack, false, true><<<blocks_sh_cnt_, kTraceBlock, 0, s>>>(B, B.jobs);
            else if (any_nee)
                with_trace_variant(trace_, [&](auto BS, auto SS) {
                    kb_shadow<BS.value, SS.value, false><<<blocks_sh_, BS.value, 0, s>>>(B, B.jobs);
                });
            cur ^= 1;
        }
    };
    if (!use_graphs_) {
        sequence(st);
        check_cuda(cudaGetLastError(), "batch wave launch");
        return;
    }
    GraphSlot* slot = nullptr;
    for (auto& g : L.graphs)
        if (g.bounces == h.max_bounces && g.nee == any_nee && g.two == two && g.count == count) slot = &g;
    if (!slot) {
        cudaStream_t cap;
        check_cuda(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking), "cudaStreamCreate");
        cudaGraph_t graph;
        check_cuda(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
        sequence(cap);
        check_cuda(cudaStreamEndCapture(cap, &graph), "cudaStreamEndCapture");
        cudaStreamDestroy(cap);
        GraphSlot g;
        g.bounces = h.max_bounces;
        g.nee = any_nee;
        g.two = two;
        g.count = count;
        check_cuda(cudaGraphInstantiate(&g.exec, graph, 0), "cudaGraphInstantiate");
        cudaGraphDestroy(graph);
        L.graphs.push_back(g);
        slot = &L.graphs.back();
    }
    check_cuda(cudaGraphLaunch(slot->exec, st), "cudaGraphLaunch");
}

void BatchEngine::launch_finish(Lane& L, const Packed& pk, cudaStream_t st) {
    const uint8_t* d = L.desc.as<uint8_t>();
    BatchLaunch B;
    B.bp = layout_batch(L.paths.as<uint32_t>(), capacity_);
    B.hdr = reinterpret_cast<const WaveHeader*>(d);
    B.segs = reinterpret_cast<const WaveSeg*>(d + sizeof(WaveHeader));
    B.jobs = reinterpret_cast<const JobGpu*>(d + sizeof(WaveHeader) + kMaxWaveSegments * sizeof(WaveSeg));
    B.P = capacity_;
    const int simple = std::min<int>(blocks_simple_, (int)((capacity_ + kBlock - 1) / kBlock));
    kb_finish<<<simple, kBlock, 0, st>>>(B, B.jobs);
    for (BatchJob* j : pk.completed) {   // resolve the jobs this wave completed
        const JobGpu g = job_record(*j);
        const uint32_t px = g.W * g.H;
        const int blocks = (int)std::min<uint32_t>((px + kBlock - 1) / kBlock, (uint32_t)blocks_simple_);
        kb_resolve<<<blocks, kBlock, 0, st>>>(g);
    }
    check_cuda(cudaGetLastError(), "batch launch");
    check_cuda(cudaEventRecord(L.finished, st), "cudaEventRecord");
    check_cuda(cudaMemcpyAsync(L.host_counters, L.paths.get(), kNumCounters * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                               st), "D2H counters");
    check_cuda(cudaEventRecord(L.done, st), "cudaEventRecord");
    L.pending = true;
}

void BatchEngine::collect(Lane& L) {
    if (!L.pending) return;
    L.pending = false;
    const uint32_t* c = L.host_counters;
    auto u64 = [&](int at) { uint64_t v; std::memcpy(&v, c + at, 8); return v; };
    rays_ += u64(kCntRays);
    shadow_rays_ += u64(kCntShadowRays);
    work_.nodes += u64(kCntNodes);
    work_.tris += u64(kCntTris);
    work_.shadow_nodes += u64(kCntShadowNodes);
    work_.shadow_tris += u64(kCntShadowTris);
    work_.shaded += u64(kCntShaded);
    waves_++;
    if (c[kCntError])
        fail(REINA_ERR_DEVICE, "batch wave kernels raised error flag " + std::to_string(c[kCntError]) +
                                   device_error_text(c[kCntError]));
}

BatchEngine::Packed BatchEngine::pack(const std::vector<BatchJob*>& jobs, bool fifo, Lane& L) {
    Packed pk;
    std::memset(&pk.hdr, 0, sizeof(pk.hdr));
    // active jobs (at most kMaxWaveJobs per wave; the rest wait for a later wave)
    std::vector<BatchJob*> active;
    for (BatchJob* j : jobs)
        if (j->cursor < j->total && active.size() < kMaxWaveJobs) active.push_back(j);
    if (active.empty()) return pk;
    // fair share of the capacity, then leftovers to the oldest jobs (or, first-come first-served, each
    // job in order takes all it can use)
    // A job's samples per pixel in one wave: any number when its samples are independent (NEE+MIS: seeded
    // by (pixel, sample); the finish kernel sums a pixel's samples of the wave in order); one in the
    // reference's mode, where a pixel's next sample starts from the state its previous one left.
    auto cap = [](const BatchJob* j) -> uint64_t {
        return j->opt.mode == kModeNeeMis ? UINT64_MAX : (uint64_t)j->opt.width * j->opt.height;
    };
    std::vector<uint64_t> take(active.size(), 0);
    const uint64_t fair = fifo ? (uint64_t)capacity_ : std::max<uint64_t>(1, capacity_ / active.size());
    uint64_t used = 0;
    for (size_t a = 0; a < active.size(); ++a) {
        const BatchJob* j = active[a];
        take[a] = std::min({fair, cap(j), j->total - j->cursor, (uint64_t)capacity_ - used});
        used += take[a];
    }
    for (size_t a = 0; a < active.size() && used < capacity_; ++a) {
        const BatchJob* j = active[a];
        const uint64_t more = std::min(std::min(cap(j), j->total - j->cursor) - take[a], (uint64_t)capacity_ - used);
        take[a] += more;
        used += more;
    }
    uint8_t* h = static_cast<uint8_t*>(L.host_desc);
    WaveHeader* hdr = reinterpret_cast<WaveHeader*>(h);
    WaveSeg* segs = reinterpret_cast<WaveSeg*>(h + sizeof(WaveHeader));
    JobGpu* jt = reinterpret_cast<JobGpu*>(h + sizeof(WaveHeader) + kMaxWaveSegments * sizeof(WaveSeg));
    uint32_t nseg = 0, njobs = 0, wave_pos = 0, bounces = 0, finish = 0;
    for (size_t a = 0; a < active.size(); ++a) {
        if (take[a] == 0) continue;
        if (nseg >= kMaxWaveSegments) break;   // the descriptor is full: later jobs wait for the next wave
        BatchJob* j = active[a];
        const uint64_t px = (uint64_t)j->opt.width * j->opt.height;
        const uint32_t ji = njobs++;
        jt[ji] = job_record(*j);
        pk.members.push_back(j);
        bounces = std::max(bounces, j->pc.maxBounces);
        pk.any_nee = pk.any_nee || j->opt.mode == kModeNeeMis;
        pk.two = pk.two || j->scene.inst_trav != nullptr;
        const uint64_t c0 = j->cursor;
        const uint32_t ws = wave_pos;
        uint64_t m = take[a];
        while (m > 0 && nseg < kMaxWaveSegments) {
            const uint64_t sample = j->cursor / px, pixel = j->cursor % px;
            const uint64_t c = std::min(m, px - pixel);
            WaveSeg& s = segs[nseg++];
            s.job = ji;
            s.wave_start = wave_pos;
            s.pixel_start = (uint32_t)pixel;
            s.count = (uint32_t)c;
            s.sample = (uint32_t)sample;
            wave_pos += (uint32_t)c;
            j->cursor += c;
            m -= c;
        }
        const uint64_t placed = j->cursor - c0;
        jt[ji].cursor0 = c0;
        jt[ji].wave_start = ws;
        jt[ji].take = (uint32_t)placed;
        jt[ji].finish_start = finish;
        finish += (uint32_t)std::min(placed, px);
        // samples after a pixel's first start from the state its previous sample left (reference mode)
        pk.carries = pk.carries || (j->opt.mode != kModeNeeMis && c0 + placed > px);
        if (j->cursor == j->total && !j->resolved) {
            pk.completed.push_back(j);
            j->resolved = true;
        }
    }
    hdr->count = wave_pos;
    hdr->nseg = nseg;
    hdr->njobs = njobs;
    hdr->max_bounces = bounces;
    hdr->finish_total = finish;
    pk.hdr = *hdr;
    return pk;
}

bool BatchEngine::submit_wave(const std::vector<BatchJob*>& jobs, bool fifo, std::vector<BatchJob*>* members,
                              std::vector<BatchJob*>* completed) {
    Lane& L = lanes_[submitted_ % lanes_.size()];
    if (L.pending) fail(REINA_ERR_STATE, "batch engine: no free lane");
    Packed pk = pack(jobs, fifo, L);
    if (pk.hdr.count == 0) return false;
    Lane* prev = submitted_ > 0 ? &lanes_[(submitted_ - 1) % lanes_.size()] : nullptr;
    if (prev == &L) prev = nullptr;   // one lane: stream order already chains the waves
    if (prev && pk.carries) check_cuda(cudaStreamWaitEvent(L.stream, prev->finished, 0), "cudaStreamWaitEvent");
    launch_body(L, pk, L.stream);
    if (prev) check_cuda(cudaStreamWaitEvent(L.stream, prev->finished, 0), "cudaStreamWaitEvent");
    launch_finish(L, pk, L.stream);
    ++submitted_;
    if (members) *members = std::move(pk.members);
    if (completed) *completed = std::move(pk.completed);
    return true;
}

void BatchEngine::wait_oldest() {
    if (!pending()) return;
    Lane& L = lanes_[retired_ % lanes_.size()];
    ++retired_;
    check_cuda(cudaEventSynchronize(L.done), "cudaEventSynchronize");
    collect(L);
}

void BatchEngine::drain() {
    for (Lane& L : lanes_) {
        cudaStreamSynchronize(L.stream);
        L.pending = false;
    }
    retired_ = submitted_;
}

void BatchEngine::order_after(cudaStream_t st) {
    cudaEvent_t e;
    check_cuda(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate");
    cudaError_t err = cudaEventRecord(e, st);
    for (Lane& L : lanes_)
        if (err == cudaSuccess) err = cudaStreamWaitEvent(L.stream, e, 0);
    cudaEventDestroy(e);
    check_cuda(err, "ordering the lanes after the caller's stream");
}

void BatchEngine::order_before(cudaStream_t st) {
    for (Lane& L : lanes_) {
        check_cuda(cudaEventRecord(L.done, L.stream), "cudaEventRecord");
        check_cuda(cudaStreamWaitEvent(st, L.done, 0), "cudaStreamWaitEvent");
    }
}

void BatchEngine::run_all(const std::vector<BatchJob*>& jobs, cudaStream_t st, bool fifo) {
    try {
        order_after(st);
        for (;;) {
            if (!lane_free()) wait_oldest();   // reuse the lane of the wave two back
            if (!submit_wave(jobs, fifo)) break;
        }
        while (pending()) wait_oldest();
        order_before(st);
    } catch (...) {
        drain();   // nothing of this call stays in flight
        throw;
    }
}

}  // namespace rt
