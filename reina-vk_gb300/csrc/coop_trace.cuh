// Warp-cooperative persistent BVH8 traversal: the default launch form for flat scenes.
//
// The per-thread traversal of trace_device.cuh loses most of a warp's issue slots to divergence on
// incoherent rays: lanes whose rays have ended wait for the warp's longest ray, and the triangle tests
// run with the few lanes whose node had leaf children.  Here a warp keeps 32 rays in flight and shares
// the work that diverges:
//   * refill (Aila and Laine, "Understanding the Efficiency of Ray Traversal on GPUs", HPG 2009): when at
//     most `refill_at` lanes still trace, the idle lanes take the next rays from a warp-private chunk of
//     the global fetch counter;
//   * node visits: every tracing lane visits its nearest pending child node (the step of trace_device.cuh:
//     box test of the 8 quantized children, near-to-far order by ray octant), kCoopVisits times between
//     two rounds of the warp's bookkeeping (refill, list tests, finishing), so that the bookkeeping is
//     paid once per several visits;
//   * triangle tests: a node's leaf triangles are not tested by the lane that found them; the warp
//     collects (ray, triangle group) pairs in a shared list and, once it holds kFlushTris triangles (or a
//     lane with groups in the list has no nodes left), tests them with one (ray, triangle) pair per lane,
//     the closest (t, prim) per ray kept by a 64-bit atomic minimum in shared memory;
//   * finishing: ended rays go to a shared list that the warp refines (refine_hit) and stores one per
//     lane once it is full, so the hit refinement also runs at full width.
// The closest hit is the lowest (t, prim) over the triangles hit in [tmin, tmax], as in every other form,
// so hits are bit-identical to the per-thread traversal; any-hit rays end at the first triangle found.
#pragma once

#include <stdint.h>

#include "trace_device.cuh"

namespace rt {

// Per-warp shared state of the cooperative traversal.
struct CoopWarp {
    float4 ray_a[32];                 // per lane: origin, tmin of its ray (for the triangle tests)
    float4 ray_b[32];                 // per lane: shear constants sx, sy, sz, axes kx | ky << 2 | kz << 4
    unsigned long long best[32];      // per lane: ordered(t) << 32 | prim of the closest hit so far
    float4 best_hit[32];              // per lane: triangle record (bits), t, u, v of that hit
    const float4* tris[32];           // per lane: triangle records of its ray's scene
    uint32_t gbase[64];               // triangle groups: first triangle record
    uint32_t gmo[64];                 // triangle groups: owner lane << 24 | triangle hit mask
    uint32_t gprefix[64];             // inclusive prefix of the groups' triangle counts
    float4 fin_o[32];                 // finished rays: origin, t
    float4 fin_d[32];                 // finished rays: direction, u
    uint4 fin_i[32];                  // finished rays: item, prim, triangle record, v (bits)
    const float4* fin_tris[32];       // finished rays: triangle records of their scene
};

// Scene of one item (per lane: batched waves mix scenes).
struct CoopScene {
    const Bvh8Node* nodes;
    const TriRecord* tris;
    uint32_t node_count;
};

// Items per warp-private fetch chunk.  Small chunks interleave the warps over the item list, so the last
// items end together (1.3M-triangle ray cast: chunks of 32 0.568 ms, 128 0.656 ms, 512 0.822 ms).
constexpr uint32_t kCoopChunk = 32;
// Blocks of 128 threads per SM the cooperative kernels are compiled for: 7 (at most 72 registers; 30 KB of
// shared memory each, 210 KB per SM).
#ifndef RT_COOP_MINB
#define RT_COOP_MINB 7
#endif
constexpr int kCoopMinBlocks = RT_COOP_MINB;
#ifndef RT_COOP_FLUSH_TRIS
#define RT_COOP_FLUSH_TRIS 24
#endif
constexpr uint32_t kFlushTris = RT_COOP_FLUSH_TRIS;   // triangles collected before the warp tests them
// Node visits per lane per round of bookkeeping (1.3M-triangle ray cast, closest hit: 1 visit 0.539 ms,
// 2 visits 0.505 ms with 0.7 % more node visits, 3 visits 0.556 ms, 4 visits 0.620 ms).
#ifndef RT_COOP_VISITS
#define RT_COOP_VISITS 2
#endif
constexpr int kCoopVisits = RT_COOP_VISITS;

__device__ __forceinline__ uint32_t coop_ordered(float f) {
    const uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float coop_unordered(uint32_t o) {
    return __uint_as_float((o & 0x80000000u) ? (o & 0x7FFFFFFFu) : ~o);
}
__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Adds a warp's traversal counts to two u64 device counters (one atomic per warp).
__device__ __forceinline__ void coop_add_counts(const TraceCounters& c, uint32_t* counters, int nodes_at, int tris_at) {
    unsigned long long nv = c.nodes, tv = c.tris;
    for (int o = 16; o > 0; o >>= 1) {
        nv += __shfl_down_sync(0xFFFFFFFFu, nv, o);
        tv += __shfl_down_sync(0xFFFFFFFFu, tv, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (nv) atomicAdd(reinterpret_cast<unsigned long long*>(counters + nodes_at), nv);
        if (tv) atomicAdd(reinterpret_cast<unsigned long long*>(counters + tris_at), tv);
    }
}

// Tests the collected triangle groups, one (ray, triangle) pair per lane per round.  MIXED: each lane's ray
// has its own scene (S.tris); otherwise every ray uses `tris`.  Not inlined, like coop_store_finished: both
// run once per several traversal steps, and kept out of the traversal loop they leave it more registers
// (1.3M-triangle ray cast: 0.566 -> 0.534 ms, the loop's register copies moved off the ALU pipe).
template <bool COUNT, bool MIXED>
__device__ __noinline__ void coop_test_groups(CoopWarp& S, uint32_t lane, uint32_t n_groups, const float4* tris,
                                                 TraceCounters& cnt) {
    const uint32_t c0 = lane < n_groups ? __popc(S.gmo[lane] & 0x00FFFFFFu) : 0u;
    const uint32_t c1 = lane + 32u < n_groups ? __popc(S.gmo[lane + 32u] & 0x00FFFFFFu) : 0u;
    uint32_t i0 = c0, i1 = c1;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y0 = __shfl_up_sync(0xFFFFFFFFu, i0, o);
        const uint32_t y1 = __shfl_up_sync(0xFFFFFFFFu, i1, o);
        if (lane >= (uint32_t)o) { i0 += y0; i1 += y1; }
    }
    const uint32_t t0 = __shfl_sync(0xFFFFFFFFu, i0, 31);
    const uint32_t total = t0 + __shfl_sync(0xFFFFFFFFu, i1, 31);
    S.gprefix[lane] = i0;
    S.gprefix[lane + 32u] = i1 + t0;
    __syncwarp();
    for (uint32_t b0 = 0; b0 < total; b0 += 32u) {
        const uint32_t p = b0 + lane;
        bool hit = false;
        uint32_t o = 0, rec = 0;
        unsigned long long key = 0;
        float t = 0.0f, u = 0.0f, v = 0.0f;
        if (p < total) {
            uint32_t g = 0;   // the group holding pair p: binary search over the prefix
#pragma unroll
            for (uint32_t s = 32; s; s >>= 1)
                if (g + s - 1 < n_groups && S.gprefix[g + s - 1] <= p) g += s;
            const uint32_t k = p - (g ? S.gprefix[g - 1] : 0u);
            const uint32_t mo = S.gmo[g];
            o = mo >> 24;
            rec = S.gbase[g] + (uint32_t)__fns(mo & 0x00FFFFFFu, 0u, (int)k + 1);
            const float4* tp = (MIXED ? S.tris[o] : tris) + 3ull * rec;
            const float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
            const float4 ra = S.ray_a[o], rb = S.ray_b[o];
            TraceRay q;
            q.ox = ra.x; q.oy = ra.y; q.oz = ra.z; q.tmin = ra.w;
            q.sx = rb.x; q.sy = rb.y; q.sz = rb.z;
            const uint32_t kk = __float_as_uint(rb.w);
            q.kx = (int)(kk & 3u); q.ky = (int)((kk >> 2) & 3u); q.kz = (int)((kk >> 4) & 3u);
            if (COUNT) cnt.tris++;
            if (intersect_triangle(q, a, b, c, coop_unordered((uint32_t)(S.best[o] >> 32)), t, u, v)) {
                hit = true;
                key = ((unsigned long long)coop_ordered(t + 0.0f) << 32) | __float_as_uint(a.w);
                atomicMin(&S.best[o], key);
            }
        }
        __syncwarp();
        if (hit && S.best[o] == key) S.best_hit[o] = make_float4(__uint_as_float(rec), t, u, v);
        __syncwarp();
    }
}

// Refines (REFINE) and stores the finished rays of the list, one per lane; store is called by all lanes.
template <bool REFINE, bool MIXED, class Store>
__device__ __noinline__ void coop_store_finished(CoopWarp& S, uint32_t lane, uint32_t n_fin, const float4* tris,
                                                    Store& store) {
    __syncwarp();
    const bool valid = lane < n_fin;
    Hit h;
    h.prim = kMiss; h.t = 0.0f; h.u = 0.0f; h.v = 0.0f;
    uint32_t item = 0;
    if (valid) {
        const float4 o = S.fin_o[lane], d = S.fin_d[lane];
        const uint4 fi = S.fin_i[lane];
        item = fi.x;
        h.prim = fi.y;
        h.t = o.w;
        h.u = d.w;
        h.v = __uint_as_float(fi.w);
        if (REFINE && h.prim != kMiss) {
            TraceRay r;
            r.ox = o.x; r.oy = o.y; r.oz = o.z;
            r.dx = d.x; r.dy = d.y; r.dz = d.z;
            const float4* tp = (MIXED ? S.fin_tris[lane] : tris) + 3ull * fi.z;
            refine_hit(r, __ldg(tp), __ldg(tp + 1), __ldg(tp + 2), h);
        }
    }
    __syncwarp();
    store(item, h, valid);
}

// Traces items [0, n) of the caller's list: load(i, ray, scene) -> false if item i has no ray to trace (it
// is stored as a miss with t = its tmax); with MIXED, load also names the item's scene (batched waves mix
// scenes), otherwise every item uses `uniform`; store(i, hit, valid) is called by all 32 lanes together with
// up to 32 finished items (valid marks the lanes holding one).  `next` is the global fetch counter (zero
// at launch); a warp refills its idle lanes once at most `refill_at` lanes still trace.  Requires
// blockDim.x to be a multiple of 32; `stack` points at this thread's first shared stack entry, entries
// `stride` apart.  Returns the device error bits of the warp's rays.
// CHUNK, FLUSH: the fetch chunk and the triangle flush size; VISITS: node visits per lane between two
// rounds of the warp's bookkeeping (the triangles found meanwhile are tested at the next flush, so the
// closest distance a visit culls with may lag by up to VISITS - 1 visits: a few more nodes, same hits).
template <bool ANY, bool COUNT, bool REFINE, bool MIXED, int SS, uint32_t CHUNK = kCoopChunk, uint32_t FLUSH = kFlushTris,
          int VISITS = kCoopVisits, class Load, class Store>
__device__ __forceinline__ uint32_t coop_trace(const CoopScene& uniform, uint32_t n, uint32_t* next, uint32_t refill_at,
                                               CoopWarp& S, uint2* stack, int stride, Load load, Store store,
                                               TraceCounters& cnt) {
    const uint32_t lane = threadIdx.x & 31u;
    uint2 spill[kTotalStack - SS];
    uint32_t err = 0;
    bool has = false;
    TraceRay r;
    CoopScene sc = uniform;
    const float4* utris = reinterpret_cast<const float4*>(uniform.tris);
    uint32_t item = 0;
    uint2 group = make_uint2(0u, 0u);
    int sp = 0;
    uint32_t steps = 0;
    float best_t = 0.0f;
    uint32_t my_groups = 0;                         // this lane's groups in the list
    uint32_t n_groups = 0, n_tris = 0, n_fin = 0;   // warp-uniform list sizes
    uint32_t chunk_next = 0, chunk_end = 0;         // warp-uniform: unclaimed items [next, end) of the chunk
    bool exhausted = false;
    // tests the warp's triangle list (all lanes together) and takes each lane's result
    auto flush = [&]() {
        __syncwarp();
        coop_test_groups<COUNT, MIXED>(S, lane, n_groups, utris, cnt);
        n_groups = 0;
        n_tris = 0;
        if (has && my_groups) {
            const unsigned long long key = S.best[lane];
            if (ANY) {
                if ((uint32_t)key != 0xFFFFFFFFu) { group = make_uint2(0u, 0u); sp = 0; }
            } else {
                best_t = coop_unordered((uint32_t)(key >> 32));
            }
        }
        my_groups = 0;
    };
    for (;;) {
        // refill idle lanes
        const uint32_t active = __ballot_sync(0xFFFFFFFFu, has);
        const uint32_t n_active = (uint32_t)__popc(active);
        if (!exhausted && n_active <= refill_at) {
            const uint32_t idle = ~active;
            const uint32_t n_idle = 32u - n_active;
            const uint32_t rem = chunk_end - chunk_next;
            uint32_t base = 0;
            if (rem < n_idle) {
                if (lane == 0) base = atomicAdd(next, CHUNK);
                base = __shfl_sync(0xFFFFFFFFu, base, 0);
            }
            bool empty_item = false;
            if (!has) {
                const uint32_t rank = (uint32_t)__popc(idle & lanemask_lt());
                const uint32_t i = rank < rem ? chunk_next + rank : base + (rank - rem);
                if (i < n && (rank < rem || base < n)) {
                    item = i;
                    CoopScene own = uniform;
                    const bool loaded = load(i, r, own);
                    if (MIXED) sc = own;
                    const bool traced = loaded && (MIXED ? own.node_count : uniform.node_count) != 0;
                    if (traced) {
                        has = true;
                        group = make_uint2(0u, 0x80000000u);
                        sp = 0;
                        steps = 0;
                        best_t = r.tmax;
                        S.ray_a[lane] = make_float4(r.ox, r.oy, r.oz, r.tmin);
                        S.ray_b[lane] = make_float4(r.sx, r.sy, r.sz,
                                                    __uint_as_float((uint32_t)r.kx | ((uint32_t)r.ky << 2) | ((uint32_t)r.kz << 4)));
                        S.best[lane] = ((unsigned long long)coop_ordered(r.tmax) << 32) | 0xFFFFFFFFull;
                        if (MIXED) S.tris[lane] = reinterpret_cast<const float4*>(sc.tris);
                    } else {
                        empty_item = true;   // no ray: stored as a miss
                    }
                }
            }
            if (rem < n_idle) {
                chunk_next = base + (n_idle - rem);
                chunk_end = base + CHUNK;
                if (base >= n) exhausted = true;
                if (chunk_end > n) chunk_end = n > chunk_next ? n : chunk_next;
            } else {
                chunk_next += n_idle;
            }
            // items without a ray go straight to the finished list
            const uint32_t em = __ballot_sync(0xFFFFFFFFu, empty_item);
            if (em) {
                if (n_fin + (uint32_t)__popc(em) > 32u) {
                    coop_store_finished<REFINE, MIXED>(S, lane, n_fin, utris, store);
                    n_fin = 0;
                }
                if (empty_item) {
                    const uint32_t pos = n_fin + (uint32_t)__popc(em & lanemask_lt());
                    S.fin_o[pos] = make_float4(0.0f, 0.0f, 0.0f, r.tmax);
                    S.fin_d[pos] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    S.fin_i[pos] = make_uint4(item, kMiss, 0u, 0u);
                    if (MIXED) S.fin_tris[pos] = nullptr;
                }
                n_fin += (uint32_t)__popc(em);
            }
        }
        if (!__any_sync(0xFFFFFFFFu, has)) {
            if (exhausted) break;
            continue;
        }
        // watchdog: a ray's traversal ends with kErrStepLimit after kMaxTraversalSteps visit slots
        if (has) {
            steps += VISITS;
            if (steps > kMaxTraversalSteps) {
                err |= kErrStepLimit;
                group = make_uint2(0u, 0u);
                sp = 0;
            }
        }
        // VISITS node visits per tracing lane, each followed by its stack pop; every visit's leaf triangles
        // join the warp's list (tested before the list could overflow, between visits if need be)
#pragma unroll
        for (int v = 0; v < VISITS; ++v) {
            uint32_t tbase = 0, tmask = 0;
            if (has && group.y > 0x00FFFFFFu) {
                const uint32_t slot_bit = 31u - __clz(group.y);
                const uint32_t slot = (slot_bit - 24u) ^ r.oct_inv;
                const uint32_t child = group.x + (uint32_t)__popc(group.y & ((1u << slot) - 1u));
                group.y &= ~(1u << slot_bit);
                if (group.y > 0x00FFFFFFu) {
                    if (sp < SS) {
                        stack[sp * stride] = group;
                        ++sp;
                    } else if (sp < kTotalStack) {
                        spill[sp - SS] = group;
                        ++sp;
                    } else {
                        err |= kErrStackOverflow;
                    }
                }
                const uint4* np = reinterpret_cast<const uint4*>(MIXED ? sc.nodes : uniform.nodes) + 5ull * child;
                const uint4 w0 = __ldg(np + 0), w1 = __ldg(np + 1), w2 = __ldg(np + 2), w3 = __ldg(np + 3),
                            w4 = __ldg(np + 4);
                if (COUNT) cnt.nodes++;
                const uint32_t hm = intersect_children(r, w0, w1, w2, w3, w4, best_t);
                group = make_uint2(w1.x, (hm & 0xFF000000u) | (w0.w >> 24));
                tbase = w1.y;
                tmask = hm & 0x00FFFFFFu;
            }
            if (has && group.y <= 0x00FFFFFFu && sp > 0) {
                --sp;
                group = sp < SS ? stack[sp * stride] : spill[sp - SS];
            }
            const uint32_t app = __ballot_sync(0xFFFFFFFFu, tmask != 0u);
            if (app) {
                if (tmask) {
                    const uint32_t pos = n_groups + (uint32_t)__popc(app & lanemask_lt());
                    S.gbase[pos] = tbase;
                    S.gmo[pos] = (lane << 24) | tmask;
                    ++my_groups;
                }
                n_groups += (uint32_t)__popc(app);
                n_tris += __reduce_add_sync(0xFFFFFFFFu, (uint32_t)__popc(tmask));
            }
            if (v + 1 < VISITS && n_groups > 32u) flush();
        }
        // test the list when it is full enough, could overflow next step, or holds groups of a finished lane
        const bool waiting = has && group.y <= 0x00FFFFFFu && sp == 0 && my_groups > 0;
        if (n_groups && (__any_sync(0xFFFFFFFFu, waiting) || n_tris >= FLUSH || n_groups > 32u)) flush();
        // finished rays join the warp's finished list
        const bool done = has && group.y <= 0x00FFFFFFu && sp == 0 && my_groups == 0;
        const uint32_t dm = __ballot_sync(0xFFFFFFFFu, done);
        if (dm) {
            if (n_fin + (uint32_t)__popc(dm) > 32u) {
                coop_store_finished<REFINE, MIXED>(S, lane, n_fin, utris, store);
                n_fin = 0;
            }
            if (done) {
                const uint32_t pos = n_fin + (uint32_t)__popc(dm & lanemask_lt());
                const unsigned long long key = S.best[lane];
                const float4 bh = S.best_hit[lane];
                const bool miss = (uint32_t)key == 0xFFFFFFFFu;
                S.fin_o[pos] = make_float4(r.ox, r.oy, r.oz, miss ? r.tmax : bh.y);
                S.fin_d[pos] = make_float4(r.dx, r.dy, r.dz, miss ? 0.0f : bh.z);
                S.fin_i[pos] = make_uint4(item, miss ? kMiss : (uint32_t)key, miss ? 0u : __float_as_uint(bh.x),
                                          miss ? 0u : __float_as_uint(bh.w));
                if (MIXED) S.fin_tris[pos] = S.tris[lane];
                has = false;
            }
            n_fin += (uint32_t)__popc(dm);
        }
    }
    if (n_fin) coop_store_finished<REFINE, MIXED>(S, lane, n_fin, utris, store);
    return err;
}

}  // namespace rt
