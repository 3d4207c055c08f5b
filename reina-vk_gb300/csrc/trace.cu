// Ray-cast kernels (closest hit / any hit) over the BVH8, in two launch forms — one thread per ray
// (grid) and persistent warps with dynamic ray fetch — and, for the grid form, in several block sizes
// and shared-memory stack depths (the autotuner's choices; every variant computes the same hits).
#include <cuda_runtime.h>

#include <algorithm>

#include "kernels.h"
#include "trace_device.cuh"

namespace rt {

static_assert(kSmemStack == kDefaultTraceStack, "default traversal stack depth");

// Minimum resident blocks per SM requested from the compiler (register cap), when set.
#ifdef RT_TRACE_MINB
#define RT_TRACE_BOUNDS(B) __launch_bounds__(B, RT_TRACE_MINB)
#else
#define RT_TRACE_BOUNDS(B) __launch_bounds__(B)
#endif

template <bool COUNT>
__device__ __forceinline__ void reduce_counters(const TraceCounters& c, unsigned long long* counters) {
    if (COUNT) {
        unsigned long long nodes_v = c.nodes, tris_v = c.tris;
        for (int o = 16; o > 0; o >>= 1) {
            nodes_v += __shfl_down_sync(0xFFFFFFFFu, nodes_v, o);
            tris_v += __shfl_down_sync(0xFFFFFFFFu, tris_v, o);
        }
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(counters + 0, nodes_v);
            atomicAdd(counters + 1, tris_v);
        }
    }
}

template <bool ANY, bool COUNT>
__global__ void RT_TRACE_BOUNDS(kTraceBlock) raycast_kernel(const Bvh8Node* __restrict__ nodes,
                                                           const TriRecord* __restrict__ tris, uint32_t node_count,
                                                           const Ray* __restrict__ rays, uint32_t n,
                                                           Hit* __restrict__ hits, unsigned long long* counters,
                                                           uint32_t* err_flag, uint32_t* next, int refill) {
    __shared__ uint2 stack[kSmemStack * kTraceBlock];
    TraceCounters c{0u, 0u};
    auto load = [&](uint32_t i, TraceRay& r) {
        const float4* rp = reinterpret_cast<const float4*>(rays) + 2ull * i;
        const float4 a = __ldcs(rp), b = __ldcs(rp + 1);
        r = make_trace_ray(a.x, a.y, a.z, b.x, b.y, b.z, a.w, b.w);
        return true;
    };
    auto store = [&](uint32_t i, const Hit& h, bool valid) {
        if (valid && hits) __stcs(reinterpret_cast<float4*>(hits) + i, make_float4(__uint_as_float(h.prim), h.t, h.u, h.v));
    };
    const uint32_t e = persistent_trace<ANY, COUNT, true>(nodes, tris, node_count, n, next, stack + threadIdx.x,
                                                         kTraceBlock, refill, load, store, c);
    if (e) atomicOr(err_flag, e);
    reduce_counters<COUNT>(c, counters);
}

// One thread per ray (the hardware block scheduler balances the load at block granularity).
template <bool ANY, bool COUNT, int BLOCK, int SS>
__global__ void RT_TRACE_BOUNDS(BLOCK) raycast_kernel_grid(const Bvh8Node* __restrict__ nodes,
                                                          const TriRecord* __restrict__ tris, uint32_t node_count,
                                                          const Ray* __restrict__ rays, uint32_t n,
                                                          Hit* __restrict__ hits, unsigned long long* counters,
                                                          uint32_t* err_flag) {
    __shared__ uint2 stack[SS * BLOCK];
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    TraceCounters c{0u, 0u};
    if (i < n) {
        const float4* rp = reinterpret_cast<const float4*>(rays) + 2ull * i;
        const float4 a = __ldcs(rp), b = __ldcs(rp + 1);
        const TraceRay r = make_trace_ray(a.x, a.y, a.z, b.x, b.y, b.z, a.w, b.w);
        Hit h;
        uint32_t e = 0;
        if (node_count) {
            e = traverse<ANY, COUNT, true, SS>(nodes, tris, r, stack + threadIdx.x, BLOCK, h, c);
        } else {
            h.prim = kMiss; h.t = r.tmax; h.u = 0.0f; h.v = 0.0f;
        }
        if (hits) __stcs(reinterpret_cast<float4*>(hits) + i, make_float4(__uint_as_float(h.prim), h.t, h.u, h.v));
        if (e) atomicOr(err_flag, e);
    }
    reduce_counters<COUNT>(c, counters);
}

template <bool ANY, bool COUNT>
static int persistent_grid(int sm_count) {
    static int per_sm = -1;
    if (per_sm < 0) {
        int b = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, raycast_kernel<ANY, COUNT>, kTraceBlock, 0);
        per_sm = std::max(1, b);
    }
    return per_sm * std::max(1, sm_count);
}

template <bool ANY, bool COUNT, int BLOCK, int SS>
static void launch_grid(const DeviceScene& s, const Ray* d_rays, uint64_t n, Hit* d_hits,
                        unsigned long long* d_counters, uint32_t* d_err, cudaStream_t st) {
    const uint64_t blocks = (n + BLOCK - 1) / BLOCK;
    raycast_kernel_grid<ANY, COUNT, BLOCK, SS><<<(unsigned)blocks, BLOCK, 0, st>>>(s.nodes, s.tris, s.node_count, d_rays,
                                                                                 (uint32_t)n, d_hits, d_counters, d_err);
}

template <bool ANY, int BLOCK>
static void launch_grid_stack(int stack, const DeviceScene& s, const Ray* d_rays, uint64_t n, Hit* d_hits,
                              uint32_t* d_err, cudaStream_t st) {
    if (stack == 8) launch_grid<ANY, false, BLOCK, 8>(s, d_rays, n, d_hits, nullptr, d_err, st);
    else if (stack == 16) launch_grid<ANY, false, BLOCK, 16>(s, d_rays, n, d_hits, nullptr, d_err, st);
    else launch_grid<ANY, false, BLOCK, kSmemStack>(s, d_rays, n, d_hits, nullptr, d_err, st);
}

template <bool ANY>
static void launch(const DeviceScene& s, const Ray* d_rays, uint64_t n, Hit* d_hits, uint32_t* d_err, uint32_t* d_next,
                   int sm_count, const TraceConfig& cfg, cudaStream_t st) {
    // grid form (also for more than 2^31 rays, where the persistent form's fetch counter could wrap)
    if (cfg.refill <= 0 || n > (1ull << 31)) {
        if (cfg.block == 64) launch_grid_stack<ANY, 64>(cfg.stack, s, d_rays, n, d_hits, d_err, st);
        else if (cfg.block == 256) launch_grid_stack<ANY, 256>(cfg.stack, s, d_rays, n, d_hits, d_err, st);
        else launch_grid_stack<ANY, kTraceBlock>(cfg.stack, s, d_rays, n, d_hits, d_err, st);
        return;
    }
    const uint64_t needed = (n + kTraceBlock - 1) / kTraceBlock;
    check_cuda(cudaMemsetAsync(d_next, 0, sizeof(uint32_t), st), "cudaMemsetAsync");
    const int grid = (int)std::min<uint64_t>(needed, (uint64_t)persistent_grid<ANY, false>(sm_count));
    raycast_kernel<ANY, false><<<grid, kTraceBlock, 0, st>>>(s.nodes, s.tris, s.node_count, d_rays, (uint32_t)n, d_hits,
                                                             nullptr, d_err, d_next, cfg.refill);
}

bool valid_trace_config(const TraceConfig& c) {
    const bool block_ok = c.block == 0 || c.block == 64 || c.block == 128 || c.block == 256;
    const bool stack_ok = c.stack == 0 || c.stack == 8 || c.stack == 12 || c.stack == 16;
    return block_ok && stack_ok && c.refill >= 0 && c.refill <= 32;
}

void launch_raycast(const DeviceScene& s, const Ray* d_rays, uint64_t n, Hit* d_hits, bool any, uint32_t* d_err,
                    uint32_t* d_next, int sm_count, const TraceConfig& cfg, cudaStream_t st) {
    if (n == 0) return;
    if (!valid_trace_config(cfg)) fail(REINA_ERR_INVALID, "invalid traversal launch configuration");
    if (any) launch<true>(s, d_rays, n, d_hits, d_err, d_next, sm_count, cfg, st);
    else launch<false>(s, d_rays, n, d_hits, d_err, d_next, sm_count, cfg, st);
}

void launch_raycast_counters(const DeviceScene& s, const Ray* d_rays, uint64_t n, bool any,
                             unsigned long long* d_counters, uint32_t* d_err, uint32_t* d_next, int sm_count,
                             cudaStream_t st) {
    (void)d_next;
    (void)sm_count;
    if (n == 0) return;
    // The counting build uses the default grid form: visit counts do not depend on block size or stack
    // depth (warps hold the same 32 consecutive rays in every grid variant).
    if (any) launch_grid<true, true, kTraceBlock, kSmemStack>(s, d_rays, n, nullptr, d_counters, d_err, st);
    else launch_grid<false, true, kTraceBlock, kSmemStack>(s, d_rays, n, nullptr, d_counters, d_err, st);
}

}  // namespace rt
