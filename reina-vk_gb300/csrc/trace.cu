// Ray-cast kernels (closest hit / any hit) over the BVH8: persistent warps with dynamic ray fetch.
#include <cuda_runtime.h>

#include <algorithm>

#include "kernels.h"
#include "trace_device.cuh"

namespace rt {

template <bool ANY, bool COUNT>
__global__ void __launch_bounds__(kTraceBlock) raycast_kernel(const Bvh8Node* __restrict__ nodes,
                                                             const TriRecord* __restrict__ tris,
                                                             uint32_t node_count, const Ray* __restrict__ rays,
                                                             uint32_t n, Hit* __restrict__ hits,
                                                             unsigned long long* counters, uint32_t* err_flag,
                                                             uint32_t* next, int refill) {
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

// One thread per ray (the hardware block scheduler balances the load at block granularity).
template <bool ANY, bool COUNT>
__global__ void __launch_bounds__(kTraceBlock) raycast_kernel_grid(const Bvh8Node* __restrict__ nodes,
                                                                  const TriRecord* __restrict__ tris,
                                                                  uint32_t node_count, const Ray* __restrict__ rays,
                                                                  uint32_t n, Hit* __restrict__ hits,
                                                                  unsigned long long* counters, uint32_t* err_flag) {
    __shared__ uint2 stack[kSmemStack * kTraceBlock];
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    TraceCounters c{0u, 0u};
    if (i < n) {
        const float4* rp = reinterpret_cast<const float4*>(rays) + 2ull * i;
        const float4 a = __ldcs(rp), b = __ldcs(rp + 1);
        const TraceRay r = make_trace_ray(a.x, a.y, a.z, b.x, b.y, b.z, a.w, b.w);
        Hit h;
        uint32_t e = 0;
        if (node_count) {
            e = traverse<ANY, COUNT>(nodes, tris, r, stack + threadIdx.x, kTraceBlock, h, c);
        } else {
            h.prim = kMiss; h.t = r.tmax; h.u = 0.0f; h.v = 0.0f;
        }
        if (hits) __stcs(reinterpret_cast<float4*>(hits) + i, make_float4(__uint_as_float(h.prim), h.t, h.u, h.v));
        if (e) atomicOr(err_flag, e);
    }
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
static int raycast_grid(int sm_count) {
    static int per_sm = -1;
    if (per_sm < 0) {
        int b = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, raycast_kernel<ANY, COUNT>, kTraceBlock, 0);
        per_sm = std::max(1, b);
    }
    return per_sm * std::max(1, sm_count);
}

template <bool ANY, bool COUNT>
static void launch(const DeviceScene& s, const Ray* d_rays, uint64_t n, Hit* d_hits, unsigned long long* d_counters,
                   uint32_t* d_err, uint32_t* d_next, int sm_count, int refill, cudaStream_t st) {
    const uint64_t needed = (n + kTraceBlock - 1) / kTraceBlock;
    if (refill <= 0) {   // grid form
        raycast_kernel_grid<ANY, COUNT><<<(unsigned)needed, kTraceBlock, 0, st>>>(s.nodes, s.tris, s.node_count, d_rays,
                                                                               (uint32_t)n, d_hits, d_counters, d_err);
        return;
    }
    check_cuda(cudaMemsetAsync(d_next, 0, sizeof(uint32_t), st), "cudaMemsetAsync");
    const int grid = (int)std::min<uint64_t>(needed, (uint64_t)raycast_grid<ANY, COUNT>(sm_count));
    raycast_kernel<ANY, COUNT><<<grid, kTraceBlock, 0, st>>>(s.nodes, s.tris, s.node_count, d_rays, (uint32_t)n, d_hits,
                                                             d_counters, d_err, d_next, refill);
}

void launch_raycast(const DeviceScene& s, const Ray* d_rays, uint64_t n, Hit* d_hits, bool any, uint32_t* d_err,
                    uint32_t* d_next, int sm_count, int refill, cudaStream_t st) {
    if (n == 0) return;
    if (any) launch<true, false>(s, d_rays, n, d_hits, nullptr, d_err, d_next, sm_count, refill, st);
    else launch<false, false>(s, d_rays, n, d_hits, nullptr, d_err, d_next, sm_count, refill, st);
}

void launch_raycast_counters(const DeviceScene& s, const Ray* d_rays, uint64_t n, bool any,
                             unsigned long long* d_counters, uint32_t* d_err, uint32_t* d_next, int sm_count,
                             cudaStream_t st) {
    if (n == 0) return;
    // the counting build uses the grid form: its visit counts do not depend on the launch form
    if (any) launch<true, true>(s, d_rays, n, nullptr, d_counters, d_err, d_next, sm_count, 0, st);
    else launch<false, true>(s, d_rays, n, nullptr, d_counters, d_err, d_next, sm_count, 0, st);
}

}  // namespace rt
