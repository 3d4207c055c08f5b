// Ray-cast kernels (closest hit / any hit) over the BVH8, one thread per ray.
#include <cuda_runtime.h>

#include "kernels.h"
#include "trace_device.cuh"

namespace rt {

template <bool ANY, bool COUNT>
__global__ void __launch_bounds__(kTraceBlock) raycast_kernel(const Bvh8Node* __restrict__ nodes,
                                                             const TriRecord* __restrict__ tris,
                                                             uint32_t node_count, const Ray* __restrict__ rays,
                                                             uint64_t n, Hit* __restrict__ hits,
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

void launch_raycast(const DeviceScene& s, const Ray* d_rays, uint64_t n, Hit* d_hits, bool any,
                    uint32_t* d_err, cudaStream_t st) {
    if (n == 0) return;
    const uint64_t blocks = (n + kTraceBlock - 1) / kTraceBlock;
    if (any)
        raycast_kernel<true, false><<<(unsigned)blocks, kTraceBlock, 0, st>>>(s.nodes, s.tris, s.node_count, d_rays, n,
                                                                             d_hits, nullptr, d_err);
    else
        raycast_kernel<false, false><<<(unsigned)blocks, kTraceBlock, 0, st>>>(s.nodes, s.tris, s.node_count, d_rays, n,
                                                                              d_hits, nullptr, d_err);
}

void launch_raycast_counters(const DeviceScene& s, const Ray* d_rays, uint64_t n, bool any,
                             unsigned long long* d_counters, uint32_t* d_err, cudaStream_t st) {
    if (n == 0) return;
    const uint64_t blocks = (n + kTraceBlock - 1) / kTraceBlock;
    if (any)
        raycast_kernel<true, true><<<(unsigned)blocks, kTraceBlock, 0, st>>>(s.nodes, s.tris, s.node_count, d_rays, n,
                                                                            nullptr, d_counters, d_err);
    else
        raycast_kernel<false, true><<<(unsigned)blocks, kTraceBlock, 0, st>>>(s.nodes, s.tris, s.node_count, d_rays, n,
                                                                             nullptr, d_counters, d_err);
}

}  // namespace rt
