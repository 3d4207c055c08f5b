// Ray-cast kernels (closest hit / any hit) over the BVH8, in two launch forms — one thread per ray
// (grid) and persistent warps with dynamic ray fetch — and, for the grid form, in several block sizes
// and shared-memory stack depths (the autotuner's choices; every variant computes the same hits).
#include <cuda_runtime.h>

#include <algorithm>

#include "coop_trace.cuh"
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

// Warp-cooperative persistent form (coop_trace.cuh): warps refill idle lanes once at most `refill_at` of
// their lanes still trace; triangle tests and hit refinement are spread over the warp.
template <bool ANY, bool COUNT>
__global__ void __launch_bounds__(kTraceBlock, kCoopMinBlocks) raycast_kernel(const Bvh8Node* __restrict__ nodes,
                                                              const TriRecord* __restrict__ tris, uint32_t node_count,
                                                              const Ray* __restrict__ rays, uint32_t n,
                                                              Hit* __restrict__ hits, unsigned long long* counters,
                                                              uint32_t* err_flag, uint32_t* next, uint32_t refill_at) {
    __shared__ CoopWarp warps[kTraceBlock / 32];
    __shared__ uint2 stack[kSmemStack * kTraceBlock];
    TraceCounters c{0u, 0u};
    auto load = [&](uint32_t i, TraceRay& r, CoopScene& sc) {
        const float4* rp = reinterpret_cast<const float4*>(rays) + 2ull * i;
        const float4 a = __ldcs(rp), b = __ldcs(rp + 1);
        r = make_trace_ray(a.x, a.y, a.z, b.x, b.y, b.z, a.w, b.w);
        (void)sc;
        return true;
    };
    auto store = [&](uint32_t i, const Hit& h, bool valid) {
        if (valid && hits) __stcs(reinterpret_cast<float4*>(hits) + i, make_float4(__uint_as_float(h.prim), h.t, h.u, h.v));
    };
    const uint32_t e = coop_trace<ANY, COUNT, true, false, kSmemStack>(CoopScene{nodes, tris, node_count}, n, next, refill_at,
                                                                       warps[threadIdx.x >> 5], stack + threadIdx.x,
                                                                       kTraceBlock, load, store, c);
    if (e) atomicOr(err_flag, e);
    reduce_counters<COUNT>(c, counters);
}

// One thread per ray (the hardware block scheduler balances the load at block granularity).
template <bool ANY, bool COUNT, int BLOCK, int SS>
__global__ void RT_TRACE_BOUNDS(BLOCK) raycast_kernel_grid(const Bvh8Node* __restrict__ nodes,
                                                          const TriRecord* __restrict__ tris, uint32_t node_count,
                                                          const Ray* __restrict__ rays, uint32_t n,
                                                          Hit* __restrict__ hits, unsigned long long* counters,
                                                          uint32_t* err_flag, const uint32_t* __restrict__ order) {
    __shared__ uint2 stack[SS * BLOCK];
    const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    TraceCounters c{0u, 0u};
    if (k < n) {
        const uint64_t i = order ? order[k] : k;   // thread k traces the k-th ray of the coherence order
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

// The same for two-level scenes (top level over instances, bottom levels per model).  Closest hit is
// held to 64 registers (8 blocks per SM): 4 % faster than the 80 it takes unbounded on 256 instances;
// any hit was 1 % slower when bounded, so it keeps its own allocation.
template <bool ANY, bool COUNT>
__global__ void __launch_bounds__(kTraceBlock, ANY ? 1 : 8) raycast_kernel_two_level(DeviceScene sc, const Ray* __restrict__ rays,
                                                                      uint32_t n, Hit* __restrict__ hits,
                                                                      unsigned long long* counters, uint32_t* err_flag,
                                                                      const uint32_t* __restrict__ order) {
    __shared__ uint2 stack[kSmemStack * kTraceBlock];
    const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    TraceCounters c{0u, 0u};
    if (k < n) {
        const uint64_t i = order ? order[k] : k;
        const float4* rp = reinterpret_cast<const float4*>(rays) + 2ull * i;
        const float4 a = __ldcs(rp), b = __ldcs(rp + 1);
        const TraceRay r = make_trace_ray(a.x, a.y, a.z, b.x, b.y, b.z, a.w, b.w);
        Hit h;
        uint32_t e = 0;
        if (sc.node_count) {
            e = traverse_two_level<ANY, COUNT, true, kSmemStack>(sc, r, stack + threadIdx.x, kTraceBlock, h, c);
        } else {
            h.prim = kMiss; h.t = r.tmax; h.u = 0.0f; h.v = 0.0f;
        }
        if (hits) __stcs(reinterpret_cast<float4*>(hits) + i, make_float4(__uint_as_float(h.prim), h.t, h.u, h.v));
        if (e) atomicOr(err_flag, e);
    }
    reduce_counters<COUNT>(c, counters);
}

// ------------------------------------------------------------------------------------------------
// Coherence order: rays binned by (direction octant, Morton code of the origin's cell on an 8^3 grid
// over the bounds of the ray origins), bins in Morton order, rays in input order within a bin per warp.
// Threads that trace consecutive rays of this order follow similar paths through the tree; hits are
// written to each ray's own slot, so results do not depend on the order.
constexpr int kBinBits = 12;
constexpr uint32_t kBins = 1u << kBinBits;
constexpr int kBinBlock = 256;

// Float bits mapped to an unsigned key with the same order (min/max by integer atomics).
__device__ __forceinline__ uint32_t ordered_bits(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float from_ordered(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}

// bounds[0..2] = ordered min of the origins, bounds[3..5] = ordered max (pre-set to 0xFFFFFFFF / 0).
__global__ void __launch_bounds__(kBinBlock) k_ray_bounds(const Ray* __restrict__ rays, uint32_t n,
                                                          uint32_t* __restrict__ bounds) {
    uint32_t lo[3] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu}, hi[3] = {0u, 0u, 0u};
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const float4 a = __ldg(reinterpret_cast<const float4*>(rays) + 2ull * i);
        const uint32_t k[3] = {ordered_bits(a.x), ordered_bits(a.y), ordered_bits(a.z)};
        for (int c = 0; c < 3; ++c) {
            lo[c] = min(lo[c], k[c]);
            hi[c] = max(hi[c], k[c]);
        }
    }
    for (int c = 0; c < 3; ++c)
        for (int o = 16; o > 0; o >>= 1) {
            lo[c] = min(lo[c], __shfl_xor_sync(0xFFFFFFFFu, lo[c], o));
            hi[c] = max(hi[c], __shfl_xor_sync(0xFFFFFFFFu, hi[c], o));
        }
    if ((threadIdx.x & 31) == 0)
        for (int c = 0; c < 3; ++c) {
            atomicMin(bounds + c, lo[c]);
            atomicMax(bounds + 3 + c, hi[c]);
        }
}

__device__ __forceinline__ uint32_t spread3(uint32_t v) {   // 3 bits -> bits 0, 3, 6
    return (v & 1u) | ((v & 2u) << 2) | ((v & 4u) << 4);
}

__device__ __forceinline__ uint32_t ray_bin(const Ray* rays, uint64_t i, const uint32_t* bounds) {
    const float4* rp = reinterpret_cast<const float4*>(rays) + 2ull * i;
    const float4 a = __ldg(rp), b = __ldg(rp + 1);
    const uint32_t oct = (b.x < 0.0f ? 4u : 0u) | (b.y < 0.0f ? 2u : 0u) | (b.z < 0.0f ? 1u : 0u);
    auto cell = [&](float x, int c) {
        const float lo = from_ordered(bounds[c]), hi = from_ordered(bounds[3 + c]);
        const float t = hi > lo ? (x - lo) / (hi - lo) * 8.0f : 0.0f;
        return t >= 7.0f ? 7u : (t > 0.0f ? (uint32_t)t : 0u);   // NaN -> 0
    };
    return (oct << 9) | (spread3(cell(a.x, 0)) << 2) | (spread3(cell(a.y, 1)) << 1) | spread3(cell(a.z, 2));
}

// Per-block shared histograms, added to the global one with one atomic per non-empty bin and block.
__global__ void __launch_bounds__(kBinBlock) k_ray_bins(const Ray* __restrict__ rays, uint32_t n,
                                                        const uint32_t* __restrict__ bounds, uint32_t* __restrict__ bin_of,
                                                        uint32_t* __restrict__ hist) {
    __shared__ uint32_t h[kBins];
    for (uint32_t b = threadIdx.x; b < kBins; b += blockDim.x) h[b] = 0;
    __syncthreads();
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t b = ray_bin(rays, i, bounds);
        bin_of[i] = b;
        atomicAdd(h + b, 1u);
    }
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < kBins; b += blockDim.x)
        if (h[b]) atomicAdd(hist + b, h[b]);
}

// Exclusive prefix sum of the kBins counts, in place (one block of 1024 threads, 4 bins each).
__global__ void __launch_bounds__(1024) k_bin_offsets(uint32_t* __restrict__ hist) {
    __shared__ uint32_t part[1024];
    constexpr uint32_t per = kBins / 1024;
    uint32_t local[per];
    uint32_t sum = 0;
    for (uint32_t j = 0; j < per; ++j) {
        local[j] = hist[threadIdx.x * per + j];
        sum += local[j];
    }
    part[threadIdx.x] = sum;
    __syncthreads();
    for (uint32_t off = 1; off < 1024; off <<= 1) {   // Hillis-Steele inclusive scan
        const uint32_t v = threadIdx.x >= off ? part[threadIdx.x - off] : 0u;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    uint32_t run = part[threadIdx.x] - sum;
    for (uint32_t j = 0; j < per; ++j) {
        hist[threadIdx.x * per + j] = run;
        run += local[j];
    }
}

__global__ void __launch_bounds__(kBinBlock) k_ray_scatter(const uint32_t* __restrict__ bin_of, uint32_t n,
                                                           uint32_t* __restrict__ cursor, uint32_t* __restrict__ order) {
    for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < n; base += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i = base + threadIdx.x;
        const bool valid = i < n;
        const uint32_t b = valid ? bin_of[i] : 0xFFFFFFFFu;
        const unsigned same = __match_any_sync(0xFFFFFFFFu, b);
        const int lane = threadIdx.x & 31, leader = __ffs(same) - 1;
        uint32_t pos = 0;
        if (valid && lane == leader) pos = atomicAdd(cursor + b, (uint32_t)__popc(same));
        pos = __shfl_sync(0xFFFFFFFFu, pos, leader);
        if (valid) order[pos + __popc(same & ((1u << lane) - 1u))] = (uint32_t)i;
    }
}

// Builds the coherence order of n rays in `order` (scratch: n bin ids, kBins counters, 6 bound words).
static void ray_order(const Ray* d_rays, uint64_t n, uint32_t* bin_of, uint32_t* hist, uint32_t* bounds,
                      uint32_t* order, int sm_count, cudaStream_t st) {
    const int grid = std::max(1, std::min<int>((int)((n + kBinBlock - 1) / kBinBlock), 2 * std::max(1, sm_count)));
    check_cuda(cudaMemsetAsync(hist, 0, kBins * sizeof(uint32_t), st), "cudaMemsetAsync");
    check_cuda(cudaMemsetAsync(bounds, 0xFF, 3 * sizeof(uint32_t), st), "cudaMemsetAsync");
    check_cuda(cudaMemsetAsync(bounds + 3, 0, 3 * sizeof(uint32_t), st), "cudaMemsetAsync");
    k_ray_bounds<<<grid, kBinBlock, 0, st>>>(d_rays, (uint32_t)n, bounds);
    k_ray_bins<<<grid, kBinBlock, 0, st>>>(d_rays, (uint32_t)n, bounds, bin_of, hist);
    k_bin_offsets<<<1, 1024, 0, st>>>(hist);
    k_ray_scatter<<<grid * 4, kBinBlock, 0, st>>>(bin_of, (uint32_t)n, hist, order);
}

template <bool ANY, bool COUNT>
static int persistent_grid(int sm_count) {
    static const int per_sm = [] {   // initialised once, thread-safely (a function-local static)
        int b = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, raycast_kernel<ANY, COUNT>, kTraceBlock, 0);
        return std::max(1, b);
    }();
    return per_sm * std::max(1, sm_count);
}

// Two-level scenes always run the default block size and stack depth.
template <bool ANY, bool COUNT, int BLOCK, int SS>
static void launch_grid(const DeviceScene& s, const Ray* d_rays, uint64_t n, Hit* d_hits,
                        unsigned long long* d_counters, uint32_t* d_err, const uint32_t* order, cudaStream_t st) {
    if (s.inst_trav) {
        const uint64_t blocks = (n + kTraceBlock - 1) / kTraceBlock;
        raycast_kernel_two_level<ANY, COUNT><<<(unsigned)blocks, kTraceBlock, 0, st>>>(s, d_rays, (uint32_t)n, d_hits,
                                                                                     d_counters, d_err, order);
        return;
    }
    const uint64_t blocks = (n + BLOCK - 1) / BLOCK;
    raycast_kernel_grid<ANY, COUNT, BLOCK, SS><<<(unsigned)blocks, BLOCK, 0, st>>>(
        s.nodes, s.tris, s.node_count, d_rays, (uint32_t)n, d_hits, d_counters, d_err, order);
}

template <bool ANY, int BLOCK>
static void launch_grid_stack(int stack, const DeviceScene& s, const Ray* d_rays, uint64_t n, Hit* d_hits,
                              uint32_t* d_err, const uint32_t* order, cudaStream_t st) {
    if (stack == 8) launch_grid<ANY, false, BLOCK, 8>(s, d_rays, n, d_hits, nullptr, d_err, order, st);
    else if (stack == 16) launch_grid<ANY, false, BLOCK, 16>(s, d_rays, n, d_hits, nullptr, d_err, order, st);
    else launch_grid<ANY, false, BLOCK, kSmemStack>(s, d_rays, n, d_hits, nullptr, d_err, order, st);
}

template <bool ANY>
static void launch(const DeviceScene& s, const Ray* d_rays, uint64_t n, Hit* d_hits, uint32_t* d_err, uint32_t* d_next,
                   int sm_count, const TraceConfig& cfg, cudaStream_t st) {
    // grid form (also for more than 2^31 rays, where the persistent form's fetch counter could wrap, and
    // for two-level scenes)
    if (cfg.refill <= 0 || n > (1ull << 31) || s.inst_trav) {
        uint32_t* scratch = nullptr;
        const uint32_t* order = nullptr;
        if (cfg.sort) {   // stream-ordered scratch: concurrent calls on other streams do not share it
            check_cuda(cudaMallocAsync((void**)&scratch, (2 * n + kBins + 8) * sizeof(uint32_t), st), "cudaMallocAsync");
            ray_order(d_rays, n, scratch, scratch + 2 * n, scratch + 2 * n + kBins, scratch + n, sm_count, st);
            order = scratch + n;
        }
        if (cfg.block == 64) launch_grid_stack<ANY, 64>(cfg.stack, s, d_rays, n, d_hits, d_err, order, st);
        else if (cfg.block == 256) launch_grid_stack<ANY, 256>(cfg.stack, s, d_rays, n, d_hits, d_err, order, st);
        else launch_grid_stack<ANY, kTraceBlock>(cfg.stack, s, d_rays, n, d_hits, d_err, order, st);
        if (scratch) check_cuda(cudaFreeAsync(scratch, st), "cudaFreeAsync");
        return;
    }
    const uint64_t needed = (n + kTraceBlock - 1) / kTraceBlock;
    check_cuda(cudaMemsetAsync(d_next, 0, sizeof(uint32_t), st), "cudaMemsetAsync");
    const int grid = (int)std::min<uint64_t>(needed, (uint64_t)persistent_grid<ANY, false>(sm_count));
    raycast_kernel<ANY, false><<<grid, kTraceBlock, 0, st>>>(s.nodes, s.tris, s.node_count, d_rays, (uint32_t)n, d_hits,
                                                             nullptr, d_err, d_next, (uint32_t)(32 - cfg.refill));
}

bool valid_trace_config(const TraceConfig& c) {
    const bool block_ok = c.block == 0 || c.block == 64 || c.block == 128 || c.block == 256;
    const bool stack_ok = c.stack == 0 || c.stack == 8 || c.stack == 12 || c.stack == 16;
    return block_ok && stack_ok && c.refill >= 0 && c.refill <= 32 && (c.sort == 0 || c.sort == 1);
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
    if (n == 0) return;
    // The counting build of the default form: the cooperative form for flat scenes (its deferred triangle
    // tests cull later, so it may visit a few more nodes than the grid form), the grid form otherwise.
    if (s.inst_trav || n > (1ull << 31)) {
        if (any) launch_grid<true, true, kTraceBlock, kSmemStack>(s, d_rays, n, nullptr, d_counters, d_err, nullptr, st);
        else launch_grid<false, true, kTraceBlock, kSmemStack>(s, d_rays, n, nullptr, d_counters, d_err, nullptr, st);
        return;
    }
    check_cuda(cudaMemsetAsync(d_next, 0, sizeof(uint32_t), st), "cudaMemsetAsync");
    const uint64_t needed = (n + kTraceBlock - 1) / kTraceBlock;
    const uint32_t refill_at = (uint32_t)(32 - kDefaultRefill);
    if (any) {
        const int grid = (int)std::min<uint64_t>(needed, (uint64_t)persistent_grid<true, true>(sm_count));
        raycast_kernel<true, true><<<grid, kTraceBlock, 0, st>>>(s.nodes, s.tris, s.node_count, d_rays, (uint32_t)n,
                                                                 nullptr, d_counters, d_err, d_next, refill_at);
    } else {
        const int grid = (int)std::min<uint64_t>(needed, (uint64_t)persistent_grid<false, true>(sm_count));
        raycast_kernel<false, true><<<grid, kTraceBlock, 0, st>>>(s.nodes, s.tris, s.node_count, d_rays, (uint32_t)n,
                                                                  nullptr, d_counters, d_err, d_next, refill_at);
    }
}

}  // namespace rt
