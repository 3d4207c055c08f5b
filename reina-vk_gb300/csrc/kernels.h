// Host-callable launchers of the CUDA kernels (implemented in the .cu files).
#pragma once

#include <cstdint>

#include <cuda_runtime_api.h>

#include "device_scene.h"
#include "errors.h"
#include "rt_common.h"

namespace rt {

constexpr int kTraceBlock = 128;
// Traversal launch form: 0 = one thread per ray (grid); 1..32 = the warp-cooperative persistent form
// (coop_trace.cuh), whose warps fetch new rays once this many of their 32 lanes are idle.  The
// cooperative form is the default for flat scenes (two-level scenes always run the grid form): on the
// 1.3M-triangle ray cast, closest hit 0.58 ms against 0.82 ms for the grid form, any hit 0.36 / 0.51 ms.
constexpr int kDefaultRefill = 8;
// Launch form of the wavefront extension and shadow kernels (renders, batches, the server): the grid
// form.  The cooperative form's refill costs more than it saves there, where a wave's queue holds many
// paths per scene and rays of one bounce are coherent: 1920x1080 64-spp frame of the 1.3M-triangle scene
// 318 ms grid against 352 ms cooperative (refill 8), 256x256 Cornell room 2.48 against 3.79 ms.
constexpr int kDefaultWaveRefill = 0;

// Launch configuration of the traversal kernels: block size (64, 128, 256) and shared-memory stack
// entries per thread (8, 12, 16) of the grid form, or the cooperative persistent form with its refill
// threshold (refill > 0; block 128, stack 12).
constexpr int kDefaultTraceStack = 12;
struct TraceConfig {
    int block = kTraceBlock;
    int stack = kDefaultTraceStack;
    int refill = kDefaultRefill;
    int sort = 0;                 // ray casts (grid form): 1 = trace the rays in coherence order
};
bool valid_trace_config(const TraceConfig& c);

// `d_next` is a device u32 used as the ray-fetch counter (reset by the launcher); n < 2^32.
void launch_raycast(const DeviceScene& s, const Ray* d_rays, uint64_t n, Hit* d_hits, bool any, uint32_t* d_err,
                    uint32_t* d_next, int sm_count, const TraceConfig& cfg, cudaStream_t st);
void launch_raycast_counters(const DeviceScene& s, const Ray* d_rays, uint64_t n, bool any,
                             unsigned long long* d_counters, uint32_t* d_err, uint32_t* d_next, int sm_count,
                             cudaStream_t st);

}  // namespace rt
