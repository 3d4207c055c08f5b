// Host-callable launchers of the CUDA kernels (implemented in the .cu files).
#pragma once

#include <cstdint>

#include <cuda_runtime_api.h>

#include "device_scene.h"
#include "rt_common.h"

namespace rt {

constexpr int kTraceBlock = 128;

void launch_raycast(const DeviceScene& s, const Ray* d_rays, uint64_t n, Hit* d_hits, bool any,
                    uint32_t* d_err, cudaStream_t st);
void launch_raycast_counters(const DeviceScene& s, const Ray* d_rays, uint64_t n, bool any,
                             unsigned long long* d_counters, uint32_t* d_err, cudaStream_t st);

}  // namespace rt
