// Device self-check of single shading functions (kat.cu).
#pragma once

#include <cstdint>

#include <cuda_runtime_api.h>

namespace rt {

constexpr int kKatRecordFloats = 40;
void launch_kat(int kind, const float* d_records, uint32_t n, float* d_out, cudaStream_t st);

}  // namespace rt
