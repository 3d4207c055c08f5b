// Post-process (bloom + ACES tone map) launcher and its intermediate images.
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime_api.h>

#include "errors.h"
#include "../../include/reina/polyglot.h"

namespace rt {

struct PostWorkspace {
    DeviceBuffer ping, pong, weights;
    void ensure(size_t pixels, int k);

private:
    size_t cap_px_ = 0, cap_w_ = 0;
};

// accum (W*H RGBA32F) -> rgba8 (W*H*4 bytes); `d_combined` (optional) receives the bloomed HDR image.
void postprocess(PostWorkspace& ws, const float* d_accum, int W, int H, const BloomPushConsts& bloom,
                 const TonemappingPushConsts& tm, uint8_t* d_rgba8, float* d_combined, int sm_count, cudaStream_t st);

}  // namespace rt
