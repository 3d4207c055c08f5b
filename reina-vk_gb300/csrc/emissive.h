// Emissive CDFs on the GPU: Instance::computeCDF (src/scene/Instance.cpp:15-53) for every emissive
// instance of a scene, and the duplicate search of Instances::computeSamplingDataEmissives
// (src/scene/Instances.cpp:52-90), with results bit-identical to the host build in scene.cpp.
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

namespace rt {

struct EmissiveInput {
    const float* vertices = nullptr;   // model vertices, xyzw
    size_t nv = 0;
    const uint32_t* indices = nullptr;
    size_t ntri = 0;
    uint32_t model = 0;                // instances of one model share its upload
    float transform[16];               // column-major instance transform
    float brightness = 0.0f;           // luminance of the emission
};

struct EmissiveOutput {
    std::vector<float> cdf;            // normalized cumulative area x brightness, one entry per triangle
    float area = 0.0f;                 // sum of the triangle areas, in the host's order
    float weight = 0.0f;               // cumulative area x brightness before normalization
};

// Builds the CDFs of `in` on `device`, and for every pair i < j of equal triangle count whether the two
// CDFs agree within `tol` on every entry (same[i * n + j]).  A zero weight is returned as is (the
// caller rejects it).  Synchronous.
void emissive_cdfs_device(int device, const std::vector<EmissiveInput>& in, float tol, std::vector<EmissiveOutput>& out,
                          std::vector<uint8_t>& same);

}  // namespace rt
