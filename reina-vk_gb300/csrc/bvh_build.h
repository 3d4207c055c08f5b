// Host BVH builder: binned-SAH binary BVH -> 8-wide collapse -> conservatively quantized BVH8 nodes.
// Replaces the opaque driver builds of the reference (BLAS per model, src/graphics/Blas.cpp:41-113;
// TLAS over instances, src/tools/vktools.cpp:460-596) with an explicit structure that software
// traversal on the GB300 can read.
#pragma once

#include <cstdint>
#include <vector>

#include "bvh_sah.h"
#include "rt_common.h"

namespace rt {

struct Bvh8 {
    std::vector<Bvh8Node> nodes;   // node 0 is the root (empty vector for an empty scene)
    std::vector<TriRecord> tris;   // leaf-ordered traversal triangles
    uint32_t depth = 0;            // number of BVH8 levels
    uint32_t binary_nodes = 0;
    double seconds = 0.0;
};

// How the binary BVH is collapsed into 8-wide nodes: greedily (open the largest-area internal child until
// 8 children), or by the SAH-optimal dynamic programme of Ylitie, Karras and Laine (HPG 2017, section
// 3.1), which also merges subtrees of up to 3 triangles into one leaf child.
enum BvhCollapse : int { kCollapseGreedy = 0, kCollapseSahDp = 1 };
#ifndef RT_COLLAPSE
#define RT_COLLAPSE 1
#endif

struct BvhBuildOptions {
    int sah_bins = 32;
    int max_threads = 0;           // 0 = std::thread::hardware_concurrency()
    int collapse = RT_COLLAPSE;
    int median_depth = sah::kForceMedianDepth;   // binary depth from which every split is an object median
};

// `verts` holds 9 floats per triangle (v0, v1, v2 in world space); triangle i gets id i.
Bvh8 build_bvh8(const float* verts, uint64_t tri_count, const BvhBuildOptions& opt = BvhBuildOptions());

// BVH8 over axis-aligned boxes (6 floats each: lo x, y, z, hi x, y, z), for the top level of a two-level
// scene: leaf children reference boxes instead of triangles — their entries (box indices) are appended
// to `refs`, and a leaf child's offset indexes refs from the node's tri_base.  The result has no
// triangle records.
Bvh8 build_bvh8_boxes(const float* boxes6, uint64_t box_count, std::vector<uint32_t>& refs,
                      const BvhBuildOptions& opt = BvhBuildOptions());

// Maximum BVH8 depth the traversal kernels accept (their stack holds one entry per level).
constexpr uint32_t kMaxBvhDepth = 64;
// Largest quantization exponent of a node (scale 2^e): the traversal forms 2^(e+15) in single precision.
constexpr int kMaxQuantExponent = sah::kMaxQuantExponent;

// The same BVH8 built on the GPU `device` (bvh_gpu.cu): byte-identical nodes and triangle records for the
// same input and options (SAH collapse only, at most 64 bins).  `kernel_seconds` receives the device
// time of the build kernels.  Synchronous.
Bvh8 build_bvh8_device(int device, const float* verts, uint64_t tri_count, const BvhBuildOptions& opt = BvhBuildOptions(),
                       double* kernel_seconds = nullptr);
constexpr int kMaxDeviceSahBins = 64;

}  // namespace rt
