// Plain-pointer view of a built scene in device memory, passed by value to the kernels.
#pragma once

#include <stdint.h>

#include <vector_types.h>

#include "rt_common.h"
#include "../../include/reina/polyglot.h"

namespace rt {

// Per-instance data for hit reconstruction (the gl_ObjectToWorldEXT of the reference, plus the
// normal matrix transpose(inverse(mat3(M))) that closestHitCommon.h.glsl:131-132 computes per hit).
struct alignas(16) InstanceGpu {
    float m[12];          // object-to-world, row-major 3x4: world_r = sum_c m[r*4+c] * p_c + m[r*4+3]
    float nrm[9];         // normal matrix, row-major 3x3
    uint32_t props;       // InstanceProperties index used by faces without a per-face material
    uint32_t first_prim;  // global triangle id of the object's primitive 0
    uint32_t object;      // object (model) id
    float light_weight;   // emissive weight (Σ area·luminance, src/scene/Instance.cpp:15-53), 0 if not emissive
    float light_area;     // emissive area of the instance, 0 if not emissive
};

struct DeviceScene {
    // traversal
    const Bvh8Node* nodes = nullptr;
    const TriRecord* tris = nullptr;
    uint32_t node_count = 0;
    uint32_t tri_count = 0;
    // global model buffers, identical in content to the reference's (src/scene/Models.cpp:24-92)
    const float* vertices = nullptr;        // 4 per vertex
    const uint32_t* indices = nullptr;      // offset by firstVertex
    const float* tbns = nullptr;            // 9 per entry, column-major
    const uint32_t* tbn_indices = nullptr;  // offset by the model's first TBN
    const float* tex_coords = nullptr;      // 2 per entry
    const uint32_t* tex_indices = nullptr;  // offset by the model's first texcoord (0xFFFFFFFF kept)
    // instances
    const InstanceProperties* props = nullptr;
    const InstanceGpu* instances = nullptr;
    const uint32_t* prim_instance = nullptr;  // per global triangle
    const uint32_t* prim_props = nullptr;     // per global triangle: InstanceProperties index
    const uint32_t* props_material = nullptr; // per InstanceProperties: material_idx (the SBT offset)
    const uint8_t* has_tbn = nullptr;         // per object: 1 if the model supplied TBN data
    uint32_t instance_count = 0;
    uint32_t props_count = 0;
    // emissive sampling data (src/scene/Instances.cpp:129-191, packed as in :197-232)
    const EmissiveInstanceData* emissive = nullptr;
    const float* cdf_triangles = nullptr;
    const float* cdf_instances = nullptr;     // numInstances entries
    uint32_t emissive_count = 0;
    float emissive_weight = 0.0f;             // the `allInstancesArea` field = Σ weights
    // two-level scenes: per-instance traversal records and the top-level leaf entries (instance ids);
    // null for a flat scene (one BVH over world-space triangles)
    const InstanceTrav* inst_trav = nullptr;
    const uint32_t* tlas_refs = nullptr;
    // textures (src/scene/Scene.cpp:59-80; sampled as R8G8B8A8_UNORM, src/graphics/Image.cpp:56)
    const uint32_t* tex_texels = nullptr;     // RGBA8 texels of all textures, one word each
    const uint4* tex_info = nullptr;          // per texture: first texel, width, height, 0
    uint32_t tex_count = 0;
    float bounds_lo[3] = {0.0f, 0.0f, 0.0f};  // world-space triangle bounds (ray binning frame)
    float bounds_hi[3] = {0.0f, 0.0f, 0.0f};
};

}  // namespace rt
