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
    uint32_t face_base;   // per-face instances: first entry in DeviceScene::face_props; else 0xFFFFFFFF
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
    const uint32_t* prim_instance = nullptr;  // per global triangle (flat scenes; null in two-level scenes)
    const uint32_t* prim_props = nullptr;     // per global triangle: InstanceProperties index (flat scenes)
    const uint32_t* face_props = nullptr;     // per-face instances' InstanceProperties ids, concatenated
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

#if defined(__CUDACC__)
// Instance and InstanceProperties index of global triangle `prim`: the per-triangle tables of a flat
// scene, or (two-level scenes, which keep no per-triangle tables) a binary search over the instances'
// first triangles and the instance's material or per-face table.
__device__ __forceinline__ void prim_lookup(const DeviceScene& s, uint32_t prim, uint32_t& inst, uint32_t& props) {
    if (s.prim_instance) {
        inst = s.prim_instance[prim];
        props = s.prim_props[prim];
        return;
    }
    uint32_t lo = 0, hi = s.instance_count - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) / 2;
        if (s.instances[mid].first_prim <= prim) lo = mid;
        else hi = mid - 1;
    }
    inst = lo;
    const InstanceGpu& g = s.instances[lo];
    props = g.face_base == 0xFFFFFFFFu ? g.props : s.face_props[g.face_base + (prim - g.first_prim)];
}
__device__ __forceinline__ uint32_t prim_props_of(const DeviceScene& s, uint32_t prim) {
    uint32_t inst, props;
    prim_lookup(s, prim, inst, props);
    return props;
}
#endif

}  // namespace rt
