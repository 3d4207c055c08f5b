// Scene assembly on the host (the reference's Scene/Models/Instance/Instances classes) and the upload
// of the assembled buffers plus the BVH8 to the GPU.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "bvh_build.h"
#include "device_scene.h"
#include "errors.h"
#include "image.h"

namespace rt {

// ModelData (src/scene/Models.h:23-30).
struct ModelData {
    std::vector<float> vertices;        // 4 per vertex
    std::vector<uint32_t> indices;
    std::vector<float> tbns;            // 9 per entry (column-major T, B, N)
    std::vector<uint32_t> tbn_indices;
    std::vector<float> tex_coords;      // 2 per entry
    std::vector<uint32_t> tex_indices;
};

// ModelRange (src/scene/Models.h:9-18).
struct ModelRange {
    uint32_t first_vertex, first_normal, index_offset, tbns_index_offset, tex_index_offset;
    uint32_t index_count, tbns_index_count, tex_index_count;
};

// One emissive instance's sampling data before packing (src/scene/Instance.cpp:5-53).
struct EmissiveInfo {
    bool emissive = false;
    std::vector<float> cdf;
    float area = 0.0f;
    float weight = 0.0f;
};

struct InstanceRecord {
    uint32_t object = 0;
    uint32_t props_id = 0;         // instanceCustomIndex (src/tools/vktools.cpp:481)
    uint32_t material_idx = 0;     // SBT offset (src/tools/vktools.cpp:483)
    float transform[16];           // column-major object-to-world
    bool per_face = false;
    std::vector<uint32_t> face_props;   // per-face InstanceProperties ids when per_face
    EmissiveInfo light;
    uint32_t first_prim = 0;
};

class Scene {
public:
    explicit Scene(int device) : device_(device) {}

    uint32_t define_object(ModelData&& model);
    // Scene::defineTexture (src/scene/Scene.cpp:15-25): RGBA8 texels, first row at v = 0.  Returns the id
    // materials refer to (texture_id, normal_map_id, bump_map_id).
    uint32_t define_texture(Image&& image);
    size_t texture_count() const { return textures_.size(); }
    const Image& texture(uint32_t id) const;
    void add_instance(uint32_t object, const float transform[16], const reina_material& mat);
    void add_instance_per_face(uint32_t object, const float transform[16], const reina_material* mats,
                               uint32_t mat_count, const uint32_t* face_material);
    void build(bool require_emissive);
    // Acceleration structure (REINA_ACCEL_*): one BVH over world-space triangles, or a top level over
    // instances with one bottom level per model; set before the build.
    void set_accel(int mode);
    // Where build() computes the emissive CDFs and their duplicate search: the host (default) or the
    // scene's GPU (emissive.cu); both give the same bits.
    void set_emissive_on_device(bool on) { emissive_device_ = on; }
    bool emissive_on_device() const { return emissive_device_; }
    double emissive_seconds() const { return emissive_seconds_; }
    // Where build() builds the triangle BVHs (the flat BVH, or every bottom level of a two-level scene;
    // the top level over instance boxes stays on the host): the host (default) or the scene's GPU
    // (bvh_gpu.cu); both give the same bytes.  `opt` carries the SAH bin count and the median depth.
    void set_bvh_build(bool on_device, const BvhBuildOptions& opt) {
        bvh_device_ = on_device;
        bvh_opt_ = opt;
    }
    bool bvh_on_device() const { return bvh_device_; }
    double bvh_kernel_seconds() const { return bvh_kernel_seconds_; }
    bool two_level() const { return two_level_; }
    uint32_t blas_count() const { return blas_count_; }
    const std::vector<InstanceTrav>& instance_records() const { return inst_trav_; }
    const std::vector<uint32_t>& tlas_refs() const { return tlas_refs_; }

    bool built() const { return built_; }
    float emissive_weight() const { return emissive_total_; }
    const DeviceScene& device_view() const { return dev_; }
    const Bvh8& bvh() const { return bvh_; }
    uint64_t triangle_count() const { return tri_total_; }
    size_t instance_count() const { return instances_.size(); }
    size_t device_bytes() const;
    // Device residency (used by the request server's LRU): the host keeps every assembled buffer, so a
    // released scene can be uploaded again.  upload_bytes() is the device memory an upload takes.
    bool resident() const { return resident_; }
    size_t upload_bytes() const;
    void upload();
    void release_device();
    int device() const { return device_; }
    void prim_info(uint32_t prim, uint32_t* inst, uint32_t* local) const;
    size_t object_count() const { return models_.size(); }
    const ModelData& model(uint32_t object) const;
    void bounds(float lo[3], float hi[3]) const;

    // Host copies of the assembled buffers (as uploaded), used by the C ABI's inspection calls.
    const std::vector<InstanceProperties>& instance_properties() const { return props_; }
    const std::vector<EmissiveInstanceData>& emissive_data() const { return emissive_data_; }
    const std::vector<float>& cdf_triangles() const { return cdf_triangles_; }
    const std::vector<float>& cdf_instances() const { return cdf_instances_; }

private:
    InstanceProperties make_props(uint32_t object, const reina_material& mat) const;
    void compute_emissive(InstanceRecord& inst, const float emission[3]);
    void compute_emissives_device();
    // `same` (optional, from the device build): same[i * n + j] for emissive positions i < j.
    void pack_emissives(const std::vector<uint8_t>* same = nullptr);
    bool use_two_level() const;
    void build_flat();
    void build_two_level();

    int device_;
    bool built_ = false;
    bool resident_ = false;
    // Models (src/scene/Models.cpp)
    std::vector<ModelData> models_;
    std::vector<ModelRange> ranges_;
    std::vector<float> all_vertices_, all_tbns_, all_tex_coords_;
    std::vector<uint32_t> all_indices_offset_, all_tex_indices_offset_, all_tbns_indices_offset_, all_indices_non_offset_;
    // Instances
    std::vector<InstanceProperties> props_;
    std::vector<uint32_t> props_material_;
    std::vector<InstanceRecord> instances_;
    // Emissive packing (src/scene/Instances.cpp)
    std::vector<EmissiveInstanceData> emissive_data_;
    std::vector<float> cdf_triangles_, cdf_instances_;
    float emissive_total_ = 0.0f;
    // Flattened traversal data
    uint64_t tri_total_ = 0;
    std::vector<uint32_t> prim_instance_, prim_props_;
    float bounds_lo_[3] = {0, 0, 0}, bounds_hi_[3] = {0, 0, 0};
    Bvh8 bvh_;
    std::vector<InstanceGpu> inst_gpu_;
    std::vector<uint8_t> has_tbn_;
    // Two-level acceleration structure
    int accel_mode_ = REINA_ACCEL_AUTO;
    bool emissive_device_ = false;
    bool bvh_device_ = false;
    BvhBuildOptions bvh_opt_;
    double bvh_kernel_seconds_ = 0.0;
    Bvh8 build_triangles(const float* verts, uint64_t tri_count);
    double emissive_seconds_ = 0.0;
    std::vector<uint8_t> emissive_same_;   // device build: pairwise same-CDF table of the emissive instances
    bool two_level_ = false;
    uint32_t blas_count_ = 0;
    std::vector<InstanceTrav> inst_trav_;
    std::vector<uint32_t> tlas_refs_;   // top-level leaf entries: instance indices
    std::vector<uint32_t> face_props_;  // two-level: per-face instances' material ids, concatenated
    // Textures: all texels in one array (one RGBA8 word each) and per texture its first texel and size
    std::vector<Image> textures_;
    std::vector<uint32_t> tex_texels_;
    std::vector<uint32_t> tex_info_;   // 4 per texture: first texel, width, height, 0
    // Device buffers
    DeviceBuffer d_nodes_, d_tris_, d_vertices_, d_indices_, d_tbns_, d_tbn_indices_, d_tex_coords_,
        d_tex_indices_, d_props_, d_instances_, d_prim_instance_, d_prim_props_, d_emissive_, d_cdf_tris_,
        d_cdf_inst_, d_props_material_, d_has_tbn_, d_tex_texels_, d_tex_info_, d_inst_trav_, d_tlas_refs_,
        d_face_props_;
    DeviceScene dev_;
};

// glm-style column-major helpers shared by the scene code and the C ABI.
void mat4_identity(float m[16]);
bool affine_inverse(const float T[16], float inv[12]);

}  // namespace rt
