// Host scene assembly, following src/scene/{Models,Scene,Instance,Instances}.cpp of the reference, and
// the upload of the assembled buffers and the BVH8 to the device.
#include "scene.h"

#include "emissive.h"

#include <array>
#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>
#include <unordered_map>

namespace rt {

void mat4_identity(float m[16]) {
    for (int i = 0; i < 16; ++i) m[i] = (i % 5 == 0) ? 1.0f : 0.0f;
}

// Models::addModel (src/scene/Models.cpp:24-92): append to the global buffers with offsets.
uint32_t Scene::define_object(ModelData&& model) {
    if (built_) fail(REINA_ERR_STATE, "Could not add model; buffers are already built");
    if (model.vertices.size() % 4 != 0) fail(REINA_ERR_INVALID, "vertices must hold 4 floats per vertex");
    if (model.indices.size() % 3 != 0) fail(REINA_ERR_INVALID, "indices must hold 3 entries per triangle");
    if (model.tbns.size() % 9 != 0) fail(REINA_ERR_INVALID, "tbns must hold 9 floats per entry");
    if (model.tex_coords.size() % 2 != 0) fail(REINA_ERR_INVALID, "tex_coords must hold 2 floats per entry");
    const uint64_t nv = model.vertices.size() / 4;
    for (uint32_t i : model.indices)
        if (i >= nv) fail(REINA_ERR_INVALID, "vertex index out of range");
    const uint64_t ntri = model.indices.size() / 3;
    if (!model.tbn_indices.empty()) {
        if (model.tbn_indices.size() != model.indices.size()) fail(REINA_ERR_INVALID, "tbn_indices must have one entry per index");
        for (uint32_t i : model.tbn_indices)
            if (i >= model.tbns.size() / 9) fail(REINA_ERR_INVALID, "tbn index out of range");
    }
    if (!model.tex_indices.empty()) {
        if (model.tex_indices.size() != model.indices.size()) fail(REINA_ERR_INVALID, "tex_indices must have one entry per index");
        for (uint32_t i : model.tex_indices)
            if (i != 0xFFFFFFFFu && i >= model.tex_coords.size() / 2) fail(REINA_ERR_INVALID, "tex index out of range");
    }
    (void)ntri;

    const size_t vertex_offset = all_vertices_.size();
    const size_t tbns_offset = all_tbns_.size() / 9;
    const size_t tex_offset = all_tex_coords_.size();
    const size_t index_offset = all_indices_offset_.size();
    const size_t tbns_indices_offset = all_tbns_indices_offset_.size();
    const size_t tex_index_offset = all_tex_indices_offset_.size();

    ModelRange r;
    r.first_vertex = (uint32_t)(vertex_offset / 4);
    r.first_normal = (uint32_t)tbns_offset;
    r.index_offset = (uint32_t)index_offset;
    r.tbns_index_offset = (uint32_t)tbns_indices_offset;
    // A model without texture coordinates (or without the per-corner indices into them) reconstructs UV
    // (0, 0) at every hit (closestHitCommon.h.glsl:96-98).
    r.tex_index_offset = (model.tex_coords.empty() || model.tex_indices.empty()) ? 0xFFFFFFFFu : (uint32_t)tex_index_offset;
    r.index_count = (uint32_t)(model.indices.size() / 3);
    r.tbns_index_count = (uint32_t)(model.indices.size() / 3);
    r.tex_index_count = (uint32_t)(model.tex_indices.size() / 3);
    ranges_.push_back(r);

    all_vertices_.insert(all_vertices_.end(), model.vertices.begin(), model.vertices.end());
    all_tex_coords_.insert(all_tex_coords_.end(), model.tex_coords.begin(), model.tex_coords.end());
    all_tbns_.insert(all_tbns_.end(), model.tbns.begin(), model.tbns.end());
    for (uint32_t idx : model.indices) {
        all_indices_offset_.push_back(idx + (uint32_t)(vertex_offset / 4));
        all_indices_non_offset_.push_back(idx);
    }
    for (uint32_t idx : model.tbn_indices) all_tbns_indices_offset_.push_back(idx + (uint32_t)tbns_offset);
    for (uint32_t idx : model.tex_indices)
        all_tex_indices_offset_.push_back(idx == 0xFFFFFFFFu ? idx : idx + (uint32_t)(tex_offset / 2));

    models_.push_back(std::move(model));
    return (uint32_t)(ranges_.size() - 1);
}

// Scene::addInstance (src/scene/Scene.cpp:27-54): Material -> InstanceProperties.
InstanceProperties Scene::make_props(uint32_t object, const reina_material& m) const {
    const ModelRange& r = ranges_[object];
    InstanceProperties p;
    std::memset(&p, 0, sizeof(p));
    p.indicesOffset = r.index_offset;
    for (int k = 0; k < 3; ++k) {
        p.albedo[k] = m.albedo[k];
        p.emission[k] = m.emission[k];
        p.sheenTint[k] = m.sheen_tint[k];
        p.specularTint[k] = m.specular_tint[k];
    }
    p.tbnsIndicesOffset = r.tbns_index_offset;
    p.texIndicesOffset = r.tex_index_offset;
    p.roughness = m.roughness;
    p.ior = m.ior;
    p.interpNormals = m.interp_normals ? 1u : 0u;
    p.absorption = m.absorption;
    p.textureID = m.texture_id;
    p.normalMapTexID = m.normal_map_id;
    p.bumpMapTexID = m.bump_map_id;
    p.cullBackface = m.cull_backface ? 1u : 0u;
    p.anisotropic = m.anisotropic;
    p.subsurface = m.subsurface;
    p.clearcoatGloss = m.clearcoat_gloss;
    p.metallic = m.metallic;
    p.clearcoat = m.clearcoat;
    p.specularTransmission = m.specular_transmission;
    p.sheen = m.sheen;
    return p;
}

// Texture ids are checked against the scene's textures at build(), since textures may be defined after
// the instances that use them (as with Scene::defineTexture).
static void check_material(const reina_material& m) {
    if (m.material_idx > 3) fail(REINA_ERR_INVALID, "material_idx must be 0 (Lambertian), 1 (metal), 2 (dielectric) or 3 (Disney)");
}

uint32_t Scene::define_texture(Image&& image) {
    if (built_) fail(REINA_ERR_STATE, "cannot define a texture in a built scene");
    if (image.width == 0 || image.height == 0) fail(REINA_ERR_INVALID, "texture has zero size");
    if (image.rgba.size() != (size_t)image.width * image.height * 4) fail(REINA_ERR_INVALID, "texture data size mismatch");
    size_t total = 0;
    for (const Image& t : textures_) total += (size_t)t.width * t.height;
    if (total + (size_t)image.width * image.height > 0xFFFFFFFFull) fail(REINA_ERR_INVALID, "textures exceed 2^32 texels in total");
    textures_.push_back(std::move(image));
    return (uint32_t)(textures_.size() - 1);
}

const Image& Scene::texture(uint32_t id) const {
    if (id >= textures_.size()) fail(REINA_ERR_INVALID, "texture id out of range");
    return textures_[id];
}

void Scene::add_instance(uint32_t object, const float transform[16], const reina_material& mat) {
    if (built_) fail(REINA_ERR_STATE, "cannot add an instance to a built scene");
    if (object >= ranges_.size()) fail(REINA_ERR_INVALID, "Index " + std::to_string(object) + " out of range for models");
    check_material(mat);
    props_.push_back(make_props(object, mat));
    props_material_.push_back(mat.material_idx);
    InstanceRecord inst;
    inst.object = object;
    inst.props_id = (uint32_t)(props_.size() - 1);
    inst.material_idx = mat.material_idx;
    std::memcpy(inst.transform, transform, sizeof(inst.transform));
    instances_.push_back(std::move(inst));
}

void Scene::add_instance_per_face(uint32_t object, const float transform[16], const reina_material* mats,
                                  uint32_t mat_count, const uint32_t* face_material) {
    if (built_) fail(REINA_ERR_STATE, "cannot add an instance to a built scene");
    if (object >= ranges_.size()) fail(REINA_ERR_INVALID, "Index " + std::to_string(object) + " out of range for models");
    if (mat_count == 0 || !mats || !face_material) fail(REINA_ERR_INVALID, "per-face instance needs materials and a face table");
    const uint32_t nfaces = ranges_[object].index_count;
    for (uint32_t f = 0; f < nfaces; ++f)
        if (face_material[f] >= mat_count) fail(REINA_ERR_INVALID, "face material index out of range");
    const uint32_t base = (uint32_t)props_.size();
    for (uint32_t i = 0; i < mat_count; ++i) {
        check_material(mats[i]);
        const float* e = mats[i].emission;
        if (e[0] != 0.0f || e[1] != 0.0f || e[2] != 0.0f)
            fail(REINA_ERR_INVALID, "per-face materials must not be emissive");
        props_.push_back(make_props(object, mats[i]));
        props_material_.push_back(mats[i].material_idx);
    }
    InstanceRecord inst;
    inst.object = object;
    inst.props_id = base;
    inst.material_idx = mats[0].material_idx;
    std::memcpy(inst.transform, transform, sizeof(inst.transform));
    inst.per_face = true;
    inst.face_props.resize(nfaces);
    for (uint32_t f = 0; f < nfaces; ++f) inst.face_props[f] = base + face_material[f];
    instances_.push_back(std::move(inst));
}

// Instance::Instance + Instance::computeCDF (src/scene/Instance.cpp:5-53).  The area uses the row-vector
// product vec4(v, 1) * transform, i.e. the transpose of the transform applied by NEE (nee.h.glsl:113-115).
static bool is_emissive(const float emission[3]) {
    const float dot = emission[0] * emission[0] + emission[1] * emission[1] + emission[2] * emission[2];
    return dot > 0.00001f * 0.00001f;
}

static float luminance(const float emission[3]) {
    return (float)(0.2126 * emission[0] + 0.7152 * emission[1] + 0.0722 * emission[2]);
}

void Scene::compute_emissive(InstanceRecord& inst, const float emission[3]) {
    inst.light = EmissiveInfo{};
    if (!is_emissive(emission)) return;
    inst.light.emissive = true;
    const float brightness = luminance(emission);
    const ModelData& md = models_[inst.object];
    const float* T = inst.transform;
    const size_t nv = md.vertices.size() / 4;
    std::vector<float> tv(3 * nv);
    for (size_t i = 0; i < nv; ++i) {
        const float v[4] = {md.vertices[4 * i + 0], md.vertices[4 * i + 1], md.vertices[4 * i + 2], 1.0f};
        for (int c = 0; c < 3; ++c) {
            const float* col = T + 4 * c;
            float s = col[0] * v[0];
            s = s + col[1] * v[1];
            s = s + col[2] * v[2];
            s = s + col[3] * v[3];
            tv[3 * i + c] = s;
        }
    }
    const size_t ntri = md.indices.size() / 3;
    inst.light.cdf.resize(ntri);
    float cumulative = 0.0f;
    float area = 0.0f;
    for (size_t t = 0; t < ntri; ++t) {
        const float* a = &tv[3 * md.indices[3 * t + 0]];
        const float* b = &tv[3 * md.indices[3 * t + 1]];
        const float* c = &tv[3 * md.indices[3 * t + 2]];
        const float ab[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
        const float ac[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
        const float cr[3] = {ab[1] * ac[2] - ac[1] * ab[2], ab[2] * ac[0] - ac[2] * ab[0], ab[0] * ac[1] - ac[0] * ab[1]};
        const float tri_area = std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]) / 2.0f;
        area += tri_area;
        cumulative += tri_area * brightness;
        inst.light.cdf[t] = cumulative;
    }
    if (cumulative == 0.0f) fail(REINA_ERR_INVALID, "Cannot calculate CDF for a mesh because the cumulative area is 0");
    for (float& v : inst.light.cdf) v /= cumulative;
    inst.light.area = area;
    inst.light.weight = cumulative;
}

// The same CDFs, areas and weights for every emissive instance on the scene's GPU (emissive.cu), and the
// duplicate search there; returns the pairwise "same CDF" table for pack_emissives.
void Scene::compute_emissives_device() {
    if (device_ < 0) fail(REINA_ERR_STATE, "the emissive CDF build on the device needs a GPU context");
    std::vector<EmissiveInput> in;
    std::vector<InstanceRecord*> targets;
    for (InstanceRecord& inst : instances_) {
        inst.light = EmissiveInfo{};
        if (inst.per_face) continue;
        const float* emission = props_[inst.props_id].emission;
        if (!is_emissive(emission)) continue;
        const ModelData& md = models_[inst.object];
        EmissiveInput e;
        e.vertices = md.vertices.data();
        e.nv = md.vertices.size() / 4;
        e.indices = md.indices.data();
        e.ntri = md.indices.size() / 3;
        e.model = inst.object;
        std::memcpy(e.transform, inst.transform, sizeof(e.transform));
        e.brightness = luminance(emission);
        in.push_back(e);
        targets.push_back(&inst);
    }
    std::vector<EmissiveOutput> out;
    emissive_cdfs_device(device_, in, std::numeric_limits<float>::epsilon(), out, emissive_same_);
    for (size_t k = 0; k < in.size(); ++k) {
        EmissiveInfo& l = targets[k]->light;
        l.emissive = true;
        if (out[k].weight == 0.0f)
            fail(REINA_ERR_INVALID, "Cannot calculate CDF for a mesh because the cumulative area is 0");
        l.cdf = std::move(out[k].cdf);
        l.area = out[k].area;
        l.weight = out[k].weight;
    }
}

// Instances::computeSamplingDataEmissives (src/scene/Instances.cpp:52-114), including its lookup of
// duplicates by position in the emissive list (`duplicates.contains(instanceIdxIdx)`) and by instance
// index (`duplicates.at(instanceIdx)`), which agree whenever every instance is emissive.
void Scene::pack_emissives(const std::vector<uint8_t>* same) {
    std::vector<int> emissive_idx;
    for (size_t i = 0; i < instances_.size(); ++i)
        if (instances_[i].light.emissive) emissive_idx.push_back((int)i);

    auto same_cdf = [](const std::vector<float>& a, const std::vector<float>& b) {
        if (a.size() != b.size()) return false;
        const float tol = std::numeric_limits<float>::epsilon();
        for (size_t i = 0; i < a.size(); ++i)
            if (std::fabs(a[i] - b[i]) > tol) return false;
        return true;
    };
    std::unordered_map<size_t, size_t> dup;
    const size_t ne = emissive_idx.size();
    if (same && same->size() != ne * ne) fail(REINA_ERR_INVALID, "emissive CDF deduplication: table size mismatch");
    for (size_t ii = 0; ii < ne; ++ii) {
        const int i = emissive_idx[ii];
        for (size_t jj = ii + 1; jj < ne; ++jj) {
            const int j = emissive_idx[jj];
            if (same ? !(*same)[ii * ne + jj] : !same_cdf(instances_[i].light.cdf, instances_[j].light.cdf)) continue;
            if (dup.find(j) == dup.end()) dup[j] = i;
        }
    }

    cdf_triangles_.clear();
    emissive_data_.assign(emissive_idx.size(), EmissiveInstanceData{});
    for (size_t pos = 0; pos < emissive_idx.size(); ++pos) {
        const int ii = emissive_idx[pos];
        const InstanceRecord& inst = instances_[ii];
        EmissiveInstanceData& d = emissive_data_[pos];
        std::memset(&d, 0, sizeof(d));
        std::memcpy(d.transform, inst.transform, sizeof(d.transform));
        d.materialOffset = inst.material_idx;
        d.indexOffset = ranges_[inst.object].index_offset;
        for (int k = 0; k < 3; ++k) d.emission[k] = props_[inst.props_id].emission[k];
        d.weight = inst.light.weight;
        d.area = inst.light.area;
        d.cullBackface = props_[inst.props_id].cullBackface ? 1u : 0u;
        if (dup.count(pos)) {
            auto it = dup.find((size_t)ii);
            if (it == dup.end())
                fail(REINA_ERR_INVALID, "emissive CDF deduplication: no canonical entry for a duplicate instance");
            if (it->second >= emissive_data_.size())
                fail(REINA_ERR_INVALID, "emissive CDF deduplication: canonical index out of range");
            const EmissiveInstanceData& of = emissive_data_[it->second];
            d.cdfRangeStart = of.cdfRangeStart;
            d.cdfRangeEnd = of.cdfRangeEnd;
            continue;
        }
        const std::vector<float>& cdf = inst.light.cdf;
        d.cdfRangeStart = (uint32_t)cdf_triangles_.size();
        d.cdfRangeEnd = d.cdfRangeStart + (uint32_t)cdf.size() - 1;
        cdf_triangles_.insert(cdf_triangles_.end(), cdf.begin(), cdf.end());
    }
    cdf_instances_.assign(emissive_idx.size(), 0.0f);
    float cumulative = 0.0f;
    for (size_t i = 0; i < cdf_instances_.size(); ++i) {
        cumulative += instances_[emissive_idx[i]].light.weight;
        cdf_instances_[i] = cumulative;
    }
    for (float& v : cdf_instances_) v /= cumulative;
    emissive_total_ = cumulative;
}

// Normal matrix transpose(inverse(mat3(M))) in float, via cofactors / determinant.
static void normal_matrix(const float T[16], float out[9]) {
    auto M = [&](int r, int c) { return T[c * 4 + r]; };
    float cof[3][3];
    for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 3; ++c) {
            const int r1 = (r + 1) % 3, r2 = (r + 2) % 3, c1 = (c + 1) % 3, c2 = (c + 2) % 3;
            cof[r][c] = M(r1, c1) * M(r2, c2) - M(r1, c2) * M(r2, c1);
        }
    }
    const float det = M(0, 0) * cof[0][0] + M(0, 1) * cof[0][1] + M(0, 2) * cof[0][2];
    // inverse = adj / det with adj = cof^T, so transpose(inverse) = cof / det.
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) out[r * 3 + c] = det != 0.0f ? cof[r][c] / det : 0.0f;
}

void Scene::set_accel(int mode) {
    if (built_) fail(REINA_ERR_STATE, "the acceleration structure is chosen before the build");
    if (mode < REINA_ACCEL_AUTO || mode > REINA_ACCEL_TWO_LEVEL) fail(REINA_ERR_INVALID, "unknown acceleration structure mode");
    accel_mode_ = mode;
}

// Inverse of an affine transform (column-major 4x4) as a row-major 3x4 world-to-object matrix: the
// 3x3 inverse by cofactors over the determinant and the translation -inverse * t, in double, each entry
// rounded to float.  Returns false for a singular (or non-finite) transform.
bool affine_inverse(const float T[16], float inv[12]) {
    auto M = [&](int r, int c) { return (double)T[c * 4 + r]; };
    double cof[3][3];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            const int r1 = (r + 1) % 3, r2 = (r + 2) % 3, c1 = (c + 1) % 3, c2 = (c + 2) % 3;
            cof[r][c] = M(r1, c1) * M(r2, c2) - M(r1, c2) * M(r2, c1);
        }
    const double det = M(0, 0) * cof[0][0] + M(0, 1) * cof[0][1] + M(0, 2) * cof[0][2];
    if (!(std::fabs(det) > 0.0) || !std::isfinite(det)) return false;
    double m[3][3];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) m[r][c] = cof[c][r] / det;   // inverse = adjugate / det
    for (int r = 0; r < 3; ++r) {
        const double t = -(m[r][0] * M(0, 3) + m[r][1] * M(1, 3) + m[r][2] * M(2, 3));
        for (int c = 0; c < 3; ++c) inv[r * 4 + c] = (float)m[r][c];
        inv[r * 4 + 3] = (float)t;
        for (int c = 0; c < 4; ++c)
            if (!std::isfinite(inv[r * 4 + c])) return false;
    }
    return true;
}

// Two levels when asked for, or (automatic) when instancing repeats models enough that the flattened
// triangle records would take at least twice the memory of one copy per model, and every instance
// transform is invertible.
bool Scene::use_two_level() const {
    if (accel_mode_ == REINA_ACCEL_FLAT || instances_.empty()) return false;
    uint64_t unique = 0;
    std::vector<uint8_t> used(models_.size(), 0);
    for (const InstanceRecord& inst : instances_)
        if (!used[inst.object]) {
            used[inst.object] = 1;
            unique += ranges_[inst.object].index_count;
        }
    bool invertible = true;
    float inv[12];
    for (const InstanceRecord& inst : instances_) invertible = invertible && affine_inverse(inst.transform, inv);
    if (accel_mode_ == REINA_ACCEL_TWO_LEVEL) {
        if (!invertible) fail(REINA_ERR_INVALID, "a two-level scene needs invertible instance transforms");
        return true;
    }
    return invertible && tri_total_ >= 2 * unique;
}

// A triangle BVH on the host or on the scene's GPU (same bytes either way).
Bvh8 Scene::build_triangles(const float* verts, uint64_t tri_count) {
    if (!bvh_device_) return build_bvh8(verts, tri_count, bvh_opt_);
    double k = 0.0;
    Bvh8 b = build_bvh8_device(device_, verts, tri_count, bvh_opt_, &k);
    bvh_kernel_seconds_ += k;
    return b;
}

// One BVH over all instances' world-space triangles.
void Scene::build_flat() {
    std::vector<float> world(9 * tri_total_);
    for (int k = 0; k < 3; ++k) { bounds_lo_[k] = INFINITY; bounds_hi_[k] = -INFINITY; }
    for (size_t ii = 0; ii < instances_.size(); ++ii) {
        const InstanceRecord& inst = instances_[ii];
        const ModelData& md = models_[inst.object];
        const float* T = inst.transform;
        const uint32_t ntri = ranges_[inst.object].index_count;
        for (uint32_t t = 0; t < ntri; ++t) {
            const uint64_t g = inst.first_prim + t;
            for (int j = 0; j < 3; ++j) {
                const uint32_t vi = md.indices[3 * t + j];
                const float x = md.vertices[4 * vi + 0], y = md.vertices[4 * vi + 1], z = md.vertices[4 * vi + 2];
                for (int r = 0; r < 3; ++r) {
                    float s = T[0 * 4 + r] * x;
                    s = s + T[1 * 4 + r] * y;
                    s = s + T[2 * 4 + r] * z;
                    s = s + T[3 * 4 + r];
                    world[9 * g + 3 * j + r] = s;
                    bounds_lo_[r] = std::min(bounds_lo_[r], s);
                    bounds_hi_[r] = std::max(bounds_hi_[r], s);
                }
            }
        }
    }
    bvh_ = build_triangles(world.data(), tri_total_);
    inst_trav_.clear();
    tlas_refs_.clear();
    blas_count_ = 0;
}

// The reference's structure (src/scene/Scene.cpp:93-116; BLAS per model, src/graphics/Blas.cpp; TLAS
// over instances, src/tools/vktools.cpp:460-596): one bottom-level BVH8 per instanced model over its
// object-space triangles (record ids = triangle index within the model), one top-level BVH8 over the
// instances' world-space boxes, all nodes in one array (top-level root = node 0, each model's nodes
// after it with their child and triangle bases offset) and all triangle records in one array.
void Scene::build_two_level() {
    const size_t ninst = instances_.size();
    std::vector<int64_t> blas_of(models_.size(), -1);
    std::vector<std::array<float, 6>> model_box(models_.size());
    // object-space boxes of the used models
    for (const InstanceRecord& inst : instances_) {
        if (blas_of[inst.object] == -2) continue;
        blas_of[inst.object] = -2;
        const ModelData& md = models_[inst.object];
        std::array<float, 6> b = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
        for (uint32_t vi : md.indices)
            for (int k = 0; k < 3; ++k) {
                b[k] = std::min(b[k], md.vertices[4 * vi + k]);
                b[3 + k] = std::max(b[3 + k], md.vertices[4 * vi + k]);
            }
        model_box[inst.object] = b;
    }
    // world boxes of the instances, in double and rounded outward: the box of the model's transformed
    // vertices when that is affordable (at most 2^26 vertex transforms in all), else of the 8 transformed
    // corners of the model box (looser for rotated instances)
    uint64_t transforms = 0;
    for (const InstanceRecord& inst : instances_) transforms += models_[inst.object].vertices.size() / 4;
    const bool exact = transforms <= (1ull << 26);
    std::vector<float> boxes(6 * ninst);
    for (int k = 0; k < 3; ++k) { bounds_lo_[k] = INFINITY; bounds_hi_[k] = -INFINITY; }
    for (size_t ii = 0; ii < ninst; ++ii) {
        const InstanceRecord& inst = instances_[ii];
        const std::array<float, 6>& mb = model_box[inst.object];
        const float* T = inst.transform;
        double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        const bool empty = ranges_[inst.object].index_count == 0;
        auto add = [&](const double p[3]) {
            for (int r = 0; r < 3; ++r) {
                const double w = T[0 * 4 + r] * p[0] + T[1 * 4 + r] * p[1] + T[2 * 4 + r] * p[2] + T[3 * 4 + r];
                lo[r] = std::min(lo[r], w);
                hi[r] = std::max(hi[r], w);
            }
        };
        if (!empty && exact) {
            const ModelData& md = models_[inst.object];   // every vertex (unreferenced ones only loosen the box)
            for (size_t vi = 0; vi < md.vertices.size() / 4; ++vi) {
                const double p[3] = {md.vertices[4 * vi], md.vertices[4 * vi + 1], md.vertices[4 * vi + 2]};
                add(p);
            }
        }
        for (int c = 0; c < 8 && !empty && !exact; ++c) {
            const double p[3] = {mb[(c & 1) ? 3 : 0], mb[(c & 2) ? 4 : 1], mb[(c & 4) ? 5 : 2]};
            add(p);
        }
        for (int r = 0; r < 3; ++r) {
            if (empty) { lo[r] = hi[r] = T[3 * 4 + r]; }
            float fl = (float)lo[r], fh = (float)hi[r];
            if ((double)fl > lo[r]) fl = std::nextafter(fl, -INFINITY);
            if ((double)fh < hi[r]) fh = std::nextafter(fh, INFINITY);
            boxes[6 * ii + r] = fl;
            boxes[6 * ii + 3 + r] = fh;
            bounds_lo_[r] = std::min(bounds_lo_[r], fl);
            bounds_hi_[r] = std::max(bounds_hi_[r], fh);
        }
    }
    Bvh8 tlas = build_bvh8_boxes(boxes.data(), ninst, tlas_refs_);
    Bvh8 out;
    out.nodes = std::move(tlas.nodes);
    out.binary_nodes = tlas.binary_nodes;
    double seconds = tlas.seconds;
    uint32_t blas_depth = 0;
    blas_count_ = 0;
    for (size_t o = 0; o < models_.size(); ++o) {
        if (blas_of[o] != -2) continue;
        const ModelData& md = models_[o];
        const size_t ntri = md.indices.size() / 3;
        std::vector<float> tris(9 * ntri);
        for (size_t t = 0; t < ntri; ++t)
            for (int j = 0; j < 3; ++j)
                for (int k = 0; k < 3; ++k) tris[9 * t + 3 * j + k] = md.vertices[4 * md.indices[3 * t + j] + k];
        Bvh8 b = build_triangles(tris.data(), ntri);
        const uint32_t node_base = (uint32_t)out.nodes.size(), tri_base = (uint32_t)out.tris.size();
        if (b.nodes.empty()) {   // a model without triangles: no bottom level (its instances have empty boxes)
            blas_of[o] = -1;
            continue;
        }
        for (Bvh8Node& n : b.nodes) {
            n.child_base += node_base;
            n.tri_base += tri_base;
        }
        out.nodes.insert(out.nodes.end(), b.nodes.begin(), b.nodes.end());
        out.tris.insert(out.tris.end(), b.tris.begin(), b.tris.end());
        blas_of[o] = node_base;
        blas_depth = std::max(blas_depth, b.depth);
        out.binary_nodes += b.binary_nodes;
        seconds += b.seconds;
        ++blas_count_;
    }
    out.depth = tlas.depth + blas_depth;
    // the traversal stack holds both levels plus one marker between them
    if (out.depth + 1 > kMaxBvhDepth) fail(REINA_ERR_INVALID, "two-level BVH deeper than the traversal stack");
    out.seconds = seconds;
    bvh_ = std::move(out);
    inst_trav_.assign(ninst, InstanceTrav{});
    for (size_t ii = 0; ii < ninst; ++ii) {
        const InstanceRecord& inst = instances_[ii];
        InstanceTrav& it = inst_trav_[ii];
        affine_inverse(inst.transform, it.inv);
        it.blas_root = blas_of[inst.object] >= 0 ? (uint32_t)blas_of[inst.object] : 0xFFFFFFFFu;
        it.first_prim = inst.first_prim;
    }
}

void Scene::build(bool require_emissive) {
    if (built_) fail(REINA_ERR_STATE, "Cannot call build more than once");
    const bool host_only = device_ < 0;
    if (!host_only) check_cuda(cudaSetDevice(device_), "cudaSetDevice");
    if (host_only && bvh_device_) fail(REINA_ERR_STATE, "device BVH build requested on a host-only context");
    bvh_kernel_seconds_ = 0.0;

    const int64_t ntex = (int64_t)textures_.size();
    for (const InstanceProperties& p : props_)
        for (int32_t id : {p.textureID, p.normalMapTexID, p.bumpMapTexID})
            if (id >= ntex) fail(REINA_ERR_INVALID, "material texture id " + std::to_string(id) + " out of range (" +
                                                        std::to_string(ntex) + " textures defined)");
    // All textures in one texel array (first texel, width, height per texture).
    tex_texels_.clear();
    tex_info_.clear();
    for (const Image& t : textures_) {
        tex_info_.insert(tex_info_.end(), {(uint32_t)tex_texels_.size(), t.width, t.height, 0u});
        const size_t n = (size_t)t.width * t.height;
        const size_t base = tex_texels_.size();
        tex_texels_.resize(base + n);
        for (size_t i = 0; i < n; ++i) {
            const uint8_t* c = &t.rgba[4 * i];
            tex_texels_[base + i] = (uint32_t)c[0] | ((uint32_t)c[1] << 8) | ((uint32_t)c[2] << 16) | ((uint32_t)c[3] << 24);
        }
    }

    // Emissive CDFs and packing (src/scene/Scene.cpp:102-114 -> Instances).
    const auto t_em = std::chrono::steady_clock::now();
    if (emissive_device_) {
        compute_emissives_device();
        pack_emissives(&emissive_same_);
    } else {
        for (InstanceRecord& inst : instances_) {
            if (inst.per_face) inst.light = EmissiveInfo{};
            else compute_emissive(inst, props_[inst.props_id].emission);
        }
        pack_emissives();
    }
    emissive_seconds_ = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_em).count();
    if (cdf_triangles_.empty() && require_emissive) fail(REINA_ERR_NO_EMISSIVE, "Scene must have at least one emissive object");

    tri_total_ = 0;
    for (InstanceRecord& inst : instances_) {
        inst.first_prim = (uint32_t)tri_total_;
        tri_total_ += ranges_[inst.object].index_count;
    }
    if (tri_total_ >= 0x7FFFFFFFull) fail(REINA_ERR_INVALID, "scene has too many triangles");
    two_level_ = use_two_level();
    // Per-triangle instance and material tables for flat scenes; two-level scenes (whose point is not
    // to hold per-triangle data for every instance) look both up from the instance records and keep only
    // the per-face tables of per-face instances.
    prim_instance_.clear();
    prim_props_.clear();
    face_props_.clear();
    if (!two_level_) {
        prim_instance_.resize(tri_total_);
        prim_props_.resize(tri_total_);
    }
    for (size_t ii = 0; ii < instances_.size(); ++ii) {
        const InstanceRecord& inst = instances_[ii];
        const uint32_t ntri = ranges_[inst.object].index_count;
        if (two_level_) {
            if (inst.per_face) face_props_.insert(face_props_.end(), inst.face_props.begin(), inst.face_props.end());
            continue;
        }
        for (uint32_t t = 0; t < ntri; ++t) {
            prim_instance_[inst.first_prim + t] = (uint32_t)ii;
            prim_props_[inst.first_prim + t] = inst.per_face ? inst.face_props[t] : inst.props_id;
        }
    }
    try {
        if (two_level_) build_two_level();
        else build_flat();
    } catch (const Error&) {
        throw;
    } catch (const std::exception& e) {
        fail(REINA_ERR_INVALID, e.what());
    }

    inst_gpu_.assign(instances_.size(), InstanceGpu{});
    uint32_t face_base = 0;
    for (size_t ii = 0; ii < instances_.size(); ++ii) {
        const InstanceRecord& inst = instances_[ii];
        InstanceGpu& g = inst_gpu_[ii];
        std::memset(&g, 0, sizeof(g));
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 4; ++c) g.m[r * 4 + c] = inst.transform[c * 4 + r];
        normal_matrix(inst.transform, g.nrm);
        g.props = inst.props_id;
        g.first_prim = inst.first_prim;
        g.object = inst.object;
        g.light_weight = inst.light.emissive ? inst.light.weight : 0.0f;
        g.light_area = inst.light.emissive ? inst.light.area : 0.0f;
        g.face_base = 0xFFFFFFFFu;
        if (two_level_ && inst.per_face) {
            g.face_base = face_base;
            face_base += (uint32_t)inst.face_props.size();
        }
    }

    has_tbn_.resize(models_.size());
    for (size_t o = 0; o < models_.size(); ++o) has_tbn_[o] = models_[o].tbn_indices.empty() ? 0 : 1;
    built_ = true;
    if (host_only) {   // host-only scenes keep the assembled buffers and the BVH, nothing is uploaded
        dev_ = DeviceScene{};
        dev_.node_count = (uint32_t)bvh_.nodes.size();
        dev_.tri_count = (uint32_t)bvh_.tris.size();
        return;
    }
    upload();
}

size_t Scene::upload_bytes() const {
    return bvh_.nodes.size() * sizeof(Bvh8Node) + bvh_.tris.size() * sizeof(TriRecord) +
           (all_vertices_.size() + all_tbns_.size() + std::max<size_t>(1, all_tex_coords_.size()) +
            cdf_triangles_.size() + cdf_instances_.size()) * sizeof(float) +
           (all_indices_offset_.size() + all_tbns_indices_offset_.size() + all_tex_indices_offset_.size() +
            prim_instance_.size() + prim_props_.size() + props_material_.size()) * sizeof(uint32_t) +
           props_.size() * sizeof(InstanceProperties) + inst_gpu_.size() * sizeof(InstanceGpu) +
           emissive_data_.size() * sizeof(EmissiveInstanceData) + has_tbn_.size() +
           (tex_texels_.size() + tex_info_.size() + tlas_refs_.size() + face_props_.size()) * sizeof(uint32_t) +
           inst_trav_.size() * sizeof(InstanceTrav);
}

void Scene::release_device() {
    for (DeviceBuffer* b : {&d_nodes_, &d_tris_, &d_vertices_, &d_indices_, &d_tbns_, &d_tbn_indices_, &d_tex_coords_,
                            &d_tex_indices_, &d_props_, &d_instances_, &d_prim_instance_, &d_prim_props_, &d_emissive_,
                            &d_cdf_tris_, &d_cdf_inst_, &d_props_material_, &d_has_tbn_, &d_tex_texels_, &d_tex_info_,
                            &d_inst_trav_, &d_tlas_refs_, &d_face_props_})
        b->release();
    const uint32_t nodes = dev_.node_count, tris = dev_.tri_count;
    dev_ = DeviceScene{};
    dev_.node_count = nodes;
    dev_.tri_count = tris;
    resident_ = false;
}

void Scene::upload() {
    if (!built_) fail(REINA_ERR_STATE, "scene is not built");
    if (device_ < 0) fail(REINA_ERR_STATE, "host-only scene cannot be uploaded");
    if (resident_) return;
    check_cuda(cudaSetDevice(device_), "cudaSetDevice");
    // Upload (src/scene/Models.cpp:94-115 uploads the same arrays; an empty texcoord buffer gets one
    // float there and here so that the pointer stays valid).
    auto up = [](DeviceBuffer& b, const void* p, size_t bytes) { b.upload(p, bytes); };
    up(d_nodes_, bvh_.nodes.data(), bvh_.nodes.size() * sizeof(Bvh8Node));
    up(d_tris_, bvh_.tris.data(), bvh_.tris.size() * sizeof(TriRecord));
    up(d_vertices_, all_vertices_.data(), all_vertices_.size() * sizeof(float));
    up(d_indices_, all_indices_offset_.data(), all_indices_offset_.size() * sizeof(uint32_t));
    up(d_tbns_, all_tbns_.data(), all_tbns_.size() * sizeof(float));
    up(d_tbn_indices_, all_tbns_indices_offset_.data(), all_tbns_indices_offset_.size() * sizeof(uint32_t));
    const float zero = 0.0f;
    if (all_tex_coords_.empty()) up(d_tex_coords_, &zero, sizeof(float));
    else up(d_tex_coords_, all_tex_coords_.data(), all_tex_coords_.size() * sizeof(float));
    up(d_tex_indices_, all_tex_indices_offset_.data(), all_tex_indices_offset_.size() * sizeof(uint32_t));
    up(d_props_, props_.data(), props_.size() * sizeof(InstanceProperties));
    up(d_instances_, inst_gpu_.data(), inst_gpu_.size() * sizeof(InstanceGpu));
    up(d_prim_instance_, prim_instance_.data(), prim_instance_.size() * sizeof(uint32_t));
    up(d_prim_props_, prim_props_.data(), prim_props_.size() * sizeof(uint32_t));
    up(d_emissive_, emissive_data_.data(), emissive_data_.size() * sizeof(EmissiveInstanceData));
    up(d_cdf_tris_, cdf_triangles_.data(), cdf_triangles_.size() * sizeof(float));
    up(d_cdf_inst_, cdf_instances_.data(), cdf_instances_.size() * sizeof(float));
    up(d_props_material_, props_material_.data(), props_material_.size() * sizeof(uint32_t));
    up(d_has_tbn_, has_tbn_.data(), has_tbn_.size());
    up(d_inst_trav_, inst_trav_.data(), inst_trav_.size() * sizeof(InstanceTrav));
    up(d_face_props_, face_props_.data(), face_props_.size() * sizeof(uint32_t));
    up(d_tlas_refs_, tlas_refs_.data(), tlas_refs_.size() * sizeof(uint32_t));
    up(d_tex_texels_, tex_texels_.data(), tex_texels_.size() * sizeof(uint32_t));
    up(d_tex_info_, tex_info_.data(), tex_info_.size() * sizeof(uint32_t));

    dev_ = DeviceScene{};
    dev_.nodes = d_nodes_.as<Bvh8Node>();
    dev_.tris = d_tris_.as<TriRecord>();
    dev_.node_count = (uint32_t)bvh_.nodes.size();
    dev_.tri_count = (uint32_t)bvh_.tris.size();
    dev_.vertices = d_vertices_.as<float>();
    dev_.indices = d_indices_.as<uint32_t>();
    dev_.tbns = d_tbns_.as<float>();
    dev_.tbn_indices = d_tbn_indices_.as<uint32_t>();
    dev_.tex_coords = d_tex_coords_.as<float>();
    dev_.tex_indices = d_tex_indices_.as<uint32_t>();
    dev_.props = d_props_.as<InstanceProperties>();
    dev_.instances = d_instances_.as<InstanceGpu>();
    dev_.prim_instance = two_level_ ? nullptr : d_prim_instance_.as<uint32_t>();
    dev_.prim_props = two_level_ ? nullptr : d_prim_props_.as<uint32_t>();
    dev_.face_props = d_face_props_.as<uint32_t>();
    dev_.props_material = d_props_material_.as<uint32_t>();
    dev_.has_tbn = d_has_tbn_.as<uint8_t>();
    dev_.instance_count = (uint32_t)instances_.size();
    dev_.props_count = (uint32_t)props_.size();
    dev_.emissive = d_emissive_.as<EmissiveInstanceData>();
    dev_.cdf_triangles = d_cdf_tris_.as<float>();
    dev_.cdf_instances = d_cdf_inst_.as<float>();
    dev_.emissive_count = (uint32_t)emissive_data_.size();
    dev_.emissive_weight = emissive_total_;
    dev_.inst_trav = two_level_ ? d_inst_trav_.as<InstanceTrav>() : nullptr;
    dev_.tlas_refs = two_level_ ? d_tlas_refs_.as<uint32_t>() : nullptr;
    dev_.tex_texels = d_tex_texels_.as<uint32_t>();
    dev_.tex_info = d_tex_info_.as<uint4>();
    dev_.tex_count = (uint32_t)textures_.size();
    for (int k = 0; k < 3; ++k) {
        dev_.bounds_lo[k] = bounds_lo_[k];
        dev_.bounds_hi[k] = bounds_hi_[k];
    }
    resident_ = true;
}

size_t Scene::device_bytes() const {
    return d_nodes_.bytes() + d_tris_.bytes() + d_vertices_.bytes() + d_indices_.bytes() + d_tbns_.bytes() +
           d_tbn_indices_.bytes() + d_tex_coords_.bytes() + d_tex_indices_.bytes() + d_props_.bytes() +
           d_instances_.bytes() + d_prim_instance_.bytes() + d_prim_props_.bytes() + d_emissive_.bytes() +
           d_cdf_tris_.bytes() + d_cdf_inst_.bytes() + d_props_material_.bytes() + d_has_tbn_.bytes() +
           d_tex_texels_.bytes() + d_tex_info_.bytes() + d_inst_trav_.bytes() + d_tlas_refs_.bytes() +
           d_face_props_.bytes();
}

const ModelData& Scene::model(uint32_t object) const {
    if (object >= models_.size()) fail(REINA_ERR_INVALID, "object id out of range");
    return models_[object];
}

void Scene::prim_info(uint32_t prim, uint32_t* inst, uint32_t* local) const {
    if (!built_) fail(REINA_ERR_STATE, "scene is not built");
    if (prim >= tri_total_) fail(REINA_ERR_INVALID, "triangle id out of range");
    uint32_t ii;
    if (!prim_instance_.empty()) {
        ii = prim_instance_[prim];
    } else {   // two-level: the last instance whose first triangle is at or before prim
        size_t lo = 0, hi = instances_.size() - 1;
        while (lo < hi) {
            const size_t mid = (lo + hi + 1) / 2;
            if (instances_[mid].first_prim <= prim) lo = mid;
            else hi = mid - 1;
        }
        ii = (uint32_t)lo;
    }
    if (inst) *inst = ii;
    if (local) *local = prim - instances_[ii].first_prim;
}

void Scene::bounds(float lo[3], float hi[3]) const {
    for (int k = 0; k < 3; ++k) { lo[k] = bounds_lo_[k]; hi[k] = bounds_hi_[k]; }
}

}  // namespace rt
