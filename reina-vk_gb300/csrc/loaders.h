// Scene loaders at the reference's boundary: Wavefront OBJ models (Scene::defineObject(path),
// src/scene/Models.cpp:117-175) and glTF 2.0 scenes (gltf::loadScene, src/scene/gltf/gltfloader.cpp).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "scene.h"

namespace rt {

// One OBJ file as one model: polygons fanned into triangles, one vertex per distinct (position, UV,
// normal) triple, smooth normals where the file has none (normalized sum of the unit face normals of all
// faces sharing the position), UVs flipped (v -> 1 - v), and per-vertex tangent frames from the UVs
// (zero tangent and bitangent when the file has no UVs).
ModelData load_obj(const std::string& path);
ModelData parse_obj(const std::string& text, const std::string& name);

struct GltfLoadStats {
    uint32_t meshes = 0, primitives = 0, instances = 0, skipped_primitives = 0, ignored_textures = 0;
};

// Adds the default scene of a .gltf / .glb file to `scene`: one object per triangle primitive of every
// mesh the scene's nodes use, one instance per (node, primitive) with the node's world matrix, and the
// primitive's material mapped as the reference maps it.
GltfLoadStats load_gltf(const std::string& path, Scene& scene);
GltfLoadStats load_gltf_memory(const uint8_t* data, size_t size, const std::string& base_dir, Scene& scene);

// Per-vertex tangent frames for an indexed triangle mesh: tangent and bitangent accumulated from the UV
// gradients of the incident triangles (Lengyel's method), then the tangent made orthogonal to the
// normal and the bitangent set to +-cross(N, T) by the UV handedness.  Where a vertex has no usable UV
// gradient, T is any unit vector orthogonal to N.  Outputs 9 floats per vertex (columns T, B, N).
void tangent_frames(const std::vector<float>& pos4, const std::vector<float>& normals3, const std::vector<float>& uv2,
                    const std::vector<uint32_t>& idx, std::vector<float>& tbn9);

}  // namespace rt
