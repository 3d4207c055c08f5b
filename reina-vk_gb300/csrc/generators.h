// Seeded synthetic workloads (icospheres, ray sets, camera matrices).
#pragma once

#include <cstdint>
#include <vector>

#include "rt_common.h"

namespace rt {

uint64_t splitmix64(uint64_t& state);
double splitmix_unit(uint64_t& state);
double fractal_noise3(double x, double y, double z, uint64_t seed);
void icosphere_counts(uint32_t level, uint64_t& nv, uint64_t& nt);
void gen_icosphere(uint32_t level, float amplitude, uint64_t seed, float* out_vertices, uint32_t* out_indices,
                   float* out_normals);
void geodesic_counts(uint32_t frequency, uint64_t& nv, uint64_t& nt);
void gen_geodesic(uint32_t frequency, float amplitude, uint64_t seed, float* out_vertices, uint32_t* out_indices,
                  float* out_normals);
void camera_matrices(const float pos[3], const float front[3], const float up[3], float fovy, float aspect,
                     float znear, float zfar, float inv_view[16], float inv_proj[16]);
void gen_raycast_rays(uint32_t width, uint32_t height, const float cam_pos[3], const float cam_target[3],
                      float fovy_degrees, uint64_t n_random, const float box_min[3], const float box_max[3],
                      uint64_t seed, Ray* out);

}  // namespace rt
