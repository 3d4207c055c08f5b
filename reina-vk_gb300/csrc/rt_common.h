// Shared host/device definitions of the trace path: small vector math, the BVH8 node and triangle
// record layouts, and the ray/hit records.  Compiled both by g++ (host code) and nvcc (kernels).
#pragma once

#include <stdint.h>
#include <math.h>

#if defined(__CUDACC__)
#define RT_HD __host__ __device__ __forceinline__
#else
#define RT_HD inline
#endif

namespace rt {

struct V3 {
    float x, y, z;
};

RT_HD V3 v3(float x, float y, float z) { return V3{x, y, z}; }
RT_HD V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
RT_HD V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
RT_HD V3 operator-(V3 a) { return V3{-a.x, -a.y, -a.z}; }
RT_HD V3 operator*(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }
RT_HD V3 operator*(float s, V3 a) { return V3{a.x * s, a.y * s, a.z * s}; }
RT_HD V3 operator*(V3 a, V3 b) { return V3{a.x * b.x, a.y * b.y, a.z * b.z}; }
RT_HD V3 vmin(V3 a, V3 b) { return V3{fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)}; }
RT_HD V3 vmax(V3 a, V3 b) { return V3{fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)}; }
RT_HD float comp(V3 a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }

// One BVH8 node, 80 bytes = 5 x 16-byte words (compressed wide BVH in the style of Ylitie, Karras and
// Laine, "Efficient Incoherent Ray Traversal on GPUs Through Compressed Wide BVHs", HPG 2017):
//   w0: origin p (3 x f32), exponents ex, ey, ez (u8 each, scale = 2^(e - 127)), imask (u8)
//   w1: child_base (u32), tri_base (u32), meta[0..7] (u8)
//   w2: qlo_x[0..7], qlo_y[0..7]     w3: qlo_z[0..7], qhi_x[0..7]     w4: qhi_y[0..7], qhi_z[0..7]
// meta byte of child slot i:  0 = empty slot;
//   internal child: 0b001 << 5 | (24 + i)   (its node is child_base + popcount(imask & ((1 << i) - 1)))
//   leaf child:     unary(count) << 5 | offset, count in 1..3 (unary 0b001, 0b011, 0b111), triangles
//                   tri_base + offset .. tri_base + offset + count - 1.
// Child slot i holds a child whose centroid lies on the positive side of axis k iff bit k of i is set,
// so visiting slots in ascending order of (i XOR ray octant) is roughly front to back.
struct alignas(16) Bvh8Node {
    float px, py, pz;
    uint8_t ex, ey, ez, imask;
    uint32_t child_base;
    uint32_t tri_base;
    uint8_t meta[8];
    uint8_t qlo_x[8], qlo_y[8], qlo_z[8];
    uint8_t qhi_x[8], qhi_y[8], qhi_z[8];
};
static_assert(sizeof(Bvh8Node) == 80, "BVH8 node must be 80 bytes");

// Traversal triangle record, 48 bytes: world-space vertices and the global triangle id in v0.w (in a
// two-level scene: the model's object-space vertices and the triangle's index within the model).
struct alignas(16) TriRecord {
    float v0x, v0y, v0z;
    uint32_t prim;
    float v1x, v1y, v1z, pad1;
    float v2x, v2y, v2z, pad2;
};
static_assert(sizeof(TriRecord) == 48, "triangle record must be 48 bytes");

// Instance record of a two-level scene (TLAS leaves reference these): the world-to-object transform
// that carries a ray into the instance's model space, the node index of the model's bottom-level BVH
// root, and the global triangle id of the model's triangle 0 in this instance (global id = first_prim +
// the triangle record's local id).
struct alignas(16) InstanceTrav {
    float inv[12];          // row-major 3x4: object_r = sum_c inv[r*4+c] * world_c + inv[r*4+3]
    uint32_t blas_root;
    uint32_t first_prim;
    uint32_t pad0, pad1;
};
static_assert(sizeof(InstanceTrav) == 64, "instance record must be 64 bytes");

struct alignas(16) Ray {
    float ox, oy, oz, tmin;
    float dx, dy, dz, tmax;
};
static_assert(sizeof(Ray) == 32, "ray must be 32 bytes");

struct alignas(16) Hit {
    uint32_t prim;
    float t, u, v;
};
static_assert(sizeof(Hit) == 16, "hit must be 16 bytes");

constexpr uint32_t kMiss = 0xFFFFFFFFu;
constexpr int kMaxLeafTris = 3;

}  // namespace rt
