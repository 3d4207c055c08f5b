// ORACLE — test infrastructure only.  The host stand-ins for the shader interface the reference's GLSL
// uses (storage buffers, storage images, the texture array, push constants, the ray-tracing built-in
// variables and traceRayEXT), shared by every translated shader stage.  The state lives in
// glsl_runtime.cpp; the hit and miss stages are dispatched from there like the ray-tracing pipeline's
// shader binding table (hit group = the instance's SBT record offset, miss shader = the miss index).
#pragma once

#include "glsl_compat.h"

namespace glsl {

// Per-thread ray-tracing state: the launch id of the ray-generation invocation, the compute invocation
// id, and the built-ins of the hit or miss shader being run.
struct RtState {
    uvec3 launch_id;
    uvec3 global_id;
    int instance_custom_index;
    int primitive_id;
    float hit_t;
    vec2 attribs;
    mat4x3 object_to_world;
    vec3 world_ray_origin;
    vec3 world_ray_direction;
};
RtState& rt();

// storage buffers by binding: raw bytes written by the test through the C interface
const unsigned char* buffer_bytes(int binding, unsigned long long* size);
void note_out_of_range(int binding);

template <class T>
struct Field {   // a fixed member of a buffer block, at a byte offset (scalar layout)
    int binding;
    unsigned long long offset;
    Field(int b, unsigned long long o) : binding(b), offset(o) {}
    operator T() const {
        unsigned long long n = 0;
        const unsigned char* p = buffer_bytes(binding, &n);
        T v{};
        if (p && offset + sizeof(T) <= n) memcpy(&v, p + offset, sizeof(T));
        else note_out_of_range(binding);
        return v;
    }
};

template <class T>
struct View {   // the runtime-sized array member of a buffer block; out-of-range reads give T{} and are counted
    int binding;
    unsigned long long offset;
    View(int b, unsigned long long o) : binding(b), offset(o) {}
    T operator[](unsigned long long i) const {
        unsigned long long n = 0;
        const unsigned char* p = buffer_bytes(binding, &n);
        T v{};
        if (p && offset + (i + 1) * sizeof(T) <= n) memcpy(&v, p + offset + i * sizeof(T), sizeof(T));
        else note_out_of_range(binding);
        return v;
    }
    T operator[](int i) const { return (*this)[(unsigned long long)(long long)i]; }
    T operator[](uint i) const { return (*this)[(unsigned long long)i]; }
};

// storage images (rgba32f, or rgba8 written with UNORM conversion)
struct Image2D {
    int binding;
    explicit Image2D(int b) : binding(b) {}
};
vec4 imageLoad(const Image2D& im, ivec2 p);
void imageStore(const Image2D& im, ivec2 p, vec4 v);
ivec2 imageSize(const Image2D& im);

// combined image samplers: R8G8B8A8_UNORM textures, linear filter, repeat addressing, one mip level
struct sampler2D {
    int id;
};
struct SamplerArray {
    int binding;
    explicit SamplerArray(int b) : binding(b) {}
    sampler2D operator[](int i) const { return sampler2D{i}; }
};
vec4 texture(sampler2D s, vec2 uv);

// push constants: one block per dispatch
unsigned char* push_constant_bytes();
template <class T>
T& push_constants() { return *reinterpret_cast<T*>(push_constant_bytes()); }

// Vulkan ray flags used by the shaders
constexpr uint gl_RayFlagsOpaqueEXT = 1u;
constexpr uint gl_RayFlagsTerminateOnFirstHitEXT = 4u;
constexpr uint gl_RayFlagsSkipClosestHitShaderEXT = 8u;

// traceRayEXT: finds the closest hit (or, with TerminateOnFirstHit, any hit) in [tmin, tmax] and runs the
// hit group of the instance's SBT record (unless SkipClosestHitShader) or the miss shader `miss`, on the
// caller's payload bytes.
void trace_ray(uint flags, uint sbt_offset, uint miss, vec3 origin, float tmin, vec3 dir, float tmax, void* payload,
               unsigned long long payload_size);

using StageFn = void (*)(void* payload, unsigned long long size);
void register_hit_stage(int sbt_record, StageFn fn);
void register_miss_stage(int index, StageFn fn);

}  // namespace glsl

#define gl_LaunchIDEXT (glsl::rt().launch_id)
#define gl_GlobalInvocationID (glsl::rt().global_id)
#define gl_InstanceCustomIndexEXT (glsl::rt().instance_custom_index)
#define gl_PrimitiveID (glsl::rt().primitive_id)
#define gl_HitTEXT (glsl::rt().hit_t)
#define gl_ObjectToWorldEXT (glsl::rt().object_to_world)
#define gl_WorldRayOriginEXT (glsl::rt().world_ray_origin)
#define gl_WorldRayDirectionEXT (glsl::rt().world_ray_direction)
