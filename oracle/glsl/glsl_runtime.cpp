// ORACLE — test infrastructure only.  State and dispatch behind glsl_runtime.h, and the C interface of
// oracle/_ref/libref_glsl.so: the reference's own shader code (translated by build_ref.py) run on the host.
//
//   ref_set_buffer(binding, bytes, n)     storage buffer contents, by the shaders' binding numbers
//   ref_set_scene(...)                    world-space triangles with (instance, primitive) ids, instances
//                                         (object-to-world 4x3, custom index, SBT record offset)
//   ref_set_textures(...)                 RGBA8 textures (texel rows as stored, v = 0 is the first row)
//   ref_render(push, W, H, image)         the ray-generation shader over every pixel (storage image binding 0)
//   ref_postprocess(...)                  blurX, blurY, combine and tonemapping as Reina::applyBloom and
//                                         Reina::applyTonemapping chain them (src/Reina.cpp:472-577)
//   ref_kat(kind, records, n, out)        single shader functions on 40-float case records (ref_kat.inc)
//
// traceRayEXT here: a binary BVH over the given world-space triangles, the watertight test of Woop,
// Benthin and Wald (JCGT 2(1), 2013) in binary32, closest hit = the lowest (t, triangle id) in
// [tmin, tmax] (the hardware's choice between equal t is unspecified; the lower id makes it defined).
#include "glsl_runtime.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

namespace glsl {

namespace {

struct Buffer {
    std::vector<unsigned char> bytes;
};
Buffer g_buffers[32];
std::atomic<unsigned long long> g_out_of_range{0};

struct Image {
    int w = 0, h = 0;
    bool rgba8 = false;
    float* f = nullptr;
    unsigned char* u8 = nullptr;
};
Image g_images[8];

struct Texture {
    int w = 0, h = 0;
    std::vector<uint32_t> texels;
};
std::vector<Texture> g_textures;

unsigned char g_push[256];

thread_local RtState t_rt;

StageFn g_hit[16] = {};
StageFn g_miss[4] = {};

// scene
struct Tri {
    float v[9];
    uint32_t inst, prim, id;
};
struct Inst {
    mat4x3 o2w;
    uint32_t custom, sbt;
};
std::vector<Tri> g_tris;
std::vector<Inst> g_inst;

struct Node {
    float lo[3], hi[3];
    uint32_t left_or_first, count;   // count 0: inner node, children left_or_first and left_or_first + 1
};
std::vector<Node> g_nodes;
std::vector<uint32_t> g_order;

void build_bvh() {
    g_nodes.clear();
    g_order.resize(g_tris.size());
    for (size_t i = 0; i < g_order.size(); ++i) g_order[i] = (uint32_t)i;
    if (g_tris.empty()) return;
    struct Item { uint32_t node, first, count; };
    g_nodes.push_back(Node{});
    std::vector<Item> work{{0u, 0u, (uint32_t)g_tris.size()}};
    auto cen = [](const Tri& t, int a) { return (t.v[a] + t.v[3 + a] + t.v[6 + a]) / 3.0f; };
    while (!work.empty()) {
        const Item it = work.back();
        work.pop_back();
        Node& nd = g_nodes[it.node];
        for (int a = 0; a < 3; ++a) { nd.lo[a] = INFINITY; nd.hi[a] = -INFINITY; }
        float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (uint32_t k = it.first; k < it.first + it.count; ++k) {
            const Tri& t = g_tris[g_order[k]];
            for (int a = 0; a < 3; ++a) {
                for (int v = 0; v < 3; ++v) {
                    nd.lo[a] = std::min(nd.lo[a], t.v[3 * v + a]);
                    nd.hi[a] = std::max(nd.hi[a], t.v[3 * v + a]);
                }
                clo[a] = std::min(clo[a], cen(t, a));
                chi[a] = std::max(chi[a], cen(t, a));
            }
        }
        if (it.count <= 4) {
            nd.left_or_first = it.first;
            nd.count = it.count;
            continue;
        }
        int axis = 0;
        for (int a = 1; a < 3; ++a)
            if (chi[a] - clo[a] > chi[axis] - clo[axis]) axis = a;
        const uint32_t mid = it.first + it.count / 2;
        std::nth_element(g_order.begin() + it.first, g_order.begin() + mid, g_order.begin() + it.first + it.count,
                         [&](uint32_t a, uint32_t b) { return cen(g_tris[a], axis) < cen(g_tris[b], axis); });
        const uint32_t left = (uint32_t)g_nodes.size();
        g_nodes.push_back(Node{});
        g_nodes.push_back(Node{});
        g_nodes[it.node].left_or_first = left;
        g_nodes[it.node].count = 0;
        work.push_back({left, it.first, mid - it.first});
        work.push_back({left + 1, mid, it.first + it.count - mid});
    }
}

struct Ray {
    float o[3], d[3], tmin, tmax;
    int kx, ky, kz;
    float sx, sy, sz;
    float inv[3];
};

Ray make_ray(vec3 o, vec3 d, float tmin, float tmax) {
    Ray r;
    r.o[0] = o.x; r.o[1] = o.y; r.o[2] = o.z;
    r.d[0] = d.x; r.d[1] = d.y; r.d[2] = d.z;
    r.tmin = tmin; r.tmax = tmax;
    const float ax = std::fabs(d.x), ay = std::fabs(d.y), az = std::fabs(d.z);
    int kz = (ax >= ay) ? ((ax >= az) ? 0 : 2) : ((ay >= az) ? 1 : 2);
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    if (r.d[kz] < 0.0f) std::swap(kx, ky);
    r.kx = kx; r.ky = ky; r.kz = kz;
    r.sx = r.d[kx] / r.d[kz];
    r.sy = r.d[ky] / r.d[kz];
    r.sz = 1.0f / r.d[kz];
    for (int a = 0; a < 3; ++a) r.inv[a] = 1.0f / r.d[a];
    return r;
}

// watertight ray/triangle test; on a hit in [tmin, tmax] gives t and the weights of v1 (u) and v2 (v)
bool hit_triangle(const Ray& r, const float* v, float tmax, float& t, float& u, float& w) {
    float A[3], B[3], C[3];
    for (int a = 0; a < 3; ++a) { A[a] = v[a] - r.o[a]; B[a] = v[3 + a] - r.o[a]; C[a] = v[6 + a] - r.o[a]; }
    const float Ax = A[r.kx] - r.sx * A[r.kz], Ay = A[r.ky] - r.sy * A[r.kz];
    const float Bx = B[r.kx] - r.sx * B[r.kz], By = B[r.ky] - r.sy * B[r.kz];
    const float Cx = C[r.kx] - r.sx * C[r.kz], Cy = C[r.ky] - r.sy * C[r.kz];
    float U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {   // exact signs: products of floats are exact in double
        U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
        V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
        W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = U + V + W;
    if (det == 0.0f) return false;
    const float Az = r.sz * A[r.kz], Bz = r.sz * B[r.kz], Cz = r.sz * C[r.kz];
    const float T = U * Az + V * Bz + W * Cz;
    const float rcp = 1.0f / det;
    const float tt = T * rcp;
    if (!(tt >= r.tmin && tt <= tmax)) return false;
    t = tt;
    u = V * rcp;
    w = W * rcp;
    return true;
}

bool box_hit(const Ray& r, const Node& n, float tmax) {
    float t0 = r.tmin, t1 = tmax;
    for (int a = 0; a < 3; ++a) {
        float lo = (n.lo[a] - r.o[a]) * r.inv[a], hi = (n.hi[a] - r.o[a]) * r.inv[a];
        if (lo > hi) std::swap(lo, hi);
        if (std::isnan(lo) || std::isnan(hi)) { lo = -INFINITY; hi = INFINITY; }   // origin on a slab plane, d = 0
        // widen by a few ulps so that the box test is conservative for the watertight triangle test
        lo = lo - std::fabs(lo) * 1e-6f;
        hi = hi + std::fabs(hi) * 1e-6f;
        t0 = std::max(t0, lo);
        t1 = std::min(t1, hi);
    }
    return t0 <= t1;
}

// closest (or, any_hit, the first found) triangle hit; returns the triangle index or -1
long find_hit(const Ray& r, bool any_hit, float& t_out, float& u_out, float& v_out) {
    if (g_nodes.empty()) return -1;
    long best = -1;
    float best_t = r.tmax;
    uint32_t best_id = 0xFFFFFFFFu;
    uint32_t stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp) {
        const Node& n = g_nodes[stack[--sp]];
        if (!box_hit(r, n, best_t)) continue;
        if (n.count == 0) {
            if (sp + 2 > 128) return best;   // depth is bounded by the median split; never reached
            stack[sp++] = n.left_or_first;
            stack[sp++] = n.left_or_first + 1;
            continue;
        }
        for (uint32_t k = n.left_or_first; k < n.left_or_first + n.count; ++k) {
            const Tri& tr = g_tris[g_order[k]];
            float t, u, w;
            if (!hit_triangle(r, tr.v, best_t, t, u, w)) continue;
            if (best < 0 || t < best_t || tr.id < best_id) {
                best = g_order[k]; best_t = t; best_id = tr.id; t_out = t; u_out = u; v_out = w;
                if (any_hit) return best;
            }
        }
    }
    return best;
}

}  // namespace

RtState& rt() { return t_rt; }

const unsigned char* buffer_bytes(int binding, unsigned long long* size) {
    if (binding < 0 || binding >= 32) { *size = 0; return nullptr; }
    *size = g_buffers[binding].bytes.size();
    return g_buffers[binding].bytes.empty() ? nullptr : g_buffers[binding].bytes.data();
}
void note_out_of_range(int) { g_out_of_range.fetch_add(1); }

vec4 imageLoad(const Image2D& im, ivec2 p) {
    const Image& g = g_images[im.binding];
    if (p.x < 0 || p.y < 0 || p.x >= g.w || p.y >= g.h) return vec4(0.0f);   // out of range reads zero (robust access)
    const size_t i = ((size_t)p.y * g.w + p.x) * 4;
    if (g.rgba8) return vec4(g.u8[i] / 255.0f, g.u8[i + 1] / 255.0f, g.u8[i + 2] / 255.0f, g.u8[i + 3] / 255.0f);
    return vec4(g.f[i], g.f[i + 1], g.f[i + 2], g.f[i + 3]);
}
void imageStore(const Image2D& im, ivec2 p, vec4 v) {
    Image& g = g_images[im.binding];
    if (p.x < 0 || p.y < 0 || p.x >= g.w || p.y >= g.h) return;
    const size_t i = ((size_t)p.y * g.w + p.x) * 4;
    const float c[4] = {v.x, v.y, v.z, v.w};
    for (int k = 0; k < 4; ++k) {
        if (g.rgba8) {   // UNORM8: clamp to [0, 1], scale by 255, round to nearest
            float x = c[k];
            x = x != x ? 0.0f : std::min(std::max(x, 0.0f), 1.0f);
            g.u8[i + k] = (unsigned char)std::lrint(x * 255.0f);
        } else {
            g.f[i + k] = c[k];
        }
    }
}
ivec2 imageSize(const Image2D& im) { return ivec2(g_images[im.binding].w, g_images[im.binding].h); }

// Linear filtering with repeat addressing (Vulkan, "Texel Filtering"): u' = u W - 1/2, i0 = floor(u'),
// alpha = frac(u'); the four texels are converted from UNORM to float, then weighted.
vec4 texture(sampler2D s, vec2 uv) {
    if (s.id < 0 || s.id >= (int)g_textures.size() || g_textures[s.id].w == 0) { note_out_of_range(-1); return vec4(0.0f); }
    const Texture& t = g_textures[s.id];
    const float u = uv.x * (float)t.w - 0.5f, v = uv.y * (float)t.h - 0.5f;
    const float fu = std::floor(u), fv = std::floor(v);
    const float a = u - fu, b = v - fv;
    auto wrap = [](long i, int n) { long m = i % n; return (int)(m < 0 ? m + n : m); };
    const long i0 = std::isfinite(fu) ? (long)fu : 0, j0 = std::isfinite(fv) ? (long)fv : 0;
    auto texel = [&](long i, long j) {
        const uint32_t x = t.texels[(size_t)wrap(j, t.h) * t.w + wrap(i, t.w)];
        return vec4((x & 255u) / 255.0f, ((x >> 8) & 255u) / 255.0f, ((x >> 16) & 255u) / 255.0f, (x >> 24) / 255.0f);
    };
    const vec4 t00 = texel(i0, j0), t10 = texel(i0 + 1, j0), t01 = texel(i0, j0 + 1), t11 = texel(i0 + 1, j0 + 1);
    vec4 r;
    for (int k = 0; k < 4; ++k)
        (&r.x)[k] = (1.0f - a) * (1.0f - b) * (&t00.x)[k] + a * (1.0f - b) * (&t10.x)[k] + (1.0f - a) * b * (&t01.x)[k] +
                    a * b * (&t11.x)[k];
    return r;
}

unsigned char* push_constant_bytes() { return g_push; }

void register_hit_stage(int sbt_record, StageFn fn) { g_hit[sbt_record] = fn; }
void register_miss_stage(int index, StageFn fn) { g_miss[index] = fn; }

void trace_ray(uint flags, uint sbt_offset, uint miss, vec3 origin, float tmin, vec3 dir, float tmax, void* payload,
               unsigned long long payload_size) {
    const Ray r = make_ray(origin, dir, tmin, tmax);
    float t = 0.0f, u = 0.0f, v = 0.0f;
    const long k = find_hit(r, (flags & gl_RayFlagsTerminateOnFirstHitEXT) != 0, t, u, v);
    const RtState saved = t_rt;
    t_rt.world_ray_origin = origin;
    t_rt.world_ray_direction = dir;
    if (k >= 0) {
        if (flags & gl_RayFlagsSkipClosestHitShaderEXT) { t_rt = saved; return; }
        const Tri& tr = g_tris[k];
        const Inst& in = g_inst[tr.inst];
        t_rt.instance_custom_index = (int)in.custom;
        t_rt.primitive_id = (int)tr.prim;
        t_rt.hit_t = t;
        t_rt.attribs = vec2(u, v);
        t_rt.object_to_world = in.o2w;
        const uint rec = sbt_offset + in.sbt;
        if (rec < 16 && g_hit[rec]) g_hit[rec](payload, payload_size);
        else note_out_of_range(-2);
    } else {
        if (miss < 4 && g_miss[miss]) g_miss[miss](payload, payload_size);
        else note_out_of_range(-3);
    }
    t_rt = saved;
}

}  // namespace glsl

using namespace glsl;

// stage entry points of the translated shaders (ref_stages.cpp, written by build_ref.py)
void ref_register_stages();
void ref_stage_raygen();
void ref_stage_blur_x();
void ref_stage_blur_y();
void ref_stage_combine();
void ref_stage_tonemap();
extern "C" void ref_kat_dispatch(int kind, const float* records, unsigned long long n, double* out);

extern "C" {

int ref_init() {
    ref_register_stages();
    return 0;
}

void ref_set_buffer(int binding, const void* data, unsigned long long bytes) {
    if (binding < 0 || binding >= 32) return;
    const unsigned char* p = static_cast<const unsigned char*>(data);
    g_buffers[binding].bytes.assign(p, p + bytes);
}

// tris9: world-space vertices (9 floats per triangle); tri_inst / tri_prim / tri_id: the triangle's
// instance, its index within the instance's model (gl_PrimitiveID) and its global id (tie order);
// o2w12: per instance the object-to-world matrix as 4 columns of 3 rows; custom / sbt per instance.
void ref_set_scene(const float* tris9, const uint32_t* tri_inst, const uint32_t* tri_prim, const uint32_t* tri_id,
                   unsigned long long n_tris, const float* o2w12, const uint32_t* custom, const uint32_t* sbt,
                   unsigned long long n_inst) {
    g_tris.resize(n_tris);
    for (unsigned long long i = 0; i < n_tris; ++i) {
        std::memcpy(g_tris[i].v, tris9 + 9 * i, 36);
        g_tris[i].inst = tri_inst[i];
        g_tris[i].prim = tri_prim[i];
        g_tris[i].id = tri_id[i];
    }
    g_inst.resize(n_inst);
    for (unsigned long long i = 0; i < n_inst; ++i) {
        for (int c = 0; c < 4; ++c) g_inst[i].o2w.c[c] = vec3(o2w12[12 * i + 3 * c], o2w12[12 * i + 3 * c + 1], o2w12[12 * i + 3 * c + 2]);
        g_inst[i].custom = custom[i];
        g_inst[i].sbt = sbt[i];
    }
    build_bvh();
}

void ref_set_textures(unsigned long long count, const uint32_t* widths, const uint32_t* heights, const uint32_t* texels) {
    g_textures.assign(count, Texture{});
    size_t off = 0;
    for (unsigned long long i = 0; i < count; ++i) {
        g_textures[i].w = (int)widths[i];
        g_textures[i].h = (int)heights[i];
        g_textures[i].texels.assign(texels + off, texels + off + (size_t)widths[i] * heights[i]);
        off += (size_t)widths[i] * heights[i];
    }
}

unsigned long long ref_out_of_range() { return g_out_of_range.load(); }

// The ray-generation shader over a W x H launch; `image` (RGBA32F, read when sampleBatch > 0) is the
// storage image at binding 0.  Rows are shared out over `threads` host threads.
void ref_render(const void* push_consts, unsigned long long push_bytes, int W, int H, float* image, int threads) {
    std::memcpy(g_push, push_consts, std::min<unsigned long long>(push_bytes, sizeof(g_push)));
    g_images[0] = Image{W, H, false, image, nullptr};
    if (threads < 1) threads = 1;
    std::atomic<int> next_row{0};
    auto work = [&]() {
        for (;;) {
            const int y = next_row.fetch_add(1);
            if (y >= H) return;
            for (int x = 0; x < W; ++x) {
                t_rt = RtState{};
                t_rt.launch_id = uvec3{(uint)x, (uint)y, 0u};
                ref_stage_raygen();
            }
        }
    };
    std::vector<std::thread> pool;
    for (int i = 1; i < threads; ++i) pool.emplace_back(work);
    work();
    for (auto& t : pool) t.join();
}

// Reina::applyBloom + applyTonemapping: blurX (accum -> ping), blurY (ping -> pong), combine (accum, pong
// -> ping), tonemapping (ping -> rgba8).  bloom_push: radius, threshold, intensity; tonemap_push: exposure.
void ref_postprocess(const float* accum, int W, int H, const float* bloom_push, const float* tonemap_push,
                     float* bloomed, unsigned char* rgba8) {
    std::vector<float> in(accum, accum + (size_t)W * H * 4), ping((size_t)W * H * 4), pong((size_t)W * H * 4);
    auto dispatch = [&](void (*stage)()) {
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                t_rt = RtState{};
                t_rt.global_id = uvec3{(uint)x, (uint)y, 0u};
                stage();
            }
    };
    std::memcpy(g_push, bloom_push, 12);
    g_images[0] = Image{W, H, false, in.data(), nullptr};
    g_images[1] = Image{W, H, false, ping.data(), nullptr};
    dispatch(ref_stage_blur_x);
    g_images[0] = Image{W, H, false, ping.data(), nullptr};
    g_images[1] = Image{W, H, false, pong.data(), nullptr};
    dispatch(ref_stage_blur_y);
    g_images[0] = Image{W, H, false, in.data(), nullptr};
    g_images[1] = Image{W, H, false, pong.data(), nullptr};
    g_images[2] = Image{W, H, false, ping.data(), nullptr};
    dispatch(ref_stage_combine);
    if (bloomed) std::memcpy(bloomed, ping.data(), ping.size() * sizeof(float));
    std::memcpy(g_push, tonemap_push, 4);
    g_images[0] = Image{W, H, false, ping.data(), nullptr};
    g_images[1] = Image{W, H, true, nullptr, rgba8};
    dispatch(ref_stage_tonemap);
}

void ref_kat(int kind, const float* records, unsigned long long n, double* out) { ref_kat_dispatch(kind, records, n, out); }

}  // extern "C"
