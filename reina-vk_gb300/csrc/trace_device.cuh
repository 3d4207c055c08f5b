// Device-side BVH8 traversal (closest hit and any hit) with a per-thread short stack in shared memory,
// and the watertight ray/triangle test of Woop, Benthin and Wald, "Watertight Ray/Triangle
// Intersection", JCGT 2(1), 2013.  Replaces the hardware traversal behind traceRayEXT
// (shaders/raytrace/raytrace.rgen.glsl:159-171 and shaders/raytrace/nee.h.glsl:129-141).
//
// The triangle test is written with explicitly rounded intrinsics (__fmul_rn, __fadd_rn, ...), which
// nvcc never contracts into FMAs, so that its results (hit/miss, t, u, v) are bit-identical to an IEEE
// single-precision evaluation of the same expressions on the host.
#pragma once

#include <stdint.h>

#include "device_scene.h"
#include "rt_common.h"

namespace rt {

// Shared-memory stack entries per thread; deeper levels spill to a small local array.
#ifndef RT_SMEM_STACK
#define RT_SMEM_STACK 12
#endif
constexpr int kSmemStack = RT_SMEM_STACK;
constexpr int kTotalStack = 64;          // == kMaxBvhDepth: one entry per BVH8 level at most
// Watchdog: a ray's traversal ends with kErrStepLimit after this many steps (a node visit and its
// triangle tests each).  Far above any finite traversal of a valid tree; a build may lower it
// (-DRT_MAX_TRAVERSAL_STEPS=n) to exercise the error path on ordinary scenes.
#ifndef RT_MAX_TRAVERSAL_STEPS
#define RT_MAX_TRAVERSAL_STEPS (1u << 22)
#endif
constexpr uint32_t kMaxTraversalSteps = RT_MAX_TRAVERSAL_STEPS;

constexpr uint32_t kErrStackOverflow = 1u;
constexpr uint32_t kErrStepLimit = 2u;

struct TraceRay {
    float ox, oy, oz;
    float dx, dy, dz;
    float idx, idy, idz;        // reciprocal direction (box test only)
    float tmin, tmax;
    float sx, sy, sz;           // watertight shear constants
    int kx, ky, kz;
    uint32_t oct_inv;
};

__device__ __forceinline__ float pick3(float x, float y, float z, int k) { return k == 0 ? x : (k == 1 ? y : z); }
__device__ __forceinline__ double pick3d(double x, double y, double z, int k) { return k == 0 ? x : (k == 1 ? y : z); }

__device__ __forceinline__ float safe_rcp(float d) {
    // Only the box test uses this reciprocal; zero components become a huge finite value.  __frcp_rn is
    // the correctly rounded 1/d, the same value as the division, in fewer instructions.
    const float ad = fabsf(d);
    return ad > 1e-30f ? __frcp_rn(d) : copysignf(1e30f, d);
}

__device__ __forceinline__ TraceRay make_trace_ray(float ox, float oy, float oz, float dx, float dy, float dz,
                                                   float tmin, float tmax) {
    TraceRay r;
    r.ox = ox; r.oy = oy; r.oz = oz;
    r.dx = dx; r.dy = dy; r.dz = dz;
    r.tmin = tmin; r.tmax = tmax;
    r.idx = safe_rcp(dx); r.idy = safe_rcp(dy); r.idz = safe_rcp(dz);
    const float ax = fabsf(dx), ay = fabsf(dy), az = fabsf(dz);
    int kz = (ax >= ay) ? ((ax >= az) ? 0 : 2) : ((ay >= az) ? 1 : 2);
    int kx = kz + 1; if (kx == 3) kx = 0;
    int ky = kx + 1; if (ky == 3) ky = 0;
    const float dkz = pick3(dx, dy, dz, kz);
    if (dkz < 0.0f) { int t = kx; kx = ky; ky = t; }
    r.kx = kx; r.ky = ky; r.kz = kz;
    r.sx = __fdiv_rn(pick3(dx, dy, dz, kx), dkz);
    r.sy = __fdiv_rn(pick3(dx, dy, dz, ky), dkz);
    r.sz = __frcp_rn(dkz);
    const uint32_t oct = (dx < 0.0f ? 1u : 0u) | (dy < 0.0f ? 2u : 0u) | (dz < 0.0f ? 4u : 0u);
    r.oct_inv = 7u - oct;
    return r;
}

// Watertight test; on a hit within [tmin, tmax] writes t and the barycentric weights (u of v1, v of v2).
__device__ __forceinline__ bool intersect_triangle(const TraceRay& r, const float4& a4, const float4& b4,
                                                   const float4& c4, float tmax, float& t_out, float& u_out,
                                                   float& v_out) {
    const float Ax0 = __fsub_rn(a4.x, r.ox), Ay0 = __fsub_rn(a4.y, r.oy), Az0 = __fsub_rn(a4.z, r.oz);
    const float Bx0 = __fsub_rn(b4.x, r.ox), By0 = __fsub_rn(b4.y, r.oy), Bz0 = __fsub_rn(b4.z, r.oz);
    const float Cx0 = __fsub_rn(c4.x, r.ox), Cy0 = __fsub_rn(c4.y, r.oy), Cz0 = __fsub_rn(c4.z, r.oz);
    const float Akx = pick3(Ax0, Ay0, Az0, r.kx), Aky = pick3(Ax0, Ay0, Az0, r.ky), Akz = pick3(Ax0, Ay0, Az0, r.kz);
    const float Bkx = pick3(Bx0, By0, Bz0, r.kx), Bky = pick3(Bx0, By0, Bz0, r.ky), Bkz = pick3(Bx0, By0, Bz0, r.kz);
    const float Ckx = pick3(Cx0, Cy0, Cz0, r.kx), Cky = pick3(Cx0, Cy0, Cz0, r.ky), Ckz = pick3(Cx0, Cy0, Cz0, r.kz);
    const float Ax = __fsub_rn(Akx, __fmul_rn(r.sx, Akz));
    const float Ay = __fsub_rn(Aky, __fmul_rn(r.sy, Akz));
    const float Bx = __fsub_rn(Bkx, __fmul_rn(r.sx, Bkz));
    const float By = __fsub_rn(Bky, __fmul_rn(r.sy, Bkz));
    const float Cx = __fsub_rn(Ckx, __fmul_rn(r.sx, Ckz));
    const float Cy = __fsub_rn(Cky, __fmul_rn(r.sy, Ckz));
    float U = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
    float V = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
    float W = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        // Exact-sign fallback of the paper: float products are exact in double.
        const double CxBy = __dmul_rn((double)Cx, (double)By), CyBx = __dmul_rn((double)Cy, (double)Bx);
        const double AxCy = __dmul_rn((double)Ax, (double)Cy), AyCx = __dmul_rn((double)Ay, (double)Cx);
        const double BxAy = __dmul_rn((double)Bx, (double)Ay), ByAx = __dmul_rn((double)By, (double)Ax);
        U = __double2float_rn(__dsub_rn(CxBy, CyBx));
        V = __double2float_rn(__dsub_rn(AxCy, AyCx));
        W = __double2float_rn(__dsub_rn(BxAy, ByAx));
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = __fadd_rn(__fadd_rn(U, V), W);
    if (det == 0.0f) return false;
    const float Az = __fmul_rn(r.sz, Akz), Bz = __fmul_rn(r.sz, Bkz), Cz = __fmul_rn(r.sz, Ckz);
    const float T = __fadd_rn(__fadd_rn(__fmul_rn(U, Az), __fmul_rn(V, Bz)), __fmul_rn(W, Cz));
    const float rcp = __frcp_rn(det);
    const float t = __fmul_rn(T, rcp);
    if (!(t >= r.tmin && t <= tmax)) return false;
    t_out = t;
    u_out = __fmul_rn(V, rcp);
    v_out = __fmul_rn(W, rcp);
    return true;
}

// Re-evaluates t, u, v of the selected triangle from an origin moved along the ray onto the hit point.
// The FP32 test above decides which triangle is hit; this only sharpens the reported values (with a far
// origin, FP32 barycentrics lose ~1e-5 of the triangle's size to cancellation).  The moved origin
// o + t0 d is formed exactly as hi + lo with FMA-based TwoProduct and TwoSum (error-free transforms,
// Ogita, Rump and Oishi, SIAM J. Sci. Comput. 26(6), 2005), so the vertex offsets are small and accurate;
// a Möller–Trumbore evaluation there, with Kahan's FMA difference of products for the cross products
// and the compensated dot product Dot2, gives barycentrics within ~1e-5 of exact, and t = t0 + t'.
// Single precision only: GB300's FP64 rate is too low for a per-ray double evaluation.
__device__ __forceinline__ void two_sum_f(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void two_prod_f(float a, float b, float& p, float& e) {
    p = __fmul_rn(a, b);
    e = __fmaf_rn(a, b, -p);
}
__device__ __forceinline__ float diff_prod_f(float a, float b, float c, float d) {   // a*b - c*d
    const float w = __fmul_rn(c, d);
    const float e = __fmaf_rn(-c, d, w);
    const float f = __fmaf_rn(a, b, -w);
    return __fadd_rn(f, e);
}
__device__ __forceinline__ float dot2_f(float x0, float x1, float x2, float y0, float y1, float y2) {
    float p, s, h, r, q;
    two_prod_f(x0, y0, p, s);
    two_prod_f(x1, y1, h, r);
    two_sum_f(p, h, p, q);
    s = __fadd_rn(s, __fadd_rn(q, r));
    two_prod_f(x2, y2, h, r);
    two_sum_f(p, h, p, q);
    s = __fadd_rn(s, __fadd_rn(q, r));
    return __fadd_rn(p, s);
}

__device__ __forceinline__ void refine_hit(const TraceRay& r, const float4& a4, const float4& b4, const float4& c4,
                                           Hit& h) {
    const float t0 = h.t;
    auto moved = [&](float o, float d, float v0) {   // (o + t0 d) - v0 with the moved origin kept exactly
        float ph, pl, sh, sl;
        two_prod_f(t0, d, ph, pl);
        two_sum_f(o, ph, sh, sl);
        return __fadd_rn(__fsub_rn(sh, v0), __fadd_rn(sl, pl));
    };
    const float s0 = moved(r.ox, r.dx, a4.x), s1 = moved(r.oy, r.dy, a4.y), s2 = moved(r.oz, r.dz, a4.z);
    const float e10 = __fsub_rn(b4.x, a4.x), e11 = __fsub_rn(b4.y, a4.y), e12 = __fsub_rn(b4.z, a4.z);
    const float e20 = __fsub_rn(c4.x, a4.x), e21 = __fsub_rn(c4.y, a4.y), e22 = __fsub_rn(c4.z, a4.z);
    const float p0 = diff_prod_f(r.dy, e22, r.dz, e21), p1 = diff_prod_f(r.dz, e20, r.dx, e22),
                p2 = diff_prod_f(r.dx, e21, r.dy, e20);
    const float det = dot2_f(e10, e11, e12, p0, p1, p2);
    if (det == 0.0f) return;
    const float q0 = diff_prod_f(s1, e12, s2, e11), q1 = diff_prod_f(s2, e10, s0, e12), q2 = diff_prod_f(s0, e11, s1, e10);
    h.u = __fdiv_rn(dot2_f(s0, s1, s2, p0, p1, p2), det);
    h.v = __fdiv_rn(dot2_f(r.dx, r.dy, r.dz, q0, q1, q2), det);
    h.t = __fadd_rn(t0, __fdiv_rn(dot2_f(e20, e21, e22, q0, q1, q2), det));
}

// The bits of 1.0f, read by the byte permutes of the box test from the constant bank: as an immediate the
// compiler materialises it in a register before each permute (one register move per plane, 48 per node
// visit), as a constant-bank operand the permute reads it directly (1.3M-triangle ray cast: 426 M -> 394 M
// warp instructions, 0.507 -> 0.487 ms).
static __constant__ uint32_t kOneBits = 0x3F800000u;

// Byte `byte` of `word` as the float 1 + q * 2^-15, exactly: the byte placed in mantissa bits 8..15 of
// 1.0 by one byte permute (no conversion or subtraction).
__device__ __forceinline__ float q15(uint32_t word, int byte) {
    return __uint_as_float(__byte_perm(word, kOneBits, 0x7604u | ((uint32_t)byte << 4)));
}

// Node meta bytes with the octant applied: internal children (meta bits 3 and 4 both set; leaf offsets
// are below 24) get their bit index XOR-ed with the ray's inverse octant, four children per word.
__device__ __forceinline__ uint32_t octant_meta(uint32_t m, uint32_t oct_inv) {
    const uint32_t inner = (m & (m << 1)) & 0x10101010u;
    return m ^ ((inner >> 4) * oct_inv);
}

// Intersects the 8 quantized child boxes of one node; returns the hit mask in the CWBVH layout
// (bits 24..31: internal children, reordered by the ray octant; bits 0..23: leaf triangles).
// A child plane at q quanta is at t = (1 + q 2^-15) S + O with S = 2^15 quanta in t units and
// O = (p - o) / d - S: one byte permute and one FMA per plane.  Forming O adds one rounding of at most
// 2^-9 quanta (2^-24 of |S|), which the builder's 2^-8-quantum margin around every child box covers.
// Empty slots have meta 0 and contribute nothing to the mask.
__device__ __forceinline__ uint32_t intersect_children(const TraceRay& r, const uint4& w0, const uint4& w1,
                                                       const uint4& w2, const uint4& w3, const uint4& w4,
                                                       float tmax) {
    const float px = __uint_as_float(w0.x), py = __uint_as_float(w0.y), pz = __uint_as_float(w0.z);
    const uint32_t ex = w0.w & 0xFFu, ey = (w0.w >> 8) & 0xFFu, ez = (w0.w >> 16) & 0xFFu;
    const float sx = __uint_as_float((ex + 15u) << 23) * r.idx;
    const float sy = __uint_as_float((ey + 15u) << 23) * r.idy;
    const float sz = __uint_as_float((ez + 15u) << 23) * r.idz;
    const float ox = (px - r.ox) * r.idx - sx;
    const float oy = (py - r.oy) * r.idy - sy;
    const float oz = (pz - r.oz) * r.idz - sz;
    // Near/far plane words by direction sign (qlo_x = w2.xy, qlo_y = w2.zw, qlo_z = w3.xy,
    // qhi_x = w3.zw, qhi_y = w4.xy, qhi_z = w4.zw).
    const bool nx = r.idx < 0.0f, ny = r.idy < 0.0f, nz = r.idz < 0.0f;
    const uint32_t nearx0 = nx ? w3.z : w2.x, nearx1 = nx ? w3.w : w2.y;
    const uint32_t farx0 = nx ? w2.x : w3.z, farx1 = nx ? w2.y : w3.w;
    const uint32_t neary0 = ny ? w4.x : w2.z, neary1 = ny ? w4.y : w2.w;
    const uint32_t fary0 = ny ? w2.z : w4.x, fary1 = ny ? w2.w : w4.y;
    const uint32_t nearz0 = nz ? w4.z : w3.x, nearz1 = nz ? w4.w : w3.y;
    const uint32_t farz0 = nz ? w3.x : w4.z, farz1 = nz ? w3.y : w4.w;
    const uint32_t meta0 = octant_meta(w1.z, r.oct_inv), meta1 = octant_meta(w1.w, r.oct_inv);
    uint32_t hitmask = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int b = i & 3;
        const float tnx = fmaf(q15(i < 4 ? nearx0 : nearx1, b), sx, ox);
        const float tny = fmaf(q15(i < 4 ? neary0 : neary1, b), sy, oy);
        const float tnz = fmaf(q15(i < 4 ? nearz0 : nearz1, b), sz, oz);
        const float tfx = fmaf(q15(i < 4 ? farx0 : farx1, b), sx, ox);
        const float tfy = fmaf(q15(i < 4 ? fary0 : fary1, b), sy, oy);
        const float tfz = fmaf(q15(i < 4 ? farz0 : farz1, b), sz, oz);
        const float tn = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, r.tmin));
        const float tf = fminf(fminf(tfx, tfy), fminf(tfz, tmax));
        if (tn <= tf) {
            const uint32_t meta = ((i < 4 ? meta0 : meta1) >> (8 * b)) & 0xFFu;
            hitmask |= (meta >> 5) << (meta & 31u);
        }
    }
    return hitmask;
}

struct TraceCounters {
    uint32_t nodes;
    uint32_t tris;
};

// Resumable traversal state of one ray (the shared-memory stack and the local spill array live with
// the caller).  Closest hit: the lowest (t, prim) over all triangles hit in [tmin, tmax].  Any hit: the
// first triangle found hit in [tmin, tmax].
struct TravState {
    uint2 group;        // current node group: child base, node hits (bits 24..31) | internal mask
    float best_t;
    uint32_t best_rec;  // triangle record of the current best hit
    int sp;
    uint32_t steps;
};

__device__ __forceinline__ void trav_init(const TraceRay& r, TravState& s, Hit& hit) {
    s.group = make_uint2(0u, 0x80000000u);
    s.best_t = r.tmax;
    s.best_rec = 0;
    s.sp = 0;
    s.steps = 0;
    hit.prim = kMiss;
    hit.t = r.tmax;
    hit.u = 0.0f;
    hit.v = 0.0f;
}

// Triangle postponing (Ylitie, Karras and Laine, "Efficient Incoherent Ray Traversal on GPUs Through
// Compressed Wide BVHs", HPG 2017): a lane with triangles to test defers them (pushes its triangle group
// on the stack and goes on with nodes) while fewer than kPostpone/32 of the warp's traversing lanes have
// triangles too, so that triangle tests run with more lanes active.  0 disables postponing; any-hit
// traversal never postpones (its rays end at the first hit found).
#ifndef RT_POSTPONE
#define RT_POSTPONE 6
#endif
constexpr int kPostpone = RT_POSTPONE;


// One traversal step.  Stack entries and the current group are node groups (child base, node hits in
// bits 24..31 | internal mask) or postponed triangle groups (triangle base, triangle hits in bits
// 0..23, bits 24..31 zero).  A step visits the nearest pending child node (or takes a popped triangle
// group) and tests the group's triangles unless it postpones them.  Returns true when the ray is done.
template <bool ANY, bool COUNT, int SS = kSmemStack>
__device__ __forceinline__ bool trav_step(const Bvh8Node* __restrict__ nodes, const TriRecord* __restrict__ tris,
                                          const TraceRay& r, TravState& s, Hit& hit, uint2* stack, int stride,
                                          uint2* spill, TraceCounters& cnt, uint32_t& err) {
    if (++s.steps > kMaxTraversalSteps) { err |= kErrStepLimit; return true; }
    constexpr bool kPost = kPostpone > 0 && !ANY;   // any-hit rays stop at their first hit: never postpone
    const uint32_t traversing = kPost ? (uint32_t)__popc(__activemask()) : 0u;
    const uint4* nptr = reinterpret_cast<const uint4*>(nodes);
    const float4* tptr = reinterpret_cast<const float4*>(tris);
    uint2 tgroup;
    if (s.group.y > 0x00FFFFFFu) {
        const uint32_t slot_bit = 31u - __clz(s.group.y);
        const uint32_t slot = (slot_bit - 24u) ^ r.oct_inv;
        const uint32_t rel = __popc(s.group.y & ((1u << slot) - 1u));
        const uint32_t child = s.group.x + rel;
        s.group.y &= ~(1u << slot_bit);
        if (s.group.y > 0x00FFFFFFu) {
            if (s.sp < SS) stack[s.sp * stride] = s.group;
            else if (s.sp < kTotalStack) spill[s.sp - SS] = s.group;
            else { err |= kErrStackOverflow; return true; }
            ++s.sp;
        }
        const uint4* np = nptr + 5ull * child;
        const uint4 w0 = __ldg(np + 0), w1 = __ldg(np + 1), w2 = __ldg(np + 2), w3 = __ldg(np + 3), w4 = __ldg(np + 4);
        if (COUNT) cnt.nodes++;
        const uint32_t hm = intersect_children(r, w0, w1, w2, w3, w4, s.best_t);
        s.group = make_uint2(w1.x, (hm & 0xFF000000u) | (w0.w >> 24));
        tgroup = make_uint2(w1.y, hm & 0x00FFFFFFu);
    } else {
        tgroup = s.group;   // a postponed triangle group
        s.group = make_uint2(0u, 0u);
    }
    while (tgroup.y) {
        if constexpr (kPost) {
            if (s.sp < kTotalStack) {
                const uint32_t with_tris = (uint32_t)__popc(__activemask());
                if (with_tris * 32u < traversing * (uint32_t)kPostpone) {
                    if (s.sp < SS) stack[s.sp * stride] = tgroup;
                    else spill[s.sp - SS] = tgroup;
                    ++s.sp;
                    break;
                }
            }
        }
        const int k = __ffs(tgroup.y) - 1;
        tgroup.y &= tgroup.y - 1u;
        const float4* tp = tptr + 3ull * (tgroup.x + (uint32_t)k);
        const float4 a = __ldg(tp + 0), b = __ldg(tp + 1), c = __ldg(tp + 2);
        if (COUNT) cnt.tris++;
        float t, u, v;
        if (intersect_triangle(r, a, b, c, s.best_t, t, u, v)) {
            const uint32_t prim = __float_as_uint(a.w);
            if (ANY) {
                hit.prim = prim; hit.t = t; hit.u = u; hit.v = v;
                s.best_rec = tgroup.x + (uint32_t)k;
                return true;
            }
            if (t < s.best_t || prim < hit.prim) {   // t <= best_t holds; equal t: lower id wins
                s.best_t = t;
                hit.prim = prim; hit.t = t; hit.u = u; hit.v = v;
                s.best_rec = tgroup.x + (uint32_t)k;
            }
        }
    }
    if (s.group.y <= 0x00FFFFFFu) {
        if (s.sp == 0) return true;
        --s.sp;
        s.group = s.sp < SS ? stack[s.sp * stride] : spill[s.sp - SS];
    }
    return false;
}

// After the last step: a miss reports t = tmax; a hit gets its reported t, u, v refined (refine_hit).
template <bool REFINE>
__device__ __forceinline__ void trav_finish(const Bvh8Node* __restrict__ nodes, const TriRecord* __restrict__ tris,
                                            const TraceRay& r, const TravState& s, Hit& hit) {
    (void)nodes;
    if (hit.prim == kMiss) {
        hit.t = r.tmax;
    } else if (REFINE) {
        const float4* tp = reinterpret_cast<const float4*>(tris) + 3ull * s.best_rec;
        refine_hit(r, __ldg(tp + 0), __ldg(tp + 1), __ldg(tp + 2), hit);
    }
}

// Traverses the BVH8 for one ray to completion.  `stack` points at this thread's first shared-memory
// stack entry; consecutive entries are `stride` elements apart.  Returns an error code (0 = ok).
template <bool ANY, bool COUNT, bool REFINE = true, int SS = kSmemStack>
__device__ __forceinline__ uint32_t traverse(const Bvh8Node* __restrict__ nodes, const TriRecord* __restrict__ tris,
                                             const TraceRay& r, uint2* stack, int stride, Hit& hit,
                                             TraceCounters& cnt) {
    TravState s;
    trav_init(r, s, hit);
    uint2 spill[kTotalStack - SS];
    uint32_t err = 0;
    while (!trav_step<ANY, COUNT, SS>(nodes, tris, r, s, hit, stack, stride, spill, cnt, err)) {
    }
    trav_finish<REFINE>(nodes, tris, r, s, hit);
    return err;
}

// ------------------------------------------------------------------------------------------------
// Two-level scenes: a top-level BVH8 over instances (leaf entries index DeviceScene::tlas_refs, which
// holds instance ids) and one bottom-level BVH8 per model in object space, in the same node and triangle
// arrays.  A ray enters an instance through the instance's world-to-object matrix; t is the same in both
// spaces (the direction is transformed, not normalized), so the closest distance found so far culls
// boxes at both levels.  The stack entry (kLevelMarker, 0) separates an instance's bottom-level entries
// from the top-level entries below it; popping it returns to the world-space ray.

constexpr uint32_t kLevelMarker = 0xFFFFFFFFu;

// The world ray in an instance's model space: origin and direction through the 3x4 matrix with
// explicitly rounded products and sums in a fixed order (the host restatement evaluates the same), and
// the traversal constants of the new ray.
__device__ __forceinline__ TraceRay instance_ray(const TraceRay& w, const InstanceTrav* __restrict__ it) {
    const float4* q = reinterpret_cast<const float4*>(it);
    const float4 m0 = __ldg(q), m1 = __ldg(q + 1), m2 = __ldg(q + 2);
    auto row = [](float4 m, float x, float y, float z) {
        return __fadd_rn(__fadd_rn(__fmul_rn(m.x, x), __fmul_rn(m.y, y)), __fmul_rn(m.z, z));
    };
    return make_trace_ray(__fadd_rn(row(m0, w.ox, w.oy, w.oz), m0.w), __fadd_rn(row(m1, w.ox, w.oy, w.oz), m1.w),
                          __fadd_rn(row(m2, w.ox, w.oy, w.oz), m2.w), row(m0, w.dx, w.dy, w.dz),
                          row(m1, w.dx, w.dy, w.dz), row(m2, w.dx, w.dy, w.dz), w.tmin, w.tmax);
}

// Closest / any hit through both levels; hit ids are global (instance's first triangle + the record's
// triangle index within the model).  Ties in t go to the lower global id, as in the flat traversal.
// Triangles are tested as soon as they are reached (no postponing).
template <bool ANY, bool COUNT, bool REFINE = true, int SS = kSmemStack>
__device__ __forceinline__ uint32_t traverse_two_level(const DeviceScene& sc, const TraceRay& wr, uint2* stack, int stride,
                                                       Hit& hit, TraceCounters& cnt) {
    const uint4* nptr = reinterpret_cast<const uint4*>(sc.nodes);
    const float4* tptr = reinterpret_cast<const float4*>(sc.tris);
    uint2 spill[kTotalStack - SS];
    uint32_t err = 0, steps = 0;
    TraceRay r = wr;
    bool in_blas = false;
    uint32_t cur_first = 0, cur_inst = 0, best_inst = 0, best_rec = 0;
    float best_t = wr.tmax;
    hit.prim = kMiss;
    hit.t = wr.tmax;
    hit.u = 0.0f;
    hit.v = 0.0f;
    uint2 group = make_uint2(0u, 0x80000000u);
    int sp = 0;
    auto push = [&](uint2 g) {
        if (sp < SS) stack[sp * stride] = g;
        else if (sp < kTotalStack) spill[sp - SS] = g;
        else { err |= kErrStackOverflow; return false; }
        ++sp;
        return true;
    };
    auto pop = [&]() {
        --sp;
        return sp < SS ? stack[sp * stride] : spill[sp - SS];
    };
    for (;;) {
        if (++steps > kMaxTraversalSteps) { err |= kErrStepLimit; break; }
        uint2 tgroup;
        if (group.y > 0x00FFFFFFu) {
            const uint32_t slot_bit = 31u - __clz(group.y);
            const uint32_t slot = (slot_bit - 24u) ^ r.oct_inv;
            const uint32_t child = group.x + __popc(group.y & ((1u << slot) - 1u));
            group.y &= ~(1u << slot_bit);
            if (group.y > 0x00FFFFFFu && !push(group)) break;
            const uint4* np = nptr + 5ull * child;
            const uint4 w0 = __ldg(np + 0), w1 = __ldg(np + 1), w2 = __ldg(np + 2), w3 = __ldg(np + 3), w4 = __ldg(np + 4);
            if (COUNT) cnt.nodes++;
            const uint32_t hm = intersect_children(r, w0, w1, w2, w3, w4, best_t);
            group = make_uint2(w1.x, (hm & 0xFF000000u) | (w0.w >> 24));
            tgroup = make_uint2(w1.y, hm & 0x00FFFFFFu);
        } else {
            tgroup = group;   // a pending leaf group
            group = make_uint2(0u, 0u);
        }
        if (!in_blas) {
            if (tgroup.y) {   // enter the nearest pending instance; the rest of the top level waits below a marker
                const int k = __ffs(tgroup.y) - 1;
                tgroup.y &= tgroup.y - 1u;
                if (group.y > 0x00FFFFFFu && !push(group)) break;
                if (tgroup.y && !push(tgroup)) break;
                group = make_uint2(0u, 0u);
                const uint32_t ii = __ldg(sc.tlas_refs + tgroup.x + (uint32_t)k);
                const uint4 tail = __ldg(reinterpret_cast<const uint4*>(sc.inst_trav + ii) + 3);
                if (tail.x != 0xFFFFFFFFu) {   // a model without triangles has no bottom level
                    if (!push(make_uint2(kLevelMarker, 0u))) break;
                    r = instance_ray(wr, sc.inst_trav + ii);
                    in_blas = true;
                    cur_inst = ii;
                    cur_first = tail.y;
                    group = make_uint2(tail.x, 0x80000000u);
                    continue;
                }
            }
        } else {
            bool done = false;
            while (tgroup.y) {
                const int k = __ffs(tgroup.y) - 1;
                tgroup.y &= tgroup.y - 1u;
                const float4* tp = tptr + 3ull * (tgroup.x + (uint32_t)k);
                const float4 a = __ldg(tp + 0), b = __ldg(tp + 1), c = __ldg(tp + 2);
                if (COUNT) cnt.tris++;
                float t, u, v;
                if (intersect_triangle(r, a, b, c, best_t, t, u, v)) {
                    const uint32_t prim = cur_first + __float_as_uint(a.w);
                    if (ANY || t < best_t || prim < hit.prim) {   // t <= best_t holds; equal t: lower id wins
                        best_t = t;
                        hit.prim = prim; hit.t = t; hit.u = u; hit.v = v;
                        best_rec = tgroup.x + (uint32_t)k;
                        best_inst = cur_inst;
                        if (ANY) { done = true; break; }
                    }
                }
            }
            if (done) break;
        }
        if (group.y <= 0x00FFFFFFu) {
            if (sp == 0) break;
            group = pop();
            if (group.x == kLevelMarker && group.y == 0u) {   // back to the top level
                r = wr;
                in_blas = false;
                if (sp == 0) break;
                group = pop();
            }
        }
    }
    if (hit.prim == kMiss) {
        hit.t = wr.tmax;
    } else if (REFINE) {
        const TraceRay ri = instance_ray(wr, sc.inst_trav + best_inst);
        const float4* tp = tptr + 3ull * best_rec;
        refine_hit(ri, __ldg(tp + 0), __ldg(tp + 1), __ldg(tp + 2), hit);
    }
    return err;
}

// Either traversal, by the scene's structure.  Kernels instantiated with TWO = false handle flat scenes
// only (the two-level path costs registers: the world ray is kept while inside an instance); the
// launchers pick TWO = true when a scene of the launch is two-level.
template <bool ANY, bool COUNT, bool REFINE = true, int SS = kSmemStack, bool TWO = false>
__device__ __forceinline__ uint32_t trace_scene(const DeviceScene& sc, const TraceRay& r, uint2* stack, int stride, Hit& hit,
                                                TraceCounters& cnt) {
    if constexpr (TWO) {
        if (sc.inst_trav) return traverse_two_level<ANY, COUNT, REFINE, SS>(sc, r, stack, stride, hit, cnt);
    }
    return traverse<ANY, COUNT, REFINE, SS>(sc.nodes, sc.tris, r, stack, stride, hit, cnt);
}

}  // namespace rt
