// Arithmetic of the BVH build shared by the host builder (bvh_build.cpp) and the device builder
// (bvh_gpu.cu): binned-SAH costs, the collapse's dynamic programme, the octant slot assignment and the
// child-box quantization.  Every float and double operation is explicitly rounded (never contracted into
// an FMA) and evaluated in one fixed order, so that both builders take the same decisions and write the
// same bytes.  Host code is compiled with -ffp-contract=off; device code uses the _rn intrinsics.
#pragma once

#include <stdint.h>
#include <math.h>

#include "rt_common.h"

namespace rt {
namespace sah {

RT_HD float mul(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
RT_HD float add(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
RT_HD float sub(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}
RT_HD float div(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fdiv_rn(a, b);
#else
    return a / b;
#endif
}
RT_HD float u2f(uint32_t n) {
#ifdef __CUDA_ARCH__
    return __uint2float_rn(n);
#else
    return (float)n;
#endif
}
RT_HD double dadd(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
}
RT_HD double dsub(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dsub_rn(a, b);
#else
    return a - b;
#endif
}
RT_HD double ddiv(double a, double b) {
#ifdef __CUDA_ARCH__
    return __ddiv_rn(a, b);
#else
    return a / b;
#endif
}

RT_HD float pos(float x) { return x > 0.0f ? x : 0.0f; }

// Half the surface area of a box (0 for an empty or inverted box).
RT_HD float half_area(const float lo[3], const float hi[3]) {
    const float d0 = pos(sub(hi[0], lo[0])), d1 = pos(sub(hi[1], lo[1])), d2 = pos(sub(hi[2], lo[2]));
    return add(add(mul(d0, d1), mul(d1, d2)), mul(d2, d0));
}

RT_HD float centroid(float lo, float hi) { return mul(0.5f, add(lo, hi)); }

// Centroid key of the object-median split: -0 and +0 compare equal, so both map to +0.
RT_HD float median_key(float c) { return add(c, 0.0f); }

// Binning frame of one axis over the centroid bounds [lo, hi]: false when the axis cannot be binned
// (no extent, or an extent so small that bins / extent overflows).
RT_HD bool bin_scale(float lo, float hi, int bins, float& scale) {
    const float ext = sub(hi, lo);
    if (!(ext > 0.0f)) return false;
    scale = div((float)bins, ext);
    return isfinite(scale);
}

RT_HD int bin_of(float c, float lo, float scale, int bins) {
    const float f = mul(sub(c, lo), scale);
    if (!(f > 0.0f)) return 0;
    if (f >= (float)(bins - 1)) return bins - 1;
    return (int)f;
}

// SAH cost of splitting a node of half area `parent` into (area_l, n_l) and (area_r, n_r):
// 1 + (A_L n_L + A_R n_R) / A.
RT_HD float split_cost(float area_l, uint32_t n_l, float area_r, uint32_t n_r, float parent) {
    return add(1.0f, div(add(mul(area_l, u2f(n_l)), mul(area_r, u2f(n_r))), parent));
}

// Past this depth of the binary build every split is an object median (bounds the tree depth).
constexpr int kForceMedianDepth = 48;

// SAH costs of the collapse: one node test = 1, one triangle test = 1 (Ylitie et al. use 0.3; on the
// 1.3M-triangle ray cast 0.6-1.2 measured 2 % faster than 0.3, as fewer 3-triangle leaves are merged).
#ifndef RT_COST_TRI
#define RT_COST_TRI 1.0f
#endif
constexpr float kCostNode = 1.0f, kCostTri = RT_COST_TRI;
constexpr uint32_t kLeafMax = 3;   // triangles per leaf child (3 bits of the node's meta byte)

// Dynamic-programme table of one binary node (Ylitie, Karras and Laine, HPG 2017, section 3.1):
// cost[i] = cost of the subtree as at most i + 1 wide children; how[i] = 0 one leaf child, 1 one wide
// node, 2 split between the two binary children with left[i] slots on the left and used[i] slots in all.
struct Dp {
    float cost[8];
    uint8_t how[8], left[8], used[8];
};

RT_HD void dp_leaf(Dp& d, float area, uint32_t count) {
    const float c = mul(mul(area, u2f(count)), kCostTri);
    for (int i = 0; i < 8; ++i) {
        d.cost[i] = c;
        d.how[i] = 0;
        d.left[i] = 0;
        d.used[i] = 1;
    }
}

RT_HD void dp_inner(Dp& d, const Dp& L, const Dp& R, float area, uint32_t count) {
    float dist[9];
    uint8_t dist_k[9];
    for (int j = 2; j <= 8; ++j) {
        dist[j] = INFINITY;
        dist_k[j] = 1;
        for (int k = 1; k < j; ++k) {
            const float c = add(L.cost[k - 1], R.cost[j - k - 1]);
            if (c < dist[j]) { dist[j] = c; dist_k[j] = (uint8_t)k; }
        }
    }
    const float leaf = count <= kLeafMax ? mul(mul(area, u2f(count)), kCostTri) : INFINITY;
    const float inner = add(dist[8], mul(area, kCostNode));
    const bool as_leaf = count <= kLeafMax && leaf <= inner;
    d.cost[0] = as_leaf ? leaf : inner;
    d.how[0] = as_leaf ? 0 : 1;
    d.left[0] = 0;
    d.used[0] = 1;
    for (int i = 2; i <= 8; ++i) {
        if (dist[i] < d.cost[i - 2]) {
            d.cost[i - 1] = dist[i];
            d.how[i - 1] = 2;
            d.left[i - 1] = dist_k[i];
            d.used[i - 1] = (uint8_t)i;
        } else {
            d.cost[i - 1] = d.cost[i - 2];
            d.how[i - 1] = d.how[i - 2];
            d.left[i - 1] = d.left[i - 2];
            d.used[i - 1] = d.used[i - 2];
        }
    }
}

// Slots given to the left binary child when an internal node spreads its subtree over 8 children.
RT_HD int dp_root_split(const Dp& L, const Dp& R) {
    int best_k = 1;
    float best = INFINITY;
    for (int k = 1; k < 8; ++k) {
        const float c = add(L.cost[k - 1], R.cost[8 - k - 1]);
        if (c < best) { best = c; best_k = k; }
    }
    return best_k;
}

// Octant slot assignment of `nch` children (boxes lo/hi): repeatedly the (child, free slot) pair of
// largest dot(child centroid - union centre, slot direction) over the still unassigned children, where
// bit k of the slot selects the positive direction of axis k; ties go to the lower child, then the lower
// slot.  child_in_slot[s] = child or -1.  The unassigned children and free slots are bit masks.
RT_HD void assign_slots(int nch, const float (*lo)[3], const float (*hi)[3], int child_in_slot[8]) {
    float ulo[3] = {INFINITY, INFINITY, INFINITY}, uhi[3] = {-INFINITY, -INFINITY, -INFINITY};
    float c[8][3];
    for (int i = 0; i < nch; ++i)
        for (int k = 0; k < 3; ++k) {
            ulo[k] = lo[i][k] < ulo[k] ? lo[i][k] : ulo[k];
            uhi[k] = hi[i][k] > uhi[k] ? hi[i][k] : uhi[k];
        }
    float centre[3];
    for (int k = 0; k < 3; ++k) centre[k] = centroid(ulo[k], uhi[k]);
    for (int i = 0; i < nch; ++i)
        for (int k = 0; k < 3; ++k) c[i][k] = sub(centroid(lo[i][k], hi[i][k]), centre[k]);
    int result[8] = {-1, -1, -1, -1, -1, -1, -1, -1};
    uint32_t unassigned = nch >= 8 ? 0xFFu : ((1u << nch) - 1u), free_slots = 0xFFu;
    while (unassigned) {
        float best = -INFINITY;
        int bc = -1, bs = -1;
        for (int i = 0; i < 8; ++i) {
            if (!((unassigned >> i) & 1u)) continue;
            for (int s = 0; s < 8; ++s) {
                if (!((free_slots >> s) & 1u)) continue;
                const float score = add(add((s & 1) ? c[i][0] : -c[i][0], (s & 2) ? c[i][1] : -c[i][1]),
                                        (s & 4) ? c[i][2] : -c[i][2]);
                if (score > best) { best = score; bc = i; bs = s; }
            }
        }
        if (bc < 0) {   // non-finite scores: first free slot for the first unassigned child
            for (int i = 7; i >= 0; --i)
                if ((unassigned >> i) & 1u) bc = i;
            for (int s = 7; s >= 0; --s)
                if ((free_slots >> s) & 1u) bs = s;
        }
        unassigned &= ~(1u << bc);
        free_slots &= ~(1u << bs);
        result[bs] = bc;
    }
    for (int s = 0; s < 8; ++s) child_in_slot[s] = result[s];
}

// Largest quantization exponent of a node (scale 2^e): the traversal forms 2^(e+15) in single precision.
constexpr int kMaxQuantExponent = 110;

// Quantization frame of one axis of a node whose children's union is [ulo, uhi]: origin p and scale 2^e
// with 255 * 2^e >= extent + 2 delta + 2 slack, where slack = 2^-7 quanta.  The slack keeps every child's
// quantized box at least 2^-8 quanta outside its (delta-dilated) bounds without clamping at 0 or 255,
// which covers the extra rounding of the traversal's plane offsets (at most 2^-9 quanta).  False when
// the exponent exceeds kMaxQuantExponent.
RT_HD bool quant_axis(float ulo, float uhi, double delta, float& p, int& e) {
    const double lo = dsub((double)ulo, delta);
    const double hi = dadd((double)uhi, delta);
    e = 0;
    frexp(ddiv(dsub(hi, lo), 255.0), &e);
    if (e < -126) e = -126;
    for (;;) {
        if (e > kMaxQuantExponent) return false;
        const double slack = ldexp(1.0, e - 7);
        const double target = dsub(lo, slack);
        float pf = (float)target;
        if ((double)pf > target) pf = nextafterf(pf, -INFINITY);
        if (ldexp(255.0, e) >= dsub(dadd(hi, slack), (double)pf)) {
            p = pf;
            return true;
        }
        ++e;
    }
}

// Conservative 8-bit bounds of [lo, hi] (dilated by delta) in the frame (p, scale).
RT_HD void quant_child(float lo, float hi, double delta, float p, double scale, uint8_t& qlo, uint8_t& qhi) {
    double a = floor(dsub(ddiv(dsub(dsub((double)lo, delta), (double)p), scale), 0.00390625));
    double b = ceil(dadd(ddiv(dsub(dadd((double)hi, delta), (double)p), scale), 0.00390625));
    a = a < 0.0 ? 0.0 : (a > 255.0 ? 255.0 : a);
    b = b < 0.0 ? 0.0 : (b > 255.0 ? 255.0 : b);
    qlo = (uint8_t)a;
    qhi = (uint8_t)b;
}

// Dilation of quantized boxes: 2^-18 of the scene's coordinate magnitude, which covers the float
// rounding of the slab test for ray origins within ~20x that magnitude.
RT_HD double quant_delta(float mag) { return ldexp((double)mag < 1e-20 ? 1e-20 : (double)mag, -18); }

}  // namespace sah
}  // namespace rt
