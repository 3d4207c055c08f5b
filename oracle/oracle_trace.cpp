// ORACLE — test infrastructure only (see oracle_common.h).
//
// CPU ray casting: the watertight ray/triangle test of Woop, Benthin and Wald (JCGT 2013) templated on
// float/double, a brute-force closest/any hit over all triangles, and an independent binary SAH BVH
// with a conservative slab test.  Restates the traversal semantics of traceRayEXT as the reference
// uses it: closest hit with tmin 0 / tmax 1e4 (shaders/raytrace/raytrace.rgen.glsl:159-171) and the
// terminate-on-first-hit shadow query (shaders/raytrace/nee.h.glsl:126-144).  Ties in t are broken
// towards the lower triangle id so that the closest hit does not depend on traversal order.
//
// In float mode every operation is a single IEEE binary32 operation in a fixed order (this file must be
// compiled with -ffp-contract=off), so its hits are bit-identical to any other IEEE evaluation of the
// same expressions.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <limits>
#include <memory>
#include <thread>
#include <vector>

#include "oracle_common.h"

namespace oracle {

template <class T>
struct PreRay {
    Vec3<T> o, d;
    T tmin, tmax;
    int kx, ky, kz;
    T sx, sy, sz;
};

template <class T>
PreRay<T> precompute(const RayRec& r) {
    PreRay<T> p;
    p.o = Vec3<T>((T)r.ox, (T)r.oy, (T)r.oz);
    p.d = Vec3<T>((T)r.dx, (T)r.dy, (T)r.dz);
    p.tmin = (T)r.tmin;
    p.tmax = (T)r.tmax;
    const T ax = std::fabs(p.d.x), ay = std::fabs(p.d.y), az = std::fabs(p.d.z);
    int kz;
    if (ax >= ay) kz = (ax >= az) ? 0 : 2;
    else kz = (ay >= az) ? 1 : 2;
    int kx = (kz + 1) % 3, ky = (kx + 1) % 3;
    if (p.d[kz] < (T)0) std::swap(kx, ky);
    p.kx = kx; p.ky = ky; p.kz = kz;
    p.sx = p.d[kx] / p.d[kz];
    p.sy = p.d[ky] / p.d[kz];
    p.sz = (T)1 / p.d[kz];
    return p;
}

// Returns true on a hit with t in [tmin, tmax_now]; u weights vertex 1, v weights vertex 2.
template <class T>
bool watertight(const PreRay<T>& r, const float* tri, T tmax_now, T& t_out, T& u_out, T& v_out) {
    const Vec3<T> A = Vec3<T>((T)tri[0], (T)tri[1], (T)tri[2]) - r.o;
    const Vec3<T> B = Vec3<T>((T)tri[3], (T)tri[4], (T)tri[5]) - r.o;
    const Vec3<T> C = Vec3<T>((T)tri[6], (T)tri[7], (T)tri[8]) - r.o;
    const T Ax = A[r.kx] - r.sx * A[r.kz];
    const T Ay = A[r.ky] - r.sy * A[r.kz];
    const T Bx = B[r.kx] - r.sx * B[r.kz];
    const T By = B[r.ky] - r.sy * B[r.kz];
    const T Cx = C[r.kx] - r.sx * C[r.kz];
    const T Cy = C[r.ky] - r.sy * C[r.kz];
    T U = Cx * By - Cy * Bx;
    T V = Ax * Cy - Ay * Cx;
    T W = Bx * Ay - By * Ax;
    if (sizeof(T) == sizeof(float) && (U == (T)0 || V == (T)0 || W == (T)0)) {
        const double CxBy = (double)Cx * (double)By, CyBx = (double)Cy * (double)Bx;
        const double AxCy = (double)Ax * (double)Cy, AyCx = (double)Ay * (double)Cx;
        const double BxAy = (double)Bx * (double)Ay, ByAx = (double)By * (double)Ax;
        U = (T)(float)(CxBy - CyBx);
        V = (T)(float)(AxCy - AyCx);
        W = (T)(float)(BxAy - ByAx);
    }
    if ((U < (T)0 || V < (T)0 || W < (T)0) && (U > (T)0 || V > (T)0 || W > (T)0)) return false;
    const T det = (U + V) + W;
    if (det == (T)0) return false;
    const T Az = r.sz * A[r.kz], Bz = r.sz * B[r.kz], Cz = r.sz * C[r.kz];
    const T Tn = (U * Az + V * Bz) + W * Cz;
    const T rcp = (T)1 / det;
    const T t = Tn * rcp;
    if (!(t >= r.tmin && t <= tmax_now)) return false;
    t_out = t;
    u_out = V * rcp;
    v_out = W * rcp;
    return true;
}

// The reported t, u, v of a float-mode hit: the same watertight expressions evaluated in double for the
// selected triangle (no range or sign checks) and rounded to float.  Ray-cast APIs report these values;
// the float test above only decides which triangle is hit.
// Re-evaluation of the selected triangle from an origin moved along the ray onto the hit point.  The
// moved origin o + t0 d (t0 from the watertight test) is formed exactly as hi + lo with FMA-based
// TwoProduct and TwoSum (error-free transforms, Ogita/Rump/Oishi 2005), so the vertex offsets
// s = o' - v0 are small and accurate; a Möller–Trumbore evaluation there gives barycentrics without the
// cancellation that a far origin causes, and t = t0 + t'.  Every step is one IEEE binary32 operation
// (std::fma is correctly rounded), so the GPU's evaluation of the same sequence gives the same bits.
inline void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}
inline void two_prod(float a, float b, float& p, float& e) {
    p = a * b;
    e = std::fma(a, b, -p);
}

// a*b - c*d with one rounding error (Kahan's FMA algorithm).
inline float diff_prod(float a, float b, float c, float d) {
    const float w = c * d;
    const float e = std::fma(-c, d, w);
    const float f = std::fma(a, b, -w);
    return f + e;
}
// Compensated dot product Dot2 (Ogita, Rump, Oishi): as if computed in twice the working precision.
inline float dot2(const float x[3], const float y[3]) {
    float p, s;
    two_prod(x[0], y[0], p, s);
    for (int i = 1; i < 3; ++i) {
        float h, r, q;
        two_prod(x[i], y[i], h, r);
        two_sum(p, h, p, q);
        s = s + (q + r);
    }
    return p + s;
}

inline void refine64(const RayRec& ray, const float* tri, float& t, float& u, float& v) {
    const float o[3] = {ray.ox, ray.oy, ray.oz}, d[3] = {ray.dx, ray.dy, ray.dz};
    const float t0 = t;
    float s[3], e1[3], e2[3];
    for (int k = 0; k < 3; ++k) {
        float ph, pl, sh, sl;
        two_prod(t0, d[k], ph, pl);
        two_sum(o[k], ph, sh, sl);
        const float lo = sl + pl;
        s[k] = (sh - tri[k]) + lo;          // o' - v0
        e1[k] = tri[3 + k] - tri[k];
        e2[k] = tri[6 + k] - tri[k];
    }
    const float p[3] = {diff_prod(d[1], e2[2], d[2], e2[1]), diff_prod(d[2], e2[0], d[0], e2[2]),
                        diff_prod(d[0], e2[1], d[1], e2[0])};
    const float det = dot2(e1, p);
    if (det == 0.0f) return;
    const float q[3] = {diff_prod(s[1], e1[2], s[2], e1[1]), diff_prod(s[2], e1[0], s[0], e1[2]),
                        diff_prod(s[0], e1[1], s[1], e1[0])};
    u = dot2(s, p) / det;
    v = dot2(d, q) / det;
    t = t0 + dot2(e2, q) / det;
}

template <class T>
struct BestHit {
    uint32_t prim = kMiss;
    T t, u = 0, v = 0;
};

template <class T>
inline void consider(const PreRay<T>& r, const float* tris9, uint32_t id, bool any, BestHit<T>& best, bool& done) {
    T t, u, v;
    if (!watertight(r, tris9 + 9ull * id, best.t, t, u, v)) return;
    if (any) {
        best.prim = id; best.t = t; best.u = u; best.v = v;
        done = true;
        return;
    }
    if (t < best.t || id < best.prim) {
        best.prim = id; best.t = t; best.u = u; best.v = v;
    }
}

// ---------------------------------------------------------------------------------------------------
// Independent binary BVH (binned SAH over the largest centroid axis, leaves of up to 4 triangles).
struct BNode {
    float lo[3], hi[3];
    uint32_t left_or_first;
    uint32_t count;        // 0 = internal (children left_or_first, left_or_first + 1)
};

struct Bvh {
    std::vector<BNode> nodes;
    std::vector<uint32_t> order;
    std::vector<float> tris;   // 9 per triangle, original ids
};

static void build_node(Bvh& b, const std::vector<float>& cen, uint32_t node, uint32_t first, uint32_t count) {
    BNode& n = b.nodes[node];
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t i = first; i < first + count; ++i) {
        const uint32_t p = b.order[i];
        for (int j = 0; j < 3; ++j)
            for (int k = 0; k < 3; ++k) {
                lo[k] = std::min(lo[k], b.tris[9ull * p + 3 * j + k]);
                hi[k] = std::max(hi[k], b.tris[9ull * p + 3 * j + k]);
            }
        for (int k = 0; k < 3; ++k) {
            clo[k] = std::min(clo[k], cen[3ull * p + k]);
            chi[k] = std::max(chi[k], cen[3ull * p + k]);
        }
    }
    for (int k = 0; k < 3; ++k) { n.lo[k] = lo[k]; n.hi[k] = hi[k]; }
    if (count <= 4) { n.left_or_first = first; n.count = count; return; }
    int axis = 0;
    for (int k = 1; k < 3; ++k)
        if (chi[k] - clo[k] > chi[axis] - clo[axis]) axis = k;
    uint32_t mid = first + count / 2;
    const float ext = chi[axis] - clo[axis];
    if (ext > 0.0f) {
        constexpr int NB = 12;
        float blo[NB][3], bhi[NB][3];
        uint32_t bc[NB] = {0};
        for (int i = 0; i < NB; ++i)
            for (int k = 0; k < 3; ++k) { blo[i][k] = INFINITY; bhi[i][k] = -INFINITY; }
        auto bin_of = [&](uint32_t p) { return std::min(NB - 1, (int)((cen[3ull * p + axis] - clo[axis]) * (NB / ext))); };
        for (uint32_t i = first; i < first + count; ++i) {
            const uint32_t p = b.order[i];
            const int bi = bin_of(p);
            bc[bi]++;
            for (int j = 0; j < 3; ++j)
                for (int k = 0; k < 3; ++k) {
                    blo[bi][k] = std::min(blo[bi][k], b.tris[9ull * p + 3 * j + k]);
                    bhi[bi][k] = std::max(bhi[bi][k], b.tris[9ull * p + 3 * j + k]);
                }
        }
        auto area = [](const float* l, const float* h) {
            const double dx = std::max(0.0f, h[0] - l[0]), dy = std::max(0.0f, h[1] - l[1]), dz = std::max(0.0f, h[2] - l[2]);
            return dx * dy + dy * dz + dz * dx;
        };
        double best = INFINITY;
        int best_split = -1;
        for (int s = 1; s < NB; ++s) {
            float l0[3] = {INFINITY, INFINITY, INFINITY}, h0[3] = {-INFINITY, -INFINITY, -INFINITY};
            float l1[3] = {INFINITY, INFINITY, INFINITY}, h1[3] = {-INFINITY, -INFINITY, -INFINITY};
            uint32_t c0 = 0, c1 = 0;
            for (int i = 0; i < NB; ++i) {
                float* L = i < s ? l0 : l1;
                float* H = i < s ? h0 : h1;
                (i < s ? c0 : c1) += bc[i];
                for (int k = 0; k < 3; ++k) { L[k] = std::min(L[k], blo[i][k]); H[k] = std::max(H[k], bhi[i][k]); }
            }
            if (c0 == 0 || c1 == 0) continue;
            const double cost = area(l0, h0) * c0 + area(l1, h1) * c1;
            if (cost < best) { best = cost; best_split = s; }
        }
        if (best_split > 0) {
            auto it = std::partition(b.order.begin() + first, b.order.begin() + first + count,
                                     [&](uint32_t p) { return bin_of(p) < best_split; });
            mid = (uint32_t)(it - b.order.begin());
            if (mid == first || mid == first + count) mid = first + count / 2;
        }
    }
    const uint32_t left = (uint32_t)b.nodes.size();
    b.nodes.push_back(BNode{});
    b.nodes.push_back(BNode{});
    b.nodes[node].left_or_first = left;
    b.nodes[node].count = 0;
    build_node(b, cen, left, first, mid - first);
    build_node(b, cen, left + 1, mid, first + count - mid);
}

static Bvh* build_bvh(const float* tris9, uint64_t n) {
    auto b = std::make_unique<Bvh>();
    b->tris.assign(tris9, tris9 + 9 * n);
    b->order.resize(n);
    std::vector<float> cen(3 * n);
    for (uint64_t i = 0; i < n; ++i) {
        b->order[i] = (uint32_t)i;
        for (int k = 0; k < 3; ++k) {
            float lo = std::min(std::min(tris9[9 * i + k], tris9[9 * i + 3 + k]), tris9[9 * i + 6 + k]);
            float hi = std::max(std::max(tris9[9 * i + k], tris9[9 * i + 3 + k]), tris9[9 * i + 6 + k]);
            cen[3 * i + k] = 0.5f * (lo + hi);
        }
    }
    b->nodes.reserve(2 * n + 1);
    b->nodes.push_back(BNode{});
    if (n > 0) build_node(*b, cen, 0, 0, (uint32_t)n);
    return b.release();
}

// Slab test with generous slack so that it never culls a box containing a hit the triangle test
// accepts (the entry distance is lowered and the exit distance raised by a relative 1e-5).
template <class T>
inline bool box_hit(const PreRay<T>& r, const BNode& n, T tmax_now, T& tnear) {
    T t0 = r.tmin, t1 = tmax_now;
    for (int k = 0; k < 3; ++k) {
        const T o = r.o[k], d = r.d[k];
        const T lo = (T)n.lo[k], hi = (T)n.hi[k];
        if (d == (T)0) {
            if (o < lo || o > hi) return false;
            continue;
        }
        T a = (lo - o) / d, b = (hi - o) / d;
        if (a > b) std::swap(a, b);
        a = a - std::fabs(a) * (T)1e-5 - (T)1e-30;
        b = b + std::fabs(b) * (T)1e-5 + (T)1e-30;
        t0 = std::max(t0, a);
        t1 = std::min(t1, b);
        if (t0 > t1) return false;
    }
    tnear = t0;
    return true;
}

template <class T>
BestHit<T> trace_bvh(const Bvh& b, const RayRec& ray, bool any, uint64_t* nodes_visited) {
    const PreRay<T> r = precompute<T>(ray);
    BestHit<T> best;
    best.t = r.tmax;
    if (b.tris.empty()) return best;
    uint32_t stack[128];
    int sp = 0;
    stack[sp++] = 0;
    bool done = false;
    while (sp > 0 && !done) {
        const BNode& n = b.nodes[stack[--sp]];
        T tn;
        if (nodes_visited) (*nodes_visited)++;
        if (!box_hit(r, n, best.t + std::fabs(best.t) * (T)1e-5, tn)) continue;
        if (n.count > 0) {
            for (uint32_t i = 0; i < n.count && !done; ++i) consider(r, b.tris.data(), b.order[n.left_or_first + i], any, best, done);
            continue;
        }
        // push far child first (by the sign of the ray direction on the node's largest axis)
        const BNode& l = b.nodes[n.left_or_first];
        const BNode& rr = b.nodes[n.left_or_first + 1];
        int axis = 0;
        float best_ext = -1.0f;
        for (int k = 0; k < 3; ++k) {
            const float e = n.hi[k] - n.lo[k];
            if (e > best_ext) { best_ext = e; axis = k; }
        }
        const bool left_first = (l.lo[axis] + l.hi[axis]) <= (rr.lo[axis] + rr.hi[axis]) ? (r.d[axis] >= (T)0) : (r.d[axis] < (T)0);
        if (sp + 2 > 128) break;
        if (left_first) { stack[sp++] = n.left_or_first + 1; stack[sp++] = n.left_or_first; }
        else { stack[sp++] = n.left_or_first; stack[sp++] = n.left_or_first + 1; }
    }
    return best;
}

template <class T>
BestHit<T> trace_brute(const float* tris9, uint64_t ntri, const RayRec& ray, bool any) {
    const PreRay<T> r = precompute<T>(ray);
    BestHit<T> best;
    best.t = r.tmax;
    bool done = false;
    for (uint64_t i = 0; i < ntri && !done; ++i) consider(r, tris9, (uint32_t)i, any, best, done);
    return best;
}

inline HitRec finish32(const BestHit<float>& r, const RayRec& ray, const float* tri) {
    HitRec h{r.prim, r.t, r.u, r.v};
    if (tri) refine64(ray, tri, h.t, h.u, h.v);
    return h;
}

// Closest hit as the renderer sees it: float mode reports the refined t/u/v (what the GPU reports).
int trace_closest_f(void* bvh, const RayRec& r, uint32_t& prim, double& t, double& u, double& v, int precision) {
    const Bvh& b = *static_cast<Bvh*>(bvh);
    if (precision == 64) {
        const BestHit<double> h = trace_bvh<double>(b, r, false, nullptr);
        prim = h.prim; t = h.t; u = h.u; v = h.v;
    } else {
        const BestHit<float> h = trace_bvh<float>(b, r, false, nullptr);
        const HitRec f = finish32(h, r, h.prim == kMiss ? nullptr : b.tris.data() + 9ull * h.prim);
        prim = f.prim; t = f.t; u = f.u; v = f.v;
    }
    return prim != kMiss;
}

bool trace_occluded(void* bvh, const RayRec& r, int precision) {
    const Bvh& b = *static_cast<Bvh*>(bvh);
    if (precision == 64) return trace_bvh<double>(b, r, true, nullptr).prim != kMiss;
    return trace_bvh<float>(b, r, true, nullptr).prim != kMiss;
}

template <class F>
static void parallel_for(uint64_t n, int threads, F&& f) {
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    if (threads == 1 || n < 256) { for (uint64_t i = 0; i < n; ++i) f(i); return; }
    std::atomic<uint64_t> next{0};
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t)
        pool.emplace_back([&] {
            for (;;) {
                const uint64_t b = next.fetch_add(256);
                if (b >= n) break;
                const uint64_t e = std::min(n, b + 256);
                for (uint64_t i = b; i < e; ++i) f(i);
            }
        });
    for (auto& th : pool) th.join();
}

// ---------------------------------------------------------------------------------------------------
// Traversal of the product's exported BVH8 (the compressed 8-wide layout of Ylitie, Karras and Laine,
// HPG 2017, as the library's C ABI documents it: 80-byte nodes with a power-of-two quantization frame,
// 8 child slots assigned by octant, meta byte per slot = triangle-count unary code << 5 | bit index,
// internal children at bit indices 24 + slot; 48-byte triangle records v0 | id, v1, v2).  Written
// from that description to count the node visits and triangle tests behind the ray cast's byte
// accounting, and to check on the CPU that the exported tree finds the same hits as the oracle's own
// BVH.  Closest hit visits children nearest-first by octant order and tests a node's triangles as soon
// as it reaches them (no postponing).
struct Bvh8View {
    const uint8_t* nodes;
    uint64_t node_count;
    const float* tris;   // 12 floats per record
};

inline float f32_bits(uint32_t u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

inline uint32_t bvh8_children(const uint8_t* n, const PreRay<float>& r, float idx, float idy, float idz,
                              uint32_t oct_inv, float tmax) {
    float p[3];
    std::memcpy(p, n, 12);
    const float id[3] = {idx, idy, idz};
    const float o[3] = {r.o.x, r.o.y, r.o.z};
    float sc[3], of[3];
    for (int k = 0; k < 3; ++k) {
        sc[k] = f32_bits(((uint32_t)n[12 + k] + 15u) << 23) * id[k];   // 2^(e+15) in t units
        of[k] = std::fma(p[k] - o[k], id[k], -sc[k]);
    }
    const uint8_t* meta = n + 24;
    const uint8_t* qlo[3] = {n + 32, n + 40, n + 48};
    const uint8_t* qhi[3] = {n + 56, n + 64, n + 72};
    uint32_t hitmask = 0;
    for (int i = 0; i < 8; ++i) {
        float tn = r.tmin, tf = tmax;
        for (int k = 0; k < 3; ++k) {
            const uint8_t qn = id[k] < 0.0f ? qhi[k][i] : qlo[k][i];
            const uint8_t qf = id[k] < 0.0f ? qlo[k][i] : qhi[k][i];
            const float a = std::fma(1.0f + (float)qn * (1.0f / 32768.0f), sc[k], of[k]);
            const float b = std::fma(1.0f + (float)qf * (1.0f / 32768.0f), sc[k], of[k]);
            tn = std::fmax(tn, a);
            tf = std::fmin(tf, b);
        }
        if (tn <= tf && meta[i] != 0) {
            uint32_t m = meta[i];
            if ((m & 0x18u) == 0x18u) m ^= oct_inv;   // internal child: bit index 24 + (slot ^ octant)
            hitmask |= (m >> 5) << (m & 31u);
        }
    }
    return hitmask;
}

BestHit<float> trace_bvh8_from(const Bvh8View& b, uint32_t root, const RayRec& ray, bool any, uint64_t& visited,
                               uint64_t& tested) {
    const PreRay<float> r = precompute<float>(ray);
    BestHit<float> best;
    best.t = r.tmax;
    if (b.node_count == 0) return best;
    auto rcp = [](float d) { return std::fabs(d) > 1e-30f ? 1.0f / d : std::copysign(1e30f, d); };
    const float idx = rcp(ray.dx), idy = rcp(ray.dy), idz = rcp(ray.dz);
    const uint32_t oct = (ray.dx < 0.0f ? 1u : 0u) | (ray.dy < 0.0f ? 2u : 0u) | (ray.dz < 0.0f ? 4u : 0u);
    const uint32_t oct_inv = 7u - oct;
    uint32_t gbase = root, gbits = 0x80000000u;   // node group: child base, hit bits 24..31 | internal mask
    std::vector<std::pair<uint32_t, uint32_t>> stack;
    for (;;) {
        uint32_t tbase = 0, tbits = 0;
        if (gbits > 0x00FFFFFFu) {
            const uint32_t slot_bit = 31u - (uint32_t)__builtin_clz(gbits);
            const uint32_t slot = (slot_bit - 24u) ^ oct_inv;
            const uint32_t rel = (uint32_t)__builtin_popcount(gbits & ((1u << slot) - 1u));
            const uint32_t child = gbase + rel;
            gbits &= ~(1u << slot_bit);
            if (gbits > 0x00FFFFFFu) stack.emplace_back(gbase, gbits);
            if (child >= b.node_count) return best;   // malformed tree
            const uint8_t* n = b.nodes + 80ull * child;
            ++visited;
            const uint32_t hm = bvh8_children(n, r, idx, idy, idz, oct_inv, best.t);
            uint32_t cb, tb;
            std::memcpy(&cb, n + 16, 4);
            std::memcpy(&tb, n + 20, 4);
            gbase = cb;
            gbits = (hm & 0xFF000000u) | n[15];
            tbase = tb;
            tbits = hm & 0x00FFFFFFu;
        }
        while (tbits) {
            const int k = __builtin_ctz(tbits);
            tbits &= tbits - 1u;
            const float* rec = b.tris + 12ull * (tbase + (uint32_t)k);
            const float tri[9] = {rec[0], rec[1], rec[2], rec[4], rec[5], rec[6], rec[8], rec[9], rec[10]};
            uint32_t id;
            std::memcpy(&id, rec + 3, 4);
            ++tested;
            float t, u, v;
            if (!watertight(r, tri, best.t, t, u, v)) continue;
            if (any) {
                best.prim = id; best.t = t; best.u = u; best.v = v;
                return best;
            }
            if (t < best.t || id < best.prim) {
                best.prim = id; best.t = t; best.u = u; best.v = v;
            }
        }
        if (gbits <= 0x00FFFFFFu) {
            if (stack.empty()) return best;
            gbase = stack.back().first;
            gbits = stack.back().second;
            stack.pop_back();
        }
    }
}

BestHit<float> trace_bvh8(const Bvh8View& b, const RayRec& ray, bool any, uint64_t& visited, uint64_t& tested) {
    return trace_bvh8_from(b, 0u, ray, any, visited, tested);
}

// ---------------------------------------------------------------------------------------------------
// Two-level scenes.  A ray enters an instance through the instance's world-to-object matrix (row-major
// 3x4), evaluated as ((m0 x + m1 y) + m2 z) + m3 per row in IEEE binary32; t is unchanged by the affine
// change of space.  Hit ids are global: the instance's first triangle + the triangle's index in its model.
inline RayRec to_instance(const RayRec& w, const float* m) {
    auto row = [&](int r, float x, float y, float z) { return (m[4 * r] * x + m[4 * r + 1] * y) + m[4 * r + 2] * z; };
    RayRec o;
    o.ox = row(0, w.ox, w.oy, w.oz) + m[3];
    o.oy = row(1, w.ox, w.oy, w.oz) + m[7];
    o.oz = row(2, w.ox, w.oy, w.oz) + m[11];
    o.dx = row(0, w.dx, w.dy, w.dz);
    o.dy = row(1, w.dx, w.dy, w.dz);
    o.dz = row(2, w.dx, w.dy, w.dz);
    o.tmin = w.tmin;
    o.tmax = w.tmax;
    return o;
}

// The oracle's own two-level restatement: per model its binary BVH over object-space triangles; every
// instance is tried (no top level), keeping the closest hit (ties: lower global id) or the first hit.
struct InstancedScene {
    std::vector<std::unique_ptr<Bvh>> models;
    struct Inst {
        uint32_t model;
        float inv[12];
        uint32_t first_prim;
    };
    std::vector<Inst> insts;
};

inline HitRec trace_instanced(const InstancedScene& s, const RayRec& w, bool any) {
    HitRec best{kMiss, w.tmax, 0.0f, 0.0f};
    float best_t = w.tmax;
    uint32_t best_inst = 0;
    BestHit<float> bh;
    for (size_t i = 0; i < s.insts.size(); ++i) {
        const InstancedScene::Inst& in = s.insts[i];
        RayRec r = to_instance(w, in.inv);
        r.tmax = best_t;
        const Bvh& b = *s.models[in.model];
        const BestHit<float> h = trace_bvh<float>(b, r, any, nullptr);
        if (h.prim == kMiss) continue;
        const uint32_t g = in.first_prim + h.prim;
        if (h.t < best_t || g < best.prim) {
            best_t = h.t;
            best = HitRec{g, h.t, h.u, h.v};
            best_inst = (uint32_t)i;
            bh = h;
            if (any) break;
        }
    }
    if (best.prim != kMiss) {   // refined in the instance's space, as the device reports it
        const InstancedScene::Inst& in = s.insts[best_inst];
        const RayRec r = to_instance(w, in.inv);
        const Bvh& b = *s.models[in.model];
        const HitRec f = finish32(bh, r, b.tris.data() + 9ull * (best.prim - in.first_prim));
        best.t = f.t;
        best.u = f.u;
        best.v = f.v;
    }
    return best;
}

// Traversal of an exported two-level BVH8 (the device's layout: top-level root = node 0, its leaf entries
// index `refs` (instance ids); per instance a 64-byte record: world-to-object matrix, bottom-level root
// node, first global triangle).  Counts node visits and triangle tests; unrefined t/u/v.
BestHit<float> trace_bvh8_two_level(const Bvh8View& b, const uint32_t* refs, const uint8_t* inst, const RayRec& wray,
                                    bool any, uint64_t& visited, uint64_t& tested) {
    BestHit<float> best;
    best.t = wray.tmax;
    // the top level with the world ray: gather every instance whose box the ray reaches (in the device's
    // order the culling distance can be smaller; this is conservative), then traverse the instances
    std::vector<uint32_t> pending;
    {
        const PreRay<float> r = precompute<float>(wray);
        auto rcp = [](float d) { return std::fabs(d) > 1e-30f ? 1.0f / d : std::copysign(1e30f, d); };
        const float idx = rcp(wray.dx), idy = rcp(wray.dy), idz = rcp(wray.dz);
        const uint32_t oct = (wray.dx < 0.0f ? 1u : 0u) | (wray.dy < 0.0f ? 2u : 0u) | (wray.dz < 0.0f ? 4u : 0u);
        std::vector<uint32_t> st = {0u};
        while (!st.empty()) {
            const uint32_t ni = st.back();
            st.pop_back();
            const uint8_t* n = b.nodes + 80ull * ni;
            ++visited;
            const uint32_t hm = bvh8_children(n, r, idx, idy, idz, 7u - oct, wray.tmax);
            uint32_t cb, tb;
            std::memcpy(&cb, n + 16, 4);
            std::memcpy(&tb, n + 20, 4);
            for (uint32_t bit = 24; bit < 32; ++bit)
                if (hm >> bit & 1u) {
                    const uint32_t slot = (bit - 24u) ^ (7u - oct);
                    st.push_back(cb + (uint32_t)__builtin_popcount(n[15] & ((1u << slot) - 1u)));
                }
            for (uint32_t bit = 0; bit < 24; ++bit)
                if (hm >> bit & 1u) pending.push_back(refs[tb + bit]);
        }
    }
    std::sort(pending.begin(), pending.end());
    for (uint32_t ii : pending) {
        const uint8_t* rec = inst + 64ull * ii;
        float m[12];
        uint32_t root, first;
        std::memcpy(m, rec, 48);
        std::memcpy(&root, rec + 48, 4);
        std::memcpy(&first, rec + 52, 4);
        if (root == 0xFFFFFFFFu) continue;
        RayRec r = to_instance(wray, m);
        r.tmax = best.t;
        // the instance's bottom level, nearest child first (the flat traversal from its root)
        Bvh8View sub{b.nodes, b.node_count, b.tris};
        const uint64_t v0 = visited;
        BestHit<float> h = trace_bvh8_from(sub, root, r, any, visited, tested);
        (void)v0;
        if (h.prim == kMiss) continue;
        const uint32_t g = first + h.prim;
        if (h.t < best.t || g < best.prim) {
            best.prim = g;
            best.t = h.t;
            best.u = h.u;
            best.v = h.v;
            if (any) break;
        }
    }
    return best;
}

}  // namespace oracle

using namespace oracle;

extern "C" {

void* oracle_instanced_new(void) { return new InstancedScene(); }
void oracle_instanced_free(void* h) { delete static_cast<InstancedScene*>(h); }
uint32_t oracle_instanced_add_model(void* h, const float* tris9, uint64_t n) {
    InstancedScene* s = static_cast<InstancedScene*>(h);
    s->models.emplace_back(build_bvh(tris9, n));
    return (uint32_t)(s->models.size() - 1);
}
void oracle_instanced_add_instance(void* h, uint32_t model, const float* inv12, uint32_t first_prim) {
    InstancedScene* s = static_cast<InstancedScene*>(h);
    InstancedScene::Inst in;
    in.model = model;
    std::memcpy(in.inv, inv12, sizeof(in.inv));
    in.first_prim = first_prim;
    s->insts.push_back(in);
}
void oracle_instanced_raycast(void* h, const RayRec* rays, uint64_t n, int any, int threads, HitRec* hits) {
    const InstancedScene& s = *static_cast<InstancedScene*>(h);
    parallel_for(n, threads, [&](uint64_t i) { hits[i] = trace_instanced(s, rays[i], any != 0); });
}

// Exported two-level BVH8: hits (unrefined) and visit counts.
void oracle_bvh8_two_level_raycast(const uint8_t* nodes, uint64_t node_count, const float* tris, const uint32_t* refs,
                                   const uint8_t* inst, const RayRec* rays, uint64_t n, int any, int threads,
                                   HitRec* hits, uint64_t* visited, uint64_t* tested) {
    const Bvh8View b{nodes, node_count, tris};
    std::atomic<uint64_t> nv{0}, nt{0};
    parallel_for(n, threads, [&](uint64_t i) {
        uint64_t v = 0, t = 0;
        const BestHit<float> h = trace_bvh8_two_level(b, refs, inst, rays[i], any != 0, v, t);
        hits[i] = HitRec{h.prim, h.t, h.u, h.v};
        nv += v;
        nt += t;
    });
    *visited += nv.load();
    *tested += nt.load();
}

// Casts rays through an exported BVH8 (float mode, unrefined t/u/v); adds the node visits and triangle
// tests to *visited and *tested.
void oracle_bvh8_raycast(const uint8_t* nodes, uint64_t node_count, const float* tris, const RayRec* rays, uint64_t n,
                         int any, int threads, HitRec* hits, uint64_t* visited, uint64_t* tested) {
    const Bvh8View b{nodes, node_count, tris};
    std::atomic<uint64_t> nv{0}, nt{0};
    parallel_for(n, threads, [&](uint64_t i) {
        uint64_t v = 0, t = 0;
        const BestHit<float> h = trace_bvh8(b, rays[i], any != 0, v, t);
        hits[i] = HitRec{h.prim, h.t, h.u, h.v};
        nv += v;
        nt += t;
    });
    *visited += nv.load();
    *tested += nt.load();
}

int oracle_hw_threads(void) { return (int)std::max(1u, std::thread::hardware_concurrency()); }

void oracle_rng(uint32_t seed, int n, uint32_t* words, float* values, double* values64) {
    uint32_t s = seed;
    for (int i = 0; i < n; ++i) {
        const uint32_t w = rng_step(s);
        if (words) words[i] = w;
        if (values) values[i] = (float)w / 4294967295.0f;
        if (values64) values64[i] = (double)w / 4294967295.0;
    }
}

void* oracle_bvh_build(const float* tris9, uint64_t n) { return build_bvh(tris9, n); }

void oracle_bvh_destroy(void* h) { delete static_cast<Bvh*>(h); }

// precision: 32 -> HitRec (float) output in hits32; 64 -> HitRec64 output in hits64.
void oracle_raycast(void* h, const RayRec* rays, uint64_t n, int any, int precision, int threads, HitRec* hits32,
                    HitRec64* hits64) {
    const Bvh& b = *static_cast<Bvh*>(h);
    auto tris_of = [&](uint32_t p) { return p == kMiss ? nullptr : b.tris.data() + 9ull * p; };
    parallel_for(n, threads, [&](uint64_t i) {
        if (precision == 64) {
            BestHit<double> r = trace_bvh<double>(b, rays[i], any != 0, nullptr);
            hits64[i] = HitRec64{r.prim, 0u, r.t, r.u, r.v};
        } else {
            BestHit<float> r = trace_bvh<float>(b, rays[i], any != 0, nullptr);
            hits32[i] = finish32(r, rays[i], tris_of(r.prim));
        }
    });
}

void oracle_raycast_brute(const float* tris9, uint64_t ntri, const RayRec* rays, uint64_t n, int any, int precision,
                          int threads, HitRec* hits32, HitRec64* hits64) {
    auto tris_of = [&](uint32_t p) { return p == kMiss ? nullptr : tris9 + 9ull * p; };
    parallel_for(n, threads, [&](uint64_t i) {
        if (precision == 64) {
            BestHit<double> r = trace_brute<double>(tris9, ntri, rays[i], any != 0);
            hits64[i] = HitRec64{r.prim, 0u, r.t, r.u, r.v};
        } else {
            BestHit<float> r = trace_brute<float>(tris9, ntri, rays[i], any != 0);
            hits32[i] = finish32(r, rays[i], tris_of(r.prim));
        }
    });
}

// Tests one ray against one triangle (float mode) with the full [tmin, tmax] range; returns 1 on a hit.
int oracle_test_triangle(const float* tri9, const RayRec* ray, HitRec* out) {
    const PreRay<float> r = precompute<float>(*ray);
    float t, u, v;
    if (!watertight(r, tri9, r.tmax, t, u, v)) return 0;
    refine64(*ray, tri9, t, u, v);
    if (out) *out = HitRec{0u, t, u, v};
    return 1;
}

}  // extern "C"
