// Device BVH build: the host builder of bvh_build.cpp (binned-SAH binary BVH, SAH dynamic-programme
// collapse to 8-wide nodes, conservative 8-bit quantization) as CUDA kernels, writing the same bytes.
//
// Why the bytes agree: every decision depends only on the set of primitives of a binary node (bounds are
// minima and maxima, bin counts are counts, the SAH sweeps run serially in one lane in the host's order,
// and all arithmetic is the shared, explicitly rounded code of bvh_sah.h); the leaf triangles of a leaf
// child are written in ascending id order by both builders; and the wide nodes are laid out in the host's
// depth-first order from subtree sizes (below).
//
// Binary build, level-synchronous: each binary node of the current level is a task over a contiguous
// range of the primitive index array.  A task of at most kSmall primitives is handled by one warp
// (bounds, bins in shared memory, SAH sweeps, stable ballot partition, child allocation); a larger task
// is cut into work items of kItem primitives, which accumulate its bounds and bins with global atomics
// before one warp chooses the split and the items partition their ranges at offsets from a scan.  An
// object-median split (forced past the median depth, or when no axis can be binned) selects the pivot
// key (centroid, id) by rank in a warp, or by an 8-pass radix select in a block for larger tasks.
// Children are numbered level by level, so the bottom-up collapse runs one launch per level.
//
// Wide tree: top-down, each wide node gathers its children from the dynamic programme's decisions and
// assigns slots; bottom-up, each node sums the nodes and triangles its subtree allocates; top-down, the
// host's pre-order allocation (a node's inner children get consecutive indices when it is visited, its
// leaf triangles are appended then) gives every node its index, child base and triangle base; finally
// every node quantizes its children and writes its record and triangles.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <stdexcept>
#include <vector>

#include <cuda_runtime.h>

#include "bvh_build.h"
#include "bvh_sah.h"
#include "errors.h"

namespace rt {
namespace {

constexpr int kBT = 128;                 // threads per block (4 warps)
constexpr int kWarps = kBT / 32;
constexpr uint32_t kSmall = 2048;        // tasks of at most this many primitives: one warp per level step
constexpr uint32_t kItem = 4096;         // primitives per work item of a larger task
constexpr int kMaxBins = kMaxDeviceSahBins;
constexpr uint32_t kNone = 0xFFFFFFFFu;

enum : uint32_t {
    kCtrNodes = 0,       // binary nodes allocated
    kCtrLarge = 1,       // large tasks of the current level
    kCtrItems = 2,       // their work items
    kCtrNextLarge = 3,   // large tasks created for the next level
    kCtrErr = 4,         // error bits
    kCtrWide = 5,        // wide nodes allocated
    kCtrMag = 6,         // largest |coordinate| (float bits)
    kCtrSite = 7,        // first failed access check: site << 24 | low 24 bits of the index
    kCtrWords = 8
};
enum : uint32_t { kErrNonFinite = 1, kErrRange = 2, kErrInternal = 4 };
enum : uint32_t { kModeLeaf = 0, kModeSplit = 1, kModeMedian = 2 };

struct BNodeD {
    float lo[3], hi[3];
    uint32_t first, count;   // range of the primitive index array
    uint32_t left;           // internal node: left child (the right child is left + 1); leaf: 0
};

struct LargeTask {
    uint32_t node, item0, nitems, pad;
    uint32_t box[6], cbox[6];   // order-preserving unsigned encodings: lo by atomicMin, hi by atomicMax
    uint32_t mode;
    int axis, bin;
    float lo, scale;            // binning frame of the split axis
    unsigned long long pivot;   // median split: keys below the pivot go left
};

struct Item {
    uint32_t task, begin, count;
    uint32_t nleft;             // elements of the item going left
    uint32_t lpos, rpos;        // destinations of its first left and first right element
};

struct Ctx {
    const float4* plo;          // primitive boxes (xyz; w unused)
    const float4* phi;
    uint32_t* idx;
    uint32_t* tmp;
    BNodeD* nodes;
    uint32_t* ctr;
    LargeTask* large;
    Item* items;
    uint32_t* lbins;            // per large task: [3][kMaxBins][7] words (box lo, box hi, count)
    uint32_t max_large, max_items, max_nodes;
    uint32_t n;                 // primitives
    int bins, median_depth;
};

// Every index the build computes from its own tables is checked before use: a failed check records the
// site and the index (ctr[kCtrSite]) and raises kErrInternal, and the access is skipped or redirected to
// element 0, so that an inconsistent table (which a correct build never produces) ends in an error
// instead of a stray access.
__device__ __noinline__ void record_fault(uint32_t* ctr, uint32_t site, uint64_t x) {
    atomicOr(&ctr[kCtrErr], kErrInternal);
    atomicCAS(&ctr[kCtrSite], 0u, (site << 24) | (uint32_t)(x & 0xFFFFFFu));
}
__device__ __forceinline__ bool checked(const Ctx& c, uint64_t x, uint64_t lim, uint32_t site) {
    if (x < lim) return true;
    record_fault(c.ctr, site, x);
    return false;
}
__device__ __forceinline__ uint32_t idx_at(const Ctx& c, uint64_t x, uint32_t site) {
    return checked(c, x, c.n, site) ? c.idx[x] : 0u;
}

__device__ __forceinline__ uint32_t ord(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float unord(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}
__device__ __forceinline__ float fmin_h(float acc, float v) { return v < acc ? v : acc; }   // std::min(acc, v)
__device__ __forceinline__ float fmax_h(float acc, float v) { return acc < v ? v : acc; }   // std::max(acc, v)

__device__ __forceinline__ void load_box(const Ctx& c, uint32_t p, float lo[3], float hi[3]) {
    if (!checked(c, p, c.n, 1)) p = 0;
    const float4 a = c.plo[p], b = c.phi[p];
    lo[0] = a.x; lo[1] = a.y; lo[2] = a.z;
    hi[0] = b.x; hi[1] = b.y; hi[2] = b.z;
}

__device__ __forceinline__ float prim_centroid(const Ctx& c, uint32_t p, int axis) {
    if (!checked(c, p, c.n, 2)) p = 0;
    const float4 a = c.plo[p], b = c.phi[p];
    const float l = axis == 0 ? a.x : (axis == 1 ? a.y : a.z);
    const float h = axis == 0 ? b.x : (axis == 1 ? b.y : b.z);
    return sah::centroid(l, h);
}

// Median order: (centroid with -0 folded into +0, primitive id).
__device__ __forceinline__ unsigned long long median_key(const Ctx& c, uint32_t p, int axis) {
    return ((unsigned long long)ord(sah::median_key(prim_centroid(c, p, axis))) << 32) | p;
}

__device__ __forceinline__ float warp_min(float v) {
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
    return v;
}
__device__ __forceinline__ float warp_max(float v) {
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
    return v;
}

// Box and centroid bounds of idx[b, b + n), reduced over the warp (every lane gets the result).
__device__ void warp_bounds(const Ctx& c, uint32_t b, uint32_t n, int lane, float lo[3], float hi[3], float clo[3],
                            float chi[3]) {
    for (int k = 0; k < 3; ++k) {
        lo[k] = INFINITY; hi[k] = -INFINITY; clo[k] = INFINITY; chi[k] = -INFINITY;
    }
    for (uint32_t i = lane; i < n; i += 32) {
        float pl[3], ph[3];
        load_box(c, idx_at(c, (uint64_t)b + i, 3), pl, ph);
        for (int k = 0; k < 3; ++k) {
            lo[k] = fmin_h(lo[k], pl[k]);
            hi[k] = fmax_h(hi[k], ph[k]);
            const float ce = sah::centroid(pl[k], ph[k]);
            clo[k] = fmin_h(clo[k], ce);
            chi[k] = fmax_h(chi[k], ce);
        }
    }
    for (int k = 0; k < 3; ++k) {
        lo[k] = warp_min(lo[k]); hi[k] = warp_max(hi[k]);
        clo[k] = warp_min(clo[k]); chi[k] = warp_max(chi[k]);
    }
}

// The host's two sweeps over the bins of one axis (bins[i * 7 + 0..5] encoded box, [6] count): the first
// cheapest split (bin index of its last left bin) and its cost, INFINITY when no split has both sides.
__device__ void sah_axis(const uint32_t* bins, int nb, float parent, float* rarea, uint32_t* rcnt, float& best_cost,
                         int& best_bin) {
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    uint32_t cnt = 0;
    for (int i = nb - 1; i > 0; --i) {
        const uint32_t* b = bins + 7 * i;
        for (int k = 0; k < 3; ++k) {
            lo[k] = fmin_h(lo[k], unord(b[k]));
            hi[k] = fmax_h(hi[k], unord(b[3 + k]));
        }
        cnt += b[6];
        rarea[i] = sah::half_area(lo, hi);
        rcnt[i] = cnt;
    }
    for (int k = 0; k < 3; ++k) { lo[k] = INFINITY; hi[k] = -INFINITY; }
    cnt = 0;
    best_cost = INFINITY;
    best_bin = -1;
    for (int i = 0; i < nb - 1; ++i) {
        const uint32_t* b = bins + 7 * i;
        for (int k = 0; k < 3; ++k) {
            lo[k] = fmin_h(lo[k], unord(b[k]));
            hi[k] = fmax_h(hi[k], unord(b[3 + k]));
        }
        cnt += b[6];
        if (cnt == 0 || rcnt[i + 1] == 0) continue;
        const float cost = sah::split_cost(sah::half_area(lo, hi), cnt, rarea[i + 1], rcnt[i + 1], parent);
        if (cost < best_cost) { best_cost = cost; best_bin = i; }
    }
}

__device__ __forceinline__ void init_bins(uint32_t* bins, int nb, int lane, int stride) {
    for (int i = lane; i < 3 * kMaxBins; i += stride) {
        if ((i % kMaxBins) >= nb) continue;
        uint32_t* b = bins + 7 * i;
        b[0] = b[1] = b[2] = ord(INFINITY);
        b[3] = b[4] = b[5] = ord(-INFINITY);
        b[6] = 0;
    }
}

// Adds primitive p to the bins of every binnable axis.
__device__ __forceinline__ void bin_prim(const Ctx& c, uint32_t p, uint32_t* bins, const bool ok[3], const float blo[3],
                                         const float sc[3]) {
    float pl[3], ph[3];
    load_box(c, p, pl, ph);
    for (int k = 0; k < 3; ++k) {
        if (!ok[k]) continue;
        const int bi = sah::bin_of(sah::centroid(pl[k], ph[k]), blo[k], sc[k], c.bins);
        uint32_t* b = bins + 7 * (k * kMaxBins + bi);
        atomicMin(&b[0], ord(pl[0])); atomicMin(&b[1], ord(pl[1])); atomicMin(&b[2], ord(pl[2]));
        atomicMax(&b[3], ord(ph[0])); atomicMax(&b[4], ord(ph[1])); atomicMax(&b[5], ord(ph[2]));
        atomicAdd(&b[6], 1u);
    }
}

// Picks the split from the three axes' sweeps (lanes 0..2), the host's order: axis 0, 1, 2, strict less.
__device__ void choose_split(const uint32_t* bins, int nb, float parent, const bool ok[3], float* rarea,
                             uint32_t* rcnt, int lane, float& best_cost, int& best_axis, int& best_bin) {
    float cost = INFINITY;
    int bin = -1;
    if (lane < 3 && ok[lane])
        sah_axis(bins + 7 * lane * kMaxBins, nb, parent, rarea + lane * kMaxBins, rcnt + lane * kMaxBins, cost, bin);
    best_cost = INFINITY;
    best_axis = -1;
    best_bin = -1;
    for (int k = 0; k < 3; ++k) {
        const float ck = __shfl_sync(0xFFFFFFFFu, cost, k);
        const int bk = __shfl_sync(0xFFFFFFFFu, bin, k);
        if (bk >= 0 && ck < best_cost) { best_cost = ck; best_axis = k; best_bin = bk; }
    }
}

__device__ __forceinline__ int median_axis(const float clo[3], const float chi[3]) {
    int axis = 0;
    float best = -1.0f;
    for (int k = 0; k < 3; ++k) {
        const float ext = sah::sub(chi[k], clo[k]);
        if (ext > best) { best = ext; axis = k; }
    }
    return axis;
}

__device__ __forceinline__ bool goes_left(const Ctx& c, uint32_t p, uint32_t mode, int axis, int bin, float blo,
                                          float scale, unsigned long long pivot) {
    if (mode == kModeSplit) return sah::bin_of(prim_centroid(c, p, axis), blo, scale, c.bins) <= bin;
    return median_key(c, p, axis) < pivot;
}

// Two children over [first, first + nl) and [first + nl, first + count); returns the left child.
__device__ void alloc_children(const Ctx& c, uint32_t node, uint32_t first, uint32_t count, uint32_t nl) {
    const uint32_t l = atomicAdd(&c.ctr[kCtrNodes], 2u);
    if (!checked(c, (uint64_t)l + 1u, c.max_nodes, 4) || !checked(c, node, c.max_nodes, 5)) return;
    BNodeD* L = c.nodes + l;
    L[0].first = first;
    L[0].count = nl;
    L[0].left = 0;
    L[1].first = first + nl;
    L[1].count = count - nl;
    L[1].left = 0;
    c.nodes[node].left = l;
    if (nl > kSmall) atomicAdd(&c.ctr[kCtrNextLarge], 1u);
    if (count - nl > kSmall) atomicAdd(&c.ctr[kCtrNextLarge], 1u);
}

__device__ __forceinline__ uint32_t lanemask_lt_() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

struct WarpShared {
    uint32_t bins[3 * kMaxBins * 7];
    float rarea[3 * kMaxBins];
    uint32_t rcnt[3 * kMaxBins];
    unsigned long long pivot;
};

// The counters and the root node (a kernel on the build's stream, so that they are in place before the
// first level whatever the copy engine does with small host copies).
__global__ void k_init(uint32_t* ctr, BNodeD* root, uint32_t n) {
    if (threadIdx.x != 0) return;
    for (int k = 0; k < (int)kCtrWords; ++k) ctr[k] = 0u;
    ctr[kCtrNodes] = 1u;
    for (int k = 0; k < 3; ++k) {
        root->lo[k] = 0.0f;
        root->hi[k] = 0.0f;
    }
    root->first = 0u;
    root->count = n;
    root->left = 0u;
}

// Primitive boxes, the identity permutation, the coordinate magnitude and the finiteness check.
__global__ void __launch_bounds__(kBT) k_prims(const float* __restrict__ verts, uint32_t n, float4* plo, float4* phi,
                                               uint32_t* idx, uint32_t* ctr) {
    const uint32_t i = blockIdx.x * kBT + threadIdx.x;
    if (i >= n) return;
    const float* v = verts + 9ull * i;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    float mag = 0.0f;
    bool finite = true;
    for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 3; ++k) {
            const float x = v[3 * j + k];
            finite = finite && isfinite(x);
            lo[k] = fmin_h(lo[k], x);
            hi[k] = fmax_h(hi[k], x);
            mag = fmaxf(mag, fabsf(x));
        }
    idx[i] = i;
    plo[i] = make_float4(lo[0], lo[1], lo[2], 0.0f);
    phi[i] = make_float4(hi[0], hi[1], hi[2], 0.0f);
    if (!finite) {
        atomicOr(&ctr[kCtrErr], kErrNonFinite);
        return;
    }
    atomicMax(&ctr[kCtrMag], __float_as_uint(mag));
}

// The per-level counters (large tasks, their items, large tasks of the next level).
__global__ void k_level_reset(uint32_t* ctr) {
    if (threadIdx.x == 0) ctr[kCtrLarge] = ctr[kCtrItems] = ctr[kCtrNextLarge] = 0u;
}

// One level of the binary build for the tasks of at most kSmall primitives (one warp each); larger tasks
// are queued with their work items.
__global__ void __launch_bounds__(kBT) k_level_small(Ctx c, uint32_t lb, uint32_t le, int depth) {
    __shared__ WarpShared ws[kWarps];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t node = lb + blockIdx.x * kWarps + wid;
    if (node >= le) return;
    WarpShared& S = ws[wid];
    if (!checked(c, node, c.max_nodes, 6)) return;
    const uint32_t first = c.nodes[node].first, count = c.nodes[node].count;
    if (!checked(c, (uint64_t)first + count, (uint64_t)c.n + 1u, 7)) return;

    if (count > kSmall) {
        uint32_t t = 0, i0 = 0;
        const uint32_t nit = (count + kItem - 1) / kItem;
        if (lane == 0) {
            t = atomicAdd(&c.ctr[kCtrLarge], 1u);
            i0 = atomicAdd(&c.ctr[kCtrItems], nit);
        }
        t = __shfl_sync(0xFFFFFFFFu, t, 0);
        i0 = __shfl_sync(0xFFFFFFFFu, i0, 0);
        if (t >= c.max_large || i0 + nit > c.max_items) {
            if (lane == 0) record_fault(c.ctr, 41, 0);
            return;
        }
        LargeTask& T = c.large[t];
        if (lane == 0) {
            T.node = node;
            T.item0 = i0;
            T.nitems = nit;
            for (int k = 0; k < 3; ++k) {
                T.box[k] = ord(INFINITY); T.box[3 + k] = ord(-INFINITY);
                T.cbox[k] = ord(INFINITY); T.cbox[3 + k] = ord(-INFINITY);
            }
            T.mode = kModeLeaf;
            T.pivot = 0;
        }
        for (uint32_t j = lane; j < nit; j += 32) {
            Item& I = c.items[i0 + j];
            I.task = t;
            I.begin = first + j * kItem;
            I.count = min(kItem, count - j * kItem);
        }
        init_bins(c.lbins + (size_t)t * 3 * kMaxBins * 7, c.bins, lane, 32);
        return;
    }

    float lo[3], hi[3], clo[3], chi[3];
    warp_bounds(c, first, count, lane, lo, hi, clo, chi);
    if (lane == 0) {
        BNodeD& N = c.nodes[node];
        for (int k = 0; k < 3; ++k) { N.lo[k] = lo[k]; N.hi[k] = hi[k]; }
        N.left = 0;
    }
    if (count <= 1) return;

    uint32_t mode;
    int axis = 0, bin = -1;
    float blo = 0.0f, bscale = 0.0f;
    if (depth >= c.median_depth) {
        mode = count <= (uint32_t)kMaxLeafTris ? kModeLeaf : kModeMedian;
    } else {
        bool ok[3];
        float sc[3] = {0.0f, 0.0f, 0.0f};
        for (int k = 0; k < 3; ++k) ok[k] = sah::bin_scale(clo[k], chi[k], c.bins, sc[k]);
        init_bins(S.bins, c.bins, lane, 32);
        __syncwarp();
        for (uint32_t i = lane; i < count; i += 32) bin_prim(c, idx_at(c, (uint64_t)first + i, 8), S.bins, ok, clo, sc);
        __syncwarp();
        const float ha = sah::half_area(lo, hi);
        const float parent = ha < 1e-30f ? 1e-30f : ha;
        float best_cost;
        int best_axis, best_bin;
        choose_split(S.bins, c.bins, parent, ok, S.rarea, S.rcnt, lane, best_cost, best_axis, best_bin);
        if (count <= (uint32_t)kMaxLeafTris && sah::u2f(count) <= best_cost) mode = kModeLeaf;
        else if (best_axis < 0) mode = count <= (uint32_t)kMaxLeafTris ? kModeLeaf : kModeMedian;
        else {
            mode = kModeSplit;
            axis = best_axis;
            bin = best_bin;
            blo = clo[axis];
            bscale = sc[axis];
        }
    }
    if (mode == kModeLeaf) return;

    // Elements going left.
    unsigned long long pivot = 0;
    uint32_t nl = 0;
    if (mode == kModeSplit) {
        for (uint32_t s = 0; s < count; s += 32) {
            const uint32_t i = s + lane;
            const bool pred = i < count && goes_left(c, idx_at(c, (uint64_t)first + i, 9), mode, axis, bin, blo, bscale, 0);
            nl += __popc(__ballot_sync(0xFFFFFFFFu, pred));
        }
        if (nl == 0 || nl == count) mode = kModeMedian;   // (cannot happen: the bins counted both sides)
    }
    if (mode == kModeMedian) {
        axis = median_axis(clo, chi);
        const uint32_t kth = count / 2;
        if (lane == 0) S.pivot = 0;
        __syncwarp();
        for (uint32_t i = lane; i < count; i += 32) {
            const unsigned long long ki = median_key(c, idx_at(c, (uint64_t)first + i, 10), axis);
            uint32_t rank = 0;
            for (uint32_t j = 0; j < count; ++j)
                rank += median_key(c, idx_at(c, (uint64_t)first + j, 10), axis) < ki ? 1u : 0u;
            if (rank == kth) S.pivot = ki;
        }
        __syncwarp();
        pivot = S.pivot;
        nl = 0;
        for (uint32_t s = 0; s < count; s += 32) {
            const uint32_t i = s + lane;
            const bool pred = i < count && goes_left(c, idx_at(c, (uint64_t)first + i, 11), mode, axis, bin, blo, bscale, pivot);
            nl += __popc(__ballot_sync(0xFFFFFFFFu, pred));
        }
        if (nl != kth) {
            if (lane == 0) record_fault(c.ctr, 42, 0);
            return;
        }
    }

    // Stable partition into tmp, then back.
    uint32_t lpos = first, rpos = first + nl;
    for (uint32_t s = 0; s < count; s += 32) {
        const uint32_t i = s + lane;
        const bool valid = i < count;
        const uint32_t p = valid ? idx_at(c, (uint64_t)first + i, 12) : 0u;
        const bool pred = valid && goes_left(c, p, mode, axis, bin, blo, bscale, pivot);
        const uint32_t bl = __ballot_sync(0xFFFFFFFFu, pred), br = __ballot_sync(0xFFFFFFFFu, valid && !pred);
        const uint64_t dst = pred ? lpos + __popc(bl & lanemask_lt_()) : rpos + __popc(br & lanemask_lt_());
        if (valid && checked(c, dst, (uint64_t)first + count, 13)) c.tmp[dst] = p;
        lpos += __popc(bl);
        rpos += __popc(br);
    }
    __syncwarp();
    for (uint32_t i = lane; i < count; i += 32) c.idx[first + i] = c.tmp[first + i];
    if (lane == 0) alloc_children(c, node, first, count, nl);
}

__device__ __forceinline__ uint32_t global_warp() { return (blockIdx.x * kBT + threadIdx.x) >> 5; }

// Large tasks: bounds of every work item into its task.
__global__ void __launch_bounds__(kBT) k_large_bounds(Ctx c) {
    const int lane = threadIdx.x & 31;
    const uint32_t w = global_warp();
    if (w >= min(c.ctr[kCtrItems], c.max_items)) return;
    const Item I = c.items[w];
    if (!checked(c, (uint64_t)I.begin + I.count, (uint64_t)c.n + 1u, 14) || !checked(c, I.task, c.max_large, 15)) return;
    float lo[3], hi[3], clo[3], chi[3];
    warp_bounds(c, I.begin, I.count, lane, lo, hi, clo, chi);
    if (lane == 0) {
        LargeTask& T = c.large[I.task];
        for (int k = 0; k < 3; ++k) {
            atomicMin(&T.box[k], ord(lo[k]));
            atomicMax(&T.box[3 + k], ord(hi[k]));
            atomicMin(&T.cbox[k], ord(clo[k]));
            atomicMax(&T.cbox[3 + k], ord(chi[k]));
        }
    }
}

__device__ __forceinline__ void task_bounds(const LargeTask& T, float lo[3], float hi[3], float clo[3], float chi[3]) {
    for (int k = 0; k < 3; ++k) {
        lo[k] = unord(T.box[k]); hi[k] = unord(T.box[3 + k]);
        clo[k] = unord(T.cbox[k]); chi[k] = unord(T.cbox[3 + k]);
    }
}

// Large tasks: bins of every work item (shared per warp, then added into the task's bins).
__global__ void __launch_bounds__(kBT) k_large_bins(Ctx c, int depth) {
    __shared__ WarpShared ws[kWarps];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t w = global_warp();
    if (w >= min(c.ctr[kCtrItems], c.max_items) || depth >= c.median_depth) return;
    WarpShared& S = ws[wid];
    const Item I = c.items[w];
    if (!checked(c, (uint64_t)I.begin + I.count, (uint64_t)c.n + 1u, 16) || !checked(c, I.task, c.max_large, 17)) return;
    float lo[3], hi[3], clo[3], chi[3];
    task_bounds(c.large[I.task], lo, hi, clo, chi);
    bool ok[3];
    float sc[3] = {0.0f, 0.0f, 0.0f};
    for (int k = 0; k < 3; ++k) ok[k] = sah::bin_scale(clo[k], chi[k], c.bins, sc[k]);
    init_bins(S.bins, c.bins, lane, 32);
    __syncwarp();
    for (uint32_t i = lane; i < I.count; i += 32) bin_prim(c, idx_at(c, (uint64_t)I.begin + i, 18), S.bins, ok, clo, sc);
    __syncwarp();
    uint32_t* g = c.lbins + (size_t)I.task * 3 * kMaxBins * 7;
    for (int i = lane; i < 3 * kMaxBins; i += 32) {
        const uint32_t* b = S.bins + 7 * i;
        if ((i % kMaxBins) >= c.bins || b[6] == 0) continue;
        uint32_t* d = g + 7 * i;
        for (int k = 0; k < 3; ++k) {
            atomicMin(&d[k], b[k]);
            atomicMax(&d[3 + k], b[3 + k]);
        }
        atomicAdd(&d[6], b[6]);
    }
}

// Large tasks: the split decision (one warp per task).
__global__ void __launch_bounds__(kBT) k_large_split(Ctx c, int depth) {
    __shared__ WarpShared ws[kWarps];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t t = global_warp();
    if (t >= min(c.ctr[kCtrLarge], c.max_large)) return;
    LargeTask& T = c.large[t];
    float lo[3], hi[3], clo[3], chi[3];
    task_bounds(T, lo, hi, clo, chi);
    if (!checked(c, T.node, c.max_nodes, 19)) return;
    BNodeD& N = c.nodes[T.node];
    if (lane == 0) {
        for (int k = 0; k < 3; ++k) { N.lo[k] = lo[k]; N.hi[k] = hi[k]; }
        N.left = 0;
    }
    uint32_t mode = kModeMedian;
    int axis = median_axis(clo, chi), bin = -1;
    float blo = 0.0f, bscale = 0.0f;
    if (depth < c.median_depth) {
        bool ok[3];
        float sc[3] = {0.0f, 0.0f, 0.0f};
        for (int k = 0; k < 3; ++k) ok[k] = sah::bin_scale(clo[k], chi[k], c.bins, sc[k]);
        const float ha = sah::half_area(lo, hi);
        const float parent = ha < 1e-30f ? 1e-30f : ha;
        float best_cost;
        int best_axis, best_bin;
        choose_split(c.lbins + (size_t)t * 3 * kMaxBins * 7, c.bins, parent, ok, ws[wid].rarea, ws[wid].rcnt, lane,
                     best_cost, best_axis, best_bin);
        if (best_axis >= 0) {
            mode = kModeSplit;
            axis = best_axis;
            bin = best_bin;
            blo = clo[axis];
            bscale = sc[axis];
        }
    }
    if (lane == 0) {
        T.mode = mode;
        T.axis = axis;
        T.bin = bin;
        T.lo = blo;
        T.scale = bscale;
    }
}

// Large tasks split at the object median: the pivot key by an 8-pass radix select (one block per task).
constexpr int kSelBlock = 512;
__global__ void __launch_bounds__(kSelBlock) k_large_select(Ctx c) {
    __shared__ uint32_t hist[256];
    __shared__ unsigned long long prefix_s;
    __shared__ uint32_t k_s;
    const uint32_t t = blockIdx.x;
    if (t >= min(c.ctr[kCtrLarge], c.max_large)) return;
    const LargeTask& T = c.large[t];
    if (T.mode != kModeMedian || T.node >= c.max_nodes) return;
    const uint32_t first = c.nodes[T.node].first, count = c.nodes[T.node].count;
    unsigned long long prefix = 0, mask = 0;
    uint32_t k = count / 2;
    for (int pass = 0; pass < 8; ++pass) {
        const int shift = 56 - 8 * pass;
        for (int i = threadIdx.x; i < 256; i += kSelBlock) hist[i] = 0;
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < count; i += kSelBlock) {
            const unsigned long long key = median_key(c, idx_at(c, (uint64_t)first + i, 20), T.axis);
            if ((key & mask) == prefix) atomicAdd(&hist[(key >> shift) & 255u], 1u);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t cum = 0;
            int d = 0;
            for (; d < 255; ++d) {
                if (cum + hist[d] > k) break;
                cum += hist[d];
            }
            prefix_s = prefix | ((unsigned long long)d << shift);
            k_s = k - cum;
        }
        __syncthreads();
        prefix = prefix_s;
        k = k_s;
        mask |= 255ull << shift;
        __syncthreads();
    }
    if (threadIdx.x == 0) c.large[t].pivot = prefix;
}

// Large tasks: left count of every work item.
__global__ void __launch_bounds__(kBT) k_large_count(Ctx c) {
    const int lane = threadIdx.x & 31;
    const uint32_t w = global_warp();
    if (w >= min(c.ctr[kCtrItems], c.max_items)) return;
    Item& I = c.items[w];
    if (!checked(c, (uint64_t)I.begin + I.count, (uint64_t)c.n + 1u, 21) || !checked(c, I.task, c.max_large, 22)) return;
    const LargeTask& T = c.large[I.task];
    uint32_t nl = 0;
    for (uint32_t s = 0; s < I.count; s += 32) {
        const uint32_t i = s + lane;
        const bool pred = i < I.count &&
                          goes_left(c, idx_at(c, (uint64_t)I.begin + i, 23), T.mode, T.axis, T.bin, T.lo, T.scale, T.pivot);
        nl += __popc(__ballot_sync(0xFFFFFFFFu, pred));
    }
    if (lane == 0) I.nleft = nl;
}

// Large tasks: destinations of every item (scan over the task's items) and the children.
__global__ void __launch_bounds__(kBT) k_large_alloc(Ctx c) {
    const int lane = threadIdx.x & 31;
    const uint32_t t = global_warp();
    if (t >= min(c.ctr[kCtrLarge], c.max_large)) return;
    const LargeTask& T = c.large[t];
    if (!checked(c, T.node, c.max_nodes, 24) || !checked(c, (uint64_t)T.item0 + T.nitems, (uint64_t)c.max_items + 1u, 25))
        return;
    const uint32_t first = c.nodes[T.node].first, count = c.nodes[T.node].count;
    uint32_t total = 0;
    for (uint32_t s = 0; s < T.nitems; s += 32) {
        const uint32_t j = s + lane;
        const uint32_t v = j < T.nitems ? c.items[T.item0 + j].nleft : 0u;
        uint32_t incl = v;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= o) incl += u;
        }
        if (j < T.nitems) {   // lpos: left elements before the item, made absolute below
            c.items[T.item0 + j].lpos = total + incl - v;
        }
        total += __shfl_sync(0xFFFFFFFFu, incl, 31);
    }
    __syncwarp();
    // left destination: first + (left elements before it); right destination: first + (left elements in
    // all) + (right elements before it)
    for (uint32_t j = lane; j < T.nitems; j += 32) {
        Item& I = c.items[T.item0 + j];
        const uint32_t left_before = I.lpos;
        I.lpos = first + left_before;
        I.rpos = first + total + (I.begin - first) - left_before;
    }
    if (lane == 0) {
        if (total == 0 || total == count || (T.mode == kModeMedian && total != count / 2))
            record_fault(c.ctr, 43, 0);
        else alloc_children(c, T.node, first, count, total);
    }
}

// Large tasks: stable partition of every work item into tmp.
__global__ void __launch_bounds__(kBT) k_large_scatter(Ctx c) {
    const int lane = threadIdx.x & 31;
    const uint32_t w = global_warp();
    if (w >= min(c.ctr[kCtrItems], c.max_items)) return;
    const Item I = c.items[w];
    if (!checked(c, (uint64_t)I.begin + I.count, (uint64_t)c.n + 1u, 26) || !checked(c, I.task, c.max_large, 27)) return;
    const LargeTask& T = c.large[I.task];
    uint32_t lpos = I.lpos, rpos = I.rpos;
    for (uint32_t s = 0; s < I.count; s += 32) {
        const uint32_t i = s + lane;
        const bool valid = i < I.count;
        const uint32_t p = valid ? idx_at(c, (uint64_t)I.begin + i, 28) : 0u;
        const bool pred = valid && goes_left(c, p, T.mode, T.axis, T.bin, T.lo, T.scale, T.pivot);
        const uint32_t bl = __ballot_sync(0xFFFFFFFFu, pred), br = __ballot_sync(0xFFFFFFFFu, valid && !pred);
        const uint64_t dst = pred ? lpos + __popc(bl & lanemask_lt_()) : rpos + __popc(br & lanemask_lt_());
        if (valid && checked(c, dst, c.n, 29)) c.tmp[dst] = p;
        lpos += __popc(bl);
        rpos += __popc(br);
    }
}

__global__ void __launch_bounds__(kBT) k_large_copy(Ctx c) {
    const int lane = threadIdx.x & 31;
    const uint32_t w = global_warp();
    if (w >= min(c.ctr[kCtrItems], c.max_items)) return;
    const Item I = c.items[w];
    if (!checked(c, (uint64_t)I.begin + I.count, (uint64_t)c.n + 1u, 30)) return;
    for (uint32_t i = lane; i < I.count; i += 32) c.idx[I.begin + i] = c.tmp[I.begin + i];
}

// Collapse: the dynamic programme of one level of binary nodes (children are one level deeper).
__global__ void __launch_bounds__(kBT) k_dp(const BNodeD* __restrict__ nodes, sah::Dp* dp, uint32_t lb, uint32_t le,
                                            uint32_t nb, uint32_t* ctr) {
    const uint32_t n = lb + blockIdx.x * kBT + threadIdx.x;
    if (n >= le) return;
    const BNodeD N = nodes[n];
    const float area = sah::half_area(N.lo, N.hi);
    sah::Dp d;
    if (N.left == 0) {
        sah::dp_leaf(d, area, N.count);
    } else if (N.left <= n || (uint64_t)N.left + 1u >= nb) {   // children are numbered after their parent
        record_fault(ctr, 31, N.left);
        sah::dp_leaf(d, area, N.count);
    } else {
        sah::dp_inner(d, dp[N.left], dp[N.left + 1], area, N.count);
    }
    dp[n] = d;
}

struct WideRec {
    uint32_t bn;              // binary node
    uint32_t ch[8];           // child binary node of every slot (kNone = empty)
    uint32_t cw[8];           // wide records of the internal children, in slot order
    uint32_t leafmask, n_inner, n_tris;
    uint32_t sub_nodes, sub_tris;
    uint32_t index, node_ptr, tri_ptr;
};

// Children of wide node w (binary nodes, as-leaf flags) in the host's gather order.
__device__ int gather_children(const BNodeD* nodes, const sah::Dp* dp, uint32_t nb, uint32_t bn, uint32_t ch[8],
                                bool leaf[8]) {
    if (bn >= nb) return 0;
    if (nodes[bn].left == 0) {
        ch[0] = bn;
        leaf[0] = true;
        return 1;
    }
    uint32_t st_n[16];
    int st_s[16];
    int sp = 0, nch = 0;
    const uint32_t l = nodes[bn].left;
    if (l + 1u >= nb) return 0;
    const int k = sah::dp_root_split(dp[l], dp[l + 1]);
    st_n[sp] = l + 1; st_s[sp++] = 8 - k;
    st_n[sp] = l; st_s[sp++] = k;
    while (sp > 0 && nch < 8) {
        --sp;
        const uint32_t n = st_n[sp];
        const int i = st_s[sp] - 1;
        if (n >= nb || i < 0 || i > 7) return 0;
        const sah::Dp& d = dp[n];
        if (d.how[i] == 0 || d.how[i] == 1) {
            ch[nch] = n;
            leaf[nch++] = d.how[i] == 0;
            continue;
        }
        if (sp + 2 > 16) break;
        const uint32_t nl = nodes[n].left;
        if (nl == 0 || nl + 1u >= nb) return 0;
        st_n[sp] = nl + 1; st_s[sp++] = d.used[i] - d.left[i];
        st_n[sp] = nl; st_s[sp++] = d.left[i];
    }
    return nch;
}

// Wide nodes of one level: children, slots, and the records of the next level.
__global__ void __launch_bounds__(kBT) k_wide_expand(const BNodeD* __restrict__ nodes, const sah::Dp* __restrict__ dp,
                                                     uint32_t nb, WideRec* w, uint32_t wb, uint32_t we, uint32_t* ctr,
                                                     uint32_t cap) {
    const uint32_t r = wb + blockIdx.x * kBT + threadIdx.x;
    if (r >= we) return;
    WideRec& W = w[r];
    uint32_t ch[8];
    bool leaf[8];
    const int nch = gather_children(nodes, dp, nb, W.bn, ch, leaf);
    if (nch == 0) {   // (a corrupt table: cannot happen for a consistent build)
        record_fault(ctr, 44, 0);
        W.leafmask = 0;
        W.n_inner = 0;
        W.n_tris = 0;
        for (int s = 0; s < 8; ++s) W.ch[s] = kNone;
        return;
    }
    float lo[8][3], hi[8][3];
    for (int i = 0; i < nch; ++i)
        for (int k = 0; k < 3; ++k) {
            lo[i][k] = nodes[ch[i]].lo[k];
            hi[i][k] = nodes[ch[i]].hi[k];
        }
    int slot[8];
    sah::assign_slots(nch, lo, hi, slot);
    uint32_t n_inner = 0, n_tris = 0, leafmask = 0;
    for (int s = 0; s < 8; ++s) {
        W.ch[s] = slot[s] < 0 ? kNone : ch[slot[s]];
        if (slot[s] < 0) continue;
        if (leaf[slot[s]]) {
            leafmask |= 1u << s;
            n_tris += nodes[ch[slot[s]]].count;
        } else {
            ++n_inner;
        }
    }
    const uint32_t base = n_inner ? atomicAdd(&ctr[kCtrWide], n_inner) : 0u;
    if (base + n_inner > cap) {
        record_fault(ctr, 45, 0);
        n_inner = 0;
    }
    uint32_t j = 0;
    for (int s = 0; s < 8 && j < n_inner; ++s) {
        if (slot[s] < 0 || leaf[slot[s]]) continue;
        w[base + j].bn = ch[slot[s]];
        W.cw[j] = base + j;
        ++j;
    }
    W.leafmask = leafmask;
    W.n_inner = n_inner;
    W.n_tris = n_tris;
}

// The root record (binary root, node 0, children from node 1, triangles from 0) and the record counter.
__global__ void k_init_wide(WideRec* w, uint32_t* ctr) {
    if (threadIdx.x != 0) return;
    WideRec& r = w[0];
    r.bn = 0u;
    for (int s = 0; s < 8; ++s) { r.ch[s] = kNone; r.cw[s] = 0u; }
    r.leafmask = r.n_inner = r.n_tris = r.sub_nodes = r.sub_tris = 0u;
    r.index = 0u;
    r.node_ptr = 1u;
    r.tri_ptr = 0u;
    ctr[kCtrWide] = 1u;
}

__global__ void __launch_bounds__(kBT) k_wide_sums(WideRec* w, uint32_t wb, uint32_t we) {
    const uint32_t r = wb + blockIdx.x * kBT + threadIdx.x;
    if (r >= we) return;
    WideRec& W = w[r];
    uint32_t sn = W.n_inner, st = W.n_tris;
    for (uint32_t j = 0; j < W.n_inner; ++j) {
        sn += w[W.cw[j]].sub_nodes;
        st += w[W.cw[j]].sub_tris;
    }
    W.sub_nodes = sn;
    W.sub_tris = st;
}

__global__ void __launch_bounds__(kBT) k_wide_offsets(WideRec* w, uint32_t wb, uint32_t we) {
    const uint32_t r = wb + blockIdx.x * kBT + threadIdx.x;
    if (r >= we) return;
    const WideRec& W = w[r];
    uint32_t np = W.node_ptr + W.n_inner, tp = W.tri_ptr + W.n_tris;
    for (uint32_t j = 0; j < W.n_inner; ++j) {
        WideRec& C = w[W.cw[j]];
        C.index = W.node_ptr + j;
        C.node_ptr = np;
        C.tri_ptr = tp;
        np += C.sub_nodes;
        tp += C.sub_tris;
    }
}

// Quantized node record and leaf triangles of every wide node.
__global__ void __launch_bounds__(kBT) k_wide_emit(const BNodeD* __restrict__ nodes, const sah::Dp* __restrict__ dp,
                                                   uint32_t nb, const WideRec* __restrict__ w, uint32_t nw, const uint32_t* __restrict__ idx,
                                                   const float* __restrict__ verts, double delta, Bvh8Node* out_nodes,
                                                   TriRecord* out_tris, uint32_t n_tris_total, uint32_t* ctr) {
    const uint32_t r = blockIdx.x * kBT + threadIdx.x;
    if (r >= nw) return;
    const WideRec& W = w[r];
    if (W.index >= nw || W.n_tris > n_tris_total || W.tri_ptr > n_tris_total - W.n_tris) {
        record_fault(ctr, 46, 0);
        return;
    }
    uint32_t ch[8];
    bool leaf[8];
    const int nch = gather_children(nodes, dp, nb, W.bn, ch, leaf);
    if (nch == 0) {
        record_fault(ctr, 47, 0);
        return;
    }
    float ulo[3] = {INFINITY, INFINITY, INFINITY}, uhi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int i = 0; i < nch; ++i)
        for (int k = 0; k < 3; ++k) {
            ulo[k] = fmin_h(ulo[k], nodes[ch[i]].lo[k]);
            uhi[k] = fmax_h(uhi[k], nodes[ch[i]].hi[k]);
        }
    Bvh8Node node;
    memset(&node, 0, sizeof(node));
    float p[3];
    double scale[3];
    for (int k = 0; k < 3; ++k) {
        int e = 0;
        if (!sah::quant_axis(ulo[k], uhi[k], delta, p[k], e)) {
            atomicOr(&ctr[kCtrErr], kErrRange);
            return;
        }
        scale[k] = ldexp(1.0, e);
        const uint8_t eb = (uint8_t)(e + 127);
        if (k == 0) node.ex = eb;
        else if (k == 1) node.ey = eb;
        else node.ez = eb;
    }
    node.px = p[0];
    node.py = p[1];
    node.pz = p[2];
    node.child_base = W.node_ptr;
    node.tri_base = W.tri_ptr;
    uint32_t tri_off = 0;
    uint8_t imask = 0;
    for (int s = 0; s < 8; ++s) {
        const uint32_t c = W.ch[s];
        if (c == kNone) continue;
        if (c >= nb) {
            record_fault(ctr, 48, 0);
            return;
        }
        const BNodeD& C = nodes[c];
        sah::quant_child(C.lo[0], C.hi[0], delta, p[0], scale[0], node.qlo_x[s], node.qhi_x[s]);
        sah::quant_child(C.lo[1], C.hi[1], delta, p[1], scale[1], node.qlo_y[s], node.qhi_y[s]);
        sah::quant_child(C.lo[2], C.hi[2], delta, p[2], scale[2], node.qlo_z[s], node.qhi_z[s]);
        if (!(W.leafmask & (1u << s))) {
            imask |= (uint8_t)(1u << s);
            node.meta[s] = (uint8_t)((1u << 5) | (24u + (uint32_t)s));
            continue;
        }
        const uint32_t cnt = C.count;   // 1..3
        if (cnt == 0 || cnt > 3 || tri_off + cnt > W.n_tris || (uint64_t)C.first + cnt > n_tris_total) {
            record_fault(ctr, 49, 0);
            return;
        }
        node.meta[s] = (uint8_t)((((1u << cnt) - 1u) << 5) | tri_off);
        uint32_t prims[3] = {0u, 0u, 0u};
        for (uint32_t j = 0; j < cnt && j < 3; ++j) prims[j] = idx[C.first + j] < n_tris_total ? idx[C.first + j] : 0u;
        for (uint32_t a = 1; a < cnt && a < 3; ++a)   // ascending ids
            for (uint32_t b = a; b > 0 && prims[b - 1] > prims[b]; --b) {
                const uint32_t t = prims[b];
                prims[b] = prims[b - 1];
                prims[b - 1] = t;
            }
        for (uint32_t j = 0; j < cnt && j < 3; ++j) {
            const float* v = verts + 9ull * prims[j];
            TriRecord t;
            t.v0x = v[0]; t.v0y = v[1]; t.v0z = v[2]; t.prim = prims[j];
            t.v1x = v[3]; t.v1y = v[4]; t.v1z = v[5]; t.pad1 = 0.0f;
            t.v2x = v[6]; t.v2y = v[7]; t.v2z = v[8]; t.pad2 = 0.0f;
            out_tris[W.tri_ptr + tri_off + j] = t;
        }
        tri_off += cnt;
    }
    node.imask = imask;
    out_nodes[W.index] = node;
}

inline uint32_t blocks_for(uint64_t n, int per_block) { return (uint32_t)((n + per_block - 1) / per_block); }

}  // namespace

Bvh8 build_bvh8_device(int device, const float* verts, uint64_t tri_count, const BvhBuildOptions& opt,
                       double* kernel_seconds) {
    const auto t0 = std::chrono::steady_clock::now();
    if (kernel_seconds) *kernel_seconds = 0.0;
    if (tri_count == 0) return Bvh8{};
    if (tri_count >= 0x7FFFFFFFull) throw std::runtime_error("BVH build: too many triangles");
    if (opt.collapse != kCollapseSahDp) fail(REINA_ERR_INVALID, "device BVH build: only the SAH collapse is implemented");
    const int bins = std::max(4, std::min(256, opt.sah_bins));
    if (bins > kMaxDeviceSahBins)
        fail(REINA_ERR_INVALID, "device BVH build: at most " + std::to_string(kMaxDeviceSahBins) + " SAH bins");
    const uint32_t n = (uint32_t)tri_count;
    check_cuda(cudaSetDevice(device), "cudaSetDevice");

    cudaStream_t st;
    check_cuda(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
    struct StreamGuard {
        cudaStream_t s;
        ~StreamGuard() {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
    } guard{st};
    cudaEvent_t e0, e1;
    check_cuda(cudaEventCreate(&e0), "cudaEventCreate");
    check_cuda(cudaEventCreate(&e1), "cudaEventCreate");
    struct EventGuard {
        cudaEvent_t a, b;
        ~EventGuard() {
            cudaEventDestroy(a);
            cudaEventDestroy(b);
        }
    } eguard{e0, e1};

    const uint32_t max_nodes = 2u * n;
    const uint32_t max_large = n / kSmall + 2;
    const uint32_t max_items = n / kItem + max_large + 2;
    DeviceBuffer d_verts(9ull * n * sizeof(float)), d_plo(16ull * n), d_phi(16ull * n), d_idx(4ull * n), d_tmp(4ull * n),
        d_nodes((size_t)max_nodes * sizeof(BNodeD)), d_ctr(kCtrWords * sizeof(uint32_t)),
        d_large((size_t)max_large * sizeof(LargeTask)), d_items((size_t)max_items * sizeof(Item)),
        d_lbins((size_t)max_large * 3 * kMaxBins * 7 * sizeof(uint32_t));
    // The vertices are the stream's first work; every later piece of state is written by kernels on the
    // stream, and counters are read back only after a stream synchronization, so that no copy from or to
    // pageable host memory is ever ordered against queued device work.
    check_cuda(cudaMemcpyAsync(d_verts.get(), verts, 9ull * n * sizeof(float), cudaMemcpyHostToDevice, st), "H2D vertices");
    check_cuda(cudaEventRecord(e0, st), "cudaEventRecord");

    uint32_t* ctr = d_ctr.as<uint32_t>();
    k_init<<<1, 32, 0, st>>>(ctr, d_nodes.as<BNodeD>(), n);
    k_prims<<<blocks_for(n, kBT), kBT, 0, st>>>(d_verts.as<float>(), n, d_plo.as<float4>(), d_phi.as<float4>(),
                                                d_idx.as<uint32_t>(), ctr);
    check_cuda(cudaGetLastError(), "BVH build: primitive boxes");

    Ctx c{};
    c.plo = d_plo.as<float4>();
    c.phi = d_phi.as<float4>();
    c.idx = d_idx.as<uint32_t>();
    c.tmp = d_tmp.as<uint32_t>();
    c.nodes = d_nodes.as<BNodeD>();
    c.ctr = ctr;
    c.large = d_large.as<LargeTask>();
    c.items = d_items.as<Item>();
    c.lbins = d_lbins.as<uint32_t>();
    c.max_large = max_large;
    c.max_items = max_items;
    c.max_nodes = max_nodes;
    c.n = n;
    c.bins = bins;
    c.median_depth = opt.median_depth;

    uint32_t h_ctr[kCtrWords];
    auto read_ctr = [&]() {
        check_cuda(cudaStreamSynchronize(st), "BVH build");
        check_cuda(cudaMemcpy(h_ctr, ctr, sizeof(h_ctr), cudaMemcpyDeviceToHost), "D2H counters");
        if (h_ctr[kCtrErr] & kErrNonFinite) throw std::runtime_error("BVH build: non-finite vertex coordinate");
        if (h_ctr[kCtrErr] & kErrRange) throw std::runtime_error("BVH build: scene coordinates out of range");
        if (h_ctr[kCtrErr])
            fail(REINA_ERR_DEVICE, "device BVH build: inconsistent state (check " + std::to_string(h_ctr[kCtrSite] >> 24) +
                                       ", index " + std::to_string(h_ctr[kCtrSite] & 0xFFFFFFu) + ")");
    };
    read_ctr();
    float mag = 0.0f;
    std::memcpy(&mag, &h_ctr[kCtrMag], sizeof(float));

    // Binary build, one level per iteration.
    std::vector<uint32_t> level_begin{0u, 1u};   // level L = nodes [level_begin[L], level_begin[L + 1])
    uint32_t lb = 0, le = 1, n_large = n > kSmall ? 1u : 0u;
    for (int depth = 0; lb < le; ++depth) {
        k_level_reset<<<1, 32, 0, st>>>(ctr);
        k_level_small<<<blocks_for(le - lb, kWarps), kBT, 0, st>>>(c, lb, le, depth);
        if (n_large > 0) {
            const uint32_t item_blocks = blocks_for(std::min<uint64_t>(max_items, (uint64_t)n / kItem + n_large + 1), kWarps);
            const uint32_t task_blocks = blocks_for(n_large, kWarps);
            k_large_bounds<<<item_blocks, kBT, 0, st>>>(c);
            k_large_bins<<<item_blocks, kBT, 0, st>>>(c, depth);
            k_large_split<<<task_blocks, kBT, 0, st>>>(c, depth);
            k_large_select<<<n_large, kSelBlock, 0, st>>>(c);
            k_large_count<<<item_blocks, kBT, 0, st>>>(c);
            k_large_alloc<<<task_blocks, kBT, 0, st>>>(c);
            k_large_scatter<<<item_blocks, kBT, 0, st>>>(c);
            k_large_copy<<<item_blocks, kBT, 0, st>>>(c);
        }
        check_cuda(cudaGetLastError(), "BVH build: binary level");
        read_ctr();
        lb = le;
        le = h_ctr[kCtrNodes];
        n_large = h_ctr[kCtrNextLarge];
        level_begin.push_back(le);
        if (le > max_nodes || depth > 4096) fail(REINA_ERR_DEVICE, "device BVH build: node overflow");
    }
    const uint32_t nb = le;

    // Collapse: dynamic programme bottom-up.
    DeviceBuffer d_dp((size_t)nb * sizeof(sah::Dp));
    for (size_t L = level_begin.size() - 1; L-- > 0;) {
        const uint32_t a = level_begin[L], b = level_begin[L + 1];
        if (b > a) k_dp<<<blocks_for(b - a, kBT), kBT, 0, st>>>(c.nodes, d_dp.as<sah::Dp>(), a, b, nb, ctr);
    }
    check_cuda(cudaGetLastError(), "BVH build: collapse");

    // Wide tree: records level by level from the root.
    const uint32_t wcap = n + 1;
    DeviceBuffer d_w((size_t)wcap * sizeof(WideRec));
    k_init_wide<<<1, 32, 0, st>>>(d_w.as<WideRec>(), ctr);
    std::vector<uint32_t> wlevel{0u, 1u};   // wide level L = records [wlevel[L], wlevel[L + 1])
    uint32_t wb = 0, we = 1;
    while (wb < we) {
        k_wide_expand<<<blocks_for(we - wb, kBT), kBT, 0, st>>>(c.nodes, d_dp.as<sah::Dp>(), nb, d_w.as<WideRec>(), wb, we,
                                                               ctr, wcap);
        check_cuda(cudaGetLastError(), "BVH build: wide level");
        read_ctr();
        wb = we;
        we = h_ctr[kCtrWide];
        wlevel.push_back(we);
    }
    const uint32_t nw = we;
    const uint32_t depth = (uint32_t)wlevel.size() - 2;   // the last entry repeats the end
    if (depth > kMaxBvhDepth) throw std::runtime_error("BVH build: tree deeper than the traversal stack");
    for (size_t L = wlevel.size() - 1; L-- > 0;)
        if (wlevel[L + 1] > wlevel[L])
            k_wide_sums<<<blocks_for(wlevel[L + 1] - wlevel[L], kBT), kBT, 0, st>>>(d_w.as<WideRec>(), wlevel[L],
                                                                                  wlevel[L + 1]);
    for (size_t L = 0; L + 1 < wlevel.size(); ++L)
        if (wlevel[L + 1] > wlevel[L])
            k_wide_offsets<<<blocks_for(wlevel[L + 1] - wlevel[L], kBT), kBT, 0, st>>>(d_w.as<WideRec>(), wlevel[L],
                                                                                     wlevel[L + 1]);
    DeviceBuffer d_out_nodes((size_t)nw * sizeof(Bvh8Node)), d_out_tris((size_t)n * sizeof(TriRecord));
    k_wide_emit<<<blocks_for(nw, kBT), kBT, 0, st>>>(c.nodes, d_dp.as<sah::Dp>(), nb, d_w.as<WideRec>(), nw, c.idx,
                                                     d_verts.as<float>(), sah::quant_delta(mag), d_out_nodes.as<Bvh8Node>(),
                                                     d_out_tris.as<TriRecord>(), n, ctr);
    check_cuda(cudaGetLastError(), "BVH build: emit");
    check_cuda(cudaEventRecord(e1, st), "cudaEventRecord");
    read_ctr();

    Bvh8 out;
    out.nodes.resize(nw);
    out.tris.resize(n);
    check_cuda(cudaMemcpy(out.nodes.data(), d_out_nodes.get(), (size_t)nw * sizeof(Bvh8Node), cudaMemcpyDeviceToHost),
               "D2H nodes");
    check_cuda(cudaMemcpy(out.tris.data(), d_out_tris.get(), (size_t)n * sizeof(TriRecord), cudaMemcpyDeviceToHost),
               "D2H triangles");
    float ms = 0.0f;
    check_cuda(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
    if (kernel_seconds) *kernel_seconds = ms * 1e-3;
    out.depth = depth;
    out.binary_nodes = nb;
    out.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return out;
}

}  // namespace rt
