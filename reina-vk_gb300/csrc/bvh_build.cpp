// Binned-SAH BVH build, 8-wide collapse and conservative 8-bit child-box quantization (host C++).  The
// arithmetic lives in bvh_sah.h, shared with the device builder (bvh_gpu.cu), which writes the same bytes.
#include "bvh_build.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <thread>

#include "bvh_sah.h"

namespace rt {
namespace {

struct Box {
    float lo[3], hi[3];
};

inline Box empty_box() {
    Box b;
    for (int k = 0; k < 3; ++k) {
        b.lo[k] = INFINITY;
        b.hi[k] = -INFINITY;
    }
    return b;
}

inline void grow(Box& b, const Box& o) {
    for (int k = 0; k < 3; ++k) {
        b.lo[k] = std::min(b.lo[k], o.lo[k]);
        b.hi[k] = std::max(b.hi[k], o.hi[k]);
    }
}

inline float half_area(const Box& b) { return sah::half_area(b.lo, b.hi); }

struct BNode {
    Box box;
    uint32_t left;    // internal: index of the left child (the right child is left + 1)
    uint32_t first;   // leaf: first entry of the primitive index array
    uint32_t count;   // leaf: primitive count (0 for internal nodes)
};

struct BinaryBuilder {
    const float* verts = nullptr;
    std::vector<Box> prim_box;
    std::vector<float> centroid;        // 3 per primitive
    std::vector<uint32_t> idx;
    std::vector<BNode> nodes;
    std::atomic<uint32_t> next{1};
    std::atomic<int> spare_threads{0};
    int bins = 32;
    int median_depth = sah::kForceMedianDepth;

    void range_bounds(uint32_t b, uint32_t e, Box& box, Box& cbox) const {
        box = empty_box();
        cbox = empty_box();
        for (uint32_t i = b; i < e; ++i) {
            uint32_t p = idx[i];
            grow(box, prim_box[p]);
            for (int k = 0; k < 3; ++k) {
                float c = centroid[3 * p + k];
                cbox.lo[k] = std::min(cbox.lo[k], c);
                cbox.hi[k] = std::max(cbox.hi[k], c);
            }
        }
    }

    void make_leaf(uint32_t node, uint32_t b, uint32_t e) {
        nodes[node].first = b;
        nodes[node].count = e - b;
        nodes[node].left = 0;
    }

    // Splits idx[b, e) at its middle along the largest centroid axis (object median; ties by index).
    uint32_t median_split(uint32_t b, uint32_t e, const Box& cbox) {
        int axis = 0;
        float best = -1.0f;
        for (int k = 0; k < 3; ++k) {
            const float ext = sah::sub(cbox.hi[k], cbox.lo[k]);
            if (ext > best) { best = ext; axis = k; }
        }
        uint32_t mid = b + (e - b) / 2;
        std::nth_element(idx.begin() + b, idx.begin() + mid, idx.begin() + e, [&](uint32_t x, uint32_t y) {
            const float cx = sah::median_key(centroid[3 * x + axis]), cy = sah::median_key(centroid[3 * y + axis]);
            return cx < cy || (cx == cy && x < y);
        });
        return mid;
    }

    void build(uint32_t node, uint32_t b, uint32_t e, int depth) {
        Box box, cbox;
        range_bounds(b, e, box, cbox);
        nodes[node].box = box;
        const uint32_t n = e - b;
        if (n <= 1) { make_leaf(node, b, e); return; }

        uint32_t mid = b;
        if (depth >= median_depth) {
            if (n <= (uint32_t)kMaxLeafTris) { make_leaf(node, b, e); return; }
            mid = median_split(b, e, cbox);
        } else {
            // Binned SAH over the three axes: cost(split) = 1 + (A_L n_L + A_R n_R) / A, cost(leaf) = n.
            float best_cost = INFINITY;
            int best_axis = -1, best_bin = -1;
            const float parent_area = std::max(half_area(box), 1e-30f);
            std::vector<Box> bin_box(bins);
            std::vector<uint32_t> bin_cnt(bins);
            std::vector<float> right_area(bins);
            std::vector<uint32_t> right_cnt(bins);
            for (int axis = 0; axis < 3; ++axis) {
                const float lo = cbox.lo[axis];
                float scale;
                if (!sah::bin_scale(lo, cbox.hi[axis], bins, scale)) continue;
                for (int i = 0; i < bins; ++i) { bin_box[i] = empty_box(); bin_cnt[i] = 0; }
                for (uint32_t i = b; i < e; ++i) {
                    uint32_t p = idx[i];
                    const int bi = sah::bin_of(centroid[3 * p + axis], lo, scale, bins);
                    grow(bin_box[bi], prim_box[p]);
                    bin_cnt[bi]++;
                }
                Box acc = empty_box();
                uint32_t cnt = 0;
                for (int i = bins - 1; i > 0; --i) {
                    grow(acc, bin_box[i]);
                    cnt += bin_cnt[i];
                    right_area[i] = half_area(acc);
                    right_cnt[i] = cnt;
                }
                acc = empty_box();
                cnt = 0;
                for (int i = 0; i < bins - 1; ++i) {
                    grow(acc, bin_box[i]);
                    cnt += bin_cnt[i];
                    if (cnt == 0 || right_cnt[i + 1] == 0) continue;
                    const float cost = sah::split_cost(half_area(acc), cnt, right_area[i + 1], right_cnt[i + 1], parent_area);
                    if (cost < best_cost) { best_cost = cost; best_axis = axis; best_bin = i; }
                }
            }
            if (n <= (uint32_t)kMaxLeafTris && (float)n <= best_cost) { make_leaf(node, b, e); return; }
            if (best_axis < 0) {
                if (n <= (uint32_t)kMaxLeafTris) { make_leaf(node, b, e); return; }
                mid = median_split(b, e, cbox);
            } else {
                const float lo = cbox.lo[best_axis];
                float scale = 0.0f;
                sah::bin_scale(lo, cbox.hi[best_axis], bins, scale);
                auto it = std::partition(idx.begin() + b, idx.begin() + e, [&](uint32_t p) {
                    return sah::bin_of(centroid[3 * p + best_axis], lo, scale, bins) <= best_bin;
                });
                mid = (uint32_t)(it - idx.begin());
                if (mid == b || mid == e) mid = median_split(b, e, cbox);
            }
        }

        const uint32_t left = next.fetch_add(2);
        nodes[node].left = left;
        nodes[node].count = 0;
        if (n > 65536 && spare_threads.fetch_sub(1) > 0) {
            std::thread t([&, left, b, mid, depth] { build(left, b, mid, depth + 1); });
            build(left + 1, mid, e, depth + 1);
            t.join();
        } else {
            build(left, b, mid, depth + 1);
            build(left + 1, mid, e, depth + 1);
        }
    }
};

using sah::kLeafMax;

struct WideBuilder {
    const BinaryBuilder& bb;
    Bvh8& out;
    double delta;   // conservative dilation of every quantized child box, in world units
    int collapse = kCollapseSahDp;
    std::vector<uint32_t>* refs = nullptr;   // box mode: leaf entries are box indices appended here

    std::vector<sah::Dp> dp;
    std::vector<uint32_t> sub_first, sub_count;   // triangle range of every binary subtree

    bool is_leaf(uint32_t n) const { return bb.nodes[n].count > 0; }

    void solve(uint32_t n) {
        const BNode& b = bb.nodes[n];
        const float area = half_area(b.box);
        if (b.count > 0) {
            sub_first[n] = b.first;
            sub_count[n] = b.count;
            sah::dp_leaf(dp[n], area, b.count);
            return;
        }
        const uint32_t l = b.left, r = b.left + 1;
        solve(l);
        solve(r);
        sub_first[n] = std::min(sub_first[l], sub_first[r]);
        sub_count[n] = sub_count[l] + sub_count[r];
        sah::dp_inner(dp[n], dp[l], dp[r], area, sub_count[n]);
    }

    // Wide children of binary subtree `n` given `slots`: (binary node, as one leaf child).
    void gather(uint32_t n, int slots, uint32_t* ch, bool* leaf, int& nch) const {
        const sah::Dp& d = dp[n];
        const int i = slots - 1;
        if (d.how[i] == 0) { ch[nch] = n; leaf[nch++] = true; return; }
        if (d.how[i] == 1) { ch[nch] = n; leaf[nch++] = false; return; }
        const uint32_t l = bb.nodes[n].left;
        gather(l, d.left[i], ch, leaf, nch);
        gather(l + 1, d.used[i] - d.left[i], ch, leaf, nch);
    }

    void prepare() {
        if (collapse != kCollapseSahDp) return;
        const size_t nb = bb.next.load();
        dp.resize(nb);
        sub_first.resize(nb);
        sub_count.resize(nb);
        solve(0);
    }

    void emit(uint32_t wi, uint32_t bn, uint32_t depth) {
        out.depth = std::max(out.depth, depth);
        uint32_t ch[8];
        bool leaf[8];
        int nch = 0;
        if (is_leaf(bn)) {
            ch[nch] = bn;
            leaf[nch++] = true;
        } else if (collapse == kCollapseSahDp) {
            // The node itself is internal: distribute its subtree over 8 slots (dist(n, 8)).
            const int best_k = sah::dp_root_split(dp[bb.nodes[bn].left], dp[bb.nodes[bn].left + 1]);
            gather(bb.nodes[bn].left, best_k, ch, leaf, nch);
            gather(bb.nodes[bn].left + 1, 8 - best_k, ch, leaf, nch);
        } else {
            ch[nch] = bb.nodes[bn].left;
            leaf[nch++] = is_leaf(ch[0]);
            ch[nch] = bb.nodes[bn].left + 1;
            leaf[nch++] = is_leaf(ch[1]);
            // Greedy collapse: open the internal child of largest surface area until 8 children.
            while (nch < 8) {
                int pick = -1;
                float best = -1.0f;
                for (int i = 0; i < nch; ++i) {
                    if (leaf[i]) continue;
                    float a = half_area(bb.nodes[ch[i]].box);
                    if (a > best) { best = a; pick = i; }
                }
                if (pick < 0) break;
                uint32_t l = bb.nodes[ch[pick]].left;
                ch[pick] = l;
                leaf[pick] = is_leaf(l);
                ch[nch] = l + 1;
                leaf[nch++] = is_leaf(l + 1);
            }
        }

        // Union box and octant-based slot assignment.
        float clo[8][3], chi[8][3];
        Box u = empty_box();
        for (int i = 0; i < nch; ++i) {
            const Box& cb = bb.nodes[ch[i]].box;
            grow(u, cb);
            for (int k = 0; k < 3; ++k) {
                clo[i][k] = cb.lo[k];
                chi[i][k] = cb.hi[k];
            }
        }
        int child_in_slot[8];
        sah::assign_slots(nch, clo, chi, child_in_slot);

        Bvh8Node node;
        std::memset(&node, 0, sizeof(node));
        double scale[3];
        float p[3];
        uint8_t ebias[3];
        for (int k = 0; k < 3; ++k) {
            int e = 0;
            if (!sah::quant_axis(u.lo[k], u.hi[k], delta, p[k], e))
                throw std::runtime_error("BVH build: scene coordinates out of range");
            scale[k] = std::ldexp(1.0, e);
            ebias[k] = (uint8_t)(e + 127);
        }
        node.px = p[0];
        node.py = p[1];
        node.pz = p[2];
        node.ex = ebias[0];
        node.ey = ebias[1];
        node.ez = ebias[2];

        // Children in slot order: internal ones get consecutive node indices, leaf triangles are
        // appended to the triangle array.
        uint32_t inner_bnodes[8];
        int n_inner = 0;
        node.tri_base = (uint32_t)(refs ? refs->size() : out.tris.size());
        uint32_t tri_off = 0;
        uint8_t imask = 0;
        for (int s = 0; s < 8; ++s) {
            int ci = child_in_slot[s];
            if (ci < 0) continue;
            const BNode& c = bb.nodes[ch[ci]];
            const bool as_leaf = leaf[ci];
            auto q = [&](int k, float lo, float hi, uint8_t& qlo, uint8_t& qhi) {
                sah::quant_child(lo, hi, delta, p[k], scale[k], qlo, qhi);
            };
            q(0, c.box.lo[0], c.box.hi[0], node.qlo_x[s], node.qhi_x[s]);
            q(1, c.box.lo[1], c.box.hi[1], node.qlo_y[s], node.qhi_y[s]);
            q(2, c.box.lo[2], c.box.hi[2], node.qlo_z[s], node.qhi_z[s]);
            if (!as_leaf) {
                imask |= (uint8_t)(1u << s);
                node.meta[s] = (uint8_t)((1u << 5) | (24u + (uint32_t)s));
                inner_bnodes[n_inner++] = ch[ci];
            } else {
                // a binary leaf, or (dynamic programme) a whole subtree of at most 3 triangles
                const uint32_t first = is_leaf(ch[ci]) ? c.first : sub_first[ch[ci]];
                const uint32_t cnt = is_leaf(ch[ci]) ? c.count : sub_count[ch[ci]];   // 1..3
                const uint32_t unary = (1u << cnt) - 1u;
                node.meta[s] = (uint8_t)((unary << 5) | tri_off);
                uint32_t prims[kLeafMax];   // a leaf child's triangles in ascending id order
                for (uint32_t j = 0; j < cnt; ++j) prims[j] = bb.idx[first + j];
                std::sort(prims, prims + cnt);
                for (uint32_t j = 0; j < cnt; ++j) {
                    const uint32_t prim = prims[j];
                    if (refs) {
                        refs->push_back(prim);
                        continue;
                    }
                    const float* v = bb.verts + 9ull * prim;
                    TriRecord r;
                    r.v0x = v[0]; r.v0y = v[1]; r.v0z = v[2]; r.prim = prim;
                    r.v1x = v[3]; r.v1y = v[4]; r.v1z = v[5]; r.pad1 = 0.0f;
                    r.v2x = v[6]; r.v2y = v[7]; r.v2z = v[8]; r.pad2 = 0.0f;
                    out.tris.push_back(r);
                }
                tri_off += cnt;
            }
        }
        node.imask = imask;
        node.child_base = (uint32_t)out.nodes.size();
        out.nodes.resize(out.nodes.size() + n_inner);
        out.nodes[wi] = node;
        const uint32_t base = node.child_base;
        for (int i = 0; i < n_inner; ++i) emit(base + (uint32_t)i, inner_bnodes[i], depth + 1);
    }
};

}  // namespace

// Binary SAH build over primitive boxes, collapse and quantization; leaves become triangle records
// (verts) or entries of `refs` (box mode).
static Bvh8 build_core(std::vector<Box>&& boxes, double mag, const float* verts, std::vector<uint32_t>* refs,
                       const BvhBuildOptions& opt) {
    auto t0 = std::chrono::steady_clock::now();
    Bvh8 out;
    const uint32_t n = (uint32_t)boxes.size();
    if (n == 0) return out;
    BinaryBuilder bb;
    bb.verts = verts;
    bb.bins = std::max(4, std::min(256, opt.sah_bins));
    bb.median_depth = opt.median_depth;
    bb.prim_box = std::move(boxes);
    bb.centroid.resize(3ull * n);
    bb.idx.resize(n);
    for (uint32_t i = 0; i < n; ++i) {
        const Box& b = bb.prim_box[i];
        for (int k = 0; k < 3; ++k) bb.centroid[3ull * i + k] = sah::centroid(b.lo[k], b.hi[k]);
        bb.idx[i] = i;
    }
    bb.nodes.resize(2ull * n);
    int hw = opt.max_threads > 0 ? opt.max_threads : (int)std::thread::hardware_concurrency();
    bb.spare_threads = std::max(0, hw - 1);
    bb.build(0, 0, n, 0);
    out.binary_nodes = bb.next.load();

    const double delta = sah::quant_delta((float)mag);
    out.nodes.resize(1);
    if (!refs) out.tris.reserve(n);
    WideBuilder wb{bb, out, delta, opt.collapse, refs};
    wb.prepare();
    wb.emit(0, 0, 1);
    if (out.depth > kMaxBvhDepth) throw std::runtime_error("BVH build: tree deeper than the traversal stack");
    out.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return out;
}

Bvh8 build_bvh8(const float* verts, uint64_t tri_count, const BvhBuildOptions& opt) {
    if (tri_count == 0) return Bvh8{};
    if (tri_count >= 0x7FFFFFFFull) throw std::runtime_error("BVH build: too many triangles");
    const uint32_t n = (uint32_t)tri_count;
    std::vector<Box> boxes(n);
    double mag = 0.0;
    for (uint32_t i = 0; i < n; ++i) {
        const float* v = verts + 9ull * i;
        Box b = empty_box();
        for (int j = 0; j < 3; ++j) {
            for (int k = 0; k < 3; ++k) {
                float c = v[3 * j + k];
                if (!std::isfinite(c)) throw std::runtime_error("BVH build: non-finite vertex coordinate");
                b.lo[k] = std::min(b.lo[k], c);
                b.hi[k] = std::max(b.hi[k], c);
                mag = std::max(mag, (double)std::fabs(c));
            }
        }
        boxes[i] = b;
    }
    return build_core(std::move(boxes), mag, verts, nullptr, opt);
}

Bvh8 build_bvh8_boxes(const float* boxes6, uint64_t box_count, std::vector<uint32_t>& refs, const BvhBuildOptions& opt) {
    refs.clear();
    if (box_count == 0) return Bvh8{};
    if (box_count >= 0x7FFFFFFFull) throw std::runtime_error("BVH build: too many boxes");
    const uint32_t n = (uint32_t)box_count;
    std::vector<Box> boxes(n);
    double mag = 0.0;
    for (uint32_t i = 0; i < n; ++i) {
        for (int k = 0; k < 3; ++k) {
            const float lo = boxes6[6ull * i + k], hi = boxes6[6ull * i + 3 + k];
            if (!std::isfinite(lo) || !std::isfinite(hi) || lo > hi) throw std::runtime_error("BVH build: invalid box");
            boxes[i].lo[k] = lo;
            boxes[i].hi[k] = hi;
            mag = std::max(mag, std::max((double)std::fabs(lo), (double)std::fabs(hi)));
        }
    }
    return build_core(std::move(boxes), mag, nullptr, &refs, opt);
}

}  // namespace rt
