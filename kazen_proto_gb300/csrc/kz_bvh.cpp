// kz_bvh.cpp — binned-SAH BVH build and device layout (see kz_bvh.h).
#include "kz_bvh.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>

namespace kz {
namespace {

constexpr int kBins = 32;
constexpr float kInf = std::numeric_limits<float>::infinity();

struct Box {
    float lo[3] = {kInf, kInf, kInf};
    float hi[3] = {-kInf, -kInf, -kInf};
    void grow(const Box& b) {
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], b.lo[a]);
            hi[a] = std::max(hi[a], b.hi[a]);
        }
    }
    void grow(const float* p) {
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], p[a]);
            hi[a] = std::max(hi[a], p[a]);
        }
    }
    float area() const {
        if (lo[0] > hi[0]) return 0.f;
        float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        return 2.f * (dx * dy + dy * dz + dz * dx);
    }
};

struct BNode {
    Box box;
    int32_t left = -1, right = -1;
    uint32_t first = 0, count = 0;
};

struct Builder {
    const BvhBuildInput& in;
    int max_leaf;
    std::vector<Box> tb;           // per-triangle bounds
    std::vector<float> cen;        // per-triangle centroid * 3
    std::vector<uint32_t> idx;     // permutation
    std::vector<BNode> nodes;
    uint32_t max_depth = 0;

    Builder(const BvhBuildInput& i, int ml) : in(i), max_leaf(ml) {}

    void run() {
        const uint32_t n = in.ntris;
        tb.resize(n);
        cen.resize((size_t)n * 3);
        idx.resize(n);
        for (uint32_t t = 0; t < n; ++t) {
            const float* v = in.tri_verts + (size_t)t * 9;
            Box b;
            b.grow(v);
            b.grow(v + 3);
            b.grow(v + 6);
            tb[t] = b;
            for (int a = 0; a < 3; ++a) cen[(size_t)t * 3 + a] = 0.5f * (b.lo[a] + b.hi[a]);
            idx[t] = t;
        }
        nodes.reserve(n ? 2 * (size_t)n / (size_t)std::max(1, max_leaf / 2) + 8 : 1);
        nodes.emplace_back();
        struct Task { uint32_t node, first, count, depth; };
        std::vector<Task> stack;
        stack.push_back({0, 0, n, 1});
        while (!stack.empty()) {
            Task tk = stack.back();
            stack.pop_back();
            max_depth = std::max(max_depth, tk.depth);
            Box bb, cb;
            for (uint32_t i = tk.first; i < tk.first + tk.count; ++i) {
                bb.grow(tb[idx[i]]);
                cb.grow(&cen[(size_t)idx[i] * 3]);
            }
            nodes[tk.node].box = bb;
            uint32_t mid = 0;
            bool split = tk.count > 1 && (int)tk.depth < kMaxBvhDepth - 1 && choose_split(tk.first, tk.count, bb, cb, mid);
            if (!split) {
                nodes[tk.node].first = tk.first;
                nodes[tk.node].count = tk.count;
                continue;
            }
            int32_t l = (int32_t)nodes.size();
            nodes.emplace_back();
            int32_t r = (int32_t)nodes.size();
            nodes.emplace_back();
            nodes[tk.node].left = l;
            nodes[tk.node].right = r;
            stack.push_back({(uint32_t)r, mid, tk.first + tk.count - mid, tk.depth + 1});
            stack.push_back({(uint32_t)l, tk.first, mid - tk.first, tk.depth + 1});
        }
    }

    // Returns true and the partition point when the node should be split.
    bool choose_split(uint32_t first, uint32_t count, const Box& bb, const Box& cb, uint32_t& mid) {
        int best_axis = -1, best_bin = -1;
        float best_cost = kInf;
        for (int a = 0; a < 3; ++a) {
            float ext = cb.hi[a] - cb.lo[a];
            if (!(ext > 0.f)) continue;
            float scale = (float)kBins / ext;
            Box bins[kBins];
            uint32_t cnt[kBins] = {0};
            for (uint32_t i = first; i < first + count; ++i) {
                uint32_t t = idx[i];
                int b = (int)((cen[(size_t)t * 3 + a] - cb.lo[a]) * scale);
                b = std::min(std::max(b, 0), kBins - 1);
                cnt[b]++;
                bins[b].grow(tb[t]);
            }
            float rarea[kBins];
            uint32_t rcnt[kBins];
            Box acc;
            uint32_t c = 0;
            for (int b = kBins - 1; b > 0; --b) {
                acc.grow(bins[b]);
                c += cnt[b];
                rarea[b] = acc.area();
                rcnt[b] = c;
            }
            Box lacc;
            uint32_t lc = 0;
            for (int b = 0; b < kBins - 1; ++b) {
                lacc.grow(bins[b]);
                lc += cnt[b];
                if (lc == 0 || rcnt[b + 1] == 0) continue;
                float cost = lacc.area() * (float)lc + rarea[b + 1] * (float)rcnt[b + 1];
                if (cost < best_cost) {
                    best_cost = cost;
                    best_axis = a;
                    best_bin = b;
                }
            }
        }
        const float parent_area = bb.area();
        // SAH: traversal cost 1, intersection cost 1 per triangle
        const float leaf_cost = (float)count;
        const bool must_split = (int)count > max_leaf;
        if (best_axis >= 0) {
            float split_cost = 1.f + (parent_area > 0.f ? best_cost / parent_area : (float)count);
            if (!must_split && split_cost >= leaf_cost) return false;
            const int a = best_axis;
            const float scale = (float)kBins / (cb.hi[a] - cb.lo[a]);
            auto it = std::partition(idx.begin() + first, idx.begin() + first + count, [&](uint32_t t) {
                int b = (int)((cen[(size_t)t * 3 + a] - cb.lo[a]) * scale);
                b = std::min(std::max(b, 0), kBins - 1);
                return b <= best_bin;
            });
            mid = (uint32_t)(it - idx.begin());
            if (mid > first && mid < first + count) return true;
        }
        if (!must_split) return false;
        // coincident centroids or a failed partition: split by count
        int a = 0;
        for (int k = 1; k < 3; ++k)
            if (bb.hi[k] - bb.lo[k] > bb.hi[a] - bb.lo[a]) a = k;
        mid = first + count / 2;
        std::nth_element(idx.begin() + first, idx.begin() + mid, idx.begin() + first + count,
                         [&](uint32_t p, uint32_t q) {
                             float cp = cen[(size_t)p * 3 + a], cq = cen[(size_t)q * 3 + a];
                             return cp < cq || (cp == cq && p < q);
                         });
        return true;
    }
};

inline float u2f(uint32_t u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

}  // namespace

void build_bvh(const BvhBuildInput& in, int max_leaf, BvhBuildOutput& out) {
    Builder b(in, max_leaf);
    b.run();
    const auto& bn = b.nodes;

    // Device layout: one device node per inner build node, preorder; a leaf
    // root becomes child 0 of a synthetic root.
    out.nodes.clear();
    out.tris.clear();
    out.order.clear();
    out.tris.reserve((size_t)in.ntris * 12);
    out.order.reserve(in.ntris);

    auto emit_leaf = [&](const BNode& nd) -> int32_t {
        uint32_t rec = (uint32_t)out.order.size();
        for (uint32_t i = nd.first; i < nd.first + nd.count; ++i) {
            uint32_t t = b.idx[i];
            const float* v = in.tri_verts + (size_t)t * 9;
            uint32_t geom = in.tri_geom ? in.tri_geom[t] : 0u;
            uint32_t mat = in.geom_material ? (uint32_t)in.geom_material[geom] : 0u;
            float r[12] = {v[0], v[1], v[2], u2f(t), v[3], v[4], v[5], u2f(geom), v[6], v[7], v[8], u2f(mat)};
            out.tris.insert(out.tris.end(), r, r + 12);
            out.order.push_back(t);
        }
        return ~(int32_t)rec;
    };

    struct Item { int32_t build_node; uint32_t dev_node; };
    std::vector<Item> stack;
    auto alloc_dev = [&]() -> uint32_t {
        uint32_t id = (uint32_t)(out.nodes.size() / 16);
        out.nodes.resize(out.nodes.size() + 16, 0.f);
        return id;
    };
    auto set_child = [&](uint32_t dev, int slot, const Box& box, int32_t link, uint32_t count) {
        float* n = &out.nodes[(size_t)dev * 16];
        const Box& bx = box;
        float* xy = n + slot * 4;
        xy[0] = bx.lo[0];
        xy[1] = bx.hi[0];
        xy[2] = bx.lo[1];
        xy[3] = bx.hi[1];
        n[8 + slot * 2] = bx.lo[2];
        n[9 + slot * 2] = bx.hi[2];
        n[12 + slot] = u2f((uint32_t)link);
        n[14 + slot] = u2f(count);
    };

    uint32_t root = alloc_dev();
    if (bn.empty() || bn[0].left < 0) {
        // Leaf root (few triangles): child 0 is the leaf, child 1 repeats its
        // box with no triangles (finite boxes only; the slab test has no
        // empty-box encoding). An empty scene keeps an all-zero root and is
        // never traversed.
        if (!bn.empty() && bn[0].count > 0) {
            int32_t link = emit_leaf(bn[0]);
            set_child(root, 0, bn[0].box, link, bn[0].count);
            set_child(root, 1, bn[0].box, link, 0);
        } else {
            Box point;  // empty scene: two empty leaves, never an inner link
            for (int a = 0; a < 3; ++a) point.lo[a] = point.hi[a] = 0.f;
            set_child(root, 0, point, ~0, 0);
            set_child(root, 1, point, ~0, 0);
        }
    } else {
        stack.push_back({0, root});
        while (!stack.empty()) {
            Item it = stack.back();
            stack.pop_back();
            const BNode& nd = bn[(size_t)it.build_node];
            const int32_t ch[2] = {nd.left, nd.right};
            // children that are inner nodes get device nodes; push right first
            // so the left subtree is laid out directly after its parent
            int32_t links[2];
            for (int s = 0; s < 2; ++s) {
                const BNode& c = bn[(size_t)ch[s]];
                if (c.left < 0) {
                    links[s] = emit_leaf(c);
                    set_child(it.dev_node, s, c.box, links[s], c.count);
                }
            }
            uint32_t dev_children[2] = {0, 0};
            for (int s = 0; s < 2; ++s) {
                const BNode& c = bn[(size_t)ch[s]];
                if (c.left >= 0) {
                    dev_children[s] = alloc_dev();
                    set_child(it.dev_node, s, c.box, (int32_t)dev_children[s], 0);
                }
            }
            for (int s = 1; s >= 0; --s) {
                const BNode& c = bn[(size_t)ch[s]];
                if (c.left >= 0) stack.push_back({ch[s], dev_children[s]});
            }
        }
    }
    out.n_nodes = (uint32_t)(out.nodes.size() / 16);
    out.depth = b.max_depth;
}

}  // namespace kz
