// kz_bvh.cpp — binned-SAH BVH build and device layout (see kz_bvh.h).
#include "kz_bvh.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <memory>
#include <stdexcept>
#include <utility>

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
            nodes[tk.node].first = tk.first;  // inner nodes keep their range too
            nodes[tk.node].count = tk.count;
            uint32_t mid = 0;
            bool split = tk.count > 1 && (int)tk.depth < kMaxBvhDepth - 1 && choose_split(tk.first, tk.count, bb, cb, mid);
            if (!split) continue;
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

inline uint32_t f2u(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}

void emit_tri(const BvhBuildInput& in, uint32_t t, std::vector<float>& tris, std::vector<uint32_t>& order) {
    const float* v = in.tri_verts + (size_t)t * 9;
    uint32_t geom = in.tri_geom ? in.tri_geom[t] : 0u;
    uint32_t mat = in.geom_material ? (uint32_t)in.geom_material[geom] : 0u;
    float r[12] = {v[0], v[1], v[2], u2f(t), v[3], v[4], v[5], u2f(geom), v[6], v[7], v[8], u2f(mat)};
    tris.insert(tris.end(), r, r + 12);
    order.push_back(t);
}

// A subtree of the binary build seen by the wide collapse: an inner build
// node (bnode >= 0) or a run of triangles idx[first, first + count).
struct WItem {
    int32_t bnode = -1;
    uint32_t first = 0, count = 0;
    Box box;
};

constexpr uint32_t kWideLeafMax = 3;

struct Collapser {
    Builder& b;
    explicit Collapser(Builder& bb) : b(bb) {}

    WItem item_of(int32_t id) const {
        const BNode& c = b.nodes[(size_t)id];
        WItem w;
        w.box = c.box;
        if (c.left >= 0) {
            w.bnode = id;
        } else {
            w.first = c.first;
            w.count = c.count;
        }
        return w;
    }
    static bool expandable(const WItem& w) { return w.bnode >= 0 || w.count > kWideLeafMax; }

    Box range_box(uint32_t first, uint32_t count) const {
        Box bx;
        for (uint32_t i = first; i < first + count; ++i) bx.grow(b.tb[b.idx[i]]);
        return bx;
    }

    void expand(const WItem& w, WItem& l, WItem& r) {
        if (w.bnode >= 0) {
            const BNode& n = b.nodes[(size_t)w.bnode];
            l = item_of(n.left);
            r = item_of(n.right);
            return;
        }
        // a leaf left larger than 3 triangles by the depth cap: halve it by
        // count along the widest centroid axis
        Box cb;
        for (uint32_t i = w.first; i < w.first + w.count; ++i) cb.grow(&b.cen[(size_t)b.idx[i] * 3]);
        int a = 0;
        for (int k = 1; k < 3; ++k)
            if (cb.hi[k] - cb.lo[k] > cb.hi[a] - cb.lo[a]) a = k;
        const uint32_t mid = w.first + w.count / 2;
        std::nth_element(b.idx.begin() + w.first, b.idx.begin() + mid, b.idx.begin() + w.first + w.count,
                         [&](uint32_t p, uint32_t q) {
                             float cp = b.cen[(size_t)p * 3 + a], cq = b.cen[(size_t)q * 3 + a];
                             return cp < cq || (cp == cq && p < q);
                         });
        l = WItem{-1, w.first, mid - w.first, range_box(w.first, mid - w.first)};
        r = WItem{-1, mid, w.first + w.count - mid, range_box(mid, w.first + w.count - mid)};
    }
};

// Leaves the depth cap left larger than kWideLeafMax become inner nodes,
// halved by count along the widest centroid axis until every leaf fits a
// wide slot. Children are appended after their parent, as in the build.
void split_big_leaves(Builder& b) {
    for (size_t id = 0; id < b.nodes.size(); ++id) {
        if (b.nodes[id].left >= 0 || b.nodes[id].count <= kWideLeafMax) continue;
        const uint32_t first = b.nodes[id].first, count = b.nodes[id].count;
        Box cb;
        for (uint32_t i = first; i < first + count; ++i) cb.grow(&b.cen[(size_t)b.idx[i] * 3]);
        int a = 0;
        for (int k = 1; k < 3; ++k)
            if (cb.hi[k] - cb.lo[k] > cb.hi[a] - cb.lo[a]) a = k;
        const uint32_t mid = first + count / 2;
        std::nth_element(b.idx.begin() + first, b.idx.begin() + mid, b.idx.begin() + first + count,
                         [&](uint32_t p, uint32_t q) {
                             float cp = b.cen[(size_t)p * 3 + a], cq = b.cen[(size_t)q * 3 + a];
                             return cp < cq || (cp == cq && p < q);
                         });
        const uint32_t rng[2][2] = {{first, mid - first}, {mid, first + count - mid}};
        int32_t kids[2];
        for (int c = 0; c < 2; ++c) {
            BNode n;
            n.first = rng[c][0];
            n.count = rng[c][1];
            for (uint32_t i = n.first; i < n.first + n.count; ++i) n.box.grow(b.tb[b.idx[i]]);
            kids[c] = (int32_t)b.nodes.size();
            b.nodes.push_back(n);
        }
        b.nodes[id].left = kids[0];
        b.nodes[id].right = kids[1];
    }
}

// SAH-optimal assignment of binary subtrees to the 8 slots of wide nodes
// (H. Ylitie, T. Karras, S. Laine, HPG 2017, section 4.1): cost(n, i) is the
// least SAH cost of covering subtree n with at most i slots, each a leaf of
// <= 3 triangles or a wide node; a wide node costs node_cost * area plus the
// best 8-slot distribution of its two children, a leaf tri_cost * area *
// triangles. Filled bottom-up (children follow parents in the node array).
struct SahCollapse {
    const Builder& b;
    float node_cost, tri_cost;
    std::vector<float> cost;        // [node][i - 1], i = 1..8
    std::vector<uint8_t> split;     // [node][i - 1]: k slots to the left child of the best distribution of i
    std::vector<uint8_t> from_prev; // [node][i - 1]: cost(n, i) == cost(n, i - 1)
    std::vector<uint8_t> as_leaf;   // cost(n, 1) is the leaf's

    SahCollapse(const Builder& bb, float cn, float ct) : b(bb), node_cost(cn), tri_cost(ct) {
        const size_t n = b.nodes.size();
        cost.assign(n * 8, 0.f);
        split.assign(n * 8, 0);
        from_prev.assign(n * 8, 0);
        as_leaf.assign(n, 0);
        const float inf = std::numeric_limits<float>::infinity();
        for (size_t id = n; id-- > 0;) {
            const BNode& nd = b.nodes[id];
            const float A = nd.box.area();
            const float leaf = nd.count <= kWideLeafMax ? tri_cost * A * (float)nd.count : inf;
            float* c = &cost[id * 8];
            if (nd.left < 0) {
                for (int i = 0; i < 8; ++i) c[i] = leaf;
                as_leaf[id] = 1;
                continue;
            }
            const float* cl = &cost[(size_t)nd.left * 8];
            const float* cr = &cost[(size_t)nd.right * 8];
            float dist[9];
            for (int j = 2; j <= 8; ++j) {
                dist[j] = inf;
                for (int k = 1; k < j; ++k) {
                    const float v = cl[k - 1] + cr[j - k - 1];
                    if (v < dist[j]) {
                        dist[j] = v;
                        split[id * 8 + j - 1] = (uint8_t)k;
                    }
                }
            }
            const float inner = dist[8] + node_cost * A;
            as_leaf[id] = leaf <= inner ? 1 : 0;
            c[0] = std::min(leaf, inner);
            for (int i = 2; i <= 8; ++i) {
                if (c[i - 2] <= dist[i]) {
                    c[i - 1] = c[i - 2];
                    from_prev[id * 8 + i - 1] = 1;
                } else {
                    c[i - 1] = dist[i];
                }
            }
        }
    }

    WItem slot_of(int32_t id) const {
        const BNode& nd = b.nodes[(size_t)id];
        WItem w;
        w.box = nd.box;
        if (as_leaf[(size_t)id]) {
            w.first = nd.first;
            w.count = nd.count;
        } else {
            w.bnode = id;
        }
        return w;
    }
    // Slots covering subtree id with at most i of them.
    void gather(int32_t id, int i, WItem* out, int& n) const {
        const BNode& nd = b.nodes[(size_t)id];
        while (i > 1 && from_prev[(size_t)id * 8 + i - 1]) --i;
        if (i == 1 || nd.left < 0) {
            out[n++] = slot_of(id);
            return;
        }
        const int k = split[(size_t)id * 8 + i - 1];
        gather(nd.left, k, out, n);
        gather(nd.right, i - k, out, n);
    }
    // The slots of the wide node made from inner build node id.
    int children(int32_t id, WItem* out) const {
        const BNode& nd = b.nodes[(size_t)id];
        const int k = split[(size_t)id * 8 + 7];
        int n = 0;
        gather(nd.left, k, out, n);
        gather(nd.right, 8 - k, out, n);
        return n;
    }
};

// Smallest power-of-two quantum q with 255 * q >= ext (>= 2^-100).
int quantum_exponent(double ext) {
    int e = -100;
    if (ext > 0.0) {
        e = std::max(-100, (int)std::ceil(std::log2(ext / 255.0)));
        while (std::ldexp(255.0, e) < ext) ++e;
        while (e > -100 && std::ldexp(255.0, e - 1) >= ext) --e;
    }
    if (e > 112) throw std::length_error("scene extent too large for the wide BVH");
    return e;
}

}  // namespace

void build_wide_bvh(const BvhBuildInput& in, WideBvhOutput& out, const WideBuildOptions& opt) {
    Builder b(in, opt.sah_collapse ? std::max(1, std::min(opt.binary_max_leaf, (int)kWideLeafMax)) : (int)kWideLeafMax);
    b.run();
    split_big_leaves(b);
    Collapser col(b);
    std::unique_ptr<SahCollapse> sah;
    if (opt.sah_collapse && !b.nodes.empty()) sah.reset(new SahCollapse(b, opt.node_cost, opt.tri_cost));
    out.nodes.assign(kWideWords, 0u);
    out.tris.clear();
    out.order.clear();
    out.tris.reserve((size_t)in.ntris * 12);
    out.order.reserve(in.ntris);
    out.depth = 1;

    WItem root;
    if (!b.nodes.empty()) root = sah ? sah->slot_of(0) : col.item_of(0);
    struct Pending {
        WItem item;
        uint32_t node, depth;
    };
    std::vector<Pending> queue{{root, 0u, 1u}};
    for (size_t head = 0; head < queue.size(); ++head) {
        const Pending pd = queue[head];
        out.depth = std::max(out.depth, pd.depth);
        WItem ch[8];
        int nch = 0;
        if (sah && pd.item.bnode >= 0) nch = sah->children(pd.item.bnode, ch);
        else ch[nch++] = pd.item;
        // greedy collapse: open the largest expandable child until 8 slots
        while (!sah && nch < 8) {
            int best = -1;
            float best_area = -1.f;
            for (int k = 0; k < nch; ++k)
                if (Collapser::expandable(ch[k]) && ch[k].box.area() > best_area) {
                    best = k;
                    best_area = ch[k].box.area();
                }
            if (best < 0) break;
            WItem l, r;
            col.expand(ch[best], l, r);
            ch[best] = l;
            ch[nch++] = r;
        }
        // drop empty runs (an empty scene only)
        int m = 0;
        for (int k = 0; k < nch; ++k)
            if (ch[k].bnode >= 0 || ch[k].count > 0) ch[m++] = ch[k];
        nch = m;

        uint32_t* w = &out.nodes[(size_t)pd.node * kWideWords];
        if (nch == 0) {  // empty scene: a node with no slots, never hit
            w[3] = 127u | 127u << 8 | 127u << 16;
            continue;
        }

        // slot assignment: child towards octant s of the node centre
        Box nb;
        for (int k = 0; k < nch; ++k) nb.grow(ch[k].box);
        float cen[8][3];
        for (int k = 0; k < nch; ++k)
            for (int a = 0; a < 3; ++a)
                cen[k][a] = 0.5f * (ch[k].box.lo[a] + ch[k].box.hi[a]) - 0.5f * (nb.lo[a] + nb.hi[a]);
        struct Cand { float score; int child, slot; };
        std::vector<Cand> cand;
        cand.reserve((size_t)nch * 8);
        for (int k = 0; k < nch; ++k)
            for (int sl = 0; sl < 8; ++sl) {
                float sc = 0.f;
                for (int a = 0; a < 3; ++a) sc += ((sl >> a) & 1) ? cen[k][a] : -cen[k][a];
                cand.push_back({sc, k, sl});
            }
        std::stable_sort(cand.begin(), cand.end(), [](const Cand& x, const Cand& y) { return x.score > y.score; });
        int slot_child[8];
        bool child_done[8] = {false};
        for (int sl = 0; sl < 8; ++sl) slot_child[sl] = -1;
        for (const Cand& c : cand)
            if (!child_done[c.child] && slot_child[c.slot] < 0) {
                slot_child[c.slot] = c.child;
                child_done[c.child] = true;
            }

        // quantization frame
        int ex[3];
        for (int a = 0; a < 3; ++a) {
            ex[a] = quantum_exponent((double)nb.hi[a] - (double)nb.lo[a]);
            w[a] = f2u(nb.lo[a]);
        }
        uint32_t imask = 0, meta[8] = {0};
        uint8_t qlo[3][8] = {{0}}, qhi[3][8] = {{0}};
        const uint32_t child_base = (uint32_t)(out.nodes.size() / kWideWords);
        const uint32_t tri_base = (uint32_t)out.order.size();
        uint32_t n_inner = 0, tri_off = 0;
        for (int sl = 0; sl < 8; ++sl) {
            const int k = slot_child[sl];
            if (k < 0) continue;
            const WItem& c = ch[k];
            for (int a = 0; a < 3; ++a) {
                const double q = std::ldexp(1.0, ex[a]);
                double lo = std::floor(((double)c.box.lo[a] - (double)nb.lo[a]) / q);
                double hi = std::ceil(((double)c.box.hi[a] - (double)nb.lo[a]) / q);
                qlo[a][sl] = (uint8_t)std::min(255.0, std::max(0.0, lo));
                qhi[a][sl] = (uint8_t)std::min(255.0, std::max(0.0, hi));
            }
            if (Collapser::expandable(c)) {
                imask |= 1u << sl;
                meta[sl] = 0x20u | (24u + (uint32_t)sl);
                out.nodes.resize(out.nodes.size() + kWideWords, 0u);
                queue.push_back({c, child_base + n_inner, pd.depth + 1});
                ++n_inner;
            } else {
                meta[sl] = (((1u << c.count) - 1u) << 5) | tri_off;
                for (uint32_t i = c.first; i < c.first + c.count; ++i) emit_tri(in, b.idx[i], out.tris, out.order);
                tri_off += c.count;
            }
        }
        w = &out.nodes[(size_t)pd.node * kWideWords];  // the resize above may move the array
        w[3] = (uint32_t)(ex[0] + 127) | (uint32_t)(ex[1] + 127) << 8 | (uint32_t)(ex[2] + 127) << 16 | imask << 24;
        w[4] = child_base;
        w[5] = tri_base;
        for (int sl = 0; sl < 8; ++sl) w[6 + sl / 4] |= meta[sl] << (8 * (sl % 4));
        for (int a = 0; a < 3; ++a)
            for (int sl = 0; sl < 8; ++sl) {
                w[8 + 4 * a + sl / 4] |= (uint32_t)qlo[a][sl] << (8 * (sl % 4));
                w[10 + 4 * a + sl / 4] |= (uint32_t)qhi[a][sl] << (8 * (sl % 4));
            }
    }
    out.n_nodes = (uint32_t)(out.nodes.size() / kWideWords);
    if (out.depth > (uint32_t)kWideDepthCap) throw std::length_error("wide BVH deeper than the traversal stack");
}

}  // namespace kz
