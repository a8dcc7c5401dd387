// Host-side structural check of the device BVH layout produced by
// kazen_proto_gb300/csrc/kz_bvh.cpp (compiled together by tests/test_bvh_layout.py).
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../kazen_proto_gb300/csrc/kz_bvh.h"

static float u2f(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
static uint32_t f2u(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }

extern "C" int kzt_check_layout(const float* tv, uint32_t ntris, char* msg, int msglen, uint32_t* out_nodes,
                                uint32_t* out_depth) {
    std::vector<uint32_t> geom(ntris);
    for (uint32_t i = 0; i < ntris; ++i) geom[i] = i % 3;
    std::vector<int32_t> gmat = {7, 8, 9};
    kz::BvhBuildInput in{tv, ntris, geom.data(), gmat.data()};
    kz::BvhBuildOutput out;
    kz::build_bvh(in, 4, out);
    *out_nodes = out.n_nodes;
    *out_depth = out.depth;
    auto bad = [&](const char* why, long a, long b) {
        std::snprintf(msg, msglen, "%s (%ld, %ld)", why, a, b);
        return 1;
    };
    if (out.n_nodes < 1 || out.nodes.size() != (size_t)out.n_nodes * 16) return bad("node array size", out.n_nodes, 0);
    if (out.tris.size() != (size_t)ntris * 12 || out.order.size() != ntris) return bad("record array size", 0, 0);
    if (out.depth > (uint32_t)kz::kMaxBvhDepth) return bad("depth", out.depth, 0);
    // records: a permutation of the input, carrying exact vertices and ids
    std::vector<int> seen(ntris, 0);
    for (uint32_t r = 0; r < ntris; ++r) {
        const float* rec = &out.tris[(size_t)r * 12];
        uint32_t t = f2u(rec[3]);
        if (t >= ntris || seen[t]++) return bad("record prim id", r, t);
        if (t != out.order[r]) return bad("order", r, t);
        for (int v = 0; v < 3; ++v)
            for (int a = 0; a < 3; ++a)
                if (f2u(rec[v * 4 + a]) != f2u(tv[(size_t)t * 9 + v * 3 + a])) return bad("vertex bits", r, v);
        if (f2u(rec[7]) != geom[t] || f2u(rec[11]) != (uint32_t)gmat[geom[t]]) return bad("geom/material", r, t);
    }
    // tree: every inner node reached exactly once from the root; leaves
    // partition the records; child boxes contain their triangles
    std::vector<int> visited(out.n_nodes, 0), covered(ntris, 0);
    struct It { uint32_t node; uint32_t depth; };
    std::vector<It> st = {{0, 1}};
    while (!st.empty()) {
        It it = st.back();
        st.pop_back();
        if (it.node >= out.n_nodes) return bad("inner link out of range", it.node, out.n_nodes);
        if (visited[it.node]++) return bad("inner node reached twice", it.node, 0);
        if (it.depth > 64) return bad("traversal depth", it.depth, 0);
        const float* n = &out.nodes[(size_t)it.node * 16];
        for (int s = 0; s < 2; ++s) {
            int32_t link = (int32_t)f2u(n[12 + s]);
            uint32_t cnt = f2u(n[14 + s]);
            float lo[3] = {n[s * 4 + 0], n[s * 4 + 2], n[8 + s * 2]};
            float hi[3] = {n[s * 4 + 1], n[s * 4 + 3], n[9 + s * 2]};
            if (link >= 0) {
                if (link == 0) return bad("link to root", it.node, s);
                if (cnt != 0) return bad("inner child with count", it.node, cnt);
                // box must contain the inner child's two boxes
                const float* c = &out.nodes[(size_t)link * 16];
                for (int cs = 0; cs < 2; ++cs) {
                    float clo[3] = {c[cs * 4 + 0], c[cs * 4 + 2], c[8 + cs * 2]};
                    float chi[3] = {c[cs * 4 + 1], c[cs * 4 + 3], c[9 + cs * 2]};
                    uint32_t ccnt = f2u(c[14 + cs]);
                    int32_t clink = (int32_t)f2u(c[12 + cs]);
                    if (clink < 0 && ccnt == 0) continue;
                    for (int a = 0; a < 3; ++a)
                        if (clo[a] < lo[a] || chi[a] > hi[a]) return bad("child box not contained", link, a);
                }
                st.push_back({(uint32_t)link, it.depth + 1});
            } else {
                uint32_t first = (uint32_t)(~link);
                if ((uint64_t)first + cnt > ntris) return bad("leaf range", first, cnt);
                for (uint32_t r = first; r < first + cnt; ++r) {
                    if (covered[r]++) return bad("record in two leaves", r, 0);
                    const float* rec = &out.tris[(size_t)r * 12];
                    for (int v = 0; v < 3; ++v)
                        for (int a = 0; a < 3; ++a)
                            if (rec[v * 4 + a] < lo[a] || rec[v * 4 + a] > hi[a]) return bad("leaf box", r, a);
                }
            }
        }
    }
    for (uint32_t i = 0; i < out.n_nodes; ++i)
        if (!visited[i]) return bad("unreachable inner node", i, 0);
    for (uint32_t r = 0; r < ntris; ++r)
        if (!covered[r]) return bad("record in no leaf", r, 0);
    (void)u2f;
    return 0;
}
