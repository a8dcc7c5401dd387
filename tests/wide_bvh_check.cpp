// Host-side checks of the 8-wide BVH produced by
// kazen_proto_gb300/csrc/kz_bvh.cpp (compiled together by tests/test_bvh_layout.py):
//  * kzt_check_wide: structure (every node reached once, slot encodings,
//    leaves partition the triangle records, every triangle of a slot's
//    subtree inside the slot's dequantized box, depth within the stack);
//  * kzt_wide_trace: a float emulation of the device traversal
//    (kz_traverse.cuh: wide_axis / wide_slot / wide_pop_child, same operation
//    order, built with -ffp-contract=off) against a brute-force loop over all
//    triangles with the same watertight test: closest triangle id and t bits
//    must agree for every ray.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../kazen_proto_gb300/csrc/kz_bvh.h"

namespace {

float u2f(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
uint32_t f2u(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }

struct Built {
    std::vector<uint32_t> geom;
    std::vector<int32_t> gmat{7, 8, 9};
    kz::WideBvhOutput out;
};

void build(const float* tv, uint32_t ntris, Built& b) {
    b.geom.resize(ntris);
    for (uint32_t i = 0; i < ntris; ++i) b.geom[i] = i % 3;
    kz::BvhBuildInput in{tv, ntris, b.geom.data(), b.gmat.data()};
    kz::build_wide_bvh(in, b.out);
}

uint32_t byte_of(uint32_t w, int j) { return (w >> (8 * j)) & 0xFFu; }

// dequantized slot box, exact in double
void slot_box(const uint32_t* w, int s, double lo[3], double hi[3]) {
    for (int a = 0; a < 3; ++a) {
        const double p = (double)u2f(w[a]);
        const int e = (int)((w[3] >> (8 * a)) & 0xFFu) - 127;
        const double q = std::ldexp(1.0, e);
        lo[a] = p + q * (double)byte_of(w[8 + 4 * a + s / 4], s % 4);
        hi[a] = p + q * (double)byte_of(w[10 + 4 * a + s / 4], s % 4);
    }
}

struct Checker {
    const float* tv;
    uint32_t ntris;
    const kz::WideBvhOutput& o;
    std::vector<int> visited, covered;
    char* msg;
    int msglen;
    bool failed = false;

    bool bad(const char* why, long a, long b) {
        if (!failed) std::snprintf(msg, msglen, "%s (%ld, %ld)", why, a, b);
        failed = true;
        return false;
    }

    // Appends the records of node's subtree to recs; checks the node.
    bool walk(uint32_t node, uint32_t depth, std::vector<uint32_t>& recs) {
        if (node >= o.n_nodes) return bad("node index out of range", node, o.n_nodes);
        if (visited[node]++) return bad("node reached twice", node, 0);
        if (depth > (uint32_t)kz::kWideStack) return bad("depth", depth, 0);
        const uint32_t* w = &o.nodes[(size_t)node * kz::kWideWords];
        const uint32_t imask = w[3] >> 24, child_base = w[4], tri_base = w[5];
        for (int a = 0; a < 3; ++a) {
            const int e = (int)((w[3] >> (8 * a)) & 0xFFu);
            if (e < 27 || e > 239) return bad("quantum exponent", node, e);
        }
        uint32_t n_inner = 0, tri_used = 0;
        for (int s = 0; s < 8; ++s) {
            const uint32_t m = byte_of(w[6 + s / 4], s % 4);
            const bool inner = (imask >> s) & 1u;
            std::vector<uint32_t> sub;
            if (inner) {
                if (m != 0x20u + 24u + (uint32_t)s) return bad("inner meta", node, s);
                if (!walk(child_base + n_inner, depth + 1, sub)) return false;
                ++n_inner;
            } else if (m != 0) {
                const uint32_t cnt_bits = m >> 5, off = m & 31u;
                if (cnt_bits != 1 && cnt_bits != 3 && cnt_bits != 7) return bad("leaf count bits", node, s);
                if (off > 23u || (cnt_bits << off) > 0x00FFFFFFu) return bad("leaf offset", node, s);
                if (tri_used & (cnt_bits << off)) return bad("leaf triangles overlap", node, s);
                tri_used |= cnt_bits << off;
                for (uint32_t k = 0; k < 3; ++k)
                    if ((cnt_bits >> k) & 1u) {
                        const uint32_t r = tri_base + off + k;
                        if (r >= ntris) return bad("record out of range", node, r);
                        if (covered[r]++) return bad("record in two leaves", r, 0);
                        sub.push_back(r);
                    }
            } else {
                continue;
            }
            double lo[3], hi[3];
            slot_box(w, s, lo, hi);
            for (uint32_t r : sub) {
                const float* rec = &o.tris[(size_t)r * 12];
                for (int v = 0; v < 3; ++v)
                    for (int a = 0; a < 3; ++a)
                        if ((double)rec[v * 4 + a] < lo[a] || (double)rec[v * 4 + a] > hi[a])
                            return bad("triangle outside slot box", node, s);
            }
            recs.insert(recs.end(), sub.begin(), sub.end());
        }
        if (tri_used && (tri_used & (tri_used + 1u))) return bad("leaf triangles not contiguous", node, tri_used);
        return true;
    }
};

// ---- float emulation of the device traversal ------------------------------

struct TRay {
    float o[3], inv[3], tmin;
    int kx, ky, kz;
    float Sx, Sy, Sz;
};

float safe_inv(float c) {
    if (std::fabs(c) < 1e-30f) c = std::copysign(1e-30f, c);
    return 1.0f / c;
}

TRay make_tray(const float* o, const float* d, float tmin) {
    TRay r;
    for (int a = 0; a < 3; ++a) {
        r.o[a] = o[a];
        r.inv[a] = safe_inv(d[a]);
    }
    r.tmin = tmin;
    float ax = std::fabs(d[0]), ay = std::fabs(d[1]), az = std::fabs(d[2]);
    int kz = 0;
    float m = ax;
    if (ay > m) { kz = 1; m = ay; }
    if (az > m) kz = 2;
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    if (d[kz] < 0.f) std::swap(kx, ky);
    r.kx = kx; r.ky = ky; r.kz = kz;
    r.Sx = d[kx] / d[kz];
    r.Sy = d[ky] / d[kz];
    r.Sz = 1.0f / d[kz];
    return r;
}

bool tri_test(const TRay& r, const float* a, const float* b, const float* c, float& t) {
    const float okx = r.o[r.kx], oky = r.o[r.ky], okz = r.o[r.kz];
    const float Akx = a[r.kx] - okx, Aky = a[r.ky] - oky, Akz = a[r.kz] - okz;
    const float Bkx = b[r.kx] - okx, Bky = b[r.ky] - oky, Bkz = b[r.kz] - okz;
    const float Ckx = c[r.kx] - okx, Cky = c[r.ky] - oky, Ckz = c[r.kz] - okz;
    const float Ax = Akx - r.Sx * Akz, Ay = Aky - r.Sy * Akz;
    const float Bx = Bkx - r.Sx * Bkz, By = Bky - r.Sy * Bkz;
    const float Cx = Ckx - r.Sx * Ckz, Cy = Cky - r.Sy * Ckz;
    float U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
    if (U == 0.f || V == 0.f || W == 0.f) {
        U = (float)((double)Cx * By - (double)Cy * Bx);
        V = (float)((double)Ax * Cy - (double)Ay * Cx);
        W = (float)((double)Bx * Ay - (double)By * Ax);
    }
    if ((U < 0.f || V < 0.f || W < 0.f) && (U > 0.f || V > 0.f || W > 0.f)) return false;
    const float det = U + V + W;
    if (det == 0.f) return false;
    const float T = U * (r.Sz * Akz) + V * (r.Sz * Bkz) + W * (r.Sz * Ckz);
    t = T / det;
    return true;
}

struct Axis { float A, Bn, Bf; uint32_t n0, n1, f0, f1; };

Axis wide_axis(float p, uint32_t e, float o, float inv, const uint32_t* q) {
    Axis ax;
    ax.A = u2f((e + 15u) << 23) * inv;
    const float b = (p - o) * inv;
    const float B = b - ax.A;
    const float d = (std::fabs(b) + std::fabs(ax.A) * 0.03125f) * 1.52587890625e-05f;
    ax.Bn = B - d;
    ax.Bf = B + d;
    const bool neg = inv < 0.f;
    ax.n0 = neg ? q[2] : q[0];
    ax.n1 = neg ? q[3] : q[1];
    ax.f0 = neg ? q[0] : q[2];
    ax.f1 = neg ? q[1] : q[3];
    return ax;
}

float wide_t(const Axis& ax, int s, bool near_plane) {
    const uint32_t w = near_plane ? (s < 4 ? ax.n0 : ax.n1) : (s < 4 ? ax.f0 : ax.f1);
    const float f = u2f(0x3F800000u | (byte_of(w, s & 3) << 8));  // the device's byte permute
    return std::fma(f, ax.A, near_plane ? ax.Bn : ax.Bf);
}

uint32_t wide_node(const uint32_t* w, const TRay& r, uint32_t octp, float tcur, uint32_t& child_base,
                   uint32_t& tri_base, uint32_t& imask) {
    child_base = w[4];
    tri_base = w[5];
    imask = w[3] >> 24;
    Axis ax[3];
    for (int a = 0; a < 3; ++a) ax[a] = wide_axis(u2f(w[a]), (w[3] >> (8 * a)) & 0xFFu, r.o[a], r.inv[a], w + 8 + 4 * a);
    uint32_t mw[2] = {w[6], w[7]};
    for (auto& m : mw) m ^= ((m >> 4) & (m >> 3) & 0x01010101u) * octp;
    uint32_t hits = 0;
    for (int s = 0; s < 8; ++s) {
        const float tn = std::fmax(std::fmax(std::fmax(wide_t(ax[0], s, true), wide_t(ax[1], s, true)), wide_t(ax[2], s, true)), r.tmin);
        const float tf = std::fmin(std::fmin(std::fmin(wide_t(ax[0], s, false), wide_t(ax[1], s, false)), wide_t(ax[2], s, false)), tcur);
        const uint32_t m = byte_of(mw[s / 4], s & 3);
        if (tn <= tf) hits |= (m >> 5) << (m & 31u);
    }
    return hits;
}

bool wide_closest(const kz::WideBvhOutput& o, const TRay& r, float tmax, float& best_t, uint32_t& best_prim,
                  uint32_t& visits) {
    best_t = tmax;
    best_prim = 0xFFFFFFFFu;
    const uint32_t octp = 7u ^ ((r.inv[0] < 0.f ? 1u : 0u) | (r.inv[1] < 0.f ? 2u : 0u) | (r.inv[2] < 0.f ? 4u : 0u));
    std::vector<std::pair<uint32_t, uint32_t>> stack;
    uint32_t gbase = 0, gbits = 0x80000000u;
    visits = 0;
    for (;;) {
        const uint32_t pos = 31u - (uint32_t)__builtin_clz(gbits);
        gbits ^= 1u << pos;
        const uint32_t slot = (pos - 24u) ^ octp;
        const uint32_t node = gbase + (uint32_t)__builtin_popcount(gbits & ((1u << slot) - 1u));
        if (gbits > 0x00FFFFFFu) {
            if (stack.size() >= (size_t)kz::kWideStack) return false;
            stack.push_back({gbase, gbits});
        }
        if (++visits > o.n_nodes || node >= o.n_nodes) return false;
        uint32_t tri_base, imask;
        const uint32_t hm = wide_node(&o.nodes[(size_t)node * kz::kWideWords], r, octp, best_t, gbase, tri_base, imask);
        gbits = (hm & 0xFF000000u) | imask;
        for (uint32_t tb = hm & 0x00FFFFFFu; tb; tb &= tb - 1u) {
            const uint32_t rec = tri_base + (uint32_t)__builtin_ctz(tb);
            const float* q = &o.tris[(size_t)rec * 12];
            float t;
            if (!tri_test(r, q, q + 4, q + 8, t)) continue;
            const uint32_t prim = f2u(q[3]);
            if (t > r.tmin && (t < best_t || (t == best_t && prim < best_prim))) {
                best_t = t;
                best_prim = prim;
            }
        }
        while (gbits <= 0x00FFFFFFu && !stack.empty()) {
            gbase = stack.back().first;
            gbits = stack.back().second;
            stack.pop_back();
        }
        if (gbits <= 0x00FFFFFFu) return true;
    }
}

}  // namespace

extern "C" int kzt_check_wide(const float* tv, uint32_t ntris, char* msg, int msglen, uint32_t* out_nodes,
                              uint32_t* out_depth) {
    Built b;
    build(tv, ntris, b);
    const kz::WideBvhOutput& o = b.out;
    *out_nodes = o.n_nodes;
    *out_depth = o.depth;
    Checker c{tv, ntris, o, std::vector<int>(o.n_nodes, 0), std::vector<int>(ntris, 0), msg, msglen};
    if (o.n_nodes < 1 || o.nodes.size() != (size_t)o.n_nodes * kz::kWideWords) return c.bad("node array size", o.n_nodes, 0), 1;
    if (o.tris.size() != (size_t)ntris * 12 || o.order.size() != ntris) return c.bad("record array size", 0, 0), 1;
    std::vector<int> seen(ntris, 0);
    for (uint32_t r = 0; r < ntris; ++r) {
        const float* rec = &o.tris[(size_t)r * 12];
        const uint32_t t = f2u(rec[3]);
        if (t >= ntris || seen[t]++) return c.bad("record prim id", r, t), 1;
        if (t != o.order[r]) return c.bad("order", r, t), 1;
        for (int v = 0; v < 3; ++v)
            for (int a = 0; a < 3; ++a)
                if (f2u(rec[v * 4 + a]) != f2u(tv[(size_t)t * 9 + v * 3 + a])) return c.bad("vertex bits", r, v), 1;
        if (f2u(rec[7]) != b.geom[t] || f2u(rec[11]) != (uint32_t)b.gmat[b.geom[t]]) return c.bad("geom/material", r, t), 1;
    }
    std::vector<uint32_t> all;
    if (!c.walk(0, 1, all)) return 1;
    for (uint32_t i = 0; i < o.n_nodes; ++i)
        if (!c.visited[i]) return c.bad("unreachable node", i, 0), 1;
    for (uint32_t r = 0; r < ntris; ++r)
        if (!c.covered[r]) return c.bad("record in no leaf", r, 0), 1;
    return 0;
}

// rays: n * 8 floats (o.xyz, tmin, d.xyz, tmax). Returns the number of rays
// whose emulated traversal disagrees with the brute-force closest hit (or
// that aborted); mean node visits in *out_visits.
extern "C" int64_t kzt_wide_trace(const float* tv, uint32_t ntris, const float* rays, uint32_t n, double* out_visits,
                                  uint32_t* out_hits) {
    Built b;
    build(tv, ntris, b);
    int64_t bad = 0;
    double visits = 0;
    uint32_t hits = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const float* ry = rays + (size_t)i * 8;
        const TRay r = make_tray(ry, ry + 4, ry[3]);
        float bt = ry[7];
        uint32_t bp = 0xFFFFFFFFu;
        for (uint32_t t = 0; t < ntris; ++t) {
            const float* v = tv + (size_t)t * 9;
            float th;
            if (tri_test(r, v, v + 3, v + 6, th) && th > r.tmin && (th < bt || (th == bt && t < bp))) {
                bt = th;
                bp = t;
            }
        }
        float wt;
        uint32_t wp, vis;
        const bool ok = wide_closest(b.out, r, ry[7], wt, wp, vis);
        visits += vis;
        if (bp != 0xFFFFFFFFu) ++hits;
        if (!ok || wp != bp || (bp != 0xFFFFFFFFu && f2u(wt) != f2u(bt))) ++bad;
    }
    *out_visits = n ? visits / n : 0.0;
    *out_hits = hits;
    return bad;
}
