// kz_oracle.cpp — CPU restatement of the kazen_proto rendering hot path.
//
// TEST INFRASTRUCTURE ONLY. This library is the parity checker for the CUDA
// path in kazen_proto_gb300/ and the timed CPU baseline of bench.py. Nothing
// in the product links, loads or calls it.
//
// Parity status: the reference (kazen_proto) cannot be compiled here — its
// hot path depends on Embree 4, OSL, boost and pcg32, none of which are
// present — so this restatement is pinned against the reference's own
// known-answer tests (microfacet white-furnace integrals,
// tests/render_tests/microfacet_tests.cpp:8-21; the Embree single-triangle
// hit, tests/libusage_tests/embree_tests.cpp:19-76) and against analytic
// identities in tests/. Formula-level parity with the reference binary is
// otherwise unpinned.
//
// Written independently of the product's device code: its own BVH (object
// median split), its own traversal, its own closure code. Compile with
// -ffp-contract=off so FP32 expressions round exactly as written.
//
// Reference files restated (paths within kazen_proto):
//   ray epsilon ............ src/core/ray.h:10-45, src/base/basic_types.h:9
//   shading frame .......... src/base/utils.h:83-210
//   closures ............... src/shading/bsdfs.cpp:27-223, 254-319, 359-554, 563-780
//                            src/shading/microfacet.cpp:3-38 (Beckmann pdf, Walter G1)
//   glass helpers .......... src/shading/bsdfs.h:541-599
//   microfacet ............. src/shading/microfacet.h:60-291
//   fresnel ................ src/shading/fresnel.h:12-187, src/base/utils.h:153-177
//   mixture ................ src/shading/bsdf.h:132-196, src/shading/bsdf.cpp:17-74
//   lights ................. src/core/light.cpp:46-86, src/core/shape.cpp:591-613,
//                            src/base/dpdf.h:8-58, src/core/integrator.cpp:25-34
//   path loop .............. src/core/integrator.cpp:362-561
//   camera ................. src/core/camera.h:50-96, src/core/camera.cpp:5-37
//   furnace tests .......... src/shading/white_furnace.h:12-38, white_furnace.cpp:3-36
// Ray/triangle: the watertight test of Woop, Benthin & Wald, "Watertight
// Ray/Triangle Intersection", JCGT 2(1), 2013, double-sided, closest hit in
// (tmin, tmax], equal t resolved to the smaller triangle index.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

#include "../include/kazen_gb300.h"

namespace {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kInvPi = 0.318309886183790671538f;
constexpr float kRayEps = 1e-4f;  // epsilon<float>, src/base/basic_types.h:9

struct V3 {
    float x, y, z;
    V3() : x(0), y(0), z(0) {}
    V3(float a, float b, float c) : x(a), y(b), z(c) {}
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
inline V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline V3 mul(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline V3 normalize(V3 a) {
    float l = std::sqrt(dot(a, a));
    return {a.x / l, a.y / l, a.z / l};
}
// base::Vec::normalized(), src/base/vec.h:784-790: reciprocal length in
// double, rounded once to float
inline V3 normalize_ref(V3 a) {
    const float rcp = (float)(1.0 / std::sqrt((double)dot(a, a)));
    return {a.x * rcp, a.y * rcp, a.z * rcp};
}
template <bool kRefNorm>
inline V3 nrm(V3 a) {
    return kRefNorm ? normalize_ref(a) : normalize(a);
}
inline float sq(float a) { return a * a; }
inline bool is_zero(V3 a) { return a.x == 0.f && a.y == 0.f && a.z == 0.f; }
inline float max_comp(V3 a) { return std::max(a.x, std::max(a.y, a.z)); }

// ---------------------------------------------------------------- PCG32
// PCG-XSH-RR 64/32 (O'Neill 2014), seeded like pcg32_srandom(initstate, initseq).
struct Pcg32 {
    uint64_t state, inc;
    void seed(uint64_t initstate, uint64_t initseq) {
        state = 0u;
        inc = (initseq << 1u) | 1u;
        next();
        state += initstate;
        next();
    }
    uint32_t next() {
        uint64_t old = state;
        state = old * 6364136223846793005ULL + inc;
        uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = (uint32_t)(old >> 59u);
        return (xorshifted >> rot) | (xorshifted << ((32u - rot) & 31u));
    }
    // pcg32::nextFloat (Jakob's pcg32.h, used by Sampler, src/core/sampler.cpp:22-27):
    // 23 random mantissa bits in [1, 2), minus 1.
    float nextf() {
        uint32_t u = (next() >> 9) | 0x3f800000u;
        float f;
        std::memcpy(&f, &u, 4);
        return f - 1.0f;
    }
};

// ---------------------------------------------------------------- triangle test
struct RayPre {
    V3 o, d;
    int kx, ky, kz;
    float Sx, Sy, Sz;
};

inline RayPre ray_pre(V3 o, V3 d) {
    RayPre r;
    r.o = o;
    r.d = d;
    float ad[3] = {std::fabs(d.x), std::fabs(d.y), std::fabs(d.z)};
    int kz = 0;
    if (ad[1] > ad[kz]) kz = 1;
    if (ad[2] > ad[kz]) kz = 2;
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    if (d[kz] < 0.f) std::swap(kx, ky);
    r.kx = kx; r.ky = ky; r.kz = kz;
    r.Sx = d[kx] / d[kz];
    r.Sy = d[ky] / d[kz];
    r.Sz = 1.0f / d[kz];
    return r;
}

// Returns true with (t, u, v) when the triangle is hit at t in (tmin, +inf).
inline bool tri_hit(const RayPre& r, V3 v0, V3 v1, V3 v2, float& t, float& bu, float& bv) {
    const V3 A = v0 - r.o, B = v1 - r.o, C = v2 - r.o;
    const float Ax = A[r.kx] - r.Sx * A[r.kz];
    const float Ay = A[r.ky] - r.Sy * A[r.kz];
    const float Bx = B[r.kx] - r.Sx * B[r.kz];
    const float By = B[r.ky] - r.Sy * B[r.kz];
    const float Cx = C[r.kx] - r.Sx * C[r.kz];
    const float Cy = C[r.ky] - r.Sy * C[r.kz];
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.f || V == 0.f || W == 0.f) {
        U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
        V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
        W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
    }
    if ((U < 0.f || V < 0.f || W < 0.f) && (U > 0.f || V > 0.f || W > 0.f)) return false;
    const float det = U + V + W;
    if (det == 0.f) return false;
    const float Az = r.Sz * A[r.kz];
    const float Bz = r.Sz * B[r.kz];
    const float Cz = r.Sz * C[r.kz];
    const float T = U * Az + V * Bz + W * Cz;
    t = T / det;
    bu = V / det;
    bv = W / det;
    return true;
}

// ---------------------------------------------------------------- oracle BVH
// Binary BVH: binned SAH (16 bins on the largest centroid axis), leaves of at
// most 4 triangles, object median when the bins cannot separate; traversal
// visits the nearer child first and skips stacked nodes whose entry distance
// is beyond the current closest hit. Written independently of the product's
// builder and traversal.
struct OBox {
    float lo[3], hi[3];
};
struct ONode {
    OBox box;
    int32_t left, right;     // children (internal) or -1
    uint32_t first, count;   // leaf triangle range in `order`
};

struct OBvh {
    std::vector<float> verts;  // ntris * 9, world space
    uint32_t ntris = 0;
    std::vector<ONode> nodes;
    std::vector<uint32_t> order;

    V3 v(uint32_t tri, int k) const {
        const float* p = &verts[(size_t)tri * 9 + k * 3];
        return {p[0], p[1], p[2]};
    }

    static float half_area(const OBox& b) {
        if (b.lo[0] > b.hi[0]) return 0.f;
        float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
        return dx * dy + dy * dz + dz * dx;
    }
    static OBox empty_box() {
        OBox b;
        for (int a = 0; a < 3; ++a) {
            b.lo[a] = std::numeric_limits<float>::infinity();
            b.hi[a] = -std::numeric_limits<float>::infinity();
        }
        return b;
    }
    static void grow(OBox& b, const OBox& c) {
        for (int a = 0; a < 3; ++a) {
            b.lo[a] = std::min(b.lo[a], c.lo[a]);
            b.hi[a] = std::max(b.hi[a], c.hi[a]);
        }
    }

    void build() {
        order.resize(ntris);
        for (uint32_t i = 0; i < ntris; ++i) order[i] = i;
        std::vector<float> cen((size_t)ntris * 3);
        std::vector<OBox> tb(ntris);
        for (uint32_t i = 0; i < ntris; ++i) {
            OBox b = empty_box();
            for (int k = 0; k < 3; ++k)
                for (int a = 0; a < 3; ++a) {
                    b.lo[a] = std::min(b.lo[a], v(i, k)[a]);
                    b.hi[a] = std::max(b.hi[a], v(i, k)[a]);
                }
            tb[i] = b;
            for (int a = 0; a < 3; ++a) cen[(size_t)i * 3 + a] = (v(i, 0)[a] + v(i, 1)[a] + v(i, 2)[a]) * (1.0f / 3.0f);
        }
        nodes.clear();
        nodes.reserve(ntris ? ntris : 1);
        struct Task { uint32_t node, first, count; };
        std::vector<Task> stack;
        nodes.push_back(ONode{});
        stack.push_back({0, 0, ntris});
        constexpr int kB = 16;
        while (!stack.empty()) {
            Task tk = stack.back();
            stack.pop_back();
            OBox b = empty_box(), cb = empty_box();
            for (uint32_t i = tk.first; i < tk.first + tk.count; ++i) {
                uint32_t tri = order[i];
                grow(b, tb[tri]);
                for (int a = 0; a < 3; ++a) {
                    float c = cen[(size_t)tri * 3 + a];
                    cb.lo[a] = std::min(cb.lo[a], c);
                    cb.hi[a] = std::max(cb.hi[a], c);
                }
            }
            nodes[tk.node].box = b;
            if (tk.count <= 4) {
                nodes[tk.node].left = nodes[tk.node].right = -1;
                nodes[tk.node].first = tk.first;
                nodes[tk.node].count = tk.count;
                continue;
            }
            int axis = 0;
            for (int a = 1; a < 3; ++a)
                if (cb.hi[a] - cb.lo[a] > cb.hi[axis] - cb.lo[axis]) axis = a;
            const float ext = cb.hi[axis] - cb.lo[axis];
            uint32_t mid = tk.first + tk.count / 2;
            bool done = false;
            if (ext > 0.f) {
                OBox bins[kB];
                uint32_t cnt[kB] = {0};
                for (int k = 0; k < kB; ++k) bins[k] = empty_box();
                const float sc = (float)kB / ext;
                auto bin_of = [&](uint32_t tri) {
                    int k = (int)((cen[(size_t)tri * 3 + axis] - cb.lo[axis]) * sc);
                    return std::min(std::max(k, 0), kB - 1);
                };
                for (uint32_t i = tk.first; i < tk.first + tk.count; ++i) {
                    int k = bin_of(order[i]);
                    cnt[k]++;
                    grow(bins[k], tb[order[i]]);
                }
                float best = std::numeric_limits<float>::infinity();
                int best_k = -1;
                for (int k = 0; k < kB - 1; ++k) {
                    OBox l = empty_box(), r = empty_box();
                    uint32_t nl = 0, nr = 0;
                    for (int j = 0; j <= k; ++j) { grow(l, bins[j]); nl += cnt[j]; }
                    for (int j = k + 1; j < kB; ++j) { grow(r, bins[j]); nr += cnt[j]; }
                    if (!nl || !nr) continue;
                    float c = half_area(l) * nl + half_area(r) * nr;
                    if (c < best) { best = c; best_k = k; }
                }
                if (best_k >= 0) {
                    auto it = std::partition(order.begin() + tk.first, order.begin() + tk.first + tk.count,
                                             [&](uint32_t t) { return bin_of(t) <= best_k; });
                    mid = (uint32_t)(it - order.begin());
                    done = mid > tk.first && mid < tk.first + tk.count;
                }
            }
            if (!done) {
                mid = tk.first + tk.count / 2;
                std::nth_element(order.begin() + tk.first, order.begin() + mid,
                                 order.begin() + tk.first + tk.count, [&](uint32_t p, uint32_t q) {
                                     float cp = cen[(size_t)p * 3 + axis], cq = cen[(size_t)q * 3 + axis];
                                     return cp < cq || (cp == cq && p < q);
                                 });
            }
            int32_t l = (int32_t)nodes.size();
            nodes.push_back(ONode{});
            int32_t r = (int32_t)nodes.size();
            nodes.push_back(ONode{});
            nodes[tk.node].left = l;
            nodes[tk.node].right = r;
            nodes[tk.node].first = nodes[tk.node].count = 0;
            stack.push_back({(uint32_t)l, tk.first, mid - tk.first});
            stack.push_back({(uint32_t)r, mid, tk.first + tk.count - mid});
        }
    }

    // Conservative slab test: box distances are widened by a relative margin
    // far larger than their rounding error, so a box that holds a triangle hit
    // at t <= tbest is never culled.
    static bool box_hit(const OBox& b, const V3& o, const V3& inv, float tmin, float tbest, float& tnear) {
        float t0 = -std::numeric_limits<float>::infinity(), t1 = std::numeric_limits<float>::infinity();
        for (int a = 0; a < 3; ++a) {
            float ta = (b.lo[a] - o[a]) * inv[a];
            float tb = (b.hi[a] - o[a]) * inv[a];
            if (ta > tb) std::swap(ta, tb);
            t0 = std::max(t0, ta);
            t1 = std::min(t1, tb);
        }
        t0 = t0 > 0.f ? t0 * (1.0f - 1e-4f) : t0 * (1.0f + 1e-4f);
        t1 = t1 > 0.f ? t1 * (1.0f + 1e-4f) : t1 * (1.0f - 1e-4f);
        tnear = std::max(t0, tmin);
        return tnear <= std::min(t1, tbest);
    }

    static V3 inv_dir(V3 d) {
        auto f = [](float c) {
            if (std::fabs(c) < 1e-30f) c = std::copysign(1e-30f, c);
            return 1.0f / c;
        };
        return {f(d.x), f(d.y), f(d.z)};
    }

    // Closest hit in (tmin, tmax]; ties in t go to the smaller triangle index.
    bool closest(V3 o, V3 d, float tmin, float tmax, float& t_out, uint32_t& prim, float& u_out, float& v_out) const {
        prim = KZ_INVALID_ID;
        t_out = tmax;
        if (ntris == 0) return false;
        RayPre rp = ray_pre(o, d);
        V3 inv = inv_dir(d);
        uint32_t stack[128];
        float stack_t[128];
        int sp = 0;
        float tn;
        if (!box_hit(nodes[0].box, o, inv, tmin, t_out, tn)) return false;
        stack[sp] = 0;
        stack_t[sp++] = tn;
        while (sp) {
            --sp;
            if (stack_t[sp] > t_out) continue;
            const ONode& nd = nodes[stack[sp]];
            if (nd.left < 0) {
                for (uint32_t i = nd.first; i < nd.first + nd.count; ++i) {
                    uint32_t tri = order[i];
                    float t, bu, bv;
                    if (!tri_hit(rp, v(tri, 0), v(tri, 1), v(tri, 2), t, bu, bv)) continue;
                    if (!(t > tmin) || !(t <= tmax)) continue;
                    if (t < t_out || (t == t_out && tri < prim)) {
                        t_out = t; prim = tri; u_out = bu; v_out = bv;
                    }
                }
                continue;
            }
            float tl, tr;
            bool hl = box_hit(nodes[nd.left].box, o, inv, tmin, t_out, tl);
            bool hr = box_hit(nodes[nd.right].box, o, inv, tmin, t_out, tr);
            if (hl && hr) {
                if (tl <= tr) {
                    stack[sp] = nd.right; stack_t[sp++] = tr;
                    stack[sp] = nd.left; stack_t[sp++] = tl;
                } else {
                    stack[sp] = nd.left; stack_t[sp++] = tl;
                    stack[sp] = nd.right; stack_t[sp++] = tr;
                }
            } else if (hl) {
                stack[sp] = nd.left; stack_t[sp++] = tl;
            } else if (hr) {
                stack[sp] = nd.right; stack_t[sp++] = tr;
            }
        }
        return prim != KZ_INVALID_ID;
    }

    bool any(V3 o, V3 d, float tmin, float tmax) const {
        if (ntris == 0) return false;
        RayPre rp = ray_pre(o, d);
        V3 inv = inv_dir(d);
        uint32_t stack[128];
        int sp = 0;
        stack[sp++] = 0;
        while (sp) {
            const ONode& nd = nodes[stack[--sp]];
            float tn;
            if (!box_hit(nd.box, o, inv, tmin, tmax, tn)) continue;
            if (nd.left < 0) {
                for (uint32_t i = nd.first; i < nd.first + nd.count; ++i) {
                    uint32_t tri = order[i];
                    float t, bu, bv;
                    if (!tri_hit(rp, v(tri, 0), v(tri, 1), v(tri, 2), t, bu, bv)) continue;
                    if (t > tmin && t <= tmax) return true;
                }
            } else {
                stack[sp++] = (uint32_t)nd.right;
                stack[sp++] = (uint32_t)nd.left;
            }
        }
        return false;
    }
};

template <typename F>
void parallel_for(uint64_t n, int nthreads, F&& fn) {
    if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
    if (n < 2 || nthreads == 1) {
        for (uint64_t i = 0; i < n; ++i) fn(i);
        return;
    }
    std::atomic<uint64_t> next{0};
    const uint64_t chunk = std::max<uint64_t>(1, std::min<uint64_t>(256, n / (8 * (uint64_t)nthreads)));
    std::vector<std::thread> th;
    for (int k = 0; k < nthreads; ++k)
        th.emplace_back([&]() {
            for (;;) {
                uint64_t b = next.fetch_add(chunk);
                if (b >= n) break;
                uint64_t e = std::min(n, b + chunk);
                for (uint64_t i = b; i < e; ++i) fn(i);
            }
        });
    for (auto& t : th) t.join();
}

// ---------------------------------------------------------------- shading frame
// Frame(n): src/base/utils.h:191-201 (normal -> y, tangent t, s = cross(t, n)).
struct Frame {
    V3 s, t, n;
    explicit Frame(V3 nn) : n(nn) {
        if (std::fabs(n.x) > std::fabs(n.y)) {
            float inv_len = 1.f / std::sqrt(n.x * n.x + n.z * n.z);
            t = V3(n.z * inv_len, 0.f, -n.x * inv_len);
        } else {
            float inv_len = 1.f / std::sqrt(n.y * n.y + n.z * n.z);
            t = V3(0.f, n.z * inv_len, -n.y * inv_len);
        }
        s = cross(t, n);
    }
    V3 to_local(V3 v) const { return V3(dot(v, s), dot(v, n), dot(v, t)); }
    V3 to_world(V3 v) const { return s * v.x + n * v.y + t * v.z; }
};

// ---------------------------------------------------------------- fresnel
// fresnel(cos, ext, int): src/base/utils.h:153-177
float fresnel_utils(float cos_theta_i, float ext_ior, float int_ior) {
    float etai = ext_ior, etat = int_ior;
    if (ext_ior == int_ior) return 0.f;
    if (cos_theta_i < 0.f) {
        std::swap(etai, etat);
        cos_theta_i = -cos_theta_i;
    }
    float eta = etai / etat;
    float sin_theta_t2 = (float)(eta * eta * (1. - cos_theta_i * cos_theta_i));
    if (sin_theta_t2 > 1.f) return 1.f;
    float cos_theta_t = std::sqrt(1.f - sin_theta_t2);
    float Rs = (etai * cos_theta_i - etat * cos_theta_t) / (etai * cos_theta_i + etat * cos_theta_t);
    float Rp = (etat * cos_theta_i - etai * cos_theta_t) / (etat * cos_theta_i + etai * cos_theta_t);
    return (Rs * Rs + Rp * Rp) / 2.f;
}

// fresnel_refl_dielectric(eta, cos_i, cos_t) / (eta, cos_i): src/shading/fresnel.h:75-131
float fr_p(float eta, float ci, float ct) {
    float fac = eta * ct;
    float r = (ci - fac) / (ci + fac);
    return r * r;
}
float fr_s(float eta, float ci, float ct) {
    float fac = eta * ci;
    float r = (ct - fac) / (ct + fac);
    return r * r;
}
float fresnel_refl3(float eta, float ci, float ct) {
    if (ci == 0.f && ct == 0.f) return 0.f;
    return 0.5f * (fr_p(eta, ci, ct) + fr_s(eta, ci, ct));
}
float fresnel_refl(float eta, float ci) {
    const float sin_i2 = 1.f - sq(ci);
    const float sin_t2 = sin_i2 * sq(eta);
    const float cos_t2 = 1.f - sin_t2;
    if (cos_t2 < 0.f) return 1.f;
    return fresnel_refl3(eta, ci, std::sqrt(cos_t2));
}
// fresnel_schlick(eta, cos): fresnel.h:180-183 (computed in double like the reference)
float fresnel_schlick_eta(float eta, float c) {
    double F0 = ((1. - eta) / (1. + eta)) * ((1. - eta) / (1. + eta));
    return (float)(F0 + (1. - F0) * std::pow(1. - c, 5.));
}
// schlick_weight / fresnel_schlick(RGB F0, cos): fresnel.h:176-187
float schlick_weight(float c) {
    double x = std::min(std::max(1. - (double)c, 0.), 1.);
    return (float)std::pow(x, 5.);
}

// ---------------------------------------------------------------- microfacet
// src/shading/microfacet.h:60-291
enum Dist { GGX = 0, BECKMANN = 1 };

float stretched_roughness(V3 m, float sin_v, float ax, float ay) {
    if (ax == ay) return 1.f / sq(ax);
    const float c = sq(m.x / (sin_v * ax));
    const float s = sq(m.z / (sin_v * ay));
    return c + s;
}
float projected_roughness(V3 m, float sin_v, float ax, float ay) {
    if (ax == ay || sin_v == 0.f) return ax;
    const float c = sq((m.x * ax) / sin_v);
    const float s = sq((m.z * ay) / sin_v);
    return std::sqrt(c + s);
}
float dist_D(int dist, float tan2m_a) {
    if (dist == GGX) {
        float tmp = 1 + tan2m_a;
        return 1.f / (kPi * tmp * tmp);
    }
    return kInvPi * std::exp(-tan2m_a);
}
float dist_lambda(int dist, float a_rcp) {
    if (dist == GGX) {
        const float a2_rcp = sq(a_rcp);
        return (-1.f + std::sqrt(1.f + a2_rcp)) * 0.5f;
    }
    const float a = 1.f / a_rcp;
    if (a < 1.6f) {
        const float a2 = sq(a);
        return (1.f - 1.259f * a + 0.396f * a2) / (3.535f * a + 2.181f * a2);
    }
    return 0.f;
}

struct Mdf {
    int dist;
    V3 wi;
    float ax, ay;
    float lambda(V3 m) const {
        float c = m.y;
        if (c == 0.f) return 0.f;
        const float s = std::sqrt(std::max(0.f, 1.f - sq(c)));
        if (s == 0.f) return 0.f;
        const float alpha = projected_roughness(m, s, ax, ay);
        const float tan_v = std::fabs(s / c);
        return dist_lambda(dist, alpha * tan_v);
    }
    float G(V3 wo) const { return 1.f / (lambda(wi) + lambda(wo) + 1.f); }
    float G1(V3 w) const { return 1.f / (lambda(w) + 1.f); }
    float D(V3 m) const {
        const float c = m.y;
        if (c == 0.f) return dist == BECKMANN ? 0.f : sq(ax) * kInvPi;
        const float c2 = sq(c);
        const float s = std::sqrt(std::max(0.f, 1.f - c2));
        const float c4 = sq(c2);
        const float tan2 = (1.f - c2) / c2;
        const float A = stretched_roughness(m, s, ax, ay);
        return dist_D(dist, tan2 * A) / (c4 * ax * ay);
    }
    // VNDF pdf of m (no Jacobian), microfacet.h:227-241
    float pdf(V3 m) const {
        const float c = wi.y;
        if (c == 0.f) return 0.f;
        return G1(wi) * std::fabs(dot(wi, m)) * D(m) / std::fabs(c);
    }
};

// inverse error function: Winitzki's closed-form start (2008) refined by Newton
// steps on erf in double precision.
double erfinv_d(double x) {
    if (x <= -1.0) return -std::numeric_limits<double>::infinity();
    if (x >= 1.0) return std::numeric_limits<double>::infinity();
    const double a = 0.147;
    double ln = std::log(1.0 - x * x);
    double t1 = 2.0 / (M_PI * a) + 0.5 * ln;
    double y = std::copysign(std::sqrt(std::sqrt(t1 * t1 - ln / a) - t1), x);
    for (int i = 0; i < 4; ++i) {
        double err = std::erf(y) - x;
        y -= err / (2.0 / std::sqrt(M_PI) * std::exp(-y * y));
    }
    return y;
}

// Visible-normal sampling (Heitz & d'Eon 2014 stretch / sample slope / rotate /
// unstretch). GGX slopes use the exact construction of Heitz 2018 ("Sampling
// the GGX Distribution of Visible Normals", JCGT 7(4)); Beckmann slopes invert
// the visible-slope CDF by Newton-bisection in the erf domain.
V3 sample_vndf(int dist, V3 wi, float ax, float ay, float u1, float u2) {
    if (dist == GGX) {
        // z-up working frame: (x, z, y) of the y-up local frame
        V3 V(wi.x, wi.z, wi.y);
        V3 Vh = normalize(V3(ax * V.x, ay * V.y, V.z));
        float lensq = Vh.x * Vh.x + Vh.y * Vh.y;
        V3 T1 = lensq > 0.f ? V3(-Vh.y, Vh.x, 0.f) * (1.f / std::sqrt(lensq)) : V3(1.f, 0.f, 0.f);
        V3 T2 = cross(Vh, T1);
        float r = std::sqrt(u1);
        float phi = 2.f * kPi * u2;
        float t1 = r * std::cos(phi);
        float t2 = r * std::sin(phi);
        float s = 0.5f * (1.f + Vh.z);
        t2 = (1.f - s) * std::sqrt(1.f - t1 * t1) + s * t2;
        V3 Nh = T1 * t1 + T2 * t2 + Vh * std::sqrt(std::max(0.f, 1.f - t1 * t1 - t2 * t2));
        V3 Ne = normalize(V3(ax * Nh.x, ay * Nh.y, std::max(0.f, Nh.z)));
        return V3(Ne.x, Ne.z, Ne.y);
    }
    // Beckmann
    V3 ws = normalize(V3(wi.x * ax, wi.y, wi.z * ay));
    float cos_t = ws.y;
    float sin_t = std::sqrt(std::max(0.f, 1.f - cos_t * cos_t));
    float sx, sy;
    if (cos_t > 0.99999f) {
        double r = std::sqrt(-std::log(std::max(1e-12, 1.0 - (double)u1)));
        double p = 2.0 * M_PI * u2;
        sx = (float)(r * std::cos(p));
        sy = (float)(r * std::sin(p));
    } else {
        double tan_t = sin_t / cos_t, cot_t = cos_t / sin_t;
        double c = std::erf(cot_t);
        double K = tan_t / std::sqrt(M_PI);
        double Z = 1.0 + c + K * std::exp(-cot_t * cot_t);
        double lo = -1.0, hi = c;
        double uu = std::min(std::max((double)u1, 1e-7), 1.0 - 1e-7);
        double b = -1.0 + 2.0 * uu * (c + 1.0) * 0.5;
        for (int it = 0; it < 40; ++it) {
            if (!(b > lo && b < hi)) b = 0.5 * (lo + hi);
            double ei = erfinv_d(b);
            double val = (1.0 + b + K * std::exp(-ei * ei)) / Z - uu;
            if (std::fabs(val) < 1e-9) break;
            if (val > 0) hi = b; else lo = b;
            double der = (1.0 - ei * tan_t) / Z;
            b -= val / der;
        }
        sx = (float)erfinv_d(b);
        sy = (float)erfinv_d(2.0 * std::min(std::max((double)u2, 1e-7), 1.0 - 1e-7) - 1.0);
    }
    float phi = std::atan2(ws.z, ws.x);
    float cp = std::cos(phi), spn = std::sin(phi);
    if (sin_t == 0.f) { cp = 1.f; spn = 0.f; }
    float rx = cp * sx - spn * sy;
    float ry = spn * sx + cp * sy;
    return normalize(V3(-rx * ax, 1.f, -ry * ay));
}

inline V3 reflect_n(V3 wi, V3 n) { return -wi + 2.f * dot(wi, n) * n; }
// refract(wi, n, eta): src/base/utils.h:142-151
inline V3 refract_u(V3 wi, V3 n, float eta) {
    float ci = dot(n, wi);
    if (ci < 0) eta = 1.f / eta;
    float co2 = 1 - (1 - ci * ci) * (eta * eta);
    if (co2 <= 0.f) return V3(0.f, 0.f, 0.f);
    float sign = ci >= 0.f ? 1.f : -1.f;
    return n * (-ci * eta + sign * std::sqrt(co2)) + wi * eta;
}

// ---------------------------------------------------------------- closures
struct LobeEval {
    V3 f;       // value (convention dependent)
    float pdf;  // pdf (convention dependent)
};

bool lobe_is_delta(uint32_t id) {
    switch (id) {
    case KZ_CLOSURE_KP_MIRROR: case KZ_CLOSURE_KP_DIELECTRIC: case KZ_CLOSURE_REFLECTION:
    case KZ_CLOSURE_REFRACTION: case KZ_CLOSURE_TRANSPARENT:
        return true;
    default:
        return false;
    }
}

// ---- helpers of the further closures (src/shading/microfacet.cpp:3-38,
// src/base/utils.h:83-125, src/shading/bsdfs.cpp:706-733)
float tan_theta_ref(V3 w) {
    float tmp = 1 - w.y * w.y;
    if (tmp < 0.f) return 0.f;
    return std::sqrt(tmp) / w.y;
}
float tan2_theta_ref(V3 w) { return std::max(0.f, 1.f - w.y * w.y) / (w.y * w.y); }
// BeckmannPDF: D(m) cos(theta_m)
float beckmann_pdf_ref(V3 m, float alpha) {
    float c = m.y;
    if (c <= 0.) return 0.f;
    float a2 = alpha * alpha;
    float t = tan_theta_ref(m);
    double lon = std::exp((-t * t) / a2) / (a2 * std::pow(c, 3));
    return (float)(kInvPi * lon);
}
// G1 of Walter et al. 2007 (rational fit)
float walter_g1_ref(V3 wh, V3 wv, float alpha) {
    if (dot(wv, wh) / wv.y <= 0.f) return 0.f;
    double b = 1. / (alpha * tan_theta_ref(wv));
    if (b >= 1.6f) return 1.f;
    double b2 = b * b;
    return (float)((3.535 * b + 2.181 * b2) / (1. + 2.276 * b + 2.577 * b2));
}
float gtr1_ref(float alpha, float c) {
    float a2 = alpha * alpha;
    return (float)((a2 - 1.) / (kPi * std::log(a2) * (1. + (a2 - 1.) * c)));
}
float clearcoat_g1_ref(float c) {
    double s = std::sqrt(std::max(0., 1. - (double)(c * c)));
    double t = s / c;
    return (float)(2. / (1. + std::sqrt(1. + 0.0625 * t)));
}
float schlick5(float c) { return (float)std::pow(1. - c, 5.); }
V3 cosine_dir(float u0, float u1) {
    float r = std::sqrt(u0);
    float phi = 2.f * kPi * u1;
    float x = r * std::cos(phi), z = r * std::sin(phi);
    return V3(x, std::sqrt(std::max(0.f, 1.f - x * x - z * z)), z);
}

Mdf make_mdf(const kz_lobe& l, V3 wi, int& dist, float& eta) {
    Mdf m;
    if (l.closure_id == KZ_CLOSURE_KP_GLOSS || l.closure_id == KZ_CLOSURE_KP_GLASS) {
        dist = (int)l.params[0];
        m.ax = l.params[7]; m.ay = l.params[8];
        eta = l.params[9];
    } else if (l.closure_id == KZ_CLOSURE_KP_PRINCIPLE_SPECULAR_REFL) {
        dist = GGX;
        m.ax = l.params[6]; m.ay = l.params[7];
        eta = l.params[8];
    } else {  // CONDUCTOR_GGX
        dist = GGX;
        m.ax = l.params[3]; m.ay = l.params[4];
        eta = 1.f;
    }
    m.dist = dist;
    m.wi = wi;
    return m;
}

// Reference-convention value and pdf of one lobe (eval functions of
// src/shading/bsdfs.cpp; on a rejected configuration the reference leaves
// its pdf untouched, here it is 0).
// kRefNorm: the reference's normalisation of half vectors (reference-convention
// queries); the path loop uses the float form, as the shading kernels do.
template <bool kRefNorm = false>
LobeEval eval_reference(const kz_lobe& l, V3 wi, V3 wo) {
    LobeEval r{V3(0, 0, 0), 0.f};
    switch (l.closure_id) {
    case KZ_CLOSURE_DIFFUSE: {
        V3 n(l.params[0], l.params[1], l.params[2]);
        float p = std::max(dot(wo, n), 0.f) * kInvPi;
        r.f = V3(p, p, p);
        r.pdf = p;
        return r;
    }
    case KZ_CLOSURE_KP_MIRROR:
    case KZ_CLOSURE_KP_DIELECTRIC:
        return r;
    case KZ_CLOSURE_KP_GLOSS: {
        int dist; float eta;
        Mdf mdf = make_mdf(l, wi, dist, eta);
        float ci = wi.y, co = wo.y;
        if (ci <= 0 || co <= 0) return r;
        V3 m = nrm<kRefNorm>(wi + wo);
        if (dot(wo, m) == 0.f) return r;
        float D = mdf.D(m), G = mdf.G(wo);
        float F = dist == BECKMANN ? fresnel_refl(eta, dot(m, wi)) : fresnel_refl(eta, std::fabs(dot(m, wi)));
        float v = D * G * F / (4.f * ci * co);
        r.f = V3(v, v, v);
        r.pdf = mdf.pdf(m);
        return r;
    }
    case KZ_CLOSURE_KP_GLASS: {
        int dist; float eta;
        Mdf mdf = make_mdf(l, wi, dist, eta);
        float ci = wi.y, co = wo.y;
        if (eta == 1.f) return r;
        if (ci < 0) eta = 1.f / eta;
        if (ci * co >= 0.f) {
            V3 m = nrm<kRefNorm>(wi + wo);
            float cmi = dot(wi, m);
            float F = fresnel_refl(eta, cmi);
            // reflection_pdf / eval_reflection, bsdfs.h:541-562
            r.pdf = cmi == 0.f ? 0.f : (1.f / (4.f * std::fabs(cmi))) * mdf.pdf(m);
            float denom = std::fabs(4.f * wi.y * wo.y);
            float v = denom == 0.f ? 0.f : F * mdf.D(m) * mdf.G(wo) / denom;
            r.f = V3(v, v, v);
        } else {
            V3 m = nrm<kRefNorm>(wi + eta * wo);
            if (m.y < 0.f) m = -m;
            float cmi = dot(wi, m);
            float F = fresnel_refl(eta, cmi);
            // refraction_pdf / eval_refraction, bsdfs.h:564-599
            float cmo = dot(m, wo);
            float dn = cmi + eta * cmo;
            r.pdf = std::fabs(dn) < 1.0e-6f ? 0.f : std::fabs(cmo) * sq(eta / dn) * mdf.pdf(m);
            float v = 0.f;
            if (wi.y != 0.f && wo.y != 0.f) {
                float c = std::fabs((cmi * cmo) / (wi.y * wo.y));
                float d2 = sq(dn);
                if (!(std::fabs(d2) < 1.0e-6f)) v = c * mdf.D(m) * mdf.G(wo) * (1.f - F) * sq(eta) / sq(d2);
            }
            r.f = V3(v, v, v);
        }
        return r;
    }
    case KZ_CLOSURE_KP_PRINCIPLE_SPECULAR_REFL: {
        int dist; float eta;
        Mdf mdf = make_mdf(l, wi, dist, eta);
        V3 F0(l.params[0], l.params[1], l.params[2]);
        float co = wo.y, ci = wi.y;
        if (ci * co < 0.) return r;
        V3 wh = nrm<kRefNorm>(wi + wo);
        float com = dot(wo, wh);
        if (com == 0.f) return r;
        float D = std::min(4.f, mdf.D(wh));
        float G = mdf.G(wo);
        float s = fresnel_schlick_eta(eta, com);
        V3 F(F0.x + (1.f - F0.x) * s, F0.y + (1.f - F0.y) * s, F0.z + (1.f - F0.z) * s);
        r.pdf = std::max(0.f, mdf.pdf(wh));
        float k = D * G / (4.f * ci * co);
        r.f = V3(std::min(1.f, k * F.x), std::min(1.f, k * F.y), std::min(1.f, k * F.z));
        return r;
    }
    case KZ_CLOSURE_CONDUCTOR_GGX: {
        int dist; float eta;
        Mdf mdf = make_mdf(l, wi, dist, eta);
        float ci = wi.y, co = wo.y;
        if (ci <= 0 || co <= 0) return r;
        V3 m = nrm<kRefNorm>(wi + wo);
        float com = dot(wo, m);
        if (com <= 0.f) return r;
        float w = schlick_weight(com);
        V3 F(l.params[0] + (1.f - l.params[0]) * w, l.params[1] + (1.f - l.params[1]) * w,
             l.params[2] + (1.f - l.params[2]) * w);
        float k = mdf.D(m) * mdf.G(wo) / (4.f * ci * co);
        r.f = V3(k * F.x, k * F.y, k * F.z);
        r.pdf = mdf.pdf(m);
        return r;
    }
    case KZ_CLOSURE_PHONG: {  // bsdfs.cpp:43-59
        V3 N(l.params[0], l.params[1], l.params[2]);
        float ex = l.params[3];
        float cos_ni = wo.y;
        float cos_no = dot(N, wi);
        if (cos_ni > 0 && cos_no > 0) {
            V3 R = (2 * cos_no) * N - wi;
            float cos_ri = dot(R, wo);
            if (cos_ri > 0) {
                r.pdf = (ex + 1) * (1.f / (2.f * kPi)) * std::pow(cos_ri, ex);
                float v = cos_ni * (ex + 2) / (ex + 1);
                r.f = V3(v, v, v);
            }
        }
        return r;
    }
    case KZ_CLOSURE_WARD: {  // bsdfs.cpp:92-112
        float ax = l.params[6], ay = l.params[7];
        float ci = wi.y, co = wo.y;
        if (ci <= 0 || co <= 0) return r;
        V3 m = nrm<kRefNorm>(wi + wo);
        float sin_v = std::sqrt(std::max(0.f, 1.f - ci * ci));
        float A = stretched_roughness(m, sin_v, ax, ay);
        float tmp = std::exp(-tan2_theta_ref(m) * A) / (4.f * kPi * ax * ay);
        r.pdf = (float)std::max(tmp / (dot(m, wi) * std::pow(m.y, 3)), 0.);
        float v = tmp / std::sqrt(ci * co);
        r.f = V3(v, v, v);
        return r;
    }
    case KZ_CLOSURE_TRANSPARENT:  // bsdfs.cpp:205-209
        r.f = V3(1, 1, 1);
        r.pdf = 1.f;
        return r;
    case KZ_CLOSURE_TRANSLUCENT:  // bsdfs.cpp:219-223
        r.pdf = std::max(wo.y, 0.f) * kInvPi;
        r.f = V3(kInvPi, kInvPi, kInvPi);
        return r;
    case KZ_CLOSURE_KP_MICROFACET: {  // bsdfs.cpp:300-319
        float alpha = l.params[0], int_ior = l.params[1], ext_ior = l.params[2], kd = l.params[3];
        float ci = wi.y, co = wo.y;
        if (ci <= 0 || co <= 0) return r;
        V3 wh = nrm<kRefNorm>(wi + wo);
        float D = beckmann_pdf_ref(wh, alpha);
        float F = fresnel_utils(dot(wh, wi), ext_ior, int_ior);
        float G = walter_g1_ref(wh, wi, alpha) * walter_g1_ref(wh, wo, alpha);
        double ks = 1. - kd;
        double Jh = 1. / (4. * dot(wh, wo));
        r.pdf = (float)(ks * D * Jh + kd * co * kInvPi);
        float v = (float)(kInvPi + ks * D * F * G / (4. * ci * co * wh.y));
        r.f = V3(v, v, v);
        return r;
    }
    case KZ_CLOSURE_KP_PRINCIPLE_DIFFUSE: {  // bsdfs.cpp:563-576
        float ci = wi.y, co = wo.y;
        if (co <= 0 || ci <= 0) return r;
        r.pdf = std::max(co, 0.f) * kInvPi;
        float v = (float)(kInvPi * (1.f - 0.5f * std::pow(1 - ci, 5)));
        r.f = V3(v, v, v);
        return r;
    }
    case KZ_CLOSURE_KP_PRINCIPLE_RETRO: {  // bsdfs.cpp:586-605
        float ci = wi.y, co = wo.y;
        if (co <= 0 || ci <= 0) return r;
        r.pdf = std::max(co, 0.f) * kInvPi;
        double FL = std::pow(1. - co, 5.), FV = std::pow(1. - ci, 5.);
        V3 wh = nrm<kRefNorm>(wi + wo);
        float d = dot(wo, wh);
        float RR = 2.f * l.params[3] * (d * d);
        float v = (float)(kInvPi * RR * (FL + FV + FL * FV * (RR - 1.)));
        r.f = V3(v, v, v);
        return r;
    }
    case KZ_CLOSURE_KP_PRINCIPLE_FAKESS: {  // bsdfs.cpp:614-640
        V3 wh = nrm<kRefNorm>(wi + wo);
        float ch = dot(wh, wo);
        float fss90 = ch * ch * l.params[0];
        float aco = std::fabs(wo.y), aci = std::fabs(wi.y);
        float fi = schlick5(aci), fo = schlick5(aco);
        float fss = std::lerp(1.f, fss90, fi) * std::lerp(1.f, fss90, fo);
        double ss = 1.25f * (fss * (1. / (aci + aco) - .5f) + .5f);
        r.pdf = std::max(wo.y, 0.f) * kInvPi;
        float v = (float)(ss * kInvPi);
        r.f = V3(v, v, v);
        return r;
    }
    case KZ_CLOSURE_KP_PRINCIPLE_SHEEN: {  // bsdfs.cpp:649-666
        float ci = wi.y, co = wo.y;
        if (co <= 0 || ci <= 0) return r;
        r.pdf = std::max(co, 0.f) * kInvPi;
        V3 wh = nrm<kRefNorm>(wi + wo);
        float cv = dot(wh, wo);
        float v = cv < 1e-6 ? l.params[3] : (float)(l.params[3] * std::pow(1. - cv, 5.));
        r.f = V3(v, v, v);
        return r;
    }
    case KZ_CLOSURE_KP_PRINCIPLE_CLEARCOAT: {  // bsdfs.cpp:736-780
        float ci = wi.y, co = wo.y;
        if (ci <= 0 || co <= 0) return r;
        V3 wh = nrm<kRefNorm>(wi + wo);
        float ch = wh.y;
        float D = gtr1_ref(l.params[3], ch);
        float G = clearcoat_g1_ref(ci) * clearcoat_g1_ref(co);
        double F = 0.04 + 0.96 * std::pow(1. - ci, 5.);
        r.pdf = (float)std::max(0., D * ch / (4. * dot(wo, wh)));
        float v = (float)std::clamp(D * G * F * 0.25, 0., 0.25);
        r.f = V3(v, v, v);
        return r;
    }
    default:
        return r;
    }
}

// Integrator convention: f*|cos(wo)| and the solid-angle pdf of wo under the
// lobe's own sampling routine.
LobeEval eval_integrator(const kz_lobe& l, V3 wi, V3 wo) {
    LobeEval r = eval_reference(l, wi, wo);
    switch (l.closure_id) {
    case KZ_CLOSURE_DIFFUSE:
        return r;  // already f*cos with pdf cos/pi
    case KZ_CLOSURE_KP_GLOSS:
    case KZ_CLOSURE_CONDUCTOR_GGX:
    case KZ_CLOSURE_KP_PRINCIPLE_SPECULAR_REFL: {
        if (r.pdf == 0.f) return LobeEval{V3(0, 0, 0), 0.f};
        if (wi.y <= 0.f || wo.y <= 0.f) return LobeEval{V3(0, 0, 0), 0.f};
        V3 m = normalize(wi + wo);
        float wom = std::fabs(dot(wo, m));
        if (wom == 0.f) return LobeEval{V3(0, 0, 0), 0.f};
        r.pdf = r.pdf / (4.f * wom);
        r.f = r.f * std::fabs(wo.y);
        return r;
    }
    case KZ_CLOSURE_KP_GLASS: {
        // the sampling routine picks reflection with probability F and
        // refraction with 1-F (bsdfs.cpp:499-553); fold that into the pdf.
        float eta = l.params[9];
        if (eta == 1.f) return LobeEval{V3(0, 0, 0), 0.f};
        if (wi.y < 0) eta = 1.f / eta;
        V3 m;
        if (wi.y * wo.y >= 0.f) m = normalize(wi + wo);
        else {
            m = normalize(wi + eta * wo);
            if (m.y < 0.f) m = -m;
        }
        float F = fresnel_refl(eta, std::min(std::max(dot(m, wi), -1.f), 1.f));
        r.pdf *= (wi.y * wo.y >= 0.f) ? F : (1.f - F);
        r.f = r.f * std::fabs(wo.y);
        return r;
    }
    case KZ_CLOSURE_PHONG: {
        // modified Phong: f = (e+2)/(2 pi) cos_r^e; pdf (e+1)/(2 pi) cos_r^e
        V3 N(l.params[0], l.params[1], l.params[2]);
        float ex = l.params[3];
        float cos_no = dot(N, wi), cos_ni = dot(N, wo);
        if (cos_no <= 0 || cos_ni <= 0) return LobeEval{V3(0, 0, 0), 0.f};
        float cos_ri = dot((2 * cos_no) * N - wi, wo);
        if (cos_ri <= 0) return LobeEval{V3(0, 0, 0), 0.f};
        float lobe = std::pow(cos_ri, ex) / (2.f * kPi);
        float v = (ex + 2) * lobe * cos_ni;
        return LobeEval{V3(v, v, v), (ex + 1) * lobe};
    }
    case KZ_CLOSURE_WARD: {
        // Walter, "Notes on the Ward BRDF": the exponent uses phi of m
        float ax = l.params[6], ay = l.params[7];
        float ci = wi.y, co = wo.y;
        if (ci <= 0 || co <= 0) return LobeEval{V3(0, 0, 0), 0.f};
        V3 m = normalize(wi + wo);
        float ex = -((m.x / ax) * (m.x / ax) + (m.z / ay) * (m.z / ay)) / (m.y * m.y);
        float k = std::exp(ex) / (4.f * kPi * ax * ay);
        float v = k / std::sqrt(ci * co) * co;
        return LobeEval{V3(v, v, v), k / (dot(m, wi) * m.y * m.y * m.y)};
    }
    case KZ_CLOSURE_TRANSLUCENT: {
        if (wi.y * wo.y >= 0) return LobeEval{V3(0, 0, 0), 0.f};
        float v = std::fabs(wo.y) * kInvPi;
        return LobeEval{V3(v, v, v), v};
    }
    case KZ_CLOSURE_KP_MICROFACET: {
        // Nori's microfacet: kd / pi + ks D F G / (4 ci co cos_h)
        float alpha = l.params[0], kd = l.params[3];
        float ci = wi.y, co = wo.y;
        if (ci <= 0 || co <= 0) return LobeEval{V3(0, 0, 0), 0.f};
        V3 wh = normalize(wi + wo);
        float D = beckmann_pdf_ref(wh, alpha);
        float F = fresnel_utils(dot(wh, wi), l.params[2], l.params[1]);
        float G = walter_g1_ref(wh, wi, alpha) * walter_g1_ref(wh, wo, alpha);
        float ks = 1.f - kd;
        float v = (kd * kInvPi + ks * D * F * G / (4.f * ci * co * wh.y)) * co;
        return LobeEval{V3(v, v, v), ks * D / (4.f * dot(wh, wo)) + kd * co * kInvPi};
    }
    case KZ_CLOSURE_KP_PRINCIPLE_DIFFUSE: {
        float ci = wi.y, co = wo.y;
        if (co <= 0 || ci <= 0) return LobeEval{V3(0, 0, 0), 0.f};
        float v = kInvPi * (1.f - 0.5f * schlick5(co)) * (1.f - 0.5f * schlick5(ci)) * co;
        return LobeEval{V3(v, v, v), co * kInvPi};
    }
    case KZ_CLOSURE_KP_PRINCIPLE_RETRO:
    case KZ_CLOSURE_KP_PRINCIPLE_SHEEN:
    case KZ_CLOSURE_KP_PRINCIPLE_FAKESS: {
        if (wi.y <= 0 || wo.y <= 0) return LobeEval{V3(0, 0, 0), 0.f};
        r.f = r.f * wo.y;
        return r;
    }
    case KZ_CLOSURE_KP_PRINCIPLE_CLEARCOAT: {
        // Burley 2012 clearcoat: GTR1(cos^2), Smith GGX G1 (alpha 0.25, tan^2), F0 0.04 at cos_d
        float ci = wi.y, co = wo.y;
        if (ci <= 0 || co <= 0) return LobeEval{V3(0, 0, 0), 0.f};
        V3 wh = normalize(wi + wo);
        float cd = dot(wo, wh);
        if (cd <= 0) return LobeEval{V3(0, 0, 0), 0.f};
        float a2 = l.params[3] * l.params[3];
        // 1 + (a2 - 1) cos^2 = a2 cos^2 + sin^2, without cancellation at small alpha
        float D = (a2 - 1.f) / (kPi * std::log(a2) * (a2 * wh.y * wh.y + (wh.x * wh.x + wh.z * wh.z)));
        auto g1 = [](float c) { return 2.f / (1.f + std::sqrt(1.f + 0.0625f * ((1.f - c * c) / (c * c)))); };
        float F = 0.04f + 0.96f * schlick5(cd);
        float v = 0.25f * D * F * g1(ci) * g1(co) / (4.f * ci);
        return LobeEval{V3(v, v, v), D * wh.y / (4.f * cd)};
    }
    default:
        return LobeEval{V3(0, 0, 0), 0.f};
    }
}

struct LobeSample {
    V3 wo;
    V3 weight;  // f*|cos|/pdf (or delta weight)
    float pdf;  // 0 for delta
    bool valid, delta;
};

LobeSample sample_lobe(const kz_lobe& l, V3 wi, float u0, float u1, float u2) {
    LobeSample s{V3(0, 0, 0), V3(0, 0, 0), 0.f, false, false};
    switch (l.closure_id) {
    case KZ_CLOSURE_DIFFUSE:
    case KZ_CLOSURE_KP_PRINCIPLE_DIFFUSE:
    case KZ_CLOSURE_KP_PRINCIPLE_RETRO:
    case KZ_CLOSURE_KP_PRINCIPLE_FAKESS:
    case KZ_CLOSURE_KP_PRINCIPLE_SHEEN:
    case KZ_CLOSURE_TRANSLUCENT: {
        // cosine-weighted hemisphere about +y (the pdf the reference declares);
        // the translucent lobe mirrors it to the side away from wi
        s.wo = cosine_dir(u0, u1);
        if (l.closure_id == KZ_CLOSURE_TRANSLUCENT) {
            if (wi.y == 0.f) return s;
            if (wi.y > 0.f) s.wo.y = -s.wo.y;
        }
        LobeEval e = eval_integrator(l, wi, s.wo);
        if (e.pdf <= 0.f) return s;
        s.pdf = e.pdf;
        s.weight = e.f * (1.f / e.pdf);
        s.valid = true;
        return s;
    }
    case KZ_CLOSURE_KP_MIRROR: {
        s.wo = reflect_n(wi, V3(0, 1, 0));
        s.weight = V3(1, 1, 1);
        s.valid = s.delta = true;
        return s;
    }
    case KZ_CLOSURE_KP_DIELECTRIC: {
        float ior_in = l.params[0], ior_ex = l.params[1];
        V3 n(0, 1, 0);
        float ci = dot(wi, n);
        float F = fresnel_utils(ci, ior_ex, ior_in);
        if (u0 < F) {
            s.wo = reflect_n(wi, n);
        } else {
            float fac = ior_in / ior_ex;
            if (ci < 0.f) {
                fac = ior_ex / ior_in;
                n = -n;
            }
            s.wo = refract_u(-wi, n, fac);
            if (is_zero(s.wo)) return s;
        }
        s.weight = V3(1, 1, 1);
        s.valid = s.delta = true;
        return s;
    }
    case KZ_CLOSURE_REFLECTION: {  // bsdfs.cpp:150-167
        if (wi.y <= 0.f) return s;
        s.wo = reflect_n(wi, V3(0, 1, 0));
        s.weight = V3(1, 1, 1);
        s.valid = s.delta = true;
        return s;
    }
    case KZ_CLOSURE_REFRACTION: {
        // Snell transmission, eta = inside / outside (the OSL refraction()
        // convention); bsdfs.cpp:178-203 refracts with the normal on wi's side
        V3 n(0, 1, 0);
        float fac = l.params[3];
        if (wi.y < 0.f) {
            fac = 1.f / fac;
            n = -n;
        }
        s.wo = refract_u(-wi, n, fac);
        if (is_zero(s.wo)) return s;
        s.weight = V3(1, 1, 1);
        s.valid = s.delta = true;
        return s;
    }
    case KZ_CLOSURE_TRANSPARENT: {  // bsdfs.cpp:211-217
        s.wo = -wi;
        s.weight = V3(1, 1, 1);
        s.valid = s.delta = true;
        return s;
    }
    case KZ_CLOSURE_PHONG: {
        if (wi.y <= 0.f) return s;
        V3 N(l.params[0], l.params[1], l.params[2]);
        float cos_no = dot(N, wi);
        if (cos_no <= 0.f) return s;
        V3 R = (2 * cos_no) * N - wi;
        // frame about R (Duff et al. 2017)
        float sg = R.z >= 0.f ? 1.f : -1.f;
        float a = -1.f / (sg + R.z);
        float b = R.x * R.y * a;
        V3 t1(1.f + sg * R.x * R.x * a, sg * b, -sg * R.x);
        V3 t2(b, sg + R.y * R.y * a, -R.y);
        float ct = std::pow(u1, 1.f / (l.params[3] + 1.f));
        float st = std::sqrt(std::max(0.f, 1.f - ct * ct));
        float phi = 2.f * kPi * u0;
        s.wo = t1 * (st * std::cos(phi)) + t2 * (st * std::sin(phi)) + R * ct;
        if (s.wo.y <= 0.f) return s;
        LobeEval e = eval_integrator(l, wi, s.wo);
        if (e.pdf <= 0.f) return s;
        s.pdf = e.pdf;
        s.weight = e.f * (1.f / e.pdf);
        s.valid = true;
        return s;
    }
    case KZ_CLOSURE_WARD:
    case KZ_CLOSURE_KP_MICROFACET:
    case KZ_CLOSURE_KP_PRINCIPLE_CLEARCOAT: {
        if (wi.y <= 0.f) return s;
        V3 m(0, 0, 0);
        if (l.closure_id == KZ_CLOSURE_WARD) {
            // Walter's notes eqs. 6-7 with the quadrant of 2 pi u0 kept
            float ax = l.params[6], ay = l.params[7];
            float px = ax * std::cos(2.f * kPi * u0), pz = ay * std::sin(2.f * kPi * u0);
            float len = std::sqrt(px * px + pz * pz);
            float cphi = px / len, sphi = pz / len;
            float A = (cphi / ax) * (cphi / ax) + (sphi / ay) * (sphi / ay);
            float theta = std::atan(std::sqrt(-std::log(1.f - u1) / A));
            m = V3(std::sin(theta) * cphi, std::cos(theta), std::sin(theta) * sphi);
        } else if (l.closure_id == KZ_CLOSURE_KP_MICROFACET) {
            if (u2 >= 1.f - l.params[3]) {
                s.wo = cosine_dir(u0, u1);
            } else {
                float theta = std::atan(std::sqrt(-l.params[0] * l.params[0] * std::log(1.f - u1)));
                float phi = 2.f * kPi * u0;
                m = V3(std::sin(theta) * std::cos(phi), std::cos(theta), std::sin(theta) * std::sin(phi));
            }
        } else {
            // GTR1 half vector (Burley 2012, appendix B)
            float a2 = l.params[3] * l.params[3];
            float ct = std::sqrt(std::max(0.f, (1.f - std::pow(a2, 1.f - u1)) / (1.f - a2)));
            float st = std::sqrt(std::max(0.f, 1.f - ct * ct));
            float phi = 2.f * kPi * u0;
            m = V3(st * std::cos(phi), ct, st * std::sin(phi));
        }
        if (!is_zero(m)) s.wo = reflect_n(wi, m);
        if (s.wo.y <= 0.f) return s;
        LobeEval e = eval_integrator(l, wi, s.wo);
        if (e.pdf <= 0.f) return s;
        s.pdf = e.pdf;
        s.weight = e.f * (1.f / e.pdf);
        s.valid = true;
        return s;
    }
    case KZ_CLOSURE_KP_GLOSS:
    case KZ_CLOSURE_CONDUCTOR_GGX:
    case KZ_CLOSURE_KP_PRINCIPLE_SPECULAR_REFL: {
        if (wi.y <= 0.f) return s;
        int dist; float eta;
        Mdf mdf = make_mdf(l, wi, dist, eta);
        V3 m = sample_vndf(dist, wi, mdf.ax, mdf.ay, u0, u1);
        s.wo = reflect_n(wi, m);
        if (s.wo.y <= 0.f) return s;
        LobeEval e = eval_integrator(l, wi, s.wo);
        if (e.pdf <= 0.f) return s;
        s.pdf = e.pdf;
        s.weight = e.f * (1.f / e.pdf);
        s.valid = true;
        return s;
    }
    case KZ_CLOSURE_KP_GLASS: {
        int dist; float eta;
        Mdf mdf = make_mdf(l, wi, dist, eta);
        if (eta == 1.f) return s;
        if (wi.y < 0.f) eta = 1.f / eta;
        // sample_m flips wi into the upper hemisphere (microfacet.h:200-203)
        V3 wis = wi.y < 0.f ? -wi : wi;
        V3 m = sample_vndf(dist, wis, mdf.ax, mdf.ay, u0, u1);
        float cmi = std::min(std::max(dot(m, wi), -1.f), 1.f);
        float F = fresnel_refl(eta, cmi);
        if (u2 < F) {
            s.wo = reflect_n(wi, m);
            if (wi.y * s.wo.y <= 0.f) return s;
        } else {
            s.wo = refract_u(wi, m, eta);
            if (is_zero(s.wo) || wi.y * s.wo.y > 0.f) return s;
            s.wo = normalize(s.wo);
        }
        LobeEval e = eval_integrator(l, wi, s.wo);
        if (e.pdf <= 0.f) return s;
        s.pdf = e.pdf;
        s.weight = e.f * (1.f / e.pdf);
        s.valid = true;
        return s;
    }
    default:
        return s;
    }
}

// ---------------------------------------------------------------- scene
struct OLight {
    uint32_t geom;
    std::vector<uint32_t> tris;  // global triangle ids (empty for a point light)
    std::vector<float> cdf;      // normalised running sum of areas, cdf[0] = 0
    float area;
    V3 Le;
    bool point = false;          // PointLight (src/core/light.cpp:18-31) at `pos`
    V3 pos{0, 0, 0};
};

struct OTexture {
    int kind = KZ_TEX_CHECKER;
    uint32_t w = 0, h = 0;
    std::vector<float> rgb;
    float scale_s = 1.f, scale_t = 1.f;
    V3 Ca{1, 1, 1}, Cb{0, 0, 0};
};

struct OScene {
    OBvh bvh;
    std::vector<uint32_t> tri_geom;
    std::vector<int32_t> geom_material;
    std::vector<int32_t> geom_light;  // light index or -1
    std::vector<kz_material> materials;
    std::vector<OLight> lights;
    std::vector<float> tri_uv;        // 6 floats per triangle (global order), or empty
    std::vector<float> tri_nrm;       // 9 floats per triangle (global order), or empty
    std::vector<uint8_t> tri_has_nrm; // per triangle: its mesh has vertex normals
    std::vector<OTexture> textures;
    V3 env{0, 0, 0};
    int env_tex = -1;
};

// Texture lookup: the OSL checkerboard shader's rule, or bilinear filtering
// with periodic wrap and texel centres at (i + 0.5) / w.
V3 texture_lookup(const OTexture& t, float s, float u) {
    if (!std::isfinite(s)) s = 0.f;
    if (!std::isfinite(u)) u = 0.f;
    if (t.kind == KZ_TEX_CHECKER) {
        float cs = std::fmod(s * t.scale_s, 2.f), ct = std::fmod(u * t.scale_t, 2.f);
        int a = std::isfinite(cs) ? (int)cs : 0, b = std::isfinite(ct) ? (int)ct : 0;
        return (a ^ b) == 0 ? t.Ca : t.Cb;
    }
    s -= std::floor(s);
    u -= std::floor(u);
    float x = s * (float)t.w - 0.5f, y = u * (float)t.h - 0.5f;
    float fx = std::floor(x), fy = std::floor(y);
    float ax = x - fx, ay = y - fy;
    uint32_t x0 = fx < 0.f ? t.w - 1 : std::min((uint32_t)fx, t.w - 1);
    uint32_t y0 = fy < 0.f ? t.h - 1 : std::min((uint32_t)fy, t.h - 1);
    uint32_t x1 = (x0 + 1) % t.w, y1 = (y0 + 1) % t.h;
    auto px = [&](uint32_t xx, uint32_t yy) {
        const float* p = &t.rgb[((size_t)yy * t.w + xx) * 3];
        return V3(p[0], p[1], p[2]);
    };
    return (px(x0, y0) * (1.f - ax) + px(x1, y0) * ax) * (1.f - ay) + (px(x0, y1) * (1.f - ax) + px(x1, y1) * ax) * ay;
}

// The environment seen along d (latitude-longitude, +y up).
V3 environment(const OScene& sc, V3 d) {
    V3 e = sc.env;
    if (sc.env_tex >= 0) {
        float s = 0.5f + std::atan2(d.x, -d.z) * (0.5f * kInvPi);
        float t = std::acos(std::min(std::max(d.y, -1.f), 1.f)) * kInvPi;
        e = mul(e, texture_lookup(sc.textures[(size_t)sc.env_tex], s, t));
    }
    return e;
}

// Texture of a material: the one its lobes reference through
// params[KZ_LOBE_TEXTURE_PARAM] = index + 1, or -1.
int material_texture(const kz_material& m) {
    for (uint32_t k = 0; k < std::min<uint32_t>(m.n_lobes, KZ_MAX_LOBES); ++k)
        if (m.lobes[k].params[KZ_LOBE_TEXTURE_PARAM] != 0.f) return (int)m.lobes[k].params[KZ_LOBE_TEXTURE_PARAM] - 1;
    return -1;
}

V3 weight_of(const kz_lobe& lb, int mtex, V3 tint) {
    V3 w(lb.weight[0], lb.weight[1], lb.weight[2]);
    return (mtex >= 0 && lb.params[KZ_LOBE_TEXTURE_PARAM] != 0.f) ? mul(w, tint) : w;
}

float tri_area(const OBvh& b, uint32_t tri) {
    V3 p0 = b.v(tri, 0), p1 = b.v(tri, 1), p2 = b.v(tri, 2);
    V3 c = cross(p1 - p0, p2 - p0);
    return 0.5f * std::sqrt(dot(c, c));
}

// DiscrectPDF::sample, src/base/dpdf.h:31-36 (lower_bound over the cdf)
uint32_t cdf_sample(const std::vector<float>& cdf, float u) {
    auto it = std::lower_bound(cdf.begin(), cdf.end(), u);
    long idx = (long)(it - cdf.begin()) - 1;
    if (idx < 0) idx = 0;
    long last = (long)cdf.size() - 2;
    return (uint32_t)std::min(idx, last);
}

struct CamBasis {
    V3 eye, x, y, z;
    float tan_half, aspect;
    float flip;
};

CamBasis cam_basis(const kz_camera& c, uint32_t W, uint32_t H) {
    CamBasis b;
    V3 eye(c.eye[0], c.eye[1], c.eye[2]);
    V3 look(c.lookat[0], c.lookat[1], c.lookat[2]);
    V3 up = normalize(V3(c.up[0], c.up[1], c.up[2]));
    b.eye = eye;
    b.z = normalize(eye - look);
    b.x = normalize(cross(up, b.z));
    b.y = cross(b.z, b.x);
    b.tan_half = (float)std::tan((double)c.fov_deg * 0.5 * M_PI / 180.0);
    b.aspect = (float)W / (float)H;
    b.flip = c.flip ? -1.f : 1.f;
    return b;
}

V3 cam_dir(const CamBasis& b, uint32_t px, uint32_t py, uint32_t W, uint32_t H, float jx, float jy) {
    float sx = ((float)px + jx) / (float)W;
    float sy = ((float)py + jy) / (float)H;
    float nx = 2.0f * sx - 1.0f;
    float ny = b.flip * ((1.0f - 2.0f * sy) / b.aspect);
    float cx = nx * b.tan_half;
    float cy = ny * b.tan_half;
    V3 d = b.x * cx + b.y * cy + b.z * (-1.0f);
    return normalize(d);
}

inline float power_heuristic(float f, float g) {
    // power_heuristic(1, f, 1, g), src/core/sampling.h:61-64
    return (f * f) / (f * f + g * g);
}

struct PathCounters {
    uint64_t bounces = 0, shadow = 0;
};

// ---- the reference's loop as written (compat modes of Li below)
//
// Bits of `compat`; 0 is the corrected loop the GPU path computes.
enum : uint32_t {
    // next-event estimation of integrator.cpp:465-481: the composite closure's
    // reference-convention value (Diffuse already includes cos) times
    // cos(light, shading normal) again, lights below the shading normal
    // skipped, MIS against the reference-convention composite pdf
    COMPAT_NEE = 1,
    // BSDF sampling of integrator.cpp:503-506 with CompositeClosure::sample
    // (bsdf.cpp:17-55): lobe picked uniformly and divided by its selection
    // probability, the other lobes' values added undivided, throughput times
    // that value with no division by the direction pdf; Diffuse samples
    // uniform theta (sample_hemisphere, sampling.h:25-32), microfacet lobes
    // MicrofacetInterface::sample_m (microfacet.h:103-213)
    COMPAT_BSDF = 2,
    // emission hit of integrator.cpp:444-459: MIS weight from the previous
    // vertex's BSDF pdf and the light pdf its next-event sample left behind
    COMPAT_EMISSION = 4,
    // depth of integrator.cpp:407-420 and :555: max_depth fixed at 8 and
    // stepped twice per vertex (at most 4 shaded vertices), roulette from the
    // second vertex on (depth >= 3)
    COMPAT_DEPTH = 8,
};

// sample_hemisphere(u), src/core/sampling.h:25-32: theta uniform in [0, pi/2]
V3 sample_hemisphere_ref(float u0, float u1) {
    float theta = u0 * (float)M_PI_2;
    float phi = u1 * (float)M_PI * 2.f;
    float ct = std::cos(theta), st = std::sin(theta);
    return normalize_ref(V3(st * std::cos(phi), ct, st * std::sin(phi)));
}

// GGXDist::sample_slope, src/shading/microfacet.h:103-126
void ggx_slope_ref(float cos_theta, float s0, float s1, float& sx, float& sy) {
    float c = cos_theta < 1e-6f ? 1e-6f : cos_theta;
    float Q = (1 + c) * s0 - c;
    float num = c * std::sqrt((1 - c) * (1 + c)) - Q * std::sqrt((1 - Q) * (1 + Q));
    float den = (Q - c) * (Q + c);
    float eps = 1.f / 4294967296.0f;
    den = std::fabs(den) < eps ? std::copysign(eps, den) : den;
    sx = num / den;
    float Ru = 1 - 2 * s1;
    float u2 = std::fabs(Ru);
    float z = (u2 * (u2 * (u2 * 0.27385f - 0.73369f) + 0.46341f)) /
              (u2 * (u2 * (u2 * 0.093073f + 0.309420f) - 1.0f) + 0.597999f);
    sy = std::copysign(1.0f, Ru) * z * std::sqrt(1.0f + sx * sx);
}

// BeckmannDist::sample_slope, src/shading/microfacet.h:128-171, 1/erf where an
// inverse erf is meant as written; OIIO::fast_exp (:169) taken as exp
void beckmann_slope_ref(float cos_theta_i, float s0, float s1, float& sx, float& sy) {
    float ct = cos_theta_i < 1e-6f ? 1e-6f : cos_theta_i;
    float tan_theta_i = std::sqrt(1 - ct * ct) / ct;
    float cot_theta_i = 1 / tan_theta_i;
    float c = std::erf(cot_theta_i);
    float K = tan_theta_i * 0.564189583547756286948f;
    float y_approx = s0 * (1.f + c + K * (1 - c * c));
    float y_exact = s0 * (1.f + c + K * std::exp(-cot_theta_i * cot_theta_i));
    float b = K > 0 ? (0.5f - std::sqrt(K * (K - y_approx + 1.f) + 0.25f)) / K : y_approx - 1.f;
    float inv_erf = 1.f / std::erf(b);
    float value = 1.f + b + K * std::exp(-inv_erf * inv_erf) - y_exact;
    if (std::fabs(value) > 1e-6f) {
        b -= value / (1 - inv_erf * tan_theta_i);
        inv_erf = 1.f / std::erf(b);
        value = 1.0f + b + K * std::exp(-inv_erf * inv_erf) - y_exact;
        b -= value / (1 - inv_erf * tan_theta_i);
        sx = 1.f / std::erf(b);
    } else {
        sx = inv_erf;
    }
    sy = 1.f / std::erf(2.0f * s1 - 1.0f);
}

// MicrofacetInterface::sample_m, src/shading/microfacet.h:173-213: the slope
// is sampled for the unstretched angle and rotated by wi's azimuth
V3 sample_m_ref(int dist, V3 wi, float ax, float ay, float u0, float u1) {
    float cos_theta_i = wi.y;
    float phi = 0.f;
    if (cos_theta_i < 0.9999f) phi = std::atan2(wi.z, wi.x);
    float sx, sy;
    if (dist == BECKMANN) beckmann_slope_ref(cos_theta_i, u0, u1, sx, sy);
    else ggx_slope_ref(cos_theta_i, u0, u1, sx, sy);
    const float cp = std::cos(phi), sp = std::sin(phi);
    const float rx = cp * sx - sp * sy, ry = sp * sx + cp * sy;
    return normalize_ref(V3(-rx * ax, 1.f, -ry * ay));
}

// The reference's own sampler for one lobe (the sample functions of
// bsdfs.cpp): the direction; its value and pdf are the reference-convention
// eval at that direction, which is what those functions return.
V3 sample_dir_ref(const kz_lobe& l, V3 wi, float u0, float u1, float u2, bool& ok) {
    ok = true;
    switch (l.closure_id) {
    case KZ_CLOSURE_DIFFUSE:
        return sample_hemisphere_ref(u0, u1);
    case KZ_CLOSURE_KP_GLOSS:
    case KZ_CLOSURE_KP_PRINCIPLE_SPECULAR_REFL:
    case KZ_CLOSURE_CONDUCTOR_GGX: {
        int dist;
        float eta;
        Mdf m = make_mdf(l, wi, dist, eta);
        V3 h = sample_m_ref(dist, wi, m.ax, m.ay, u0, u1);
        return reflect_n(wi, h);
    }
    default: {  // the restatement's sampler gives the direction of the other lobes
        LobeSample smp = sample_lobe(l, wi, u0, u1, u2);
        ok = smp.valid;
        return smp.wo;
    }
    }
}

// One path of the corrected PathIntegrator::Li (src/core/integrator.cpp:362-561).
// Random numbers: 9 per shaded vertex, in a fixed order, whatever branches run:
//   [0] light pick  [1] light triangle  [2,3] point on triangle  [4] roulette
//   [5] lobe pick   [6,7,8] lobe sample
// est: 0 NEE + BSDF sampling with MIS (PathIntegrator), 1 NEE only
// (PathEmsIntegrator, integrator.cpp:264-360), 2 BSDF sampling only
// (PathMatsIntegrator, integrator.cpp:213-262).
V3 Li(const OScene& sc, V3 o, V3 d, Pcg32& rng, uint32_t max_depth, uint32_t rr_min, PathCounters& pc,
      int est = 0, uint32_t compat = 0) {
    V3 L(0, 0, 0), beta(1, 1, 1);
    float prev_pdf = 0.f;
    bool prev_specular = true;
    const uint32_t nl = (uint32_t)sc.lights.size();
    // compat state: the previous vertex's light pdf (per light, as
    // GeometryLight::sample leaves it) and BSDF pdf (as bsdf_sample.pdf)
    float stale_lpdf = 0.f, stale_mpdf = 1.f;
    if (compat & COMPAT_DEPTH) max_depth = 4;
    for (uint32_t depth = 0; depth < max_depth; ++depth) {
        float t, bu, bv;
        uint32_t prim;
        pc.bounces++;
        if (!sc.bvh.closest(o, d, kRayEps, std::numeric_limits<float>::infinity(), t, prim, bu, bv)) {
            // background shader on a miss, no MIS (integrator.cpp:545-552)
            if (sc.env.x > 0.f || sc.env.y > 0.f || sc.env.z > 0.f) L = L + mul(beta, environment(sc, d));
            break;
        }
        float u[9];
        for (int k = 0; k < 9; ++k) u[k] = rng.nextf();
        const uint32_t geom = sc.tri_geom[prim];
        const kz_material& mat = sc.materials[(size_t)sc.geom_material[geom]];
        V3 v0 = sc.bvh.v(prim, 0), v1 = sc.bvh.v(prim, 1), v2 = sc.bvh.v(prim, 2);
        V3 Ng = normalize(cross(v1 - v0, v2 - v0));
        V3 P = o + d * t;
        // shading normal and shadow-terminator offset, TriangleMesh::post_hit
        // (shape.cpp:628-656): P' = P_bary - sum_i b_i min(0, (P_bary - v_i).n_i) n_i
        V3 Ns = Ng;
        if (!sc.tri_has_nrm.empty() && sc.tri_has_nrm[prim]) {
            const float* q = &sc.tri_nrm[(size_t)prim * 9];
            V3 n0(q[0], q[1], q[2]), n1(q[3], q[4], q[5]), n2(q[6], q[7], q[8]);
            float b0 = 1.f - bu - bv;
            Ns = normalize(n0 * b0 + n1 * bu + n2 * bv);
            V3 Pb = v0 * b0 + v1 * bu + v2 * bv;
            float e0 = std::min(0.f, dot(Pb - v0, n0)), e1 = std::min(0.f, dot(Pb - v1, n1)),
                  e2 = std::min(0.f, dot(Pb - v2, n2));
            P = Pb - (n0 * (b0 * e0) + n1 * (bu * e1) + n2 * (bv * e2));
        }
        // texture tint at the hit's uv (vertex uvs interpolated by the hit's
        // barycentrics; the barycentrics themselves for meshes without uvs)
        const int mtex = sc.textures.empty() ? -1 : material_texture(mat);
        V3 tint(1, 1, 1);
        if (mtex >= 0) {
            float b0 = 1.f - bu - bv;
            float s0 = 0.f, t0 = 0.f, s1 = 1.f, t1 = 0.f, s2 = 0.f, t2 = 1.f;
            if (!sc.tri_uv.empty()) {
                const float* q = &sc.tri_uv[(size_t)prim * 6];
                s0 = q[0]; t0 = q[1]; s1 = q[2]; t1 = q[3]; s2 = q[4]; t2 = q[5];
            }
            tint = texture_lookup(sc.textures[(size_t)mtex], b0 * s0 + bu * s1 + bv * s2, b0 * t0 + bu * t1 + bv * t2);
        }
        Frame fr(Ns);
        V3 wi = -fr.to_local(d);
        // 1. emission on hit (front side of the shading normal, single_emissive_surface)
        V3 Le(mat.Le[0], mat.Le[1], mat.Le[2]);
        if (!is_zero(Le) && dot(d, Ns) < 0.f && (compat & COMPAT_EMISSION)) {
            float w = prev_specular ? 1.f : power_heuristic(stale_mpdf, stale_lpdf);
            L = L + mul(beta, Le) * w;
        } else if (!is_zero(Le) && dot(d, Ns) < 0.f) {
            float w = 1.f;
            if (!prev_specular && est != 2) {
                int li = sc.geom_light[geom];
                if (li >= 0) {
                    if (est == 1) {
                        w = 0.f;  // found by next-event estimation instead
                    } else {
                        float cos_l = -dot(d, Ng);
                        float lpdf = (t * t) / (cos_l * sc.lights[(size_t)li].area) * (1.0f / (float)nl);
                        w = power_heuristic(prev_pdf, lpdf);
                    }
                }
            }
            L = L + mul(beta, Le) * w;
        }
        // lobe selection probabilities, CompositeClosure::compute_pdfs (bsdf.h:157-176)
        const uint32_t nlobes = std::min<uint32_t>(mat.n_lobes, KZ_MAX_LOBES);
        float lp[KZ_MAX_LOBES];
        float bsum = beta.x + beta.y + beta.z;
        float winv = 1.f / bsum;
        float wsum = 0.f;
        bool any_smooth = false;
        for (uint32_t i = 0; i < nlobes; ++i) {
            const kz_lobe& lb = mat.lobes[i];
            V3 lw = weight_of(lb, mtex, tint);
            lp[i] = (lw.x * beta.x + lw.y * beta.y + lw.z * beta.z) * winv;
            wsum += lp[i];
            if (!lobe_is_delta(lb.closure_id)) any_smooth = true;
        }
        if (wsum > 0.f)
            for (uint32_t i = 0; i < nlobes; ++i) lp[i] /= wsum;
        // 2. next-event estimation (not when sampling the BSDF only)
        if ((compat & COMPAT_NEE) && nl > 0) {
            // integrator.cpp:465-481 with GeometryLight::sample (light.cpp:52-76)
            uint32_t li = std::min((uint32_t)(u[0] * (float)nl), nl - 1);
            const OLight& lt = sc.lights[li];
            if (!lt.point) {
                uint32_t k = cdf_sample(lt.cdf, u[1]);
                uint32_t ltri = lt.tris[k];
                V3 a0 = sc.bvh.v(ltri, 0), a1 = sc.bvh.v(ltri, 1), a2 = sc.bvh.v(ltri, 2);
                float su0 = std::sqrt(u[2]);
                float bu0 = 1.f - su0;
                float bv0 = u[3] * su0;
                V3 p = a0 * bu0 + a1 * bv0 + a2 * (1.f - bu0 - bv0);
                V3 nlgt = normalize(cross(a1 - a0, a2 - a0));
                V3 lv = p - P;
                float dist2 = dot(lv, lv);
                float dist = std::sqrt(dist2);
                V3 ldir = normalize_ref(lv);
                stale_lpdf = 1.f / lt.area;
                pc.shadow++;
                float cos_l = dot(-ldir, nlgt);
                if (!sc.bvh.any(P, ldir, kRayEps, dist - kRayEps) && cos_l > 0.f) {
                    stale_lpdf = stale_lpdf * dist2 / cos_l;
                    V3 Ls = lt.Le * (1.f / stale_lpdf);
                    float cos_v = dot(ldir, Ns);
                    if (cos_v > 0.f) {
                        V3 wo = fr.to_local(ldir);
                        V3 f(0, 0, 0);
                        float bpdf = 0.f;
                        for (uint32_t i = 0; i < nlobes; ++i) {
                            const kz_lobe& lb = mat.lobes[i];
                            LobeEval e = eval_reference<true>(lb, wi, wo);
                            f = f + mul(weight_of(lb, mtex, tint), e.f);
                            bpdf += lp[i] * e.pdf;
                        }
                        float w = power_heuristic(stale_lpdf, bpdf);
                        if (std::isnan(w)) w = 0.f;
                        L = L + mul(mul(beta, Ls), f) * (w * cos_v * (float)nl);
                    }
                }
            }
        } else if (est != 2 && nl > 0 && any_smooth && wsum > 0.f) {
            uint32_t li = std::min((uint32_t)(u[0] * (float)nl), nl - 1);
            const OLight& lt = sc.lights[li];
            V3 p = lt.pos, nlgt(0, 0, 0);
            if (!lt.point) {
                uint32_t k = cdf_sample(lt.cdf, u[1]);
                uint32_t ltri = lt.tris[k];
                V3 a0 = sc.bvh.v(ltri, 0), a1 = sc.bvh.v(ltri, 1), a2 = sc.bvh.v(ltri, 2);
                float su0 = std::sqrt(u[2]);
                float bu0 = 1.f - su0;
                float bv0 = u[3] * su0;
                p = a0 * bu0 + a1 * bv0 + a2 * (1.f - bu0 - bv0);
                nlgt = normalize(cross(a1 - a0, a2 - a0));
            }
            V3 lv = p - P;
            float dist2 = dot(lv, lv);
            float dist = std::sqrt(dist2);
            V3 ldir(lv.x / dist, lv.y / dist, lv.z / dist);
            float cos_l = lt.point ? 1.f : -dot(ldir, nlgt);
            if (cos_l > 0.f && dist2 > 0.f) {
                // a point light: picked with probability 1/nl, no MIS (a delta light)
                float lpdf = lt.point ? 1.0f / (float)nl : dist2 / (cos_l * lt.area) * (1.0f / (float)nl);
                V3 wo = fr.to_local(ldir);
                V3 f(0, 0, 0);
                float bpdf = 0.f;
                for (uint32_t i = 0; i < nlobes; ++i) {
                    const kz_lobe& lb = mat.lobes[i];
                    if (lobe_is_delta(lb.closure_id)) continue;
                    LobeEval e = eval_integrator(lb, wi, wo);
                    f = f + mul(weight_of(lb, mtex, tint), e.f);
                    bpdf += lp[i] * e.pdf;
                }
                if (!is_zero(f)) {
                    pc.shadow++;
                    if (!sc.bvh.any(P, ldir, kRayEps, dist - kRayEps)) {
                        float w = lt.point || est == 1 ? 1.f : power_heuristic(lpdf, bpdf);
                        // PointLight::sample returns radiance / (0.1 |d|^2)
                        V3 Le = lt.point ? lt.Le * (1.f / (dist2 * 0.1f)) : lt.Le;
                        V3 c = mul(mul(beta, f), Le) * (w / lpdf);
                        L = L + c;
                    }
                }
            }
        }
        if (depth + 1 >= max_depth) break;
        // 3. Russian roulette (integrator.cpp:491-498)
        if ((compat & COMPAT_DEPTH) ? depth >= 1 : depth >= rr_min) {
            float prob = std::min(max_comp(beta) * 0.9025f, 0.99f);
            if (prob < u[4]) break;
            beta = beta * (1.f / prob);
        }
        // 4. BSDF sampling: lobe by its selection probability, then the
        // one-sample mixture over all non-delta lobes.
        if (compat & COMPAT_BSDF) {
            // integrator.cpp:503-506 with CompositeClosure::sample (bsdf.cpp:17-55)
            if (nlobes == 0) break;
            uint32_t idx = std::min((uint32_t)(u[5] * 0.9999999f * (float)nlobes), nlobes - 1);
            const kz_lobe& ls = mat.lobes[idx];
            bool ok;
            V3 wo = sample_dir_ref(ls, wi, u[6], u[7], u[8], ok);
            if (!ok) break;
            LobeEval e = eval_reference<true>(ls, wi, wo);
            V3 ret = mul(weight_of(ls, mtex, tint), e.f) * (1.f / lp[idx]);
            float pdf_acc = e.pdf * lp[idx];
            for (uint32_t i = 0; i < nlobes; ++i) {
                if (i == idx) continue;
                const float before = pdf_acc;  // other_sample copies bsdf_sample first
                const kz_lobe& lb = mat.lobes[i];
                LobeEval eo = eval_reference<true>(lb, wi, wo);  // and eval overwrites its pdf
                ret = ret + mul(weight_of(lb, mtex, tint), eo.f);
                pdf_acc = eo.pdf + lp[i] * before;
            }
            beta = mul(beta, ret);
            stale_mpdf = pdf_acc;
            prev_pdf = pdf_acc;
            prev_specular = lobe_is_delta(ls.closure_id);
            if (is_zero(beta) || !std::isfinite(beta.x + beta.y + beta.z)) break;
            o = P;
            d = normalize_ref(fr.to_world(wo));
            continue;
        }
        if (!(wsum > 0.f)) break;
        uint32_t sel = nlobes - 1;
        {
            float acc = 0.f;
            for (uint32_t i = 0; i < nlobes; ++i) {
                acc += lp[i];
                if (u[5] < acc) { sel = i; break; }
            }
            while (sel > 0 && lp[sel] == 0.f) --sel;
        }
        const kz_lobe& ls = mat.lobes[sel];
        LobeSample smp = sample_lobe(ls, wi, u[6], u[7], u[8]);
        if (!smp.valid) break;
        V3 weight;
        float pdf_dir;
        if (smp.delta) {
            weight = mul(weight_of(ls, mtex, tint), smp.weight) * (1.f / lp[sel]);
            pdf_dir = 0.f;
        } else {
            V3 f(0, 0, 0);
            float pdf = 0.f;
            for (uint32_t i = 0; i < nlobes; ++i) {
                const kz_lobe& lb = mat.lobes[i];
                if (lobe_is_delta(lb.closure_id)) continue;
                LobeEval e = eval_integrator(lb, wi, smp.wo);
                f = f + mul(weight_of(lb, mtex, tint), e.f);
                pdf += lp[i] * e.pdf;
            }
            if (!(pdf > 0.f)) break;
            weight = f * (1.f / pdf);
            pdf_dir = pdf;
        }
        beta = mul(beta, weight);
        if (is_zero(beta)) break;
        prev_pdf = pdf_dir;
        stale_mpdf = pdf_dir;
        prev_specular = smp.delta;
        o = P;
        d = normalize(fr.to_world(smp.wo));
    }
    return L;
}

int estimator_of(const kz_render_config* cfg) {
    return (cfg->flags & KZ_RENDER_FLAG_NEE_ONLY) ? 1 : (cfg->flags & KZ_RENDER_FLAG_BSDF_ONLY) ? 2 : 0;
}

}  // namespace

// =================================================================== C API
extern "C" {

void* kzo_bvh_build(const float* tri_verts, uint32_t ntris) {
    OBvh* b = new OBvh();
    b->ntris = ntris;
    b->verts.assign(tri_verts, tri_verts + (size_t)ntris * 9);
    b->build();
    return b;
}

void kzo_bvh_free(void* h) { delete static_cast<OBvh*>(h); }

void kzo_closest(void* h, const kz_ray* rays, uint64_t n, int nthreads, float* t, uint32_t* prim, float* u, float* v) {
    const OBvh* b = static_cast<const OBvh*>(h);
    parallel_for(n, nthreads, [&](uint64_t i) {
        const kz_ray& r = rays[i];
        float tt, uu = 0.f, vv = 0.f;
        uint32_t p;
        b->closest(V3(r.ox, r.oy, r.oz), V3(r.dx, r.dy, r.dz), r.tmin, r.tmax, tt, p, uu, vv);
        t[i] = tt;
        prim[i] = p;
        if (u) u[i] = p == KZ_INVALID_ID ? 0.f : uu;
        if (v) v[i] = p == KZ_INVALID_ID ? 0.f : vv;
    });
}

void kzo_any(void* h, const kz_ray* rays, uint64_t n, int nthreads, uint8_t* occ) {
    const OBvh* b = static_cast<const OBvh*>(h);
    parallel_for(n, nthreads, [&](uint64_t i) {
        const kz_ray& r = rays[i];
        occ[i] = b->any(V3(r.ox, r.oy, r.oz), V3(r.dx, r.dy, r.dz), r.tmin, r.tmax) ? 1 : 0;
    });
}

// Brute force over all triangles (small cases only): same tie rule.
void kzo_closest_brute(const float* tri_verts, uint32_t ntris, const kz_ray* rays, uint64_t n, float* t, uint32_t* prim) {
    for (uint64_t i = 0; i < n; ++i) {
        const kz_ray& r = rays[i];
        RayPre rp = ray_pre(V3(r.ox, r.oy, r.oz), V3(r.dx, r.dy, r.dz));
        float best = r.tmax;
        uint32_t bp = KZ_INVALID_ID;
        for (uint32_t k = 0; k < ntris; ++k) {
            const float* p = tri_verts + (size_t)k * 9;
            float tt, bu, bv;
            if (!tri_hit(rp, V3(p[0], p[1], p[2]), V3(p[3], p[4], p[5]), V3(p[6], p[7], p[8]), tt, bu, bv)) continue;
            if (!(tt > r.tmin) || !(tt <= r.tmax)) continue;
            if (tt < best || (tt == best && k < bp)) { best = tt; bp = k; }
        }
        t[i] = best;
        prim[i] = bp;
    }
}

void kzo_closure_eval(const kz_lobe* lobes, const float* wi, const float* wo, uint64_t n, int conv, float* f, float* pdf) {
    for (uint64_t i = 0; i < n; ++i) {
        V3 a(wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]), b(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]);
        LobeEval e = conv == KZ_CONVENTION_REFERENCE ? eval_reference<true>(lobes[i], a, b) : eval_integrator(lobes[i], a, b);
        f[3 * i] = e.f.x; f[3 * i + 1] = e.f.y; f[3 * i + 2] = e.f.z;
        pdf[i] = e.pdf;
    }
}

void kzo_closure_sample(const kz_lobe* lobes, const float* wi, const float* u, uint64_t n, float* wo, float* weight,
                        float* pdf, uint8_t* flags) {
    for (uint64_t i = 0; i < n; ++i) {
        V3 a(wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]);
        LobeSample s = sample_lobe(lobes[i], a, u[3 * i], u[3 * i + 1], u[3 * i + 2]);
        wo[3 * i] = s.wo.x; wo[3 * i + 1] = s.wo.y; wo[3 * i + 2] = s.wo.z;
        weight[3 * i] = s.weight.x; weight[3 * i + 1] = s.weight.y; weight[3 * i + 2] = s.weight.z;
        pdf[i] = s.pdf;
        flags[i] = (uint8_t)((s.valid ? 1 : 0) | (s.delta ? 2 : 0));
    }
}

// Microfacet white-furnace integrals, src/shading/white_furnace.{h,cpp}.
// weak test: sum over (theta, phi) grid of sin*D(h)*G1(h)/|4 V.y| (y-up).
double kzo_furnace_weak(int dist, float theta_deg, float alpha) {
    float th = theta_deg / 180.f * kPi;
    Mdf mdf;
    mdf.dist = dist;
    mdf.wi = V3(std::sin(th), std::cos(th), 0.f);
    mdf.ax = mdf.ay = alpha;
    V3 V = mdf.wi;
    float integral = 0.f;
    const float dth = 0.05f, dph = 0.05f;
    for (int i = 0; i * dth < kPi; ++i) {
        float theta = i * dth;
        float st = std::sin(theta), ct = std::cos(theta);
        for (int j = 0; j * dph < 2.f * kPi; ++j) {
            float phi = j * dph;
            float sp = std::sin(phi), cp = std::cos(phi);
            V3 Lv(cp * st, ct, sp * st);
            V3 H = normalize(V + Lv);
            integral += st * mdf.D(H) * mdf.G1(H) / std::fabs(4.f * V.y);
        }
    }
    return (double)(integral * dth * dph);
}

// fixed_beckmann_white_furnace_test(alpha, theta_o), white_furnace.cpp:3-36 (z-up)
double kzo_furnace_fixed_beckmann(float alpha, float theta_o) {
    float so = std::sin(theta_o), co = std::cos(theta_o);
    V3 V(so, 0.f, co);
    float a = 1.f / (alpha * std::tan(theta_o));
    float a2 = a * a;
    float lambda = 0.f;
    if (a < 1.6f) lambda = (1 - 1.259f * a + 0.396f * a2) / (3.535f * a + 2.181f * a2);
    float G = 1.f / (1.f + lambda);
    float integral = 0.f;
    const float dth = 0.05f, dph = 0.05f;
    for (int i = 0; i * dth < kPi; ++i) {
        float ti = i * dth;
        for (int j = 0; j * dph < 2.f * kPi; ++j) {
            float phi = j * dph;
            float si = std::sin(ti), ci = std::cos(ti), sp = std::sin(phi), cp = std::cos(phi);
            V3 Lv(cp * si, sp * si, ci);
            V3 H = normalize(V + Lv);
            if (H.z <= 0) continue;
            float th = std::acos(H.z);
            float D = std::exp(-std::pow(std::tan(th) / alpha, 2.f)) / (kPi * alpha * alpha * std::pow(H.z, 4.f));
            integral += si * D * G / std::fabs(4 * V.z);
        }
    }
    return (double)(integral * dth * dph);
}

void* kzo_scene_create(const float* tri_verts, uint32_t ntris, const uint32_t* tri_geom, const int32_t* geom_material,
                       const int32_t* geom_is_light, uint32_t ngeom, const kz_material* mats, uint32_t nmats) {
    OScene* s = new OScene();
    s->bvh.ntris = ntris;
    s->bvh.verts.assign(tri_verts, tri_verts + (size_t)ntris * 9);
    s->bvh.build();
    s->tri_geom.assign(tri_geom, tri_geom + ntris);
    s->geom_material.assign(geom_material, geom_material + ngeom);
    s->materials.assign(mats, mats + nmats);
    s->geom_light.assign(ngeom, -1);
    // one GeometryLight per emissive mesh, in mesh order; area CDF in triangle
    // order (TriangleMesh::setup_dpdf, shape.cpp:700-709)
    for (uint32_t g = 0; g < ngeom; ++g) {
        if (!geom_is_light[g]) continue;
        OLight lt;
        lt.geom = g;
        const kz_material& m = mats[geom_material[g]];
        lt.Le = V3(m.Le[0], m.Le[1], m.Le[2]);
        for (uint32_t k = 0; k < ntris; ++k)
            if (tri_geom[k] == g) lt.tris.push_back(k);
        if (lt.tris.empty()) continue;
        lt.cdf.push_back(0.f);
        for (uint32_t k : lt.tris) lt.cdf.push_back(lt.cdf.back() + tri_area(s->bvh, k));
        float sum = lt.cdf.back();
        lt.area = sum;
        if (sum > 0.f) {
            float nrm = 1.f / sum;
            for (size_t k = 1; k < lt.cdf.size(); ++k) lt.cdf[k] *= nrm;
            lt.cdf.back() = 1.f;
        }
        s->geom_light[g] = (int32_t)s->lights.size();
        s->lights.push_back(std::move(lt));
    }
    return s;
}

void kzo_scene_free(void* h) { delete static_cast<OScene*>(h); }

// Vertex normals per triangle (9 floats, global order) and a per-triangle
// flag (0: the mesh has none, shade with the geometric normal).
void kzo_scene_set_normals(void* h, const float* tri_nrm, const uint8_t* has) {
    OScene* s = static_cast<OScene*>(h);
    s->tri_nrm.assign(tri_nrm, tri_nrm + (size_t)s->bvh.ntris * 9);
    s->tri_has_nrm.assign(has, has + s->bvh.ntris);
}

// Point lights follow the area lights in the light list.
void kzo_scene_add_point_light(void* h, const float* position, const float* radiance) {
    OScene* s = static_cast<OScene*>(h);
    OLight lt;
    lt.geom = 0xffffffffu;
    lt.area = 0.f;
    lt.point = true;
    lt.pos = V3(position[0], position[1], position[2]);
    lt.Le = V3(radiance[0], radiance[1], radiance[2]);
    s->lights.push_back(std::move(lt));
}

// Textures, per-triangle vertex uvs (6 floats per triangle in global order,
// NULL = barycentrics) and the environment of a restatement scene.
void kzo_scene_set_textures(void* h, const kz_texture* tex, uint32_t n, const float* tri_uv, const float* env_rgb,
                            int32_t env_tex) {
    OScene* s = static_cast<OScene*>(h);
    s->textures.clear();
    for (uint32_t k = 0; k < n; ++k) {
        OTexture t;
        t.kind = tex[k].kind;
        t.w = tex[k].width;
        t.h = tex[k].height;
        if (t.kind == KZ_TEX_IMAGE) t.rgb.assign(tex[k].rgb, tex[k].rgb + (size_t)t.w * t.h * 3);
        t.scale_s = tex[k].scale_s;
        t.scale_t = tex[k].scale_t;
        t.Ca = V3(tex[k].Ca[0], tex[k].Ca[1], tex[k].Ca[2]);
        t.Cb = V3(tex[k].Cb[0], tex[k].Cb[1], tex[k].Cb[2]);
        s->textures.push_back(std::move(t));
    }
    if (tri_uv) s->tri_uv.assign(tri_uv, tri_uv + (size_t)s->bvh.ntris * 6);
    else s->tri_uv.clear();
    s->env = env_rgb ? V3(env_rgb[0], env_rgb[1], env_rgb[2]) : V3(0, 0, 0);
    s->env_tex = env_tex;
}

// Renders rows [row_begin, row_end) of a W x H frame; out: W*H*3 doubles
// (spp average, FP64 accumulation); stats[0] = path bounces, stats[1] = shadow rays.
void kzo_render_compat(void* h, const kz_camera* cam, uint32_t W, uint32_t H, const kz_render_config* cfg,
                       int nthreads, uint32_t row_begin, uint32_t row_end, uint32_t compat, double* out,
                       uint64_t* stats);
void kzo_render(void* h, const kz_camera* cam, uint32_t W, uint32_t H, const kz_render_config* cfg, int nthreads,
                uint32_t row_begin, uint32_t row_end, double* out, uint64_t* stats) {
    kzo_render_compat(h, cam, W, H, cfg, nthreads, row_begin, row_end, 0, out, stats);
}
// The frame with the path loop in a reference-as-written mode (COMPAT_* bits).
void kzo_render_compat(void* h, const kz_camera* cam, uint32_t W, uint32_t H, const kz_render_config* cfg,
                       int nthreads, uint32_t row_begin, uint32_t row_end, uint32_t compat, double* out,
                       uint64_t* stats) {
    const OScene* sc = static_cast<const OScene*>(h);
    CamBasis cb = cam_basis(*cam, W, H);
    row_end = std::min(row_end, H);
    const uint64_t npix = (uint64_t)(row_end - row_begin) * W;
    const uint32_t spp = cfg->spp;
    std::atomic<uint64_t> nb{0}, ns{0};
    parallel_for(npix, nthreads, [&](uint64_t i) {
        uint64_t pix = (uint64_t)row_begin * W + i;
        uint32_t px = (uint32_t)(pix % W), py = (uint32_t)(pix / W);
        double acc[3] = {0, 0, 0};
        PathCounters pc;
        for (uint32_t s = 0; s < spp; ++s) {
            Pcg32 rng;
            rng.seed(cfg->seed, pix * spp + s);
            float jx = rng.nextf(), jy = rng.nextf();
            V3 d = cam_dir(cb, px, py, W, H, jx, jy);
            V3 L = Li(*sc, cb.eye, d, rng, cfg->max_depth, cfg->rr_min_depth, pc, estimator_of(cfg), compat);
            acc[0] += L.x; acc[1] += L.y; acc[2] += L.z;
        }
        for (int c = 0; c < 3; ++c) out[pix * 3 + c] = acc[c] / (double)spp;
        nb += pc.bounces;
        ns += pc.shadow;
    });
    if (stats) {
        stats[0] = nb.load();
        stats[1] = ns.load();
    }
}

// Camera rays of a frame, exactly as the renderer generates them (first two
// draws of each stream); rays: W*H*spp records.
void kzo_camera_rays(const kz_camera* cam, uint32_t W, uint32_t H, uint32_t spp, uint64_t seed, kz_ray* rays) {
    CamBasis cb = cam_basis(*cam, W, H);
    for (uint64_t pix = 0; pix < (uint64_t)W * H; ++pix)
        for (uint32_t s = 0; s < spp; ++s) {
            Pcg32 rng;
            rng.seed(seed, pix * spp + s);
            float jx = rng.nextf(), jy = rng.nextf();
            V3 d = cam_dir(cb, (uint32_t)(pix % W), (uint32_t)(pix / W), W, H, jx, jy);
            kz_ray& r = rays[pix * spp + s];
            r.ox = cb.eye.x; r.oy = cb.eye.y; r.oz = cb.eye.z; r.tmin = kRayEps;
            r.dx = d.x; r.dy = d.y; r.dz = d.z; r.tmax = std::numeric_limits<float>::infinity();
        }
}

// Li of explicit rays; ray i uses PCG32 stream (seed, i).
void kzo_li(void* h, const kz_ray* rays, uint64_t n, const kz_render_config* cfg, int nthreads, double* out,
            uint64_t* stats) {
    const OScene* sc = static_cast<const OScene*>(h);
    std::atomic<uint64_t> nb{0}, ns{0};
    parallel_for(n, nthreads, [&](uint64_t i) {
        Pcg32 rng;
        rng.seed(cfg->seed, i);
        PathCounters pc;
        const kz_ray& r = rays[i];
        V3 L = Li(*sc, V3(r.ox, r.oy, r.oz), V3(r.dx, r.dy, r.dz), rng, cfg->max_depth, cfg->rr_min_depth, pc,
                  estimator_of(cfg));
        out[3 * i] = L.x; out[3 * i + 1] = L.y; out[3 * i + 2] = L.z;
        nb += pc.bounces;
        ns += pc.shadow;
    });
    if (stats) {
        stats[0] = nb.load();
        stats[1] = ns.load();
    }
}

// First 16 outputs of a PCG32 stream (known-answer check of the generator).
void kzo_pcg32_outputs(uint64_t initstate, uint64_t initseq, uint32_t* out, int n) {
    Pcg32 r;
    r.seed(initstate, initseq);
    for (int i = 0; i < n; ++i) out[i] = r.next();
}

// ---- the reference's own ray/triangle test (compat intersection mode)
// moller_trumbore_intersect, src/core/shape.cpp:373-408: single-sided (a
// determinant below 1e-6 misses, so back faces and grazing hits are culled),
// hits with t in [0, tmax]; u, v barycentrics of v1, v2.
bool moller_trumbore_ref(V3 o, V3 d, V3 v0, V3 v1, V3 v2, float tmax, float& t, float& u, float& v) {
    V3 v1v0 = v1 - v0, v2v0 = v2 - v0;
    V3 pvec = cross(d, v2v0);
    float det = dot(v1v0, pvec);
    if (det < 0.000001) return false;
    float det_inv = 1.f / det;
    V3 tvec = o - v0;
    u = dot(tvec, pvec) * det_inv;
    if (u < 0.f || u > 1.f) return false;
    V3 qvec = cross(tvec, v1v0);
    v = dot(d, qvec) * det_inv;
    if (v < 0.f || u + v > 1.f) return false;
    t = dot(v2v0, qvec) * det_inv;
    if (t < 0 || t > tmax) return false;
    return true;
}

// Rays against a triangle list with the reference's test. mode 0: the closest
// such hit (what a correct traversal over moller_trumbore_intersect gives);
// mode 1: TriangleMesh::intersect as written (shape.cpp:533-557), the first
// triangle in index order that the test accepts -- not the closest.
void kzo_mt_intersect(const float* tri_verts, uint32_t ntris, const kz_ray* rays, uint64_t n, int mode, float* t,
                      uint32_t* prim, float* u, float* v) {
    for (uint64_t i = 0; i < n; ++i) {
        const kz_ray& r = rays[i];
        V3 o(r.ox, r.oy, r.oz), d(r.dx, r.dy, r.dz);
        float best = std::numeric_limits<float>::infinity();
        uint32_t bp = KZ_INVALID_ID;
        float bu = 0.f, bv = 0.f;
        for (uint32_t k = 0; k < ntris; ++k) {
            const float* q = tri_verts + 9 * (size_t)k;
            float tt, uu, vv;
            if (!moller_trumbore_ref(o, d, V3(q[0], q[1], q[2]), V3(q[3], q[4], q[5]), V3(q[6], q[7], q[8]),
                                     mode == 1 ? r.tmax : best, tt, uu, vv))
                continue;
            if (mode == 1 || tt < best) {
                best = tt; bp = k; bu = uu; bv = vv;
                if (mode == 1) break;
            }
        }
        t[i] = best;
        prim[i] = bp;
        u[i] = bu;
        v[i] = bv;
    }
}

// ---- the restatement's scalar building blocks, for the known-answer vectors
// computed by the reference's own header code (oracle/ref_harness.cpp)

// in: n x 11 (wi, wo, m, ax, ay); out: n x 7 (D(m), lambda(wi), lambda(wo),
// G1(wi), G1(wo), G(wo), pdf(m)) of MicrofacetInterface (microfacet.h:215-291)
void kzo_mdf_terms(int dist, const float* in, uint64_t n, float* out) {
    for (uint64_t i = 0; i < n; ++i) {
        const float* a = in + 11 * i;
        Mdf m;
        m.dist = dist;
        m.wi = V3(a[0], a[1], a[2]);
        m.ax = a[9];
        m.ay = a[10];
        V3 wo(a[3], a[4], a[5]), h(a[6], a[7], a[8]);
        float* o = out + 7 * i;
        o[0] = m.D(h);
        o[1] = m.lambda(m.wi);
        o[2] = m.lambda(wo);
        o[3] = m.G1(m.wi);
        o[4] = m.G1(wo);
        o[5] = m.G(wo);
        o[6] = m.pdf(h);
    }
}

// in: n x 4 (cos, eta, ext, int); out: n x 4 (fresnel_refl_dielectric(eta, |cos|),
// fresnel(cos, ext, int), fresnel_schlick(eta, |cos|), schlick_weight(|cos|))
void kzo_fresnel_terms(const float* in, uint64_t n, float* out) {
    for (uint64_t i = 0; i < n; ++i) {
        const float* a = in + 4 * i;
        const float ac = std::fabs(a[0]);
        float* o = out + 4 * i;
        o[0] = fresnel_refl(a[1], ac);
        o[1] = fresnel_utils(a[0], a[2], a[3]);
        o[2] = fresnel_schlick_eta(a[1], ac);
        o[3] = schlick_weight(ac);
    }
}

// in: n x 7 (wi, n, eta); out: n x 3 refract(wi, n, eta) (utils.h:142-151)
void kzo_refract(const float* in, uint64_t n, float* out) {
    for (uint64_t i = 0; i < n; ++i) {
        const float* a = in + 7 * i;
        V3 t = refract_u(V3(a[0], a[1], a[2]), V3(a[3], a[4], a[5]), a[6]);
        out[3 * i] = t.x; out[3 * i + 1] = t.y; out[3 * i + 2] = t.z;
    }
}

// in: n x 6 (n, v); out: n x 9 (Frame(n).s, .t, to_local(v)) (utils.h:183-210)
void kzo_frame(const float* in, uint64_t n, float* out) {
    for (uint64_t i = 0; i < n; ++i) {
        const float* a = in + 6 * i;
        Frame f(V3(a[0], a[1], a[2]));
        V3 l = f.to_local(V3(a[3], a[4], a[5]));
        float* o = out + 9 * i;
        o[0] = f.s.x; o[1] = f.s.y; o[2] = f.s.z;
        o[3] = f.t.x; o[4] = f.t.y; o[5] = f.t.z;
        o[6] = l.x; o[7] = l.y; o[8] = l.z;
    }
}

// in: n x 4 (u1, u2, a, b); out: n x 4 (cosine_dir(u2, u1) in the y-up frame,
// power_heuristic(1, a, 1, b)) -- the cosine warp with the disk mapping of
// to_uniform_disk / to_cosine_hemisphere (sampling.h:66-108), which returns
// its cosine in z
void kzo_warps(const float* in, uint64_t n, float* out) {
    for (uint64_t i = 0; i < n; ++i) {
        const float* a = in + 4 * i;
        V3 c = cosine_dir(a[1], a[0]);
        float* o = out + 4 * i;
        o[0] = c.x; o[1] = c.y; o[2] = c.z;
        o[3] = power_heuristic(a[2], a[3]);
    }
}

}  // extern "C"
