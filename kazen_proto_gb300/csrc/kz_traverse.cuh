// kz_traverse.cuh — BVH traversal and watertight ray/triangle test (device).
//
// Replaces EmbreeAccel::intersect / occluded (src/core/accel.cpp:348-432,
// src/core/hitable.h:25-33) and the Moller-Trumbore routine
// (src/core/shape.cpp:373-450) with:
//  * the watertight test of S. Woop, C. Benthin, I. Wald, "Watertight
//    Ray/Triangle Intersection", JCGT 2(1), 2013 — double-sided, double
//    precision fallback when an edge function is exactly zero;
//  * closest hit in (tmin, tmax], equal t resolved to the smaller global
//    triangle id, so the result is independent of traversal order and of the
//    BVH shape (bit-exact against any exact restatement);
//  * a binary BVH with both child boxes in one 64-byte node, read with
//    16-byte non-coherent loads, near-child-first order and a short stack of
//    (node, entry distance) pairs in local memory.
// Box distances are widened by a relative margin far above their rounding
// error, so no box holding a hit at t <= t_best is culled.
#pragma once

#include "kz_device.cuh"

namespace kz {

constexpr int kStackSize = 64;
constexpr float kBoxLo = 1.0f - 1.0f / 65536.0f;
constexpr float kBoxHi = 1.0f + 1.0f / 65536.0f;

struct TRay {
    f3 o, inv;
    float tmin;
    int kx, ky, kz;
    float Sx, Sy, Sz;
};

__device__ __forceinline__ float safe_inv(float c) {
    if (fabsf(c) < 1e-30f) c = copysignf(1e-30f, c);
    return 1.0f / c;
}

__device__ __forceinline__ TRay make_tray(f3 o, f3 d, float tmin) {
    TRay r;
    r.o = o;
    r.tmin = tmin;
    r.inv = mk(safe_inv(d.x), safe_inv(d.y), safe_inv(d.z));
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    int kz = 0;
    float m = ax;
    if (ay > m) { kz = 1; m = ay; }
    if (az > m) { kz = 2; }
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    float dz = comp(d, kz);
    if (dz < 0.f) { int t = kx; kx = ky; ky = t; }
    r.kx = kx; r.ky = ky; r.kz = kz;
    r.Sx = comp(d, kx) / dz;
    r.Sy = comp(d, ky) / dz;
    r.Sz = 1.0f / dz;
    return r;
}

__device__ __forceinline__ float pick(float4 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

// Watertight test against a triangle record; t, u, v valid when it returns true.
__device__ __forceinline__ bool tri_test(const TRay& r, float4 a, float4 b, float4 c, float& t, float& bu, float& bv) {
    const float okx = comp(r.o, r.kx), oky = comp(r.o, r.ky), okz = comp(r.o, r.kz);
    const float Akx = pick(a, r.kx) - okx, Aky = pick(a, r.ky) - oky, Akz = pick(a, r.kz) - okz;
    const float Bkx = pick(b, r.kx) - okx, Bky = pick(b, r.ky) - oky, Bkz = pick(b, r.kz) - okz;
    const float Ckx = pick(c, r.kx) - okx, Cky = pick(c, r.ky) - oky, Ckz = pick(c, r.kz) - okz;
    const float Ax = Akx - r.Sx * Akz, Ay = Aky - r.Sy * Akz;
    const float Bx = Bkx - r.Sx * Bkz, By = Bky - r.Sy * Bkz;
    const float Cx = Ckx - r.Sx * Ckz, Cy = Cky - r.Sy * Ckz;
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
    const float T = U * (r.Sz * Akz) + V * (r.Sz * Bkz) + W * (r.Sz * Ckz);
    t = T / det;
    bu = V / det;
    bv = W / det;
    return true;
}

__device__ __forceinline__ bool box_test(float lx, float hx, float ly, float hy, float lz, float hz, const TRay& r,
                                         float tcur, float& tnear) {
    const float tx0 = (lx - r.o.x) * r.inv.x, tx1 = (hx - r.o.x) * r.inv.x;
    const float ty0 = (ly - r.o.y) * r.inv.y, ty1 = (hy - r.o.y) * r.inv.y;
    const float tz0 = (lz - r.o.z) * r.inv.z, tz1 = (hz - r.o.z) * r.inv.z;
    float tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fminf(tz0, tz1));
    float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fmaxf(tz0, tz1));
    tn *= tn > 0.f ? kBoxLo : kBoxHi;
    tf *= tf > 0.f ? kBoxHi : kBoxLo;
    tnear = fmaxf(tn, r.tmin);
    return tnear <= fminf(tf, tcur);
}

struct HitRec {
    float t, u, v;
    uint32_t prim;  // global triangle id, KZ_INVALID_ID on a miss
    int32_t rec;    // triangle record, -1 on a miss
};

template <bool kCount>
__device__ __forceinline__ void leaf_closest(const float4* __restrict__ tris, const TRay& r, int first, int count,
                                             HitRec& h, uint32_t& ntri) {
    for (int k = 0; k < count; ++k) {
        const float4* tp = tris + (size_t)(first + k) * 3;
        const float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
        if (kCount) ++ntri;
        float t, bu, bv;
        if (!tri_test(r, a, b, c, t, bu, bv)) continue;
        const uint32_t prim = __float_as_uint(a.w);
        if (t > r.tmin && (t < h.t || (t == h.t && prim < h.prim))) {
            h.t = t;
            h.u = bu;
            h.v = bv;
            h.prim = prim;
            h.rec = first + k;
        }
    }
}

// Closest hit. Returns false only if the stack would overflow (ruled out by
// the builder's depth cap) or more nodes are visited than the tree holds (a
// corrupt node array); the caller reports KZ_ERR_STACK and the ray misses.
template <bool kCount>
__device__ bool trace_closest(const DevScene& s, const TRay& r, float tmax, HitRec& h, uint32_t& nnode,
                              uint32_t& ntri) {
    h.t = tmax;
    h.u = h.v = 0.f;
    h.prim = KZ_INVALID_ID;
    h.rec = -1;
    int stack_node[kStackSize];
    float stack_t[kStackSize];
    int sp = 0;
    int node = 0;
    uint32_t visits = 0;
    for (;;) {
        if (++visits > s.n_nodes || (uint32_t)node >= s.n_nodes) return false;
        const float4* np = s.nodes + (size_t)node * 4;
        const float4 n0 = __ldg(np), n1 = __ldg(np + 1), n2 = __ldg(np + 2);
        const int4 n3 = __ldg(reinterpret_cast<const int4*>(np + 3));
        if (kCount) ++nnode;
        float tn0, tn1;
        const bool h0 = box_test(n0.x, n0.y, n0.z, n0.w, n2.x, n2.y, r, h.t, tn0);
        const bool h1 = box_test(n1.x, n1.y, n1.z, n1.w, n2.z, n2.w, r, h.t, tn1);
        if (h0 && n3.x < 0) leaf_closest<kCount>(s.tris, r, ~n3.x, n3.z, h, ntri);
        if (h1 && n3.y < 0) leaf_closest<kCount>(s.tris, r, ~n3.y, n3.w, h, ntri);
        const bool g0 = h0 && n3.x >= 0 && tn0 <= h.t;
        const bool g1 = h1 && n3.y >= 0 && tn1 <= h.t;
        if (g0 && g1) {
            int near = n3.x, far = n3.y;
            float tfar = tn1;
            if (tn1 < tn0) {
                near = n3.y;
                far = n3.x;
                tfar = tn0;
            }
            if (sp >= kStackSize) return false;
            stack_node[sp] = far;
            stack_t[sp] = tfar;
            ++sp;
            node = near;
            continue;
        }
        if (g0) { node = n3.x; continue; }
        if (g1) { node = n3.y; continue; }
        for (;;) {
            if (sp == 0) return true;
            --sp;
            if (stack_t[sp] <= h.t) break;
        }
        node = stack_node[sp];
    }
}

// Any hit in (tmin, tmax].
template <bool kCount>
__device__ bool trace_any(const DevScene& s, const TRay& r, float tmax, bool& overflow, uint32_t& nnode,
                          uint32_t& ntri) {
    int stack_node[kStackSize];
    int sp = 0;
    int node = 0;
    uint32_t visits = 0;
    overflow = false;
    for (;;) {
        if (++visits > s.n_nodes || (uint32_t)node >= s.n_nodes) {
            overflow = true;
            return false;
        }
        const float4* np = s.nodes + (size_t)node * 4;
        const float4 n0 = __ldg(np), n1 = __ldg(np + 1), n2 = __ldg(np + 2);
        const int4 n3 = __ldg(reinterpret_cast<const int4*>(np + 3));
        if (kCount) ++nnode;
        float tn0, tn1;
        const bool h0 = box_test(n0.x, n0.y, n0.z, n0.w, n2.x, n2.y, r, tmax, tn0);
        const bool h1 = box_test(n1.x, n1.y, n1.z, n1.w, n2.z, n2.w, r, tmax, tn1);
        for (int side = 0; side < 2; ++side) {
            const bool hit = side ? h1 : h0;
            const int link = side ? n3.y : n3.x;
            const int cnt = side ? n3.w : n3.z;
            if (!hit || link >= 0) continue;
            const int first = ~link;
            for (int k = 0; k < cnt; ++k) {
                const float4* tp = s.tris + (size_t)(first + k) * 3;
                if (kCount) ++ntri;
                float t, bu, bv;
                if (tri_test(r, __ldg(tp), __ldg(tp + 1), __ldg(tp + 2), t, bu, bv) && t > r.tmin && t <= tmax)
                    return true;
            }
        }
        const bool g0 = h0 && n3.x >= 0;
        const bool g1 = h1 && n3.y >= 0;
        if (g0 && g1) {
            if (sp >= kStackSize) {
                overflow = true;
                return false;
            }
            stack_node[sp++] = n3.y;
            node = n3.x;
            continue;
        }
        if (g0) { node = n3.x; continue; }
        if (g1) { node = n3.y; continue; }
        if (sp == 0) return false;
        node = stack_node[--sp];
    }
}

}  // namespace kz
