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
//  * an 8-wide BVH with quantized child boxes (80-byte nodes, five 16-byte
//    non-coherent loads), in the manner of H. Ylitie, T. Karras, S. Laine,
//    "Efficient Incoherent Ray Traversal on GPUs Through Compressed Wide
//    BVHs", HPG 2017: one node test yields a 32-bit mask of inner children
//    (in an octant-derived near-first order) and leaf triangles; a stack of
//    (child base, mask) groups in local memory.
// Box distances are widened by a margin above their rounding error (see
// wide_axis), so no box holding a hit at t <= t_best is culled.
#pragma once

#include "kz_bvh.h"
#include "kz_device.cuh"

namespace kz {

static_assert(kWideWords == 20, "a wide node is five 16-byte vectors");

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

// The per-ray terms of the watertight test: the origin in the permuted axes
// (kx, ky, kz), the shear and the ray's lower bound.
struct TriRay {
    float okx, oky, okz, tmin;
    float Sx, Sy, Sz;
    int kx, ky, kz;
};

__device__ __forceinline__ TriRay tri_ray(const TRay& r) {
    TriRay q;
    q.okx = comp(r.o, r.kx);
    q.oky = comp(r.o, r.ky);
    q.okz = comp(r.o, r.kz);
    q.tmin = r.tmin;
    q.Sx = r.Sx;
    q.Sy = r.Sy;
    q.Sz = r.Sz;
    q.kx = r.kx;
    q.ky = r.ky;
    q.kz = r.kz;
    return q;
}

// The same test with the barycentric divisions left to the caller:
// u = V / det, v = W / det for the hit that is kept.
__device__ __forceinline__ bool tri_test_t(const TriRay& r, float4 a, float4 b, float4 c, float& t, float& V_,
                                           float& W_, float& det_) {
    const float okx = r.okx, oky = r.oky, okz = r.okz;
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
    V_ = V;
    W_ = W;
    det_ = det;
    return true;
}
__device__ __forceinline__ bool tri_test_t(const TRay& r, float4 a, float4 b, float4 c, float& t, float& V_, float& W_,
                                           float& det_) {
    return tri_test_t(tri_ray(r), a, b, c, t, V_, W_, det_);
}

struct HitRec {
    float t, u, v;
    uint32_t prim;  // global triangle id, KZ_INVALID_ID on a miss
    int32_t rec;    // triangle record, -1 on a miss
};

// ---- 8-wide quantized BVH (layout in kz_bvh.h) ------------------------------
//
// A child box plane at p + q * 2^E on one axis is reached at
//   t(q) = (p + q 2^E - o) / d = b + q 2^E inv,  b = (p - o) inv.
// The byte q becomes f = 1 + q 2^-15 with one byte permute (0x3F80_qq00 as
// float bits), so t(q) = fma(f, A, B) with A = 2^(E+15) inv (exact: a power
// of two times inv) and B = b - A. Each term carries rounding error below
// 2^-24 (6 |b| + 3 |A|); the per-node margin 2^-16 (|b| + |A| / 32) exceeds it,
// so the near plane is lowered and the far plane raised by more than any
// rounding and no box holding a hit at t <= t_best is culled. An overflowing
// A or b turns the axis' distances into NaN, which the min/max below ignore:
// such an axis culls nothing.
struct WideAxis {
    float A, Bn, Bf;
    uint32_t n0, n1, f0, f1;  // near / far plane bytes (slots 0-3, 4-7)
};

__device__ __forceinline__ WideAxis wide_axis(float p, uint32_t e, float o, float inv, uint4 q) {
    WideAxis ax;
    ax.A = __uint_as_float((e + 15u) << 23) * inv;
    const float b = (p - o) * inv;
    const float B = b - ax.A;
    const float d = (fabsf(b) + fabsf(ax.A) * 0.03125f) * 1.52587890625e-05f;
    ax.Bn = B - d;
    ax.Bf = B + d;
    const bool neg = inv < 0.f;  // entering through the high plane
    ax.n0 = neg ? q.z : q.x;
    ax.n1 = neg ? q.w : q.y;
    ax.f0 = neg ? q.x : q.z;
    ax.f1 = neg ? q.y : q.w;
    return ax;
}

template <int kSlot>
__device__ __forceinline__ float wide_t(const WideAxis& ax, bool near_plane) {
    const uint32_t w = near_plane ? (kSlot < 4 ? ax.n0 : ax.n1) : (kSlot < 4 ? ax.f0 : ax.f1);
    const float f = __uint_as_float(__byte_perm(w, 0x3F800000u, 0x7604u | ((kSlot & 3) << 4)));
    return fmaf(f, ax.A, near_plane ? ax.Bn : ax.Bf);
}

// KZ_MINMAX3: the slot test's entry / exit distances through three-input
// min.f32 / max.f32 (sm_100 and later; bit-identical to the fminf / fmaxf
// chains on every combination of NaN, infinities, signed zeros, denormals and
// finite values). Measured on the terrain frame: 1,764 against 1,778
// Mpaths*bounces/s for the chains, which take the ray's bound first.
#ifndef KZ_MINMAX3
#define KZ_MINMAX3 0
#endif
__device__ __forceinline__ float max3f(float a, float b, float c) {
#if KZ_MINMAX3
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
#else
    return fmaxf(fmaxf(a, b), c);
#endif
}
__device__ __forceinline__ float min3f(float a, float b, float c) {
#if KZ_MINMAX3
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
#else
    return fminf(fminf(a, b), c);
#endif
}

template <int kSlot>
__device__ __forceinline__ void wide_slot(const WideAxis& X, const WideAxis& Y, const WideAxis& Z, uint32_t meta,
                                          float tmin, float tcur, uint32_t& hits) {
    const float tn = max3f(fmaxf(wide_t<kSlot>(X, true), tmin), wide_t<kSlot>(Y, true), wide_t<kSlot>(Z, true));
    const float tf = min3f(fminf(wide_t<kSlot>(X, false), tcur), wide_t<kSlot>(Y, false), wide_t<kSlot>(Z, false));
    const uint32_t m = (meta >> (8 * (kSlot & 3))) & 0xFFu;
    if (tn <= tf) hits |= (m >> 5) << (m & 31u);
}

// Tests the 8 child boxes of a node. Returns the hit mask: bits 24-31 the
// inner children in visiting order (bit 31 first), bits 0-23 the triangles
// (relative to tri_base) of the leaves hit.
__device__ __forceinline__ uint32_t wide_node(const uint4* __restrict__ np, const TRay& r, uint32_t octp, float tcur,
                                              uint32_t& child_base, uint32_t& tri_base, uint32_t& imask) {
    const uint4 h0 = __ldg(np), h1 = __ldg(np + 1);
    const uint4 qx = __ldg(np + 2), qy = __ldg(np + 3), qz = __ldg(np + 4);
    child_base = h1.x;
    tri_base = h1.y;
    imask = h0.w >> 24;
    const WideAxis X = wide_axis(__uint_as_float(h0.x), h0.w & 0xFFu, r.o.x, r.inv.x, qx);
    const WideAxis Y = wide_axis(__uint_as_float(h0.y), (h0.w >> 8) & 0xFFu, r.o.y, r.inv.y, qy);
    const WideAxis Z = wide_axis(__uint_as_float(h0.z), (h0.w >> 16) & 0xFFu, r.o.z, r.inv.z, qz);
    // inner slots carry 24 + slot in their low bits; XOR the ray's octant in
    // so that the nearest octant lands on bit 31
    uint32_t m0 = h1.z, m1 = h1.w;
    m0 ^= ((m0 >> 4) & (m0 >> 3) & 0x01010101u) * octp;
    m1 ^= ((m1 >> 4) & (m1 >> 3) & 0x01010101u) * octp;
    uint32_t hits = 0;
    wide_slot<0>(X, Y, Z, m0, r.tmin, tcur, hits);
    wide_slot<1>(X, Y, Z, m0, r.tmin, tcur, hits);
    wide_slot<2>(X, Y, Z, m0, r.tmin, tcur, hits);
    wide_slot<3>(X, Y, Z, m0, r.tmin, tcur, hits);
    wide_slot<4>(X, Y, Z, m1, r.tmin, tcur, hits);
    wide_slot<5>(X, Y, Z, m1, r.tmin, tcur, hits);
    wide_slot<6>(X, Y, Z, m1, r.tmin, tcur, hits);
    wide_slot<7>(X, Y, Z, m1, r.tmin, tcur, hits);
    return hits;
}

// XOR mask that maps a slot to its visiting rank: 7 for the octant the ray
// enters first (slot bits set on the axes whose direction is negative).
__device__ __forceinline__ uint32_t wide_octant(const TRay& r) {
    return 7u ^ ((r.inv.x < 0.f ? 1u : 0u) | (r.inv.y < 0.f ? 2u : 0u) | (r.inv.z < 0.f ? 4u : 0u));
}

// Next inner child of a node group (base, bits): bits 24-31 the remaining
// hits in visiting order, bits 0-7 the node's inner-slot mask.
__device__ __forceinline__ uint32_t wide_pop_child(uint32_t base, uint32_t& bits, uint32_t octp) {
    const uint32_t pos = 31u - __clz(bits);
    bits ^= 1u << pos;
    const uint32_t slot = (pos - 24u) ^ octp;
    return base + __popc(bits & ((1u << slot) - 1u));
}

// Traversal stack of node groups: a per-thread local array (LocalStack), or
// its first kSmem entries in shared memory, entry i of thread t at
// i * blockDim.x + t, and the rest local (SplitStack).
struct LocalStack {
    uint2* p;
    __device__ __forceinline__ uint2 get(int i) const { return p[i]; }
    __device__ __forceinline__ void put(int i, uint2 e) const { p[i] = e; }
};
template <int kSmem>
struct SplitStack {
    uint2* sm;
    uint2* lm;
    __device__ __forceinline__ uint2 get(int i) const {
        return i < kSmem ? sm[i * blockDim.x + threadIdx.x] : lm[i - kSmem];
    }
    __device__ __forceinline__ void put(int i, uint2 e) const {
        if (i < kSmem) sm[i * blockDim.x + threadIdx.x] = e;
        else lm[i - kSmem] = e;
    }
};

// Closest-hit traversal state, advanced one node at a time (closest_step) so
// that persistent kernels can interleave rays; trace_closest runs it to the
// end. The barycentric divisions are deferred to closest_finish (the same
// IEEE divisions as tri_test, for the kept hit only).
struct ClosestState {
    float t, V, W, det;
    uint32_t prim;
    int32_t rec;
    uint32_t gbase, gbits;  // current node group
    uint32_t visits;
    int sp;
};

__device__ __forceinline__ void closest_begin(ClosestState& c, float tmax) {
    c.t = tmax;
    c.V = c.W = 0.f;
    c.det = 1.f;
    c.prim = KZ_INVALID_ID;
    c.rec = -1;
    c.gbase = 0;
    c.gbits = 0x80000000u;  // the root as the only child of a virtual node
    c.visits = 0;
    c.sp = 0;
}

// Visits one node and tests its leaf triangles. Returns 0 while nodes remain,
// 1 when the traversal is complete, -1 if it must abort: the stack would
// overflow (the builder bounds the depth by the stack size), more nodes are
// visited than the tree holds, or a record index is out of range (a corrupt
// node array).
template <bool kCount, typename Stack>
__device__ __forceinline__ int closest_step(const DevScene& s, const TRay& r, uint32_t octp, ClosestState& c,
                                            const Stack& stack, uint32_t& nnode, uint32_t& ntri) {
    const uint32_t node = wide_pop_child(c.gbase, c.gbits, octp);
    if (c.gbits > 0x00FFFFFFu) {
        if (c.sp >= kWideStack) return -1;
        stack.put(c.sp++, make_uint2(c.gbase, c.gbits));
    }
    if (++c.visits > s.n_nodes || node >= s.n_nodes) return -1;
    uint32_t tri_base, imask;
    const uint32_t hm = wide_node(s.nodes + (size_t)node * 5, r, octp, c.t, c.gbase, tri_base, imask);
    if (kCount) ++nnode;
    c.gbits = (hm & 0xFF000000u) | imask;
    uint32_t tbits = hm & 0x00FFFFFFu;
    while (tbits) {
        const uint32_t rec = tri_base + (__ffs(tbits) - 1);
        tbits &= tbits - 1u;
        if (rec >= s.n_tris) return -1;
        const float4* tp = s.tris + (size_t)rec * 3;
        const float4 a = __ldg(tp), b = __ldg(tp + 1), cc = __ldg(tp + 2);
        if (kCount) ++ntri;
        float t, V, W, det;
        if (!tri_test_t(r, a, b, cc, t, V, W, det)) continue;
        const uint32_t prim = __float_as_uint(a.w);
        if (t > r.tmin && (t < c.t || (t == c.t && prim < c.prim))) {
            c.t = t;
            c.V = V;
            c.W = W;
            c.det = det;
            c.prim = prim;
            c.rec = (int32_t)rec;
        }
    }
    while (c.gbits <= 0x00FFFFFFu && c.sp > 0) {
        const uint2 e = stack.get(--c.sp);
        c.gbase = e.x;
        c.gbits = e.y;
    }
    return c.gbits <= 0x00FFFFFFu ? 1 : 0;
}

// Hit record of a finished traversal; an aborted one (ok == false) misses.
__device__ __forceinline__ void closest_finish(const ClosestState& c, bool ok, float tmax, HitRec& h) {
    if (!ok || c.rec < 0) {
        h.t = ok ? c.t : tmax;
        h.u = h.v = 0.f;
        h.prim = KZ_INVALID_ID;
        h.rec = -1;
        return;
    }
    h.t = c.t;
    h.u = c.V / c.det;
    h.v = c.W / c.det;
    h.prim = c.prim;
    h.rec = c.rec;
}

// Closest hit in (tmin, tmax]. Returns false if the traversal aborted
// (closest_step == -1); the caller reports KZ_ERR_STACK and the ray misses.
template <bool kCount>
__device__ bool trace_closest(const DevScene& s, const TRay& r, float tmax, HitRec& h, uint32_t& nnode,
                              uint32_t& ntri) {
    const uint32_t octp = wide_octant(r);
    uint2 stack[kWideStack];
    ClosestState c;
    closest_begin(c, tmax);
    int rc;
    do {
        rc = closest_step<kCount>(s, r, octp, c, LocalStack{stack}, nnode, ntri);
    } while (rc == 0);
    closest_finish(c, rc > 0, tmax, h);
    return rc > 0;
}

// Any-hit traversal state, advanced one node at a time like ClosestState.
struct AnyState {
    uint32_t gbase, gbits;
    uint32_t visits;
    int sp;
};

__device__ __forceinline__ void any_begin(AnyState& c) {
    c.gbase = 0;
    c.gbits = 0x80000000u;
    c.visits = 0;
    c.sp = 0;
}

// One node of an any-hit query in (tmin, tmax]: 0 while nodes remain, 1 no
// hit (complete), 2 hit, -1 abort (as closest_step).
template <bool kCount, typename Stack>
__device__ __forceinline__ int any_step(const DevScene& s, const TRay& r, uint32_t octp, float tmax, AnyState& c,
                                        const Stack& stack, uint32_t& nnode, uint32_t& ntri) {
    const uint32_t node = wide_pop_child(c.gbase, c.gbits, octp);
    if (c.gbits > 0x00FFFFFFu) {
        if (c.sp >= kWideStack) return -1;
        stack.put(c.sp++, make_uint2(c.gbase, c.gbits));
    }
    if (++c.visits > s.n_nodes || node >= s.n_nodes) return -1;
    uint32_t tri_base, imask;
    const uint32_t hm = wide_node(s.nodes + (size_t)node * 5, r, octp, tmax, c.gbase, tri_base, imask);
    if (kCount) ++nnode;
    c.gbits = (hm & 0xFF000000u) | imask;
    uint32_t tbits = hm & 0x00FFFFFFu;
    while (tbits) {
        const uint32_t rec = tri_base + (__ffs(tbits) - 1);
        tbits &= tbits - 1u;
        if (rec >= s.n_tris) return -1;
        const float4* tp = s.tris + (size_t)rec * 3;
        if (kCount) ++ntri;
        float t, V, W, det;
        if (tri_test_t(r, __ldg(tp), __ldg(tp + 1), __ldg(tp + 2), t, V, W, det) && t > r.tmin && t <= tmax)
            return 2;
    }
    while (c.gbits <= 0x00FFFFFFu && c.sp > 0) {
        const uint2 e = stack.get(--c.sp);
        c.gbase = e.x;
        c.gbits = e.y;
    }
    return c.gbits <= 0x00FFFFFFu ? 1 : 0;
}

// Any hit in (tmin, tmax]; `overflow` is set when the traversal aborted
// (any_step == -1; the caller reports KZ_ERR_STACK).
template <bool kCount>
__device__ bool trace_any(const DevScene& s, const TRay& r, float tmax, bool& overflow, uint32_t& nnode,
                          uint32_t& ntri) {
    const uint32_t octp = wide_octant(r);
    uint2 stack[kWideStack];
    AnyState c;
    any_begin(c);
    int rc;
    do {
        rc = any_step<kCount>(s, r, octp, tmax, c, LocalStack{stack}, nnode, ntri);
    } while (rc == 0);
    overflow = rc < 0;
    return rc == 2;
}

// ---- warp-shared leaf tests ---------------------------------------------------
//
// In the persistent kernels a traversal step is split into a node part (the
// lane's node test; its leaf triangles are left pending), a warp-wide part in
// which all 32 lanes, busy or idle, test the pending (ray, triangle) pairs of
// the whole warp, 32 at a time, and a pop of the next node group. A per-lane
// triangle loop would run for the warp's largest leaf count with a few lanes
// active; sharing the pairs spreads them over the warp.
//
// Each lane publishes its ray (TriRay) in shared memory when it starts one.
// The closest hit of a step is exact and independent of which lane tested
// what: candidates are combined by a 64-bit atomicMin of (t in a total order,
// global triangle id) on the owner's slot, the lexicographic minimum that the
// sequential loop keeps (smaller t, then smaller id), then the lane whose
// candidate won writes its record, its unrounded t and the barycentric terms.
struct LeafShare {
    float4* ray;              // [2 * 256]: (okx, oky, okz, tmin), (Sx, Sy, Sz, kx | ky << 2 | kz << 4)
    unsigned long long* key;  // [256] closest: best (t, id); any hit: tmax bits
    uint32_t* rec;            // [256] closest: record of the best; any hit: mask of the triangles hit
    float4* vwdt;             // [256] closest: V, W, det, t of the best
};

__device__ __forceinline__ void publish_ray(const LeafShare& sh, const TRay& r) {
    const TriRay q = tri_ray(r);
    sh.ray[2 * threadIdx.x] = make_float4(q.okx, q.oky, q.okz, q.tmin);
    sh.ray[2 * threadIdx.x + 1] =
        make_float4(q.Sx, q.Sy, q.Sz, __uint_as_float((uint32_t)q.kx | ((uint32_t)q.ky << 2) | ((uint32_t)q.kz << 4)));
}

__device__ __forceinline__ TriRay shared_ray(const LeafShare& sh, uint32_t slot) {
    const float4 a = sh.ray[2 * slot], b = sh.ray[2 * slot + 1];
    const uint32_t k = __float_as_uint(b.w);
    TriRay q;
    q.okx = a.x;
    q.oky = a.y;
    q.okz = a.z;
    q.tmin = a.w;
    q.Sx = b.x;
    q.Sy = b.y;
    q.Sz = b.z;
    q.kx = (int)(k & 3u);
    q.ky = (int)((k >> 2) & 3u);
    q.kz = (int)((k >> 4) & 3u);
    return q;
}

// (t, id) as one 64-bit key whose unsigned order is float order of t (-0 as
// +0), then id.
__device__ __forceinline__ unsigned long long hit_key(float t, uint32_t prim) {
    const uint32_t u = __float_as_uint(t == 0.f ? 0.f : t);
    const uint32_t o = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
    return ((unsigned long long)o << 32) | prim;
}

// Position of the (k+1)-th set bit of m (k < popc(m), m below bit 31).
__device__ __forceinline__ uint32_t nth_set_bit(uint32_t m, uint32_t k) {
    uint32_t pos = 0;
#pragma unroll
    for (uint32_t s = 16; s; s >>= 1)
        if ((uint32_t)__popc(m & ((1u << (pos + s)) - 1u)) <= k) pos += s;
    return pos;
}

// Assignment of pair p (0 <= p < total) of a warp whose lanes hold cnt pairs
// each (inclusive prefix incl): the owner lane and the owner's bit. Every
// lane must call it (full-warp shuffles).
struct LeafPair {
    uint32_t owner, bit, rec;
};
__device__ __forceinline__ LeafPair leaf_pair(uint32_t p, uint32_t incl, uint32_t cnt, uint32_t tbits, uint32_t tbase) {
    uint32_t o = 0;
#pragma unroll
    for (uint32_t s = 16; s; s >>= 1) {
        const uint32_t v = __shfl_sync(0xFFFFFFFFu, incl, o + s - 1);
        if (v <= p) o += s;
    }
    const uint32_t o_incl = __shfl_sync(0xFFFFFFFFu, incl, o);
    const uint32_t o_cnt = __shfl_sync(0xFFFFFFFFu, cnt, o);
    const uint32_t o_bits = __shfl_sync(0xFFFFFFFFu, tbits, o);
    const uint32_t o_base = __shfl_sync(0xFFFFFFFFu, tbase, o);
    LeafPair lp;
    lp.owner = o;
    lp.bit = nth_set_bit(o_bits, p - (o_incl - o_cnt));
    lp.rec = o_base + lp.bit;
    return lp;
}

// Lane's pair count and its inclusive prefix over the warp; returns the total.
__device__ __forceinline__ uint32_t leaf_scan(uint32_t tbits, uint32_t& cnt, uint32_t& incl) {
    const uint32_t lane = threadIdx.x & 31u;
    cnt = __popc(tbits);
    incl = cnt;
#pragma unroll
    for (uint32_t o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o) incl += v;
    }
    return __shfl_sync(0xFFFFFFFFu, incl, 31);
}

// Node part of a closest-hit step: visits one node; its leaf triangles are
// returned in tbits (relative to tbase) for the warp-wide test. Returns -1 on
// an abort (as closest_step), else 0.
template <bool kCount, typename Stack>
__device__ __forceinline__ int closest_node(const DevScene& s, const TRay& r, uint32_t octp, ClosestState& c,
                                            const Stack& stack, uint32_t& tbits, uint32_t& tbase, uint32_t& nnode,
                                            uint32_t& ntri) {
    const uint32_t node = wide_pop_child(c.gbase, c.gbits, octp);
    if (c.gbits > 0x00FFFFFFu) {
        if (c.sp >= kWideStack) return -1;
        stack.put(c.sp++, make_uint2(c.gbase, c.gbits));
    }
    if (++c.visits > s.n_nodes || node >= s.n_nodes) return -1;
    uint32_t imask;
    const uint32_t hm = wide_node(s.nodes + (size_t)node * 5, r, octp, c.t, c.gbase, tbase, imask);
    if (kCount) ++nnode;
    c.gbits = (hm & 0xFF000000u) | imask;
    const uint32_t tb = hm & 0x00FFFFFFu;
    if (tb && (uint64_t)tbase + (31u - __clz(tb)) >= s.n_tris) return -1;
    if (kCount) ntri += __popc(tb);
    tbits = tb;
    return 0;
}

// Next node group from the stack: 1 when the traversal is complete, else 0.
template <typename State, typename Stack>
__device__ __forceinline__ int group_pop(State& c, const Stack& stack) {
    while (c.gbits <= 0x00FFFFFFu && c.sp > 0) {
        const uint2 e = stack.get(--c.sp);
        c.gbase = e.x;
        c.gbits = e.y;
    }
    return c.gbits <= 0x00FFFFFFu ? 1 : 0;
}

// Warp-wide closest-hit leaf tests; every lane of the warp calls it, lanes
// without pending triangles with tbits = 0. `tris` is the calling lane's
// triangle array: with kOwnScene each owner's array is fetched from its lane
// (batched jobs trace different scenes in one warp).
template <bool kOwnScene>
__device__ __forceinline__ void closest_leaves(const LeafShare& sh, const float4* tris, uint32_t tbits, uint32_t tbase,
                                               ClosestState& c) {
    if (__ballot_sync(0xFFFFFFFFu, tbits != 0) == 0) return;
    const uint32_t lane = threadIdx.x & 31u, wbase = threadIdx.x - lane;
    uint32_t cnt, incl;
    const uint32_t total = leaf_scan(tbits, cnt, incl);
    unsigned long long init = 0;
    if (tbits) {
        init = hit_key(c.t, c.prim);
        sh.key[threadIdx.x] = init;
    }
    __syncwarp();
    for (uint32_t base = 0; base < total; base += 32) {
        const uint32_t p = base + lane;
        const LeafPair lp = leaf_pair(p, incl, cnt, tbits, tbase);
        const float4* tp = tris;
        if (kOwnScene) {
            const uint64_t tv = reinterpret_cast<uint64_t>(tris);
            const uint32_t lo = __shfl_sync(0xFFFFFFFFu, (uint32_t)tv, lp.owner);
            const uint32_t hi = __shfl_sync(0xFFFFFFFFu, (uint32_t)(tv >> 32), lp.owner);
            tp = reinterpret_cast<const float4*>(((uint64_t)hi << 32) | lo);
        }
        const uint32_t slot = wbase + lp.owner;
        bool cand = false;
        unsigned long long key = 0;
        float t = 0.f, V = 0.f, W = 0.f, det = 0.f;
        if (p < total) {
            const TriRay q = shared_ray(sh, slot);
            const float4* tr = tp + (size_t)lp.rec * 3;
            const float4 a = __ldg(tr), b = __ldg(tr + 1), cc = __ldg(tr + 2);
            if (tri_test_t(q, a, b, cc, t, V, W, det) && t > q.tmin) {
                key = hit_key(t, __float_as_uint(a.w));
                atomicMin(sh.key + slot, key);
                cand = true;
            }
        }
        __syncwarp();
        if (cand && sh.key[slot] == key) {
            sh.rec[slot] = lp.rec;
            sh.vwdt[slot] = make_float4(V, W, det, t);
        }
        __syncwarp();
    }
    if (tbits) {
        const unsigned long long k = sh.key[threadIdx.x];
        if (k != init) {
            const float4 w = sh.vwdt[threadIdx.x];
            const uint32_t prim = (uint32_t)k;
            if (w.w < c.t || (w.w == c.t && prim < c.prim)) {
                c.t = w.w;
                c.V = w.x;
                c.W = w.y;
                c.det = w.z;
                c.prim = prim;
                c.rec = (int32_t)sh.rec[threadIdx.x];
            }
        }
    }
    __syncwarp();
}

// Node part of an any-hit step (as closest_node, culling against tmax).
template <bool kCount, typename Stack>
__device__ __forceinline__ int any_node(const DevScene& s, const TRay& r, uint32_t octp, float tmax, AnyState& c,
                                        const Stack& stack, uint32_t& tbits, uint32_t& tbase, uint32_t& nnode,
                                        uint32_t& ntri) {
    const uint32_t node = wide_pop_child(c.gbase, c.gbits, octp);
    if (c.gbits > 0x00FFFFFFu) {
        if (c.sp >= kWideStack) return -1;
        stack.put(c.sp++, make_uint2(c.gbase, c.gbits));
    }
    if (++c.visits > s.n_nodes || node >= s.n_nodes) return -1;
    uint32_t imask;
    const uint32_t hm = wide_node(s.nodes + (size_t)node * 5, r, octp, tmax, c.gbase, tbase, imask);
    if (kCount) ++nnode;
    c.gbits = (hm & 0xFF000000u) | imask;
    const uint32_t tb = hm & 0x00FFFFFFu;
    if (tb && (uint64_t)tbase + (31u - __clz(tb)) >= s.n_tris) return -1;
    tbits = tb;
    return 0;
}

// Triangles a sequential any-hit loop over tbits (lowest bit first) tests
// before it stops at the first hit of `hits`.
__device__ __forceinline__ uint32_t any_tested(uint32_t tbits, uint32_t hits) {
    return hits ? __popc(tbits & (((hits & (0u - hits)) << 1) - 1u)) : __popc(tbits);
}

// Warp-wide any-hit leaf tests: the mask of the lane's pending triangles
// (bits of tbits) with a hit in (tmin, tmax]. The lane's tmax is in key[] as
// float bits (publish_tmax).
__device__ __forceinline__ void publish_tmax(const LeafShare& sh, float tmax) {
    sh.key[threadIdx.x] = __float_as_uint(tmax);
}
template <bool kOwnScene>
__device__ __forceinline__ uint32_t any_leaves(const LeafShare& sh, const float4* tris, uint32_t tbits,
                                               uint32_t tbase) {
    if (__ballot_sync(0xFFFFFFFFu, tbits != 0) == 0) return 0u;
    const uint32_t lane = threadIdx.x & 31u, wbase = threadIdx.x - lane;
    uint32_t cnt, incl;
    const uint32_t total = leaf_scan(tbits, cnt, incl);
    if (tbits) sh.rec[threadIdx.x] = 0u;
    __syncwarp();
    for (uint32_t base = 0; base < total; base += 32) {
        const uint32_t p = base + lane;
        const LeafPair lp = leaf_pair(p, incl, cnt, tbits, tbase);
        const float4* tp = tris;
        if (kOwnScene) {
            const uint64_t tv = reinterpret_cast<uint64_t>(tris);
            const uint32_t lo = __shfl_sync(0xFFFFFFFFu, (uint32_t)tv, lp.owner);
            const uint32_t hi = __shfl_sync(0xFFFFFFFFu, (uint32_t)(tv >> 32), lp.owner);
            tp = reinterpret_cast<const float4*>(((uint64_t)hi << 32) | lo);
        }
        const uint32_t slot = wbase + lp.owner;
        if (p < total) {
            const TriRay q = shared_ray(sh, slot);
            const float tmax = __uint_as_float((uint32_t)sh.key[slot]);
            const float4* tr = tp + (size_t)lp.rec * 3;
            float t, V, W, det;
            if (tri_test_t(q, __ldg(tr), __ldg(tr + 1), __ldg(tr + 2), t, V, W, det) && t > q.tmin && t <= tmax)
                atomicOr(sh.rec + slot, 1u << lp.bit);
        }
    }
    __syncwarp();
    const uint32_t hits = tbits ? sh.rec[threadIdx.x] : 0u;
    __syncwarp();
    return hits;
}

// Persistent ray loop: each warp keeps its lanes busy by fetching new rays
// (one atomic per warp) whenever at least `refill` of its lanes are idle,
// instead of running until its slowest ray ends. Warp-synchronous: one ballot
// per step; start(k) sets up ray k on the calling lane, step() advances it by
// one node and returns true once the ray is finished and its result written.
// Every traversal is bounded, so a warp leaves once the queue [0, n) is
// drained. Refilling only in groups (8 lanes) keeps the set-up code from
// running for one or two lanes at a time.
// Stack entries of a persistent closest-hit thread kept in shared memory
// (16 KB per block of 256 threads at 8). Measured: the terrain frame's trace
// stage 130.6 -> 129.7 ms, the incoherent-ray microbenchmark 1.190 -> 1.242
// Grays/s; the any-hit kernels keep the local stack (their frame stage lost
// 1 % with it).
#ifndef KZ_SMEM_STACK
#define KZ_SMEM_STACK 8
#endif

#ifndef KZ_TRACE_REFILL
#define KZ_TRACE_REFILL 8
#endif
constexpr uint32_t kTraceRefill = KZ_TRACE_REFILL;
// Refill group of the any-hit (shadow ray) kernels.
#ifndef KZ_ANY_REFILL
#define KZ_ANY_REFILL KZ_TRACE_REFILL
#endif
constexpr uint32_t kAnyRefill = KZ_ANY_REFILL;

template <typename Ctr, typename Start, typename Step>
__device__ __forceinline__ void persistent_rays(Ctr n, Ctr* next, uint32_t refill, Start start, Step step) {
    const uint32_t lane = threadIdx.x & 31u;
    bool busy = false, more = true;
    for (;;) {
        const uint32_t idle = __ballot_sync(0xFFFFFFFFu, !busy);
        if (!more && idle == 0xFFFFFFFFu) break;
        const uint32_t n_idle = __popc(idle);
        if (more && n_idle >= refill) {
            Ctr base = 0;
            if (lane == 0) base = atomicAdd(next, (Ctr)n_idle);
            base = __shfl_sync(0xFFFFFFFFu, base, 0);
            if (base + n_idle >= n) more = false;
            if (!busy) {
                const Ctr k = base + __popc(idle & ((1u << lane) - 1u));
                if (k < n) {
                    busy = true;
                    start(k);
                }
            }
        }
        if (busy && step()) busy = false;
    }
}

// persistent_rays with the warp-wide leaf part: node(tbits, tbase) runs on
// the busy lanes and returns -1 on an abort, else 0; leaves(tbits, tbase)
// runs on all 32 lanes; finish(rc) on the busy lanes returns true once the
// ray is finished and its result written.
template <typename Ctr, typename Start, typename Node, typename Leaves, typename Finish>
__device__ __forceinline__ void persistent_rays_shared(Ctr n, Ctr* next, uint32_t refill, Start start, Node node,
                                                       Leaves leaves, Finish finish) {
    const uint32_t lane = threadIdx.x & 31u;
    bool busy = false, more = true;
    for (;;) {
        const uint32_t idle = __ballot_sync(0xFFFFFFFFu, !busy);
        if (!more && idle == 0xFFFFFFFFu) break;
        const uint32_t n_idle = __popc(idle);
        if (more && n_idle >= refill) {
            Ctr base = 0;
            if (lane == 0) base = atomicAdd(next, (Ctr)n_idle);
            base = __shfl_sync(0xFFFFFFFFu, base, 0);
            if (base + n_idle >= n) more = false;
            if (!busy) {
                const Ctr k = base + __popc(idle & ((1u << lane) - 1u));
                if (k < n) {
                    busy = true;
                    start(k);
                }
            }
        }
        uint32_t tbits = 0, tbase = 0;
        int rc = 0;
        if (busy) rc = node(tbits, tbase);
        leaves(tbits, tbase);
        if (busy && finish(rc)) busy = false;
    }
}

}  // namespace kz
