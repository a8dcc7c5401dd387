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

// The same test with the barycentric divisions left to the caller:
// u = V / det, v = W / det for the hit that is kept.
__device__ __forceinline__ bool tri_test_t(const TRay& r, float4 a, float4 b, float4 c, float& t, float& V_, float& W_,
                                           float& det_) {
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
    V_ = V;
    W_ = W;
    det_ = det;
    return true;
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

template <int kSlot>
__device__ __forceinline__ void wide_slot(const WideAxis& X, const WideAxis& Y, const WideAxis& Z, uint32_t meta,
                                          float tmin, float tcur, uint32_t& hits) {
    const float tn = fmaxf(fmaxf(fmaxf(wide_t<kSlot>(X, true), wide_t<kSlot>(Y, true)), wide_t<kSlot>(Z, true)), tmin);
    const float tf = fminf(fminf(fminf(wide_t<kSlot>(X, false), wide_t<kSlot>(Y, false)), wide_t<kSlot>(Z, false)), tcur);
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
#if KZ_SMEM_STACK > 0 && KZ_SMEM_STACK < KZ_WIDE_STACK
#define KZ_CLOSEST_STACK(name)                       \
    __shared__ uint2 name##_sm[KZ_SMEM_STACK * 256]; \
    uint2 name##_lm[kWideStack - KZ_SMEM_STACK];     \
    const SplitStack<KZ_SMEM_STACK> name{name##_sm, name##_lm}
#else
#define KZ_CLOSEST_STACK(name)   \
    uint2 name##_lm[kWideStack]; \
    const LocalStack name { name##_lm }
#endif

#ifndef KZ_TRACE_REFILL
#define KZ_TRACE_REFILL 8
#endif
constexpr uint32_t kTraceRefill = KZ_TRACE_REFILL;

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

}  // namespace kz
