// kz_stages.cuh — device helpers shared by the wavefront stage kernels
// (kz_trace.cu: traversal kernels; kz_kernels.cu: generation, shading and the
// loop kernels): path-state flags, warp-aggregated counters and appends, film
// accumulation, camera path generation, the shaded vertex (shade_vertex), job
// lookup for batched renders, the persistent closest-hit driver and grid
// sizing. Each translation unit gets its own copy (internal linkage).
//
// The wavefront stages restate PathIntegrator::Li
// (src/core/integrator.cpp:362-561 in kazen_proto) with the estimator
// corrections listed at the top of k_shade. Random numbers: PCG32 stream
// (seed, path id); a camera path first draws the pixel jitter (2 floats,
// Renderer::render, src/core/renderer.cpp:57), then 9 floats per shaded
// vertex in a fixed order whatever branches run:
//   [0] light pick  [1] light triangle  [2,3] point on triangle  [4] roulette
//   [5] lobe pick   [6,7,8] lobe sample
#pragma once

#include <algorithm>

#include "kz_guide.cuh"
#include "kz_internal.h"
#include "kz_traverse.cuh"

namespace kz {
namespace {

constexpr uint32_t kSpecularFlag = 1u << 8;
// Batched wavefront: bits 12-31 of a path's d4.w hold its job index (0 for a
// single render); continuations keep them, shadow rays carry the job in c4.w.
constexpr uint32_t kJobShift = 12;
constexpr uint32_t kJobMask = 0xFFFFF000u;

__device__ __forceinline__ void set_status(uint32_t* status, uint32_t code) {
    if (status) atomicCAS(status, 0u, code);
}

__device__ __forceinline__ f3 ld3(const float* p) { return mk(p[0], p[1], p[2]); }
__device__ __forceinline__ f3 xyz(float4 v) { return mk(v.x, v.y, v.z); }

// Warp-aggregated append: one atomic per warp, lanes get consecutive slots.
__device__ __forceinline__ uint32_t warp_append(bool pred, uint32_t* counter) {
    const unsigned mask = __activemask();
    const unsigned ballot = __ballot_sync(mask, pred);
    if (!pred) return 0xFFFFFFFFu;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(ballot) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(ballot));
    base = __shfl_sync(ballot, base, leader);
    return base + (uint32_t)__popc(ballot & ((1u << lane) - 1u));
}

__device__ __forceinline__ void store_hit(const DevScene& s, kz_hits hits, uint64_t i, const HitRec& h) {
    hits.t[i] = h.t;
    uint32_t geom = KZ_INVALID_ID, local = KZ_INVALID_ID;
    if (h.rec >= 0) {
        geom = __float_as_uint(__ldg(s.tris + (size_t)h.rec * 3 + 1).w);
        local = h.prim - __ldg(s.geom_offset + geom);
    }
    hits.prim_id[i] = local;
    if (hits.geom_id) hits.geom_id[i] = geom;
    if (hits.u) hits.u[i] = h.u;
    if (hits.v) hits.v[i] = h.v;
}

// ------------------------------------------------------------------ wavefront stages
__device__ __forceinline__ void generate_camera_path(const DevCamera& cam, const PathParams& pp, PathSoA dst,
                                                     uint32_t k, uint64_t pid) {
    const uint64_t pix = pid / pp.spp;
    const uint32_t px = (uint32_t)(pix % cam.W), py = (uint32_t)(pix / cam.W);
    Pcg rng;
    rng.seed(pp.seed, pid);
    const float jx = rng.nextf(), jy = rng.nextf();
    // Camera::generate_ray (src/core/camera.cpp:5-37): horizontal fov,
    // row 0 at the top unless flipped.
    const float sx = ((float)px + jx) / (float)cam.W;
    const float sy = ((float)py + jy) / (float)cam.H;
    const float nx = 2.0f * sx - 1.0f;
    const float ny = cam.flip * ((1.0f - 2.0f * sy) / cam.aspect);
    const float cx = nx * cam.tan_half;
    const float cy = ny * cam.tan_half;
    const f3 d = normalize(ld3(cam.x) * cx + ld3(cam.y) * cy + ld3(cam.z) * (-1.0f));
    dst.o4[k] = make_float4(cam.eye[0], cam.eye[1], cam.eye[2], 0.f);
    dst.d4[k] = make_float4(d.x, d.y, d.z, __uint_as_float(kSpecularFlag));
    dst.b4[k] = make_float4(1.f, 1.f, 1.f, __uint_as_float((uint32_t)pid));
    dst.rng[k] = rng.state;
}

__device__ __forceinline__ void generate_ray_path(const kz_ray* __restrict__ rays, const PathParams& pp, PathSoA dst,
                                                  uint32_t k, uint64_t pid) {
    Pcg rng;
    rng.seed(pp.seed, pid);
    const kz_ray r = rays[pid];
    dst.o4[k] = make_float4(r.ox, r.oy, r.oz, 0.f);
    dst.d4[k] = make_float4(r.dx, r.dy, r.dz, __uint_as_float(kSpecularFlag));
    dst.b4[k] = make_float4(1.f, 1.f, 1.f, __uint_as_float((uint32_t)pid));
    dst.rng[k] = rng.state;
}

// Sums two per-thread counters over the warp; one 64-bit atomic each.
__device__ __forceinline__ void warp_count(uint32_t a, uint32_t b, unsigned long long* dst) {
    unsigned long long x = a, y = b;
    for (int o = 16; o > 0; o >>= 1) {
        x += __shfl_down_sync(0xffffffffu, x, o);
        y += __shfl_down_sync(0xffffffffu, y, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(dst, x);
        atomicAdd(dst + 1, y);
    }
}

// Leaf triangles of the persistent kernels tested warp-wide
// (persistent_rays_shared) rather than per lane (persistent_rays).
#ifndef KZ_SHARE_LEAVES
#define KZ_SHARE_LEAVES 1
#endif

// Shared memory of the persistent traversal loops: the closest-hit loop's
// first stack entries and warp-shared leaf arrays, and the any-hit loop's
// leaf arrays (blocks of 256 threads). A kernel that runs both loops one
// after the other (the single-launch batch kernel) overlays them.
struct ClosestSmem {
    uint2 stack[(KZ_SMEM_STACK > 0 ? KZ_SMEM_STACK : 1) * 256];
    float4 ray[2 * 256];
    unsigned long long key[256];
    uint32_t rec[256];
    float4 vwdt[256];
};
// KZ_ANY_SMEM_STACK: the any-hit loop's first stack entries in shared memory
// (off: the terrain frame's shadow stage measured 29.1 ms with 4 or 8 entries
// against 28.9 ms with the whole stack in local memory).
#ifndef KZ_ANY_SMEM_STACK
#define KZ_ANY_SMEM_STACK 0
#endif
struct AnySmem {
    float4 ray[2 * 256];
    unsigned long long key[256];
    uint32_t rec[256];
#if KZ_ANY_SMEM_STACK > 0 && KZ_ANY_SMEM_STACK < KZ_WIDE_STACK
    uint2 stack[KZ_ANY_SMEM_STACK * 256];
#endif
};

// Closest hit of ray k through persistent_rays: load(k, r, tmax) sets the
// ray up, store(k, hit) writes the result; m is the block's shared memory.
// `s` is the lane's scene; load may repoint it per ray (batched jobs: kOwnScene).
template <bool kCount, bool kOwnScene, typename Ctr, typename Load, typename Store>
__device__ __forceinline__ void persistent_closest_in(ClosestSmem& m, DevScene& s, Ctr n, Ctr* next,
                                                      uint32_t* status, Load load, Store store, uint32_t& dn,
                                                      uint32_t& dt) {
#if KZ_SMEM_STACK > 0 && KZ_SMEM_STACK < KZ_WIDE_STACK
    uint2 stack_lm[kWideStack - KZ_SMEM_STACK];
    const SplitStack<KZ_SMEM_STACK> stack{m.stack, stack_lm};
#else
    uint2 stack_lm[kWideStack];
    const LocalStack stack{stack_lm};
#endif
#if KZ_SHARE_LEAVES
    const LeafShare sh{m.ray, m.key, m.rec, m.vwdt};
    ClosestState c;
    TRay r;
    float tmax = 0.f;
    uint32_t octp = 0;
    Ctr ray = 0;
    persistent_rays_shared(
        n, next, kTraceRefill,
        [&](Ctr k) {
            ray = k;
            load(k, r, tmax);
            octp = wide_octant(r);
            closest_begin(c, tmax);
            publish_ray(sh, r);
        },
        [&](uint32_t& tbits, uint32_t& tbase) {
            return closest_node<kCount>(s, r, octp, c, stack, tbits, tbase, dn, dt);
        },
        [&](uint32_t tbits, uint32_t tbase) { closest_leaves<kOwnScene>(sh, s.tris, tbits, tbase, c); },
        [&](int rc) {
            if (rc == 0) rc = group_pop(c, stack);
            if (rc == 0) return false;
            HitRec h;
            closest_finish(c, rc > 0, tmax, h);
            if (rc < 0) set_status(status, KZ_ERR_STACK);
            store(ray, h);
            return true;
        });
#else
    ClosestState c;
    TRay r;
    float tmax = 0.f;
    uint32_t octp = 0;
    Ctr ray = 0;
    persistent_rays(
        n, next, kTraceRefill,
        [&](Ctr k) {
            ray = k;
            load(k, r, tmax);
            octp = wide_octant(r);
            closest_begin(c, tmax);
        },
        [&]() {
            const int rc = closest_step<kCount>(s, r, octp, c, stack, dn, dt);
            if (rc == 0) return false;
            HitRec h;
            closest_finish(c, rc > 0, tmax, h);
            if (rc < 0) set_status(status, KZ_ERR_STACK);
            store(ray, h);
            return true;
        });
#endif
}

// The same with the block's own static shared memory.
template <bool kCount, bool kOwnScene = false, typename Ctr, typename Load, typename Store>
__device__ __forceinline__ void persistent_closest(DevScene& s, Ctr n, Ctr* next, uint32_t* status, Load load,
                                                   Store store, uint32_t& dn, uint32_t& dt) {
    __shared__ ClosestSmem m;
    persistent_closest_in<kCount, kOwnScene>(m, s, n, next, status, load, store, dn, dt);
}

// Any hit of ray k through persistent_rays_shared: load(k, r, tmax) sets the
// ray up, done(k, rc) gets 1 (no hit), 2 (hit) or -1 (aborted: miss).
template <bool kCount, bool kOwnScene, typename Ctr, typename Load, typename Done>
__device__ __forceinline__ void persistent_any_in(AnySmem& m, DevScene& s, Ctr n, Ctr* next, Load load, Done done,
                                                  uint32_t& dn, uint32_t& dt) {
#if KZ_ANY_SMEM_STACK > 0 && KZ_ANY_SMEM_STACK < KZ_WIDE_STACK
    uint2 stack_lm[kWideStack - KZ_ANY_SMEM_STACK];
    const SplitStack<KZ_ANY_SMEM_STACK> stack{m.stack, stack_lm};
#else
    uint2 stack_lm[kWideStack];
    const LocalStack stack{stack_lm};
#endif
    const LeafShare sh{m.ray, m.key, m.rec, nullptr};
    AnyState c;
    TRay r;
    float tmax = 0.f;
    uint32_t octp = 0;
    Ctr ray = 0;
    bool hit = false;
    persistent_rays_shared(
        n, next, kAnyRefill,
        [&](Ctr k) {
            ray = k;
            load(k, r, tmax);
            octp = wide_octant(r);
            any_begin(c);
            publish_ray(sh, r);
            publish_tmax(sh, tmax);
        },
        [&](uint32_t& tbits, uint32_t& tbase) {
            return any_node<kCount>(s, r, octp, tmax, c, stack, tbits, tbase, dn, dt);
        },
        [&](uint32_t tbits, uint32_t tbase) {
            const uint32_t hits = any_leaves<kOwnScene>(sh, s.tris, tbits, tbase);
            hit = hits != 0u;
            if (kCount) dt += any_tested(tbits, hits);
        },
        [&](int rc) {
            if (rc == 0) rc = hit ? 2 : group_pop(c, stack);
            if (rc == 0) return false;
            done(ray, rc);
            return true;
        });
}

template <bool kCount, bool kOwnScene = false, typename Ctr, typename Load, typename Done>
__device__ __forceinline__ void persistent_any(DevScene& s, Ctr n, Ctr* next, Load load, Done done, uint32_t& dn,
                                               uint32_t& dt) {
    __shared__ AnySmem m;
    persistent_any_in<kCount, kOwnScene>(m, s, n, next, load, done, dn, dt);
}

// Closest-hit pass of the device-driven loop (k_plan zeroes trace_next).

__device__ __forceinline__ void film_add(float* film, double* film64, uint32_t idx, f3 c) {
    atomicAdd(film + 3 * (size_t)idx, c.x);
    atomicAdd(film + 3 * (size_t)idx + 1, c.y);
    atomicAdd(film + 3 * (size_t)idx + 2, c.z);
    if (film64) {
        atomicAdd(film64 + 3 * (size_t)idx, (double)c.x);
        atomicAdd(film64 + 3 * (size_t)idx + 1, (double)c.y);
        atomicAdd(film64 + 3 * (size_t)idx + 2, (double)c.z);
    }
}

// DiscrectPDF::sample (src/base/dpdf.h:31-36): lower_bound over cdf[0..n].
__device__ __forceinline__ uint32_t cdf_sample(const float* cdf, uint32_t n, float u) {
    uint32_t lo = 0, cnt = n + 1;
    while (cnt > 0) {
        uint32_t step = cnt / 2, it = lo + step;
        if (__ldg(cdf + it) < u) {
            lo = it + 1;
            cnt -= step + 1;
        } else {
            cnt = step;
        }
    }
    int idx = (int)lo - 1;
    if (idx < 0) idx = 0;
    return min((uint32_t)idx, n - 1);
}

// One shaded vertex per thread. Estimator corrections relative to the
// reference loop (each one keeps the estimator unbiased):
//  * NEE uses f*|cos| once (the reference multiplies Diffuse's f*cos by cos
//    again, integrator.cpp:475-480) and divides by the light pick pdf inside
//    the MIS weight as well as outside;
//  * BSDF sampling divides by the direction pdf (integrator.cpp:503-505
//    multiplies by f only) and picks the lobe by its selection probability;
//  * emission hits weigh against the light pdf of the sampled direction
//    (integrator.cpp:452-462 reuses the previous light sample's pdf);
//  * max_depth counts shaded vertices (the reference steps depth twice per
//    loop, integrator.cpp:420,555).
// Guided mode (learned path guiding, not in the reference) additionally:
//  * on materials without delta lobes, samples the direction from the
//    network's vMF mixture with probability alpha and from the BSDF mixture
//    otherwise, with the one-sample MIS pdf alpha*q + (1-alpha)*p_bsdf in the
//    path weight, the NEE MIS weight and the next emission hit's MIS weight;
//  * records every such vertex (position, normal, direction, pdf,
//    throughput after it) and adds each later contribution, divided by that
//    throughput, to the vertex's incident-radiance estimate: the training
//    data of the network.
__device__ __forceinline__ void propagate(VRec* recs, uint64_t rbase, uint32_t depth, f3 c) {
    for (uint32_t k = 0; k < depth; ++k) {
        VRec& r = recs[rbase + k];
        if (r.n.w == 0.f) continue;
        const float4 b = r.beta;
        r.L.x += b.x > 0.f ? c.x / b.x : 0.f;
        r.L.y += b.y > 0.f ? c.y / b.y : 0.f;
        r.L.z += b.z > 0.f ? c.z / b.z : 0.f;
    }
}

// ------------------------------------------------------------------ textures
// OSL checkerboard (int() truncates, as the shader's int(fmod(..)) does) or
// a bilinear lookup with periodic wrap, texel centres at (i + 0.5) / w.
__device__ __noinline__ f3 tex_eval(const DevScene& s, int32_t k, float u, float v) {
    const DevTexture& tx = s.textures[k];
    if (!isfinite(u)) u = 0.f;
    if (!isfinite(v)) v = 0.f;
    if (tx.kind == KZ_TEX_CHECKER) {
        const float cs = fmodf(u * tx.scale_s, 2.f), ct = fmodf(v * tx.scale_t, 2.f);
        const int a = isfinite(cs) ? (int)cs : 0, b = isfinite(ct) ? (int)ct : 0;
        return (a ^ b) == 0 ? mk(tx.Ca[0], tx.Ca[1], tx.Ca[2]) : mk(tx.Cb[0], tx.Cb[1], tx.Cb[2]);
    }
    u -= floorf(u);
    v -= floorf(v);
    const float x = u * (float)tx.w - 0.5f, y = v * (float)tx.h - 0.5f;
    const float fx = floorf(x), fy = floorf(y);
    const float ax = x - fx, ay = y - fy;
    const uint32_t x0 = fx < 0.f ? tx.w - 1 : min((uint32_t)fx, tx.w - 1), x1 = x0 + 1 == tx.w ? 0 : x0 + 1;
    const uint32_t y0 = fy < 0.f ? tx.h - 1 : min((uint32_t)fy, tx.h - 1), y1 = y0 + 1 == tx.h ? 0 : y0 + 1;
    const float* d = s.tex_data + tx.offset;
    const f3 c00 = ld3(d + ((size_t)y0 * tx.w + x0) * 3), c10 = ld3(d + ((size_t)y0 * tx.w + x1) * 3);
    const f3 c01 = ld3(d + ((size_t)y1 * tx.w + x0) * 3), c11 = ld3(d + ((size_t)y1 * tx.w + x1) * 3);
    return (c00 * (1.f - ax) + c10 * ax) * (1.f - ay) + (c01 * (1.f - ax) + c11 * ax) * ay;
}

// Radiance of a ray leaving the scene: the environment in latitude-longitude form.
__device__ __noinline__ f3 env_radiance(const DevScene& s, f3 d) {
    f3 e = mk(s.env.x, s.env.y, s.env.z);
    if (s.env_tex >= 0) {
        const float u = 0.5f + atan2f(d.x, -d.z) * (0.5f * kInvPi);
        const float v = acosf(fminf(fmaxf(d.y, -1.f), 1.f)) * kInvPi;
        e = hmul(e, tex_eval(s, s.env_tex, u, v));
    }
    return e;
}

// Weight of lobe k at this vertex: the texture tint applies to the lobes
// that reference the material's texture.
__device__ __forceinline__ f3 lobe_weight(const kz_lobe& lb, bool textured, f3 tint) {
    const f3 w = ld3(lb.weight);
    return textured && lb.params[KZ_LOBE_TEXTURE_PARAM] != 0.f ? hmul(w, tint) : w;
}

struct ShadeOut {
    bool cont = false, shadow = false;
    float4 o_next, d_next, b_next, s_o, s_d, s_c;
    unsigned long long rng_next = 0;
    f3 Lsum = {0.f, 0.f, 0.f};  // contribution to the film pixel film_idx
    uint32_t film_idx = 0;
};

// One shaded path vertex: emission, next-event estimation (the shadow ray is
// returned, not traced), roulette and direction sampling. `raw` holds the
// guiding network's outputs for this path (guided mode only). kAttr = false
// compiles the vertex attributes out (texture tint, shading normals) for
// scenes that have neither.
template <bool kGuided, bool kAttr = true>
__device__ __forceinline__ void shade_vertex(const DevScene& s, const PathParams& pp, const float4 hit,
                                             const float4 o4, const float4 d4, const float4 b4,
                                             unsigned long long rng_state, const GuideShade& gs, const float* raw,
                                             ShadeOut& out) {
    const int rec = __float_as_int(hit.w);
    if (rec >= 0) {
        const uint32_t pid = __float_as_uint(b4.w);
        const uint32_t film_idx = pid / pp.spp;
        const uint32_t flags = __float_as_uint(d4.w);
        const uint32_t depth = flags & 0xffu;
        const bool prev_spec = (flags & kSpecularFlag) != 0;
        const float prev_pdf = o4.w;
        Pcg rng;
        rng.state = rng_state;
        rng.inc = ((uint64_t)pid << 1u) | 1u;
        float u[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) u[k] = rng.nextf();

        const float4* tp = s.tris + (size_t)rec * 3;
        const float4 ta = __ldg(tp), tb = __ldg(tp + 1), tc = __ldg(tp + 2);
        const uint32_t geom = __float_as_uint(tb.w);
        const kz_material& mat = s.materials[__float_as_uint(tc.w)];
        const f3 v0 = xyz(ta), v1 = xyz(tb), v2 = xyz(tc);
        const f3 Ng = normalize(cross(v1 - v0, v2 - v0));
        const f3 d = xyz(d4);
        f3 P = xyz(o4) + d * hit.x;
        // shading normal: the interpolated vertex normal, with the shading
        // point moved off the flat triangle by the shadow-terminator offset
        // (Hanika 2021), as TriangleMesh::post_hit does (shape.cpp:628-656)
        f3 Ns = Ng;
        if (kAttr && s.tri_nrm) {
            const float4 m0 = __ldg(s.tri_nrm + (size_t)rec * 3);
            if (m0.w != 0.f) {
                const f3 n0 = xyz(m0), n1 = xyz(__ldg(s.tri_nrm + (size_t)rec * 3 + 1)),
                         n2 = xyz(__ldg(s.tri_nrm + (size_t)rec * 3 + 2));
                const float b0 = 1.f - hit.y - hit.z;
                Ns = normalize(n0 * b0 + n1 * hit.y + n2 * hit.z);
                const f3 Pb = v0 * b0 + v1 * hit.y + v2 * hit.z;
                const float e0 = fminf(0.f, dot(Pb - v0, n0)), e1 = fminf(0.f, dot(Pb - v1, n1)),
                            e2 = fminf(0.f, dot(Pb - v2, n2));
                P = Pb - (n0 * (b0 * e0) + n1 * (hit.y * e1) + n2 * (hit.z * e2));
            }
        }
        // texture tint of the material at the hit's uv (interpolated vertex
        // uvs; the barycentrics of vertices 1, 2 when the mesh has none)
        const int32_t mtex = kAttr && s.mat_tex ? __ldg(s.mat_tex + __float_as_uint(tc.w)) : -1;
        const bool textured = mtex >= 0;
        f3 tint = mk(1.f, 1.f, 1.f);
        if (textured) {
            const float2 q0 = s.tri_uv[(size_t)rec * 3], q1 = s.tri_uv[(size_t)rec * 3 + 1],
                         q2 = s.tri_uv[(size_t)rec * 3 + 2];
            const float b0 = 1.f - hit.y - hit.z;
            tint = tex_eval(s, mtex, b0 * q0.x + hit.y * q1.x + hit.z * q2.x, b0 * q0.y + hit.y * q1.y + hit.z * q2.y);
        }
        const Frame fr(Ns);
        const f3 wi = -fr.to_local(d);
        f3 beta = xyz(b4);
        f3 Lsum = mk(0.f, 0.f, 0.f);
        const uint32_t nl = s.n_lights;
        const uint64_t rbase = kGuided ? ((uint64_t)pid - gs.pass_first) * pp.max_depth : 0;

        // 1. emission (front face only, against the shading normal:
        // single_emissive_surface, integrator.cpp:454)
        const f3 Le = ld3(mat.Le);
        if (!is_zero(Le) && dot(d, Ns) < 0.f) {
            float w = 1.f;
            if (!prev_spec && pp.estimator != 2u) {
                const int li = __ldg(s.geom_light + geom);
                if (li >= 0) {
                    if (pp.estimator == 1u) {
                        w = 0.f;  // NEE only: after a non-specular bounce this light was sampled directly
                    } else {
                        const float cos_l = -dot(d, Ng);
                        const float lpdf = (hit.x * hit.x) / (cos_l * s.lights[li].area) * (1.0f / (float)nl);
                        w = power_heuristic(prev_pdf, lpdf);
                    }
                }
            }
            Lsum = Lsum + hmul(beta, Le) * w;
            // MIS-weighted, like the next-event samples it pairs with
            if (kGuided && gs.recs) propagate(gs.recs, rbase, depth, Lsum);
        }

        // lobe selection probabilities (CompositeClosure::compute_pdfs)
        const uint32_t nlobes = min(mat.n_lobes, (uint32_t)KZ_MAX_LOBES);
        float lp[KZ_MAX_LOBES];
        const float winv = 1.f / (beta.x + beta.y + beta.z);
        float wsum = 0.f;
        bool any_smooth = false, any_delta = false;
        for (uint32_t k = 0; k < nlobes; ++k) {
            const kz_lobe& lb = mat.lobes[k];
            const f3 lw = lobe_weight(lb, textured, tint);
            lp[k] = (lw.x * beta.x + lw.y * beta.y + lw.z * beta.z) * winv;
            wsum += lp[k];
            const bool dl = lobe_is_delta(lb.closure_id);
            any_smooth |= !dl;
            any_delta |= dl;
        }
        if (wsum > 0.f)
            for (uint32_t k = 0; k < nlobes; ++k) lp[k] /= wsum;
        const bool guided = kGuided && any_smooth && !any_delta && wsum > 0.f;
        VmfMixture mix;
        if (kGuided && guided)
            mixture_for_shading(raw, hmul(P - mk(s.box_lo.x, s.box_lo.y, s.box_lo.z), mk(s.box_inv.x, s.box_inv.y, s.box_inv.z)),
                                mk(1.f / s.box_inv.x, 1.f / s.box_inv.y, 1.f / s.box_inv.z), mix);
        const float alpha = gs.alpha;

        // 2. next-event estimation (none when sampling the BSDF only)
        if (pp.estimator != 2u && nl > 0 && any_smooth && wsum > 0.f) {
            const uint32_t li = min((uint32_t)(u[0] * (float)nl), nl - 1);
            const DevLight lt = s.lights[li];
            // a point light (PointLight, light.cpp:18-31) has no triangles:
            // its position is the one light_tris record it names
            const bool point = lt.tri_count == 0;
            f3 p, nlgt = mk(0.f, 0.f, 0.f);
            if (point) {
                p = xyz(__ldg(s.light_tris + (size_t)lt.tri_begin * 3));
            } else {
                const uint32_t kk = cdf_sample(s.light_cdf + lt.cdf_begin, lt.tri_count, u[1]);
                const float4* lq = s.light_tris + (size_t)(lt.tri_begin + kk) * 3;
                const f3 a0 = xyz(__ldg(lq)), a1 = xyz(__ldg(lq + 1)), a2 = xyz(__ldg(lq + 2));
                const float su0 = sqrtf(u[2]);
                const float bu0 = 1.f - su0;
                const float bv0 = u[3] * su0;
                p = a0 * bu0 + a1 * bv0 + a2 * (1.f - bu0 - bv0);
                nlgt = normalize(cross(a1 - a0, a2 - a0));
            }
            const f3 lv = p - P;
            const float dist2 = dot(lv, lv);
            const float dist = sqrtf(dist2);
            const f3 ldir = mk(lv.x / dist, lv.y / dist, lv.z / dist);
            const float cos_l = point ? 1.f : -dot(ldir, nlgt);
            if (cos_l > 0.f && dist2 > 0.f) {
                // a delta light is picked with probability 1/nl and weighs no MIS
                const float lpdf = point ? 1.0f / (float)nl : dist2 / (cos_l * lt.area) * (1.0f / (float)nl);
                const f3 wo = fr.to_local(ldir);
                f3 f = mk(0.f, 0.f, 0.f);
                float bpdf = 0.f;
                for (uint32_t k = 0; k < nlobes; ++k) {
                    const kz_lobe& lb = mat.lobes[k];
                    if (lobe_is_delta(lb.closure_id)) continue;
                    const LobeEval e = lobe_eval(lb, wi, wo);
                    f = f + hmul(lobe_weight(lb, textured, tint), e.f);
                    bpdf += lp[k] * e.pdf;
                }
                // the MIS partner of this light sample is the next direction,
                // sampled from the guide mixture; at the last vertex no
                // direction follows, so the weight is the plain one and the
                // guided image converges to the plain image at every depth
                if (kGuided && guided && depth + 1 < pp.max_depth)
                    bpdf = alpha * mixture_pdf_shading(mix, ldir) + (1.f - alpha) * bpdf;
                if (!is_zero(f)) {
                    const float w = point || pp.estimator == 1u ? 1.f : power_heuristic(lpdf, bpdf);
                    // PointLight::sample's falloff: radiance / (0.1 |d|^2)
                    const f3 Le_l = point ? ld3(lt.Le) * (1.f / (dist2 * 0.1f)) : ld3(lt.Le);
                    const f3 c = hmul(hmul(beta, f), Le_l) * (w / lpdf);
                    out.shadow = true;
                    out.s_o = make_float4(P.x, P.y, P.z, dist - kRayEps);
                    out.s_d = make_float4(ldir.x, ldir.y, ldir.z, __uint_as_float(film_idx));
                    const uint32_t tag = kGuided ? (uint32_t)(((uint64_t)pid - gs.pass_first) << 4 | (depth & 15u))
                                                 : flags >> kJobShift;
                    out.s_c = make_float4(c.x, c.y, c.z, __uint_as_float(tag));
                    if (kGuided && gs.nee && guided) {
                        // training sample: the light direction with its
                        // MIS-weighted share of L*f*cos over the light pdf
                        const f3 fl = hmul(f, Le_l);
                        const float wt = (0.2126f * fl.x + 0.7152f * fl.y + 0.0722f * fl.z) * (w / lpdf);
                        const f3 p01 = hmul(P - mk(s.box_lo.x, s.box_lo.y, s.box_lo.z),
                                            mk(s.box_inv.x, s.box_inv.y, s.box_inv.z));
                        NRec& nr = gs.nee[rbase + depth];
                        nr.p = make_float4(p01.x, p01.y, p01.z, wt);
                        nr.n = make_float4(Ng.x, Ng.y, Ng.z, 0.f);
                        nr.d = make_float4(ldir.x, ldir.y, ldir.z, 0.f);
                    }
                }
            }
        }

        bool alive = depth + 1 < pp.max_depth;
        // 3. Russian roulette (integrator.cpp:491-498)
        if (alive && depth >= pp.rr_min) {
            const float prob = fminf(max_comp(beta) * 0.9025f, 0.99f);
            if (prob < u[4]) alive = false;
            else beta = beta * (1.f / prob);
        }
        // 4. direction sampling
        if (kGuided && guided && alive) {
            // one-sample MIS of the learned vMF mixture and the BSDF mixture
            f3 wo, wdir;
            bool ok = true;
            if (u[5] < alpha) {
                wdir = mixture_sample(mix, u[5] / alpha, u[6], u[7]);
                wo = fr.to_local(wdir);
            } else {
                const float us = (u[5] - alpha) / (1.f - alpha);
                uint32_t sel = nlobes - 1;
                float acc = 0.f;
                for (uint32_t k = 0; k < nlobes; ++k) {
                    acc += lp[k];
                    if (us < acc) {
                        sel = k;
                        break;
                    }
                }
                while (sel > 0 && lp[sel] == 0.f) --sel;
                const LobeSample smp = lobe_sample(mat.lobes[sel], wi, u[6], u[7], u[8]);
                ok = smp.valid;
                wo = smp.wo;
                wdir = normalize(fr.to_world(wo));
            }
            f3 f = mk(0.f, 0.f, 0.f);
            float pdf = 0.f;
            if (ok) {
                for (uint32_t k = 0; k < nlobes; ++k) {
                    const kz_lobe& lb = mat.lobes[k];
                    const LobeEval e = lobe_eval(lb, wi, wo);
                    f = f + hmul(lobe_weight(lb, textured, tint), e.f);
                    pdf += lp[k] * e.pdf;
                }
                pdf = alpha * mixture_pdf_shading(mix, wdir) + (1.f - alpha) * pdf;
            }
            alive = ok && pdf > 0.f && !is_zero(f);
            if (alive) {
                beta = hmul(beta, f * (1.f / pdf));
                alive = !is_zero(beta);
            }
            if (alive) {
                out.cont = true;
                out.o_next = make_float4(P.x, P.y, P.z, pdf);
                out.d_next = make_float4(wdir.x, wdir.y, wdir.z, __uint_as_float((depth + 1) | (flags & kJobMask)));
                out.b_next = make_float4(beta.x, beta.y, beta.z, b4.w);
                out.rng_next = rng.state;
            }
            if (alive && gs.recs) {
                VRec& r = gs.recs[rbase + depth];
                const f3 p01 = hmul(P - mk(s.box_lo.x, s.box_lo.y, s.box_lo.z),
                                    mk(s.box_inv.x, s.box_inv.y, s.box_inv.z));
                r.p = make_float4(p01.x, p01.y, p01.z, pdf);
                r.n = make_float4(Ng.x, Ng.y, Ng.z, 1.f);
                // d.w: luminance of f*|cos| along the sampled direction,
                // so the network learns the whole integrand L*f*cos
                r.d = make_float4(wdir.x, wdir.y, wdir.z, 0.2126f * f.x + 0.7152f * f.y + 0.0722f * f.z);
                r.beta = make_float4(beta.x, beta.y, beta.z, 0.f);
                r.L = make_float4(0.f, 0.f, 0.f, 0.f);
            }
        } else if (alive && wsum > 0.f) {
            // BSDF sample (one-sample mixture over the non-delta lobes)
            uint32_t sel = nlobes - 1;
            float acc = 0.f;
            for (uint32_t k = 0; k < nlobes; ++k) {
                acc += lp[k];
                if (u[5] < acc) {
                    sel = k;
                    break;
                }
            }
            while (sel > 0 && lp[sel] == 0.f) --sel;
            const kz_lobe& ls = mat.lobes[sel];
            const LobeSample smp = lobe_sample(ls, wi, u[6], u[7], u[8]);
            alive = smp.valid;
            f3 weight = mk(0.f, 0.f, 0.f);
            float pdf_dir = 0.f;
            if (alive) {
                if (smp.delta) {
                    weight = hmul(lobe_weight(ls, textured, tint), smp.weight) * (1.f / lp[sel]);
                } else {
                    f3 f = mk(0.f, 0.f, 0.f);
                    float pdf = 0.f;
                    for (uint32_t k = 0; k < nlobes; ++k) {
                        const kz_lobe& lb = mat.lobes[k];
                        if (lobe_is_delta(lb.closure_id)) continue;
                        const LobeEval e = lobe_eval(lb, wi, smp.wo);
                        f = f + hmul(lobe_weight(lb, textured, tint), e.f);
                        pdf += lp[k] * e.pdf;
                    }
                    alive = pdf > 0.f;
                    if (alive) weight = f * (1.f / pdf);
                    pdf_dir = pdf;
                }
            }
            if (alive) {
                beta = hmul(beta, weight);
                alive = !is_zero(beta);
            }
            if (alive) {
                const f3 dn = normalize(fr.to_world(smp.wo));
                out.cont = true;
                out.o_next = make_float4(P.x, P.y, P.z, pdf_dir);
                out.d_next = make_float4(
                    dn.x, dn.y, dn.z,
                    __uint_as_float((depth + 1) | (smp.delta ? kSpecularFlag : 0u) | (flags & kJobMask)));
                out.b_next = make_float4(beta.x, beta.y, beta.z, b4.w);
                out.rng_next = rng.state;
            }
        }
        out.Lsum = Lsum;
        out.film_idx = film_idx;
    } else if (s.has_env) {
        // a miss: throughput times the environment, without MIS (the
        // environment is not sampled as a light), integrator.cpp:545-552
        const uint32_t pid = __float_as_uint(b4.w);
        out.Lsum = hmul(xyz(b4), env_radiance(s, xyz(d4)));
        out.film_idx = pid / pp.spp;
        if (kGuided && gs.recs) {
            const uint32_t depth = __float_as_uint(d4.w) & 0xffu;
            propagate(gs.recs, ((uint64_t)pid - gs.pass_first) * pp.max_depth, depth, out.Lsum);
        }
    }
}

__device__ __forceinline__ uint32_t find_job(const DevJob* __restrict__ jobs, uint32_t n_jobs, unsigned long long g) {
    uint32_t lo = 0, hi = n_jobs;  // last job with path_begin <= g
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (jobs[mid].path_begin <= g) lo = mid;
        else hi = mid;
    }
    return lo;
}

// The traversal reads only these fields of a scene.
__device__ __forceinline__ void trace_fields(DevScene& dst, const DevScene& src) {
    dst.nodes = src.nodes;
    dst.tris = src.tris;
    dst.n_nodes = src.n_nodes;
    dst.n_tris = src.n_tris;
}

// ---- stages of the batched wavefront (jobs of several scenes in one
// wavefront), as device functions shared by the per-stage kernels and the
// single persistent kernel of KZ_BATCH_PERSISTENT.

// Closest hits of the wavefront's paths; each path's scene through its job.
__device__ __forceinline__ void batch_trace_paths(ClosestSmem& m, const DevJob* __restrict__ jobs, PathSoA p,
                                                  DevCounters* ctr) {
    uint32_t dn = 0, dt = 0;
    DevScene ls;
    persistent_closest_in<false, true>(
        m, ls, ctr->n_active, &ctr->trace_next, &ctr->status,
        [&](uint32_t k, TRay& r, float& tmax) {
            const float4 o = p.o4[k], d = p.d4[k];
            trace_fields(ls, jobs[__float_as_uint(d.w) >> kJobShift].scene);
            r = make_tray(xyz(o), xyz(d), kRayEps);
            tmax = __int_as_float(0x7f800000);
        },
        [&](uint32_t k, const HitRec& h) { p.hit[k] = make_float4(h.t, h.u, h.v, __int_as_float(h.rec)); }, dn, dt);
}

// Shadow rays of the wavefront; an unoccluded one adds its contribution to
// its job's film.
__device__ __forceinline__ void batch_trace_shadow(AnySmem& m, const DevJob* __restrict__ jobs, ShadowSoA sq,
                                                   DevCounters* ctr) {
    uint32_t dn = 0, dt = 0;
    DevScene ls;
    persistent_any_in<false, true>(
        m, ls, ctr->n_shadow, &ctr->shadow_next,
        [&](uint32_t k, TRay& r, float& tmax) {
            const float4 o = sq.o4[k], d = sq.d4[k];
            trace_fields(ls, jobs[__float_as_uint(sq.c4[k].w)].scene);
            r = make_tray(xyz(o), xyz(d), kRayEps);
            tmax = o.w;
        },
        [&](uint32_t ray, int rc) {
            if (rc < 0) set_status(&ctr->status, KZ_ERR_STACK);
            if (rc == 1)
                film_add(jobs[__float_as_uint(sq.c4[ray].w)].film, nullptr, __float_as_uint(sq.d4[ray].w),
                         xyz(sq.c4[ray]));
        },
        dn, dt);
}

// Camera path j of this iteration's generation (j < gen_count).
__device__ __forceinline__ void batch_generate(const DevJob* __restrict__ jobs, uint32_t n_jobs, PathSoA dst,
                                               const DevCounters* c, uint32_t j) {
    const unsigned long long g = c->gen_first + j;
    const uint32_t job = find_job(jobs, n_jobs, g);
    const DevJob& J = jobs[job];
    const uint32_t k = c->gen_slot + j;
    generate_camera_path(J.cam, J.pp, dst, k, g - J.path_begin);
    dst.d4[k].w = __uint_as_float(__float_as_uint(dst.d4[k].w) | (job << kJobShift));
}

// Counters of one iteration of the device-driven loop: how many new paths
// fill the free slots (when `generate`), and the per-iteration cursors reset.
__device__ __forceinline__ void plan_iteration(DevCounters* c, uint32_t cap, bool generate) {
    const uint64_t remaining = c->total - c->next_path;
    const uint32_t room = cap - c->n_active;
    const uint32_t n_new = generate ? (uint32_t)(remaining < room ? remaining : room) : 0u;
    c->gen_first = c->next_path;
    c->gen_count = n_new;
    c->gen_slot = c->n_active;
    c->next_path += n_new;
    c->n_active += n_new;
    c->n_next = 0;
    c->n_shadow = 0;
    c->trace_next = 0;
    c->shadow_next = 0;
    if (c->n_active) {
        c->iterations += 1;
        c->path_bounces += c->n_active;
    }
}

// End of an iteration: the continuing paths become the next wavefront.
__device__ __forceinline__ void finish_iteration(DevCounters* c) {
    c->shadow_rays += c->n_shadow;
    c->n_active = c->n_next;
}

inline unsigned grid_for(uint64_t n, unsigned block) { return (unsigned)((n + block - 1) / block); }

// Blocks of `block` threads resident on the whole device for kernel f.
template <typename F>
static unsigned resident_grid(F f, unsigned block) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, f, (int)block, 0);
    return (unsigned)(sms > 0 ? sms : 1) * (unsigned)(per_sm > 0 ? per_sm : 1);
}

// Shading kind of a traced path: 0 a miss, 1 + the material's shading class
// for a hit (diffuse-like, glossy, delta, no lobe).
__device__ __forceinline__ uint32_t shade_kind(const DevScene& s, const float4 hit) {
    const int rec = __float_as_int(hit.w);
    if (rec < 0) return 0u;
    const uint32_t m = __float_as_uint(__ldg(reinterpret_cast<const float*>(s.tris + (size_t)rec * 3 + 2) + 3));
    return 1u + __ldg(s.mat_class + m);
}

// Regroups a block's paths by kind (0..5, 5 = no path) before they are
// shaded, so each warp runs one branch of shade_vertex: a counting sort in
// shared memory; returns the path index this thread shades. The order within
// a kind is arbitrary; each path's result is not. blockDim.x <= 256.
__device__ __forceinline__ uint32_t block_group_by_kind(uint32_t i, uint32_t kind) {
    __shared__ uint32_t s_cnt[6];
    __shared__ uint32_t s_perm[256];
    if (threadIdx.x < 6) s_cnt[threadIdx.x] = 0u;
    __syncthreads();
    const uint32_t rank = atomicAdd(&s_cnt[kind], 1u);
    __syncthreads();
    uint32_t first = 0u;
    for (uint32_t k = 0; k < kind; ++k) first += s_cnt[k];
    s_perm[first + rank] = i;
    __syncthreads();
    return s_perm[threadIdx.x];
}

// Plain shading runs 6 blocks per SM (40 registers, ~770 bytes of spills to
// L1): the kernel waits on dependent loads, and more warps hide more of
// them. Terrain frame shade stage at 4 / 5 / 6 / 7 / 8 blocks per SM: 32.5 /
// 31.6 / 31.1 / 31.9 / 31.9 ms (3 and 2 blocks, more registers: slower).
#ifndef KZ_SHADE_MIN_BLOCKS
#define KZ_SHADE_MIN_BLOCKS 6
#endif
// The guided variant at 3 blocks per SM (80 registers, ~200 bytes of spills):
// slit room 1024^2, 64 spp, shade stage 88.2 ms at 1 or 2 blocks (126 / 114
// registers), 80.9 ms at 3, 84.0 ms at 4 (64 registers, 728 bytes of spills).
#ifndef KZ_SHADE_GUIDED_MIN_BLOCKS
#define KZ_SHADE_GUIDED_MIN_BLOCKS 3
#endif
// KZ_SHADE_SORT: group each block's paths by kind (miss, material shading
// class) before shading them. Measured on the terrain frame: shade stage
// 40.4 -> 33.4 ms, trace +1.3 ms (the next wavefront's order changes), frame
// 1,441 -> 1,480 Mpaths*bounces/s. (Also writing the continuing paths
// grouped by the octant of their next direction, one atomic per block,
// measured trace -3.0 ms but shade +4.2 ms: not kept.)
#ifndef KZ_SHADE_SORT
#define KZ_SHADE_SORT 1
#endif
template <bool kGuided, bool kAttr = true>
__global__ void __launch_bounds__(256, kGuided ? KZ_SHADE_GUIDED_MIN_BLOCKS : KZ_SHADE_MIN_BLOCKS)
    k_shade(DevScene s, PathParams pp, PathSoA in, uint32_t n_in, PathSoA out,
                                               ShadowSoA sq, DevCounters* ctr, float* film, double* film64,
                                               GuideShade gs, const uint32_t* n_dev) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (n_dev) n_in = *n_dev;
#if KZ_SHADE_SORT
    i = block_group_by_kind(i, i < n_in ? shade_kind(s, in.hit[i]) : 5u);
#endif
    ShadeOut so;
    if (i < n_in) {
        shade_vertex<kGuided, kAttr>(s, pp, in.hit[i], in.o4[i], in.d4[i], in.b4[i], in.rng[i], gs,
                                     kGuided ? gs.raw + (size_t)i * kGuideOut : nullptr, so);
        if (!is_zero(so.Lsum)) film_add(film, film64, so.film_idx, so.Lsum);
    }
    const bool cont = so.cont, shadow = so.shadow;
    const uint32_t slot = warp_append(cont, &ctr->n_next);
    if (cont) {
        out.o4[slot] = so.o_next;
        out.d4[slot] = so.d_next;
        out.b4[slot] = so.b_next;
        out.rng[slot] = so.rng_next;
    }
    const uint32_t sslot = warp_append(shadow, &ctr->n_shadow);
    if (shadow) {
        sq.o4[sslot] = so.s_o;
        sq.d4[sslot] = so.s_d;
        sq.c4[sslot] = so.s_c;
    }
}

}  // namespace
}  // namespace kz
