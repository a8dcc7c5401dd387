// kz_trace.cu — sm_103a traversal kernels: batch intersection (closest,
// any, fetch counts) and the path tracer's closest-hit and shadow passes, as
// host-count kernels and as persistent kernels that refill idle lanes from a
// global cursor, for single renders and batched jobs.
#include "kz_stages.cuh"

// Resident 256-thread blocks per SM the persistent traversal kernels are
// compiled for (4: at most 64 registers a thread).
#ifndef KZ_TRACE_MINB
#define KZ_TRACE_MINB 4
#endif

namespace kz {
namespace {

// kz_intersect_any: rays (o, tmin, d, tmax) in, an occlusion byte out.
__global__ void __launch_bounds__(256, KZ_TRACE_MINB) k_intersect_any_persistent(DevScene s,
                                                                                 const kz_ray* __restrict__ rays,
                                                                                 unsigned long long n, uint8_t* occ,
                                                                                 unsigned long long* next,
                                                                                 uint32_t* status) {
    uint32_t dn = 0, dt = 0;
    persistent_any<false>(
        s, n, next,
        [&](unsigned long long k, TRay& r, float& tmax) {
            const float4* rp = reinterpret_cast<const float4*>(rays + k);
            const float4 a = __ldg(rp), b = __ldg(rp + 1);
            r = make_tray(mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), a.w);
            tmax = b.w;
        },
        [&](unsigned long long k, int rc) {
            if (rc < 0) set_status(status, KZ_ERR_STACK);
            occ[k] = rc == 2 ? 1 : 0;
        },
        dn, dt);
}

__global__ void k_intersect_stats(DevScene s, const kz_ray* __restrict__ rays, uint64_t n,
                                  unsigned long long* counters, uint32_t* status) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t nn = 0, nt = 0;
    if (i < n) {
        const float4* rp = reinterpret_cast<const float4*>(rays + i);
        const float4 a = __ldg(rp), b = __ldg(rp + 1);
        TRay r = make_tray(mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), a.w);
        HitRec h;
        if (!trace_closest<true>(s, r, b.w, h, nn, nt)) set_status(status, KZ_ERR_STACK);
    }
    // warp reduction, one atomic per warp
    unsigned long long a0 = nn, a1 = nt;
    for (int o = 16; o > 0; o >>= 1) {
        a0 += __shfl_down_sync(0xffffffffu, a0, o);
        a1 += __shfl_down_sync(0xffffffffu, a1, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(counters, a0);
        atomicAdd(counters + 1, a1);
    }
}

template <bool kCount>
__global__ void __launch_bounds__(256) k_trace_paths(DevScene s, PathSoA p, uint32_t n, DevCounters* ctr,
                                                     const uint32_t* n_dev) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (n_dev) n = *n_dev;
    uint32_t dn = 0, dt = 0;
    if (i < n) {
        const float4 o = p.o4[i], d = p.d4[i];
        TRay r = make_tray(xyz(o), xyz(d), kRayEps);
        HitRec h;
        if (!trace_closest<kCount>(s, r, __int_as_float(0x7f800000), h, dn, dt)) {
            set_status(&ctr->status, KZ_ERR_STACK);
            h.rec = -1;
        }
        p.hit[i] = make_float4(h.t, h.u, h.v, __int_as_float(h.rec));
    }
    if (kCount) warp_count(dn, dt, &ctr->fetch[0]);
}

template <bool kCount>
__global__ void __launch_bounds__(256, KZ_TRACE_MINB) k_trace_paths_persistent(DevScene s, PathSoA p, DevCounters* ctr) {
    uint32_t dn = 0, dt = 0;
    persistent_closest<kCount>(
        s, ctr->n_active, &ctr->trace_next, &ctr->status,
        [&](uint32_t k, TRay& r, float& tmax) {
            const float4 o = p.o4[k], d = p.d4[k];
            r = make_tray(xyz(o), xyz(d), kRayEps);
            tmax = __int_as_float(0x7f800000);
        },
        [&](uint32_t k, const HitRec& h) { p.hit[k] = make_float4(h.t, h.u, h.v, __int_as_float(h.rec)); }, dn, dt);
    if (kCount) warp_count(dn, dt, &ctr->fetch[0]);
}

// kz_intersect_closest: rays (o, tmin, d, tmax) in, hit fields out.
__global__ void __launch_bounds__(256, KZ_TRACE_MINB) k_intersect_closest_persistent(DevScene s, const kz_ray* __restrict__ rays,
                                                                      unsigned long long n, kz_hits hits,
                                                                      unsigned long long* next, uint32_t* status) {
    uint32_t dn = 0, dt = 0;
    persistent_closest<false>(
        s, n, next, status,
        [&](unsigned long long k, TRay& r, float& tmax) {
            const float4* rp = reinterpret_cast<const float4*>(rays + k);
            const float4 a = __ldg(rp), b = __ldg(rp + 1);
            r = make_tray(mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), a.w);
            tmax = b.w;
        },
        [&](unsigned long long k, const HitRec& h) { store_hit(s, hits, k, h); }, dn, dt);
}

template <bool kCount, bool kGuided>
__global__ void __launch_bounds__(256) k_trace_shadow(DevScene s, ShadowSoA sq, DevCounters* ctr, float* film,
                                                      double* film64, VRec* recs, NRec* nee, uint32_t max_depth) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t dn = 0, dt = 0;
    if (i < ctr->n_shadow) {
        const float4 o = sq.o4[i], d = sq.d4[i];
        TRay r = make_tray(xyz(o), xyz(d), kRayEps);
        bool overflow;
        const bool occluded = trace_any<kCount>(s, r, o.w, overflow, dn, dt);
        if (overflow) set_status(&ctr->status, KZ_ERR_STACK);
        if (!occluded && !overflow) {
            const float4 c = sq.c4[i];
            film_add(film, film64, __float_as_uint(d.w), xyz(c));
            if (kGuided && recs) {
                const uint32_t tag = __float_as_uint(c.w);
                const uint64_t rb = (uint64_t)(tag >> 4) * max_depth;
                propagate(recs, rb, tag & 15u, xyz(c));
                if (nee) nee[rb + (tag & 15u)].n.w = 1.f;
            }
        }
    }
    if (kCount) warp_count(dn, dt, &ctr->fetch[2]);
}

// Persistent form of k_trace_shadow for the device-driven loop (k_plan zeroes
// shadow_next each iteration).
template <bool kCount, bool kGuided>
__global__ void __launch_bounds__(256, KZ_TRACE_MINB) k_trace_shadow_persistent(DevScene s, ShadowSoA sq, DevCounters* ctr,
                                                                 float* film, double* film64, VRec* recs, NRec* nee,
                                                                 uint32_t max_depth) {
    uint32_t dn = 0, dt = 0;
    const auto unoccluded = [&](uint32_t ray) {
        const float4 cc = sq.c4[ray];
        film_add(film, film64, __float_as_uint(sq.d4[ray].w), xyz(cc));
        if (kGuided && recs) {
            const uint32_t tag = __float_as_uint(cc.w);
            const uint64_t rb = (uint64_t)(tag >> 4) * max_depth;
            propagate(recs, rb, tag & 15u, xyz(cc));
            if (nee) nee[rb + (tag & 15u)].n.w = 1.f;
        }
    };
#if KZ_SHARE_LEAVES
    persistent_any<kCount>(
        s, ctr->n_shadow, &ctr->shadow_next,
        [&](uint32_t k, TRay& r, float& tmax) {
            const float4 o = sq.o4[k], d = sq.d4[k];
            r = make_tray(xyz(o), xyz(d), kRayEps);
            tmax = o.w;
        },
        [&](uint32_t ray, int rc) {
            if (rc < 0) set_status(&ctr->status, KZ_ERR_STACK);
            if (rc == 1) unoccluded(ray);
        },
        dn, dt);
#else
    uint2 stack_lm[kWideStack];
    const LocalStack stack{stack_lm};
    AnyState c;
    TRay r;
    float tmax = 0.f;
    uint32_t octp = 0, ray = 0;
    persistent_rays(
        ctr->n_shadow, &ctr->shadow_next, kTraceRefill,
        [&](uint32_t k) {
            ray = k;
            const float4 o = sq.o4[k], d = sq.d4[k];
            r = make_tray(xyz(o), xyz(d), kRayEps);
            tmax = o.w;
            octp = wide_octant(r);
            any_begin(c);
        },
        [&]() {
            const int rc = any_step<kCount>(s, r, octp, tmax, c, stack, dn, dt);
            if (rc == 0) return false;
            if (rc < 0) set_status(&ctr->status, KZ_ERR_STACK);
            if (rc == 1) unoccluded(ray);
            return true;
        });
#endif
    if (kCount) warp_count(dn, dt, &ctr->fetch[2]);
}

// Training samples from the records of a guided pass: every valid vertex
// whose integrand estimate L*f*cos is positive, weighted by its luminance
// over the pdf the direction was sampled with.

__global__ void __launch_bounds__(256, KZ_TRACE_MINB) k_trace_paths_batch(const DevJob* __restrict__ jobs, PathSoA p,
                                                                          DevCounters* ctr) {
    __shared__ ClosestSmem m;
    batch_trace_paths(m, jobs, p, ctr);
}

__global__ void __launch_bounds__(256, KZ_TRACE_MINB) k_trace_shadow_batch(const DevJob* __restrict__ jobs,
                                                                           ShadowSoA sq, DevCounters* ctr) {
    __shared__ AnySmem m;
    batch_trace_shadow(m, jobs, sq, ctr);
}

}  // namespace

void launch_intersect_closest(const DevScene& s, const kz_ray* rays, uint64_t n, kz_hits hits,
                              unsigned long long* next, uint32_t* status, cudaStream_t st) {
    if (!n) return;
    static const unsigned g = resident_grid(k_intersect_closest_persistent, 256);
    k_intersect_closest_persistent<<<(unsigned)std::min<uint64_t>(g, grid_for(n, 256)), 256, 0, st>>>(s, rays, n, hits,
                                                                                                     next, status);
}

void launch_intersect_any(const DevScene& s, const kz_ray* rays, uint64_t n, uint8_t* occ,
                          unsigned long long* next, uint32_t* status, cudaStream_t st) {
    if (!n) return;
    static const unsigned g = resident_grid(k_intersect_any_persistent, 256);
    k_intersect_any_persistent<<<(unsigned)std::min<uint64_t>(g, grid_for(n, 256)), 256, 0, st>>>(s, rays, n, occ,
                                                                                                 next, status);
}

void launch_intersect_stats(const DevScene& s, const kz_ray* rays, uint64_t n, unsigned long long* counters,
                            uint32_t* status, cudaStream_t st) {
    if (!n) return;
    k_intersect_stats<<<grid_for(n, 128), 128, 0, st>>>(s, rays, n, counters, status);
}

void launch_trace_paths(const DevScene& s, PathSoA p, uint32_t n, DevCounters* ctr, bool count, uint32_t block,
                        cudaStream_t st) {
    if (!n) return;
    if (count) k_trace_paths<true><<<grid_for(n, block), block, 0, st>>>(s, p, n, ctr, nullptr);
    else k_trace_paths<false><<<grid_for(n, block), block, 0, st>>>(s, p, n, ctr, nullptr);
}

// The device-driven loop's closest-hit pass: persistent, 256-thread blocks,
// as many as are resident.
void launch_trace_paths_dev(const DevScene& s, PathSoA p, uint32_t cap, DevCounters* ctr, bool count, uint32_t,
                            cudaStream_t st) {
    if (!cap) return;
    if (count) {
        static const unsigned g = resident_grid(k_trace_paths_persistent<true>, 256);
        k_trace_paths_persistent<true><<<std::min(g, grid_for(cap, 256)), 256, 0, st>>>(s, p, ctr);
    } else {
        static const unsigned g = resident_grid(k_trace_paths_persistent<false>, 256);
        k_trace_paths_persistent<false><<<std::min(g, grid_for(cap, 256)), 256, 0, st>>>(s, p, ctr);
    }
}

void launch_trace_shadow_guided(const DevScene& s, ShadowSoA sq, uint32_t n_max, DevCounters* ctr, float* film,
                                double* film64, VRec* recs, NRec* nee, uint32_t max_depth, uint32_t block,
                                cudaStream_t st) {
    if (!n_max) return;
    static const unsigned g = resident_grid(k_trace_shadow_persistent<false, true>, 256);
    k_trace_shadow_persistent<false, true><<<std::min(g, grid_for(n_max, 256)), 256, 0, st>>>(
        s, sq, ctr, film, film64, recs, nee, max_depth);
}

void launch_trace_shadow_dev(const DevScene& s, ShadowSoA sq, uint32_t n_max, DevCounters* ctr, bool count,
                             float* film, double* film64, cudaStream_t st) {
    if (!n_max) return;
    if (count) {
        static const unsigned g = resident_grid(k_trace_shadow_persistent<true, false>, 256);
        k_trace_shadow_persistent<true, false><<<std::min(g, grid_for(n_max, 256)), 256, 0, st>>>(
            s, sq, ctr, film, film64, nullptr, nullptr, 0);
    } else {
        static const unsigned g = resident_grid(k_trace_shadow_persistent<false, false>, 256);
        k_trace_shadow_persistent<false, false><<<std::min(g, grid_for(n_max, 256)), 256, 0, st>>>(
            s, sq, ctr, film, film64, nullptr, nullptr, 0);
    }
}

void launch_trace_shadow(const DevScene& s, ShadowSoA sq, uint32_t n_max, DevCounters* ctr, bool count, float* film,
                         double* film64, uint32_t block, cudaStream_t st) {
    if (!n_max) return;
    if (count)
        k_trace_shadow<true, false><<<grid_for(n_max, block), block, 0, st>>>(s, sq, ctr, film, film64, nullptr,
                                                                              nullptr, 0);
    else
        k_trace_shadow<false, false><<<grid_for(n_max, block), block, 0, st>>>(s, sq, ctr, film, film64, nullptr,
                                                                               nullptr, 0);
}

static unsigned grid_trace_batch() {
    static const unsigned g = resident_grid(k_trace_paths_batch, 256);
    return g;
}

static unsigned grid_shadow_batch() {
    static const unsigned g = resident_grid(k_trace_shadow_batch, 256);
    return g;
}

void prepare_batch_wavefront() {
    (void)grid_trace_batch();
    (void)grid_shadow_batch();
}

void launch_trace_paths_batch(const DevJob* jobs, PathSoA p, uint32_t cap, DevCounters* ctr, cudaStream_t st) {
    if (!cap) return;
    k_trace_paths_batch<<<std::min(grid_trace_batch(), grid_for(cap, 256)), 256, 0, st>>>(jobs, p, ctr);
}

void launch_trace_shadow_batch(const DevJob* jobs, ShadowSoA sq, uint32_t cap, DevCounters* ctr, cudaStream_t st) {
    if (!cap) return;
    k_trace_shadow_batch<<<std::min(grid_shadow_batch(), grid_for(cap, 256)), 256, 0, st>>>(jobs, sq, ctr);
}

}  // namespace kz
