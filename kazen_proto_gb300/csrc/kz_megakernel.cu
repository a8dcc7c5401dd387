// kz_megakernel.cu — batched rendering, megakernel mode (KZ_BATCH_MEGAKERNEL).
#include "kz_stages.cuh"

namespace kz {
namespace {

// ------------------------------------------------------------------ persistent batch renderer
// Many independent jobs (scenes, cameras, films) in one launch. Lanes hold a
// path each; every `period` vertices (or when a warp has no live path) free
// lanes take the next global path ids with one atomic per warp, find their
// job by binary search over the jobs' first path ids, and start a camera
// path. Each vertex is traced, shaded (shade_vertex) and its shadow ray
// traced inline. Loop exit is warp-uniform: the fetch counter only grows and
// ends the loop once it passes the total with no live lane left.
__global__ void __launch_bounds__(256) k_render_batch(const DevJob* __restrict__ jobs, uint32_t n_jobs,
                                                      unsigned long long total, BatchCounters* bc, uint32_t period) {
    const int lane = threadIdx.x & 31;
    bool active = false, exhausted = false;
    uint32_t job = 0;
    float4 o4 = make_float4(0.f, 0.f, 0.f, 0.f), d4 = o4, b4 = o4;
    unsigned long long rng = 0;
    unsigned long long n_bounce = 0, n_shadow = 0;
    for (uint32_t step = 0;; ++step) {
        const bool any_live = __any_sync(0xffffffffu, active);
        if (!exhausted && (step % period == 0 || !any_live)) {
            const unsigned want = __ballot_sync(0xffffffffu, !active);
            if (want) {
                const int leader = __ffs(want) - 1;
                unsigned long long base = 0;
                if (lane == leader) base = atomicAdd(&bc->next_path, (unsigned long long)__popc(want));
                base = __shfl_sync(0xffffffffu, base, leader);
                if (!active) {
                    const unsigned long long g = base + (unsigned)__popc(want & ((1u << lane) - 1u));
                    if (g < total) {
                        job = find_job(jobs, n_jobs, g);
                        const DevJob& J = jobs[job];
                        PathSoA one;
                        one.o4 = &o4;
                        one.d4 = &d4;
                        one.b4 = &b4;
                        one.rng = &rng;
                        generate_camera_path(J.cam, J.pp, one, 0, g - J.path_begin);
                        active = true;
                    }
                }
                if (base + (unsigned)__popc(want) >= total) exhausted = true;
            }
        }
        if (!__any_sync(0xffffffffu, active)) {
            if (exhausted) break;
            continue;
        }
        if (active) {
            const DevJob& J = jobs[job];
            TRay r = make_tray(xyz(o4), xyz(d4), kRayEps);
            HitRec h;
            uint32_t dn = 0, dt = 0;
            if (!trace_closest<false>(J.scene, r, __int_as_float(0x7f800000), h, dn, dt)) {
                set_status(&bc->status, KZ_ERR_STACK);
                h.rec = -1;
            }
            ++n_bounce;
            ShadeOut so;
            shade_vertex<false>(J.scene, J.pp, make_float4(h.t, h.u, h.v, __int_as_float(h.rec)), o4, d4, b4, rng,
                                GuideShade{}, nullptr, so);
            if (!is_zero(so.Lsum)) film_add(J.film, nullptr, so.film_idx, so.Lsum);
            if (so.shadow) {
                ++n_shadow;
                TRay sr = make_tray(xyz(so.s_o), xyz(so.s_d), kRayEps);
                bool overflow;
                const bool occ = trace_any<false>(J.scene, sr, so.s_o.w, overflow, dn, dt);
                if (overflow) set_status(&bc->status, KZ_ERR_STACK);
                if (!occ && !overflow) film_add(J.film, nullptr, __float_as_uint(so.s_d.w), xyz(so.s_c));
            }
            if (so.cont) {
                o4 = so.o_next;
                d4 = so.d_next;
                b4 = so.b_next;
                rng = so.rng_next;
            } else {
                active = false;
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        n_bounce += __shfl_down_sync(0xffffffffu, n_bounce, o);
        n_shadow += __shfl_down_sync(0xffffffffu, n_shadow, o);
    }
    if (lane == 0) {
        atomicAdd(&bc->path_bounces, n_bounce);
        atomicAdd(&bc->shadow_rays, n_shadow);
    }
}

}  // namespace

void launch_render_batch(const DevJob* jobs, uint32_t n_jobs, unsigned long long total, BatchCounters* bc,
                         uint32_t period, uint32_t ctas, uint32_t block, cudaStream_t st) {
    if (!n_jobs || !total) return;
    k_render_batch<<<ctas, block, 0, st>>>(jobs, n_jobs, total, bc, period ? period : 1u);
}

}  // namespace kz
