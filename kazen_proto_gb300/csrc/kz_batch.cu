// kz_batch.cu — batched rendering, wavefront mode: generation and shading
// over a job table (the traversal passes are in kz_trace.cu, the megakernel
// mode in kz_megakernel.cu).
#include "kz_stages.cuh"

namespace kz {
namespace {

// ------------------------------------------------------------------ batched wavefront
// Many jobs in one wavefront: paths of all jobs share the path buffers and
// the stage kernels; each path finds its scene, camera, parameters and film
// through its job index (d4.w bits 12-31, c4.w for shadow rays). Global path
// ids [0, total) are generated in job order; a path's own id is local to its
// job, so every job renders exactly what kz_render renders for it.

__global__ void k_generate_batch_dev(const DevJob* __restrict__ jobs, uint32_t n_jobs, PathSoA dst,
                                     const DevCounters* c) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= c->gen_count) return;
    const unsigned long long g = c->gen_first + j;
    const uint32_t job = find_job(jobs, n_jobs, g);
    const DevJob& J = jobs[job];
    const uint32_t k = c->gen_slot + j;
    generate_camera_path(J.cam, J.pp, dst, k, g - J.path_begin);
    dst.d4[k].w = __uint_as_float(__float_as_uint(dst.d4[k].w) | (job << kJobShift));
}

template <bool kAttr>
__global__ void __launch_bounds__(256, 4) k_shade_batch(const DevJob* __restrict__ jobs, PathSoA in, PathSoA out,
                                                     ShadowSoA sq, DevCounters* ctr) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n_in = ctr->n_active;
#if KZ_SHADE_SORT
    i = block_group_by_kind(
        i, i < n_in ? shade_kind(jobs[__float_as_uint(in.d4[i].w) >> kJobShift].scene, in.hit[i]) : 5u);
#endif
    ShadeOut so;
    if (i < n_in) {
        const float4 d4 = in.d4[i];
        const DevJob& J = jobs[__float_as_uint(d4.w) >> kJobShift];
        shade_vertex<false, kAttr>(J.scene, J.pp, in.hit[i], in.o4[i], d4, in.b4[i], in.rng[i], GuideShade{}, nullptr,
                                  so);
        if (!is_zero(so.Lsum)) film_add(J.film, nullptr, so.film_idx, so.Lsum);
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

void launch_generate_batch_dev(const DevJob* jobs, uint32_t n_jobs, PathSoA dst, DevCounters* ctr, uint32_t cap,
                               uint32_t block, cudaStream_t st) {
    if (!cap) return;
    k_generate_batch_dev<<<grid_for(cap, block), block, 0, st>>>(jobs, n_jobs, dst, ctr);
}
void launch_shade_batch(const DevJob* jobs, PathSoA in, uint32_t cap, PathSoA out, ShadowSoA sq, DevCounters* ctr,
                        uint32_t block, bool textured, cudaStream_t st) {  // textured: textures or normals
    if (!cap) return;
    if (textured)
        k_shade_batch<true><<<grid_for(cap, block), block, 0, st>>>(jobs, in, out, sq, ctr);
    else
        k_shade_batch<false><<<grid_for(cap, block), block, 0, st>>>(jobs, in, out, sq, ctr);
}

}  // namespace kz
