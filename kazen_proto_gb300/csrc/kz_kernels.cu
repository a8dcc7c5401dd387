// kz_kernels.cu — sm_103a kernels of the kazen hot path other than traversal:
// closure batches, path generation, shading (shade_vertex, kz_stages.cuh),
// training-sample collection for guiding, the batched renderers (wavefront
// stages over a job table, and the persistent megakernel) and the
// device-driven loop's bookkeeping kernels.
#include "kz_stages.cuh"

namespace kz {
namespace {

__global__ void k_generate_camera(DevCamera cam, PathParams pp, PathSoA dst, uint32_t dst_offset,
                                  uint64_t first_path, uint32_t n_new) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n_new) return;
    generate_camera_path(cam, pp, dst, dst_offset + j, first_path + j);
}

__global__ void k_generate_rays(const kz_ray* __restrict__ rays, PathParams pp, PathSoA dst, uint32_t dst_offset,
                                uint64_t first_path, uint32_t n_new) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n_new) return;
    generate_ray_path(rays, pp, dst, dst_offset + j, first_path + j);
}


__global__ void k_guide_collect(const VRec* __restrict__ recs, const NRec* __restrict__ nee, uint64_t n,
                                float4* __restrict__ samples, uint32_t cap, uint32_t* count, float* wsum) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool take = false;
    float4 a, b, c;
    if (i < n) {
        const VRec r = recs[i];
        const float lum = (0.2126f * r.L.x + 0.7152f * r.L.y + 0.0722f * r.L.z) * r.d.w;
        if (r.n.w != 0.f && lum > 0.f && r.p.w > 0.f && isfinite(lum)) {
            const float w = lum / r.p.w;
            take = isfinite(w);
            a = make_float4(r.p.x, r.p.y, r.p.z, w);
            b = make_float4(r.n.x, r.n.y, r.n.z, 0.f);
            c = make_float4(r.d.x, r.d.y, r.d.z, 0.f);
        }
    } else if (i < 2 * n && nee) {
        const NRec r = nee[i - n];
        if (r.n.w != 0.f && r.p.w > 0.f && isfinite(r.p.w)) {
            take = true;
            a = r.p;
            b = make_float4(r.n.x, r.n.y, r.n.z, 0.f);
            c = r.d;
        }
    }
    const uint32_t slot = warp_append(take, count);
    if (take && slot < cap) {
        samples[3 * (size_t)slot] = a;
        samples[3 * (size_t)slot + 1] = b;
        samples[3 * (size_t)slot + 2] = c;
        atomicAdd(wsum, a.w);
    }
}

// ------------------------------------------------------------------ device-driven loop
__global__ void k_plan(DevCounters* c, uint32_t cap, bool generate) { plan_iteration(c, cap, generate); }

__global__ void k_finish(DevCounters* c) { finish_iteration(c); }

__global__ void k_generate_camera_dev(DevCamera cam, PathParams pp, PathSoA dst, const DevCounters* c) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= c->gen_count) return;
    generate_camera_path(cam, pp, dst, c->gen_slot + j, c->gen_first + j);
}

__global__ void k_generate_rays_dev(const kz_ray* __restrict__ rays, PathParams pp, PathSoA dst,
                                    const DevCounters* c) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= c->gen_count) return;
    generate_ray_path(rays, pp, dst, c->gen_slot + j, c->gen_first + j);
}

__global__ void k_scale(float* film, double* film64, uint64_t n, float sf, double sd) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (film) film[i] *= sf;
    if (film64) film64[i] *= sd;
}

}  // namespace

void launch_generate_camera(const DevCamera& cam, const PathParams& pp, PathSoA dst, uint32_t dst_offset,
                            uint64_t first_path, uint32_t n_new, uint32_t block, cudaStream_t st) {
    if (!n_new) return;
    k_generate_camera<<<grid_for(n_new, block), block, 0, st>>>(cam, pp, dst, dst_offset, first_path, n_new);
}
void launch_generate_rays(const kz_ray* rays, const PathParams& pp, PathSoA dst, uint32_t dst_offset,
                          uint64_t first_path, uint32_t n_new, uint32_t block, cudaStream_t st) {
    if (!n_new) return;
    k_generate_rays<<<grid_for(n_new, block), block, 0, st>>>(rays, pp, dst, dst_offset, first_path, n_new);
}
void launch_plan(DevCounters* ctr, uint32_t cap, cudaStream_t st, bool generate) {
    k_plan<<<1, 1, 0, st>>>(ctr, cap, generate);
}
void launch_finish(DevCounters* ctr, cudaStream_t st) { k_finish<<<1, 1, 0, st>>>(ctr); }
void launch_generate_camera_dev(const DevCamera& cam, const PathParams& pp, PathSoA dst, DevCounters* ctr,
                                uint32_t cap, uint32_t block, cudaStream_t st) {
    if (!cap) return;
    k_generate_camera_dev<<<grid_for(cap, block), block, 0, st>>>(cam, pp, dst, ctr);
}
void launch_generate_rays_dev(const kz_ray* rays, const PathParams& pp, PathSoA dst, DevCounters* ctr, uint32_t cap,
                              uint32_t block, cudaStream_t st) {
    if (!cap) return;
    k_generate_rays_dev<<<grid_for(cap, block), block, 0, st>>>(rays, pp, dst, ctr);
}
void launch_shade_dev(const DevScene& s, const PathParams& pp, PathSoA in, uint32_t cap, PathSoA out, ShadowSoA sq,
                      DevCounters* ctr, float* film, double* film64, const GuideShade* gs, uint32_t block,
                      cudaStream_t st) {
    if (!cap) return;
    if (gs) {
        launch_shade_guided_dev(s, pp, in, cap, out, sq, ctr, film, film64, *gs, block, st);
        return;
    }
    if (s.mat_tex || s.tri_nrm)
        k_shade<false, true><<<grid_for(cap, block), block, 0, st>>>(s, pp, in, cap, out, sq, ctr, film, film64,
                                                                     GuideShade{}, &ctr->n_active);
    else
        k_shade<false, false><<<grid_for(cap, block), block, 0, st>>>(s, pp, in, cap, out, sq, ctr, film, film64,
                                                                      GuideShade{}, &ctr->n_active);
}
void launch_shade(const DevScene& s, const PathParams& pp, PathSoA in, uint32_t n_in, PathSoA out, ShadowSoA sq,
                  DevCounters* ctr, float* film, double* film64, uint32_t block, cudaStream_t st) {
    if (!n_in) return;
    if (s.mat_tex || s.tri_nrm)
        k_shade<false, true><<<grid_for(n_in, block), block, 0, st>>>(s, pp, in, n_in, out, sq, ctr, film, film64,
                                                                      GuideShade{}, nullptr);
    else
        k_shade<false, false><<<grid_for(n_in, block), block, 0, st>>>(s, pp, in, n_in, out, sq, ctr, film, film64,
                                                                       GuideShade{}, nullptr);
}
void launch_guide_collect(const VRec* recs, const NRec* nee, uint64_t n_recs, float4* samples, uint32_t cap,
                          uint32_t* count, float* wsum, cudaStream_t st) {
    if (!n_recs) return;
    k_guide_collect<<<grid_for(2 * n_recs, 256), 256, 0, st>>>(recs, nee, n_recs, samples, cap, count, wsum);
}
void launch_scale(float* film, double* film64, uint64_t n, float sf, double sd, cudaStream_t st) {
    if (!n) return;
    k_scale<<<grid_for(n, 256), 256, 0, st>>>(film, film64, n, sf, sd);
}

}  // namespace kz
