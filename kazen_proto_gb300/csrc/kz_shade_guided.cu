// kz_shade_guided.cu — the guided shading kernels (k_shade<true, kAttr>,
// kz_stages.cuh) in a translation unit of their own, so they compile in
// parallel with the plain ones; the variant without vertex attributes runs
// for scenes that have no textures and no vertex normals.
// The guided kernel inlines lobe_eval / lobe_sample: called out of line they
// raise it to 162 registers and one block per SM (measured: 2,944 guided spp
// in the equal-time budget against 3,456-3,520 inlined), while the plain
// kernels gain from the single copy.
#define KZ_LOBE_INLINE
#include "kz_stages.cuh"

namespace kz {

void launch_shade_guided(const DevScene& s, const PathParams& pp, PathSoA in, uint32_t n_in, PathSoA out,
                         ShadowSoA sq, DevCounters* ctr, float* film, double* film64, const GuideShade& gs,
                         uint32_t block, cudaStream_t st) {
    if (!n_in) return;
    if (s.mat_tex || s.tri_nrm)
        k_shade<true, true><<<grid_for(n_in, block), block, 0, st>>>(s, pp, in, n_in, out, sq, ctr, film, film64, gs,
                                                                     nullptr);
    else
        k_shade<true, false><<<grid_for(n_in, block), block, 0, st>>>(s, pp, in, n_in, out, sq, ctr, film, film64,
                                                                      gs, nullptr);
}
void launch_shade_guided_dev(const DevScene& s, const PathParams& pp, PathSoA in, uint32_t cap, PathSoA out,
                             ShadowSoA sq, DevCounters* ctr, float* film, double* film64, const GuideShade& gs,
                             uint32_t block, cudaStream_t st) {
    if (!cap) return;
    if (s.mat_tex || s.tri_nrm)
        k_shade<true, true><<<grid_for(cap, block), block, 0, st>>>(s, pp, in, cap, out, sq, ctr, film, film64, gs,
                                                                    &ctr->n_active);
    else
        k_shade<true, false><<<grid_for(cap, block), block, 0, st>>>(s, pp, in, cap, out, sq, ctr, film, film64, gs,
                                                                     &ctr->n_active);
}

}  // namespace kz
