// kz_shade_guided.cu — the guided shading kernel (k_shade<true>, kz_stages.cuh)
// in a translation unit of its own, so it compiles in parallel with the plain
// one.
#include "kz_stages.cuh"

namespace kz {

void launch_shade_guided(const DevScene& s, const PathParams& pp, PathSoA in, uint32_t n_in, PathSoA out,
                         ShadowSoA sq, DevCounters* ctr, float* film, double* film64, const GuideShade& gs,
                         uint32_t block, cudaStream_t st) {
    if (!n_in) return;
    k_shade<true><<<grid_for(n_in, block), block, 0, st>>>(s, pp, in, n_in, out, sq, ctr, film, film64, gs, nullptr);
}
void launch_shade_guided_dev(const DevScene& s, const PathParams& pp, PathSoA in, uint32_t cap, PathSoA out,
                             ShadowSoA sq, DevCounters* ctr, float* film, double* film64, const GuideShade& gs,
                             uint32_t block, cudaStream_t st) {
    if (!cap) return;
    k_shade<true><<<grid_for(cap, block), block, 0, st>>>(s, pp, in, cap, out, sq, ctr, film, film64, gs,
                                                          &ctr->n_active);
}

}  // namespace kz
