// kz_closures.cu — batch closure kernels (kz_closure_eval_batch /
// kz_closure_sample_batch): one lobe, incident and outgoing direction per
// thread, in the reference or the integrator convention (kz_device.cuh).
#include "kz_stages.cuh"

namespace kz {
namespace {

// ------------------------------------------------------------------ closures
__global__ void k_closure_eval(const kz_lobe* __restrict__ lobes, const float* __restrict__ wi,
                               const float* __restrict__ wo, uint64_t n, int conv, float* f, float* pdf) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const kz_lobe l = lobes[i];
    const f3 a = ld3(wi + 3 * i), b = ld3(wo + 3 * i);
    LobeEval e = conv == KZ_CONVENTION_REFERENCE ? lobe_eval_reference<true>(l, a, b) : lobe_eval(l, a, b);
    f[3 * i] = e.f.x;
    f[3 * i + 1] = e.f.y;
    f[3 * i + 2] = e.f.z;
    pdf[i] = e.pdf;
}

__global__ void k_closure_sample(const kz_lobe* __restrict__ lobes, const float* __restrict__ wi,
                                 const float* __restrict__ u, uint64_t n, float* wo, float* weight, float* pdf,
                                 uint8_t* flags) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const kz_lobe l = lobes[i];
    LobeSample s = lobe_sample(l, ld3(wi + 3 * i), u[3 * i], u[3 * i + 1], u[3 * i + 2]);
    wo[3 * i] = s.wo.x;
    wo[3 * i + 1] = s.wo.y;
    wo[3 * i + 2] = s.wo.z;
    weight[3 * i] = s.weight.x;
    weight[3 * i + 1] = s.weight.y;
    weight[3 * i + 2] = s.weight.z;
    pdf[i] = s.pdf;
    flags[i] = (uint8_t)((s.valid ? 1 : 0) | (s.delta ? 2 : 0));
}

}  // namespace

void launch_closure_eval(const kz_lobe* lobes, const float* wi, const float* wo, uint64_t n, int convention,
                         float* f, float* pdf, cudaStream_t st) {
    if (!n) return;
    k_closure_eval<<<grid_for(n, 128), 128, 0, st>>>(lobes, wi, wo, n, convention, f, pdf);
}
void launch_closure_sample(const kz_lobe* lobes, const float* wi, const float* u, uint64_t n, float* wo,
                           float* weight, float* pdf, uint8_t* flags, cudaStream_t st) {
    if (!n) return;
    k_closure_sample<<<grid_for(n, 128), 128, 0, st>>>(lobes, wi, u, n, wo, weight, pdf, flags);
}

}  // namespace kz
