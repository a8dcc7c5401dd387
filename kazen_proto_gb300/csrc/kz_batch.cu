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
    if (j < c->gen_count) batch_generate(jobs, n_jobs, dst, c, j);
}

// Shades path i of the wavefront (i >= n_in: no path); every thread of the
// block calls it (the block groups its paths by kind first).
template <bool kAttr>
__device__ __forceinline__ void batch_shade(const DevJob* __restrict__ jobs, PathSoA in, PathSoA out, ShadowSoA sq,
                                            DevCounters* ctr, uint32_t i, uint32_t n_in) {
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

template <bool kAttr>
__global__ void __launch_bounds__(256, KZ_SHADE_MIN_BLOCKS) k_shade_batch(const DevJob* __restrict__ jobs, PathSoA in, PathSoA out,
                                                     ShadowSoA sq, DevCounters* ctr) {
    batch_shade<kAttr>(jobs, in, out, sq, ctr, blockIdx.x * blockDim.x + threadIdx.x, ctr->n_active);
}

// ------------------------------------------------------------------ one persistent launch
// KZ_BATCH_PERSISTENT: the batched wavefront's whole loop (plan, generate,
// trace, shade, shadow, finish per iteration, until every job's paths are
// done) in one cooperative launch, the stages separated by grid-wide
// barriers. All blocks are resident (cooperative launch), so a barrier only
// waits for work in progress; every wait is still bounded.

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Wait limit of one grid barrier: far above any stage's duration.
constexpr uint64_t kGridWaitNs = 20ull * 1000000000ull;

// Sense-counting grid barrier over the counters' bar_count / bar_gen words.
// Returns false on every block once any block's wait ran out (the kernel
// then returns; status KZ_ERR_TIMEOUT).
__device__ __forceinline__ bool grid_barrier(DevCounters* c) {
    __shared__ uint32_t s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile uint32_t* gen = &c->bar_gen;
        volatile uint32_t* abort = &c->bar_abort;
        uint32_t ok = *abort == 0u;
        if (ok) {
            const uint32_t g = *gen;
            __threadfence();
            if (atomicAdd(&c->bar_count, 1u) == gridDim.x - 1) {
                c->bar_count = 0u;
                __threadfence();
                atomicAdd(&c->bar_gen, 1u);
            } else {
                const uint64_t t0 = global_ns();
                for (uint32_t k = 0; *gen == g; ++k) {
                    if (*abort) {
                        ok = 0u;
                        break;
                    }
                    __nanosleep(64);
                    if ((k & 255u) == 255u && global_ns() - t0 > kGridWaitNs) {
                        *abort = 1u;
                        set_status(&c->status, KZ_ERR_TIMEOUT);
                        ok = 0u;
                        break;
                    }
                }
            }
            __threadfence();
        }
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0u;
}

// The stages as separate functions (not inlined), so that each gets the
// kernel's registers to itself instead of sharing them with the loop state.
// The trace and shadow stages overlay one dynamic shared-memory region (the
// larger of the two loops' arrays), so the kernel holds no more shared memory
// than the closest-hit kernel alone and keeps the same L1 for BVH nodes.
extern __shared__ __align__(16) unsigned char kz_batch_smem[];
constexpr size_t kBatchSmem = sizeof(ClosestSmem) > sizeof(AnySmem) ? sizeof(ClosestSmem) : sizeof(AnySmem);

__device__ __noinline__ void stage_trace_paths(const DevJob* __restrict__ jobs, PathSoA p, DevCounters* ctr) {
    batch_trace_paths(*reinterpret_cast<ClosestSmem*>(kz_batch_smem), jobs, p, ctr);
}
__device__ __noinline__ void stage_trace_shadow(const DevJob* __restrict__ jobs, ShadowSoA sq, DevCounters* ctr) {
    batch_trace_shadow(*reinterpret_cast<AnySmem*>(kz_batch_smem), jobs, sq, ctr);
}
template <bool kAttr>
__device__ __noinline__ void stage_shade(const DevJob* __restrict__ jobs, PathSoA in, PathSoA out, ShadowSoA sq,
                                         DevCounters* ctr, uint32_t n_active) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n_active; base += stride)
        batch_shade<kAttr>(jobs, in, out, sq, ctr, base + threadIdx.x, n_active);
}

template <bool kAttr>
__global__ void __launch_bounds__(256, 4) k_batch_persistent(const DevJob* __restrict__ jobs, uint32_t n_jobs,
                                                          PathSoA A, PathSoA B, ShadowSoA sq, DevCounters* ctr,
                                                          uint32_t cap, uint32_t period) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t it = 0;; ++it) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            if (it) finish_iteration(ctr);
            plan_iteration(ctr, cap, it % period == 0);
        }
        if (!grid_barrier(ctr)) return;
        const volatile DevCounters* vc = ctr;
        const uint32_t n_active = vc->n_active, gen_count = vc->gen_count;
        if (n_active == 0 && vc->next_path >= vc->total) return;
        for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < gen_count; j += stride)
            batch_generate(jobs, n_jobs, A, ctr, j);
        if (!grid_barrier(ctr)) return;
        stage_trace_paths(jobs, A, ctr);
        if (!grid_barrier(ctr)) return;
        stage_shade<kAttr>(jobs, A, B, sq, ctr, n_active);
        if (!grid_barrier(ctr)) return;
        stage_trace_shadow(jobs, sq, ctr);
        if (!grid_barrier(ctr)) return;
        const PathSoA t = A;
        A = B;
        B = t;
    }
}

}  // namespace

void launch_generate_batch_dev(const DevJob* jobs, uint32_t n_jobs, PathSoA dst, DevCounters* ctr, uint32_t cap,
                               uint32_t block, cudaStream_t st) {
    if (!cap) return;
    k_generate_batch_dev<<<grid_for(cap, block), block, 0, st>>>(jobs, n_jobs, dst, ctr);
}
// Blocks per SM of the persistent batch kernel (0: it does not fit).
int batch_persistent_blocks_per_sm(bool textured) {
    int n = 0;
    if (textured) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch_persistent<true>, 256, kBatchSmem);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch_persistent<false>, 256, kBatchSmem);
    return n;
}

cudaError_t launch_batch_persistent(const DevJob* jobs, uint32_t n_jobs, PathSoA A, PathSoA B, ShadowSoA sq,
                                   DevCounters* ctr, uint32_t cap, uint32_t period, uint32_t blocks, bool textured,
                                   cudaStream_t st) {
    void* args[] = {(void*)&jobs, (void*)&n_jobs, (void*)&A, (void*)&B, (void*)&sq, (void*)&ctr, (void*)&cap,
                    (void*)&period};
    const void* f = textured ? (const void*)k_batch_persistent<true> : (const void*)k_batch_persistent<false>;
    return cudaLaunchCooperativeKernel(f, dim3(blocks), dim3(256), args, kBatchSmem, st);
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
