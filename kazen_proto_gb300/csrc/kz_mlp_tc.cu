// kz_mlp_tc.cu — the guiding network's weight gradients on the 5th-generation
// tensor cores (sm_103a): TMA-staged BF16 operands, tcgen05.mma with FP32
// accumulators in tensor memory, tcgen05.ld epilogue.
//
// Per training step, for the four layers l:
//   dW_l[o][i] = sum_r dZ_l[r][o] * A_{l-1}[r][i],   db_l[o] = sum_r dZ_l[r][o]
// over up to 2^18 rows r. The rows are the records k_guide_train_fb writes,
// 496 BF16 each: X H1 H2 H3 dZ1 dZ2 dZ3 (64 columns each) and dO (48). In the
// product D = A * B^T of tcgen05 (A: M x K, B: N x K) the row index r is K,
// and both operands are read with their M / N index contiguous in memory
// (MN-major): a TMA box of 64 columns x 64 rows with the 128-byte swizzle is
// exactly the canonical MN-major SWIZZLE_128B layout (one 128-byte line of 64
// MN elements per K index, 8-line swizzle atoms).
//
// Two M = 128 products per 16-row K step:
//   D0 = [dZ1 | dZ2]^T x [X  | H1 | 1],   D1 = [dZ3 | dO]^T x [H2 | H3 | 1]
// with N = 144: the third N block is a constant tile of ones, so column 128 of
// each accumulator is the bias gradient. dW1 = D0[0:64, 0:64],
// dW2 = D0[64:128, 64:128], dW3 = D1[0:64, 0:64], dW4 = D1[64:104, 64:128].
// (The off-diagonal blocks are computed and dropped: the kernel is bound by
// the 992 bytes per row it reads, not by the tensor pipe.)
//
// One CTA per SM streams a contiguous range of 64-row chunks through a
// two-stage shared-memory ring: thread 0 issues the TMA loads (eight 8 KB
// boxes per chunk, one mbarrier transaction count) and the MMAs, and
// tcgen05.commit releases a stage when its MMAs have read it. The four warps
// then read their 32 TMEM lanes and add the partial gradient of the CTA into
// the FP32 gradient with atomics.
//
// Every wait is bounded: a wait that runs out records KZ_ERR_TIMEOUT in the
// status word, the kernel waits (bounded again) for the copies and products
// it has issued, frees its tensor memory and returns.
#include <cuda.h>
#include <cuda_bf16.h>

#include "kz_guide.cuh"
#include "kz_internal.h"

namespace kz {
namespace {

constexpr int kRecCols = 496;  // BF16 per training row
constexpr int kRows = 64;      // K rows per chunk (one TMA box high)
constexpr uint32_t kBox = 64 * 64 * 2;  // bytes of one 64 x 64 BF16 box
// stage layout (bytes from the stage base; every box 1024-byte aligned)
constexpr uint32_t kA0 = 0 * kBox, kB0 = 2 * kBox, kA1 = 5 * kBox, kB1 = 7 * kBox;
constexpr uint32_t kStage = 10 * kBox;  // 80 KB: A0 (2 boxes) B0 (2 + ones) A1 (2) B1 (2 + ones)
constexpr int kStages = 2;
constexpr uint32_t kTxBytes = 8 * kBox;  // loaded by TMA per stage (the ones tiles are written once)
constexpr uint32_t kTmemCols = 512;      // D0 at column 0, D1 at column 256 (144 used each)
constexpr uint32_t kN = 144, kM = 128;
constexpr size_t kSmemTc = (size_t)kStages * kStage + 1024 /*alignment*/ + 256 /*barriers*/;
constexpr int kThreads = 128;
constexpr uint32_t kWaitLimit = 1u << 22;  // try_wait rounds before a wait is declared stuck

// Instruction descriptor of tcgen05.mma .kind::f16: FP32 accumulator (bits
// 4-5 = 1), BF16 A and B (bits 7-9, 10-12 = 1), A and B MN-major (bits 15,
// 16), N >> 3 at bits 17-22, M >> 4 at bits 24-28.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | (1u << 15) | (1u << 16) | ((kN >> 3) << 17) |
                            ((kM >> 4) << 24);

// Shared-memory matrix descriptor: start address >> 4 (bits 0-13), leading
// byte offset >> 4 (16-29: the distance between 64-element MN blocks),
// stride byte offset >> 4 (32-45: the distance between 8-line K groups),
// fixed 0b001 at bits 46-48, swizzle mode 2 = 128-byte (bits 61-63).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46) | (2ull << 61);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.b32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait on one phase of an mbarrier; false when it ran out.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (uint32_t k = 0; k < kWaitLimit; ++k)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
        "[%4];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void umma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

// 32 consecutive accumulator columns of this warp's 32 TMEM lanes.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int k = 0; k < 32; ++k) v[k] = __uint_as_float(r[k]);
}
__device__ __forceinline__ float tmem_ld1(uint32_t taddr) {
    uint32_t r;
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x1.b32 {%0}, [%1];" : "=r"(r) : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    return __uint_as_float(r);
}

__global__ void __launch_bounds__(kThreads, 1) k_guide_wgrad_tc(const __grid_constant__ CUtensorMap rec_map,
                                                                 uint32_t n_chunks, uint32_t chunks_per_cta,
                                                                 float* __restrict__ grad,
                                                                 uint32_t* __restrict__ status) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned char* smem =
        reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kStages * kStage);  // full[2], empty[2], done
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 8);
    const uint32_t base = smem_u32(smem);
    const uint32_t full0 = smem_u32(&bars[0]), empty0 = smem_u32(&bars[2]), done = smem_u32(&bars[4]);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t c0 = blockIdx.x * chunks_per_cta;
    const uint32_t nloc = c0 < n_chunks ? min(chunks_per_cta, n_chunks - c0) : 0u;
    if (nloc == 0) return;  // uniform over the CTA: nothing allocated yet

    // the constant tiles of ones (B's third N block) in both stages
    const __nv_bfloat162 one2 = __floats2bfloat162_rn(1.f, 1.f);
    for (int s = 0; s < kStages; ++s)
        for (uint32_t i = threadIdx.x; i < kBox / 4; i += kThreads) {
            reinterpret_cast<__nv_bfloat162*>(smem + s * kStage + kB0 + 2 * kBox)[i] = one2;
            reinterpret_cast<__nv_bfloat162*>(smem + s * kStage + kB1 + 2 * kBox)[i] = one2;
        }
    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, 1);
        }
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // generic-proxy writes (the ones tiles) become visible to the tensor core
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    bool ok = true;
    if (threadIdx.x == 0) {
        const int col_a0 = 256, col_b0 = 0, col_a1 = 384, col_b1 = 128;  // dZ1, X, dZ3, H2
        uint32_t issued = 0, consumed = 0;                                // chunks loaded / multiplied
        for (uint32_t it = 0; it <= nloc && ok; ++it) {
            if (it < nloc) {  // load chunk `it` into stage it % 2
                const uint32_t s = it & 1;
                if (it >= kStages) ok = mbar_wait(empty0 + 8 * s, ((it >> 1) - 1) & 1);
                if (!ok) break;
                const uint32_t st = base + s * kStage, bar = full0 + 8 * s;
                const int y = (int)((c0 + it) * kRows);
                mbar_expect_tx(bar, kTxBytes);
                tma_load_2d(st + kA0, &rec_map, col_a0, y, bar);
                tma_load_2d(st + kA0 + kBox, &rec_map, col_a0 + 64, y, bar);
                tma_load_2d(st + kB0, &rec_map, col_b0, y, bar);
                tma_load_2d(st + kB0 + kBox, &rec_map, col_b0 + 64, y, bar);
                tma_load_2d(st + kA1, &rec_map, col_a1, y, bar);
                tma_load_2d(st + kA1 + kBox, &rec_map, col_a1 + 64, y, bar);  // dO and 16 zero-filled columns
                tma_load_2d(st + kB1, &rec_map, col_b1, y, bar);
                tma_load_2d(st + kB1 + kBox, &rec_map, col_b1 + 64, y, bar);
                issued = it + 1;
            }
            if (it >= 1) {  // multiply chunk it - 1
                const uint32_t j = it - 1, s = j & 1;
                ok = mbar_wait(full0 + 8 * s, (j >> 1) & 1);
                if (!ok) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t st = base + s * kStage;
#pragma unroll
                for (int ks = 0; ks < kRows / 16; ++ks) {
                    const uint32_t acc = (j > 0 || ks > 0) ? 1u : 0u;
                    const uint32_t koff = ks * 16 * 128;  // 16 K lines of 128 bytes
                    umma_bf16(tmem, smem_desc(st + kA0 + koff, kBox, 1024), smem_desc(st + kB0 + koff, kBox, 1024),
                              acc);
                    umma_bf16(tmem + 256, smem_desc(st + kA1 + koff, kBox, 1024),
                              smem_desc(st + kB1 + koff, kBox, 1024), acc);
                }
                umma_commit(empty0 + 8 * s);
                consumed = j + 1;
            }
        }
        if (ok) {
            umma_commit(done);
            ok = mbar_wait(done, 0);
        }
        if (!ok) {
            atomicExch(status, (uint32_t)KZ_ERR_TIMEOUT);
            // let the copies and products already issued finish before the
            // shared and tensor memory they use is released (bounded)
            for (uint32_t j = consumed; j < issued; ++j) mbar_wait(full0 + 8 * (j & 1), (j >> 1) & 1);
            umma_commit(done);
            mbar_wait(done, 0);
        }
        bars[5] = ok ? 1ull : 0ull;  // tell the other warps
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    ok = bars[5] != 0ull;

    if (ok) {
        // warp w reads TMEM lanes 32w..32w+31 = accumulator rows
        const uint32_t row = 32 * warp + lane;  // M index of this thread
        const uint32_t lane_addr = tmem + ((uint32_t)(32 * warp) << 16);
        const uint32_t coff = row < 64 ? 0u : 64u;  // the diagonal block's columns
#pragma unroll
        for (int pair = 0; pair < 2; ++pair) {
            const uint32_t dbase = lane_addr + (pair ? 256u : 0u);
            const int layer = 2 * pair + (row < 64 ? 0 : 1);
            const int o = (int)(row & 63);
            const int outs = layer == 3 ? 40 : 64;
            const int woff = layer == 0 ? kOffW1 : layer == 1 ? kOffW2 : layer == 2 ? kOffW3 : kOffW4;
            const int boff = layer == 0 ? kOffB1 : layer == 1 ? kOffB2 : layer == 2 ? kOffB3 : kOffB4;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                float v[32];
                tmem_ld32(dbase + coff + 32 * h, v);
                if (o < outs)
#pragma unroll
                    for (int k = 0; k < 32; ++k)
                        if (v[k] != 0.f) atomicAdd(grad + woff + o * 64 + 32 * h + k, v[k]);
            }
            const float db = tmem_ld1(dbase + 128);
            if (o < outs && db != 0.f) atomicAdd(grad + boff + o, db);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled() {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    return fn;
}

int sm_count_tc() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

}  // namespace

cudaError_t guide_wgrad_tc_setup() {
    return cudaFuncSetAttribute(k_guide_wgrad_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemTc);
}

cudaError_t launch_guide_wgrad_tc(const __nv_bfloat16* rec, uint32_t n, float* grad, uint32_t* status,
                                  cudaStream_t st) {
    if (!n) return cudaSuccess;
    EncodeTiledFn enc = encode_tiled();
    if (!enc) return cudaErrorNotSupported;
    // the records as a 2-D BF16 tensor: 496 columns (contiguous) x n rows of 992 bytes
    CUtensorMap map;
    const cuuint64_t dims[2] = {(cuuint64_t)kRecCols, (cuuint64_t)n};
    const cuuint64_t strides[1] = {(cuuint64_t)kRecCols * 2};
    const cuuint32_t box[2] = {64, (cuuint32_t)kRows};
    const cuuint32_t estr[2] = {1, 1};
    if (enc(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<__nv_bfloat16*>(rec), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return cudaErrorInvalidValue;
    const uint32_t n_chunks = (n + kRows - 1) / kRows;
    const uint32_t ctas_max = (uint32_t)sm_count_tc();
    const uint32_t per = (n_chunks + ctas_max - 1) / ctas_max;
    const uint32_t ctas = (n_chunks + per - 1) / per;
    k_guide_wgrad_tc<<<ctas, kThreads, kSmemTc, st>>>(map, n_chunks, per, grad, status);
    return cudaGetLastError();
}

}  // namespace kz
