// kz_mlp_tc.cu — the guiding network's weight gradients on the 5th-generation
// tensor cores (sm_103a) from training records: TMA-staged BF16 operands,
// tcgen05.mma with FP32 accumulators in tensor memory, tcgen05.ld epilogue.
// (The default training step runs forward, backward and these products in
// one kernel, kz_guide_tc.cu; this kernel serves the split path whose
// forward/backward kernel writes the records.)
//
// Per training step, for the four layers l:
//   dW_l[o][i] = sum_r dZ_l[r][o] * A_{l-1}[r][i],   db_l[o] = sum_r dZ_l[r][o]
// over up to 2^18 rows r. The rows are the records k_guide_train_fb writes,
// 496 BF16 each: X H1 H2 H3 dZ1 dZ2 dZ3 (64 columns each) and dO (48). In the
// product D = A * B^T of tcgen05 (A: M x K, B: N x K) the row index r is K,
// and both operands are read with their M / N index contiguous in memory
// (MN-major): a TMA box of 64 columns x 32 rows with the 128-byte swizzle is
// the canonical MN-major SWIZZLE_128B layout (one 128-byte line of 64 MN
// elements per K index, 8-line swizzle atoms; kz_tc.cuh).
//
// Two M = 128 products per 16-row K step:
//   D0 = [dZ1 | dZ2]^T x [X  | H1 | 1],   D1 = [dZ3 | dO]^T x [H2 | H3 | 1]
// with N = 144: the third N block is a constant tile of ones, so column 128 of
// each accumulator is the bias gradient. dW1 = D0[0:64, 0:64],
// dW2 = D0[64:128, 64:128], dW3 = D1[0:64, 0:64], dW4 = D1[64:104, 64:128].
// (The off-diagonal blocks are computed and dropped: the kernel is bound by
// the 992 bytes per row it reads, not by the tensor pipe.)
//
// One CTA per SM streams a contiguous range of 32-row chunks through a
// five-stage shared-memory ring: thread 0 issues the TMA loads (eight 4 KB
// boxes per chunk, one mbarrier transaction count) up to four chunks ahead
// and the MMAs, and tcgen05.commit releases a stage when its MMAs have read
// it. The four warps then read their 32 TMEM lanes and add the partial
// gradient of the CTA into the FP32 gradient with atomics.
//
// Every wait is bounded: a wait that runs out records KZ_ERR_TIMEOUT in the
// status word, the kernel waits (bounded again) for the copies and products
// it has issued, frees its tensor memory and returns.
#include <cuda.h>
#include <cuda_bf16.h>

#include "kz_guide.cuh"
#include "kz_internal.h"
#include "kz_tc.cuh"

namespace kz {
namespace {
using namespace tc;

constexpr int kRecCols = 496;              // BF16 per training row
constexpr int kRows = 32;                  // K rows per chunk (one TMA box high)
constexpr uint32_t kBox = 64 * kRows * 2;  // bytes of one 64-column x 32-row BF16 box
// stage layout (bytes from the stage base; every box 1024-byte aligned)
constexpr uint32_t kA0 = 0 * kBox, kB0 = 2 * kBox, kA1 = 5 * kBox, kB1 = 7 * kBox;
constexpr uint32_t kStage = 10 * kBox;    // 40 KB: A0 (2 boxes) B0 (2 + ones) A1 (2) B1 (2 + ones)
constexpr int kStages = 5;                // up to four stages of loads in flight per SM
constexpr uint32_t kTxBytes = 8 * kBox;   // loaded by TMA per stage (the ones tiles are written once)
constexpr uint32_t kTmemCols = 512;       // D0 at column 0, D1 at column 256 (144 used each)
constexpr uint32_t kN = 144, kM = 128;
constexpr size_t kSmemTc = (size_t)kStages * kStage + 1024 /*alignment*/ + 256 /*barriers*/;
constexpr int kThreads = 128;
constexpr uint32_t kIdesc = idesc_bf16(kM, kN, true, true);  // both operands MN-major
static_assert(kSmemTc <= 227 * 1024, "shared memory of the weight-gradient kernel");

__global__ void __launch_bounds__(kThreads, 1) k_guide_wgrad_tc(const __grid_constant__ CUtensorMap rec_map,
                                                                 uint32_t n_chunks, uint32_t chunks_per_cta,
                                                                 float* __restrict__ grad,
                                                                 uint32_t* __restrict__ status) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned char* smem =
        reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kStages * kStage);  // full[S], empty[S], done, flag
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * kStages + 2);
    volatile uint64_t* flag = &bars[2 * kStages + 1];
    const uint32_t base = smem_u32(smem);
    const uint32_t full0 = smem_u32(&bars[0]), empty0 = smem_u32(&bars[kStages]),
                   done = smem_u32(&bars[2 * kStages]);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t c0 = blockIdx.x * chunks_per_cta;
    const uint32_t nloc = c0 < n_chunks ? min(chunks_per_cta, n_chunks - c0) : 0u;
    if (nloc == 0) return;  // uniform over the CTA: nothing allocated yet

    // the constant tiles of ones (B's third N block) in every stage
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
        mbar_init_fence();
    }
    fence_async_smem();  // the ones tiles become visible to the tensor core
    if (warp == 0) tmem_alloc(tmem_slot, kTmemCols);
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = *tmem_slot;

    bool ok = true;
    if (threadIdx.x == 0) {
        const int col_a0 = 256, col_b0 = 0, col_a1 = 384, col_b1 = 128;  // dZ1, X, dZ3, H2
        uint32_t issued = 0, consumed = 0;                                // chunks loaded / multiplied
        // iteration `it` loads chunk `it` (while there is one) and then
        // multiplies the oldest loaded chunk once the loads run kStages - 1
        // chunks ahead, or once they are all issued; ends when every chunk
        // has been multiplied
        for (uint32_t it = 0; consumed < nloc && ok; ++it) {
            if (it < nloc) {  // load chunk `it` into stage it % kStages
                const uint32_t s = it % kStages;
                if (it >= kStages) ok = mbar_wait(empty0 + 8 * s, ((it / kStages) - 1) & 1);
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
            if ((it >= kStages - 1 || it >= nloc) && consumed < issued) {  // multiply the oldest loaded chunk
                const uint32_t j = consumed, s = j % kStages;
                ok = mbar_wait(full0 + 8 * s, (j / kStages) & 1);
                if (!ok) break;
                fence_after_sync();
                const uint32_t st = base + s * kStage;
#pragma unroll
                for (int ks = 0; ks < kRows / 16; ++ks) {
                    const uint32_t acc = (j > 0 || ks > 0) ? 1u : 0u;
                    const uint32_t koff = ks * 16 * 128;  // 16 K lines of 128 bytes
                    umma_bf16(tmem, desc_sw128(st + kA0 + koff, kBox, 1024), desc_sw128(st + kB0 + koff, kBox, 1024),
                              kIdesc, acc);
                    umma_bf16(tmem + 256, desc_sw128(st + kA1 + koff, kBox, 1024),
                              desc_sw128(st + kB1 + koff, kBox, 1024), kIdesc, acc);
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
            for (uint32_t j = consumed; j < issued; ++j) mbar_wait(full0 + 8 * (j % kStages), (j / kStages) & 1);
            umma_commit(done);
            mbar_wait(done, 0);
        }
        *flag = ok ? 1ull : 0ull;  // tell the other warps
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    ok = *flag != 0ull;

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
    fence_before_sync();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, kTmemCols);
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
