// kz_guide_tc.cu — one training step of the guiding network as one tcgen05
// kernel (sm_103a): forward, mixture loss, backward and weight gradients,
// with every contraction on the 5th-generation tensor cores and the weight
// gradients accumulated in tensor memory across the CTA's rows.
//
// A CTA of 256 threads owns tiles of 128 training rows; warps w and w + 4
// serve TMEM lanes 32 (w % 4) .. + 31, i.e. rows r = t % 128, and split every
// 64-column epilogue into halves (h = t / 128: columns 32h .. 32h + 31). Per
// tile:
//   X  = features (8-band sin/cos of the position, normal)   -> smem tile
//   Hl = ReLU(H(l-1) W_l^T + b_l), l = 1..3                  -> smem tiles
//   O  = H3 W4^T + b4 (40 outputs); dO = d(w * -log q)/dO     -> smem tile
//   dZ3 = (dO W4) * [H3 > 0], dZ2 = (dZ3 W3) * [H2 > 0],
//   dZ1 = (dZ2 W2) * [H1 > 0]                                 -> smem tiles
//   dW += [dZ1 | dZ2]^T [X | H1 | 1],  [dZ3 | dO]^T [H2 | H3 | 1]
// Each product is one tcgen05.mma chain issued by thread 0 (M = 128 rows);
// its FP32 result in tensor memory is read back by all eight warps
// (tcgen05.ld, 32 lanes x 32 columns each), which apply bias, ReLU or the
// ReLU mask and store the BF16 operand of the next product into shared
// memory. The mixture loss of a row is computed by its half-0 thread (the
// other half's output columns pass through shared memory). Every
// activation tile is a [128 rows][64] BF16 matrix in the 128-byte-swizzled
// layout (kz_tc.cuh): K-major for the forward and backward products, and,
// unchanged, the MN-major transpose for the weight-gradient products (rows
// are then K). The last layer has 48 columns (40 outputs and 8 zeros); the
// backward through it contracts 48 of dO's columns.
//
// BF16 rounding points are those of the warp-level kernels (and of the numpy
// restatement): features, weights, activations after ReLU, dO and the dZ;
// accumulation is FP32. The weight gradients of the CTA's rows stay in
// tensor memory (2 x 144 columns) until its last tile and are then added to
// the FP32 gradient with atomics; column 128 of each accumulator (the ones
// block) is the bias gradient. The 992-byte training records of the
// two-kernel path are never written.
//
// Every wait is bounded: a wait that runs out sets a flag, the CTA leaves
// its tile loop together, waits (bounded) for the products it issued, frees
// its tensor memory and records KZ_ERR_TIMEOUT in the status word.
#include <cuda_bf16.h>

#include "kz_guide.cuh"
#include "kz_internal.h"
#include "kz_tc.cuh"

namespace kz {
namespace {
using namespace tc;

constexpr int kT = 128;               // rows per tile = TMEM lanes
constexpr int kThreads = 256;         // two threads per row
constexpr uint32_t kTile = kT * 128;  // bytes of a [128][64] BF16 tile (16 KB)
constexpr uint32_t kWt = 64 * 128;    // bytes of a [64][64] BF16 weight tile (8 KB)
// shared-memory layout (from the 1024-byte-aligned base)
constexpr uint32_t oX = 0 * kTile, oH1 = 1 * kTile, oOne0 = 2 * kTile;   // X | H1 | ones
constexpr uint32_t oH2 = 3 * kTile, oH3 = 4 * kTile, oOne1 = 5 * kTile;  // H2 | H3 | ones
constexpr uint32_t oD1 = 6 * kTile, oD2 = 7 * kTile;                    // dZ1 | dZ2
constexpr uint32_t oD3 = 8 * kTile, oDO = 9 * kTile;                    // dZ3 | dO
constexpr uint32_t oW1 = 10 * kTile, oW2 = oW1 + kWt, oW3 = oW2 + kWt, oW4 = oW3 + kWt;  // [out][in]
constexpr uint32_t oW2T = oW4 + kWt, oW3T = oW2T + kWt, oW4T = oW3T + kWt;             // [in][out]
constexpr uint32_t oBar = oW4T + kWt;
constexpr size_t kSmemTrain = (size_t)oBar + 64 + 1024;  // barriers, TMEM slot, flag; alignment slack
constexpr uint32_t kTmemCols = 512;  // dW pair 0 at column 0, pair 1 at 256 (144 each), scratch at 160 (64)
constexpr uint32_t kScratch = 160;
constexpr uint32_t kIdF64 = idesc_bf16(128, 64, false, false);
constexpr uint32_t kIdF48 = idesc_bf16(128, 48, false, false);
constexpr uint32_t kIdW = idesc_bf16(128, 144, true, true);
static_assert(kSmemTrain <= 227 * 1024, "shared memory of the fused training kernel");

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

// store 32 floats as half `h` (chunks 4h .. 4h + 3) of the BF16 line of row `r`
__device__ __forceinline__ void store_half(unsigned char* tile, uint32_t r, uint32_t h, const float* v) {
#pragma unroll
    for (int cc = 0; cc < 4; ++cc) {
        const int c = 4 * (int)h + cc;
        uint4 q;
        q.x = pack2(v[8 * cc + 0], v[8 * cc + 1]);
        q.y = pack2(v[8 * cc + 2], v[8 * cc + 3]);
        q.z = pack2(v[8 * cc + 4], v[8 * cc + 5]);
        q.w = pack2(v[8 * cc + 6], v[8 * cc + 7]);
        *reinterpret_cast<uint4*>(tile + sw128(r, c)) = q;
    }
}

// the positive-part mask of half `h` of a stored BF16 line: bit k set where
// element 32h + k > 0
__device__ __forceinline__ uint32_t positive_mask_half(const unsigned char* tile, uint32_t r, uint32_t h) {
    uint32_t m = 0;
#pragma unroll
    for (int cc = 0; cc < 4; ++cc) {
        const uint4 q = *reinterpret_cast<const uint4*>(tile + sw128(r, 4 * h + cc));
        const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            // BF16 > 0: sign bit clear and not +0
            if (!(w[e] & 0x8000u) && (w[e] & 0x7FFFu)) m |= 1u << (8 * cc + 2 * e);
            if (!(w[e] & 0x80000000u) && (w[e] & 0x7FFF0000u)) m |= 1u << (8 * cc + 2 * e + 1);
        }
    }
    return m;
}

// D = A (tile at `a`, K-major, K = 16 * ksteps) x B^T (tile at `b`, K-major)
__device__ __forceinline__ void mma_chain(uint32_t d, uint32_t a, uint32_t b, int ksteps, uint32_t idesc) {
    for (int ks = 0; ks < ksteps; ++ks)
        umma_bf16(d, desc_sw128(a + 32u * ks, 16, 1024), desc_sw128(b + 32u * ks, 16, 1024), idesc, ks > 0);
}

__global__ void __launch_bounds__(kThreads, 1) k_guide_train_tc(const float4* __restrict__ samples, uint32_t count,
                                                                 uint32_t n, uint32_t stride, uint32_t offset,
                                                                 GuideDev gd, float inv_n, float wcap,
                                                                 float* __restrict__ grad, float* __restrict__ loss,
                                                                 uint32_t* __restrict__ status) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned char* sm =
        reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    const uint32_t base = smem_u32(sm);
    uint64_t* bars = reinterpret_cast<uint64_t*>(sm + oBar);  // [0] products, [1] weight gradients, [2] drain
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 3);
    volatile uint32_t* failed = reinterpret_cast<volatile uint32_t*>(bars + 4);
    const uint32_t bar_mma = smem_u32(&bars[0]), bar_wg = smem_u32(&bars[1]), bar_end = smem_u32(&bars[2]);
    const int t = threadIdx.x, warp = t >> 5;
    const uint32_t row = (uint32_t)t & (kT - 1);  // tile row = TMEM lane
    const uint32_t half = (uint32_t)t >> 7;       // columns 32 * half .. + 31 of each product
    const uint32_t tiles = (n + kT - 1) / kT;
    if (blockIdx.x >= tiles) return;  // uniform over the CTA

    // ---- weights, their transposes and the ones tiles, once per CTA
    const __nv_bfloat16* Wg = gd.wbf;
    const int offs[4] = {kOffW1, kOffW2, kOffW3, kOffW4};
    const uint32_t wt[4] = {oW1, oW2, oW3, oW4};
    for (int l = 0; l < 4; ++l)
        for (int i = t; i < 64 * 8; i += kThreads) {
            const int line = i >> 3, c = i & 7;
            uint4 q = make_uint4(0u, 0u, 0u, 0u);
            if (l < 3 || line < 40) q = *reinterpret_cast<const uint4*>(Wg + offs[l] + line * 64 + 8 * c);
            *reinterpret_cast<uint4*>(sm + wt[l] + sw128(line, c)) = q;
        }
    const uint32_t wtt[3] = {oW2T, oW3T, oW4T};
    for (int l = 1; l < 4; ++l)
        for (int i = t; i < 64 * 64; i += kThreads) {
            const int in = i >> 6, o = i & 63;  // line `in` of W_l^T holds W_l[o][in] over o
            __nv_bfloat16 v = __float2bfloat16_rn(0.f);
            if (l < 3 || o < 40) v = Wg[offs[l] + o * 64 + in];
            *reinterpret_cast<__nv_bfloat16*>(sm + wtt[l - 1] + sw128(in, o >> 3) + 2 * (o & 7)) = v;
        }
    const uint32_t one2 = pack2(1.f, 1.f);
    for (uint32_t i = t; i < kTile / 4; i += kThreads) {
        reinterpret_cast<uint32_t*>(sm + oOne0)[i] = one2;
        reinterpret_cast<uint32_t*>(sm + oOne1)[i] = one2;
    }
    if (t == 0) {
        mbar_init(bar_mma, 1);
        mbar_init(bar_wg, 1);
        mbar_init(bar_end, 1);
        *failed = 0u;
        mbar_init_fence();
    }
    fence_async_smem();
    if (warp == 0) tmem_alloc(tmem_slot, kTmemCols);
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = *tmem_slot;
    const uint32_t lanes = (uint32_t)(32 * (warp & 3)) << 16;  // this warp's TMEM lane quadrant
    const uint32_t S = tmem + lanes + kScratch + 32u * half;  // this thread's 32 scratch columns
    float* raw_hi = reinterpret_cast<float*>(sm + oD1);       // [128][8] outputs 32..39 (dZ1's tile is free then)

    const f3 ext = mk(1.f / gd.box_inv.x, 1.f / gd.box_inv.y, 1.f / gd.box_inv.z);
    const float* Wf = gd.wf;
    uint32_t ph_mma = 0, ph_wg = 0;
    bool any_wg = false;
    float loss_acc = 0.f;

    // all threads wait for a phase; a wait that runs out marks the CTA failed
    auto wait_phase = [&](uint32_t bar, uint32_t& ph) {
        if (!mbar_wait(bar, ph)) *failed = 1u;
        ph ^= 1u;
        fence_after_sync();
    };
    // shared-memory operands written, accumulator reads done: next product
    auto stage_sync = [&]() {
        fence_async_smem();
        fence_before_sync();
        __syncthreads();
        fence_after_sync();
        return *failed == 0u;
    };
    // one product into the scratch accumulator, then this thread's 32 columns
    // (16 for half 1 of the 48-column product; the rest zero)
    auto product = [&](uint32_t a, uint32_t b, int ksteps, uint32_t idesc, float (&v)[32], bool narrow) {
        if (t == 0) {
            mma_chain(tmem + kScratch, base + a, base + b, ksteps, idesc);
            umma_commit(bar_mma);
        }
        wait_phase(bar_mma, ph_mma);
        if (narrow && half) {
            tmem_ld16(S, v);
#pragma unroll
            for (int k = 16; k < 32; ++k) v[k] = 0.f;
        } else {
            tmem_ld32(S, v);
        }
    };

    for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const uint32_t r = tile * kT + row;
        const bool valid = r < n;
        f3 p = mk(0.5f, 0.5f, 0.5f), nn = mk(0.f, 1.f, 0.f), dir = mk(0.f, 1.f, 0.f);
        float w = 0.f;
        if (valid) {
            const size_t si = (size_t)(((uint64_t)(r + offset) * stride) % count);
            const float4 a = samples[3 * si], b = samples[3 * si + 1];
            p = mk(a.x, a.y, a.z);
            nn = mk(b.x, b.y, b.z);
            if (half == 0) {
                const float4 c = samples[3 * si + 2];
                dir = mk(c.x, c.y, c.z);
                w = fminf(a.w * inv_n, wcap);
            }
        }
        // the previous tile's weight-gradient products read the tiles rewritten below
        if (any_wg) wait_phase(bar_wg, ph_wg);
        float v[32];
        // ---- features: half 0 the x and y bands (columns 0..31), half 1 the
        // z bands, the normal and the zero padding (32..63)
        if (half == 0) {
#pragma unroll
            for (int a = 0; a < 2; ++a)
#pragma unroll
                for (int b = 0; b < 8; ++b)
                    band_sincos(comp(p, a), b, gd.band_scale, v[16 * a + 2 * b], v[16 * a + 2 * b + 1]);
        } else {
#pragma unroll
            for (int b = 0; b < 8; ++b) band_sincos(p.z, b, gd.band_scale, v[2 * b], v[2 * b + 1]);
            v[16] = nn.x;
            v[17] = nn.y;
            v[18] = nn.z;
#pragma unroll
            for (int k = 19; k < 32; ++k) v[k] = 0.f;
        }
        store_half(sm + oX, row, half, v);
        if (!stage_sync()) break;
        // ---- hidden layers
        const uint32_t ain[3] = {oX, oH1, oH2}, aout[3] = {oH1, oH2, oH3}, wl[3] = {oW1, oW2, oW3};
        const int boff[3] = {kOffB1, kOffB2, kOffB3};
        bool ok = true;
        for (int l = 0; l < 3 && ok; ++l) {
            product(ain[l], wl[l], 4, kIdF64, v, false);
            const float* bias = Wf + boff[l] + 32 * half;
#pragma unroll
            for (int k = 0; k < 32; ++k) v[k] = fmaxf(v[k] + __ldg(bias + k), 0.f);
            store_half(sm + aout[l], row, half, v);
            ok = stage_sync();
        }
        if (!ok) break;
        // ---- outputs, loss and its gradient (the half-0 thread of the row)
        product(oH3, oW4, 4, kIdF48, v, true);
        if (half) {
#pragma unroll
            for (int k = 0; k < 8; ++k) raw_hi[row * 8 + k] = v[k];  // outputs 32..39
        }
        __syncthreads();
        if (half == 0) {
            float raw[kGuideOut], g[kGuideOut];
#pragma unroll
            for (int k = 0; k < 32; ++k) raw[k] = v[k] + __ldg(Wf + kOffB4 + k);
#pragma unroll
            for (int k = 0; k < 8; ++k) raw[32 + k] = raw_hi[row * 8 + k] + __ldg(Wf + kOffB4 + 32 + k);
            if (valid) {
                loss_acc += w * mixture_nll_grad(raw, dir, w, g, p, ext);
            } else {
#pragma unroll
                for (int k = 0; k < kGuideOut; ++k) g[k] = 0.f;
            }
            float lo[32], hi[32];
#pragma unroll
            for (int k = 0; k < 32; ++k) lo[k] = g[k];
#pragma unroll
            for (int k = 0; k < 8; ++k) hi[k] = g[32 + k];
#pragma unroll
            for (int k = 8; k < 32; ++k) hi[k] = 0.f;
            store_half(sm + oDO, row, 0, lo);
            store_half(sm + oDO, row, 1, hi);
        }
        if (!stage_sync()) break;
        // ---- backward: dZ3, dZ2, dZ1
        const uint32_t bin[3] = {oDO, oD3, oD2}, bw[3] = {oW4T, oW3T, oW2T}, hmask[3] = {oH3, oH2, oH1},
                       bout[3] = {oD3, oD2, oD1};
        const int ksteps[3] = {3, 4, 4};  // dO has 48 columns
        for (int l = 0; l < 3 && ok; ++l) {
            product(bin[l], bw[l], ksteps[l], kIdF64, v, false);
            const uint32_t m = positive_mask_half(sm + hmask[l], row, half);
#pragma unroll
            for (int k = 0; k < 32; ++k) v[k] = ((m >> k) & 1u) ? v[k] : 0.f;
            store_half(sm + bout[l], row, half, v);
            ok = stage_sync();
        }
        if (!ok) break;
        // ---- weight gradients of this tile, accumulated in tensor memory
        if (t == 0) {
            for (int k = 0; k < kT / 16; ++k) {
                const uint32_t koff = 2048u * k;  // 16 rows (K lines) of 128 bytes
                const uint32_t acc = (any_wg || k > 0) ? 1u : 0u;
                umma_bf16(tmem, desc_sw128(base + oD1 + koff, kTile, 1024), desc_sw128(base + oX + koff, kTile, 1024),
                          kIdW, acc);
                umma_bf16(tmem + 256, desc_sw128(base + oD3 + koff, kTile, 1024),
                          desc_sw128(base + oH2 + koff, kTile, 1024), kIdW, acc);
            }
            umma_commit(bar_wg);
        }
        any_wg = true;
    }
    // ---- drain: every product issued by thread 0 is done before the
    // accumulators are read and the tensor memory is freed
    if (t == 0) umma_commit(bar_end);
    if (!mbar_wait(bar_end, 0)) *failed = 1u;
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const bool ok_all = *failed == 0u;
    if (ok_all && any_wg) {
        const uint32_t coff = row < 64 ? 0u : 64u;  // the diagonal block's columns
#pragma unroll
        for (int pair = 0; pair < 2; ++pair) {
            const uint32_t dbase = tmem + lanes + (pair ? 256u : 0u);
            const int layer = 2 * pair + (row < 64 ? 0 : 1);
            const int o = (int)(row & 63);
            const int outs = layer == 3 ? 40 : 64;
            const int woff = layer == 0 ? kOffW1 : layer == 1 ? kOffW2 : layer == 2 ? kOffW3 : kOffW4;
            const int bo = layer == 0 ? kOffB1 : layer == 1 ? kOffB2 : layer == 2 ? kOffB3 : kOffB4;
            float d[32];
            tmem_ld32(dbase + coff + 32 * half, d);
            if (o < outs)
#pragma unroll
                for (int k = 0; k < 32; ++k)
                    if (d[k] != 0.f) atomicAdd(grad + woff + o * 64 + 32 * half + k, d[k]);
            const float db = tmem_ld1(dbase + 128);
            if (half == 0 && o < outs && db != 0.f) atomicAdd(grad + bo + o, db);
        }
    }
    if (!ok_all && t == 0) atomicExch(status, (uint32_t)KZ_ERR_TIMEOUT);
    // the loss of the CTA's rows (the half-0 threads hold it)
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) loss_acc += __shfl_xor_sync(0xffffffffu, loss_acc, s);
    if ((t & 31) == 0 && loss_acc != 0.f) atomicAdd(loss, loss_acc);
    fence_before_sync();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, kTmemCols);
}

int sm_count_train() {
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

cudaError_t guide_train_tc_setup() {
    return cudaFuncSetAttribute(k_guide_train_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemTrain);
}

cudaError_t launch_guide_train_tc(const float4* samples, uint32_t count, uint32_t n, uint32_t stride,
                                  uint32_t offset, float wscale, float wcap, const GuideDev& gd, float* grad,
                                  float* loss, uint32_t* status, cudaStream_t st) {
    if (!n || !count) return cudaSuccess;
    const uint32_t tiles = (n + kT - 1) / kT;
    const uint32_t grid = min(tiles, (uint32_t)sm_count_train());
    k_guide_train_tc<<<grid, kThreads, kSmemTrain, st>>>(samples, count, n, stride, offset, gd, wscale, wcap, grad,
                                                         loss, status);
    return cudaGetLastError();
}

}  // namespace kz
