// kz_mlp.cu — the guiding network's kernels (sm_103a): fused BF16
// tensor-core inference, fused training forward + mixture loss + backward
// (data), split-K weight gradients, and Adam.
//
// Every layer is a warp-level product on 16-row tiles with
// mma.sync.m16n8k16 (BF16 operands, FP32 accumulation). Weights live in
// shared memory in [out][in] order (which is the column-major B operand of
// X * W^T) and, for the backward pass, also transposed. The accumulator
// fragment of one layer is, element for element, the A fragment of the next
// (rows g and g+8, columns 2t..2t+1 and 2t+8..2t+9 of each 16-column block),
// so activations never leave registers inside the fused kernels.
#include <cuda_bf16.h>

#include <cstdlib>
#include <cstring>

#include "kz_guide.cuh"
#include "kz_internal.h"

namespace kz {
static_assert(kGuideParams == KZ_GUIDE_PARAMS, "parameter blob size must match the C ABI");
namespace {

constexpr int kStrideW = 72;   // bf16 row stride of [out][64] weight tiles (bank-conflict free)
constexpr int kStrideW4T = 56; // bf16 row stride of W4^T [64][48]
constexpr int kRec = 496;      // bf16 per training row: X H1 H2 H3 dZ1 dZ2 dZ3 (64 each) + dO (48)
constexpr int kColX = 0, kColH1 = 64, kColH2 = 128, kColH3 = 192, kColD1 = 256, kColD2 = 320, kColD3 = 384,
              kColDO = 448;

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ void mma16816(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// acc[j] (16 x 8 tile j) = bias + A (16 x 16*KT) * Bt^T, Bt = smem [8*NT rows][stride] bf16.
template <int NT, int KT>
__device__ __forceinline__ void warp_layer(float (&acc)[NT][4], const uint32_t (&a)[KT][4],
                                           const __nv_bfloat16* Bt, int stride, const float* bias, int lane) {
    const int g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int j = 0; j < NT; ++j) {
        const float b0 = bias ? bias[8 * j + 2 * t] : 0.f;
        const float b1 = bias ? bias[8 * j + 2 * t + 1] : 0.f;
        acc[j][0] = b0;
        acc[j][1] = b1;
        acc[j][2] = b0;
        acc[j][3] = b1;
    }
#pragma unroll
    for (int kt = 0; kt < KT; ++kt) {
#pragma unroll
        for (int j = 0; j < NT; ++j) {
            const uint32_t* w = reinterpret_cast<const uint32_t*>(Bt + (8 * j + g) * stride + 16 * kt + 2 * t);
            mma16816(acc[j], a[kt], w[0], w[4]);
        }
    }
}

// Accumulator fragments (NT tiles of 16 x 8) -> A fragments (NT/2 tiles of 16 x 16), optional ReLU.
template <int NT>
__device__ __forceinline__ void to_afrag(const float (&c)[NT][4], uint32_t (&a)[NT / 2][4], bool relu) {
#pragma unroll
    for (int kt = 0; kt < NT / 2; ++kt) {
        float v[8] = {c[2 * kt][0], c[2 * kt][1], c[2 * kt][2], c[2 * kt][3],
                      c[2 * kt + 1][0], c[2 * kt + 1][1], c[2 * kt + 1][2], c[2 * kt + 1][3]};
        if (relu)
#pragma unroll
            for (int e = 0; e < 8; ++e) v[e] = fmaxf(v[e], 0.f);
        a[kt][0] = pack2(v[0], v[1]);
        a[kt][1] = pack2(v[2], v[3]);
        a[kt][2] = pack2(v[4], v[5]);
        a[kt][3] = pack2(v[6], v[7]);
    }
}

// Input features of rows g and g+8 straight into A fragments (4 k-tiles).
// Lane t holds columns 16 kt + 2t (+1) and 16 kt + 2t + 8 (+9): for the
// position axes kt = 0..2, the sin/cos pairs of bands t and t + 4 (the
// layout of guide_feature); k-tile 3 holds the normal and zero padding.
__device__ __forceinline__ void feature_afrag(uint32_t (&a)[4][4], f3 p0, f3 n0, f3 p1, f3 n1, float bs, int lane) {
    const int t = lane & 3;
#pragma unroll
    for (int kt = 0; kt < 3; ++kt) {
        float s0, c0, s1, c1, s2, c2, s3, c3;
        band_sincos(comp(p0, kt), t, bs, s0, c0);
        band_sincos(comp(p1, kt), t, bs, s1, c1);
        band_sincos(comp(p0, kt), t + 4, bs, s2, c2);
        band_sincos(comp(p1, kt), t + 4, bs, s3, c3);
        a[kt][0] = pack2(s0, c0);
        a[kt][1] = pack2(s1, c1);
        a[kt][2] = pack2(s2, c2);
        a[kt][3] = pack2(s3, c3);
    }
    const int c = 48 + 2 * t;
    a[3][0] = pack2(guide_feature(c, p0, n0, bs), guide_feature(c + 1, p0, n0, bs));
    a[3][1] = pack2(guide_feature(c, p1, n1, bs), guide_feature(c + 1, p1, n1, bs));
    a[3][2] = 0u;  // columns 56..63: padding
    a[3][3] = 0u;
}

// Stage the BF16 weights into shared memory: W1..W3 [64][72], W4 [40][72]
// and, when `transposed`, W2^T, W3^T [64][72] and W4^T [64][56].
struct SmemW {
    __nv_bfloat16* w[4];
    __nv_bfloat16* wt[4];  // wt[1..3] used
};

__device__ void stage_weights(const __nv_bfloat16* __restrict__ Wg, __nv_bfloat16* smem, bool transposed, SmemW& s) {
    s.w[0] = smem;
    s.w[1] = s.w[0] + 64 * kStrideW;
    s.w[2] = s.w[1] + 64 * kStrideW;
    s.w[3] = s.w[2] + 64 * kStrideW;
    s.wt[0] = nullptr;
    s.wt[1] = s.w[3] + 40 * kStrideW;  // W2^T
    s.wt[2] = s.wt[1] + 64 * kStrideW; // W3^T
    s.wt[3] = s.wt[2] + 64 * kStrideW; // W4^T [64][56]
    const int offs[4] = {kOffW1, kOffW2, kOffW3, kOffW4};
    const int rows[4] = {64, 64, 64, 40};
    for (int l = 0; l < 4; ++l)
        for (int i = threadIdx.x; i < rows[l] * 64; i += blockDim.x) {
            const int o = i >> 6, k = i & 63;
            const __nv_bfloat16 v = Wg[offs[l] + i];
            s.w[l][o * kStrideW + k] = v;
            if (transposed && l >= 1) {
                if (l < 3) s.wt[l][k * kStrideW + o] = v;
                else s.wt[3][k * kStrideW4T + o] = v;
            }
        }
    if (transposed)
        for (int i = threadIdx.x; i < 64 * 8; i += blockDim.x)  // W4^T columns 40..47 = 0
            s.wt[3][(i >> 3) * kStrideW4T + 40 + (i & 7)] = __float2bfloat16_rn(0.f);
    __syncthreads();
}

constexpr size_t kSmemInfer = (size_t)(64 * 3 + 40) * kStrideW * 2;
constexpr uint32_t kInferCtasPerSm = 6;  // 33 KB of weights each: six fit in shared memory
constexpr size_t kSmemTrainW = kSmemInfer + (size_t)(64 * 2) * kStrideW * 2 + (size_t)64 * kStrideW4T * 2;
constexpr int kTrainWarps = 4;
constexpr size_t kSmemTrain = kSmemTrainW + (size_t)kTrainWarps * 16 * 41 * 4;

// Forward of one 16-row tile from features to the 40 raw outputs.
__device__ __forceinline__ void forward_tile(const SmemW& s, const float* __restrict__ Wf, const uint32_t (&x)[4][4],
                                             float (&h1)[8][4], float (&h2)[8][4], float (&h3)[8][4],
                                             float (&o)[5][4], uint32_t (&a1)[4][4], uint32_t (&a2)[4][4],
                                             uint32_t (&a3)[4][4], int lane) {
    warp_layer<8, 4>(h1, x, s.w[0], kStrideW, Wf + kOffB1, lane);
    to_afrag<8>(h1, a1, true);
    warp_layer<8, 4>(h2, a1, s.w[1], kStrideW, Wf + kOffB2, lane);
    to_afrag<8>(h2, a2, true);
    warp_layer<8, 4>(h3, a2, s.w[2], kStrideW, Wf + kOffB3, lane);
    to_afrag<8>(h3, a3, true);
    warp_layer<5, 4>(o, a3, s.w[3], kStrideW, Wf + kOffB4, lane);
}

// ------------------------------------------------------------------ inference
// rows = points: pts[2i] = (p01.xyz, -), pts[2i+1] = (n.xyz, -); or, in path
// mode, the hit of path i (position and geometric normal from the triangle
// record). raw[i*40 ..] = network outputs.
template <bool kPaths>
__global__ void __launch_bounds__(128) k_guide_infer(DevScene sc, PathSoA ps, const float4* __restrict__ pts,
                                                     uint32_t n, GuideDev gd, float* __restrict__ raw,
                                                     const uint32_t* n_dev) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    if (n_dev) n = *n_dev;
    if ((n + 15) / 16 <= blockIdx.x * (blockDim.x >> 5)) return;  // no tile for this CTA
    SmemW s;
    stage_weights(gd.wbf, reinterpret_cast<__nv_bfloat16*>(smem_raw), false, s);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    const uint32_t tiles = (n + 15) / 16;
    const uint32_t tstride = gridDim.x * (blockDim.x >> 5);
    // the hit records of the warp's next tile are loaded one tile ahead, so
    // the triangle fetch that depends on them waits on one load, not two
    float4 hit_next[2];
    const uint32_t tile0 = blockIdx.x * (blockDim.x >> 5) + warp;
    if (kPaths)
        for (int h = 0; h < 2; ++h) {
            const uint32_t r = tile0 * 16 + g + 8 * h;
            hit_next[h] = r < n ? ps.hit[r] : make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
        }
    for (uint32_t tile = tile0; tile < tiles; tile += tstride) {
        f3 p[2], nn[2];
        float4 hit_cur[2];
        if (kPaths)
            for (int h = 0; h < 2; ++h) {
                hit_cur[h] = hit_next[h];
                const uint32_t r = (tile + tstride) * 16 + g + 8 * h;
                hit_next[h] = tile + tstride < tiles && r < n ? ps.hit[r] : make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
            }
        for (int h = 0; h < 2; ++h) {
            const uint32_t r = tile * 16 + g + 8 * h;
            p[h] = mk(0.5f, 0.5f, 0.5f);
            nn[h] = mk(0.f, 1.f, 0.f);
            if (r < n) {
                if (kPaths) {
                    const float4 hit = hit_cur[h];
                    const int rec = __float_as_int(hit.w);
                    if (rec >= 0) {
                        const float4 o4 = ps.o4[r], d4 = ps.d4[r];
                        const float4* tp = sc.tris + (size_t)rec * 3;
                        const float4 ta = __ldg(tp), tb = __ldg(tp + 1), tc = __ldg(tp + 2);
                        const f3 v0 = mk(ta.x, ta.y, ta.z), v1 = mk(tb.x, tb.y, tb.z), v2 = mk(tc.x, tc.y, tc.z);
                        nn[h] = normalize(cross(v1 - v0, v2 - v0));
                        const f3 P = mk(o4.x, o4.y, o4.z) + mk(d4.x, d4.y, d4.z) * hit.x;
                        p[h] = hmul(P - mk(gd.box_lo.x, gd.box_lo.y, gd.box_lo.z),
                                    mk(gd.box_inv.x, gd.box_inv.y, gd.box_inv.z));
                    }
                } else {
                    const float4 a = pts[2 * (size_t)r], b = pts[2 * (size_t)r + 1];
                    p[h] = mk(a.x, a.y, a.z);
                    nn[h] = mk(b.x, b.y, b.z);
                }
            }
        }
        uint32_t x[4][4], a1[4][4], a2[4][4], a3[4][4];
        float h1[8][4], h2[8][4], h3[8][4], o[5][4];
        feature_afrag(x, p[0], nn[0], p[1], nn[1], gd.band_scale, lane);
        forward_tile(s, gd.wf, x, h1, h2, h3, o, a1, a2, a3, lane);
        for (int h = 0; h < 2; ++h) {
            const uint32_t r = tile * 16 + g + 8 * h;
            if (r >= n) continue;
#pragma unroll
            for (int j = 0; j < 5; ++j)
                *reinterpret_cast<float2*>(raw + (size_t)r * kGuideOut + 8 * j + 2 * t) =
                    make_float2(o[j][2 * h], o[j][2 * h + 1]);
        }
    }
}

// ------------------------------------------------------------------ training: forward + loss + backward (data)
// samples: 3 float4 per row: (p01.xyz, weight), (n.xyz, -), (dir.xyz, -).
// Writes the bf16 operands of the weight-gradient products (kRec per row)
// and adds sum(weight * -log q) to *loss.
__global__ void __launch_bounds__(kTrainWarps * 32) k_guide_train_fb(const float4* __restrict__ samples,
                                                                     uint32_t count, uint32_t n, uint32_t stride,
                                                                     uint32_t offset, GuideDev gd, float inv_n,
                                                                     float wcap,
                                                                     __nv_bfloat16* __restrict__ rec,
                                                                     float* __restrict__ loss) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SmemW s;
    stage_weights(gd.wbf, reinterpret_cast<__nv_bfloat16*>(smem_raw), true, s);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    float* so = reinterpret_cast<float*>(smem_raw + kSmemTrainW) + warp * 16 * 41;
    const uint32_t tiles = (n + 15) / 16;
    const f3 ext = mk(1.f / gd.box_inv.x, 1.f / gd.box_inv.y, 1.f / gd.box_inv.z);
    float loss_acc = 0.f;
    for (uint32_t tile = blockIdx.x * kTrainWarps + warp; tile < tiles; tile += gridDim.x * kTrainWarps) {
        f3 p[2], nn[2];
        for (int h = 0; h < 2; ++h) {
            const uint32_t r = tile * 16 + g + 8 * h;
            p[h] = mk(0.5f, 0.5f, 0.5f);
            nn[h] = mk(0.f, 1.f, 0.f);
            if (r < n) {
                const size_t si = (size_t)(((uint64_t)(r + offset) * stride) % count);
                const float4 a = samples[3 * si], b = samples[3 * si + 1];
                p[h] = mk(a.x, a.y, a.z);
                nn[h] = mk(b.x, b.y, b.z);
            }
        }
        uint32_t x[4][4], a1[4][4], a2[4][4], a3[4][4];
        float h1[8][4], h2[8][4], h3[8][4], o[5][4];
        feature_afrag(x, p[0], nn[0], p[1], nn[1], gd.band_scale, lane);
        forward_tile(s, gd.wf, x, h1, h2, h3, o, a1, a2, a3, lane);
        // raw outputs -> shared rows; one lane per row computes d(loss)/d(raw)
#pragma unroll
        for (int j = 0; j < 5; ++j) {
            so[g * 41 + 8 * j + 2 * t] = o[j][0];
            so[g * 41 + 8 * j + 2 * t + 1] = o[j][1];
            so[(g + 8) * 41 + 8 * j + 2 * t] = o[j][2];
            so[(g + 8) * 41 + 8 * j + 2 * t + 1] = o[j][3];
        }
        __syncwarp();
        if (lane < 16) {
            const uint32_t r = tile * 16 + lane;
            float gr[kGuideOut];
            if (r < n) {
                const size_t si = (size_t)(((uint64_t)(r + offset) * stride) % count);
                const float4 a = samples[3 * si], c = samples[3 * si + 2];
                float raw[kGuideOut];
                for (int k = 0; k < kGuideOut; ++k) raw[k] = so[lane * 41 + k];
                const float w = fminf(a.w * inv_n, wcap);
                loss_acc += w * mixture_nll_grad(raw, mk(c.x, c.y, c.z), w, gr, mk(a.x, a.y, a.z), ext);
            } else {
                for (int k = 0; k < kGuideOut; ++k) gr[k] = 0.f;
            }
            for (int k = 0; k < kGuideOut; ++k) so[lane * 41 + k] = gr[k];
        }
        __syncwarp();
        float d[6][4];
#pragma unroll
        for (int j = 0; j < 5; ++j) {
            d[j][0] = so[g * 41 + 8 * j + 2 * t];
            d[j][1] = so[g * 41 + 8 * j + 2 * t + 1];
            d[j][2] = so[(g + 8) * 41 + 8 * j + 2 * t];
            d[j][3] = so[(g + 8) * 41 + 8 * j + 2 * t + 1];
        }
        d[5][0] = d[5][1] = d[5][2] = d[5][3] = 0.f;
        __syncwarp();
        uint32_t ad[3][4];
        to_afrag<6>(d, ad, false);
        // dH3 = dO W4 ; dZ3 = dH3 * [H3 > 0]
        float g3[8][4];
        warp_layer<8, 3>(g3, ad, s.wt[3], kStrideW4T, nullptr, lane);
#pragma unroll
        for (int j = 0; j < 8; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) g3[j][e] = h3[j][e] > 0.f ? g3[j][e] : 0.f;
        uint32_t ad3[4][4];
        to_afrag<8>(g3, ad3, false);
        float g2[8][4];
        warp_layer<8, 4>(g2, ad3, s.wt[2], kStrideW, nullptr, lane);
#pragma unroll
        for (int j = 0; j < 8; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) g2[j][e] = h2[j][e] > 0.f ? g2[j][e] : 0.f;
        uint32_t ad2[4][4];
        to_afrag<8>(g2, ad2, false);
        float g1[8][4];
        warp_layer<8, 4>(g1, ad2, s.wt[1], kStrideW, nullptr, lane);
#pragma unroll
        for (int j = 0; j < 8; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) g1[j][e] = h1[j][e] > 0.f ? g1[j][e] : 0.f;
        uint32_t ad1[4][4];
        to_afrag<8>(g1, ad1, false);
        // write the bf16 operands of the weight-gradient products
        for (int h = 0; h < 2; ++h) {
            const uint32_t r = tile * 16 + g + 8 * h;
            if (r >= n) continue;
            uint32_t* row = reinterpret_cast<uint32_t*>(rec + (size_t)r * kRec);
            const uint32_t(*srcs[7])[4] = {x, a1, a2, a3, ad1, ad2, ad3};
            const int cols[7] = {kColX, kColH1, kColH2, kColH3, kColD1, kColD2, kColD3};
            for (int q = 0; q < 7; ++q)
#pragma unroll
                for (int kt = 0; kt < 4; ++kt) {
                    row[(cols[q] + 16 * kt + 2 * t) / 2] = srcs[q][kt][h];
                    row[(cols[q] + 16 * kt + 8 + 2 * t) / 2] = srcs[q][kt][2 + h];
                }
#pragma unroll
            for (int kt = 0; kt < 3; ++kt) {
                row[(kColDO + 16 * kt + 2 * t) / 2] = ad[kt][h];
                row[(kColDO + 16 * kt + 8 + 2 * t) / 2] = ad[kt][2 + h];
            }
        }
    }
    if (lane < 16 && loss_acc != 0.f) atomicAdd(loss, loss_acc);
}

// ------------------------------------------------------------------ weight gradients
// dW_l[o][i] = sum_r dZ_l[r][o] * A_{l-1}[r][i]; db_l[o] = sum_r dZ_l[r][o].
// Each CTA reduces a contiguous row range in 64-row chunks staged transposed
// in shared memory; 8 warps own the 120 output tiles (16 x 8) of the four
// layers; partial sums are added to the FP32 gradient with atomics.
constexpr int kWgWarps = 8;
constexpr int kChunk = 64;
constexpr int kStrideT = kChunk + 8;  // bf16 stride of the transposed chunk
constexpr size_t kSmemWgrad = (size_t)kRec * kStrideT * 2;

__device__ __forceinline__ void wg_tile(int id, int& layer, int& mt, int& nt) {
    if (id < 96) {
        layer = id / 32;
        mt = (id % 32) / 8;
        nt = id % 8;
    } else {
        layer = 3;
        mt = (id - 96) / 8;
        nt = (id - 96) % 8;
    }
}

__global__ void __launch_bounds__(kWgWarps * 32) k_guide_wgrad(const __nv_bfloat16* __restrict__ rec, uint32_t n,
                                                               uint32_t rows_per_cta, float* __restrict__ grad) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __nv_bfloat16* T = reinterpret_cast<__nv_bfloat16*>(smem_raw);  // T[col][row]
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    constexpr int kTiles = 15;
    float acc[kTiles][4];
#pragma unroll
    for (int q = 0; q < kTiles; ++q) acc[q][0] = acc[q][1] = acc[q][2] = acc[q][3] = 0.f;
    float bias_acc = 0.f;  // thread i < 232 owns bias i (db1 64, db2 64, db3 64, db4 40)
    const int aprev[4] = {kColX, kColH1, kColH2, kColH3};
    const int dcol[4] = {kColD1, kColD2, kColD3, kColDO};
    const uint32_t r0 = blockIdx.x * rows_per_cta;
    const uint32_t r1 = min(n, r0 + rows_per_cta);
    for (uint32_t base = r0; base < r1; base += kChunk) {
        const uint32_t rows = min((uint32_t)kChunk, r1 - base);
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < (uint32_t)kChunk * (kRec / 2); i += blockDim.x) {
            const uint32_t r = i / (kRec / 2), cp = i % (kRec / 2);
            __nv_bfloat162 v = __floats2bfloat162_rn(0.f, 0.f);
            if (r < rows) v = *reinterpret_cast<const __nv_bfloat162*>(rec + (size_t)(base + r) * kRec + 2 * cp);
            T[(2 * cp) * kStrideT + r] = v.x;
            T[(2 * cp + 1) * kStrideT + r] = v.y;
        }
        __syncthreads();
        if (threadIdx.x < 232) {
            const int l = threadIdx.x / 64, o = threadIdx.x % 64;
            const __nv_bfloat16* src = T + (dcol[l] + o) * kStrideT;
            float s = 0.f;
            for (int r = 0; r < kChunk; ++r) s += __bfloat162float(src[r]);
            bias_acc += s;
        }
#pragma unroll
        for (int q = 0; q < kTiles; ++q) {
            int layer, mt, nt;
            wg_tile(warp + kWgWarps * q, layer, mt, nt);
            const __nv_bfloat16* A = T + (dcol[layer] + 16 * mt) * kStrideT;  // [m = out][k = row]
            const __nv_bfloat16* B = T + (aprev[layer] + 8 * nt) * kStrideT;  // [n = in][k = row]
#pragma unroll
            for (int ks = 0; ks < kChunk / 16; ++ks) {
                uint32_t a[4];
                a[0] = *reinterpret_cast<const uint32_t*>(A + g * kStrideT + 16 * ks + 2 * t);
                a[1] = *reinterpret_cast<const uint32_t*>(A + (g + 8) * kStrideT + 16 * ks + 2 * t);
                a[2] = *reinterpret_cast<const uint32_t*>(A + g * kStrideT + 16 * ks + 8 + 2 * t);
                a[3] = *reinterpret_cast<const uint32_t*>(A + (g + 8) * kStrideT + 16 * ks + 8 + 2 * t);
                const uint32_t* b = reinterpret_cast<const uint32_t*>(B + g * kStrideT + 16 * ks + 2 * t);
                mma16816(acc[q], a, b[0], b[4]);
            }
        }
    }
    const int woff[4] = {kOffW1, kOffW2, kOffW3, kOffW4};
    const int boff[4] = {kOffB1, kOffB2, kOffB3, kOffB4};
#pragma unroll
    for (int q = 0; q < kTiles; ++q) {
        int layer, mt, nt;
        wg_tile(warp + kWgWarps * q, layer, mt, nt);
        const int outs = layer == 3 ? 40 : 64;
        for (int e = 0; e < 4; ++e) {
            const int o = 16 * mt + g + (e >= 2 ? 8 : 0);
            const int i = 8 * nt + 2 * t + (e & 1);
            if (o < outs && acc[q][e] != 0.f) atomicAdd(grad + woff[layer] + o * 64 + i, acc[q][e]);
        }
    }
    if (threadIdx.x < 232 && bias_acc != 0.f) {
        const int l = threadIdx.x / 64, o = threadIdx.x % 64;
        atomicAdd(grad + boff[l] + o, bias_acc);
    }
}

// ------------------------------------------------------------------ Adam
__global__ void k_guide_adam(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                             const float* __restrict__ grad, __nv_bfloat16* __restrict__ wbf, int n, float lr,
                             float b1, float b2, float eps, float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    // W1 columns 51..63 multiply zero inputs: keep them at zero
    if (i < kOffB1 && (i & 63) >= kGuideIn) {
        w[i] = 0.f;
        wbf[i] = __float2bfloat16_rn(0.f);
        return;
    }
    const float gr = grad[i];
    const float mi = b1 * m[i] + (1.f - b1) * gr;
    const float vi = b2 * v[i] + (1.f - b2) * gr * gr;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    wbf[i] = __float2bfloat16_rn(wi);
}

__global__ void k_guide_to_bf16(const float* __restrict__ w, __nv_bfloat16* __restrict__ wbf, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) wbf[i] = __float2bfloat16_rn(w[i]);
}

int sm_count() {
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

cudaError_t guide_kernel_setup() {
    cudaError_t e = cudaFuncSetAttribute(k_guide_infer<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kSmemInfer);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_guide_infer<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemInfer);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_guide_train_fb, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemTrain);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_guide_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemWgrad);
    if (e == cudaSuccess) e = guide_wgrad_tc_setup();
    if (e == cudaSuccess) e = guide_train_tc_setup();
    return e;
}

void launch_guide_infer_paths(const DevScene& s, PathSoA p, uint32_t n, const GuideDev& gd, float* raw,
                              cudaStream_t st) {
    if (!n) return;
    const uint32_t tiles = (n + 15) / 16;
    const uint32_t grid = min((tiles + 3) / 4, (uint32_t)sm_count() * kInferCtasPerSm);
    k_guide_infer<true><<<grid, 128, kSmemInfer, st>>>(s, p, nullptr, n, gd, raw, nullptr);
}

void launch_guide_infer_paths_dev(const DevScene& s, PathSoA p, uint32_t cap, const DevCounters* ctr,
                                  const GuideDev& gd, float* raw, cudaStream_t st) {
    if (!cap) return;
    const uint32_t tiles = (cap + 15) / 16;
    const uint32_t grid = min((tiles + 3) / 4, (uint32_t)sm_count() * kInferCtasPerSm);
    k_guide_infer<true><<<grid, 128, kSmemInfer, st>>>(s, p, nullptr, cap, gd, raw, &ctr->n_active);
}

void launch_guide_infer_points(const float4* pts, uint32_t n, const GuideDev& gd, float* raw, cudaStream_t st) {
    if (!n) return;
    DevScene none;
    PathSoA np{};
    const uint32_t tiles = (n + 15) / 16;
    const uint32_t grid = min((tiles + 3) / 4, (uint32_t)sm_count() * kInferCtasPerSm);
    k_guide_infer<false><<<grid, 128, kSmemInfer, st>>>(none, np, pts, n, gd, raw, nullptr);
}

int guide_train_mode() {
    const char* sel = getenv("KZ_GUIDE_TRAIN");
    if (sel && strcmp(sel, "tc") == 0) return 1;
    if (sel && strcmp(sel, "mma") == 0) return 2;
    return 0;
}

cudaError_t launch_guide_train(const float4* samples, uint32_t count, uint32_t n, uint32_t stride,
                               uint32_t offset, float wscale, float wcap, const GuideDev& gd, __nv_bfloat16* rec,
                               float* grad, float* loss, uint32_t* status, cudaStream_t st) {
    if (!n || !count) return cudaSuccess;
    const int mode = guide_train_mode();
    if (mode == 0)
        return launch_guide_train_tc(samples, count, n, stride, offset, wscale, wcap, gd, grad, loss, status, st);
    const uint32_t tiles = (n + 15) / 16;
    const uint32_t grid = min((tiles + kTrainWarps - 1) / kTrainWarps, (uint32_t)sm_count() * 2);
    k_guide_train_fb<<<grid, kTrainWarps * 32, kSmemTrain, st>>>(samples, count, n, stride, offset, gd, wscale, wcap,
                                                                  rec, loss);
    if (mode == 1) return launch_guide_wgrad_tc(rec, n, grad, status, st);
    const uint32_t ctas = min((n + kChunk - 1) / kChunk, (uint32_t)sm_count() * 2);
    uint32_t rows = (n + ctas - 1) / ctas;
    rows = (rows + kChunk - 1) / kChunk * kChunk;
    const uint32_t g2 = (n + rows - 1) / rows;
    k_guide_wgrad<<<g2, kWgWarps * 32, kSmemWgrad, st>>>(rec, n, rows, grad);
    return cudaGetLastError();
}

void launch_guide_adam(float* w, float* m, float* v, const float* grad, __nv_bfloat16* wbf, float lr, int step,
                       cudaStream_t st) {
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    k_guide_adam<<<(kGuideParams + 255) / 256, 256, 0, st>>>(w, m, v, grad, wbf, kGuideParams, lr, b1, b2, 1e-8f,
                                                             c1, c2);
}

void launch_guide_to_bf16(const float* w, __nv_bfloat16* wbf, cudaStream_t st) {
    k_guide_to_bf16<<<(kGuideParams + 255) / 256, 256, 0, st>>>(w, wbf, kGuideParams);
}

}  // namespace kz
