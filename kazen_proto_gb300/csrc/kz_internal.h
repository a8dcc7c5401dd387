// kz_internal.h — device data structures shared by the C-ABI layer
// (kz_api.cu) and the kernels (kz_kernels.cu). Not part of the public ABI.
#pragma once

#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/kazen_gb300.h"

namespace kz {

// One GeometryLight (src/core/light.cpp:46-86): an emissive mesh sampled by
// triangle area (TriangleMesh::sample, src/core/shape.cpp:591-613).
struct DevLight {
    uint32_t tri_begin;   // first record in DevScene::light_tris (3 float4 each)
    uint32_t tri_count;
    uint32_t cdf_begin;   // tri_count + 1 entries in DevScene::light_cdf
    uint32_t geom;
    float area;           // world-space area of the whole mesh
    float Le[3];
};

// A texture as the kernels read it (kz_texture with the image moved into
// the scene's texel array).
struct DevTexture {
    int32_t kind = 0;
    uint32_t w = 0, h = 0;
    uint32_t pad = 0;
    uint64_t offset = 0;  // first float of the RGB image in DevScene::tex_data
    float scale_s = 1.f, scale_t = 1.f;
    float Ca[3] = {1.f, 1.f, 1.f}, Cb[3] = {0.f, 0.f, 0.f};
};

struct DevScene {
    const uint4* nodes = nullptr;       // n_nodes * 5 (80-byte 8-wide nodes)
    const float4* tris = nullptr;       // n_tris * 3, leaf order
    uint32_t n_nodes = 0, n_tris = 0;
    const uint32_t* geom_offset = nullptr;  // first global triangle id per mesh
    const int32_t* geom_light = nullptr;    // light index per mesh or -1
    const kz_material* materials = nullptr;
    const uint8_t* mat_class = nullptr;  // per material: 0 diffuse-like, 1 glossy, 2 delta, 3 no lobe
    uint32_t n_materials = 0;
    const DevLight* lights = nullptr;
    const float* light_cdf = nullptr;
    const float4* light_tris = nullptr;
    uint32_t n_lights = 0;
    float3 box_lo = {0.f, 0.f, 0.f};   // scene bounds (guiding input encoding)
    float3 box_inv = {1.f, 1.f, 1.f};  // 1 / extent per axis
    // textures: NULL / 0 when the scene has none
    const float2* tri_uv = nullptr;     // n_tris * 3 vertex uvs, leaf order
    const float4* tri_nrm = nullptr;    // n_tris * 3 vertex normals (w = 1; 0 for a mesh without), leaf order
    const int32_t* mat_tex = nullptr;   // texture of each material or -1
    const DevTexture* textures = nullptr;
    const float* tex_data = nullptr;
    uint32_t n_textures = 0;
    int32_t env_tex = -1;               // environment texture or -1
    float3 env = {0.f, 0.f, 0.f};       // environment radiance (times env_tex)
    uint32_t has_env = 0;
};

// Guiding network parameters as the kernels read them.
struct GuideDev {
    const __nv_bfloat16* wbf = nullptr;  // BF16 weights, [out][in] per layer
    const float* wf = nullptr;           // FP32 master copy (biases are read from it)
    float3 box_lo = {0.f, 0.f, 0.f};
    float3 box_inv = {1.f, 1.f, 1.f};
    float band_scale = 1.f;  // frequency of band b: 2^b * pi * band_scale
};

// One recorded path vertex of a guided pass (training data): position in the
// scene box and the pdf the direction was sampled with, geometric normal and
// a valid flag, sampled world direction, throughput after the vertex, and
// the incident radiance gathered from the rest of the path.
struct VRec {
    float4 p;     // (p01.xyz, pdf)
    float4 n;     // (n.xyz, valid ? 1 : 0)
    float4 d;     // (dir.xyz, -)
    float4 beta;  // (throughput after this vertex, -)
    float4 L;     // (incident radiance estimate, -)
};

// A next-event sample as training data: (p01.xyz, weight), (n.xyz, 1 once
// the shadow ray found the light visible), (light direction, -).
struct NRec {
    float4 p;
    float4 n;
    float4 d;
};

struct GuideShade {
    const float* raw = nullptr;  // network outputs per path slot (40 floats)
    VRec* recs = nullptr;        // [path - pass_first][vertex]
    NRec* nee = nullptr;         // [path - pass_first][vertex]
    uint64_t pass_first = 0;
    float alpha = 0.5f;          // probability of sampling the learned distribution
};

// Camera basis computed on the host (same float expressions the CPU
// restatement uses) and the film size.
struct DevCamera {
    float eye[3], x[3], y[3], z[3];
    float tan_half, aspect, flip;
    uint32_t W, H;
};

// Wavefront path state, structure of arrays (capacity entries each):
//   o4  = (origin.xyz, pdf of the BSDF sample that made this ray)
//   d4  = (direction.xyz, bits: vertex index | specular flag << 8)
//   b4  = (throughput.xyz, bits: path id)
//   hit = (t, u, v, bits: triangle record or -1)
//   rng = PCG32 state (the stream increment is recomputed from the path id)
struct PathSoA {
    float4* o4;
    float4* d4;
    float4* b4;
    float4* hit;
    unsigned long long* rng;
};

// Shadow-ray queue: (origin.xyz, tmax), (direction.xyz, bits: film index),
// (contribution.rgb, unused).
struct ShadowSoA {
    float4* o4;
    float4* d4;
    float4* c4;
};

struct PathParams {
    uint32_t spp;
    uint32_t max_depth;
    uint32_t rr_min;
    uint64_t seed;
    uint32_t camera;  // 1: paths start at the camera, 0: at rays[] (Li batch)
    uint32_t estimator = 0;  // 0: NEE + BSDF sampling with MIS, 1: NEE only, 2: BSDF sampling only
};

// Counters the stage kernels update on the device.
struct DevCounters {
    uint32_t n_next;     // continuing paths written by shade
    uint32_t n_shadow;   // shadow rays queued by shade
    uint32_t status;     // device-side error (KZ_ERR_STACK ...)
    uint32_t n_active;   // paths in the current buffer (device-driven loop)
    unsigned long long fetch[4];  // closest nodes, closest tris, shadow nodes, shadow tris
    // device-driven loop: path ids [0, total) are generated in order
    unsigned long long next_path, total;
    unsigned long long path_bounces, shadow_rays, iterations;
    unsigned long long gen_first;  // first path id generated this iteration
    uint32_t gen_count, gen_slot;  // how many, and where in the buffer
    uint32_t trace_next;           // persistent kernels: next path / shadow ray to fetch
    uint32_t shadow_next;
    uint32_t bar_count, bar_gen;   // grid barrier of the persistent batch kernel
    uint32_t bar_abort;            // set when a barrier wait ran out
};

// One job of a batched render: its scene, camera and film.
struct DevJob {
    DevScene scene;
    DevCamera cam;
    PathParams pp;
    float* film;                     // W*H*3 sums
    unsigned long long path_begin;   // first global path id of this job
};

struct BatchCounters {
    unsigned long long next_path;    // global path fetch counter
    unsigned long long path_bounces, shadow_rays;
    uint32_t status, pad;
};

// ---- launchers (kz_kernels.cu) -------------------------------------------
// `next` is a zeroed 64-bit fetch counter for the persistent kernel.
void launch_intersect_closest(const DevScene& s, const kz_ray* rays, uint64_t n, kz_hits hits,
                              unsigned long long* next, uint32_t* status, cudaStream_t st);
void launch_intersect_any(const DevScene& s, const kz_ray* rays, uint64_t n, uint8_t* occ,
                          unsigned long long* next, uint32_t* status, cudaStream_t st);
void launch_intersect_stats(const DevScene& s, const kz_ray* rays, uint64_t n,
                            unsigned long long* counters /*2*/, uint32_t* status, cudaStream_t st);
void launch_closure_eval(const kz_lobe* lobes, const float* wi, const float* wo, uint64_t n,
                         int convention, float* f, float* pdf, cudaStream_t st);
void launch_closure_sample(const kz_lobe* lobes, const float* wi, const float* u, uint64_t n,
                           float* wo, float* weight, float* pdf, uint8_t* flags, cudaStream_t st);

void launch_generate_camera(const DevCamera& cam, const PathParams& pp, PathSoA dst, uint32_t dst_offset,
                            uint64_t first_path, uint32_t n_new, uint32_t block, cudaStream_t st);
void launch_generate_rays(const kz_ray* rays, const PathParams& pp, PathSoA dst, uint32_t dst_offset,
                          uint64_t first_path, uint32_t n_new, uint32_t block, cudaStream_t st);
void launch_trace_paths(const DevScene& s, PathSoA p, uint32_t n, DevCounters* ctr, bool count, uint32_t block,
                        cudaStream_t st);
void launch_shade(const DevScene& s, const PathParams& pp, PathSoA in, uint32_t n_in, PathSoA out,
                  ShadowSoA sq, DevCounters* ctr, float* film, double* film64, uint32_t block,
                  cudaStream_t st);
void launch_shade_guided(const DevScene& s, const PathParams& pp, PathSoA in, uint32_t n_in, PathSoA out,
                         ShadowSoA sq, DevCounters* ctr, float* film, double* film64, const GuideShade& gs,
                         uint32_t block, cudaStream_t st);
void launch_trace_shadow_guided(const DevScene& s, ShadowSoA sq, uint32_t n_max, DevCounters* ctr, float* film,
                                double* film64, VRec* recs, NRec* nee, uint32_t max_depth, uint32_t block,
                                cudaStream_t st);
// Training samples from a pass's vertex and next-event records: 3 float4 per
// sample ((p01, weight), (n, -), (dir, -)); *count and the weight sum *wsum.
void launch_guide_collect(const VRec* recs, const NRec* nee, uint64_t n_recs, float4* samples, uint32_t cap,
                          uint32_t* count, float* wsum, cudaStream_t st);

// ---- guiding network (kz_mlp.cu) -------------------------------------------
cudaError_t guide_kernel_setup();
void launch_guide_infer_paths(const DevScene& s, PathSoA p, uint32_t n, const GuideDev& gd, float* raw,
                              cudaStream_t st);
void launch_guide_infer_points(const float4* pts, uint32_t n, const GuideDev& gd, float* raw, cudaStream_t st);
// One training batch of `rows` samples; row r reads sample ((r + offset) * stride) % count.
// Adds the weighted loss to *loss and the gradient to grad; a sample's weight
// is min(weight * wscale, wcap). A tcgen05 kernel that finds a wait stuck
// records it in *status. The implementation is chosen by guide_train_mode():
//   0: one tcgen05 kernel for the whole step (kz_guide_tc.cu; `rec` unused),
//   1: warp-level forward/backward writing 992-byte records to `rec`, then the
//      tcgen05 weight gradients (kz_mlp_tc.cu),
//   2: the same records, then the warp-level weight gradients.
cudaError_t launch_guide_train(const float4* samples, uint32_t count, uint32_t rows, uint32_t stride,
                               uint32_t offset, float wscale, float wcap, const GuideDev& gd, __nv_bfloat16* rec,
                               float* grad, float* loss, uint32_t* status, cudaStream_t st);
// KZ_GUIDE_TRAIN in the environment: "fused" (default) = 0, "tc" = 1, "mma" = 2
// (the split paths serve side-by-side measurement).
int guide_train_mode();
// ---- one-kernel tcgen05 training step (kz_guide_tc.cu) ---------------------
cudaError_t guide_train_tc_setup();
cudaError_t launch_guide_train_tc(const float4* samples, uint32_t count, uint32_t n, uint32_t stride,
                                  uint32_t offset, float wscale, float wcap, const GuideDev& gd, float* grad,
                                  float* loss, uint32_t* status, cudaStream_t st);
// ---- tcgen05 weight gradients (kz_mlp_tc.cu) --------------------------------
cudaError_t guide_wgrad_tc_setup();
cudaError_t launch_guide_wgrad_tc(const __nv_bfloat16* rec, uint32_t n, float* grad, uint32_t* status,
                                  cudaStream_t st);
void launch_guide_adam(float* w, float* m, float* v, const float* grad, __nv_bfloat16* wbf, float lr, int step,
                       cudaStream_t st);
void launch_guide_to_bf16(const float* w, __nv_bfloat16* wbf, cudaStream_t st);
// Persistent shadow pass of the device-driven loop.
void launch_trace_shadow_dev(const DevScene& s, ShadowSoA sq, uint32_t n_max, DevCounters* ctr, bool count,
                             float* film, double* film64, cudaStream_t st);
void launch_trace_shadow(const DevScene& s, ShadowSoA sq, uint32_t n_max, DevCounters* ctr, bool count,
                         float* film, double* film64, uint32_t block, cudaStream_t st);
void launch_scale(float* film, double* film64, uint64_t n, float sf, double sd, cudaStream_t st);

// Device-driven wavefront: one iteration = plan, generate, trace, [infer],
// shade, shadow, finish; every count lives in DevCounters, so the host can
// enqueue many iterations between synchronisations. Grids are sized for the
// capacity `cap`; threads beyond the device-side count exit.
// plan: reserve slots for new paths (unless !generate) and reset the
// iteration's queue counters
void launch_plan(DevCounters* ctr, uint32_t cap, cudaStream_t st, bool generate = true);
void launch_finish(DevCounters* ctr, cudaStream_t st);
void launch_generate_camera_dev(const DevCamera& cam, const PathParams& pp, PathSoA dst, DevCounters* ctr,
                                uint32_t cap, uint32_t block, cudaStream_t st);
void launch_generate_rays_dev(const kz_ray* rays, const PathParams& pp, PathSoA dst, DevCounters* ctr, uint32_t cap,
                              uint32_t block, cudaStream_t st);
void launch_trace_paths_dev(const DevScene& s, PathSoA p, uint32_t cap, DevCounters* ctr, bool count, uint32_t block,
                            cudaStream_t st);
void launch_shade_guided_dev(const DevScene& s, const PathParams& pp, PathSoA in, uint32_t cap, PathSoA out,
                             ShadowSoA sq, DevCounters* ctr, float* film, double* film64, const GuideShade& gs,
                             uint32_t block, cudaStream_t st);
void launch_shade_dev(const DevScene& s, const PathParams& pp, PathSoA in, uint32_t cap, PathSoA out, ShadowSoA sq,
                      DevCounters* ctr, float* film, double* film64, const GuideShade* gs, uint32_t block,
                      cudaStream_t st);
// Persistent batch renderer: grid = ctas blocks of `block` threads; each lane
// keeps one path in registers and refills from the global counter every
// `period` vertices (warp-aggregated fetch).
// Batched wavefront stages over the job table (device-driven counters).
void launch_generate_batch_dev(const DevJob* jobs, uint32_t n_jobs, PathSoA dst, DevCounters* ctr, uint32_t cap,
                               uint32_t block, cudaStream_t st);
void launch_trace_paths_batch(const DevJob* jobs, PathSoA p, uint32_t cap, DevCounters* ctr, cudaStream_t st);
void launch_shade_batch(const DevJob* jobs, PathSoA in, uint32_t cap, PathSoA out, ShadowSoA sq, DevCounters* ctr,
                        uint32_t block, bool textured, cudaStream_t st);
void launch_trace_shadow_batch(const DevJob* jobs, ShadowSoA sq, uint32_t cap, DevCounters* ctr, cudaStream_t st);
int batch_persistent_blocks_per_sm(bool textured);
cudaError_t launch_batch_persistent(const DevJob* jobs, uint32_t n_jobs, PathSoA A, PathSoA B, ShadowSoA sq,
                                   DevCounters* ctr, uint32_t cap, uint32_t period, uint32_t blocks, bool textured,
                                   cudaStream_t st);
// Queries the persistent stages' grid sizes (call before a stream capture).
void prepare_batch_wavefront();
constexpr uint32_t kMaxBatchJobs = 1u << 20;  // job index in 20 bits of a path's flags
void launch_render_batch(const DevJob* jobs, uint32_t n_jobs, unsigned long long total, BatchCounters* bc,
                         uint32_t period, uint32_t ctas, uint32_t block, cudaStream_t st);
void launch_guide_infer_paths_dev(const DevScene& s, PathSoA p, uint32_t cap, const DevCounters* ctr,
                                  const GuideDev& gd, float* raw, cudaStream_t st);

}  // namespace kz
