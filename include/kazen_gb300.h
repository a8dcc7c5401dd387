/*
 * kazen_gb300.h — C ABI of the GB300-native kazen rendering hot path.
 *
 * One shared library (libkazen_gb300.so) exports these entry points. Every
 * call returns a kz_status; kz_last_error_string() gives the message of the
 * last failing call on the calling thread. Buffers are caller-owned: inputs
 * are read, outputs are written, nothing is retained across calls except by
 * the scene handle (which owns its device copy of the geometry, BVH,
 * materials and lights). Pointers are host pointers when `mem` is
 * KZ_MEM_HOST (the library stages them through pinned memory) and device
 * pointers on the current CUDA device when `mem` is KZ_MEM_DEVICE.
 *
 * Calls on one scene handle are serialised by the library (a mutex per
 * handle) and run on that handle's CUDA stream; distinct handles may be used
 * from different threads. KZ_MEM_HOST calls are synchronous. KZ_MEM_DEVICE
 * calls are asynchronous on the scene stream; kz_scene_synchronize() waits
 * and returns any device-side status (e.g. KZ_ERR_STACK) raised since the
 * last synchronisation.
 *
 * Reference interfaces replaced (kazen_proto, paths within that project):
 *   HitableInterface::intersect / occluded ........ src/core/hitable.h:10-37
 *   Accelerator::add_trianglemesh / build ......... src/core/accel.h:13-41
 *   EmbreeAccel::intersect (closest, t-only) ...... src/core/accel.cpp:348-432
 *   Integrator::setup / Li ......................... src/core/integrator.h:23-39
 *   Renderer::render (per-pixel spp average) ....... src/core/renderer.cpp:18-90
 *   ClosureID / *Params / CompositeClosure ......... src/shading/bsdf.h:16-196,
 *                                                    src/shading/bsdfs.h:18-119
 *   Camera(position, lookat, up, near, far, fov) ... src/core/camera.h:31-96
 */
#ifndef KAZEN_GB300_H
#define KAZEN_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KZ_ABI_VERSION 3

/* ---- status codes ------------------------------------------------------ */
typedef int32_t kz_status;
#define KZ_OK               0
#define KZ_ERR_INVALID_ARG  1  /* bad pointer, size, id or non-finite input     */
#define KZ_ERR_OOM          2  /* device or pinned allocation failed           */
#define KZ_ERR_CUDA         3  /* a CUDA runtime call failed                   */
#define KZ_ERR_TIMEOUT      4  /* a bounded device-side wait gave up           */
#define KZ_ERR_STACK        5  /* a traversal stack overflowed (ray aborted)   */
#define KZ_ERR_STATE        6  /* call out of order (e.g. intersect before build) */
#define KZ_ERR_NO_DEVICE    7  /* no CUDA device is visible                    */

/* ---- memory kinds ------------------------------------------------------ */
#define KZ_MEM_HOST   0
#define KZ_MEM_DEVICE 1

#define KZ_INVALID_ID 0xFFFFFFFFu

/* ---- closure ids: the reference ClosureID values (src/shading/bsdf.h:16-75) */
#define KZ_CLOSURE_DIFFUSE                        0   /* DiffuseID                       */
#define KZ_CLOSURE_PHONG                          1   /* PhongID                         */
#define KZ_CLOSURE_WARD                           3   /* WardID                          */
#define KZ_CLOSURE_REFLECTION                     4   /* ReflectionID (delta)            */
#define KZ_CLOSURE_REFRACTION                     5   /* RefractionID (delta)            */
#define KZ_CLOSURE_TRANSPARENT                    6   /* TransparentID (delta)           */
#define KZ_CLOSURE_TRANSLUCENT                    7   /* TranslucentID                   */
#define KZ_CLOSURE_EMISSION                       10  /* EmissionID (Le only)            */
#define KZ_CLOSURE_KP_MIRROR                      14  /* KpMirrorID                      */
#define KZ_CLOSURE_KP_DIELECTRIC                  15  /* KpDielectricID                  */
#define KZ_CLOSURE_KP_MICROFACET                  16  /* KpMicrofacetID                  */
#define KZ_CLOSURE_KP_EMITTER                     17  /* KpEmitterID (Le only)           */
#define KZ_CLOSURE_KP_GLOSS                       18  /* KpGlossID  (microfacet, refract 0) */
#define KZ_CLOSURE_KP_GLASS                       19  /* KpGlassID  (microfacet, refract 1/2) */
#define KZ_CLOSURE_KP_PRINCIPLE_DIFFUSE           20  /* KpPrincipleDiffuseID            */
#define KZ_CLOSURE_KP_PRINCIPLE_RETRO             21  /* KpPrincipleRetroID              */
#define KZ_CLOSURE_KP_PRINCIPLE_FAKESS            22  /* KpPrincipleFakeSSID             */
#define KZ_CLOSURE_KP_PRINCIPLE_SHEEN             23  /* KpPrincipleSheenID              */
#define KZ_CLOSURE_KP_PRINCIPLE_SPECULAR_REFL     24  /* KpPrincipleSpecularReflectionID */
#define KZ_CLOSURE_KP_PRINCIPLE_CLEARCOAT         26  /* KpPrincipleClearcoatID          */
/* Not in the reference: GGX conductor with an RGB Schlick F0, built from the
 * reference GGX D/G/VNDF (src/shading/microfacet.h:95-291) and
 * fresnel_schlick(RGB F0) (src/shading/fresnel.h:185-187). */
#define KZ_CLOSURE_CONDUCTOR_GGX                  64

/* Microfacet distribution selector stored in params[0] of GLOSS / GLASS. */
#define KZ_DIST_GGX      0
#define KZ_DIST_BECKMANN 1

/*
 * One closure lobe (64 bytes). Parameter layouts, all in the y-up local
 * shading frame the reference shades in (N = (0,1,0)):
 *   DIFFUSE            params[0..2] = N
 *   KP_DIELECTRIC      params[0] = int_ior, params[1] = ext_ior
 *   KP_GLOSS/KP_GLASS  params[0] = dist, [1..3] = N, [4..6] = U,
 *                      [7] = xalpha, [8] = yalpha, [9] = eta, [10] = refract
 *   KP_PRINCIPLE_SPECULAR_REFL  [0..2] = F0, [3..5] = N, [6] = xalpha,
 *                      [7] = yalpha, [8] = eta, [9] = metallic
 *   CONDUCTOR_GGX      [0..2] = F0, [3] = xalpha, [4] = yalpha
 *   PHONG              [0..2] = N, [3] = exponent
 *   WARD               [0..2] = N, [3..5] = T, [6] = xalpha, [7] = yalpha
 *   REFLECTION         [0..2] = N, [3] = eta
 *   REFRACTION         [0..2] = N, [3] = eta (inside over outside)
 *   KP_MICROFACET      [0] = alpha, [1] = int_ior, [2] = ext_ior, [3] = kd
 *   KP_PRINCIPLE_DIFFUSE  [0..2] = N
 *   KP_PRINCIPLE_RETRO    [0..2] = N, [3] = roughness
 *   KP_PRINCIPLE_FAKESS   [0] = roughness
 *   KP_PRINCIPLE_SHEEN    [0..2] = N, [3] = sheen
 *   KP_PRINCIPLE_CLEARCOAT [0..2] = N, [3] = roughness (GTR1 alpha, in (0, 1))
 *   KP_MIRROR, TRANSPARENT, TRANSLUCENT  none
 * Delta lobes (KP_MIRROR, KP_DIELECTRIC, REFLECTION, REFRACTION,
 * TRANSPARENT) are sampled only; their eval is zero.
 * params[KZ_LOBE_TEXTURE_PARAM] (the last slot, used by no lobe) is a texture
 * reference: 0 = none, k = the weight is multiplied by texture k-1 of the
 * scene (kz_scene_set_textures) at the hit's uv. All textured lobes of one
 * material name the same texture.
 */
#define KZ_LOBE_TEXTURE_PARAM 11
typedef struct kz_lobe {
    uint32_t closure_id;
    float    weight[3];
    float    params[12];
} kz_lobe;

#define KZ_MAX_LOBES 8   /* reference max_closure, src/shading/bsdf.h:77 */

/* A lowered surface shader: emitted radiance + up to 8 weighted lobes
 * (the reference ShadingResult{Le, surface}, src/shading/bsdf.h:217-229). */
typedef struct kz_material {
    float    Le[3];
    uint32_t n_lobes;
    kz_lobe  lobes[KZ_MAX_LOBES];
} kz_material;

/* Ray record, 32 bytes (two 16-byte halves). Directions must be unit length:
 * the reference Ray ctor normalises (src/core/ray.h:12-22); callers normalise
 * once on the host so every consumer sees identical FP32 bits. */
typedef struct kz_ray {
    float ox, oy, oz, tmin;
    float dx, dy, dz, tmax;
} kz_ray;

/* Hit outputs, structure of arrays. Any pointer except t and prim_id may be
 * NULL. A miss writes t = tmax of the ray, prim_id = geom_id = KZ_INVALID_ID.
 * prim_id is the triangle index within its mesh; geom_id the mesh index
 * returned by kz_scene_add_mesh. u, v are the barycentrics of vertices 1, 2. */
typedef struct kz_hits {
    float*    t;
    uint32_t* prim_id;
    uint32_t* geom_id;
    float*    u;
    float*    v;
} kz_hits;

/* Pinhole camera, reference Camera(position, lookat, up, near, far, fov, flip)
 * (src/core/camera.h:31-96): fov is the horizontal field of view in degrees. */
typedef struct kz_camera {
    float   eye[3];
    float   lookat[3];
    float   up[3];
    float   fov_deg;
    float   near_clip;
    float   far_clip;
    int32_t flip;
} kz_camera;

typedef struct kz_film_desc {
    uint32_t width;
    uint32_t height;
} kz_film_desc;

/* Paths in flight by default: 2^24 (path state ~3.2 GB). On the 1080p,
 * 64-spp terrain frame 2^21 / 2^22 / 2^23 / 2^24 gave 1,532 / 1,622 / 1,666 /
 * 1,681 Mpaths*bounces/s, and 2^23 / 2^24 1,747 / 1,763 after the later
 * traversal changes: longer launches amortise each persistent kernel's tail
 * and the per-iteration launches. A render never holds more than its own
 * path count. */
#define KZ_RENDER_DEFAULT_WAVEFRONT (1u << 24)

typedef struct kz_render_config {
    uint32_t spp;            /* samples per pixel                              */
    uint32_t max_depth;      /* maximum number of shaded path vertices         */
    uint64_t seed;           /* PCG32 seed; stream = pixel * spp + sample      */
    uint32_t wavefront_size; /* paths in flight; 0 = KZ_RENDER_DEFAULT_WAVEFRONT */
    uint32_t rr_min_depth;   /* first vertex index that plays roulette (ref: 3) */
    uint32_t block_size;     /* threads per block of the stage kernels: 0 (= 256)
                              * or a multiple of 32 up to 256 (the kernels are
                              * compiled for at most 256 threads per block) */
    uint32_t flags;          /* KZ_RENDER_FLAG_* bits, 0 = none                */
} kz_render_config;

/* Record CUDA events around every stage launch (on the scene stream) and
 * report per-stage device time in kz_render_stats. */
#define KZ_RENDER_FLAG_TIMING 1u
/* Trace with the fetch-counting traversal variant and report BVH node and
 * triangle fetches (slower; for roofline accounting, not for timing). */
#define KZ_RENDER_FLAG_COUNT  2u
/* Estimator of kz_render / kz_li_batch (default: next-event estimation and
 * BSDF sampling combined by MIS, PathIntegrator, integrator.cpp:362-561).
 * NEE_ONLY is PathEmsIntegrator (integrator.cpp:264-360): lights found by
 * BSDF-sampled rays count only after a specular bounce or from the camera.
 * BSDF_ONLY is PathMatsIntegrator (integrator.cpp:213-262): no next-event
 * estimation, every emission hit counts in full. At most one of the two. */
#define KZ_RENDER_FLAG_NEE_ONLY  4u
#define KZ_RENDER_FLAG_BSDF_ONLY 8u

typedef struct kz_render_stats {
    uint64_t path_bounces;   /* closest-hit extension rays traced (camera rays included) */
    uint64_t shadow_rays;    /* any-hit rays traced for next-event estimation  */
    uint64_t iterations;     /* wavefront iterations                           */
    uint64_t paths;          /* camera paths started                           */
    uint64_t kernel_launches;/* kernels launched by the call                   */
    /* KZ_RENDER_FLAG_COUNT: fetches of 80-byte nodes / 48-byte triangles */
    uint64_t closest_node_fetches, closest_tri_fetches;
    uint64_t shadow_node_fetches, shadow_tri_fetches;
    /* KZ_RENDER_FLAG_TIMING: summed device time per stage, milliseconds */
    double   generate_ms, trace_ms, shade_ms, shadow_ms;
} kz_render_stats;

typedef struct kz_scene_info {
    uint64_t n_meshes;
    uint64_t n_triangles;
    uint64_t n_lights;
    uint64_t n_bvh_nodes;
    uint64_t bvh_bytes;       /* node array bytes on the device              */
    uint64_t triangle_bytes;  /* leaf-ordered triangle records on the device */
    uint32_t bvh_depth;
    uint32_t built;
} kz_scene_info;

typedef struct kz_scene kz_scene;

/* Texture for lobe weights and the environment, the GPU form of the OSL
 * lookups the reference's shaders make (texture(filename, u, v),
 * environment(filename, I); OIIO, src/shading/renderservices.cpp) and of the
 * OSL checkerboard shader network (resource/scene/textured_cornell_box). */
#define KZ_TEX_CHECKER 0  /* Ca where int(fmod(s*scale_s, 2)) ^ int(fmod(t*scale_t, 2)) == 0, else Cb */
#define KZ_TEX_IMAGE   1  /* RGB float image, bilinear, periodic wrap; t = 0 at row 0 (the top) */
typedef struct kz_texture {
    int32_t      kind;
    uint32_t     width, height;   /* IMAGE */
    const float* rgb;             /* IMAGE: width*height*3 floats, host memory, row-major from the top */
    float        scale_s, scale_t;  /* CHECKER */
    float        Ca[3], Cb[3];      /* CHECKER */
} kz_texture;

/* ---- library --------------------------------------------------------- */
int32_t     kz_abi_version(void);
const char* kz_last_error_string(void);
/* Number of visible CUDA devices (0 when none); never fails. */
int32_t     kz_device_count(void);

/* ---- scene (replaces Accelerator::add_trianglemesh / build,
 *      src/core/accel.h:22-32, and Scene::add_mesh / build_bvh,
 *      src/core/scene.h:144-164) ------------------------------------------ */
kz_status kz_scene_create(kz_scene** out_scene);
kz_status kz_scene_destroy(kz_scene* scene);
/* xyz: nverts*3 floats; idx: ntris*3 vertex indices; xform12: optional
 * row-major 3x4 object-to-world matrix (NULL = identity), applied on the host
 * at add time. Host pointers only. */
kz_status kz_scene_add_mesh(kz_scene* scene, const float* xyz, uint32_t nverts,
                            const uint32_t* idx, uint32_t ntris,
                            const float* xform12, int32_t material_id,
                            int32_t is_light, int32_t* out_geom_id);
kz_status kz_scene_set_materials(kz_scene* scene, const kz_material* materials,
                                 uint32_t n_materials);
/* Textures referenced by lobes and the environment; copied (images too).
 * Replaces the set. Call before kz_scene_build. */
kz_status kz_scene_set_textures(kz_scene* scene, const kz_texture* textures, uint32_t n_textures);
/* Per-vertex texture coordinates (nverts*2 floats, host) of a mesh added
 * with kz_scene_add_mesh. A mesh without them has uv = the barycentrics of
 * vertices 1 and 2, as the reference's meshes without texcoords do
 * (TriangleMesh::post_hit, src/core/shape.cpp:615-683). */
kz_status kz_scene_set_mesh_uvs(kz_scene* scene, int32_t geom_id, const float* uv, uint32_t nverts);
/* Per-vertex normals (nverts*3 floats, host, object space: the mesh's
 * xform12 is applied as its inverse transpose, then each is normalised) of a
 * mesh added with kz_scene_add_mesh. Shading then uses the interpolated
 * normal and the shading point moves off the flat triangle by the
 * shadow-terminator offset (Hanika 2021), as TriangleMesh::post_hit does
 * (src/core/shape.cpp:628-656); meshes without normals shade with the
 * geometric normal. */
kz_status kz_scene_set_mesh_normals(kz_scene* scene, int32_t geom_id, const float* normals, uint32_t nverts);
/* Radiance of a ray that leaves the scene (the background shader of
 * PathIntegrator::Li, src/core/integrator.cpp:381-388, 545-552): rgb times
 * texture `texture` (-1: none) looked up in latitude-longitude form,
 * s = 0.5 + atan2(d.x, -d.z) / (2 pi), t = acos(d.y) / pi. Default black. */
kz_status kz_scene_set_environment(kz_scene* scene, const float rgb[3], int32_t texture);
/* A point light (PointLight, src/core/light.cpp:18-36): next-event estimation
 * picks it like any light (uniformly among all lights, area lights first in
 * mesh order, then point lights in the order added) and it contributes
 * radiance / (0.1 |d|^2), the falloff PointLight::sample returns, without MIS
 * (nothing can hit it). Host pointers; call before kz_scene_build. */
kz_status kz_scene_add_point_light(kz_scene* scene, const float position[3], const float radiance[3],
                                   int32_t* out_light_id);
/* Builds the BVH and uploads geometry, materials, textures and the light table. */
kz_status kz_scene_build(kz_scene* scene);
kz_status kz_scene_get_info(kz_scene* scene, kz_scene_info* out_info);
/* Use an external cudaStream_t (NULL = the library-created stream). */
kz_status kz_scene_set_stream(kz_scene* scene, void* cuda_stream);
kz_status kz_scene_synchronize(kz_scene* scene);

/* ---- intersector (replaces HitableInterface::intersect / occluded,
 *      src/core/hitable.h:10-37, EmbreeAccel::intersect,
 *      src/core/accel.cpp:348-432) --------------------------------------- */
/* Closest hit in (tmin, tmax]; equal t resolves to the smaller global
 * triangle index. */
kz_status kz_intersect_closest(kz_scene* scene, const kz_ray* rays, uint64_t n,
                               kz_hits hits, int32_t mem);
/* occluded[i] = 1 when any triangle is hit in (tmin, tmax], else 0. */
kz_status kz_intersect_any(kz_scene* scene, const kz_ray* rays, uint64_t n,
                           uint8_t* occluded, int32_t mem);
/* Closest-hit traversal that also counts, per ray, BVH nodes fetched and
 * triangles tested (device-side counters; for roofline accounting). */
kz_status kz_intersect_stats(kz_scene* scene, const kz_ray* rays, uint64_t n,
                             int32_t mem, uint64_t* out_node_fetches,
                             uint64_t* out_triangle_fetches);

/* ---- closures (reference per-lobe eval/pdf/sample, src/shading/bsdfs.cpp) */
#define KZ_CONVENTION_REFERENCE  0  /* value and pdf exactly as the reference lobe returns them */
#define KZ_CONVENTION_INTEGRATOR 1  /* f*|cos(wo)| and solid-angle pdf of wo, as the path loop uses them */
/* One lobe per query (lobes[i]); wi, wo: n*3 floats (local frame, y-up).
 * out_f: n*3 floats (weight not applied), out_pdf: n floats. */
kz_status kz_closure_eval_batch(const kz_lobe* lobes, const float* wi,
                                const float* wo, uint64_t n, int32_t convention,
                                float* out_f, float* out_pdf, int32_t mem);
/* u: n*3 uniforms in [0,1). Outputs: wo (n*3), weight = f*|cos|/pdf (n*3, lobe
 * weight not applied), pdf (n, 0 for delta), flags (n: bit0 = valid,
 * bit1 = delta/specular). */
kz_status kz_closure_sample_batch(const kz_lobe* lobes, const float* wi,
                                  const float* u, uint64_t n, float* out_wo,
                                  float* out_weight, float* out_pdf,
                                  uint8_t* out_flags, int32_t mem);

/* ---- integrator (replaces PathIntegrator::Li, src/core/integrator.cpp:362-561,
 *      driven per pixel sample by Renderer::render, src/core/renderer.cpp:53-62) */
/* Li of n camera rays; path i draws from PCG32 stream (cfg.seed, i). */
kz_status kz_li_batch(kz_scene* scene, const kz_ray* rays, uint64_t n,
                      const kz_render_config* cfg, float* out_rgb, int32_t mem,
                      kz_render_stats* out_stats);
/* Full frame: out_rgb (W*H*3 floats, spp average, row 0 = top) and optional
 * out_rgb64 (FP64 accumulation of the same samples). */
kz_status kz_render(kz_scene* scene, const kz_camera* camera,
                    const kz_film_desc* film, const kz_render_config* cfg,
                    float* out_rgb, double* out_rgb64, int32_t mem,
                    kz_render_stats* out_stats);

/* ---- learned path guiding -------------------------------------------------
 * Not in the reference (kazen_proto has no guiding). A small network trained
 * online on the radiance samples the tracer produces maps a shading point
 * (position in the scene box, 8-band sin/cos encoding, plus the geometric
 * normal: 51 inputs) through 3 hidden layers of 64 ReLU units to an 8-lobe
 * von Mises-Fisher mixture over incident directions (anchor 3, concentration
 * 1, weight 1 per lobe: 40 outputs; a lobe's mean direction points from the
 * shading point to its anchor, both in scene-box coordinates, measured in
 * world units). BF16 weights, FP32 accumulation, Adam.
 * The renderer samples it with probability alpha and the BSDF otherwise and
 * weighs with the one-sample MIS pdf, so every image is unbiased whatever
 * the network has learned. */
typedef struct kz_guide kz_guide;

typedef struct kz_guide_config {
    float    alpha;             /* probability of sampling the network (0 = 0.5) */
    float    learning_rate;     /* Adam step size (0 = 1e-2)                     */
    uint32_t spp_per_pass;      /* spp rendered between training steps (0 = 1)   */
    uint32_t train;             /* 1: train after every pass, 0: frozen network  */
    uint32_t max_train_samples; /* samples per Adam step (0 = 2^18)               */
    uint32_t steps_per_pass;    /* Adam steps after each pass (0 = 1)            */
    uint32_t max_train_steps;   /* > 0: freeze the network after this many steps */
    double   time_budget_ms;    /* > 0: stop after the pass that reaches it       */
} kz_guide_config;

typedef struct kz_guide_stats {
    uint64_t passes;
    uint64_t spp_done;          /* the image is the average of this many spp     */
    uint64_t train_steps;
    uint64_t train_samples;     /* radiance samples collected                    */
    double   last_loss;         /* weighted -log q of the last step              */
    double   wall_ms;           /* whole call                                    */
    double   train_ms;          /* collection + training (host wall clock)       */
} kz_guide_stats;

#define KZ_GUIDE_PARAMS 15080   /* FP32 parameters: W1..W4 [out][64], b1..b4 */

kz_status kz_guide_create(kz_guide** out_guide, uint64_t seed);
kz_status kz_guide_destroy(kz_guide* guide);
kz_status kz_guide_get_params(kz_guide* guide, float* out_params /* KZ_GUIDE_PARAMS, host */);
kz_status kz_guide_set_params(kz_guide* guide, const float* params /* KZ_GUIDE_PARAMS, host */);
/* The guide's whole training state, for checkpoint and resume: the FP32
 * weights, Adam's first and second moments (KZ_GUIDE_PARAMS floats each, in
 * that order, 3 * KZ_GUIDE_PARAMS in all) and the Adam step count. Training
 * resumed from a restored state continues as the saved guide would have.
 * No counterpart in the reference (it has no guiding). */
kz_status kz_guide_get_state(kz_guide* guide, float* out_state, uint32_t* out_step);
kz_status kz_guide_set_state(kz_guide* guide, const float* state, uint32_t step);
/* points: n * 8 floats (p01.xyz, -, n.xyz, -); out_raw: n * 40 network outputs. */
kz_status kz_guide_forward(kz_guide* guide, const float* points, uint64_t n, float* out_raw, int32_t mem);
/* samples: n * 12 floats ((p01.xyz, weight), (n.xyz, -), (dir.xyz, -)).
 * Loss = mean over samples of weight * -log q(dir). Writes the loss, the
 * gradient (optional, KZ_GUIDE_PARAMS floats, host) and, when apply != 0,
 * takes one Adam step. n <= 2^20. */
kz_status kz_guide_train_step(kz_guide* guide, const float* samples, uint64_t n, float learning_rate,
                              int32_t apply, float* out_loss, float* out_grad, int32_t mem);
/* Guided render (same film contract as kz_render). cfg->spp is the target;
 * gcfg->time_budget_ms may stop it earlier (gstats->spp_done says where). */
kz_status kz_render_guided(kz_scene* scene, kz_guide* guide, const kz_camera* camera,
                           const kz_film_desc* film, const kz_render_config* cfg,
                           const kz_guide_config* gcfg, float* out_rgb, double* out_rgb64,
                           int32_t mem, kz_render_stats* out_stats, kz_guide_stats* out_gstats);

/* ---- batched rendering ------------------------------------------------------
 * Many independent jobs (each its own scene, camera, film, spp and depth) in
 * one call. Not in the reference (its renderer runs one scene at a time,
 * src/core/renderer.cpp:18-90); every job's film equals what kz_render
 * produces for it (same PCG32 streams). Two modes:
 *  KZ_BATCH_WAVEFRONT (default): one wavefront over all jobs' paths, driven
 *    by device counters; the stage kernels find each path's scene, camera and
 *    film through its job index, so small jobs share the GPU instead of
 *    underfilling it. With use_graph, each batch of iterations is one CUDA
 *    graph launch (one host synchronisation per batch).
 *  KZ_BATCH_MEGAKERNEL: one persistent kernel; lanes keep a path each and
 *    refill from a global path counter every refill_period vertices.
 *  KZ_BATCH_PERSISTENT: the wavefront's whole loop (every stage of every
 *    iteration) in one cooperative kernel launch, its stages separated by
 *    grid-wide barriers (bounded waits: KZ_ERR_TIMEOUT); wavefront_size and
 *    refill_period as in KZ_BATCH_WAVEFRONT, block_size fixed at 256. With
 *    use_graph the launch is replayed from a captured graph.
 * All scenes must be built on the same device; the call runs on the first
 * job's scene stream. */
#define KZ_BATCH_WAVEFRONT  0
#define KZ_BATCH_MEGAKERNEL 1
#define KZ_BATCH_PERSISTENT 2
typedef struct kz_batch_job {
    kz_scene* scene;
    kz_camera camera;
    uint32_t  width, height;
    uint32_t  spp, max_depth, rr_min_depth;
    uint64_t  seed;
    float*    out_rgb;          /* width*height*3 floats, spp average */
} kz_batch_job;

typedef struct kz_batch_config {
    uint32_t block_size;        /* threads per block (0 = 256 wavefront,
                                   128 megakernel)                           */
    uint32_t ctas_per_sm;       /* megakernel: resident blocks per SM (0 = 2) */
    uint32_t refill_period;     /* megakernel: vertices between lane refills;
                                   wavefront: iterations between generations
                                   of new paths into free slots (0 = 1)      */
    uint32_t use_graph;         /* 1: launch through a captured CUDA graph   */
    uint32_t mode;              /* KZ_BATCH_WAVEFRONT, _MEGAKERNEL or _PERSISTENT */
    uint32_t wavefront_size;    /* wavefront: paths in flight (0 = 2^24)     */
} kz_batch_config;

typedef struct kz_batch_stats {
    uint64_t paths;
    uint64_t path_bounces;
    uint64_t shadow_rays;
    uint64_t threads;           /* paths in flight (wavefront slots or lanes) */
    double   device_ms;         /* CUDA-event time of the launch (graph)      */
} kz_batch_stats;

kz_status kz_render_batch(const kz_batch_job* jobs, uint32_t n_jobs, const kz_batch_config* cfg,
                          int32_t mem, kz_batch_stats* out_stats);
/* Frees the scene's cached render scratch (wavefront buffers, staging);
 * geometry, BVH and materials stay. */
kz_status kz_scene_release_scratch(kz_scene* scene);

/* ---- Li batch that allocates nothing -------------------------------------
 * No counterpart in the reference: kazen_proto has no device path of its own.
 * Same result as kz_li_batch with KZ_MEM_DEVICE, for callers that cannot call
 * cudaMalloc while they render: a host application or framework that owns
 * the GPU's memory budget through its own allocator, or a latency-critical
 * loop that cannot afford cudaMalloc's implicit device synchronisation. The
 * wavefront scratch (path state and shadow-ray queue) lives in one static
 * device array of the library, about 3 MiB, that every GPU which loads the
 * library holds until the process exits; the call itself makes no
 * cudaMalloc, cudaFree or other allocating call.
 *   - rays and out_rgb are device pointers on the scene's device; the scene
 *     must be built (kz_scene_build allocates the scene, as before).
 *   - cfg->wavefront_size = 0 selects KZ_LI_NOALLOC_MAX_WAVEFRONT paths in
 *     flight; a larger value fails with KZ_ERR_INVALID_ARG. n itself may be
 *     up to 2^32-1: paths stream through the fixed wavefront.
 *   - The first call on a device looks up the array's device address (once
 *     per device and context, with that device current); make that first
 *     call before any stream capture. After a cudaDeviceReset the next call
 *     looks the address up again (the scene must be rebuilt first, as for
 *     every other entry point).
 *   - All calls share the one array and its previous contents (the counters
 *     are cleared on every call): calls that overlap on the GPU — from two
 *     threads, or on two scenes' streams — race and corrupt each other.
 *   - KZ_RENDER_FLAG_TIMING is ignored (stage times stay 0); the call
 *     returns after the work has finished on the scene stream.
 *   - The host waits for the stream after every wavefront iteration (it
 *     reads the queue counts to size the next launches), where kz_li_batch
 *     lets the device drive the loop and waits once per 2 x (max_depth + 1)
 *     iterations: for the same rays this call is slower, more so for small
 *     batches whose iterations are short. */
#define KZ_LI_NOALLOC_MAX_WAVEFRONT 16384u
kz_status kz_li_batch_noalloc(kz_scene* scene, const kz_ray* rays, uint64_t n,
                              const kz_render_config* cfg, float* out_rgb,
                              kz_render_stats* out_stats);

#ifdef __cplusplus
}
#endif

#endif /* KAZEN_GB300_H */
