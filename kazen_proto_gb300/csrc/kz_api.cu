// kz_api.cu — the C ABI of include/kazen_gb300.h: scene management, host
// validation, device memory, and the wavefront render loop driver.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>

#include <nvtx3/nvToolsExt.h>
#include <vector>

#include "kz_bvh.h"
#include "kz_internal.h"

namespace {

thread_local std::string g_last_error;

// Host range of one API call or wavefront batch, seen by NVTX-aware
// profilers (no-op without one attached).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

kz_status fail(kz_status code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

#define KZ_CUDA(call)                                                                        \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) {                                                             \
            if (e_ == cudaErrorMemoryAllocation)                                             \
                return fail(KZ_ERR_OOM, "%s: %s", #call, cudaGetErrorString(e_));           \
            return fail(KZ_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_));              \
        }                                                                                    \
    } while (0)

#define KZ_TRY(expr)                   \
    do {                               \
        kz_status s_ = (expr);         \
        if (s_ != KZ_OK) return s_;    \
    } while (0)

// A growable device allocation.
// Host-side fault injection for tests: with KZ_FAIL_ALLOC_AFTER=N in the
// environment, device allocations after the first N of the process fail as
// an out-of-memory would (KZ_ERR_OOM), without touching the GPU.
bool injected_alloc_failure() {
    static const long limit = [] {
        const char* v = std::getenv("KZ_FAIL_ALLOC_AFTER");
        return v ? std::strtol(v, nullptr, 10) : -1L;
    }();
    static std::atomic<long> count{0};
    return limit >= 0 && count.fetch_add(1) >= limit;
}

struct DevBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
    kz_status ensure(size_t want) {
        if (want <= bytes) return KZ_OK;
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
        size_t b = std::max<size_t>(want, 256);
        if (injected_alloc_failure())
            return fail(KZ_ERR_OOM, "cudaMalloc(%zu): refused by KZ_FAIL_ALLOC_AFTER (injected)", b);
        cudaError_t e = cudaMalloc(&ptr, b);
        if (e != cudaSuccess) {
            ptr = nullptr;
            return fail(e == cudaErrorMemoryAllocation ? KZ_ERR_OOM : KZ_ERR_CUDA, "cudaMalloc(%zu): %s", b,
                        cudaGetErrorString(e));
        }
        bytes = b;
        return KZ_OK;
    }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
    template <typename T>
    T* as() const {
        return static_cast<T*>(ptr);
    }
};

struct HostMesh {
    std::vector<float> verts;  // world space, nverts * 3
    std::vector<float> uv;     // nverts * 2 texture coordinates, or empty
    std::vector<float> nrm;    // nverts * 3 world-space unit normals, or empty
    float xf[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};  // object-to-world (for normals)
    std::vector<uint32_t> idx;
    int32_t material;
    int32_t is_light;
};

bool finite3(const float* p) { return std::isfinite(p[0]) && std::isfinite(p[1]) && std::isfinite(p[2]); }

kz_status validate_lobe(const kz_lobe& l, uint32_t m, uint32_t k) {
    for (int c = 0; c < 3; ++c)
        if (!std::isfinite(l.weight[c]) || l.weight[c] < 0.f)
            return fail(KZ_ERR_INVALID_ARG, "material %u lobe %u: weight must be finite and >= 0", m, k);
    for (int c = 0; c < 12; ++c)
        if (!std::isfinite(l.params[c]))
            return fail(KZ_ERR_INVALID_ARG, "material %u lobe %u: non-finite parameter %d", m, k, c);
    switch (l.closure_id) {
    case KZ_CLOSURE_DIFFUSE:
    case KZ_CLOSURE_KP_MIRROR:
        return KZ_OK;
    case KZ_CLOSURE_KP_DIELECTRIC:
        if (!(l.params[0] > 0.f) || !(l.params[1] > 0.f))
            return fail(KZ_ERR_INVALID_ARG, "material %u lobe %u: dielectric iors must be > 0", m, k);
        return KZ_OK;
    case KZ_CLOSURE_KP_GLOSS:
    case KZ_CLOSURE_KP_GLASS:
        if (l.params[0] != (float)KZ_DIST_GGX && l.params[0] != (float)KZ_DIST_BECKMANN)
            return fail(KZ_ERR_INVALID_ARG, "material %u lobe %u: unknown microfacet distribution", m, k);
        if (!(l.params[7] > 0.f) || !(l.params[8] > 0.f))
            return fail(KZ_ERR_INVALID_ARG, "material %u lobe %u: roughness must be > 0", m, k);
        return KZ_OK;
    case KZ_CLOSURE_KP_PRINCIPLE_SPECULAR_REFL:
        if (!(l.params[6] > 0.f) || !(l.params[7] > 0.f))
            return fail(KZ_ERR_INVALID_ARG, "material %u lobe %u: roughness must be > 0", m, k);
        return KZ_OK;
    case KZ_CLOSURE_CONDUCTOR_GGX:
        if (!(l.params[3] > 0.f) || !(l.params[4] > 0.f))
            return fail(KZ_ERR_INVALID_ARG, "material %u lobe %u: roughness must be > 0", m, k);
        return KZ_OK;
    case KZ_CLOSURE_PHONG:
        if (!(l.params[3] >= 0.f))
            return fail(KZ_ERR_INVALID_ARG, "material %u lobe %u: phong exponent must be >= 0", m, k);
        return KZ_OK;
    case KZ_CLOSURE_WARD:
        if (!(l.params[6] > 0.f) || !(l.params[7] > 0.f))
            return fail(KZ_ERR_INVALID_ARG, "material %u lobe %u: ward roughness must be > 0", m, k);
        return KZ_OK;
    case KZ_CLOSURE_REFRACTION:
        if (!(l.params[3] > 0.f))
            return fail(KZ_ERR_INVALID_ARG, "material %u lobe %u: refraction eta must be > 0", m, k);
        return KZ_OK;
    case KZ_CLOSURE_REFLECTION:
    case KZ_CLOSURE_TRANSPARENT:
    case KZ_CLOSURE_TRANSLUCENT:
    case KZ_CLOSURE_KP_PRINCIPLE_DIFFUSE:
    case KZ_CLOSURE_KP_PRINCIPLE_SHEEN:
        return KZ_OK;
    case KZ_CLOSURE_KP_MICROFACET:
        if (!(l.params[0] > 0.f) || !(l.params[1] > 0.f) || !(l.params[2] > 0.f))
            return fail(KZ_ERR_INVALID_ARG, "material %u lobe %u: kp_microfacet alpha and iors must be > 0", m, k);
        if (!(l.params[3] >= 0.f && l.params[3] <= 1.f))
            return fail(KZ_ERR_INVALID_ARG, "material %u lobe %u: kp_microfacet kd must be in [0, 1]", m, k);
        return KZ_OK;
    case KZ_CLOSURE_KP_PRINCIPLE_RETRO:
        if (!(l.params[3] >= 0.f))
            return fail(KZ_ERR_INVALID_ARG, "material %u lobe %u: roughness must be >= 0", m, k);
        return KZ_OK;
    case KZ_CLOSURE_KP_PRINCIPLE_FAKESS:
        if (!(l.params[0] >= 0.f))
            return fail(KZ_ERR_INVALID_ARG, "material %u lobe %u: roughness must be >= 0", m, k);
        return KZ_OK;
    case KZ_CLOSURE_KP_PRINCIPLE_CLEARCOAT:
        // GTR1 divides by log(alpha^2): alpha 1 is singular
        if (!(l.params[3] > 0.f && l.params[3] < 1.f))
            return fail(KZ_ERR_INVALID_ARG, "material %u lobe %u: clearcoat roughness must be in (0, 1)", m, k);
        return KZ_OK;
    case KZ_CLOSURE_EMISSION:
    case KZ_CLOSURE_KP_EMITTER:
        return fail(KZ_ERR_INVALID_ARG,
                    "material %u lobe %u: emission closures are lowered into kz_material.Le, not lobes", m, k);
    default:
        return fail(KZ_ERR_INVALID_ARG, "material %u lobe %u: unsupported closure id %u", m, k, l.closure_id);
    }
}

}  // namespace

struct kz_scene {
    std::mutex mu;
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    std::vector<HostMesh> meshes;
    std::vector<kz_material> materials;
    bool built = false;
    kz_scene_info info{};

    // device scene
    DevBuf nodes, tris, geom_offset, geom_light, mats, lights, light_cdf, light_tris, mat_class;
    // textures and environment
    std::vector<kz::DevTexture> textures;  // offsets into tex_texels
    std::vector<float> tex_texels;
    float env_rgb[3] = {0.f, 0.f, 0.f};
    int32_t env_tex = -1;
    std::vector<float> point_lights;  // 6 floats each: position, radiance
    DevBuf d_tri_uv, d_mat_tex, d_textures, d_texels, d_tri_nrm;
    kz::DevScene dev;
    DevBuf status;        // uint32 device status word for batch calls
    uint32_t* status_host = nullptr;  // pinned

    // batch scratch (host-memory calls)
    DevBuf s_rays, s_t, s_prim, s_geom, s_u, s_v, s_occ, s_ctr, s_next;

    // wavefront buffers
    DevBuf pa[5], pb[5], sh[3], ctr, film, film64;
    kz::DevCounters* ctr_host = nullptr;  // pinned

    bool cuda_ready = false;

    ~kz_scene() {
        if (!cuda_ready) return;
        cudaSetDevice(device);
        if (stream) cudaStreamSynchronize(stream);
        DevBuf* all[] = {&nodes, &tris, &geom_offset, &geom_light, &mats, &mat_class, &lights, &light_cdf,
                         &light_tris, &status, &s_rays, &s_t, &s_prim, &s_geom, &s_u, &s_v, &s_occ, &s_ctr, &s_next,
                         &ctr, &film, &film64, &d_tri_uv, &d_mat_tex, &d_textures, &d_texels, &d_tri_nrm};
        for (DevBuf* b : all) b->release();
        for (auto& b : pa) b.release();
        for (auto& b : pb) b.release();
        for (auto& b : sh) b.release();
        if (status_host) cudaFreeHost(status_host);
        if (ctr_host) cudaFreeHost(ctr_host);
        if (own_stream) cudaStreamDestroy(own_stream);
    }
};

namespace {

template <typename T>
kz_status upload(DevBuf& b, const std::vector<T>& v, cudaStream_t st) {
    KZ_TRY(b.ensure(std::max<size_t>(v.size() * sizeof(T), sizeof(T))));
    if (!v.empty()) KZ_CUDA(cudaMemcpyAsync(b.ptr, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st));
    return KZ_OK;
}

kz_status check_scene(kz_scene* s) {
    if (!s) return fail(KZ_ERR_INVALID_ARG, "scene is NULL");
    if (!s->built) return fail(KZ_ERR_STATE, "kz_scene_build has not been called since the last change");
    cudaError_t e = cudaSetDevice(s->device);
    if (e != cudaSuccess) return fail(KZ_ERR_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
    return KZ_OK;
}

kz_status check_mem(int32_t mem) {
    if (mem != KZ_MEM_HOST && mem != KZ_MEM_DEVICE) return fail(KZ_ERR_INVALID_ARG, "mem must be KZ_MEM_HOST or KZ_MEM_DEVICE");
    return KZ_OK;
}

// Waits for the stream and folds the device status word into the result.
kz_status sync_and_status(kz_scene* s) {
    KZ_CUDA(cudaMemcpyAsync(s->status_host, s->status.ptr, sizeof(uint32_t), cudaMemcpyDeviceToHost, s->stream));
    KZ_CUDA(cudaStreamSynchronize(s->stream));
    KZ_CUDA(cudaGetLastError());
    uint32_t st = *s->status_host;
    if (st != 0) {
        KZ_CUDA(cudaMemsetAsync(s->status.ptr, 0, sizeof(uint32_t), s->stream));
        KZ_CUDA(cudaStreamSynchronize(s->stream));
        if (st == KZ_ERR_STACK) return fail(KZ_ERR_STACK, "traversal stack overflow: affected rays were reported as misses");
        return fail((kz_status)st, "device reported status %u", st);
    }
    return KZ_OK;
}

// Host-side camera basis (the same float expressions as Camera::init,
// src/core/camera.h:50-96, restated for a horizontal field of view).
struct H3 {
    float x, y, z;
};
H3 h_sub(H3 a, H3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
H3 h_cross(H3 a, H3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
H3 h_norm(H3 a) {
    float l = std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    return {a.x / l, a.y / l, a.z / l};
}

kz_status make_camera(const kz_camera* c, uint32_t W, uint32_t H, kz::DevCamera& out) {
    for (int k = 0; k < 3; ++k)
        if (!std::isfinite(c->eye[k]) || !std::isfinite(c->lookat[k]) || !std::isfinite(c->up[k]))
            return fail(KZ_ERR_INVALID_ARG, "camera vectors must be finite");
    if (!(c->fov_deg > 0.f && c->fov_deg < 180.f)) return fail(KZ_ERR_INVALID_ARG, "fov_deg must be in (0, 180)");
    H3 eye{c->eye[0], c->eye[1], c->eye[2]}, look{c->lookat[0], c->lookat[1], c->lookat[2]};
    H3 up = h_norm(H3{c->up[0], c->up[1], c->up[2]});
    H3 z = h_norm(h_sub(eye, look));
    H3 x = h_norm(h_cross(up, z));
    H3 y = h_cross(z, x);
    if (!std::isfinite(x.x) || !std::isfinite(z.x)) return fail(KZ_ERR_INVALID_ARG, "degenerate camera basis");
    out.eye[0] = eye.x; out.eye[1] = eye.y; out.eye[2] = eye.z;
    out.x[0] = x.x; out.x[1] = x.y; out.x[2] = x.z;
    out.y[0] = y.x; out.y[1] = y.y; out.y[2] = y.z;
    out.z[0] = z.x; out.z[1] = z.y; out.z[2] = z.z;
    out.tan_half = (float)std::tan((double)c->fov_deg * 0.5 * M_PI / 180.0);
    out.aspect = (float)W / (float)H;
    out.flip = c->flip ? -1.f : 1.f;
    out.W = W;
    out.H = H;
    return KZ_OK;
}

kz_status alloc_paths(DevBuf* b, uint32_t cap, kz::PathSoA& p) {
    const size_t f4 = (size_t)cap * sizeof(float4);
    for (int k = 0; k < 4; ++k) KZ_TRY(b[k].ensure(f4));
    KZ_TRY(b[4].ensure((size_t)cap * sizeof(unsigned long long)));
    p.o4 = b[0].as<float4>();
    p.d4 = b[1].as<float4>();
    p.b4 = b[2].as<float4>();
    p.hit = b[3].as<float4>();
    p.rng = b[4].as<unsigned long long>();
    return KZ_OK;
}

// Wavefront path tracing of `total` paths; contributions are summed into
// film (and film64) on the device.
// Guiding hooks of the wavefront loop (null for plain rendering).
struct GuideHooks {
    const kz::GuideShade* gs = nullptr;
    kz::GuideDev gd;
    float* raw = nullptr;
};

// Wavefront path tracing of `total` paths, driven by device-side counters:
// the host enqueues batches of iterations (plan, generate, trace, [infer],
// shade, shadow, finish) and synchronises once per batch. Contributions are
// summed into film (and film64) on the device.
kz_status run_wavefront(kz_scene* s, const kz::DevCamera* cam, const kz_ray* rays_dev, uint64_t total,
                        const kz_render_config* cfg, float* film, double* film64, kz_render_stats* stats,
                        const kz::PathParams* pp_override = nullptr, const GuideHooks* gh = nullptr) {
    kz::PathParams pp;
    pp.spp = cam ? cfg->spp : 1u;
    pp.max_depth = cfg->max_depth;
    pp.rr_min = cfg->rr_min_depth;
    pp.seed = cfg->seed;
    pp.camera = cam ? 1u : 0u;
    pp.estimator = (cfg->flags & KZ_RENDER_FLAG_NEE_ONLY) ? 1u : (cfg->flags & KZ_RENDER_FLAG_BSDF_ONLY) ? 2u : 0u;
    if (pp_override) pp = *pp_override;
    uint64_t want = cfg->wavefront_size ? cfg->wavefront_size : KZ_RENDER_DEFAULT_WAVEFRONT;
    const uint32_t cap = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(std::min<uint64_t>(want, total), 1u << 30));
    const uint32_t block = cfg->block_size ? cfg->block_size : 256u;
    kz::PathSoA A, B;
    KZ_TRY(alloc_paths(s->pa, cap, A));
    KZ_TRY(alloc_paths(s->pb, cap, B));
    for (int k = 0; k < 3; ++k) KZ_TRY(s->sh[k].ensure((size_t)cap * sizeof(float4)));
    kz::ShadowSoA sq{s->sh[0].as<float4>(), s->sh[1].as<float4>(), s->sh[2].as<float4>()};
    KZ_TRY(s->ctr.ensure(sizeof(kz::DevCounters)));
    kz::DevCounters* ctr = s->ctr.as<kz::DevCounters>();
    cudaStream_t strm = s->stream;
    {
        kz::DevCounters init{};
        init.total = total;
        *s->ctr_host = init;
        KZ_CUDA(cudaMemcpyAsync(ctr, s->ctr_host, sizeof(kz::DevCounters), cudaMemcpyHostToDevice, strm));
    }
    const bool timing = (cfg->flags & KZ_RENDER_FLAG_TIMING) != 0;
    const bool count = (cfg->flags & KZ_RENDER_FLAG_COUNT) != 0;
    // one batch covers the life of two waves of paths: the host waits for the
    // device once per batch, and fewer waits leave fewer idle gaps
    const uint32_t batch = 2 * std::max<uint32_t>(4, cfg->max_depth + 1);
    std::vector<cudaEvent_t> ev;
    if (timing) {
        ev.assign(5 * (size_t)batch, nullptr);
        for (auto& e : ev)
            if (cudaEventCreate(&e) != cudaSuccess) {
                for (auto& f : ev)
                    if (f) cudaEventDestroy(f);
                return fail(KZ_ERR_CUDA, "cudaEventCreate failed");
            }
    }
    struct EvGuard {
        std::vector<cudaEvent_t>& e;
        ~EvGuard() {
            for (auto& x : e)
                if (x) cudaEventDestroy(x);
        }
    } guard{ev};
    kz_render_stats st{};
    st.paths = total;
    for (;;) {
        const NvtxRange batch_range("wavefront batch");
        for (uint32_t it = 0; it < batch; ++it) {
            cudaEvent_t* e = timing ? &ev[5 * (size_t)it] : nullptr;
            if (e) KZ_CUDA(cudaEventRecord(e[0], strm));
            kz::launch_plan(ctr, cap, strm);
            if (cam) kz::launch_generate_camera_dev(*cam, pp, A, ctr, cap, block, strm);
            else kz::launch_generate_rays_dev(rays_dev, pp, A, ctr, cap, block, strm);
            if (e) KZ_CUDA(cudaEventRecord(e[1], strm));
            kz::launch_trace_paths_dev(s->dev, A, cap, ctr, count, block, strm);
            if (gh) kz::launch_guide_infer_paths_dev(s->dev, A, cap, ctr, gh->gd, gh->raw, strm);
            if (e) KZ_CUDA(cudaEventRecord(e[2], strm));
            kz::launch_shade_dev(s->dev, pp, A, cap, B, sq, ctr, film, film64, gh ? gh->gs : nullptr, block, strm);
            if (e) KZ_CUDA(cudaEventRecord(e[3], strm));
            if (gh)
                kz::launch_trace_shadow_guided(s->dev, sq, cap, ctr, film, film64, gh->gs->recs, gh->gs->nee,
                                               pp.max_depth, block, strm);
            else
                kz::launch_trace_shadow_dev(s->dev, sq, cap, ctr, count, film, film64, strm);
            kz::launch_finish(ctr, strm);
            if (e) KZ_CUDA(cudaEventRecord(e[4], strm));
            st.kernel_launches += gh ? 7 : 6;
            std::swap(A, B);
        }
        KZ_CUDA(cudaGetLastError());
        KZ_CUDA(cudaMemcpyAsync(s->ctr_host, ctr, sizeof(kz::DevCounters), cudaMemcpyDeviceToHost, strm));
        KZ_CUDA(cudaStreamSynchronize(strm));
        if (timing)
            for (uint32_t it = 0; it < batch; ++it) {
                float ms[4];
                for (int k = 0; k < 4; ++k) KZ_CUDA(cudaEventElapsedTime(&ms[k], ev[5 * it + k], ev[5 * it + k + 1]));
                st.generate_ms += ms[0];
                st.trace_ms += ms[1];
                st.shade_ms += ms[2];
                st.shadow_ms += ms[3];
            }
        const kz::DevCounters& hc = *s->ctr_host;
        if (hc.status) return fail((kz_status)hc.status, "device status %u during rendering", hc.status);
        if (hc.n_active == 0 && hc.next_path >= hc.total) break;
    }
    const kz::DevCounters& hc = *s->ctr_host;
    st.path_bounces = hc.path_bounces;
    st.shadow_rays = hc.shadow_rays;
    st.iterations = hc.iterations;
    if (count) {
        st.closest_node_fetches = hc.fetch[0];
        st.closest_tri_fetches = hc.fetch[1];
        st.shadow_node_fetches = hc.fetch[2];
        st.shadow_tri_fetches = hc.fetch[3];
    }
    if (stats) *stats = st;
    return KZ_OK;
}

kz_status init_cuda(kz_scene* s) {
    if (s->cuda_ready) return KZ_OK;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return fail(KZ_ERR_NO_DEVICE, "no CUDA device is visible");
    }
    KZ_CUDA(cudaGetDevice(&s->device));
    s->cuda_ready = true;  // from here on the destructor releases what exists
    KZ_CUDA(cudaStreamCreateWithFlags(&s->own_stream, cudaStreamNonBlocking));
    KZ_CUDA(cudaMallocHost((void**)&s->status_host, sizeof(uint32_t)));
    KZ_CUDA(cudaMallocHost((void**)&s->ctr_host, sizeof(kz::DevCounters)));
    if (!s->stream) s->stream = s->own_stream;
    KZ_TRY(s->status.ensure(sizeof(uint32_t)));
    KZ_CUDA(cudaMemset(s->status.ptr, 0, sizeof(uint32_t)));
    return KZ_OK;
}

}  // namespace

extern "C" {

int32_t kz_abi_version(void) { return KZ_ABI_VERSION; }

const char* kz_last_error_string(void) { return g_last_error.c_str(); }

int32_t kz_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

// Scene handles are created without touching CUDA, so meshes and materials
// can be described (and validated) on any host; the CUDA context, stream and
// device buffers are set up by the first kz_scene_build on the then-current
// device.
kz_status kz_scene_create(kz_scene** out_scene) {
    if (!out_scene) return fail(KZ_ERR_INVALID_ARG, "out_scene is NULL");
    *out_scene = new kz_scene();
    return KZ_OK;
}

kz_status kz_scene_destroy(kz_scene* scene) {
    if (!scene) return KZ_OK;
    delete scene;
    return KZ_OK;
}

kz_status kz_scene_add_mesh(kz_scene* s, const float* xyz, uint32_t nverts, const uint32_t* idx, uint32_t ntris,
                            const float* xform12, int32_t material_id, int32_t is_light, int32_t* out_geom_id) {
    if (!s) return fail(KZ_ERR_INVALID_ARG, "scene is NULL");
    std::lock_guard<std::mutex> lk(s->mu);
    if ((nverts && !xyz) || (ntris && !idx)) return fail(KZ_ERR_INVALID_ARG, "NULL vertex or index array");
    if (material_id < 0) return fail(KZ_ERR_INVALID_ARG, "material_id must be >= 0");
    if (xform12)
        for (int k = 0; k < 12; ++k)
            if (!std::isfinite(xform12[k])) return fail(KZ_ERR_INVALID_ARG, "transform has a non-finite entry");
    HostMesh m;
    m.material = material_id;
    m.is_light = is_light ? 1 : 0;
    if (xform12) std::copy(xform12, xform12 + 12, m.xf);
    m.verts.resize((size_t)nverts * 3);
    for (uint32_t i = 0; i < nverts; ++i) {
        const float* p = xyz + (size_t)i * 3;
        if (!finite3(p)) return fail(KZ_ERR_INVALID_ARG, "vertex %u is not finite", i);
        float* q = &m.verts[(size_t)i * 3];
        if (xform12) {
            for (int r = 0; r < 3; ++r) {
                const float* row = xform12 + r * 4;
                q[r] = row[0] * p[0] + row[1] * p[1] + row[2] * p[2] + row[3];
            }
            if (!finite3(q)) return fail(KZ_ERR_INVALID_ARG, "transformed vertex %u is not finite", i);
        } else {
            q[0] = p[0];
            q[1] = p[1];
            q[2] = p[2];
        }
    }
    m.idx.assign(idx, idx + (size_t)ntris * 3);
    for (size_t k = 0; k < m.idx.size(); ++k)
        if (m.idx[k] >= nverts) return fail(KZ_ERR_INVALID_ARG, "index %zu (= %u) is out of range", k, m.idx[k]);
    s->meshes.push_back(std::move(m));
    s->built = false;
    if (out_geom_id) *out_geom_id = (int32_t)s->meshes.size() - 1;
    return KZ_OK;
}

kz_status kz_scene_set_materials(kz_scene* s, const kz_material* materials, uint32_t n) {
    if (!s) return fail(KZ_ERR_INVALID_ARG, "scene is NULL");
    if (n && !materials) return fail(KZ_ERR_INVALID_ARG, "materials is NULL");
    std::lock_guard<std::mutex> lk(s->mu);
    for (uint32_t m = 0; m < n; ++m) {
        const kz_material& mt = materials[m];
        if (mt.n_lobes > KZ_MAX_LOBES) return fail(KZ_ERR_INVALID_ARG, "material %u: more than %d lobes", m, KZ_MAX_LOBES);
        for (int c = 0; c < 3; ++c)
            if (!std::isfinite(mt.Le[c]) || mt.Le[c] < 0.f)
                return fail(KZ_ERR_INVALID_ARG, "material %u: Le must be finite and >= 0", m);
        for (uint32_t k = 0; k < mt.n_lobes; ++k) KZ_TRY(validate_lobe(mt.lobes[k], m, k));
    }
    s->materials.assign(materials, materials + n);
    s->built = false;
    return KZ_OK;
}

kz_status kz_scene_set_textures(kz_scene* s, const kz_texture* tex, uint32_t n) {
    if (!s) return fail(KZ_ERR_INVALID_ARG, "scene is NULL");
    if (n && !tex) return fail(KZ_ERR_INVALID_ARG, "textures is NULL");
    std::vector<kz::DevTexture> out(n);
    std::vector<float> texels;
    for (uint32_t k = 0; k < n; ++k) {
        const kz_texture& t = tex[k];
        kz::DevTexture& d = out[k];
        d.kind = t.kind;
        if (t.kind == KZ_TEX_CHECKER) {
            if (!std::isfinite(t.scale_s) || !std::isfinite(t.scale_t) || !finite3(t.Ca) || !finite3(t.Cb))
                return fail(KZ_ERR_INVALID_ARG, "texture %u: checker parameters must be finite", k);
            d.scale_s = t.scale_s;
            d.scale_t = t.scale_t;
            for (int c = 0; c < 3; ++c) {
                d.Ca[c] = t.Ca[c];
                d.Cb[c] = t.Cb[c];
            }
        } else if (t.kind == KZ_TEX_IMAGE) {
            if (!t.rgb || t.width == 0 || t.height == 0 || t.width > (1u << 16) || t.height > (1u << 16))
                return fail(KZ_ERR_INVALID_ARG, "texture %u: image needs pixels and 1..65536 columns and rows", k);
            const size_t nf = (size_t)t.width * t.height * 3;
            for (size_t i = 0; i < nf; ++i)
                if (!std::isfinite(t.rgb[i])) return fail(KZ_ERR_INVALID_ARG, "texture %u: texel %zu is not finite", k, i / 3);
            d.w = t.width;
            d.h = t.height;
            d.offset = texels.size();
            texels.insert(texels.end(), t.rgb, t.rgb + nf);
        } else {
            return fail(KZ_ERR_INVALID_ARG, "texture %u: unknown kind %d", k, t.kind);
        }
    }
    std::lock_guard<std::mutex> lk(s->mu);
    s->textures = std::move(out);
    s->tex_texels = std::move(texels);
    s->built = false;
    return KZ_OK;
}

kz_status kz_scene_set_mesh_uvs(kz_scene* s, int32_t geom_id, const float* uv, uint32_t nverts) {
    if (!s) return fail(KZ_ERR_INVALID_ARG, "scene is NULL");
    std::lock_guard<std::mutex> lk(s->mu);
    if (geom_id < 0 || (size_t)geom_id >= s->meshes.size())
        return fail(KZ_ERR_INVALID_ARG, "geom_id %d is not a mesh of this scene", geom_id);
    HostMesh& m = s->meshes[(size_t)geom_id];
    if ((size_t)nverts * 3 != m.verts.size())
        return fail(KZ_ERR_INVALID_ARG, "mesh %d has %zu vertices, got %u uvs", geom_id, m.verts.size() / 3, nverts);
    if (nverts && !uv) return fail(KZ_ERR_INVALID_ARG, "uv is NULL");
    for (size_t i = 0; i < (size_t)nverts * 2; ++i)
        if (!std::isfinite(uv[i])) return fail(KZ_ERR_INVALID_ARG, "uv %zu is not finite", i / 2);
    m.uv.assign(uv, uv + (size_t)nverts * 2);
    s->built = false;
    return KZ_OK;
}

kz_status kz_scene_set_mesh_normals(kz_scene* s, int32_t geom_id, const float* n, uint32_t nverts) {
    if (!s) return fail(KZ_ERR_INVALID_ARG, "scene is NULL");
    std::lock_guard<std::mutex> lk(s->mu);
    if (geom_id < 0 || (size_t)geom_id >= s->meshes.size())
        return fail(KZ_ERR_INVALID_ARG, "geom_id %d is not a mesh of this scene", geom_id);
    HostMesh& m = s->meshes[(size_t)geom_id];
    if ((size_t)nverts * 3 != m.verts.size())
        return fail(KZ_ERR_INVALID_ARG, "mesh %d has %zu vertices, got %u normals", geom_id, m.verts.size() / 3, nverts);
    if (nverts && !n) return fail(KZ_ERR_INVALID_ARG, "normals is NULL");
    // inverse transpose of the 3x3 part: the cofactor matrix (scaled by det, normalised away)
    const float* a = m.xf;
    const float c[9] = {a[5] * a[10] - a[6] * a[9], a[6] * a[8] - a[4] * a[10], a[4] * a[9] - a[5] * a[8],
                        a[2] * a[9] - a[1] * a[10], a[0] * a[10] - a[2] * a[8], a[1] * a[8] - a[0] * a[9],
                        a[1] * a[6] - a[2] * a[5], a[2] * a[4] - a[0] * a[6], a[0] * a[5] - a[1] * a[4]};
    // cofactors = det * inverse transpose: a mirroring transform (det < 0) keeps the normals' side
    const float sgn = a[0] * c[0] + a[1] * c[1] + a[2] * c[2] < 0.f ? -1.f : 1.f;
    std::vector<float> out((size_t)nverts * 3);
    for (uint32_t i = 0; i < nverts; ++i) {
        const float* p = n + (size_t)i * 3;
        if (!finite3(p)) return fail(KZ_ERR_INVALID_ARG, "normal %u is not finite", i);
        float q[3];
        for (int r = 0; r < 3; ++r) q[r] = sgn * (c[r * 3] * p[0] + c[r * 3 + 1] * p[1] + c[r * 3 + 2] * p[2]);
        const float len = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
        if (!(len > 0.f) || !std::isfinite(len)) return fail(KZ_ERR_INVALID_ARG, "normal %u has no direction", i);
        for (int r = 0; r < 3; ++r) out[(size_t)i * 3 + r] = q[r] / len;
    }
    m.nrm = std::move(out);
    s->built = false;
    return KZ_OK;
}

kz_status kz_scene_add_point_light(kz_scene* s, const float position[3], const float radiance[3],
                                   int32_t* out_light_id) {
    if (!s) return fail(KZ_ERR_INVALID_ARG, "scene is NULL");
    if (!position || !radiance || !finite3(position) || !finite3(radiance))
        return fail(KZ_ERR_INVALID_ARG, "point light position and radiance must be finite");
    if (radiance[0] < 0.f || radiance[1] < 0.f || radiance[2] < 0.f)
        return fail(KZ_ERR_INVALID_ARG, "point light radiance must be >= 0");
    std::lock_guard<std::mutex> lk(s->mu);
    s->point_lights.insert(s->point_lights.end(), position, position + 3);
    s->point_lights.insert(s->point_lights.end(), radiance, radiance + 3);
    s->built = false;
    if (out_light_id) *out_light_id = (int32_t)(s->point_lights.size() / 6) - 1;
    return KZ_OK;
}

kz_status kz_scene_set_environment(kz_scene* s, const float rgb[3], int32_t texture) {
    if (!s) return fail(KZ_ERR_INVALID_ARG, "scene is NULL");
    if (!rgb || !finite3(rgb) || rgb[0] < 0.f || rgb[1] < 0.f || rgb[2] < 0.f)
        return fail(KZ_ERR_INVALID_ARG, "environment radiance must be finite and >= 0");
    if (texture < -1) return fail(KZ_ERR_INVALID_ARG, "environment texture must be -1 or a texture index");
    std::lock_guard<std::mutex> lk(s->mu);
    for (int c = 0; c < 3; ++c) s->env_rgb[c] = rgb[c];
    s->env_tex = texture;
    s->built = false;
    return KZ_OK;
}

kz_status kz_scene_build(kz_scene* s) {
    const NvtxRange nvtx_range("kz_scene_build");
    if (!s) return fail(KZ_ERR_INVALID_ARG, "scene is NULL");
    std::lock_guard<std::mutex> lk(s->mu);
    // validate everything on the host before any device work
    for (size_t g = 0; g < s->meshes.size(); ++g)
        if ((size_t)s->meshes[g].material >= s->materials.size())
            return fail(KZ_ERR_INVALID_ARG, "mesh %zu uses material %d but only %zu are set", g,
                        s->meshes[g].material, s->materials.size());
    // texture references: params[KZ_LOBE_TEXTURE_PARAM] = texture + 1, one texture per material
    const uint32_t ntex = (uint32_t)s->textures.size();
    std::vector<int32_t> mat_tex(s->materials.size(), -1);
    bool any_tex = false;
    for (size_t m = 0; m < s->materials.size(); ++m) {
        const kz_material& mt = s->materials[m];
        for (uint32_t k = 0; k < mt.n_lobes; ++k) {
            const float r = mt.lobes[k].params[KZ_LOBE_TEXTURE_PARAM];
            if (r == 0.f) continue;
            if (!(r >= 1.f && r <= (float)ntex && r == std::floor(r)))
                return fail(KZ_ERR_INVALID_ARG, "material %zu lobe %u: texture reference %g with %u textures set", m,
                            k, (double)r, ntex);
            const int32_t t = (int32_t)r - 1;
            if (mat_tex[m] >= 0 && mat_tex[m] != t)
                return fail(KZ_ERR_INVALID_ARG, "material %zu: lobes reference textures %d and %d (one per material)",
                            m, mat_tex[m], t);
            mat_tex[m] = t;
            any_tex = true;
        }
    }
    if (s->env_tex >= (int32_t)ntex)
        return fail(KZ_ERR_INVALID_ARG, "environment texture %d with %u textures set", s->env_tex, ntex);
    KZ_TRY(init_cuda(s));
    KZ_CUDA(cudaSetDevice(s->device));
    // global triangle order = mesh order
    uint64_t total = 0;
    for (const auto& m : s->meshes) total += m.idx.size() / 3;
    if (total > 0x7fffffffull) return fail(KZ_ERR_INVALID_ARG, "too many triangles (%llu)", (unsigned long long)total);
    std::vector<float> tv((size_t)total * 9);
    std::vector<uint32_t> tgeom((size_t)total);
    std::vector<uint32_t> goff(s->meshes.size() + 1);
    std::vector<int32_t> gmat(s->meshes.size());
    size_t t = 0;
    for (size_t g = 0; g < s->meshes.size(); ++g) {
        const HostMesh& m = s->meshes[g];
        if ((size_t)m.material >= s->materials.size())
            return fail(KZ_ERR_INVALID_ARG, "mesh %zu uses material %d but only %zu are set", g, m.material,
                        s->materials.size());
        goff[g] = (uint32_t)t;
        gmat[g] = m.material;
        for (size_t k = 0; k < m.idx.size() / 3; ++k, ++t) {
            for (int c = 0; c < 3; ++c) {
                const float* p = &m.verts[(size_t)m.idx[k * 3 + c] * 3];
                tv[t * 9 + c * 3] = p[0];
                tv[t * 9 + c * 3 + 1] = p[1];
                tv[t * 9 + c * 3 + 2] = p[2];
            }
            tgeom[t] = (uint32_t)g;
        }
    }
    goff[s->meshes.size()] = (uint32_t)t;
    kz::BvhBuildInput in{tv.data(), (uint32_t)total, tgeom.data(), gmat.data()};
    kz::WideBvhOutput out;
    try {
        kz::build_wide_bvh(in, out);
    } catch (const std::bad_alloc&) {
        return fail(KZ_ERR_OOM, "host allocation failed during the BVH build");
    } catch (const std::exception& e) {
        return fail(KZ_ERR_INVALID_ARG, "BVH build: %s", e.what());
    }

    // lights: one per emissive mesh with triangles, area CDF in triangle order
    std::vector<kz::DevLight> lights;
    std::vector<float> cdf, ltris;
    std::vector<int32_t> glight(s->meshes.size(), -1);
    for (size_t g = 0; g < s->meshes.size(); ++g) {
        const HostMesh& m = s->meshes[g];
        const uint32_t nt = (uint32_t)(m.idx.size() / 3);
        if (!m.is_light || nt == 0) continue;
        kz::DevLight L{};
        L.tri_begin = (uint32_t)(ltris.size() / 12);
        L.tri_count = nt;
        L.cdf_begin = (uint32_t)cdf.size();
        L.geom = (uint32_t)g;
        const kz_material& mt = s->materials[(size_t)m.material];
        L.Le[0] = mt.Le[0];
        L.Le[1] = mt.Le[1];
        L.Le[2] = mt.Le[2];
        std::vector<float> c(1, 0.f);
        for (uint32_t k = 0; k < nt; ++k) {
            const float* q = &tv[(size_t)(goff[g] + k) * 9];
            const float e1[3] = {q[3] - q[0], q[4] - q[1], q[5] - q[2]};
            const float e2[3] = {q[6] - q[0], q[7] - q[1], q[8] - q[2]};
            const float cx = e1[1] * e2[2] - e1[2] * e2[1];
            const float cy = e1[2] * e2[0] - e1[0] * e2[2];
            const float cz = e1[0] * e2[1] - e1[1] * e2[0];
            const float area = 0.5f * std::sqrt(cx * cx + cy * cy + cz * cz);
            c.push_back(c.back() + area);
            for (int v = 0; v < 3; ++v) {
                ltris.push_back(q[v * 3]);
                ltris.push_back(q[v * 3 + 1]);
                ltris.push_back(q[v * 3 + 2]);
                ltris.push_back(0.f);
            }
        }
        const float sum = c.back();
        if (!(sum > 0.f)) return fail(KZ_ERR_INVALID_ARG, "light mesh %zu has zero area", g);
        const float nrm = 1.f / sum;
        for (size_t k = 1; k < c.size(); ++k) c[k] *= nrm;
        c.back() = 1.f;
        L.area = sum;
        cdf.insert(cdf.end(), c.begin(), c.end());
        glight[g] = (int32_t)lights.size();
        lights.push_back(L);
    }
    // point lights after the area lights: no triangles, the position in one light_tris record
    for (size_t k = 0; k < s->point_lights.size() / 6; ++k) {
        const float* q = &s->point_lights[k * 6];
        kz::DevLight L{};
        L.tri_begin = (uint32_t)(ltris.size() / 12);
        L.tri_count = 0;
        L.cdf_begin = 0;
        L.geom = KZ_INVALID_ID;
        L.area = 0.f;
        L.Le[0] = q[3];
        L.Le[1] = q[4];
        L.Le[2] = q[5];
        ltris.insert(ltris.end(), {q[0], q[1], q[2], 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f});
        lights.push_back(L);
    }

    // vertex normals per triangle record (leaf order) when any mesh has them
    bool any_nrm = false;
    for (const auto& m : s->meshes) any_nrm |= !m.nrm.empty();
    std::vector<float4> tri_nrm;
    if (any_nrm) {
        tri_nrm.assign((size_t)total * 3, make_float4(0.f, 0.f, 0.f, 0.f));
        for (size_t r = 0; r < (size_t)total; ++r) {
            const uint32_t gid = out.order[r];
            const HostMesh& m = s->meshes[tgeom[gid]];
            if (m.nrm.empty()) continue;
            const size_t k = gid - goff[tgeom[gid]];
            for (int c = 0; c < 3; ++c) {
                const float* q = &m.nrm[(size_t)m.idx[k * 3 + c] * 3];
                tri_nrm[r * 3 + c] = make_float4(q[0], q[1], q[2], 1.f);
            }
        }
    }
    // vertex uvs per triangle record (leaf order) for textured materials
    std::vector<float2> tri_uv;
    if (any_tex) {
        tri_uv.resize((size_t)total * 3);
        for (size_t r = 0; r < (size_t)total; ++r) {
            const uint32_t gid = out.order[r];
            const uint32_t g = tgeom[gid];
            const HostMesh& m = s->meshes[g];
            const size_t k = gid - goff[g];
            for (int c = 0; c < 3; ++c) {
                if (m.uv.empty()) {
                    tri_uv[r * 3 + c] = make_float2(c == 1 ? 1.f : 0.f, c == 2 ? 1.f : 0.f);
                } else {
                    const uint32_t vi = m.idx[k * 3 + c];
                    tri_uv[r * 3 + c] = make_float2(m.uv[(size_t)vi * 2], m.uv[(size_t)vi * 2 + 1]);
                }
            }
        }
    }

    cudaStream_t st = s->stream;
    KZ_TRY(upload(s->nodes, out.nodes, st));
    KZ_TRY(upload(s->tris, out.tris, st));
    KZ_TRY(upload(s->geom_offset, goff, st));
    KZ_TRY(upload(s->geom_light, glight, st));
    KZ_TRY(upload(s->mats, s->materials, st));
    {
        // shading class of each material (by its first lobe), the key the
        // shading kernel groups a block's paths by
        std::vector<uint8_t> cls(s->materials.size());
        for (size_t m = 0; m < s->materials.size(); ++m) {
            const kz_material& mt = s->materials[m];
            uint8_t c = 3;  // no lobe (emitter only)
            if (mt.n_lobes > 0) {
                switch (mt.lobes[0].closure_id) {
                case KZ_CLOSURE_KP_MIRROR: case KZ_CLOSURE_KP_DIELECTRIC: case KZ_CLOSURE_REFLECTION:
                case KZ_CLOSURE_REFRACTION: case KZ_CLOSURE_TRANSPARENT:
                    c = 2;  // delta
                    break;
                case KZ_CLOSURE_KP_GLOSS: case KZ_CLOSURE_KP_GLASS: case KZ_CLOSURE_CONDUCTOR_GGX:
                case KZ_CLOSURE_KP_PRINCIPLE_SPECULAR_REFL: case KZ_CLOSURE_WARD: case KZ_CLOSURE_KP_MICROFACET:
                case KZ_CLOSURE_KP_PRINCIPLE_CLEARCOAT: case KZ_CLOSURE_PHONG:
                    c = 1;  // glossy
                    break;
                default:
                    c = 0;  // diffuse-like
                }
            }
            cls[m] = c;
        }
        KZ_TRY(upload(s->mat_class, cls, st));
    }
    KZ_TRY(upload(s->lights, lights, st));
    KZ_TRY(upload(s->light_cdf, cdf, st));
    KZ_TRY(upload(s->light_tris, ltris, st));
    if (any_nrm) KZ_TRY(upload(s->d_tri_nrm, tri_nrm, st));
    if (any_tex) {
        KZ_TRY(upload(s->d_tri_uv, tri_uv, st));
        KZ_TRY(upload(s->d_mat_tex, mat_tex, st));
    }
    if (ntex) {
        KZ_TRY(upload(s->d_textures, s->textures, st));
        KZ_TRY(upload(s->d_texels, s->tex_texels, st));
    }
    KZ_CUDA(cudaStreamSynchronize(st));

    kz::DevScene& d = s->dev;
    {
        float lo[3] = {0.f, 0.f, 0.f}, hi[3] = {1.f, 1.f, 1.f};
        if (total) {
            for (int a = 0; a < 3; ++a) lo[a] = hi[a] = tv[a];
            for (size_t k = 0; k < tv.size(); k += 3)
                for (int a = 0; a < 3; ++a) {
                    lo[a] = std::min(lo[a], tv[k + a]);
                    hi[a] = std::max(hi[a], tv[k + a]);
                }
        }
        float inv[3];
        for (int a = 0; a < 3; ++a) inv[a] = hi[a] > lo[a] ? 1.f / (hi[a] - lo[a]) : 1.f;
        d.box_lo = make_float3(lo[0], lo[1], lo[2]);
        d.box_inv = make_float3(inv[0], inv[1], inv[2]);
    }
    d.nodes = s->nodes.as<uint4>();
    d.tris = s->tris.as<float4>();
    d.n_nodes = out.n_nodes;
    d.n_tris = (uint32_t)total;
    d.geom_offset = s->geom_offset.as<uint32_t>();
    d.geom_light = s->geom_light.as<int32_t>();
    d.materials = s->mats.as<kz_material>();
    d.mat_class = s->mat_class.as<uint8_t>();
    d.n_materials = (uint32_t)s->materials.size();
    d.lights = s->lights.as<kz::DevLight>();
    d.light_cdf = s->light_cdf.as<float>();
    d.light_tris = s->light_tris.as<float4>();
    d.n_lights = (uint32_t)lights.size();
    d.tri_uv = any_tex ? s->d_tri_uv.as<float2>() : nullptr;
    d.tri_nrm = any_nrm ? s->d_tri_nrm.as<float4>() : nullptr;
    d.mat_tex = any_tex ? s->d_mat_tex.as<int32_t>() : nullptr;
    d.textures = ntex ? s->d_textures.as<kz::DevTexture>() : nullptr;
    d.tex_data = ntex ? s->d_texels.as<float>() : nullptr;
    d.n_textures = ntex;
    d.env = make_float3(s->env_rgb[0], s->env_rgb[1], s->env_rgb[2]);
    d.env_tex = s->env_tex;
    d.has_env = (s->env_rgb[0] > 0.f || s->env_rgb[1] > 0.f || s->env_rgb[2] > 0.f) ? 1u : 0u;

    s->info.n_meshes = s->meshes.size();
    s->info.n_triangles = total;
    s->info.n_lights = lights.size();
    s->info.n_bvh_nodes = out.n_nodes;
    s->info.bvh_bytes = (uint64_t)out.n_nodes * kz::kWideWords * 4;
    s->info.triangle_bytes = total * 48;
    s->info.bvh_depth = out.depth;
    s->info.built = 1;
    s->built = true;
    return KZ_OK;
}

kz_status kz_scene_get_info(kz_scene* s, kz_scene_info* out) {
    if (!s || !out) return fail(KZ_ERR_INVALID_ARG, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->info;
    out->built = s->built ? 1 : 0;
    return KZ_OK;
}

kz_status kz_scene_set_stream(kz_scene* s, void* cuda_stream) {
    if (!s) return fail(KZ_ERR_INVALID_ARG, "scene is NULL");
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->cuda_ready) KZ_CUDA(cudaStreamSynchronize(s->stream));
    s->stream = cuda_stream ? static_cast<cudaStream_t>(cuda_stream) : s->own_stream;
    return KZ_OK;
}

kz_status kz_scene_synchronize(kz_scene* s) {
    if (!s) return fail(KZ_ERR_INVALID_ARG, "scene is NULL");
    std::lock_guard<std::mutex> lk(s->mu);
    if (!s->cuda_ready) return KZ_OK;
    KZ_CUDA(cudaSetDevice(s->device));
    return sync_and_status(s);
}

kz_status kz_intersect_closest(kz_scene* s, const kz_ray* rays, uint64_t n, kz_hits hits, int32_t mem) {
    const NvtxRange nvtx_range("kz_intersect_closest");
    KZ_TRY(check_mem(mem));
    if (!s) return fail(KZ_ERR_INVALID_ARG, "scene is NULL");
    std::lock_guard<std::mutex> lk(s->mu);
    KZ_TRY(check_scene(s));
    if (n == 0) return KZ_OK;
    if (!rays || !hits.t || !hits.prim_id) return fail(KZ_ERR_INVALID_ARG, "rays, hits.t and hits.prim_id are required");
    cudaStream_t st = s->stream;
    if (s->dev.n_tris == 0) {
        // nothing to hit: every ray misses
        std::vector<kz_ray> hr;
        const kz_ray* src = rays;
        if (mem == KZ_MEM_DEVICE) {
            hr.resize(n);
            KZ_CUDA(cudaMemcpyAsync(hr.data(), rays, n * sizeof(kz_ray), cudaMemcpyDeviceToHost, st));
            KZ_CUDA(cudaStreamSynchronize(st));
            src = hr.data();
        }
        std::vector<float> t(n);
        std::vector<uint32_t> inv(n, KZ_INVALID_ID);
        std::vector<float> z(n, 0.f);
        for (uint64_t i = 0; i < n; ++i) t[i] = src[i].tmax;
        auto put = [&](void* dst, const void* srcp, size_t bytes) -> kz_status {
            if (!dst) return KZ_OK;
            if (mem == KZ_MEM_DEVICE) KZ_CUDA(cudaMemcpyAsync(dst, srcp, bytes, cudaMemcpyHostToDevice, st));
            else std::memcpy(dst, srcp, bytes);
            return KZ_OK;
        };
        KZ_TRY(put(hits.t, t.data(), n * 4));
        KZ_TRY(put(hits.prim_id, inv.data(), n * 4));
        KZ_TRY(put(hits.geom_id, inv.data(), n * 4));
        KZ_TRY(put(hits.u, z.data(), n * 4));
        KZ_TRY(put(hits.v, z.data(), n * 4));
        KZ_CUDA(cudaStreamSynchronize(st));
        return KZ_OK;
    }
    KZ_TRY(s->s_next.ensure(sizeof(unsigned long long)));
    KZ_CUDA(cudaMemsetAsync(s->s_next.ptr, 0, sizeof(unsigned long long), st));
    if (mem == KZ_MEM_DEVICE) {
        kz::launch_intersect_closest(s->dev, rays, n, hits, s->s_next.as<unsigned long long>(),
                                     s->status.as<uint32_t>(), st);
        KZ_CUDA(cudaGetLastError());
        return KZ_OK;
    }
    KZ_TRY(s->s_rays.ensure(n * sizeof(kz_ray)));
    KZ_TRY(s->s_t.ensure(n * 4));
    KZ_TRY(s->s_prim.ensure(n * 4));
    if (hits.geom_id) KZ_TRY(s->s_geom.ensure(n * 4));
    if (hits.u) KZ_TRY(s->s_u.ensure(n * 4));
    if (hits.v) KZ_TRY(s->s_v.ensure(n * 4));
    KZ_CUDA(cudaMemcpyAsync(s->s_rays.ptr, rays, n * sizeof(kz_ray), cudaMemcpyHostToDevice, st));
    kz_hits dh{s->s_t.as<float>(), s->s_prim.as<uint32_t>(), hits.geom_id ? s->s_geom.as<uint32_t>() : nullptr,
               hits.u ? s->s_u.as<float>() : nullptr, hits.v ? s->s_v.as<float>() : nullptr};
    kz::launch_intersect_closest(s->dev, s->s_rays.as<kz_ray>(), n, dh, s->s_next.as<unsigned long long>(),
                                 s->status.as<uint32_t>(), st);
    KZ_CUDA(cudaGetLastError());
    KZ_CUDA(cudaMemcpyAsync(hits.t, dh.t, n * 4, cudaMemcpyDeviceToHost, st));
    KZ_CUDA(cudaMemcpyAsync(hits.prim_id, dh.prim_id, n * 4, cudaMemcpyDeviceToHost, st));
    if (hits.geom_id) KZ_CUDA(cudaMemcpyAsync(hits.geom_id, dh.geom_id, n * 4, cudaMemcpyDeviceToHost, st));
    if (hits.u) KZ_CUDA(cudaMemcpyAsync(hits.u, dh.u, n * 4, cudaMemcpyDeviceToHost, st));
    if (hits.v) KZ_CUDA(cudaMemcpyAsync(hits.v, dh.v, n * 4, cudaMemcpyDeviceToHost, st));
    return sync_and_status(s);
}

kz_status kz_intersect_any(kz_scene* s, const kz_ray* rays, uint64_t n, uint8_t* occluded, int32_t mem) {
    const NvtxRange nvtx_range("kz_intersect_any");
    KZ_TRY(check_mem(mem));
    if (!s) return fail(KZ_ERR_INVALID_ARG, "scene is NULL");
    std::lock_guard<std::mutex> lk(s->mu);
    KZ_TRY(check_scene(s));
    if (n == 0) return KZ_OK;
    if (!rays || !occluded) return fail(KZ_ERR_INVALID_ARG, "rays and occluded are required");
    cudaStream_t st = s->stream;
    if (s->dev.n_tris == 0) {
        if (mem == KZ_MEM_DEVICE) KZ_CUDA(cudaMemsetAsync(occluded, 0, n, st));
        else std::memset(occluded, 0, n);
        return KZ_OK;
    }
    KZ_TRY(s->s_next.ensure(sizeof(unsigned long long)));
    KZ_CUDA(cudaMemsetAsync(s->s_next.ptr, 0, sizeof(unsigned long long), st));
    if (mem == KZ_MEM_DEVICE) {
        kz::launch_intersect_any(s->dev, rays, n, occluded, s->s_next.as<unsigned long long>(),
                                 s->status.as<uint32_t>(), st);
        KZ_CUDA(cudaGetLastError());
        return KZ_OK;
    }
    KZ_TRY(s->s_rays.ensure(n * sizeof(kz_ray)));
    KZ_TRY(s->s_occ.ensure(n));
    KZ_CUDA(cudaMemcpyAsync(s->s_rays.ptr, rays, n * sizeof(kz_ray), cudaMemcpyHostToDevice, st));
    kz::launch_intersect_any(s->dev, s->s_rays.as<kz_ray>(), n, s->s_occ.as<uint8_t>(),
                             s->s_next.as<unsigned long long>(), s->status.as<uint32_t>(), st);
    KZ_CUDA(cudaGetLastError());
    KZ_CUDA(cudaMemcpyAsync(occluded, s->s_occ.ptr, n, cudaMemcpyDeviceToHost, st));
    return sync_and_status(s);
}

kz_status kz_intersect_stats(kz_scene* s, const kz_ray* rays, uint64_t n, int32_t mem, uint64_t* out_nodes,
                             uint64_t* out_tris) {
    const NvtxRange nvtx_range("kz_intersect_stats");
    KZ_TRY(check_mem(mem));
    if (!s) return fail(KZ_ERR_INVALID_ARG, "scene is NULL");
    std::lock_guard<std::mutex> lk(s->mu);
    KZ_TRY(check_scene(s));
    if (!out_nodes || !out_tris) return fail(KZ_ERR_INVALID_ARG, "output counters are required");
    *out_nodes = *out_tris = 0;
    if (n == 0 || s->dev.n_tris == 0) return KZ_OK;
    if (!rays) return fail(KZ_ERR_INVALID_ARG, "rays is NULL");
    cudaStream_t st = s->stream;
    const kz_ray* dr = rays;
    if (mem == KZ_MEM_HOST) {
        KZ_TRY(s->s_rays.ensure(n * sizeof(kz_ray)));
        KZ_CUDA(cudaMemcpyAsync(s->s_rays.ptr, rays, n * sizeof(kz_ray), cudaMemcpyHostToDevice, st));
        dr = s->s_rays.as<kz_ray>();
    }
    KZ_TRY(s->s_ctr.ensure(2 * sizeof(unsigned long long)));
    KZ_CUDA(cudaMemsetAsync(s->s_ctr.ptr, 0, 2 * sizeof(unsigned long long), st));
    kz::launch_intersect_stats(s->dev, dr, n, s->s_ctr.as<unsigned long long>(), s->status.as<uint32_t>(), st);
    KZ_CUDA(cudaGetLastError());
    unsigned long long h[2];
    KZ_CUDA(cudaMemcpyAsync(h, s->s_ctr.ptr, sizeof(h), cudaMemcpyDeviceToHost, st));
    KZ_TRY(sync_and_status(s));
    *out_nodes = h[0];
    *out_tris = h[1];
    return KZ_OK;
}

kz_status kz_closure_eval_batch(const kz_lobe* lobes, const float* wi, const float* wo, uint64_t n, int32_t convention,
                                float* out_f, float* out_pdf, int32_t mem) {
    KZ_TRY(check_mem(mem));
    if (convention != KZ_CONVENTION_REFERENCE && convention != KZ_CONVENTION_INTEGRATOR)
        return fail(KZ_ERR_INVALID_ARG, "unknown convention %d", convention);
    if (n == 0) return KZ_OK;
    if (!lobes || !wi || !wo || !out_f || !out_pdf) return fail(KZ_ERR_INVALID_ARG, "NULL argument");
    if (kz_device_count() == 0) return fail(KZ_ERR_NO_DEVICE, "no CUDA device is visible");
    cudaStream_t st = cudaStreamPerThread;
    if (mem == KZ_MEM_DEVICE) {
        kz::launch_closure_eval(lobes, wi, wo, n, convention, out_f, out_pdf, st);
        KZ_CUDA(cudaGetLastError());
        KZ_CUDA(cudaStreamSynchronize(st));
        return KZ_OK;
    }
    DevBuf bl, bi, bo, bf, bp;
    KZ_TRY(bl.ensure(n * sizeof(kz_lobe)));
    KZ_TRY(bi.ensure(n * 12));
    KZ_TRY(bo.ensure(n * 12));
    KZ_TRY(bf.ensure(n * 12));
    KZ_TRY(bp.ensure(n * 4));
    KZ_CUDA(cudaMemcpyAsync(bl.ptr, lobes, n * sizeof(kz_lobe), cudaMemcpyHostToDevice, st));
    KZ_CUDA(cudaMemcpyAsync(bi.ptr, wi, n * 12, cudaMemcpyHostToDevice, st));
    KZ_CUDA(cudaMemcpyAsync(bo.ptr, wo, n * 12, cudaMemcpyHostToDevice, st));
    kz::launch_closure_eval(bl.as<kz_lobe>(), bi.as<float>(), bo.as<float>(), n, convention, bf.as<float>(),
                            bp.as<float>(), st);
    KZ_CUDA(cudaGetLastError());
    KZ_CUDA(cudaMemcpyAsync(out_f, bf.ptr, n * 12, cudaMemcpyDeviceToHost, st));
    KZ_CUDA(cudaMemcpyAsync(out_pdf, bp.ptr, n * 4, cudaMemcpyDeviceToHost, st));
    KZ_CUDA(cudaStreamSynchronize(st));
    bl.release(); bi.release(); bo.release(); bf.release(); bp.release();
    return KZ_OK;
}

kz_status kz_closure_sample_batch(const kz_lobe* lobes, const float* wi, const float* u, uint64_t n, float* out_wo,
                                  float* out_weight, float* out_pdf, uint8_t* out_flags, int32_t mem) {
    KZ_TRY(check_mem(mem));
    if (n == 0) return KZ_OK;
    if (!lobes || !wi || !u || !out_wo || !out_weight || !out_pdf || !out_flags)
        return fail(KZ_ERR_INVALID_ARG, "NULL argument");
    if (kz_device_count() == 0) return fail(KZ_ERR_NO_DEVICE, "no CUDA device is visible");
    cudaStream_t st = cudaStreamPerThread;
    if (mem == KZ_MEM_DEVICE) {
        kz::launch_closure_sample(lobes, wi, u, n, out_wo, out_weight, out_pdf, out_flags, st);
        KZ_CUDA(cudaGetLastError());
        KZ_CUDA(cudaStreamSynchronize(st));
        return KZ_OK;
    }
    DevBuf bl, bi, bu, bo, bw, bp, bfl;
    KZ_TRY(bl.ensure(n * sizeof(kz_lobe)));
    KZ_TRY(bi.ensure(n * 12));
    KZ_TRY(bu.ensure(n * 12));
    KZ_TRY(bo.ensure(n * 12));
    KZ_TRY(bw.ensure(n * 12));
    KZ_TRY(bp.ensure(n * 4));
    KZ_TRY(bfl.ensure(n));
    KZ_CUDA(cudaMemcpyAsync(bl.ptr, lobes, n * sizeof(kz_lobe), cudaMemcpyHostToDevice, st));
    KZ_CUDA(cudaMemcpyAsync(bi.ptr, wi, n * 12, cudaMemcpyHostToDevice, st));
    KZ_CUDA(cudaMemcpyAsync(bu.ptr, u, n * 12, cudaMemcpyHostToDevice, st));
    kz::launch_closure_sample(bl.as<kz_lobe>(), bi.as<float>(), bu.as<float>(), n, bo.as<float>(), bw.as<float>(),
                              bp.as<float>(), bfl.as<uint8_t>(), st);
    KZ_CUDA(cudaGetLastError());
    KZ_CUDA(cudaMemcpyAsync(out_wo, bo.ptr, n * 12, cudaMemcpyDeviceToHost, st));
    KZ_CUDA(cudaMemcpyAsync(out_weight, bw.ptr, n * 12, cudaMemcpyDeviceToHost, st));
    KZ_CUDA(cudaMemcpyAsync(out_pdf, bp.ptr, n * 4, cudaMemcpyDeviceToHost, st));
    KZ_CUDA(cudaMemcpyAsync(out_flags, bfl.ptr, n, cudaMemcpyDeviceToHost, st));
    KZ_CUDA(cudaStreamSynchronize(st));
    bl.release(); bi.release(); bu.release(); bo.release(); bw.release(); bp.release(); bfl.release();
    return KZ_OK;
}

static kz_status check_cfg(const kz_render_config* cfg) {
    if (!cfg) return fail(KZ_ERR_INVALID_ARG, "cfg is NULL");
    if (cfg->spp == 0) return fail(KZ_ERR_INVALID_ARG, "spp must be >= 1");
    if (cfg->max_depth == 0 || cfg->max_depth > 255) return fail(KZ_ERR_INVALID_ARG, "max_depth must be in [1, 255]");
    if ((cfg->flags & KZ_RENDER_FLAG_NEE_ONLY) && (cfg->flags & KZ_RENDER_FLAG_BSDF_ONLY))
        return fail(KZ_ERR_INVALID_ARG, "KZ_RENDER_FLAG_NEE_ONLY and KZ_RENDER_FLAG_BSDF_ONLY exclude each other");
    // the stage kernels are compiled with __launch_bounds__(256): a larger
    // block would pass here and then fail at every launch
    if (cfg->block_size % 32 != 0 || cfg->block_size > 256)
        return fail(KZ_ERR_INVALID_ARG, "block_size must be 0 or a multiple of 32 that is <= 256");
    return KZ_OK;
}

kz_status kz_li_batch(kz_scene* s, const kz_ray* rays, uint64_t n, const kz_render_config* cfg, float* out_rgb,
                      int32_t mem, kz_render_stats* out_stats) {
    const NvtxRange nvtx_range("kz_li_batch");
    KZ_TRY(check_mem(mem));
    if (!s) return fail(KZ_ERR_INVALID_ARG, "scene is NULL");
    std::lock_guard<std::mutex> lk(s->mu);
    KZ_TRY(check_cfg(cfg));  // before the scene check: needs no device
    KZ_TRY(check_scene(s));
    if (n == 0) return KZ_OK;
    if (n > 0xffffffffull) return fail(KZ_ERR_INVALID_ARG, "at most 2^32-1 rays per call");
    if (!rays || !out_rgb) return fail(KZ_ERR_INVALID_ARG, "rays and out_rgb are required");
    cudaStream_t st = s->stream;
    const kz_ray* dr = rays;
    if (mem == KZ_MEM_HOST) {
        KZ_TRY(s->s_rays.ensure(n * sizeof(kz_ray)));
        KZ_CUDA(cudaMemcpyAsync(s->s_rays.ptr, rays, n * sizeof(kz_ray), cudaMemcpyHostToDevice, st));
        dr = s->s_rays.as<kz_ray>();
    }
    float* film = out_rgb;
    if (mem == KZ_MEM_HOST) {
        KZ_TRY(s->film.ensure(n * 12));
        film = s->film.as<float>();
    }
    KZ_CUDA(cudaMemsetAsync(film, 0, n * 12, st));
    KZ_TRY(run_wavefront(s, nullptr, dr, n, cfg, film, nullptr, out_stats));
    if (mem == KZ_MEM_HOST) {
        KZ_CUDA(cudaMemcpyAsync(out_rgb, film, n * 12, cudaMemcpyDeviceToHost, st));
        KZ_CUDA(cudaStreamSynchronize(st));
    }
    return KZ_OK;
}

kz_status kz_render(kz_scene* s, const kz_camera* camera, const kz_film_desc* fd, const kz_render_config* cfg,
                    float* out_rgb, double* out_rgb64, int32_t mem, kz_render_stats* out_stats) {
    const NvtxRange nvtx_range("kz_render");
    KZ_TRY(check_mem(mem));
    if (!s) return fail(KZ_ERR_INVALID_ARG, "scene is NULL");
    std::lock_guard<std::mutex> lk(s->mu);
    KZ_TRY(check_cfg(cfg));  // before the scene check: needs no device
    KZ_TRY(check_scene(s));
    if (!camera || !fd) return fail(KZ_ERR_INVALID_ARG, "camera and film are required");
    if (!out_rgb) return fail(KZ_ERR_INVALID_ARG, "out_rgb is required");
    if (fd->width == 0 || fd->height == 0) return fail(KZ_ERR_INVALID_ARG, "film size must be > 0");
    const uint64_t npix = (uint64_t)fd->width * fd->height;
    const uint64_t total = npix * cfg->spp;
    if (total > 0xffffffffull) return fail(KZ_ERR_INVALID_ARG, "width*height*spp must be < 2^32");
    kz::DevCamera cam;
    KZ_TRY(make_camera(camera, fd->width, fd->height, cam));
    cudaStream_t st = s->stream;
    float* film = out_rgb;
    double* film64 = out_rgb64;
    if (mem == KZ_MEM_HOST) {
        KZ_TRY(s->film.ensure(npix * 12));
        film = s->film.as<float>();
        if (out_rgb64) {
            KZ_TRY(s->film64.ensure(npix * 24));
            film64 = s->film64.as<double>();
        }
    }
    KZ_CUDA(cudaMemsetAsync(film, 0, npix * 12, st));
    if (film64) KZ_CUDA(cudaMemsetAsync(film64, 0, npix * 24, st));
    KZ_TRY(run_wavefront(s, &cam, nullptr, total, cfg, film, film64, out_stats));
    kz::launch_scale(film, nullptr, npix * 3, 1.0f / (float)cfg->spp, 0.0, st);
    if (film64) kz::launch_scale(nullptr, film64, npix * 3, 0.f, 1.0 / (double)cfg->spp, st);
    KZ_CUDA(cudaGetLastError());
    if (mem == KZ_MEM_HOST) {
        KZ_CUDA(cudaMemcpyAsync(out_rgb, film, npix * 12, cudaMemcpyDeviceToHost, st));
        if (out_rgb64) KZ_CUDA(cudaMemcpyAsync(out_rgb64, film64, npix * 24, cudaMemcpyDeviceToHost, st));
    }
    KZ_CUDA(cudaStreamSynchronize(st));
    return KZ_OK;
}

}  // extern "C"


// ---------------------------------------------------------------------------
// Learned path guiding: the network object and the guided render loop.
struct kz_guide {
    std::mutex mu;
    int device = 0;
    float band_scale = 1.f;
    float weight_cap = 20.f;
    cudaStream_t stream = nullptr;
    DevBuf w, m, v, grad, wbf, loss;  // parameters (FP32, BF16), Adam moments, gradient
    DevBuf train_rec, samples, raw, recs, nee, pts, ctr;
    int step = 0;
    ~kz_guide() {
        cudaSetDevice(device);
        if (stream) cudaStreamSynchronize(stream);
        DevBuf* all[] = {&w, &m, &v, &grad, &wbf, &loss, &train_rec, &samples, &raw, &recs, &nee, &pts, &ctr};
        for (DevBuf* b : all) b->release();
        if (stream) cudaStreamDestroy(stream);
    }
    kz::GuideDev dev(const kz::DevScene* sc) const {
        kz::GuideDev g;
        g.wbf = static_cast<const __nv_bfloat16*>(wbf.ptr);
        g.wf = w.as<float>();
        g.band_scale = band_scale;
        if (sc) {
            g.box_lo = sc->box_lo;
            g.box_inv = sc->box_inv;
        }
        return g;
    }
};

namespace {

// He-uniform initial weights from a PCG32 stream (host), biases 0; the
// padded inputs of layer 1 stay zero.
void guide_init_params(uint64_t seed, std::vector<float>& p) {
    p.assign(KZ_GUIDE_PARAMS, 0.f);
    uint64_t state = 0, inc = (seed << 1u) | 1u;
    auto next = [&]() {
        uint64_t old = state;
        state = old * 6364136223846793005ULL + inc;
        uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u), rot = (uint32_t)(old >> 59u);
        return (xs >> rot) | (xs << ((32u - rot) & 31u));
    };
    next();
    state += 0x853c49e6748fea9bULL;
    next();
    const int offs[4] = {0, 64 * 64 + 64, 2 * (64 * 64 + 64), 3 * (64 * 64 + 64)};
    const int rows[4] = {64, 64, 64, 40};
    const int fan_in[4] = {51, 64, 64, 64};
    for (int l = 0; l < 4; ++l) {
        const float bound = (l < 3 ? std::sqrt(6.f / (float)fan_in[l]) : 0.5f * std::sqrt(3.f / (float)fan_in[l]));
        for (int o = 0; o < rows[l]; ++o)
            for (int i = 0; i < 64; ++i) {
                const float u = (float)(next() >> 8) * (1.0f / 16777216.0f);
                p[(size_t)offs[l] + o * 64 + i] = i < fan_in[l] ? (2.f * u - 1.f) * bound : 0.f;
            }
    }
}

kz_status guide_upload_params(kz_guide* g, const float* host) {
    KZ_CUDA(cudaMemcpyAsync(g->w.ptr, host, KZ_GUIDE_PARAMS * 4, cudaMemcpyHostToDevice, g->stream));
    kz::launch_guide_to_bf16(g->w.as<float>(), static_cast<__nv_bfloat16*>(g->wbf.ptr), g->stream);
    KZ_CUDA(cudaGetLastError());
    KZ_CUDA(cudaMemsetAsync(g->m.ptr, 0, KZ_GUIDE_PARAMS * 4, g->stream));
    KZ_CUDA(cudaMemsetAsync(g->v.ptr, 0, KZ_GUIDE_PARAMS * 4, g->stream));
    g->step = 0;
    KZ_CUDA(cudaStreamSynchronize(g->stream));
    return KZ_OK;
}

// One training batch on device samples: gradient into g->grad (zeroed
// first), loss into g->loss; Adam when apply.
kz_status guide_train_device(kz_guide* g, const float4* samples, uint32_t count, uint32_t rows, uint32_t stride,
                             uint32_t offset, float wscale, float wcap, float lr, bool apply, const kz::DevScene* sc,
                             cudaStream_t st) {
    if (kz::guide_train_mode() != 0) KZ_TRY(g->train_rec.ensure((size_t)rows * 496 * 2));  // split paths only
    KZ_CUDA(cudaMemsetAsync(g->grad.ptr, 0, KZ_GUIDE_PARAMS * 4, st));
    KZ_CUDA(cudaMemsetAsync(g->loss.ptr, 0, 4, st));  // the loss sum; the status word after it is sticky
    KZ_CUDA(kz::launch_guide_train(samples, count, rows, stride, offset, wscale, wcap, g->dev(sc),
                                   static_cast<__nv_bfloat16*>(g->train_rec.ptr), g->grad.as<float>(),
                                   g->loss.as<float>(), reinterpret_cast<uint32_t*>(g->loss.as<float>() + 1), st));
    KZ_CUDA(cudaGetLastError());
    if (apply) {
        g->step += 1;
        kz::launch_guide_adam(g->w.as<float>(), g->m.as<float>(), g->v.as<float>(), g->grad.as<float>(),
                              static_cast<__nv_bfloat16*>(g->wbf.ptr), lr, g->step, st);
        KZ_CUDA(cudaGetLastError());
    }
    return KZ_OK;
}

// The loss of the last training step and the weight-gradient kernel's
// status word (set when one of its waits ran out; cleared once reported).
kz_status guide_read_loss(kz_guide* g, float* loss, cudaStream_t st) {
    uint32_t h[2] = {0, 0};
    KZ_CUDA(cudaMemcpyAsync(h, g->loss.ptr, 8, cudaMemcpyDeviceToHost, st));
    KZ_CUDA(cudaStreamSynchronize(st));
    std::memcpy(loss, &h[0], 4);
    if (h[1]) {
        KZ_CUDA(cudaMemsetAsync(g->loss.as<float>() + 1, 0, 4, st));
        return fail((kz_status)h[1], "guiding weight-gradient kernel: a wait ran out (status %u)", h[1]);
    }
    return KZ_OK;
}

uint64_t gcd64(uint64_t a, uint64_t b) {
    while (b) {
        uint64_t t = a % b;
        a = b;
        b = t;
    }
    return a;
}

}  // namespace

extern "C" {

kz_status kz_guide_create(kz_guide** out, uint64_t seed) {
    if (!out) return fail(KZ_ERR_INVALID_ARG, "out_guide is NULL");
    *out = nullptr;
    if (kz_device_count() == 0) return fail(KZ_ERR_NO_DEVICE, "no CUDA device is visible");
    kz_guide* g = new kz_guide();
    auto bail = [&](kz_status st) {
        delete g;
        return st;
    };
    if (cudaGetDevice(&g->device) != cudaSuccess) return bail(fail(KZ_ERR_CUDA, "cudaGetDevice failed"));
    if (cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking) != cudaSuccess)
        return bail(fail(KZ_ERR_CUDA, "cudaStreamCreate failed"));
    cudaError_t e = kz::guide_kernel_setup();
    if (e != cudaSuccess) return bail(fail(KZ_ERR_CUDA, "guide kernel setup: %s", cudaGetErrorString(e)));
    kz_status st = KZ_OK;
    for (DevBuf* b : {&g->w, &g->m, &g->v, &g->grad})
        if (st == KZ_OK) st = b->ensure(KZ_GUIDE_PARAMS * 4);
    if (st == KZ_OK) st = g->wbf.ensure(KZ_GUIDE_PARAMS * 2);
    if (st == KZ_OK) st = g->loss.ensure(16);
    if (st == KZ_OK && cudaMemset(g->loss.ptr, 0, 16) != cudaSuccess) st = fail(KZ_ERR_CUDA, "cudaMemset failed");
    if (st == KZ_OK) st = g->ctr.ensure(16);
    if (st != KZ_OK) return bail(st);
    std::vector<float> p;
    guide_init_params(seed, p);
    st = guide_upload_params(g, p.data());
    if (st != KZ_OK) return bail(st);
    *out = g;
    return KZ_OK;
}

kz_status kz_guide_destroy(kz_guide* g) {
    delete g;
    return KZ_OK;
}

kz_status kz_guide_get_params(kz_guide* g, float* out) {
    if (!g || !out) return fail(KZ_ERR_INVALID_ARG, "NULL argument");
    std::lock_guard<std::mutex> lk(g->mu);
    KZ_CUDA(cudaSetDevice(g->device));
    KZ_CUDA(cudaMemcpyAsync(out, g->w.ptr, KZ_GUIDE_PARAMS * 4, cudaMemcpyDeviceToHost, g->stream));
    KZ_CUDA(cudaStreamSynchronize(g->stream));
    return KZ_OK;
}

kz_status kz_guide_get_state(kz_guide* g, float* out, uint32_t* out_step) {
    if (!g || !out) return fail(KZ_ERR_INVALID_ARG, "NULL argument");
    std::lock_guard<std::mutex> lk(g->mu);
    KZ_CUDA(cudaSetDevice(g->device));
    KZ_CUDA(cudaMemcpyAsync(out, g->w.ptr, KZ_GUIDE_PARAMS * 4, cudaMemcpyDeviceToHost, g->stream));
    KZ_CUDA(cudaMemcpyAsync(out + KZ_GUIDE_PARAMS, g->m.ptr, KZ_GUIDE_PARAMS * 4, cudaMemcpyDeviceToHost, g->stream));
    KZ_CUDA(cudaMemcpyAsync(out + 2 * KZ_GUIDE_PARAMS, g->v.ptr, KZ_GUIDE_PARAMS * 4, cudaMemcpyDeviceToHost,
                            g->stream));
    KZ_CUDA(cudaStreamSynchronize(g->stream));
    if (out_step) *out_step = (uint32_t)g->step;
    return KZ_OK;
}

kz_status kz_guide_set_state(kz_guide* g, const float* in, uint32_t step) {
    if (!g || !in) return fail(KZ_ERR_INVALID_ARG, "NULL argument");
    for (int i = 0; i < 3 * KZ_GUIDE_PARAMS; ++i)
        if (!std::isfinite(in[i])) return fail(KZ_ERR_INVALID_ARG, "state value %d is not finite", i);
    for (int i = 2 * KZ_GUIDE_PARAMS; i < 3 * KZ_GUIDE_PARAMS; ++i)
        if (in[i] < 0.f) return fail(KZ_ERR_INVALID_ARG, "second moment %d is negative", i - 2 * KZ_GUIDE_PARAMS);
    std::lock_guard<std::mutex> lk(g->mu);
    KZ_CUDA(cudaSetDevice(g->device));
    KZ_TRY(guide_upload_params(g, in));  // weights (and their BF16 copy); zeroes the moments
    KZ_CUDA(cudaMemcpyAsync(g->m.ptr, in + KZ_GUIDE_PARAMS, KZ_GUIDE_PARAMS * 4, cudaMemcpyHostToDevice, g->stream));
    KZ_CUDA(cudaMemcpyAsync(g->v.ptr, in + 2 * KZ_GUIDE_PARAMS, KZ_GUIDE_PARAMS * 4, cudaMemcpyHostToDevice,
                            g->stream));
    KZ_CUDA(cudaStreamSynchronize(g->stream));
    g->step = (int)step;
    return KZ_OK;
}

kz_status kz_guide_set_params(kz_guide* g, const float* in) {
    if (!g || !in) return fail(KZ_ERR_INVALID_ARG, "NULL argument");
    for (int i = 0; i < KZ_GUIDE_PARAMS; ++i)
        if (!std::isfinite(in[i])) return fail(KZ_ERR_INVALID_ARG, "parameter %d is not finite", i);
    std::lock_guard<std::mutex> lk(g->mu);
    KZ_CUDA(cudaSetDevice(g->device));
    return guide_upload_params(g, in);
}

kz_status kz_guide_forward(kz_guide* g, const float* points, uint64_t n, float* out_raw, int32_t mem) {
    const NvtxRange nvtx_range("kz_guide_forward");
    KZ_TRY(check_mem(mem));
    if (!g) return fail(KZ_ERR_INVALID_ARG, "guide is NULL");
    if (n == 0) return KZ_OK;
    if (!points || !out_raw) return fail(KZ_ERR_INVALID_ARG, "NULL argument");
    if (n > 0xffffffffull) return fail(KZ_ERR_INVALID_ARG, "too many points");
    std::lock_guard<std::mutex> lk(g->mu);
    KZ_CUDA(cudaSetDevice(g->device));
    cudaStream_t st = g->stream;
    const float4* dp = reinterpret_cast<const float4*>(points);
    float* dr = out_raw;
    if (mem == KZ_MEM_HOST) {
        KZ_TRY(g->pts.ensure(n * 32));
        KZ_TRY(g->raw.ensure(n * 160));
        KZ_CUDA(cudaMemcpyAsync(g->pts.ptr, points, n * 32, cudaMemcpyHostToDevice, st));
        dp = g->pts.as<float4>();
        dr = g->raw.as<float>();
    }
    kz::launch_guide_infer_points(dp, (uint32_t)n, g->dev(nullptr), dr, st);
    KZ_CUDA(cudaGetLastError());
    if (mem == KZ_MEM_HOST) KZ_CUDA(cudaMemcpyAsync(out_raw, dr, n * 160, cudaMemcpyDeviceToHost, st));
    KZ_CUDA(cudaStreamSynchronize(st));
    return KZ_OK;
}

kz_status kz_guide_train_step(kz_guide* g, const float* samples, uint64_t n, float lr, int32_t apply,
                              float* out_loss, float* out_grad, int32_t mem) {
    const NvtxRange nvtx_range("kz_guide_train_step");
    KZ_TRY(check_mem(mem));
    if (!g) return fail(KZ_ERR_INVALID_ARG, "guide is NULL");
    if (n == 0 || n > (1u << 20)) return fail(KZ_ERR_INVALID_ARG, "n must be in [1, 2^20]");
    if (!samples) return fail(KZ_ERR_INVALID_ARG, "samples is NULL");
    if (!(lr > 0.f) && apply) return fail(KZ_ERR_INVALID_ARG, "learning_rate must be > 0");
    std::lock_guard<std::mutex> lk(g->mu);
    KZ_CUDA(cudaSetDevice(g->device));
    cudaStream_t st = g->stream;
    const float4* ds = reinterpret_cast<const float4*>(samples);
    if (mem == KZ_MEM_HOST) {
        KZ_TRY(g->samples.ensure(n * 48));
        KZ_CUDA(cudaMemcpyAsync(g->samples.ptr, samples, n * 48, cudaMemcpyHostToDevice, st));
        ds = g->samples.as<float4>();
    }
    KZ_TRY(guide_train_device(g, ds, (uint32_t)n, (uint32_t)n, 1, 0, 1.0f / (float)n, 3.0e38f, lr, apply != 0,
                              nullptr, st));
    float loss = 0.f;
    if (out_grad) KZ_CUDA(cudaMemcpyAsync(out_grad, g->grad.ptr, KZ_GUIDE_PARAMS * 4, cudaMemcpyDeviceToHost, st));
    KZ_TRY(guide_read_loss(g, &loss, st));
    if (out_loss) *out_loss = loss;
    return KZ_OK;
}

kz_status kz_render_guided(kz_scene* s, kz_guide* g, const kz_camera* camera, const kz_film_desc* fd,
                           const kz_render_config* cfg, const kz_guide_config* gcfg_in, float* out_rgb,
                           double* out_rgb64, int32_t mem, kz_render_stats* out_stats, kz_guide_stats* out_gstats) {
    const NvtxRange nvtx_range("kz_render_guided");
    const auto t_start = std::chrono::steady_clock::now();
    KZ_TRY(check_mem(mem));
    if (!s || !g) return fail(KZ_ERR_INVALID_ARG, "scene and guide are required");
    std::lock_guard<std::mutex> lk(s->mu);
    std::lock_guard<std::mutex> lk2(g->mu);
    KZ_TRY(check_cfg(cfg));  // before the scene check: needs no device
    KZ_TRY(check_scene(s));
    if (cfg->max_depth > 16) return fail(KZ_ERR_INVALID_ARG, "guided rendering supports max_depth <= 16");
    if (cfg->flags & (KZ_RENDER_FLAG_NEE_ONLY | KZ_RENDER_FLAG_BSDF_ONLY))
        return fail(KZ_ERR_INVALID_ARG, "guided rendering combines the guide with the MIS estimator only");
    if (g->device != s->device) return fail(KZ_ERR_INVALID_ARG, "guide and scene live on different devices");
    if (!camera || !fd || !out_rgb) return fail(KZ_ERR_INVALID_ARG, "camera, film and out_rgb are required");
    if (fd->width == 0 || fd->height == 0) return fail(KZ_ERR_INVALID_ARG, "film size must be > 0");
    kz_guide_config gc = gcfg_in ? *gcfg_in : kz_guide_config{};
    if (gc.alpha == 0.f) gc.alpha = 0.5f;
    if (!(gc.alpha > 0.f && gc.alpha < 1.f)) return fail(KZ_ERR_INVALID_ARG, "alpha must be in (0, 1)");
    if (gc.learning_rate == 0.f) gc.learning_rate = 1e-2f;
    if (gc.spp_per_pass == 0) gc.spp_per_pass = 1;
    if (gc.max_train_samples == 0) gc.max_train_samples = 1u << 18;
    if (gc.steps_per_pass == 0) gc.steps_per_pass = 1;
    const uint64_t npix = (uint64_t)fd->width * fd->height;
    const uint64_t per_pass = npix * gc.spp_per_pass;
    if (per_pass > (1ull << 28)) return fail(KZ_ERR_INVALID_ARG, "width*height*spp_per_pass must be <= 2^28");
    const uint64_t max_pass_paths = std::max<uint64_t>(per_pass, 1ull << 24);
    kz::DevCamera cam;
    KZ_TRY(make_camera(camera, fd->width, fd->height, cam));
    cudaStream_t strm = s->stream;

    // buffers
    float* film = out_rgb;
    double* film64 = out_rgb64;
    if (mem == KZ_MEM_HOST) {
        KZ_TRY(s->film.ensure(npix * 12));
        film = s->film.as<float>();
        if (out_rgb64) {
            KZ_TRY(s->film64.ensure(npix * 24));
            film64 = s->film64.as<double>();
        }
    }
    KZ_CUDA(cudaMemsetAsync(film, 0, npix * 12, strm));
    if (film64) KZ_CUDA(cudaMemsetAsync(film64, 0, npix * 24, strm));
    const uint64_t want = cfg->wavefront_size ? cfg->wavefront_size : KZ_RENDER_DEFAULT_WAVEFRONT;
    const uint32_t cap = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(want, per_pass));
    const uint32_t block = cfg->block_size ? cfg->block_size : 256u;
    const uint64_t n_recs = per_pass * cfg->max_depth;
    KZ_TRY(g->recs.ensure(n_recs * sizeof(kz::VRec)));
    KZ_TRY(g->nee.ensure(n_recs * sizeof(kz::NRec)));
    KZ_TRY(g->samples.ensure(2 * n_recs * 48));
    KZ_TRY(g->raw.ensure((size_t)cap * 160));
    kz::VRec* recs = g->recs.as<kz::VRec>();
    kz::NRec* nee = g->nee.as<kz::NRec>();
    const kz::GuideDev gdev = g->dev(&s->dev);

    kz_render_stats st{};
    kz_guide_stats gs{};
    double train_ms = 0.0;
    uint64_t spp_done = 0;
    uint32_t pass = 0;
    while (spp_done < cfg->spp) {
        const bool train = gc.train && (gc.max_train_steps == 0 || gs.train_steps < gc.max_train_steps);
        // once the network is frozen, passes only bound the time budget's
        // granularity: render them larger (up to 64 spp, within the buffers)
        uint64_t want_spp = gc.spp_per_pass;
        if (!train) want_spp = std::max<uint64_t>(want_spp, std::min<uint64_t>(64, max_pass_paths / npix));
        const uint32_t spp_pass = (uint32_t)std::min<uint64_t>(want_spp, cfg->spp - spp_done);
        const uint64_t total = npix * spp_pass;
        kz::PathParams pp;
        pp.spp = spp_pass;
        pp.max_depth = cfg->max_depth;
        pp.rr_min = cfg->rr_min_depth;
        pp.seed = cfg->seed * 0x9E3779B97F4A7C15ull + pass + 1;  // a fresh PCG32 seed per pass
        pp.camera = 1;
        if (train) {
            KZ_CUDA(cudaMemsetAsync(recs, 0, total * cfg->max_depth * sizeof(kz::VRec), strm));
            KZ_CUDA(cudaMemsetAsync(nee, 0, total * cfg->max_depth * sizeof(kz::NRec), strm));
        }
        kz::GuideShade gsh;
        gsh.raw = g->raw.as<float>();
        gsh.recs = train ? recs : nullptr;
        gsh.nee = train ? nee : nullptr;
        gsh.pass_first = 0;
        gsh.alpha = gc.alpha;
        GuideHooks hooks;
        hooks.gs = &gsh;
        hooks.gd = gdev;
        hooks.raw = g->raw.as<float>();
        kz_render_config pcfg = *cfg;
        pcfg.spp = spp_pass;
        pcfg.wavefront_size = cap;
        kz_render_stats pst{};
        KZ_TRY(run_wavefront(s, &cam, nullptr, total, &pcfg, film, film64, &pst, &pp, &hooks));
        st.path_bounces += pst.path_bounces;
        st.shadow_rays += pst.shadow_rays;
        st.iterations += pst.iterations;
        st.kernel_launches += pst.kernel_launches;
        st.generate_ms += pst.generate_ms;
        st.trace_ms += pst.trace_ms;
        st.shade_ms += pst.shade_ms;
        st.shadow_ms += pst.shadow_ms;
        st.paths += total;
        spp_done += spp_pass;
        pass += 1;
        // training on this pass's radiance samples
        if (train) {
            const auto t0 = std::chrono::steady_clock::now();
            KZ_CUDA(cudaMemsetAsync(g->ctr.ptr, 0, 16, strm));
            uint32_t* cnt = g->ctr.as<uint32_t>();
            float* wsum = reinterpret_cast<float*>(cnt + 1);
            kz::launch_guide_collect(recs, nee, total * cfg->max_depth, g->samples.as<float4>(),
                                     (uint32_t)std::min<uint64_t>(2 * n_recs, 0xffffffffull), cnt, wsum, strm);
            uint32_t hc[2] = {0, 0};
            KZ_CUDA(cudaMemcpyAsync(hc, g->ctr.ptr, 8, cudaMemcpyDeviceToHost, strm));
            KZ_CUDA(cudaStreamSynchronize(strm));
            const uint32_t count = hc[0];
            float wsum_h;
            std::memcpy(&wsum_h, &hc[1], 4);
            gs.train_samples += count;
            if (count > 0 && wsum_h > 0.f && std::isfinite(wsum_h)) {
                const uint32_t rows = std::min(count, gc.max_train_samples);
                uint64_t stride = 2654435761ull % count;
                if (stride == 0) stride = 1;
                while (gcd64(stride, count) != 1) ++stride;
                // weights normalised so each step sees mean weight 1 over its rows
                const float wscale = (float)count / (wsum_h * (float)rows);
                for (uint32_t k = 0; k < gc.steps_per_pass; ++k) {
                    // outliers (rare paths through a narrow opening) would
                    // dominate a step: cap a sample at 20x the mean weight
                    KZ_TRY(guide_train_device(g, g->samples.as<float4>(), count, rows, (uint32_t)stride,
                                              (uint32_t)(((uint64_t)k * rows) % count), wscale, g->weight_cap / (float)rows,
                                              gc.learning_rate, true, &s->dev, strm));
                    gs.train_steps += 1;
                }
                float loss = 0.f;
                KZ_TRY(guide_read_loss(g, &loss, strm));
                gs.last_loss = loss;
            }
            train_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        }
        if (gc.time_budget_ms > 0.0) {
            const double el =
                std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
            if (el >= gc.time_budget_ms) break;
        }
    }
    kz::launch_scale(film, nullptr, npix * 3, 1.0f / (float)spp_done, 0.0, strm);
    if (film64) kz::launch_scale(nullptr, film64, npix * 3, 0.f, 1.0 / (double)spp_done, strm);
    KZ_CUDA(cudaGetLastError());
    if (mem == KZ_MEM_HOST) {
        KZ_CUDA(cudaMemcpyAsync(out_rgb, film, npix * 12, cudaMemcpyDeviceToHost, strm));
        if (out_rgb64) KZ_CUDA(cudaMemcpyAsync(out_rgb64, film64, npix * 24, cudaMemcpyDeviceToHost, strm));
    }
    KZ_CUDA(cudaStreamSynchronize(strm));
    gs.passes = pass;
    gs.spp_done = spp_done;
    gs.train_ms = train_ms;
    gs.wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
    if (out_stats) *out_stats = st;
    if (out_gstats) *out_gstats = gs;
    return KZ_OK;
}

}  // extern "C"


// ---------------------------------------------------------------------------
// Batched rendering: one persistent launch over many jobs.
extern "C" kz_status kz_scene_release_scratch(kz_scene* s) {
    if (!s) return fail(KZ_ERR_INVALID_ARG, "scene is NULL");
    std::lock_guard<std::mutex> lk(s->mu);
    if (!s->cuda_ready) return KZ_OK;
    KZ_CUDA(cudaSetDevice(s->device));
    KZ_CUDA(cudaStreamSynchronize(s->stream));
    DevBuf* all[] = {&s->s_rays, &s->s_t, &s->s_prim, &s->s_geom, &s->s_u, &s->s_v, &s->s_occ, &s->s_ctr, &s->s_next,
                     &s->film, &s->film64};
    for (DevBuf* b : all) b->release();
    for (auto& b : s->pa) b.release();
    for (auto& b : s->pb) b.release();
    for (auto& b : s->sh) b.release();
    return KZ_OK;
}

namespace {

// Wavefront mode of kz_render_batch: the device-driven loop of run_wavefront
// over all jobs at once, on the first job's scene stream and scratch. One
// batch of iterations (plan, generate, trace, shade, shadow, finish) is
// enqueued, or replayed as a captured graph, between host synchronisations.
kz_status batch_wavefront(const kz_batch_job* jobs, uint32_t n_jobs, const kz_batch_config& cfg, int32_t mem,
                          const kz::DevJob* djobs, const std::vector<float*>& fptr, const std::vector<uint64_t>& npix,
                          uint64_t total, kz_batch_stats* out_stats) {
    kz_scene* s = jobs[0].scene;
    cudaStream_t strm = s->stream;
    const uint64_t want = cfg.wavefront_size ? cfg.wavefront_size : KZ_RENDER_DEFAULT_WAVEFRONT;
    const uint32_t cap = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(std::min<uint64_t>(want, total), 1u << 30));
    const uint32_t block = cfg.block_size;
    uint32_t max_depth = 1;
    for (uint32_t j = 0; j < n_jobs; ++j) max_depth = std::max(max_depth, jobs[j].max_depth);
    kz::PathSoA A, B;
    KZ_TRY(alloc_paths(s->pa, cap, A));
    KZ_TRY(alloc_paths(s->pb, cap, B));
    for (int k = 0; k < 3; ++k) KZ_TRY(s->sh[k].ensure((size_t)cap * sizeof(float4)));
    kz::ShadowSoA sq{s->sh[0].as<float4>(), s->sh[1].as<float4>(), s->sh[2].as<float4>()};
    KZ_TRY(s->ctr.ensure(sizeof(kz::DevCounters)));
    kz::DevCounters* ctr = s->ctr.as<kz::DevCounters>();
    for (uint32_t j = 0; j < n_jobs; ++j) KZ_CUDA(cudaMemsetAsync(fptr[j], 0, npix[j] * 12, strm));
    {
        kz::DevCounters init{};
        init.total = total;
        *s->ctr_host = init;
        KZ_CUDA(cudaMemcpyAsync(ctr, s->ctr_host, sizeof(kz::DevCounters), cudaMemcpyHostToDevice, strm));
    }
    // an even number of iterations per batch, so the path buffers end where
    // they started and a captured batch can be replayed as is
    uint32_t iters = std::max<uint32_t>(4, max_depth + 1);
    iters += iters & 1u;
    bool textured = false;  // the texture tint is compiled out unless a job needs it
    for (uint32_t j = 0; j < n_jobs; ++j)
        textured |= jobs[j].scene->dev.mat_tex != nullptr || jobs[j].scene->dev.tri_nrm != nullptr;
    // refill period P: free wavefront slots take new paths every P-th
    // iteration (P = 1: every iteration); in between the wavefront drains, so
    // the generation launches are fewer and the live paths fewer too
    const uint32_t period = std::max<uint32_t>(1, cfg.refill_period);
    if (iters % period) iters += period - iters % period;
    iters += iters & 1u;
    auto enqueue = [&]() {
        kz::PathSoA a = A, b = B;
        for (uint32_t it = 0; it < iters; ++it) {
            const bool gen = it % period == 0;
            kz::launch_plan(ctr, cap, strm, gen);
            if (gen) kz::launch_generate_batch_dev(djobs, n_jobs, a, ctr, cap, block, strm);
            kz::launch_trace_paths_batch(djobs, a, cap, ctr, strm);
            kz::launch_shade_batch(djobs, a, cap, b, sq, ctr, block, textured, strm);
            kz::launch_trace_shadow_batch(djobs, sq, cap, ctr, strm);
            kz::launch_finish(ctr, strm);
            std::swap(a, b);
        }
    };
    const bool persistent = cfg.mode == KZ_BATCH_PERSISTENT;
    uint32_t coop_blocks = 0;
    if (persistent) {
        int sms = 0;
        KZ_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device));
        const int per_sm = kz::batch_persistent_blocks_per_sm(textured);
        if (per_sm <= 0) return fail(KZ_ERR_CUDA, "the persistent batch kernel does not fit on an SM");
        coop_blocks = (uint32_t)sms * (uint32_t)per_sm;
    }
    // the persistent mode's one launch runs the whole loop
    auto enqueue_persistent = [&]() -> cudaError_t {
        return kz::launch_batch_persistent(djobs, n_jobs, A, B, sq, ctr, cap, period, coop_blocks, textured, strm);
    };
    kz::prepare_batch_wavefront();
    cudaGraphExec_t exec = nullptr;
    struct ExecGuard {
        cudaGraphExec_t& e;
        ~ExecGuard() {
            if (e) cudaGraphExecDestroy(e);
        }
    } xg{exec};
    if (cfg.use_graph) {
        cudaGraph_t graph = nullptr;
        KZ_CUDA(cudaStreamBeginCapture(strm, cudaStreamCaptureModeThreadLocal));
        cudaError_t le = cudaSuccess;
        if (persistent) le = enqueue_persistent();
        else enqueue();
        cudaError_t ce = cudaStreamEndCapture(strm, &graph);
        if (le != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            return fail(KZ_ERR_CUDA, "persistent batch launch (capture): %s", cudaGetErrorString(le));
        }
        if (ce != cudaSuccess) return fail(KZ_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
        ce = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ce != cudaSuccess) return fail(KZ_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ce));
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    KZ_CUDA(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return fail(KZ_ERR_CUDA, "cudaEventCreate failed");
    }
    struct Ev {
        cudaEvent_t a, b;
        ~Ev() {
            cudaEventDestroy(a);
            cudaEventDestroy(b);
        }
    } evg{e0, e1};
    KZ_CUDA(cudaEventRecord(e0, strm));
    for (;;) {
        if (exec) KZ_CUDA(cudaGraphLaunch(exec, strm));
        else if (persistent) KZ_CUDA(enqueue_persistent());
        else enqueue();
        KZ_CUDA(cudaGetLastError());
        KZ_CUDA(cudaMemcpyAsync(s->ctr_host, ctr, sizeof(kz::DevCounters), cudaMemcpyDeviceToHost, strm));
        KZ_CUDA(cudaStreamSynchronize(strm));
        const kz::DevCounters& hc = *s->ctr_host;
        if (hc.status) return fail((kz_status)hc.status, "device status %u during batched rendering", hc.status);
        if (hc.n_active == 0 && hc.next_path >= hc.total) break;
        if (persistent) return fail(KZ_ERR_CUDA, "persistent batch kernel ended with paths left");
    }
    for (uint32_t j = 0; j < n_jobs; ++j)
        kz::launch_scale(fptr[j], nullptr, npix[j] * 3, 1.0f / (float)jobs[j].spp, 0.0, strm);
    KZ_CUDA(cudaEventRecord(e1, strm));
    if (mem == KZ_MEM_HOST)
        for (uint32_t j = 0; j < n_jobs; ++j)
            KZ_CUDA(cudaMemcpyAsync(jobs[j].out_rgb, fptr[j], npix[j] * 12, cudaMemcpyDeviceToHost, strm));
    KZ_CUDA(cudaStreamSynchronize(strm));
    float ms = 0.f;
    KZ_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    if (out_stats) {
        const kz::DevCounters& hc = *s->ctr_host;
        out_stats->paths = total;
        out_stats->path_bounces = hc.path_bounces;
        out_stats->shadow_rays = hc.shadow_rays;
        out_stats->threads = cap;
        out_stats->device_ms = ms;
    }
    return KZ_OK;
}

}  // namespace

extern "C" kz_status kz_render_batch(const kz_batch_job* jobs, uint32_t n_jobs, const kz_batch_config* cfg_in,
                                     int32_t mem, kz_batch_stats* out_stats) {
    const NvtxRange nvtx_range("kz_render_batch");
    KZ_TRY(check_mem(mem));
    if (n_jobs == 0) return KZ_OK;
    if (!jobs) return fail(KZ_ERR_INVALID_ARG, "jobs is NULL");
    kz_batch_config cfg = cfg_in ? *cfg_in : kz_batch_config{};
    if (cfg.mode != KZ_BATCH_WAVEFRONT && cfg.mode != KZ_BATCH_MEGAKERNEL && cfg.mode != KZ_BATCH_PERSISTENT)
        return fail(KZ_ERR_INVALID_ARG, "unknown batch mode %u", cfg.mode);
    const bool wavefront = cfg.mode != KZ_BATCH_MEGAKERNEL;  // the persistent mode runs the wavefront's stages
    if (cfg.block_size == 0) cfg.block_size = wavefront ? 256 : 128;
    if (cfg.ctas_per_sm == 0) cfg.ctas_per_sm = 2;
    if (cfg.refill_period == 0) cfg.refill_period = 1;
    if (cfg.block_size % 32 != 0 || cfg.block_size > 256)
        return fail(KZ_ERR_INVALID_ARG, "block_size must be a multiple of 32 and <= 256");
    if (cfg.ctas_per_sm > 64) return fail(KZ_ERR_INVALID_ARG, "ctas_per_sm must be <= 64");
    if (wavefront && n_jobs > kz::kMaxBatchJobs)
        return fail(KZ_ERR_INVALID_ARG, "at most %u jobs per wavefront batch", kz::kMaxBatchJobs);
    // lock every distinct scene once, in address order
    std::vector<kz_scene*> scenes;
    for (uint32_t j = 0; j < n_jobs; ++j) {
        if (!jobs[j].scene) return fail(KZ_ERR_INVALID_ARG, "job %u has no scene", j);
        scenes.push_back(jobs[j].scene);
    }
    std::sort(scenes.begin(), scenes.end());
    scenes.erase(std::unique(scenes.begin(), scenes.end()), scenes.end());
    std::vector<std::unique_lock<std::mutex>> locks;
    for (kz_scene* sc : scenes) locks.emplace_back(sc->mu);
    for (kz_scene* sc : scenes) {
        KZ_TRY(check_scene(sc));
        if (sc->device != scenes[0]->device) return fail(KZ_ERR_INVALID_ARG, "scenes live on different devices");
    }
    kz_scene* s0 = jobs[0].scene;
    KZ_CUDA(cudaSetDevice(s0->device));
    cudaStream_t st = s0->stream;

    std::vector<kz::DevJob> dj(n_jobs);
    std::vector<uint64_t> npix(n_jobs);
    uint64_t total = 0, film_floats = 0;
    for (uint32_t j = 0; j < n_jobs; ++j) {
        const kz_batch_job& J = jobs[j];
        if (J.width == 0 || J.height == 0 || J.spp == 0) return fail(KZ_ERR_INVALID_ARG, "job %u: empty film or spp", j);
        if (J.max_depth == 0 || J.max_depth > 255) return fail(KZ_ERR_INVALID_ARG, "job %u: max_depth in [1, 255]", j);
        if (!J.out_rgb) return fail(KZ_ERR_INVALID_ARG, "job %u: out_rgb is NULL", j);
        npix[j] = (uint64_t)J.width * J.height;
        const uint64_t paths = npix[j] * J.spp;
        if (paths > 0xffffffffull) return fail(KZ_ERR_INVALID_ARG, "job %u: width*height*spp must be < 2^32", j);
        kz::DevJob& d = dj[j];
        d.scene = J.scene->dev;
        KZ_TRY(make_camera(&J.camera, J.width, J.height, d.cam));
        d.pp.spp = J.spp;
        d.pp.max_depth = J.max_depth;
        d.pp.rr_min = J.rr_min_depth;
        d.pp.seed = J.seed;
        d.pp.camera = 1;
        d.path_begin = total;
        total += paths;
        film_floats += npix[j] * 3;
    }
    // device films (the caller's when they are device pointers)
    DevBuf films, djobs, ctrs;
    std::vector<float*> fptr(n_jobs);
    if (mem == KZ_MEM_HOST) {
        KZ_TRY(films.ensure(film_floats * 4));
        uint64_t off = 0;
        for (uint32_t j = 0; j < n_jobs; ++j) {
            fptr[j] = films.as<float>() + off;
            off += npix[j] * 3;
        }
    } else {
        for (uint32_t j = 0; j < n_jobs; ++j) fptr[j] = jobs[j].out_rgb;
    }
    for (uint32_t j = 0; j < n_jobs; ++j) dj[j].film = fptr[j];
    KZ_TRY(djobs.ensure(n_jobs * sizeof(kz::DevJob)));
    KZ_TRY(ctrs.ensure(sizeof(kz::BatchCounters)));
    KZ_CUDA(cudaMemcpyAsync(djobs.ptr, dj.data(), n_jobs * sizeof(kz::DevJob), cudaMemcpyHostToDevice, st));
    if (wavefront) return batch_wavefront(jobs, n_jobs, cfg, mem, djobs.as<kz::DevJob>(), fptr, npix, total, out_stats);
    int sms = 0;
    KZ_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s0->device));
    const uint32_t ctas = (uint32_t)sms * cfg.ctas_per_sm;
    kz::BatchCounters* bc = ctrs.as<kz::BatchCounters>();

    auto enqueue = [&]() -> kz_status {
        KZ_CUDA(cudaMemsetAsync(bc, 0, sizeof(kz::BatchCounters), st));
        for (uint32_t j = 0; j < n_jobs; ++j) KZ_CUDA(cudaMemsetAsync(fptr[j], 0, npix[j] * 12, st));
        kz::launch_render_batch(djobs.as<kz::DevJob>(), n_jobs, total, bc, cfg.refill_period, ctas, cfg.block_size,
                                st);
        for (uint32_t j = 0; j < n_jobs; ++j)
            kz::launch_scale(fptr[j], nullptr, npix[j] * 3, 1.0f / (float)jobs[j].spp, 0.0, st);
        return KZ_OK;
    };
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    KZ_CUDA(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return fail(KZ_ERR_CUDA, "cudaEventCreate failed");
    }
    struct Ev {
        cudaEvent_t a, b;
        ~Ev() {
            cudaEventDestroy(a);
            cudaEventDestroy(b);
        }
    } evg{e0, e1};
    if (cfg.use_graph) {
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        KZ_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        kz_status est = enqueue();
        cudaError_t ce = cudaStreamEndCapture(st, &graph);
        if (est != KZ_OK) {
            if (graph) cudaGraphDestroy(graph);
            return est;
        }
        if (ce != cudaSuccess) return fail(KZ_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
        ce = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ce != cudaSuccess) return fail(KZ_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ce));
        KZ_CUDA(cudaEventRecord(e0, st));
        ce = cudaGraphLaunch(exec, st);
        if (ce == cudaSuccess) ce = cudaEventRecord(e1, st);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
        cudaGraphExecDestroy(exec);
        if (ce != cudaSuccess) return fail(KZ_ERR_CUDA, "graph launch: %s", cudaGetErrorString(ce));
    } else {
        KZ_CUDA(cudaEventRecord(e0, st));
        KZ_TRY(enqueue());
        KZ_CUDA(cudaEventRecord(e1, st));
        KZ_CUDA(cudaStreamSynchronize(st));
    }
    KZ_CUDA(cudaGetLastError());
    kz::BatchCounters hb;
    KZ_CUDA(cudaMemcpyAsync(&hb, bc, sizeof(hb), cudaMemcpyDeviceToHost, st));
    if (mem == KZ_MEM_HOST)
        for (uint32_t j = 0; j < n_jobs; ++j)
            KZ_CUDA(cudaMemcpyAsync(jobs[j].out_rgb, fptr[j], npix[j] * 12, cudaMemcpyDeviceToHost, st));
    KZ_CUDA(cudaStreamSynchronize(st));
    if (hb.status) return fail((kz_status)hb.status, "device status %u during batched rendering", hb.status);
    float ms = 0.f;
    KZ_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    if (out_stats) {
        out_stats->paths = total;
        out_stats->path_bounces = hb.path_bounces;
        out_stats->shadow_rays = hb.shadow_rays;
        out_stats->threads = (uint64_t)ctas * cfg.block_size;
        out_stats->device_ms = ms;
    }
    return KZ_OK;
}

// ---------------------------------------------------------------------------
// kz_li_batch_noalloc: the wavefront Li batch with its scratch in a static
// device array instead of cudaMalloc'd buffers. Layout of the array for a
// capacity of C paths: ping-pong path state A and B (four float4 arrays and
// one 64-bit RNG array each), the shadow queue (three float4 arrays), then the
// device counters. Every region starts on a 256-byte boundary.
namespace {

constexpr size_t kNoAllocCap = KZ_LI_NOALLOC_MAX_WAVEFRONT;
constexpr size_t kNoAllocPathBytes = kNoAllocCap * (4 * sizeof(float4) + sizeof(unsigned long long));
constexpr size_t kNoAllocShadowBytes = kNoAllocCap * 3 * sizeof(float4);
constexpr size_t kNoAllocCounterOffset = 2 * kNoAllocPathBytes + kNoAllocShadowBytes;
constexpr size_t kNoAllocBytes = kNoAllocCounterOffset + ((sizeof(kz::DevCounters) + 255) / 256) * 256;
static_assert(kNoAllocCap % 64 == 0, "regions must stay 256-byte aligned");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
struct NoAllocSlot {
    void* addr = nullptr;
    unsigned long long ctx_id = 0;  // cuCtxGetId of the context the address belongs to
};
NoAllocSlot g_noalloc[kNoAllocMaxDevices];

// Unique id of the calling thread's current context (cuCtxGetId), through the
// runtime's driver entry-point lookup so the library does not link libcuda.
// A context that is destroyed and created again (cudaDeviceReset) gets a new
// id, and the module holding the array is loaded again at a new address.
kz_status current_context_id(unsigned long long* id) {
    typedef int (*GetCurrentFn)(void**);
    typedef int (*GetIdFn)(void*, unsigned long long*);
    static GetCurrentFn get_current = nullptr;
    static GetIdFn get_id = nullptr;
    if (!get_current || !get_id) {
        void* a = nullptr;
        void* b = nullptr;
        cudaDriverEntryPointQueryResult qa, qb;
        cudaError_t ea = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa);
        cudaError_t eb = cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb);
        if (ea != cudaSuccess || eb != cudaSuccess || qa != cudaDriverEntryPointSuccess ||
            qb != cudaDriverEntryPointSuccess || !a || !b)
            return fail(KZ_ERR_CUDA, "driver entry points cuCtxGetCurrent/cuCtxGetId are unavailable");
        get_current = reinterpret_cast<GetCurrentFn>(a);
        get_id = reinterpret_cast<GetIdFn>(b);
    }
    void* ctx = nullptr;
    if (get_current(&ctx) != 0 || !ctx) return fail(KZ_ERR_CUDA, "no current CUDA context");
    if (get_id(ctx, id) != 0) return fail(KZ_ERR_CUDA, "cuCtxGetId failed");
    return KZ_OK;
}

// Device address of g_noalloc_scratch on `device` (which must be current):
// looked up on the first call per device, and again whenever the device's
// context has changed since (after a cudaDeviceReset the array lives at a new
// address). In host code the symbol is only a host-side stand-in, never a
// device address.
kz_status noalloc_scratch(int device, unsigned char** out) {
    if (device < 0 || device >= kNoAllocMaxDevices)
        return fail(KZ_ERR_INVALID_ARG, "device %d is beyond the %d devices the scratch table covers", device,
                    kNoAllocMaxDevices);
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    unsigned long long ctx_id = 0;
    KZ_TRY(current_context_id(&ctx_id));
    NoAllocSlot& slot = g_noalloc[device];
    if (!slot.addr || slot.ctx_id != ctx_id) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail(KZ_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
        slot.addr = p;
        slot.ctx_id = ctx_id;
    }
    *out = static_cast<unsigned char*>(slot.addr);
    return KZ_OK;
}

kz::PathSoA carve_paths(unsigned char* base) {
    kz::PathSoA p;
    p.o4 = reinterpret_cast<float4*>(base);
    p.d4 = p.o4 + kNoAllocCap;
    p.b4 = p.d4 + kNoAllocCap;
    p.hit = p.b4 + kNoAllocCap;
    p.rng = reinterpret_cast<unsigned long long*>(p.hit + kNoAllocCap);
    return p;
}

}  // namespace

extern "C" kz_status kz_li_batch_noalloc(kz_scene* s, const kz_ray* rays, uint64_t n, const kz_render_config* cfg,
                                         float* out_rgb, kz_render_stats* out_stats) {
    const NvtxRange nvtx_range("kz_li_batch_noalloc");
    if (!s) return fail(KZ_ERR_INVALID_ARG, "scene is NULL");
    std::lock_guard<std::mutex> lk(s->mu);
    KZ_TRY(check_cfg(cfg));  // before the scene check: needs no device
    KZ_TRY(check_scene(s));
    if (cfg->wavefront_size > KZ_LI_NOALLOC_MAX_WAVEFRONT)
        return fail(KZ_ERR_INVALID_ARG, "wavefront_size %u exceeds the no-allocation maximum of %u paths",
                    cfg->wavefront_size, KZ_LI_NOALLOC_MAX_WAVEFRONT);
    if (n > 0xffffffffull) return fail(KZ_ERR_INVALID_ARG, "at most 2^32-1 rays per call");
    if (out_stats) *out_stats = kz_render_stats{};
    if (n == 0) return KZ_OK;
    if (!rays || !out_rgb) return fail(KZ_ERR_INVALID_ARG, "rays and out_rgb are required");

    unsigned char* base = nullptr;
    KZ_TRY(noalloc_scratch(s->device, &base));
    kz::PathSoA A = carve_paths(base);
    kz::PathSoA B = carve_paths(base + kNoAllocPathBytes);
    float4* sh = reinterpret_cast<float4*>(base + 2 * kNoAllocPathBytes);
    kz::ShadowSoA sq{sh, sh + kNoAllocCap, sh + 2 * kNoAllocCap};
    kz::DevCounters* ctr = reinterpret_cast<kz::DevCounters*>(base + kNoAllocCounterOffset);

    kz::PathParams pp;
    pp.spp = 1;
    pp.max_depth = cfg->max_depth;
    pp.rr_min = cfg->rr_min_depth;
    pp.seed = cfg->seed;
    pp.camera = 0;
    pp.estimator = (cfg->flags & KZ_RENDER_FLAG_NEE_ONLY) ? 1u : (cfg->flags & KZ_RENDER_FLAG_BSDF_ONLY) ? 2u : 0u;
    const uint32_t cap = (uint32_t)std::min<uint64_t>(cfg->wavefront_size ? cfg->wavefront_size : kNoAllocCap, n);
    const uint32_t block = cfg->block_size ? cfg->block_size : 256u;
    const bool count = (cfg->flags & KZ_RENDER_FLAG_COUNT) != 0;
    cudaStream_t strm = s->stream;

    // the array keeps the previous call's contents: clear the counters and
    // the output this call accumulates into
    KZ_CUDA(cudaMemsetAsync(ctr, 0, sizeof(kz::DevCounters), strm));
    KZ_CUDA(cudaMemsetAsync(out_rgb, 0, n * 3 * sizeof(float), strm));
    kz_render_stats st{};
    st.paths = n;
    kz::DevCounters hc;
    uint64_t next = 0;
    uint32_t nA = 0;
    for (;;) {
        const uint32_t n_new = (uint32_t)std::min<uint64_t>(cap - nA, n - next);
        if (n_new) {
            kz::launch_generate_rays(rays, pp, A, nA, next, n_new, block, strm);
            st.kernel_launches += 1;
            nA += n_new;
            next += n_new;
        }
        if (nA == 0) break;
        kz::launch_trace_paths(s->dev, A, nA, ctr, count, block, strm);
        KZ_CUDA(cudaMemsetAsync(ctr, 0, 2 * sizeof(uint32_t), strm));
        kz::launch_shade(s->dev, pp, A, nA, B, sq, ctr, out_rgb, nullptr, block, strm);
        kz::launch_trace_shadow(s->dev, sq, nA, ctr, count, out_rgb, nullptr, block, strm);
        st.kernel_launches += 3;
        KZ_CUDA(cudaMemcpyAsync(&hc, ctr, sizeof(hc), cudaMemcpyDeviceToHost, strm));
        KZ_CUDA(cudaStreamSynchronize(strm));
        KZ_CUDA(cudaGetLastError());
        st.path_bounces += nA;
        st.shadow_rays += hc.n_shadow;
        st.iterations += 1;
        if (hc.status) return fail((kz_status)hc.status, "device status %u during Li batch", hc.status);
        nA = hc.n_next;
        std::swap(A, B);
    }
    if (count) {
        st.closest_node_fetches = hc.fetch[0];
        st.closest_tri_fetches = hc.fetch[1];
        st.shadow_node_fetches = hc.fetch[2];
        st.shadow_tri_fetches = hc.fetch[3];
    }
    if (out_stats) *out_stats = st;
    return KZ_OK;
}
