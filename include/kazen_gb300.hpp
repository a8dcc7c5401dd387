// kazen_gb300.hpp — header-only C++ adapter over the C ABI, shaped like the
// kazen_proto interfaces it replaces:
//   kz::GpuAccel      ~ Accelerator / HitableInterface (src/core/accel.h:13-41,
//                       src/core/hitable.h:10-37): intersect(Ray, Intersection&),
//                       intersect(Ray, float&), occluded(...); batch forms too.
//   kz::PathIntegrator ~ Integrator::setup / Li (src/core/integrator.h:23-39).
// Single-ray calls are batches of one (API parity); render with the batch
// forms. Errors throw kz::Error with the library's status and message.
#pragma once

#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "kazen_gb300.h"

namespace kz {

class Error : public std::runtime_error {
public:
    Error(kz_status code, const char* msg) : std::runtime_error(std::string("kazen: ") + (msg ? msg : "")), code(code) {}
    kz_status code;
};

inline void check(kz_status st) {
    if (st != KZ_OK) throw Error(st, kz_last_error_string());
}

// Ray with the reference's defaults (src/core/ray.h:12-22): the direction is
// normalised on construction, tmin = 1e-4, tmax = +inf.
inline kz_ray make_ray(const float o[3], const float d[3], float tmin = 1e-4f, float tmax = INFINITY) {
    const float l = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    return kz_ray{o[0], o[1], o[2], tmin, d[0] / l, d[1] / l, d[2] / l, tmax};
}

// Hit record: the fields of the reference Intersection that the traversal
// determines (src/core/intersection.h:24-70).
struct Intersection {
    float t = 0.f;
    uint32_t prim_id = KZ_INVALID_ID;
    uint32_t geom_id = KZ_INVALID_ID;
    float u = 0.f, v = 0.f;
    float P[3] = {0.f, 0.f, 0.f};
};

class Scene {
public:
    Scene() { check(kz_scene_create(&h_)); }
    ~Scene() { kz_scene_destroy(h_); }
    Scene(const Scene&) = delete;
    Scene& operator=(const Scene&) = delete;

    // Scene::add_mesh (src/core/scene.h:144-160); returns the geom id.
    int32_t add_mesh(const std::vector<float>& xyz, const std::vector<uint32_t>& idx, int32_t material_id,
                     bool is_light = false, const float* xform12 = nullptr) {
        int32_t gid = -1;
        check(kz_scene_add_mesh(h_, xyz.data(), (uint32_t)(xyz.size() / 3), idx.data(), (uint32_t)(idx.size() / 3),
                                xform12, material_id, is_light ? 1 : 0, &gid));
        return gid;
    }
    void set_materials(const std::vector<kz_material>& m) { check(kz_scene_set_materials(h_, m.data(), (uint32_t)m.size())); }
    // Per-vertex normals / texture coordinates of a mesh (TriangleMesh norms / uvs, src/core/shape.h)
    void set_mesh_normals(int32_t gid, const std::vector<float>& n) {
        check(kz_scene_set_mesh_normals(h_, gid, n.data(), (uint32_t)(n.size() / 3)));
    }
    void set_mesh_uvs(int32_t gid, const std::vector<float>& uv) {
        check(kz_scene_set_mesh_uvs(h_, gid, uv.data(), (uint32_t)(uv.size() / 2)));
    }
    void set_textures(const std::vector<kz_texture>& t) { check(kz_scene_set_textures(h_, t.data(), (uint32_t)t.size())); }
    void set_environment(const float rgb[3], int32_t texture = -1) { check(kz_scene_set_environment(h_, rgb, texture)); }
    // PointLight(position, radiance) (src/core/light.h:51-71); returns its index among the point lights
    int32_t add_point_light(const float position[3], const float radiance[3]) {
        int32_t id = -1;
        check(kz_scene_add_point_light(h_, position, radiance, &id));
        return id;
    }
    // Scene::build_bvh / Accelerator::build
    void build_bvh() { check(kz_scene_build(h_)); }
    kz_scene* handle() const { return h_; }

private:
    kz_scene* h_ = nullptr;
};

class GpuAccel {
public:
    explicit GpuAccel(Scene& s) : s_(s.handle()) {}

    // Closest hits of a batch (host memory).
    void intersect(const std::vector<kz_ray>& rays, std::vector<Intersection>& out) const {
        const size_t n = rays.size();
        std::vector<float> t(n), u(n), v(n);
        std::vector<uint32_t> prim(n), geom(n);
        kz_hits h{t.data(), prim.data(), geom.data(), u.data(), v.data()};
        check(kz_intersect_closest(s_, rays.data(), n, h, KZ_MEM_HOST));
        out.resize(n);
        for (size_t i = 0; i < n; ++i) {
            Intersection& it = out[i];
            it.t = t[i];
            it.prim_id = prim[i];
            it.geom_id = geom[i];
            it.u = u[i];
            it.v = v[i];
            for (int k = 0; k < 3; ++k) it.P[k] = (&rays[i].ox)[k] + t[i] * (&rays[i].dx)[k];
        }
    }
    // HitableInterface::intersect(const Ray&, Intersection&)
    bool intersect(const kz_ray& r, Intersection& isect) const {
        std::vector<Intersection> out;
        intersect(std::vector<kz_ray>{r}, out);
        isect = out[0];
        return isect.prim_id != KZ_INVALID_ID;
    }
    // HitableInterface::intersect(const Ray&, float& t)
    bool intersect(const kz_ray& r, float& t) const {
        Intersection it;
        const bool hit = intersect(r, it);
        t = it.t;
        return hit;
    }
    // HitableInterface::occluded: any hit in (tmin, tmax]
    std::vector<uint8_t> occluded(const std::vector<kz_ray>& rays) const {
        std::vector<uint8_t> occ(rays.size());
        check(kz_intersect_any(s_, rays.data(), rays.size(), occ.data(), KZ_MEM_HOST));
        return occ;
    }
    bool occluded(const kz_ray& r) const { return occluded(std::vector<kz_ray>{r})[0] != 0; }

private:
    kz_scene* s_;
};

class PathIntegrator {
public:
    explicit PathIntegrator(uint32_t max_depth = 5, uint64_t seed = 0, uint32_t rr_min_depth = 3) {
        cfg_ = kz_render_config{1, max_depth, seed, 0, rr_min_depth, 0, 0};
    }
    // Integrator::setup(Scene*)
    void setup(Scene& s) { s_ = s.handle(); }
    // Integrator::Li for a batch of camera rays; ray i uses PCG32 stream (seed, i).
    std::vector<float> Li(const std::vector<kz_ray>& rays) const {
        std::vector<float> rgb(rays.size() * 3);
        check(kz_li_batch(s_, rays.data(), rays.size(), &cfg_, rgb.data(), KZ_MEM_HOST, nullptr));
        return rgb;
    }

private:
    kz_scene* s_ = nullptr;
    kz_render_config cfg_;
};

}  // namespace kz
