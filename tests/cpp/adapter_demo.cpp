// Uses include/kazen_gb300.hpp the way kazen_proto's C++ would: build a
// scene, query the reference's single-triangle hit
// (tests/libusage_tests/embree_tests.cpp:19-76), then Li of a few rays.
#include <cstdio>

#include "../../include/kazen_gb300.hpp"

int main() {
    if (kz_device_count() == 0) {
        std::printf("no-device\n");
        return 0;
    }
    kz::Scene scene;
    scene.add_mesh({-1, 0, 1, 2, 0, 1, -1, 0, -2}, {0, 1, 2}, 0);
    kz_material m{};
    m.n_lobes = 1;
    m.lobes[0].closure_id = KZ_CLOSURE_DIFFUSE;
    m.lobes[0].weight[0] = m.lobes[0].weight[1] = m.lobes[0].weight[2] = 0.5f;
    m.lobes[0].params[1] = 1.f;
    kz_material light{};
    light.Le[0] = light.Le[1] = light.Le[2] = 3.f;
    scene.add_mesh({-1, 2, -1, -1, 2, 1, 1, 2, 1, 1, 2, -1}, {0, 1, 2, 0, 2, 3}, 1, true);
    // vertex normals equal to the face normal: the same shading through the attribute path
    scene.set_mesh_normals(0, {0, 1, 0, 0, 1, 0, 0, 1, 0});
    scene.set_materials({m, light});
    {
        kz::Scene other;  // host-side calls of the remaining wrappers
        const float p[3] = {0, 5, 0}, rad[3] = {1, 1, 1};
        if (other.add_point_light(p, rad) != 0) return 2;
    }
    scene.build_bvh();
    kz::GpuAccel accel(scene);
    const float o[3] = {0, 1, 0}, d[3] = {0, -1, 0};
    kz::Intersection it;
    const bool hit = accel.intersect(kz::make_ray(o, d, 0.f), it);
    float t = 0.f;
    accel.intersect(kz::make_ray(o, d, 0.f), t);
    const bool occ = accel.occluded(kz::make_ray(o, d, 0.f));
    kz::PathIntegrator integ(5, 7);
    integ.setup(scene);
    const float up[3] = {0, -1, 0.01f};
    std::vector<kz_ray> rays(64, kz::make_ray(o, up));
    const std::vector<float> L = integ.Li(rays);
    double sum = 0;
    for (float x : L) sum += x;
    std::printf("hit=%d geom=%u prim=%u t=%.6f occluded=%d Li_sum=%.6f\n", hit ? 1 : 0, it.geom_id, it.prim_id, t,
                occ ? 1 : 0, sum);
    return hit && it.geom_id == 0 && it.prim_id == 0 && t == 1.0f && occ ? 0 : 1;
}
