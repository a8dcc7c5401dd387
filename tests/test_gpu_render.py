"""GPU wavefront path integrator against the CPU restatement of
PathIntegrator::Li. Both draw every path from the same PCG32 stream, so the
images agree far more tightly than two independent renders: the stated bound
is relMSE <= 1e-3 (spec image tolerance), with the FP64-accumulated CPU
image as the reference."""
import numpy as np
import pytest

from kazen_proto_gb300 import api, scenes

pytestmark = pytest.mark.gpu

REL_MSE_TOL = 1e-3


def rel_mse(img, ref, eps=1e-2):
    img = np.asarray(img, np.float64)
    ref = np.asarray(ref, np.float64)
    return float(np.mean((img - ref) ** 2 / (ref ** 2 + eps)))


def oracle_camera(O, cam):
    return O.make_camera(cam.eye, cam.lookat, cam.up, cam.fov, cam.flip)


@pytest.fixture(scope="module")
def box():
    d = scenes.box_scene(64, 64, spp=16, max_depth=5)
    return d, d.build()


def test_box_scene_matches_restatement(gpu, oracle_mod, box):
    d, s = box
    W, H, spp = 64, 64, 16
    r = api.Renderer(spp=spp, max_depth=5, seed=3)
    img, img64 = r.render(s, d.camera, W, H, fp64=True)
    osc = oracle_mod.Scene.from_desc(d)
    ref, st = osc.render(oracle_camera(oracle_mod, d.camera), W, H, spp, 5, seed=3)
    e = rel_mse(img64, ref)
    assert e <= REL_MSE_TOL, e
    assert e <= 1e-5, f"same-stream renders should agree to ~1e-6, got {e}"
    assert rel_mse(img, img64) < 1e-8
    # the same paths are traced: bounce and shadow-ray counts agree closely
    g = r.last_stats
    assert abs(g["path_bounces"] - st["path_bounces"]) <= 1e-3 * st["path_bounces"]
    assert abs(g["shadow_rays"] - st["shadow_rays"]) <= 1e-3 * st["shadow_rays"]
    assert g["paths"] == W * H * spp


def test_box_scene_1024spp(gpu, oracle_mod, box):
    """Converged image at 1024 spp within relMSE 1e-3 of the FP64 CPU render."""
    d, s = box
    W, H, spp = 32, 32, 1024
    img = api.Renderer(spp=spp, max_depth=5, seed=11).render(s, d.camera, W, H)
    ref, _ = oracle_mod.Scene.from_desc(d).render(oracle_camera(oracle_mod, d.camera), W, H, spp, 5, seed=11)
    assert rel_mse(img, ref) <= REL_MSE_TOL


@pytest.fixture(scope="module")
def box256():
    """The small-box workload at its stated size: 256 x 256, pinhole fov 40,
    depth 5 (36 triangles; Lambert walls and tall box, GGX conductor box with
    alpha 0.2 and F0 (0.95, 0.64, 0.54), a 0.25 x 0.25 ceiling light of
    radiance (17, 12, 4))."""
    d = scenes.box_scene(256, 256, spp=16, max_depth=5)
    return d, d.build()


def test_box256_16spp_matches_restatement(gpu, oracle_mod, box256):
    """256 x 256 x 16 spp, depth 5: the GPU image (FP64 film) against the
    restatement's FP64 render of the same PCG32 streams."""
    d, s = box256
    W, H, spp = 256, 256, 16
    r = api.Renderer(spp=spp, max_depth=5, seed=21)
    img, img64 = r.render(s, d.camera, W, H, fp64=True)
    ref, st = oracle_mod.Scene.from_desc(d).render(oracle_camera(oracle_mod, d.camera), W, H, spp, 5, seed=21)
    e = rel_mse(img64, ref)
    assert e <= REL_MSE_TOL, e
    assert e <= 1e-5, f"same-stream renders should agree to ~1e-6, got {e}"
    assert r.last_stats["paths"] == W * H * spp
    assert abs(r.last_stats["path_bounces"] - st["path_bounces"]) <= 1e-3 * st["path_bounces"]


def test_box256_1024spp_converges(gpu, oracle_mod, box256):
    """The stated convergence bar at the stated size: the GPU's 1024-spp image
    at 256 x 256 within relMSE 1e-3 of the restatement's FP64 1024-spp render
    (same streams), and within relMSE 1e-3 of an independent 16,384-spp FP64
    GPU reference (a different seed: a true convergence check, whose error is
    the 1024-spp image's own noise)."""
    d, s = box256
    W, H = 256, 256
    img = api.Renderer(spp=1024, max_depth=5, seed=31).render(s, d.camera, W, H)
    ref, _ = oracle_mod.Scene.from_desc(d).render(oracle_camera(oracle_mod, d.camera), W, H, 1024, 5, seed=31)
    e_same = rel_mse(img, ref)
    assert e_same <= 1e-5, e_same
    hi = api.Renderer(spp=16384, max_depth=5, seed=77).render(s, d.camera, W, H, fp64=True)[1]
    e_conv = rel_mse(img, hi)
    assert e_conv <= REL_MSE_TOL, e_conv
    # and the 1024-spp noise is what is left: a 64-spp image is clearly worse
    lo = api.Renderer(spp=64, max_depth=5, seed=32).render(s, d.camera, W, H)
    assert rel_mse(lo, hi) > 4 * e_conv


def test_wavefront_refill_is_deterministic(gpu, box):
    d, s = box
    a = api.Renderer(spp=8, max_depth=5, seed=5).render(s, d.camera, 48, 40)
    b = api.Renderer(spp=8, max_depth=5, seed=5, wavefront_size=777, block_size=64).render(s, d.camera, 48, 40)
    assert rel_mse(a, b) < 1e-10
    c = api.Renderer(spp=8, max_depth=5, seed=6).render(s, d.camera, 48, 40)
    assert rel_mse(a, c) > 1e-4  # another seed is another estimate


def test_li_batch_matches_restatement(gpu, oracle_mod, box):
    d, s = box
    cam = oracle_camera(oracle_mod, d.camera)
    rays = oracle_mod.camera_rays(cam, 32, 32, 4, seed=2)
    integ = api.PathIntegrator(max_depth=5, seed=9)
    integ.setup(s)
    L = integ.Li(rays)
    Lo, st = oracle_mod.Scene.from_desc(d).li(rays, 5, seed=9)
    assert rel_mse(L, Lo) < 1e-5
    close = np.all(np.abs(L - Lo) <= 1e-3 * np.maximum(1.0, np.abs(Lo)), axis=1)
    assert close.mean() > 0.995


def test_device_memory_render_matches_host(gpu, box):
    torch = pytest.importorskip("torch")
    d, s = box
    W, H = 40, 30
    r = api.Renderer(spp=4, max_depth=5, seed=1)
    host = r.render(s, d.camera, W, H)
    rgb = torch.empty((H, W, 3), dtype=torch.float32, device="cuda")
    rgb64 = torch.empty((H, W, 3), dtype=torch.float64, device="cuda")
    r.render(s, d.camera, W, H, device_out=(rgb, rgb64))
    assert rel_mse(rgb.cpu().numpy(), host) < 1e-10
    assert rel_mse(rgb64.cpu().numpy(), host) < 1e-8
    # a caller's pinned host buffer, reused for two frames
    pinned = torch.empty((H, W, 3), dtype=torch.float32, pin_memory=True)
    for _ in range(2):
        out = r.render(s, d.camera, W, H, out=pinned)
        assert out is pinned and rel_mse(pinned.numpy(), host) < 1e-10


def test_mixture_and_delta_materials(gpu, oracle_mod):
    """The shipped cbox shaders (diffuse, rough = 0.5 diffuse + 0.1 Beckmann
    microfacet, mirror, dielectric, emitter) lowered and rendered."""
    d = scenes.box_scene(40, 40, spp=8, max_depth=6)
    rough = api.material([api.diffuse((0.35, 0.35, 0.35)), api.microfacet("beckmann", 0.28, eta=1.5,
                                                                         weight=(0.07, 0.07, 0.07))])
    d.materials[2] = rough                                          # white walls -> rough
    d.materials[3] = api.material([api.dielectric(1.5046, 1.000277)])  # metal box -> glass
    d.materials.append(api.material([api.mirror((0.9, 0.9, 0.9))]))
    v, i = scenes.box((0.1, 0.0, 0.1), (0.25, 0.15, 0.25))
    d.add(v, i, len(d.materials) - 1)
    s = d.build()
    img = api.Renderer(spp=8, max_depth=6, seed=4).render(s, d.camera, 40, 40)
    ref, _ = oracle_mod.Scene.from_desc(d).render(oracle_camera(oracle_mod, d.camera), 40, 40, 8, 6, seed=4)
    assert rel_mse(img, ref) <= REL_MSE_TOL


def test_further_closures_render(gpu, oracle_mod):
    """Phong, Ward, KpMicrofacet, the principled lobes (diffuse, retro,
    fake subsurface, sheen, clearcoat), translucent, reflection, refraction
    and transparent materials in one scene, against the restatement."""
    d = scenes.box_scene(40, 40, spp=8, max_depth=6)
    d.materials[0] = api.material([api.principle_diffuse((0.5, 0.06, 0.05)), api.principle_retro(0.6, (0.5, 0.06, 0.05)),
                                   api.principle_sheen(1.0, (0.2, 0.2, 0.2))])
    d.materials[1] = api.material([api.principle_fakess(0.4, (0.1, 0.4, 0.08)),
                                   api.principle_clearcoat(0.2, (0.8, 0.8, 0.8))])
    d.materials[2] = api.material([api.ward(0.1, 0.35, (0.4, 0.4, 0.38)), api.phong(30.0, (0.2, 0.2, 0.2))])
    d.materials[3] = api.material([api.kp_microfacet(0.25, 1.5, 1.0, 0.5, (0.8, 0.6, 0.3))])
    extra = [api.material([api.reflection(1.5, (0.9, 0.9, 0.9))]),
             api.material([api.refraction(1.5)]),
             api.material([api.transparent((0.5, 0.5, 0.5)), api.translucent((0.4, 0.4, 0.4))])]
    boxes = [((0.1, 0.0, 0.1), (0.25, 0.15, 0.25)), ((0.6, 0.35, 0.3), (0.75, 0.5, 0.45)),
             ((0.3, 0.65, 0.4), (0.45, 0.8, 0.55))]
    for m, (lo, hi) in zip(extra, boxes):
        d.materials.append(m)
        v, i = scenes.box(lo, hi)
        d.add(v, i, len(d.materials) - 1)
    s = d.build()
    img = api.Renderer(spp=8, max_depth=6, seed=5).render(s, d.camera, 40, 40)
    ref, _ = oracle_mod.Scene.from_desc(d).render(oracle_camera(oracle_mod, d.camera), 40, 40, 8, 6, seed=5)
    assert np.isfinite(img).all() and img.mean() > 0
    assert rel_mse(img, ref) <= REL_MSE_TOL


def test_reference_shader_library_render(gpu, oracle_mod):
    """The reference's own principle.osl, disney_brdf.osl and ward.osl, as
    lowered at their defaults (tests/golden/reference_shaders_lowered.json),
    on the walls and boxes of the box scene, against the restatement."""
    import json
    import os
    with open(os.path.join(os.path.dirname(__file__), "golden", "reference_shaders_lowered.json")) as f:
        g = json.load(f)

    def mat(key):
        return api.material([api.lobe(l["closure_id"], l["weight"], l["params"]) for l in g[key]["lobes"]])

    d = scenes.box_scene(40, 40, spp=8, max_depth=6)
    d.materials[0] = mat("resource/shader/src/principle.osl")
    d.materials[1] = mat("resource/shader/src/ward.osl")
    d.materials[3] = mat("resource/shader/src/disney_brdf.osl")
    s = d.build()
    img = api.Renderer(spp=8, max_depth=6, seed=6).render(s, d.camera, 40, 40)
    ref, _ = oracle_mod.Scene.from_desc(d).render(oracle_camera(oracle_mod, d.camera), 40, 40, 8, 6, seed=6)
    assert np.isfinite(img).all() and img.mean() > 0
    assert rel_mse(img, ref) <= REL_MSE_TOL


def test_textures_and_environment_render(gpu, oracle_mod):
    """Checkerboard-textured walls (uv = barycentrics), an image-textured box
    with explicit uvs, a lobe pair sharing one texture next to an untextured
    lobe, and a latitude-longitude environment seen through the open side of
    the box, against the restatement."""
    rng = np.random.default_rng(8)
    d = scenes.box_scene(40, 40, spp=8, max_depth=6)
    img = rng.random((13, 17, 3)).astype(np.float32)
    sky = (rng.random((8, 16, 3)) * 3).astype(np.float32)
    d.textures = [api.checker_texture(4, 3, (0.9, 0.9, 0.9), (0.1, 0.2, 0.3)), api.image_texture(img),
                  api.image_texture(sky)]
    d.materials[2] = api.material([api.textured(api.diffuse((0.8, 0.8, 0.8)), 0)])
    d.materials[3] = api.material([api.textured(api.principle_diffuse((0.7, 0.7, 0.7)), 1),
                                   api.textured(api.principle_retro(0.5, (0.2, 0.2, 0.2)), 1),
                                   api.conductor_ggx((0.9, 0.6, 0.5), 0.3, weight=(0.3, 0.3, 0.3))])
    d.env, d.env_texture = (0.5, 0.6, 0.7), 2
    # explicit uvs on the metal box (mesh 6): its vertex positions, scaled
    v = d.meshes[6][0]
    d.uvs[6] = (v[:, [0, 2]] * 3.0 - 0.5).astype(np.float32)
    d.camera = api.Camera(eye=(0.5, 0.5, -1.0), lookat=(0.5, 0.4, 0.5), up=(0, 1, 0), fov=70.0)
    s = d.build()
    img_g = api.Renderer(spp=8, max_depth=6, seed=7).render(s, d.camera, 40, 40)
    ref, _ = oracle_mod.Scene.from_desc(d).render(oracle_camera(oracle_mod, d.camera), 40, 40, 8, 6, seed=7)
    assert np.isfinite(img_g).all()
    assert rel_mse(img_g, ref) <= REL_MSE_TOL
    # the environment and the textures change the image
    d2 = scenes.box_scene(40, 40, spp=8, max_depth=6)
    d2.camera = d.camera
    plain = api.Renderer(spp=8, max_depth=6, seed=7).render(d2.build(), d.camera, 40, 40)
    assert rel_mse(img_g, plain) > 1e-2


@pytest.mark.parametrize("with_area", [True, False])
def test_point_lights_render(gpu, oracle_mod, with_area):
    """Point lights next to the area light (uniform pick among all lights,
    MIS only for the area light) and point lights alone."""
    d = scenes.box_scene(40, 40, spp=8, max_depth=5)
    d.point_lights = [((0.3, 0.8, 0.4), (0.4, 0.3, 0.2)), ((0.7, 0.5, 0.25), (0.1, 0.2, 0.4))]
    if not with_area:
        d.meshes = [m for m in d.meshes if not m[3]]
    s = d.build()
    img = api.Renderer(spp=8, max_depth=5, seed=9).render(s, d.camera, 40, 40)
    ref, _ = oracle_mod.Scene.from_desc(d).render(oracle_camera(oracle_mod, d.camera), 40, 40, 8, 5, seed=9)
    assert np.isfinite(img).all() and ref.mean() > 1e-3
    assert rel_mse(img, ref) <= REL_MSE_TOL


def test_shading_normals_render(gpu, oracle_mod):
    """Smooth spheres (icospheres with radial vertex normals: interpolated
    shading normals and the shadow-terminator offset), one diffuse, one
    mirror, one glass, next to flat meshes, against the restatement."""
    d = scenes.box_scene(40, 40, spp=8, max_depth=6)
    d.materials.append(api.material([api.mirror((0.9, 0.9, 0.9))]))
    d.materials.append(api.material([api.dielectric(1.5, 1.0)]))
    sv, sf = scenes.icosphere(2)
    for k, (c, r, m) in enumerate([((0.3, 0.15, 0.3), 0.15, 2), ((0.7, 0.45, 0.35), 0.12, len(d.materials) - 2),
                                    ((0.5, 0.2, 0.7), 0.14, len(d.materials) - 1)]):
        d.add(sv * r + np.asarray(c, np.float32), sf, m, normals=sv)
    s = d.build()
    img = api.Renderer(spp=8, max_depth=6, seed=11).render(s, d.camera, 40, 40)
    ref, _ = oracle_mod.Scene.from_desc(d).render(oracle_camera(oracle_mod, d.camera), 40, 40, 8, 6, seed=11)
    assert np.isfinite(img).all()
    assert rel_mse(img, ref) <= REL_MSE_TOL
    flat = scenes.box_scene(40, 40, spp=8, max_depth=6)
    flat.materials, flat.meshes = d.materials, d.meshes  # the same meshes without normals
    img_flat = api.Renderer(spp=8, max_depth=6, seed=11).render(flat.build(), d.camera, 40, 40)
    assert rel_mse(img, img_flat) > 1e-4


@pytest.mark.parametrize("flags", [0, 4, 8], ids=["mis", "nee_only", "bsdf_only"])
def test_estimators_match_restatement(gpu, oracle_mod, flags):
    """PathIntegrator (MIS), PathEmsIntegrator (NEE only) and
    PathMatsIntegrator (BSDF sampling only) on the mixed-material box."""
    d = scenes.box_scene(40, 40, spp=8, max_depth=6)
    d.materials[3] = api.material([api.dielectric(1.5, 1.0)])
    d.point_lights = [((0.3, 0.8, 0.4), (0.2, 0.2, 0.2))]
    s = d.build()
    img = api.Renderer(spp=8, max_depth=6, seed=12, flags=flags).render(s, d.camera, 40, 40)
    ref, _ = oracle_mod.Scene.from_desc(d).render(oracle_camera(oracle_mod, d.camera), 40, 40, 8, 6, seed=12,
                                                  flags=flags)
    assert np.isfinite(img).all() and ref.mean() > 1e-3
    assert rel_mse(img, ref) <= REL_MSE_TOL
    if flags == 0:
        with pytest.raises(Exception):
            api.Renderer(spp=1, max_depth=2, flags=12).render(s, d.camera, 8, 8)


def test_terrain_scene_small(gpu, oracle_mod):
    d = scenes.terrain_scene(width=64, height=36, spp=2, max_depth=8, cells=64, n_spheres=16)
    s = d.build()
    img = api.Renderer(spp=2, max_depth=8, seed=1).render(s, d.camera, 64, 36)
    ref, _ = oracle_mod.Scene.from_desc(d).render(oracle_camera(oracle_mod, d.camera), 64, 36, 2, 8, seed=1)
    assert np.isfinite(img).all()
    assert rel_mse(img, ref) <= REL_MSE_TOL
