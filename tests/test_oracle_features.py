"""Known answers for the restatement's lights, shading normals, textures and
environment: with a point light (a delta light: one next-event sample is
exact) and max_depth 1 (the first shaded vertex only), the radiance of a ray
hitting a diffuse surface is albedo/pi * cos * radiance / (0.1 d^2) exactly;
a ray leaving the scene sees the environment. These pin the checker the GPU
renders are compared with."""
import math

import numpy as np
import pytest

from kazen_proto_gb300 import api, scenes


def plane(desc, material, normals=None, uv=None):
    v = np.array([[-2, 0, -2], [2, 0, -2], [2, 0, 2], [-2, 0, 2]], np.float32)
    desc.add(v, np.array([[0, 2, 1], [0, 3, 2]], np.uint32), material, normals=normals, uv=uv)


def li(oracle_mod, desc, o, d):
    rays = api.make_rays(np.asarray(o, np.float32), np.asarray(d, np.float32))
    L, _ = oracle_mod.Scene.from_desc(desc).li(rays, max_depth=1, seed=1)
    return L


def test_point_light_over_diffuse_plane(oracle_mod):
    d = scenes.SceneDesc()
    d.materials = [api.material([api.diffuse((0.5, 0.25, 0.125))])]
    plane(d, 0)
    d.point_lights = [((0.3, 2.0, -0.4), (1.0, 2.0, 4.0))]
    # hit points straight below the camera at x in {0, 0.6}
    L = li(oracle_mod, d, [[0, 3, 0], [0.6, 3, 0]], [[0, -1, 0], [0, -1, 0]])
    for k, x in enumerate((0.0, 0.6)):
        lv = np.array([0.3 - x, 2.0, -0.4])
        d2 = float(lv @ lv)
        cos = 2.0 / math.sqrt(d2)
        want = np.array([0.5, 0.25, 0.125]) / math.pi * cos * np.array([1.0, 2.0, 4.0]) / (0.1 * d2)
        assert np.allclose(L[k], want, rtol=2e-6), (L[k], want)


def test_shading_normals_set_frame_and_point(oracle_mod):
    """Vertex normals tilted by 30 degrees: the diffuse cosine is taken against
    the shading normal, and the shading point moves by the shadow-terminator
    offset P' = P - sum_i b_i min(0, (P - v_i).n_i) n_i (Hanika 2021), from
    which the light is seen."""
    t = math.radians(30.0)
    nrm = np.array([math.sin(t), math.cos(t), 0.0])
    d = scenes.SceneDesc()
    d.materials = [api.material([api.diffuse((1.0, 1.0, 1.0))])]
    plane(d, 0, normals=np.tile(nrm.astype(np.float32), (4, 1)))
    light = np.array([0.0, 2.0, 0.0])
    d.point_lights = [(tuple(light), (1.0, 1.0, 1.0))]
    x, z = 0.7, -0.4  # inside triangle (v0, v2, v1) = ((-2,0,-2), (2,0,2), (2,0,-2))
    L = li(oracle_mod, d, [[x, 3, z]], [[0, -1, 0]])
    v = np.array([[-2, 0, -2], [2, 0, 2], [2, 0, -2]], np.float64)
    P = np.array([x, 0.0, z])
    T = np.stack([v[1] - v[0], v[2] - v[0]], 1)[[0, 2]]
    b1, b2 = np.linalg.solve(T, (P - v[0])[[0, 2]])
    b = np.array([1 - b1 - b2, b1, b2])
    assert (b >= 0).all()
    Pp = P - sum(b[i] * min(0.0, float((P - v[i]) @ nrm)) * nrm for i in range(3))
    assert np.linalg.norm(Pp - P) > 1e-3  # the offset is in play
    lv = light - Pp
    d2 = float(lv @ lv)
    want = 1.0 / math.pi * float(lv @ nrm) / math.sqrt(d2) / (0.1 * d2)
    assert np.allclose(L[0], want, rtol=1e-5), (L[0], want)


def test_checker_texture_tints_the_weight(oracle_mod):
    d = scenes.SceneDesc()
    d.textures = [api.checker_texture(2, 2, (1.0, 0.5, 0.25), (0.1, 0.2, 0.3))]
    d.materials = [api.material([api.textured(api.diffuse((0.5, 0.5, 0.5)), 0)])]
    # uv = (x, z) / 4 + 1/2 on the plane
    plane(d, 0, uv=np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32))
    d.point_lights = [((0.0, 2.0, 0.0), (1.0, 1.0, 1.0))]
    xs = [(-1.5, -1.5), (-0.5, -1.5), (0.5, 0.5)]  # uv (0.125, 0.125) Ca, (0.375, 0.125) Cb, (0.625, 0.625) Ca
    L = li(oracle_mod, d, [[x, 3, z] for x, z in xs], [[0, -1, 0]] * 3)
    for k, (x, z) in enumerate(xs):
        s_, t_ = x / 4 + 0.5, z / 4 + 0.5
        tint = (1.0, 0.5, 0.25) if (int(s_ * 2 % 2) ^ int(t_ * 2 % 2)) == 0 else (0.1, 0.2, 0.3)
        lv = np.array([-x, 2.0, -z])
        d2 = float(lv @ lv)
        want = 0.5 * np.array(tint) / math.pi * (2.0 / math.sqrt(d2)) / (0.1 * d2)
        assert np.allclose(L[k], want, rtol=2e-6), (k, L[k], want)


@pytest.mark.parametrize("direction", [(0, 1, 0), (1, 0, 0), (0, 0, -1), (0.6, 0.0, 0.8)])
def test_environment_lookup(oracle_mod, direction):
    """A miss sees rgb times the latitude-longitude texture at
    s = 1/2 + atan2(x, -z) / 2 pi, t = acos(y) / pi (texel centres, bilinear)."""
    rng = np.random.default_rng(4)
    img = rng.random((4, 8, 3)).astype(np.float32)
    d = scenes.SceneDesc()
    d.materials = [api.material([api.diffuse()])]
    plane(d, 0)  # far below every ray
    d.textures = [api.image_texture(img)]
    d.env, d.env_texture = (2.0, 1.0, 0.5), 0
    dr = np.asarray(direction, np.float64)
    dr /= np.linalg.norm(dr)
    L = li(oracle_mod, d, [[0, 5, 0]], [dr])
    s_ = 0.5 + math.atan2(dr[0], -dr[2]) / (2 * math.pi)
    t_ = math.acos(dr[1]) / math.pi
    s_ -= math.floor(s_)
    t_ -= math.floor(t_)
    x, y = s_ * 8 - 0.5, t_ * 4 - 0.5
    x0, y0 = math.floor(x), math.floor(y)
    ax, ay = x - x0, y - y0
    px = lambda i, j: img[j % 4, i % 8].astype(np.float64)  # noqa: E731
    tex = (px(x0, y0) * (1 - ax) + px(x0 + 1, y0) * ax) * (1 - ay) + (px(x0, y0 + 1) * (1 - ax) + px(x0 + 1, y0 + 1) * ax) * ay
    want = np.array([2.0, 1.0, 0.5]) * tex
    assert np.allclose(L[0], want, rtol=1e-5, atol=1e-6), (L[0], want)
