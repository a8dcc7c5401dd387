"""The restatement's reference-as-written modes (CPU, test infrastructure).

The GPU path computes the corrected estimator; these modes of the CPU
restatement reproduce the reference's path loop as written
(src/core/integrator.cpp:362-561, bsdf.cpp:17-55) and its own single-sided
Moller-Trumbore test (src/core/shape.cpp:373-408, 533-557), so the deviation
of the corrected image from what kazen_proto itself renders is a number:
on the small box (64 x 64, 256 spp, depth 5) the four defects together give
relMSE ~0.13 against the corrected image (mean 0.78x), against a noise floor
of ~2e-3 between two corrected renders."""
import numpy as np
import pytest

from kazen_proto_gb300 import api, scenes

W, SPP = 64, 256


def rel_mse(img, ref, eps=1e-2):
    return float(np.mean((np.asarray(img, np.float64) - ref) ** 2 / (ref ** 2 + eps)))


@pytest.fixture(scope="module")
def box(oracle_mod):
    d = scenes.box_scene(W, W, spp=SPP, max_depth=5)
    sc = oracle_mod.Scene.from_desc(d)
    c = d.camera
    cam = oracle_mod.make_camera(c.eye, c.lookat, c.up, c.fov, c.flip)
    ref, _ = sc.render(cam, W, W, SPP, 5, seed=1)
    ref2, _ = sc.render(cam, W, W, SPP, 5, seed=2)
    return sc, cam, ref, rel_mse(ref2, ref)


def test_compat_zero_is_the_corrected_loop(oracle_mod, box):
    sc, cam, ref, _ = box
    img, _ = sc.render_compat(cam, W, W, SPP, 5, 0, seed=1)
    assert np.array_equal(img, ref)


@pytest.mark.parametrize("name,bit,min_ratio,lo,hi", [
    # NEE times cos twice on Lambert surfaces: darker
    ("nee", 1, 5.0, 0.80, 0.97),
    # no division by the direction pdf under uniform-theta sampling: darker
    ("bsdf", 2, 20.0, 0.70, 0.95),
    # emission weighted with the stale light pdf next to the corrected NEE:
    # the weights no longer sum to one, brighter
    ("emission", 4, 50.0, 1.2, 1.7),
    # at most 4 shaded vertices instead of 5: slightly darker
    ("depth", 8, 0.0, 0.95, 0.999),
    ("all", 15, 20.0, 0.65, 0.90),
])
def test_reference_as_written_deviation(oracle_mod, box, name, bit, min_ratio, lo, hi):
    sc, cam, ref, noise = box
    img, _ = sc.render_compat(cam, W, W, SPP, 5, bit, seed=1)
    e = rel_mse(img, ref)
    ratio = img.mean() / ref.mean()
    assert np.isfinite(img).all()
    assert e >= min_ratio * noise, (name, e, noise)
    assert lo <= ratio <= hi, (name, ratio)


def test_moller_trumbore_known_answer(oracle_mod):
    # the single triangle and ray of the reference's Embree test
    # (tests/libusage_tests/embree_tests.cpp:19-76): hit at t = 1
    tri = np.array([[-1, 0, 1, 2, 0, 1, -1, 0, -2]], np.float32)
    r = api.make_rays([[0, 1, 0]], [[0, -1, 0]])
    h = oracle_mod.mt_intersect(tri, r)
    assert h["prim"][0] == 0 and h["t"][0] == 1.0
    assert abs(h["u"][0] - 1 / 3) < 1e-6 and abs(h["v"][0] - 1 / 3) < 1e-6
    # single-sided: from below the same triangle is culled, where the
    # (double-sided) watertight test of the restatement hits it
    rb = api.make_rays([[0, -1, 0]], [[0, 1, 0]])
    assert oracle_mod.mt_intersect(tri, rb)["prim"][0] == 0xFFFFFFFF
    assert oracle_mod.closest_brute(tri, rb)["prim"][0] == 0


def test_moller_trumbore_first_hit_is_not_closest(oracle_mod):
    # two parallel front-facing triangles along the ray; index 0 is the far one
    far = [-1, -2, 1, 2, -2, 1, -1, -2, -2]
    near = [-1, 0, 1, 2, 0, 1, -1, 0, -2]
    tri = np.array([far, near], np.float32)
    r = api.make_rays([[0, 1, 0]], [[0, -1, 0]])
    closest = oracle_mod.mt_intersect(tri, r)
    first = oracle_mod.mt_intersect(tri, r, first_hit=True)
    assert closest["prim"][0] == 1 and closest["t"][0] == 1.0
    assert first["prim"][0] == 0 and first["t"][0] == 3.0


def test_moller_trumbore_agrees_with_watertight_on_front_faces(oracle_mod):
    tv = scenes.triangle_soup(2000, seed=4)
    rays = scenes.soup_rays(3000, seed=5)
    mt = oracle_mod.mt_intersect(tv, rays)
    wt = oracle_mod.closest_brute(tv, rays)
    hit = wt["prim"] != 0xFFFFFFFF
    both = hit & (mt["prim"] == wt["prim"])
    # wherever the closest watertight hit is a front face the two tests agree
    # on the triangle (about half of the hits), with t within float rounding
    assert hit.sum() > 100 and both.sum() > 0.3 * hit.sum()
    assert np.allclose(mt["t"][both], wt["t"][both], rtol=1e-5, atol=1e-6)
    # back faces are hit by the watertight test only
    only_wt = (wt["prim"] != 0xFFFFFFFF) & (mt["prim"] != wt["prim"])
    assert only_wt.sum() > 0
