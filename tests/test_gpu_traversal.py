"""GPU traversal parity: closest-hit triangle ids and t bit-exact against the
CPU restatement, any-hit equal, on the traversal workload (1,048,576-triangle
soup, incoherent rays) and the edge cases the reference path meets."""
import numpy as np
import pytest

from kazen_proto_gb300 import _native as N
from kazen_proto_gb300 import api, scenes

pytestmark = pytest.mark.gpu


def soup_scene(tv):
    d = scenes.soup_desc(tv)
    return d.build()


def assert_bit_exact(g, o):
    assert np.array_equal(g["prim_id"], o["prim"]), f"{(g['prim_id'] != o['prim']).sum()} triangle ids differ"
    assert np.array_equal(g["t"].view(np.uint32), o["t"].view(np.uint32)), "t differs"
    hit = o["prim"] != N.KZ_INVALID_ID
    assert np.array_equal(g["u"][hit].view(np.uint32), o["u"][hit].view(np.uint32))
    assert np.array_equal(g["v"][hit].view(np.uint32), o["v"][hit].view(np.uint32))


def test_single_triangle_reference_case(gpu):
    # tests/libusage_tests/embree_tests.cpp:19-76
    s = api.Scene()
    s.add_mesh(np.array([[-1, 0, 1], [2, 0, 1], [-1, 0, -2]], np.float32), [[0, 1, 2]])
    s.set_materials([api.material([api.diffuse()])])
    s.build_bvh()
    h = s.intersect(api.make_rays([0, 1, 0], [0, -1, 0], tmin=0.0, tmax=np.finfo(np.float32).max))
    assert h["prim_id"][0] == 0 and h["geom_id"][0] == 0 and h["t"][0] == np.float32(1.0)


@pytest.mark.parametrize("n_tris,n_rays,seed", [(1000, 20000, 0), (50000, 200000, 1)])
def test_closest_bit_exact_small(gpu, oracle_mod, n_tris, n_rays, seed):
    tv = scenes.triangle_soup(n_tris, seed=seed)
    rays = scenes.soup_rays(n_rays, seed=seed + 100)
    s = soup_scene(tv)
    g = s.intersect(rays)
    o = oracle_mod.Bvh(tv).closest(rays)
    assert_bit_exact(g, o)
    assert (g["geom_id"][o["prim"] != N.KZ_INVALID_ID] == 0).all()
    occ = s.occluded(rays)
    assert np.array_equal(occ, oracle_mod.Bvh(tv).any(rays))


def test_closest_matches_brute_force(gpu, oracle_mod):
    rng = np.random.default_rng(3)
    tv = scenes.triangle_soup(500, seed=4)
    o = rng.uniform(-0.5, 1.5, (3000, 3)).astype(np.float32)
    rays = api.make_rays(o, rng.standard_normal((3000, 3)).astype(np.float32))
    g = soup_scene(tv).intersect(rays)
    b = oracle_mod.closest_brute(tv, rays)
    assert np.array_equal(g["prim_id"], b["prim"])
    assert np.array_equal(g["t"].view(np.uint32), b["t"].view(np.uint32))


@pytest.mark.slow
def test_traversal_workload_full_size(gpu, oracle_mod):
    """1,048,576 triangles x 16,777,216 rays: 100 % triangle-id and t match."""
    tv = scenes.triangle_soup(1 << 20, seed=1)
    rays = scenes.soup_rays(1 << 24, seed=2)
    s = soup_scene(tv)
    g = s.intersect(rays)
    ob = oracle_mod.Bvh(tv)
    o = ob.closest(rays)
    assert_bit_exact(g, o)
    # any-hit on a 2M-ray subset
    sub = rays[: 1 << 21]
    assert np.array_equal(s.occluded(sub), ob.any(sub))


def test_edge_cases(gpu, oracle_mod):
    tri = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    s = api.Scene()
    s.add_mesh(tri, [[0, 1, 2]])                                    # geom 0
    s.add_mesh(tri + np.float32([0, 0, 5]), [[0, 1, 2]])             # geom 1, farther
    s.add_mesh(tri, [[0, 1, 2]])                                    # geom 2, duplicate of geom 0
    s.add_mesh(np.array([[0, 0, 2], [1, 0, 2], [2, 0, 2]], np.float32), [[0, 1, 2]])  # degenerate
    s.set_materials([api.material([api.diffuse()])])
    s.build_bvh()
    rays = np.concatenate([
        api.make_rays([0.2, 0.2, -1], [0, 0, 1]),                   # tie between geom 0 and 2 -> geom 0
        api.make_rays([0.2, 0.2, -1], [0, 0, 1], tmax=0.5),         # tmax before the hit: miss, t = tmax
        api.make_rays([0.2, 0.2, -1], [0, 0, 1], tmin=3.0),         # tmin past the first hits: geom 1
        api.make_rays([5, 5, 5], [1, 0, 0]),                        # misses everything
        api.make_rays([0.0, 0.0, -1], [0, 0, 1]),                   # exactly through a vertex
        api.make_rays([0.5, 0.0, -1], [0, 0, 1]),                   # exactly on an edge
        api.make_rays([0.2, 0.2, -1], [0, 0, 1], tmax=1.0),         # t == tmax is inside (tmin, tmax]
    ])
    h = s.intersect(rays)
    assert (h["geom_id"][0], h["prim_id"][0]) == (0, 0)
    assert h["prim_id"][1] == N.KZ_INVALID_ID and h["t"][1] == np.float32(0.5)
    assert h["geom_id"][2] == 1
    assert h["prim_id"][3] == N.KZ_INVALID_ID and np.isinf(h["t"][3])
    assert h["geom_id"][4] == 0 and h["geom_id"][5] == 0
    assert h["geom_id"][6] == 0 and h["t"][6] == np.float32(1.0)
    occ = s.occluded(rays)
    assert list(occ) == [True, False, True, False, True, True, True]


def test_empty_scene_and_empty_batch(gpu):
    s = api.Scene()
    s.set_materials([api.material([api.diffuse()])])
    s.build_bvh()
    h = s.intersect(api.make_rays([[0, 0, 0], [1, 1, 1]], [[0, 0, 1], [0, 1, 0]], tmax=7.0))
    assert (h["prim_id"] == N.KZ_INVALID_ID).all() and (h["t"] == 7.0).all()
    assert not s.occluded(api.make_rays([0, 0, 0], [0, 0, 1])).any()
    s2 = soup_scene(scenes.triangle_soup(100, seed=1))
    h = s2.intersect(np.zeros(0, N.RAY_DTYPE))
    assert len(h["t"]) == 0


def test_watertight_closed_mesh_gpu(gpu):
    v, f = scenes.icosphere(3)
    s = api.Scene()
    s.add_mesh(v, f)
    s.set_materials([api.material([api.diffuse()])])
    s.build_bvh()
    targets = np.concatenate([v, 0.5 * (v[f[:, 0]] + v[f[:, 1]]), 0.5 * (v[f[:, 1]] + v[f[:, 2]])])
    h = s.intersect(api.make_rays(np.zeros_like(targets), targets))
    assert (h["prim_id"] != N.KZ_INVALID_ID).all()


def test_device_memory_path_matches_host(gpu):
    torch = pytest.importorskip("torch")
    tv = scenes.triangle_soup(20000, seed=5)
    rays = scenes.soup_rays(100000, seed=6)
    s = soup_scene(tv)
    hh = s.intersect(rays)
    dr = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).cuda()
    hd = s.intersect(dr)
    s.synchronize()
    assert np.array_equal(hd["prim_id"].cpu().numpy().view(np.uint32), hh["prim_id"])
    assert np.array_equal(hd["t"].cpu().numpy().view(np.uint32), hh["t"].view(np.uint32))
    od = s.occluded(dr)
    s.synchronize()
    assert np.array_equal(od.cpu().numpy().astype(bool), s.occluded(rays))


def test_multi_mesh_ids_and_transform(gpu, oracle_mod):
    rng = np.random.default_rng(9)
    s = api.Scene()
    soups = [scenes.triangle_soup(3000, seed=20 + k) for k in range(4)]
    xf = np.array([[1, 0, 0, 0.25], [0, 1, 0, 0.0], [0, 0, 1, -0.1]], np.float32)
    for k, tv in enumerate(soups):
        n = len(tv)
        s.add_mesh(tv.reshape(-1, 3), np.arange(3 * n).reshape(n, 3), 0, xform=xf if k == 2 else None)
    s.set_materials([api.material([api.diffuse()])])
    s.build_bvh()
    world = []
    for k, tv in enumerate(soups):
        v = tv.reshape(-1, 3)
        if k == 2:  # the library's transform: row . (x, y, z) + t, evaluated left to right in FP32
            v = ((xf[:, 0] * v[:, :1] + xf[:, 1] * v[:, 1:2]) + xf[:, 2] * v[:, 2:3]) + xf[:, 3]
        world.append(v.astype(np.float32).reshape(-1, 9))
    world = np.concatenate(world)
    rays = scenes.soup_rays(50000, seed=31)
    g = s.intersect(rays)
    o = oracle_mod.Bvh(world).closest(rays)
    hit = o["prim"] != N.KZ_INVALID_ID
    assert np.array_equal(g["geom_id"][hit], o["prim"][hit] // 3000)
    assert np.array_equal(g["prim_id"][hit], o["prim"][hit] % 3000)
    assert np.array_equal(g["t"].view(np.uint32), o["t"].view(np.uint32))


def test_intersect_stats_counts(gpu):
    tv = scenes.triangle_soup(20000, seed=7)
    rays = scenes.soup_rays(10000, seed=8)
    s = soup_scene(tv)
    nodes, tris = s.intersect_stats(rays)
    assert nodes >= len(rays) and tris > 0
    info = s.info()
    assert info["n_triangles"] == 20000 and info["bvh_depth"] <= 60
