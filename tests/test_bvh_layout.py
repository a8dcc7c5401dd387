"""Checks of the device BVH layout (host builder only; no GPU): every node
reachable once, slot encodings valid, leaves partition the triangle records,
dequantized slot boxes contain their subtrees, records carry the exact input
vertices, depth within the traversal stack; and a float emulation of the
device traversal agrees with brute force on closest triangle and t bits."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from kazen_proto_gb300 import scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


# ---- 8-wide quantized BVH --------------------------------------------------

WIDE_OUT = os.path.join(ROOT, "kazen_proto_gb300", "_build", "wide_bvh_check.so")


@pytest.fixture(scope="module")
def wide():
    os.makedirs(os.path.dirname(WIDE_OUT), exist_ok=True)
    srcs = [os.path.join(ROOT, "tests", "wide_bvh_check.cpp"),
            os.path.join(ROOT, "kazen_proto_gb300", "csrc", "kz_bvh.cpp")]
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-ffp-contract=off", "-o", WIDE_OUT] + srcs,
                   check=True)
    lib = C.CDLL(WIDE_OUT)
    lib.kzt_check_wide.restype = C.c_int
    lib.kzt_check_wide.argtypes = [C.c_void_p, C.c_uint32, C.c_char_p, C.c_int, C.POINTER(C.c_uint32),
                                   C.POINTER(C.c_uint32)]
    lib.kzt_wide_trace.restype = C.c_int64
    lib.kzt_wide_trace.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.POINTER(C.c_double),
                                   C.POINTER(C.c_uint32)]
    return lib


def wide_check(lib, tv):
    tv = np.ascontiguousarray(tv, np.float32).reshape(-1, 9)
    msg = C.create_string_buffer(256)
    nn, dp = C.c_uint32(), C.c_uint32()
    rc = lib.kzt_check_wide(tv.ctypes.data_as(C.c_void_p), len(tv), msg, 256, C.byref(nn), C.byref(dp))
    assert rc == 0, msg.value.decode()
    return nn.value, dp.value


def wide_trace(lib, tv, rays):
    tv = np.ascontiguousarray(tv, np.float32).reshape(-1, 9)
    r = np.ascontiguousarray(rays)
    vis, hits = C.c_double(), C.c_uint32()
    bad = lib.kzt_wide_trace(tv.ctypes.data_as(C.c_void_p), len(tv), r.ctypes.data_as(C.c_void_p), len(r),
                             C.byref(vis), C.byref(hits))
    return bad, vis.value, hits.value


@pytest.mark.parametrize("n", [0, 1, 2, 3, 4, 5, 17, 24, 25, 1000, 100000])
def test_wide_layouts(wide, n):
    nodes, depth = wide_check(wide, scenes.triangle_soup(n, seed=n + 1) if n else np.zeros((0, 9), np.float32))
    assert nodes >= 1 and depth <= 96


def test_wide_coincident_and_degenerate(wide):
    tri = np.array([0, 0, 0, 1, 0, 0, 0, 1, 0], np.float32)
    wide_check(wide, np.tile(tri, (5000, 1)))
    wide_check(wide, np.zeros((300, 9), np.float32))
    # huge and tiny extents in one scene
    big = scenes.triangle_soup(200, seed=3) * np.float32(1e6)
    tiny = scenes.triangle_soup(200, seed=4) * np.float32(1e-6)
    wide_check(wide, np.concatenate([big, tiny]))


def test_wide_terrain_layout(wide):
    d = scenes.terrain_scene(64, 36, 1, 8, cells=128, n_spheres=8)
    tv, _, _, _ = d.flatten()
    nodes, depth = wide_check(wide, tv)
    assert depth <= 40


def _axis_rays(n, seed):
    """Rays with exactly zero direction components and origins on box planes."""
    rng = np.random.default_rng(seed)
    rays = scenes.soup_rays(n, seed=seed)
    k = n // 4
    rays["dx"][:k] = 0.0
    rays["dy"][k:2 * k] = 0.0
    rays["dz"][2 * k:3 * k] = 0.0
    d = np.stack([rays["dx"], rays["dy"], rays["dz"]], 1)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays["dx"], rays["dy"], rays["dz"] = d[:, 0], d[:, 1], d[:, 2]
    rays["ox"][:k] = rng.random(k, dtype=np.float32)  # inside the soup's x range
    return rays


@pytest.mark.parametrize("n_tris,seed", [(1, 1), (7, 2), (64, 3), (3000, 4)])
def test_wide_traversal_matches_brute_force(wide, n_tris, seed):
    tv = scenes.triangle_soup(n_tris, seed=seed)
    rays = scenes.soup_rays(2000, seed=seed + 10)
    bad, visits, hits = wide_trace(wide, tv, rays)
    assert bad == 0
    assert hits > 0 or n_tris < 64  # one small triangle may be missed by all rays


def test_wide_traversal_edge_rays(wide):
    tv = scenes.triangle_soup(2000, seed=9)
    bad, _, hits = wide_trace(wide, tv, _axis_rays(4000, 21))
    assert bad == 0 and hits > 0
    # finite tmax and rays starting inside the soup
    rays = scenes.soup_rays(2000, seed=22)
    rays["ox"], rays["oy"], rays["oz"] = 0.5, 0.5, 0.5
    rays["tmax"] = np.float32(0.3)
    bad, _, hits = wide_trace(wide, tv, rays)
    assert bad == 0 and hits > 0


def test_wide_traversal_terrain(wide):
    d = scenes.terrain_scene(64, 36, 1, 8, cells=64, n_spheres=4)
    tv, _, _, _ = d.flatten()
    rng = np.random.default_rng(5)
    lo, hi = tv.reshape(-1, 3).min(0), tv.reshape(-1, 3).max(0)
    n = 1500
    rays = np.zeros(n, dtype=scenes.api.N.RAY_DTYPE)
    o = lo + (hi - lo) * rng.random((n, 3))
    dv = rng.standard_normal((n, 3))
    dv /= np.linalg.norm(dv, axis=1, keepdims=True)
    rays["ox"], rays["oy"], rays["oz"] = o[:, 0], o[:, 1], o[:, 2]
    rays["dx"], rays["dy"], rays["dz"] = dv[:, 0], dv[:, 1], dv[:, 2]
    rays["tmin"], rays["tmax"] = np.float32(1e-4), np.float32(np.inf)
    bad, visits, hits = wide_trace(wide, tv, rays)
    assert bad == 0 and hits > n // 10
