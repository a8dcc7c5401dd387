"""Structural checks of the device BVH layout (host builder only; no GPU):
links in range, no cycles, every node reachable once, leaves partition the
triangle records, boxes contain their contents, records carry the exact
input vertices, depth within the traversal stack."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from kazen_proto_gb300 import scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
OUT = os.path.join(ROOT, "kazen_proto_gb300", "_build", "bvh_layout_check.so")


@pytest.fixture(scope="module")
def checker():
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    srcs = [os.path.join(ROOT, "tests", "bvh_layout_check.cpp"),
            os.path.join(ROOT, "kazen_proto_gb300", "csrc", "kz_bvh.cpp")]
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-o", OUT] + srcs, check=True)
    lib = C.CDLL(OUT)
    f = lib.kzt_check_layout
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_uint32, C.c_char_p, C.c_int, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
    return f


def run(checker, tv):
    tv = np.ascontiguousarray(tv, np.float32).reshape(-1, 9)
    msg = C.create_string_buffer(256)
    nn, dp = C.c_uint32(), C.c_uint32()
    rc = checker(tv.ctypes.data_as(C.c_void_p), len(tv), msg, 256, C.byref(nn), C.byref(dp))
    assert rc == 0, msg.value.decode()
    return nn.value, dp.value


@pytest.mark.parametrize("n", [0, 1, 2, 4, 5, 17, 1000, 100000])
def test_soup_layouts(checker, n):
    nodes, depth = run(checker, scenes.triangle_soup(n, seed=n + 1) if n else np.zeros((0, 9), np.float32))
    assert nodes >= 1 and depth <= 60


def test_coincident_centroids_and_degenerate(checker):
    tri = np.array([0, 0, 0, 1, 0, 0, 0, 1, 0], np.float32)
    run(checker, np.tile(tri, (5000, 1)))                 # all identical
    run(checker, np.zeros((300, 9), np.float32))          # all degenerate points


def test_terrain_layout(checker):
    d = scenes.terrain_scene(64, 36, 1, 8, cells=128, n_spheres=8)
    tv, _, _, _ = d.flatten()
    nodes, depth = run(checker, tv)
    assert depth <= 60
