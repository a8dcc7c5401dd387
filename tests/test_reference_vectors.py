"""The CPU restatement against vectors that kazen_proto's own code computed.

tests/golden/reference_closure_vectors.npz holds the output of
oracle/ref_harness.cpp, compiled from the reference's header-only closure math
(microfacet.h, fresnel.h, utils.h, sampling.h) by
tests/golden/make_reference_closure_vectors.py. These tests pin the
restatement's microfacet terms, Fresnel functions, refraction, shading frame,
warps and the KpGloss / KpPrincipleSpecularReflection / Diffuse evaluations
to those executed values within 1e-5 relative (absolute floor 1e-7); the GPU
lobes are pinned to the same vectors in tests/test_gpu_closures.py."""
import os

import numpy as np
import pytest

from kazen_proto_gb300 import api

HERE = os.path.dirname(os.path.abspath(__file__))
RTOL, ATOL = 1e-5, 1e-7


@pytest.fixture(scope="module")
def vec():
    return dict(np.load(os.path.join(HERE, "golden", "reference_closure_vectors.npz")))


def close(a, b, rtol=RTOL, atol=ATOL):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b) <= np.maximum(atol, rtol * np.abs(b))


@pytest.mark.parametrize("dist,table", [(0, "mdf_ggx"), (1, "mdf_beckmann")])
def test_microfacet_terms(oracle_mod, vec, dist, table):
    t = vec[table]
    got = oracle_mod.scalar_terms("mdf_terms", t[:, :11], 7, dist=dist)
    ok = close(got, t[:, 11:])
    assert ok.all(), (np.argwhere(~ok)[:5], got[~ok.all(1)][:3], t[~ok.all(1), 11:][:3])


def test_fresnel_terms(oracle_mod, vec):
    t = vec["fresnel"]
    got = oracle_mod.scalar_terms("fresnel_terms", t[:, :4], 4)
    # columns of the table: refl_dielectric at 5, utils fresnel at 7, schlick at 8, schlick_weight at 9
    want = t[:, [5, 7, 8, 9]]
    assert close(got, want).all()


def test_refract(oracle_mod, vec):
    t = vec["refract"]
    got = oracle_mod.scalar_terms("refract", t[:, :7], 3)
    assert close(got, t[:, 7:], atol=1e-6).all()


def test_frame(oracle_mod, vec):
    t = vec["frame"]
    got = oracle_mod.scalar_terms("frame", t[:, :6], 9)
    assert close(got, t[:, 6:], atol=1e-6).all()


def test_cosine_warp_and_power_heuristic(oracle_mod, vec):
    t = vec["warps"]
    got = oracle_mod.scalar_terms("warps", t[:, :4], 4)
    # to_cosine_hemisphere returns its cosine in z; the restatement's frame is y-up
    ref_dir = t[:, [4, 6, 5]]
    assert close(got[:, :3], ref_dir, atol=2e-6).all()
    assert close(got[:, 3], t[:, 12]).all()


def lobes_kpgloss(t):
    return np.array([api.microfacet("beckmann" if d == 1 else "ggx", float(ax), float(ay), float(eta), 0)
                     for d, ax, ay, eta in zip(t[:, 0], t[:, 7], t[:, 8], t[:, 9])])


def test_kpgloss_eval_reference_convention(oracle_mod, vec):
    t = vec["kpgloss"]
    lb = lobes_kpgloss(t)
    f, pdf = oracle_mod.closure_eval(lb, t[:, 1:4], t[:, 4:7], convention=0)
    assert close(f[:, 0], t[:, 10]).all() and close(f[:, 2], t[:, 10]).all()
    assert close(pdf, t[:, 11]).all()


def test_principle_specular_eval_reference_convention(oracle_mod, vec):
    t = vec["principle_specular"]
    lb = np.array([api.principle_specular(tuple(float(x) for x in row[9:12]), float(row[6]), float(row[8]),
                                          0.0, yalpha=float(row[7])) for row in t])
    f, pdf = oracle_mod.closure_eval(lb, t[:, 0:3], t[:, 3:6], convention=0)
    assert close(f, t[:, 12:15]).all()
    assert close(pdf, t[:, 15]).all()


def test_diffuse_eval_reference_convention(oracle_mod, vec):
    t = vec["diffuse"]
    n = len(t)
    wi = np.tile(np.array([[0.3, 0.8, 0.52]], np.float32), (n, 1))
    wi /= np.linalg.norm(wi, axis=1, keepdims=True)
    f, pdf = oracle_mod.closure_eval(np.array([api.diffuse()] * n), wi, t[:, :3], convention=0)
    assert close(f[:, 0], t[:, 3]).all() and close(pdf, t[:, 3]).all()
