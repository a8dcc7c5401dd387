"""CPU checks of the guiding network's restatement (oracle/guide_oracle.py):
its analytic gradient against central finite differences in float64, and
the vMF mixture's pdf normalisation (anchor-point lobes, any box extent)."""
import numpy as np
import pytest

from oracle import guide_oracle as G


def batch(rng, n):
    p01 = rng.random((n, 3))
    nrm = rng.standard_normal((n, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    d = rng.standard_normal((n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    w = rng.random(n) + 0.1
    return p01, nrm, d, w


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = G.init_params(1).astype(np.float64)
    p01, nrm, d, w = batch(rng, 64)
    loss, g = G.loss_and_grad(p, p01, nrm, d, w, 1.0 / 64, use_bf16=False)
    idx = np.concatenate([rng.choice(np.arange(0, 4096).reshape(64, 64)[:, :51].reshape(-1), 20),
                          rng.integers(4096, G.N_PARAMS, 60)])
    for i in idx:
        h = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        lp, _ = G.loss_and_grad(pp, p01, nrm, d, w, 1.0 / 64, use_bf16=False)
        lm, _ = G.loss_and_grad(pm, p01, nrm, d, w, 1.0 / 64, use_bf16=False)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-5 + 1e-4 * abs(fd), (i, fd, g[i])


def test_mixture_pdf_integrates_to_one():
    rng = np.random.default_rng(1)
    raw = rng.standard_normal((1, 40)) * 2.0
    m = 400000
    d = rng.standard_normal((m, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    p01 = np.repeat(rng.random((1, 3)), m, 0)
    for ext in ((1.0, 1.0, 1.0), (3.0, 0.5, 2.0)):
        q = G.pdf(np.repeat(raw, m, 0), d, p01, ext)
        assert abs(q.mean() * 4 * np.pi - 1.0) < 0.02


def test_gradient_with_box_extent_matches_finite_differences():
    """The anchor gradient carries the box extent (d axis / d anchor = diag(ext))."""
    rng = np.random.default_rng(3)
    raw = rng.standard_normal((32, 40))
    p01, _, d, w = batch(rng, 32)
    ext = (3.0, 0.5, 2.0)
    _, g = G.nll_and_grad(raw, d, w, p01, ext)
    for i in rng.integers(0, 40, 25):
        h = 1e-6
        rp, rm = raw.copy(), raw.copy()
        rp[:, i] += h
        rm[:, i] -= h
        lp = (w * G.nll_and_grad(rp, d, w, p01, ext)[0]).sum()
        lm = (w * G.nll_and_grad(rm, d, w, p01, ext)[0]).sum()
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[:, i].sum()) <= 1e-5 + 1e-4 * abs(fd), (i, fd, g[:, i].sum())


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.14159], np.float32)
    y = G.bf16(x)
    assert y[0] == 1.0 and y[1] == 1.0 and y[2] == np.float32(1.0078125)
    assert abs(y[3] + 3.140625) < 1e-6
