"""Learned path guiding on the GPU: the network's forward pass and gradients
against the numpy restatement (with the kernels' BF16 rounding points), that
training reduces the loss, that guided images stay unbiased, and that the
trained network lowers the error of the narrow-aperture scene."""
import numpy as np
import pytest

from kazen_proto_gb300 import api, scenes
from oracle import guide_oracle as G

pytestmark = pytest.mark.gpu


def rand_batch(rng, n):
    p01 = rng.random((n, 3)).astype(np.float32)
    nrm = rng.standard_normal((n, 3)).astype(np.float32)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    d = rng.standard_normal((n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    w = (rng.random(n) + 0.1).astype(np.float32)
    return p01, nrm.astype(np.float32), d.astype(np.float32), w


def test_forward_matches_restatement(gpu):
    rng = np.random.default_rng(0)
    g = api.Guide(seed=3)
    p = G.init_params(5)
    g.set_params(p)
    assert np.array_equal(g.params(), p)
    p01, nrm, _, _ = rand_batch(rng, 5000)
    raw = g.forward(p01, nrm)
    ref = G.forward(p, p01, nrm, use_bf16=True)["O"]
    err = np.abs(raw - ref)
    assert err.max() <= 2e-2 * np.abs(ref).max() + 1e-3, err.max()
    assert np.median(err) <= 1e-3 * np.abs(ref).max() + 1e-5


@pytest.mark.parametrize("n", [16, 1000, 70000])
def test_gradient_matches_restatement(gpu, n):
    rng = np.random.default_rng(n)
    g = api.Guide(seed=1)
    p = G.init_params(2)
    g.set_params(p)
    p01, nrm, d, w = rand_batch(rng, n)
    loss, grad = g.train_step(p01, nrm, d, w, apply=False, want_grad=True)
    loss_o, grad_o = G.loss_and_grad(p, p01, nrm, d, w, 1.0 / n, use_bf16=True)
    assert abs(loss - loss_o) <= 1e-3 * abs(loss_o) + 1e-6, (loss, loss_o)
    rel = np.linalg.norm(grad - grad_o) / np.linalg.norm(grad_o)
    assert rel < 2e-2, rel
    # and the restatement's BF16 gradient is close to its exact (float64) gradient
    _, grad_exact = G.loss_and_grad(p.astype(np.float64), p01, nrm, d, w, 1.0 / n, use_bf16=False)
    assert np.linalg.norm(grad - grad_exact) / np.linalg.norm(grad_exact) < 0.1
    # apply=False leaves the parameters untouched
    assert np.array_equal(g.params(), p)


def test_training_fits_a_direction_field(gpu):
    """Directions drawn from a vMF whose mean depends on position: Adam on the
    GPU drives -log q well below its starting value and below the uniform
    sphere's log(4 pi)."""
    rng = np.random.default_rng(7)
    g = api.Guide(seed=11)
    c = np.array([0.5, 0.8, 0.5], np.float32)
    losses = []
    for it in range(300):
        p01 = rng.random((4096, 3)).astype(np.float32)
        nrm = np.tile(np.array([0, 1, 0], np.float32), (4096, 1))
        mu = c - p01
        mu /= np.linalg.norm(mu, axis=1, keepdims=True)
        # sample vMF(mu, 20) by perturbing and renormalising (a concentrated lobe)
        d = mu + 0.15 * rng.standard_normal((4096, 3)).astype(np.float32)
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        losses.append(g.train_step(p01, nrm, d.astype(np.float32), np.ones(4096, np.float32), lr=3e-3))
    first, last = np.mean(losses[:10]), np.mean(losses[-10:])
    assert last < first - 1.0, (first, last)
    assert last < np.log(4 * np.pi) - 1.5, last


def rel_mse(img, ref, eps=1e-2):
    return float(np.mean((np.asarray(img, np.float64) - ref) ** 2 / (ref ** 2 + eps)))


R = 64


@pytest.fixture(scope="module")
def slit():
    d = scenes.slit_room_scene(R, R, spp=16, max_depth=10, n_spheres=32)
    s = d.build()
    ref = api.Renderer(spp=16384, max_depth=10, seed=99).render(s, d.camera, R, R, fp64=True)[1]
    return d, s, ref


def test_guided_render_is_unbiased(gpu, slit):
    d, s, ref = slit
    g = api.Guide(seed=4)
    img, _, st, gst = api.render_guided(s, g, d.camera, R, R, spp=512, max_depth=10, seed=5,
                                        gcfg=api.guide_config(spp_per_pass=8))
    assert gst["spp_done"] == 512 and gst["train_steps"] > 0 and np.isfinite(img).all()
    # image mean within 3 % of the 16,384-spp plain reference
    assert abs(img.mean() / ref.mean() - 1) < 0.03, (img.mean(), ref.mean())
    # a frozen, untrained network also stays unbiased
    g2 = api.Guide(seed=6)
    img2, _, _, gst2 = api.render_guided(s, g2, d.camera, R, R, spp=512, max_depth=10, seed=8,
                                         gcfg=api.guide_config(train=False))
    assert gst2["train_steps"] == 0
    assert abs(img2.mean() / ref.mean() - 1) < 0.03, (img2.mean(), ref.mean())


def test_trained_guide_reduces_error(gpu, slit):
    """What the trained network gains: after training, at equal spp, guided
    rendering of the narrow-aperture scene has lower relMSE than plain."""
    d, s, ref = slit
    g = api.Guide(seed=9)
    _, _, _, gst = api.render_guided(s, g, d.camera, R, R, spp=4096, max_depth=10, seed=1,
                                     gcfg=api.guide_config(spp_per_pass=4, learning_rate=1e-2))
    assert gst["train_steps"] == 1024
    errs_g, errs_p = [], []
    for k in range(4):
        gi, _, _, _ = api.render_guided(s, g, d.camera, R, R, spp=64, max_depth=10, seed=100 + k,
                                        gcfg=api.guide_config(train=False, spp_per_pass=64))
        pi = api.Renderer(spp=64, max_depth=10, seed=200 + k).render(s, d.camera, R, R)
        errs_g.append(rel_mse(gi, ref))
        errs_p.append(rel_mse(pi, ref))
    assert np.mean(errs_g) < 0.75 * np.mean(errs_p), (errs_g, errs_p)
