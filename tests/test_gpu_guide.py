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


@pytest.mark.parametrize("mode", ["fused", "tc"])
@pytest.mark.parametrize("n", [64, 1000, 70000, 1 << 18])
def test_tcgen05_training_matches_warp_mma(gpu, n, mode, monkeypatch):
    """The tcgen05 training paths against the warp-level mma.sync kernels on
    the same samples: "tc" keeps the warp-level forward/backward and runs the
    weight gradients on tcgen05 (TMA-staged records, TMEM accumulators) -- the
    same BF16 products summed in another order, so FP32 rounding apart;
    "fused" (the default) runs the whole step in one tcgen05 kernel, whose
    layer sums in another order can flip a BF16 rounding of an activation, so
    it agrees to a few 1e-3 of the gradient's norm. Row counts that are not a
    multiple of the tiles exercise the tails."""
    rng = np.random.default_rng(n + 1)
    g = api.Guide(seed=1)
    p = G.init_params(4)
    g.set_params(p)
    p01, nrm, d, w = rand_batch(rng, n)
    monkeypatch.setenv("KZ_GUIDE_TRAIN", mode)
    loss_tc, grad_tc = g.train_step(p01, nrm, d, w, apply=False, want_grad=True)
    monkeypatch.setenv("KZ_GUIDE_TRAIN", "mma")
    loss_mma, grad_mma = g.train_step(p01, nrm, d, w, apply=False, want_grad=True)
    monkeypatch.delenv("KZ_GUIDE_TRAIN")
    live = np.ones_like(grad_tc, bool)
    live[:64 * 64] = (np.arange(64 * 64) % 64) < 51  # layer-1 padding columns are not parameters
    scale = np.abs(grad_mma[live]).max()
    nrm_mma = np.linalg.norm(grad_mma[live])
    b = slice(64 * 64, 64 * 64 + 64)  # layer-1 biases: the ones block of the tensor-core product
    if mode == "tc":
        # the forward/backward kernel is shared (its loss is an atomic sum)
        assert abs(loss_tc - loss_mma) <= 1e-5 * abs(loss_mma) + 1e-7
        assert np.abs(grad_tc[live] - grad_mma[live]).max() <= 1e-4 * scale + 1e-7
        assert np.linalg.norm(grad_tc[live] - grad_mma[live]) <= 1e-4 * nrm_mma + 1e-7
        assert np.allclose(grad_tc[b], grad_mma[b], rtol=1e-4, atol=1e-6 * scale)
    else:
        assert abs(loss_tc - loss_mma) <= 1e-3 * abs(loss_mma) + 1e-6, (loss_tc, loss_mma)
        assert np.linalg.norm(grad_tc[live] - grad_mma[live]) <= 5e-3 * nrm_mma, \
            np.linalg.norm(grad_tc[live] - grad_mma[live]) / nrm_mma
        assert np.linalg.norm(grad_tc[b] - grad_mma[b]) <= 5e-3 * np.linalg.norm(grad_mma[b]) + 1e-7


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
    """The slit room at 64 x 64 and a plain FP64 reference rendered as 16
    independent parts of 1024 spp: its mean and the per-pixel variance of
    that mean."""
    d = scenes.slit_room_scene(R, R, spp=16, max_depth=10, n_spheres=32)
    s = d.build()
    parts = np.stack([api.Renderer(spp=1024, max_depth=10, seed=99 + k).render(s, d.camera, R, R, fp64=True)[1]
                      for k in range(16)])
    ref = parts.mean(0)
    ref_var = parts.var(0, ddof=1) / len(parts)
    return d, s, ref, ref_var


def assert_unbiased(imgs, ref, ref_var, what):
    """Independent estimates of the same image against the reference: the
    per-pixel difference of the means, scaled by its standard error (from the
    estimates' own spread and the reference's), must look like noise over the
    whole image and in every 8 x 8 block, so a bias confined to a region
    fails as well as a global one."""
    imgs = np.asarray(imgs, np.float64)
    k = len(imgs)
    mean = imgs.mean(0).sum(-1)  # luminance-like sum of the channels
    var = (imgs.sum(-1).var(0, ddof=1) / k) + ref_var.sum(-1)
    diff = mean - ref.sum(-1)
    se_all = np.sqrt(var.sum()) / diff.size
    assert abs(diff.mean()) < 4.0 * se_all, (what, diff.mean(), se_all)
    b = 8
    db = diff.reshape(R // b, b, R // b, b).mean(axis=(1, 3))
    sb = np.sqrt(var.reshape(R // b, b, R // b, b).sum(axis=(1, 3))) / (b * b)
    zb = db / sb
    assert np.abs(zb).max() < 4.5, (what, np.abs(zb).max(), np.unravel_index(np.abs(zb).argmax(), zb.shape))
    z = diff / np.sqrt(var + 1e-30)
    assert 0.45 < np.median(np.abs(z)) < 0.95, (what, np.median(np.abs(z)))  # 0.674 for unit noise


def test_guided_render_is_unbiased(gpu, slit):
    d, s, ref, ref_var = slit
    # while it trains: every pass uses the network of that moment
    g = api.Guide(seed=4)
    img, _, st, gst = api.render_guided(s, g, d.camera, R, R, spp=512, max_depth=10, seed=5,
                                        gcfg=api.guide_config(spp_per_pass=8))
    assert gst["spp_done"] == 512 and gst["train_steps"] > 0 and np.isfinite(img).all()
    # trained and frozen: eight independent renders
    frozen = [api.render_guided(s, g, d.camera, R, R, spp=512, max_depth=10, seed=50 + k,
                                gcfg=api.guide_config(train=False, spp_per_pass=64))[0] for k in range(8)]
    assert_unbiased(frozen, ref, ref_var, "trained")
    # an untrained network (random weights) also stays unbiased
    g2 = api.Guide(seed=6)
    untrained = [api.render_guided(s, g2, d.camera, R, R, spp=512, max_depth=10, seed=80 + k,
                                   gcfg=api.guide_config(train=False, spp_per_pass=64))[0] for k in range(8)]
    assert_unbiased(untrained, ref, ref_var, "untrained")
    # and the check does fail on a biased image: 10 % darker in one corner
    biased = [f.copy() for f in frozen]
    for f in biased:
        f[:16, :16] *= 0.90
    with pytest.raises(AssertionError):
        assert_unbiased(biased, ref, ref_var, "planted bias")


def test_guided_render_is_unbiased_at_depth_2(gpu, slit):
    """Depth 2 (direct light and one bounce), where half of the shaded
    vertices are the last one: the light sample there has no sampled
    direction after it as its MIS partner, so it must weigh like the plain
    tracer's, or the guided image converges to another value than plain."""
    d, s, _, _ = slit
    parts = np.stack([api.Renderer(spp=1024, max_depth=2, seed=300 + k).render(s, d.camera, R, R, fp64=True)[1]
                      for k in range(16)])
    ref, ref_var = parts.mean(0), parts.var(0, ddof=1) / len(parts)
    g = api.Guide(seed=12)
    api.render_guided(s, g, d.camera, R, R, spp=512, max_depth=2, seed=7, gcfg=api.guide_config(spp_per_pass=8))
    frozen = [api.render_guided(s, g, d.camera, R, R, spp=512, max_depth=2, seed=400 + k,
                                gcfg=api.guide_config(train=False, spp_per_pass=64))[0] for k in range(8)]
    assert_unbiased(frozen, ref, ref_var, "trained, depth 2")


def test_trained_guide_reduces_error(gpu, slit):
    """What the trained network gains: after training, at equal spp, guided
    rendering of the narrow-aperture scene has lower relMSE than plain."""
    d, s, ref, _ = slit
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
