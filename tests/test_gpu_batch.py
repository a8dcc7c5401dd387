"""Batched rendering: many uneven jobs in one wavefront (stage kernels per
iteration, or the whole loop in one cooperative launch) or one persistent
megakernel launch, optionally through CUDA graphs, must give each job the
same film as rendering it alone."""
import numpy as np
import pytest

from kazen_proto_gb300 import api, autotune, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def jobs():
    js = scenes.batch_jobs(n_jobs=7, seed=3, tri_range=(2000, 20000), resolutions=(16, 32, 48), spps=(2, 4, 8),
                           depths=(4, 8))
    return scenes.build_batch_scenes(js, workers=4)


def rel_mse(a, b, eps=1e-2):
    return float(np.mean((np.asarray(a, np.float64) - b) ** 2 / (np.asarray(b, np.float64) ** 2 + eps)))


def singles(jobs):
    out = []
    for j in jobs:
        r = api.Renderer(spp=j["spp"], max_depth=j["max_depth"], seed=j["seed"])
        out.append((r.render(j["scene"], j["camera"], j["width"], j["height"]), r.last_stats))
    return out


MEGA = api.BATCH_MEGAKERNEL
WAVE = api.BATCH_WAVEFRONT
PERS = api.BATCH_PERSISTENT


@pytest.mark.parametrize("cfg", [dict(mode=WAVE, use_graph=True),
                                 dict(mode=WAVE, block_size=128, wavefront_size=4096, use_graph=False),
                                 dict(mode=WAVE, block_size=64, wavefront_size=1000, use_graph=True),
                                 dict(mode=WAVE, wavefront_size=3000, refill_period=2, use_graph=True),
                                 dict(mode=WAVE, block_size=128, wavefront_size=5000, refill_period=3,
                                      use_graph=False),
                                 dict(mode=MEGA, block_size=128, ctas_per_sm=2, refill_period=1, use_graph=True),
                                 dict(mode=MEGA, block_size=64, ctas_per_sm=1, refill_period=4, use_graph=False),
                                 dict(mode=MEGA, block_size=256, ctas_per_sm=4, refill_period=2, use_graph=True),
                                 dict(mode=PERS, use_graph=True),
                                 dict(mode=PERS, wavefront_size=1000, use_graph=False),
                                 dict(mode=PERS, wavefront_size=3000, refill_period=3, use_graph=True)])
def test_batch_matches_single_renders(gpu, jobs, cfg):
    imgs, st = api.render_batch(jobs, api.batch_config(**cfg))
    ref = singles(jobs)
    for img, (r, rs) in zip(imgs, ref):
        assert rel_mse(img, r) < 1e-10
    assert st["paths"] == sum(j["width"] * j["height"] * j["spp"] for j in jobs)
    assert st["path_bounces"] == sum(rs["path_bounces"] for _, rs in ref)
    assert st["shadow_rays"] == sum(rs["shadow_rays"] for _, rs in ref)
    assert st["device_ms"] > 0


def test_autotuner_picks_a_candidate(gpu, jobs, tmp_path, monkeypatch):
    monkeypatch.setattr(autotune, "PATH", str(tmp_path / "autotune.json"))
    best, table = autotune.tune(jobs, reps=1)
    assert len(table) == len(autotune.candidates())
    assert best in [c for c, _ in table] and autotune.load() == best
    imgs, _ = api.render_batch(jobs, autotune.tuned_config())
    assert all(np.isfinite(i).all() for i in imgs)


def test_batch_rejects_unknown_mode(gpu, jobs):
    with pytest.raises(api.N.KazenError):
        api.render_batch(jobs[:1], api.batch_config(mode=7))
