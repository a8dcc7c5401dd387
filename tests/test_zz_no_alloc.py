"""kz_li_batch_noalloc: the Li batch for callers that cannot allocate device
memory while they render (a host application or framework that owns the GPU
memory budget through its own allocator, or a loop that cannot absorb
cudaMalloc's implicit synchronisation). Its wavefront scratch is a static
device array inside the library; these tests call it through the C ABI and
check it against kz_li_batch, the entry point that allocates its scratch.

This file is collected last on purpose: run alone in a fresh process it does
the first-call set-up itself; run after the other tests it reuses a library
whose static array already holds an earlier call's contents."""
import ctypes as C

import numpy as np
import pytest

from kazen_proto_gb300 import _native as N
from kazen_proto_gb300 import api, scenes

pytestmark = pytest.mark.gpu

RTOL, ATOL = 1e-5, 1e-6  # the closure-level tolerance of the other GPU tests


def camera_rays(d, n, seed):
    rng = np.random.default_rng(seed)
    tgt = np.stack([rng.uniform(0.05, 0.95, n), rng.uniform(0.05, 0.95, n), np.full(n, 1.0)], -1)
    return api.make_rays(np.asarray(d.camera.eye, np.float32), tgt.astype(np.float32))


def li_batch(scene, dr, cfg, torch):
    out = torch.empty((dr.shape[0], 3), dtype=torch.float32, device="cuda")
    st = N.KzRenderStats()
    N.check(N.lib().kz_li_batch(scene.handle, C.c_void_p(dr.data_ptr()), dr.shape[0], C.byref(cfg),
                                C.c_void_p(out.data_ptr()), N.KZ_MEM_DEVICE, C.byref(st)))
    torch.cuda.synchronize()
    return out.cpu().numpy(), st


def li_noalloc(scene, dr, cfg, torch, out=None):
    if out is None:
        out = torch.full((dr.shape[0], 3), float("nan"), dtype=torch.float32, device="cuda")
    st = N.KzRenderStats()
    N.check(N.lib().kz_li_batch_noalloc(scene.handle, C.c_void_p(dr.data_ptr()), dr.shape[0], C.byref(cfg),
                                        C.c_void_p(out.data_ptr()), C.byref(st)))
    torch.cuda.synchronize()
    return out.cpu().numpy(), st


def test_noalloc_li_batch_matches_allocating_entry_point(gpu):
    torch = pytest.importorskip("torch")
    d = scenes.box_scene(16, 16, spp=1, max_depth=5)
    s = d.build()
    n = 40000  # more rays than the 16,384-path wavefront: paths stream through it
    dr = torch.from_numpy(camera_rays(d, n, 1).view(np.float32).reshape(-1, 8).copy()).cuda()
    cfg = api.render_config(spp=1, max_depth=5, seed=7)
    ref, st_ref = li_batch(s, dr, cfg, torch)
    assert np.isfinite(ref).all() and ref.mean() > 0
    # two calls in a row: the second starts from the first call's leftovers
    a, st_a = li_noalloc(s, dr, cfg, torch)
    b, st_b = li_noalloc(s, dr, cfg, torch)
    for got, st in ((a, st_a), (b, st_b)):
        assert np.allclose(got, ref, rtol=RTOL, atol=ATOL), np.abs(got - ref).max()
        assert st.path_bounces == st_ref.path_bounces and st.shadow_rays == st_ref.shadow_rays
        assert st.paths == n


def test_noalloc_other_seed_then_back(gpu):
    torch = pytest.importorskip("torch")
    d = scenes.box_scene(16, 16, spp=1, max_depth=5)
    s = d.build()
    dr = torch.from_numpy(camera_rays(d, 5000, 2).view(np.float32).reshape(-1, 8).copy()).cuda()
    cfg = api.render_config(spp=1, max_depth=5, seed=3)
    ref, _ = li_batch(s, dr, cfg, torch)
    other, _ = li_noalloc(s, dr, api.render_config(spp=1, max_depth=5, seed=4), torch)
    assert not np.allclose(other, ref, rtol=RTOL, atol=ATOL)
    again, _ = li_noalloc(s, dr, cfg, torch)
    assert np.allclose(again, ref, rtol=RTOL, atol=ATOL)


def test_noalloc_rejects_oversized_wavefront(gpu):
    torch = pytest.importorskip("torch")
    d = scenes.box_scene(16, 16, spp=1, max_depth=5)
    s = d.build()
    dr = torch.from_numpy(camera_rays(d, 100, 3).view(np.float32).reshape(-1, 8).copy()).cuda()
    cfg = api.render_config(spp=1, max_depth=5, seed=1, wavefront_size=N.KZ_LI_NOALLOC_MAX_WAVEFRONT + 1)
    with pytest.raises(N.KazenError) as e:
        li_noalloc(s, dr, cfg, torch)
    assert e.value.code == N.KZ_ERR_INVALID_ARG and "maximum" in str(e.value)
    ok, _ = li_noalloc(s, dr, api.render_config(spp=1, max_depth=5, seed=1,
                                                wavefront_size=N.KZ_LI_NOALLOC_MAX_WAVEFRONT), torch)
    ref, _ = li_batch(s, dr, api.render_config(spp=1, max_depth=5, seed=1), torch)
    assert np.allclose(ok, ref, rtol=RTOL, atol=ATOL)


def cone_rays(eye, lookat, n, seed, spread=0.35):
    """Rays from the camera eye towards jittered points around the look-at point."""
    rng = np.random.default_rng(seed)
    eye = np.asarray(eye, np.float32)
    tgt = np.asarray(lookat, np.float32)[None, :] + rng.uniform(-spread, spread, (n, 3)).astype(np.float32)
    return api.make_rays(eye, tgt)


@pytest.mark.parametrize("case", ["count", "nee_only", "bsdf_only", "block128", "textured_room"])
def test_noalloc_matches_under_flags_variants_and_block_sizes(gpu, case):
    torch = pytest.importorskip("torch")
    import os

    from kazen_proto_gb300 import scene_xml
    if case == "textured_room":
        here = os.path.dirname(os.path.abspath(__file__))
        d = scene_xml.load(os.path.join(here, "golden", "scenes", "textured_room", "scene.xml")).desc
        rays = cone_rays(d.camera.eye, d.camera.lookat, 30000, 5)
    else:
        d = scenes.box_scene(16, 16, spp=1, max_depth=5)
        rays = camera_rays(d, 30000, 4)
    s = d.build()
    dr = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).cuda()
    flags = {"count": N.KZ_RENDER_FLAG_COUNT, "nee_only": N.KZ_RENDER_FLAG_NEE_ONLY,
             "bsdf_only": N.KZ_RENDER_FLAG_BSDF_ONLY}.get(case, 0)
    block = 128 if case == "block128" else 0
    cfg = api.render_config(spp=1, max_depth=5, seed=11, block_size=block, flags=flags)
    ref, st_ref = li_batch(s, dr, cfg, torch)
    assert np.isfinite(ref).all() and ref.mean() > 0
    for _ in range(2):  # two calls in a row on the shared array
        got, st = li_noalloc(s, dr, cfg, torch)
        assert np.allclose(got, ref, rtol=RTOL, atol=ATOL), np.abs(got - ref).max()
        assert st.path_bounces == st_ref.path_bounces and st.shadow_rays == st_ref.shadow_rays
        if case == "count":
            # fetch counters accumulate in the static array over the call's
            # iterations and are cleared at the start of the next call
            assert st.closest_node_fetches > 0 and st.shadow_node_fetches > 0
            assert (st.closest_node_fetches, st.closest_tri_fetches, st.shadow_node_fetches,
                    st.shadow_tri_fetches) == (st_ref.closest_node_fetches, st_ref.closest_tri_fetches,
                                               st_ref.shadow_node_fetches, st_ref.shadow_tri_fetches)
    s.close()
