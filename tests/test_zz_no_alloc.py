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
