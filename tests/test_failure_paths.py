"""Failure paths that can be exercised without faulting a GPU.

* Traversal stack overflow: a test build of the library with a two-entry
  traversal stack (kazen_proto_gb300/build.py, variant "stack2"; the BVH
  builder's depth cap is unchanged, so ordinary trees still build) drives the
  closest-hit and any-hit kernels into their overflow path. They abort the
  ray (it misses), record KZ_ERR_STACK in the device status word, and the
  call returns that status; the scene stays usable.
* Device allocation failure, injected on the host (KZ_FAIL_ALLOC_AFTER=N:
  allocations after the first N fail as an out-of-memory would): the call
  that needed the memory returns KZ_ERR_OOM and the handle can be destroyed.
* Guiding checkpoint: weights, Adam moments and step count saved and
  restored, and training resumed from them continues as the original guide.

Each library variant and each injected failure runs in its own process."""
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

from kazen_proto_gb300 import _native as N
from kazen_proto_gb300 import api

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run_child(code, env_extra):
    env = dict(os.environ)
    env.update(env_extra)
    r = subprocess.run([sys.executable, "-c", textwrap.dedent(code)], capture_output=True, text=True, env=env,
                       cwd=ROOT, timeout=600)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    return r.stdout


def test_traversal_stack_overflow_reports_kz_err_stack(gpu):
    from kazen_proto_gb300 import build as kbuild
    lib = kbuild.build(variant="stack2")
    out = run_child("""
        import sys
        sys.path.insert(0, %r)
        import numpy as np
        from kazen_proto_gb300 import _native as N, api, scenes
        tv = scenes.triangle_soup(20000, seed=1)
        s = scenes.soup_desc(tv).build()
        rays = scenes.soup_rays(4096, seed=2)
        try:
            s.intersect(rays)
            print("closest: no error")
        except N.KazenError as e:
            print("closest:", e.code)
        try:
            s.occluded(rays)
            print("any: no error")
        except N.KazenError as e:
            print("any:", e.code)
        # the handle still answers: a ray that misses the soup's box needs no stack
        far = api.make_rays([[5.0, 5.0, 5.0]], [[1.0, 0.0, 0.0]])
        h = s.intersect(far)
        print("after:", int(h["prim_id"][0]))
        d = scenes.soup_render_scene(20000, seed=3)
        try:
            api.Renderer(spp=1, max_depth=3).render(d.build(), d.camera, 32, 32)
            print("render: no error")
        except N.KazenError as e:
            print("render:", e.code)
    """ % ROOT, {"KZ_LIBRARY": lib})
    lines = dict(l.split(": ", 1) for l in out.strip().splitlines())
    assert lines["closest"] == str(N.KZ_ERR_STACK), out
    assert lines["any"] == str(N.KZ_ERR_STACK), out
    assert lines["after"] == str(0xFFFFFFFF), out
    # the wavefront renderer's trace stage reports the same status
    assert lines["render"] == str(N.KZ_ERR_STACK), out


@pytest.mark.parametrize("after", [0, 2])
def test_injected_allocation_failure_returns_oom(gpu, after):
    out = run_child("""
        import sys
        sys.path.insert(0, %r)
        from kazen_proto_gb300 import _native as N, api, scenes
        d = scenes.box_scene(16, 16, spp=1, max_depth=3)
        try:
            sc = d.build()
            print("build: ok")
            api.Renderer(spp=1, max_depth=3).render(sc, d.camera, 16, 16)
            print("render: ok")
        except N.KazenError as e:
            print("build:", e.code, str(e))
        print("closed")
    """ % ROOT, {"KZ_FAIL_ALLOC_AFTER": str(after)})
    # with 0 the scene build's first allocation fails, with 2 a later one
    # (the build or the render's scratch): either way KZ_ERR_OOM, no crash
    assert "build: %d" % N.KZ_ERR_OOM in out and "KZ_FAIL_ALLOC_AFTER" in out, out
    assert "closed" in out


def test_guide_state_checkpoint_and_resume(gpu):
    rng = np.random.default_rng(3)

    def batch():
        p01 = rng.random((4096, 3)).astype(np.float32)
        nrm = np.tile(np.array([0, 1, 0], np.float32), (4096, 1))
        d = rng.standard_normal((4096, 3)).astype(np.float32)
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        return p01, nrm, d, np.ones(4096, np.float32)

    batches = [batch() for _ in range(8)]
    a = api.Guide(seed=5)
    for b in batches[:5]:
        a.train_step(*b, lr=1e-2)
    (w, m, v), step = a.state()
    assert step == 5 and np.abs(m).max() > 0 and v.min() >= 0 and np.abs(v).max() > 0
    b = api.Guide(seed=9)
    b.set_state(w, m, v, step)
    (w2, m2, v2), step2 = b.state()
    assert step2 == 5 and np.array_equal(w2, w) and np.array_equal(m2, m) and np.array_equal(v2, v)
    for bt in batches[5:]:
        a.train_step(*bt, lr=1e-2)
        b.train_step(*bt, lr=1e-2)
    pa, pb = a.params(), b.params()
    # same state, same batches: the same weights up to the order of the
    # gradient's atomic sums
    assert np.abs(pa - pb).max() <= 1e-5 * np.abs(pa).max()
    # a guide restored without its moments does not resume the same way
    c = api.Guide(seed=9)
    c.set_params(w)
    for bt in batches[5:]:
        c.train_step(*bt, lr=1e-2)
    assert np.abs(c.params() - pa).max() > 10 * np.abs(pa - pb).max() + 1e-7
    with pytest.raises(N.KazenError):
        b.set_state(w, m, -np.ones_like(v), 1)
    a.close()
    b.close()
    c.close()
