"""CPU-side tests of the C-ABI library: it builds for sm_103a, loads, exports
every entry point the header declares, and validates host input before any
device work. No compute calls are made without a GPU."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from kazen_proto_gb300 import _native as N
from kazen_proto_gb300 import api

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "kazen_gb300.h")


def header_functions():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(kz_[a-z_0-9]+)\s*\(", txt)))


def test_header_declares_the_boundary():
    fns = header_functions()
    for f in ["kz_scene_create", "kz_scene_add_mesh", "kz_scene_build", "kz_intersect_closest", "kz_intersect_any",
              "kz_li_batch", "kz_render", "kz_closure_eval_batch", "kz_closure_sample_batch", "kz_last_error_string"]:
        assert f in fns


def test_library_exports_every_declared_symbol(native_lib):
    for f in header_functions():
        assert hasattr(native_lib, f), f
    assert set(header_functions()) == set(N.SIGNATURES), "ctypes signature table out of sync with the header"


def test_library_is_built_for_sm_103a():
    from kazen_proto_gb300 import build as kb
    assert "arch=compute_103a,code=sm_103a" in " ".join(kb.ARCH)
    assert "--fmad=false" in kb.common_flags()


def test_struct_layouts_match_header():
    assert C.sizeof(N.KzRay) == 32
    assert C.sizeof(N.KzLobe) == 64
    assert C.sizeof(N.KzMaterial) == 16 + 8 * 64
    assert N.RAY_DTYPE.itemsize == 32
    assert C.sizeof(N.KzBatchConfig) == 24
    assert C.sizeof(N.KzTexture) == 56


def test_abi_version_and_device_query(native_lib):
    assert native_lib.kz_abi_version() == 3
    assert native_lib.kz_device_count() >= 0


def test_scene_handle_validates_on_host(native_lib):
    s = api.Scene()
    with pytest.raises(N.KazenError) as e:
        s.add_mesh(np.array([[0, 0, 0], [1, 0, 0], [0, np.nan, 0]], np.float32), [[0, 1, 2]])
    assert e.value.code == N.KZ_ERR_INVALID_ARG
    with pytest.raises(N.KazenError) as e:
        s.add_mesh(np.zeros((3, 3), np.float32), [[0, 1, 3]])
    assert e.value.code == N.KZ_ERR_INVALID_ARG and "out of range" in str(e.value)
    with pytest.raises(N.KazenError):
        s.add_mesh(np.zeros((3, 3), np.float32), [[0, 1, 2]], xform=[1, 0, 0, 0, 0, np.inf, 0, 0, 0, 0, 1, 0])
    assert s.add_mesh(np.eye(3, dtype=np.float32), [[0, 1, 2]], material_id=0) == 0
    # materials: bad closure id, emission as a lobe, zero roughness, negative Le
    with pytest.raises(N.KazenError):
        s.set_materials([api.material([api.lobe(99)])])
    with pytest.raises(N.KazenError):
        s.set_materials([api.material([api.lobe(N.KZ_CLOSURE_KP_EMITTER)])])
    with pytest.raises(N.KazenError):
        s.set_materials([api.material([api.conductor_ggx(alpha=0.0)])])
    with pytest.raises(N.KazenError):
        s.set_materials([api.material([], Le=(-1, 0, 0))])
    # a mesh that names a material that does not exist is rejected at build
    s.set_materials([])
    with pytest.raises(N.KazenError) as e:
        s.build_bvh()
    assert e.value.code == N.KZ_ERR_INVALID_ARG
    s.close()


def test_calls_before_build_report_state(native_lib):
    s = api.Scene()
    r = api.make_rays([[0, 0, 0]], [[0, 0, 1]])
    with pytest.raises(N.KazenError) as e:
        s.intersect(r)
    assert e.value.code == N.KZ_ERR_STATE
    s.close()


def test_no_gpu_fails_loudly(native_lib):
    if native_lib.kz_device_count() > 0:
        pytest.skip("a GPU is visible")
    s = api.Scene()
    s.add_mesh(np.eye(3, dtype=np.float32), [[0, 1, 2]])
    s.set_materials([api.material([api.diffuse()])])
    with pytest.raises(N.KazenError) as e:
        s.build_bvh()
    assert e.value.code == N.KZ_ERR_NO_DEVICE
    with pytest.raises(N.KazenError) as e:
        api.closure_eval([api.diffuse()], [[0, 1, 0]], [[0, 1, 0]])
    assert e.value.code == N.KZ_ERR_NO_DEVICE


def test_material_lowering_of_shipped_shaders():
    # resource/scene/cbox/{diffuse,mirror,dielectric,rough,area}.osl as lowered records
    diffuse = api.material([api.diffuse((0.5, 0.5, 0.5))])
    mirror = api.material([api.mirror()])
    diel = api.material([api.dielectric(1.5046, 1.000277)])
    rough = api.material([api.diffuse((0.35, 0.35, 0.35)), api.microfacet("beckmann", 0.28, eta=1.5,
                                                                         weight=(0.07, 0.07, 0.07))])
    area = api.material([], Le=(1.0, 1.0, 1.0))
    assert diffuse["lobes"][0]["closure_id"] == N.KZ_CLOSURE_DIFFUSE
    assert mirror["lobes"][0]["closure_id"] == N.KZ_CLOSURE_KP_MIRROR
    assert np.allclose(diel["lobes"][0]["params"][:2], [1.5046, 1.000277])
    assert rough["n_lobes"] == 2 and rough["lobes"][1]["closure_id"] == N.KZ_CLOSURE_KP_GLOSS
    assert rough["lobes"][1]["params"][0] == N.KZ_DIST_BECKMANN
    assert area["n_lobes"] == 0 and area["Le"][0] == 1.0


def test_texture_validation_on_host(native_lib):
    s = api.Scene()
    g = s.add_mesh(np.eye(3, dtype=np.float32), [[0, 1, 2]], material_id=0)
    with pytest.raises(N.KazenError):  # uv count must match the vertices
        s.set_mesh_uvs(g, np.zeros((2, 2), np.float32))
    with pytest.raises(N.KazenError):  # non-finite uv
        s.set_mesh_uvs(g, np.array([[0, 0], [1, np.nan], [0, 1]], np.float32))
    with pytest.raises(N.KazenError):  # no such mesh
        s.set_mesh_uvs(5, np.zeros((3, 2), np.float32))
    s.set_mesh_uvs(g, np.zeros((3, 2), np.float32))
    with pytest.raises(N.KazenError):  # image without pixels
        s.set_textures([api.Texture(N.KZ_TEX_IMAGE, np.zeros((0, 4, 3), np.float32))])
    with pytest.raises(N.KazenError):  # non-finite texel
        s.set_textures([api.image_texture(np.full((2, 2, 3), np.inf, np.float32))])
    with pytest.raises(N.KazenError):  # unknown kind
        s.set_textures([api.Texture(7)])
    with pytest.raises(N.KazenError):
        s.set_environment((-1, 0, 0))
    s.set_textures([api.checker_texture()])
    # a lobe naming texture 2 of 1, and two textures in one material, fail at build
    s.set_materials([api.material([api.textured(api.diffuse(), 1)])])
    with pytest.raises(N.KazenError) as e:
        s.build_bvh()
    assert e.value.code == N.KZ_ERR_INVALID_ARG and "texture" in str(e.value)
    s.set_textures([api.checker_texture(), api.checker_texture(2, 2)])
    s.set_materials([api.material([api.textured(api.diffuse(), 0), api.textured(api.phong(), 1)])])
    with pytest.raises(N.KazenError) as e:
        s.build_bvh()
    assert "one per material" in str(e.value)
    s.set_materials([api.material([api.diffuse()])])
    s.set_environment((1, 1, 1), 5)
    with pytest.raises(N.KazenError) as e:
        s.build_bvh()
    assert "environment texture" in str(e.value)


def test_point_light_validation_on_host(native_lib):
    s = api.Scene()
    assert s.add_point_light((0, 1, 0), (1, 1, 1)) == 0
    assert s.add_point_light((0, 2, 0), (0, 0, 0)) == 1
    with pytest.raises(N.KazenError):
        s.add_point_light((0, np.nan, 0), (1, 1, 1))
    with pytest.raises(N.KazenError):
        s.add_point_light((0, 1, 0), (1, -1, 1))


def test_normals_validation_on_host(native_lib):
    s = api.Scene()
    g = s.add_mesh(np.eye(3, dtype=np.float32), [[0, 1, 2]], material_id=0)
    with pytest.raises(N.KazenError):  # count must match the vertices
        s.set_mesh_normals(g, np.ones((2, 3), np.float32))
    with pytest.raises(N.KazenError):  # a zero normal has no direction
        s.set_mesh_normals(g, np.array([[0, 0, 1], [0, 0, 0], [0, 0, 1]], np.float32))
    with pytest.raises(N.KazenError):
        s.set_mesh_normals(g, np.array([[0, 0, 1], [0, np.inf, 0], [0, 0, 1]], np.float32))
    s.set_mesh_normals(g, np.array([[0, 0, 2], [0, 1, 1], [1, 0, 0]], np.float32))


@pytest.mark.parametrize("block_size", [512, 1024, 48])
def test_block_size_above_the_launch_bounds_is_rejected(native_lib, block_size):
    # the stage kernels are compiled for at most 256 threads per block; the
    # render-config check runs before any scene or device work, so an unbuilt
    # scene handle reaches it on a machine without a GPU
    s = api.Scene()
    cfg = api.render_config(spp=1, max_depth=2, block_size=block_size)
    rays = api.make_rays([[0, 0, 0]], [[0, 0, 1]])
    out = np.zeros((1, 3), np.float32)
    st = N.KzRenderStats()
    cam = N.KzCamera()
    film = N.KzFilmDesc(4, 4)
    img = np.zeros((4, 4, 3), np.float32)
    P = lambda a: a.ctypes.data  # noqa: E731
    codes = [
        native_lib.kz_li_batch(s.handle, P(rays), 1, C.byref(cfg), P(out), N.KZ_MEM_HOST, C.byref(st)),
        native_lib.kz_li_batch_noalloc(s.handle, P(rays), 1, C.byref(cfg), P(out), C.byref(st)),
        native_lib.kz_render(s.handle, C.byref(cam), C.byref(film), C.byref(cfg), P(img), None, N.KZ_MEM_HOST,
                             C.byref(st)),
    ]
    assert codes == [N.KZ_ERR_INVALID_ARG] * 3
    assert "block_size" in native_lib.kz_last_error_string().decode()
    # 256 passes the config check and stops at the scene state instead
    cfg.block_size = 256
    assert native_lib.kz_li_batch(s.handle, P(rays), 1, C.byref(cfg), P(out), N.KZ_MEM_HOST,
                                  C.byref(st)) == N.KZ_ERR_STATE
    s.close()


def test_host_output_buffer_checks():
    """Renderer.render(out=...) takes a caller's host buffer: a contiguous
    float32 numpy array or CPU tensor of H*W*3 elements, nothing else."""
    import numpy as np
    from kazen_proto_gb300 import api
    a = np.empty((4, 5, 3), np.float32)
    assert api._host_ptr(a, 60, np.float32).value == a.ctypes.data
    with pytest.raises(ValueError):
        api._host_ptr(np.empty((4, 5, 3), np.float64), 60, np.float32)
    with pytest.raises(ValueError):
        api._host_ptr(np.empty((4, 5, 2), np.float32), 60, np.float32)
    with pytest.raises(ValueError):
        api._host_ptr(np.empty((5, 4, 3), np.float32).transpose(1, 0, 2), 60, np.float32)
    torch = pytest.importorskip("torch")
    t = torch.empty((4, 5, 3), dtype=torch.float32)
    assert api._host_ptr(t, 60, np.float32).value == t.data_ptr()
    with pytest.raises(ValueError):
        api._host_ptr(t.transpose(0, 1), 60, np.float32)
    with pytest.raises(ValueError):
        api._host_ptr(torch.empty((4, 5, 3), dtype=torch.float64), 60, np.float32)


def test_python_constants_match_header():
    """The Python binding's copies of the header's flag, mode and limit
    values are the header's."""
    from kazen_proto_gb300 import _native as N
    from kazen_proto_gb300 import api
    hdr = open(os.path.join(ROOT, "include", "kazen_gb300.h")).read()
    defs = {m.group(1): m.group(2) for m in re.finditer(r"^#define\s+(KZ_\w+)\s+(.+?)\s*(?:/\*.*)?$", hdr, re.M)}

    def value(name):
        v = defs[name].strip("()")
        m = re.fullmatch(r"(\d+)u?\s*<<\s*(\d+)", v)
        return int(m.group(1)) << int(m.group(2)) if m else int(v.rstrip("u"), 0)
    for name in ("KZ_RENDER_FLAG_TIMING", "KZ_RENDER_FLAG_COUNT", "KZ_RENDER_FLAG_NEE_ONLY",
                 "KZ_RENDER_FLAG_BSDF_ONLY"):
        assert getattr(N, name) == value(name), name
    assert api.BATCH_WAVEFRONT == value("KZ_BATCH_WAVEFRONT")
    assert api.BATCH_MEGAKERNEL == value("KZ_BATCH_MEGAKERNEL")
    assert api.BATCH_PERSISTENT == value("KZ_BATCH_PERSISTENT")
    assert value("KZ_RENDER_DEFAULT_WAVEFRONT") == 1 << 24


def test_autotune_candidates_cover_every_batch_mode():
    """The batch autotuner sweeps the wavefront mode (paths in flight x block
    x refill period), the single-launch persistent mode (paths in flight x
    refill period) and the megakernel (block x blocks per SM x period), with
    no duplicate configuration."""
    from kazen_proto_gb300 import api, autotune
    cands = autotune.candidates()
    modes = {c["mode"] for c in cands}
    assert modes == {api.BATCH_WAVEFRONT, api.BATCH_PERSISTENT, api.BATCH_MEGAKERNEL}
    keys = [tuple(sorted(c.items())) for c in cands]
    assert len(keys) == len(set(keys))
    pers = [c for c in cands if c["mode"] == api.BATCH_PERSISTENT]
    assert {c["wavefront_size"] for c in pers} == set(autotune.WAVEFRONT_SIZES)
    assert {c["refill_period"] for c in pers} == set(autotune.WAVE_PERIODS)
    cfg = autotune.config_of(pers[0], use_graph=True)
    assert cfg.mode == api.BATCH_PERSISTENT and cfg.use_graph == 1 and cfg.wavefront_size == pers[0]["wavefront_size"]
