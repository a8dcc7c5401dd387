"""ctypes binding of the C ABI declared in include/kazen_gb300.h.

The shared library is built in-tree (kazen_proto_gb300/_build/); loading
fails loudly when it is missing — there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# KZ_LIBRARY selects another build of the library (the test builds of
# kazen_proto_gb300/build.py); the default is the in-tree product build.
LIB_PATH = os.environ.get("KZ_LIBRARY") or os.path.join(HERE, "_build", "libkazen_gb300.so")

KZ_OK = 0
KZ_ERR_INVALID_ARG = 1
KZ_ERR_OOM = 2
KZ_ERR_CUDA = 3
KZ_ERR_TIMEOUT = 4
KZ_ERR_STACK = 5
KZ_ERR_STATE = 6
KZ_ERR_NO_DEVICE = 7

KZ_MEM_HOST = 0
KZ_MEM_DEVICE = 1
KZ_INVALID_ID = 0xFFFFFFFF

KZ_CLOSURE_DIFFUSE = 0
KZ_CLOSURE_EMISSION = 10
KZ_CLOSURE_KP_MIRROR = 14
KZ_CLOSURE_KP_DIELECTRIC = 15
KZ_CLOSURE_KP_EMITTER = 17
KZ_CLOSURE_KP_GLOSS = 18
KZ_CLOSURE_KP_GLASS = 19
KZ_CLOSURE_KP_PRINCIPLE_SPECULAR_REFL = 24
KZ_CLOSURE_CONDUCTOR_GGX = 64
KZ_CLOSURE_PHONG = 1
KZ_CLOSURE_WARD = 3
KZ_CLOSURE_REFLECTION = 4
KZ_CLOSURE_REFRACTION = 5
KZ_CLOSURE_TRANSPARENT = 6
KZ_CLOSURE_TRANSLUCENT = 7
KZ_CLOSURE_KP_MICROFACET = 16
KZ_CLOSURE_KP_PRINCIPLE_DIFFUSE = 20
KZ_CLOSURE_KP_PRINCIPLE_RETRO = 21
KZ_CLOSURE_KP_PRINCIPLE_FAKESS = 22
KZ_CLOSURE_KP_PRINCIPLE_SHEEN = 23
KZ_CLOSURE_KP_PRINCIPLE_CLEARCOAT = 26
KZ_DIST_GGX = 0
KZ_DIST_BECKMANN = 1
KZ_MAX_LOBES = 8
KZ_CONVENTION_REFERENCE = 0
KZ_CONVENTION_INTEGRATOR = 1


class KzLobe(C.Structure):
    _fields_ = [("closure_id", C.c_uint32), ("weight", C.c_float * 3), ("params", C.c_float * 12)]


KZ_TEX_CHECKER = 0
KZ_TEX_IMAGE = 1
KZ_LOBE_TEXTURE_PARAM = 11


class KzTexture(C.Structure):
    _fields_ = [("kind", C.c_int32), ("width", C.c_uint32), ("height", C.c_uint32), ("rgb", C.c_void_p),
                ("scale_s", C.c_float), ("scale_t", C.c_float), ("Ca", C.c_float * 3), ("Cb", C.c_float * 3)]


class KzMaterial(C.Structure):
    _fields_ = [("Le", C.c_float * 3), ("n_lobes", C.c_uint32), ("lobes", KzLobe * KZ_MAX_LOBES)]


class KzRay(C.Structure):
    _fields_ = [(n, C.c_float) for n in ("ox", "oy", "oz", "tmin", "dx", "dy", "dz", "tmax")]


class KzHits(C.Structure):
    _fields_ = [("t", C.c_void_p), ("prim_id", C.c_void_p), ("geom_id", C.c_void_p),
                ("u", C.c_void_p), ("v", C.c_void_p)]


class KzCamera(C.Structure):
    _fields_ = [("eye", C.c_float * 3), ("lookat", C.c_float * 3), ("up", C.c_float * 3),
                ("fov_deg", C.c_float), ("near_clip", C.c_float), ("far_clip", C.c_float), ("flip", C.c_int32)]


class KzFilmDesc(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32)]


class KzRenderConfig(C.Structure):
    _fields_ = [("spp", C.c_uint32), ("max_depth", C.c_uint32), ("seed", C.c_uint64),
                ("wavefront_size", C.c_uint32), ("rr_min_depth", C.c_uint32), ("block_size", C.c_uint32),
                ("flags", C.c_uint32)]


KZ_RENDER_FLAG_TIMING = 1
KZ_RENDER_FLAG_COUNT = 2
KZ_RENDER_FLAG_NEE_ONLY = 4
KZ_RENDER_FLAG_BSDF_ONLY = 8


class KzRenderStats(C.Structure):
    _fields_ = [("path_bounces", C.c_uint64), ("shadow_rays", C.c_uint64), ("iterations", C.c_uint64),
                ("paths", C.c_uint64), ("kernel_launches", C.c_uint64),
                ("closest_node_fetches", C.c_uint64), ("closest_tri_fetches", C.c_uint64),
                ("shadow_node_fetches", C.c_uint64), ("shadow_tri_fetches", C.c_uint64),
                ("generate_ms", C.c_double), ("trace_ms", C.c_double), ("shade_ms", C.c_double),
                ("shadow_ms", C.c_double)]


class KzGuideConfig(C.Structure):
    _fields_ = [("alpha", C.c_float), ("learning_rate", C.c_float), ("spp_per_pass", C.c_uint32),
                ("train", C.c_uint32), ("max_train_samples", C.c_uint32), ("steps_per_pass", C.c_uint32),
                ("max_train_steps", C.c_uint32), ("time_budget_ms", C.c_double)]


class KzGuideStats(C.Structure):
    _fields_ = [("passes", C.c_uint64), ("spp_done", C.c_uint64), ("train_steps", C.c_uint64),
                ("train_samples", C.c_uint64), ("last_loss", C.c_double), ("wall_ms", C.c_double),
                ("train_ms", C.c_double)]


KZ_GUIDE_PARAMS = 15080


class KzBatchJob(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("camera", KzCamera), ("width", C.c_uint32), ("height", C.c_uint32),
                ("spp", C.c_uint32), ("max_depth", C.c_uint32), ("rr_min_depth", C.c_uint32), ("seed", C.c_uint64),
                ("out_rgb", C.c_void_p)]


class KzBatchConfig(C.Structure):
    _fields_ = [("block_size", C.c_uint32), ("ctas_per_sm", C.c_uint32), ("refill_period", C.c_uint32),
                ("use_graph", C.c_uint32), ("mode", C.c_uint32), ("wavefront_size", C.c_uint32)]


class KzBatchStats(C.Structure):
    _fields_ = [("paths", C.c_uint64), ("path_bounces", C.c_uint64), ("shadow_rays", C.c_uint64),
                ("threads", C.c_uint64), ("device_ms", C.c_double)]


class KzSceneInfo(C.Structure):
    _fields_ = [("n_meshes", C.c_uint64), ("n_triangles", C.c_uint64), ("n_lights", C.c_uint64),
                ("n_bvh_nodes", C.c_uint64), ("bvh_bytes", C.c_uint64), ("triangle_bytes", C.c_uint64),
                ("bvh_depth", C.c_uint32), ("built", C.c_uint32)]


# numpy views of the record layouts
RAY_DTYPE = np.dtype([(n, np.float32) for n in ("ox", "oy", "oz", "tmin", "dx", "dy", "dz", "tmax")])
LOBE_DTYPE = np.dtype([("closure_id", np.uint32), ("weight", np.float32, 3), ("params", np.float32, 12)])
MATERIAL_DTYPE = np.dtype([("Le", np.float32, 3), ("n_lobes", np.uint32), ("lobes", LOBE_DTYPE, KZ_MAX_LOBES)])
assert RAY_DTYPE.itemsize == C.sizeof(KzRay) == 32
assert LOBE_DTYPE.itemsize == C.sizeof(KzLobe) == 64
assert MATERIAL_DTYPE.itemsize == C.sizeof(KzMaterial)

# name -> (restype, argtypes); every entry point of the header
_P = C.c_void_p
SIGNATURES = {
    "kz_abi_version": (C.c_int32, []),
    "kz_last_error_string": (C.c_char_p, []),
    "kz_device_count": (C.c_int32, []),
    "kz_scene_create": (C.c_int32, [C.POINTER(C.c_void_p)]),
    "kz_scene_destroy": (C.c_int32, [_P]),
    "kz_scene_add_mesh": (C.c_int32, [_P, _P, C.c_uint32, _P, C.c_uint32, _P, C.c_int32, C.c_int32,
                                      C.POINTER(C.c_int32)]),
    "kz_scene_set_materials": (C.c_int32, [_P, _P, C.c_uint32]),
    "kz_scene_set_textures": (C.c_int32, [_P, _P, C.c_uint32]),
    "kz_scene_set_mesh_uvs": (C.c_int32, [_P, C.c_int32, _P, C.c_uint32]),
    "kz_scene_set_mesh_normals": (C.c_int32, [_P, C.c_int32, _P, C.c_uint32]),
    "kz_scene_set_environment": (C.c_int32, [_P, _P, C.c_int32]),
    "kz_scene_add_point_light": (C.c_int32, [_P, _P, _P, C.POINTER(C.c_int32)]),
    "kz_scene_build": (C.c_int32, [_P]),
    "kz_scene_get_info": (C.c_int32, [_P, C.POINTER(KzSceneInfo)]),
    "kz_scene_set_stream": (C.c_int32, [_P, _P]),
    "kz_scene_synchronize": (C.c_int32, [_P]),
    "kz_intersect_closest": (C.c_int32, [_P, _P, C.c_uint64, KzHits, C.c_int32]),
    "kz_intersect_any": (C.c_int32, [_P, _P, C.c_uint64, _P, C.c_int32]),
    "kz_intersect_stats": (C.c_int32, [_P, _P, C.c_uint64, C.c_int32, C.POINTER(C.c_uint64),
                                       C.POINTER(C.c_uint64)]),
    "kz_closure_eval_batch": (C.c_int32, [_P, _P, _P, C.c_uint64, C.c_int32, _P, _P, C.c_int32]),
    "kz_closure_sample_batch": (C.c_int32, [_P, _P, _P, C.c_uint64, _P, _P, _P, _P, C.c_int32]),
    "kz_li_batch": (C.c_int32, [_P, _P, C.c_uint64, C.POINTER(KzRenderConfig), _P, C.c_int32,
                                C.POINTER(KzRenderStats)]),
    "kz_render": (C.c_int32, [_P, C.POINTER(KzCamera), C.POINTER(KzFilmDesc), C.POINTER(KzRenderConfig), _P, _P,
                              C.c_int32, C.POINTER(KzRenderStats)]),
    "kz_li_batch_noalloc": (C.c_int32, [_P, _P, C.c_uint64, C.POINTER(KzRenderConfig), _P,
                                        C.POINTER(KzRenderStats)]),
    "kz_render_batch": (C.c_int32, [C.POINTER(KzBatchJob), C.c_uint32, C.POINTER(KzBatchConfig), C.c_int32,
                                    C.POINTER(KzBatchStats)]),
    "kz_scene_release_scratch": (C.c_int32, [_P]),
    "kz_guide_create": (C.c_int32, [C.POINTER(C.c_void_p), C.c_uint64]),
    "kz_guide_destroy": (C.c_int32, [_P]),
    "kz_guide_get_params": (C.c_int32, [_P, _P]),
    "kz_guide_set_params": (C.c_int32, [_P, _P]),
    "kz_guide_get_state": (C.c_int32, [_P, _P, C.POINTER(C.c_uint32)]),
    "kz_guide_set_state": (C.c_int32, [_P, _P, C.c_uint32]),
    "kz_guide_forward": (C.c_int32, [_P, _P, C.c_uint64, _P, C.c_int32]),
    "kz_guide_train_step": (C.c_int32, [_P, _P, C.c_uint64, C.c_float, C.c_int32, C.POINTER(C.c_float), _P,
                                        C.c_int32]),
    "kz_render_guided": (C.c_int32, [_P, _P, C.POINTER(KzCamera), C.POINTER(KzFilmDesc), C.POINTER(KzRenderConfig),
                                     C.POINTER(KzGuideConfig), _P, _P, C.c_int32, C.POINTER(KzRenderStats),
                                     C.POINTER(KzGuideStats)]),
}
KZ_LI_NOALLOC_MAX_WAVEFRONT = 16384


class KazenError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"kazen status {code}: {msg}")
        self.code = code


_lib = None


def lib() -> C.CDLL:
    """Load libkazen_gb300.so (built by kazen_proto_gb300.build)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run kazen_proto_gb300.build.build() first "
                              "(the library has no CPU fallback)")
        l = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(l, name)
            f.restype = res
            f.argtypes = args
        _lib = l
    return _lib


def check(code: int) -> None:
    if code != KZ_OK:
        msg = lib().kz_last_error_string()
        raise KazenError(code, msg.decode() if msg else "")
