"""ctypes wrapper of the CPU restatement (oracle/kz_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py. The product package never imports it.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_P = C.c_void_p
_lib = None

RAY_DTYPE = np.dtype([(n, np.float32) for n in ("ox", "oy", "oz", "tmin", "dx", "dy", "dz", "tmax")])
LOBE_DTYPE = np.dtype([("closure_id", np.uint32), ("weight", np.float32, 3), ("params", np.float32, 12)])
MATERIAL_DTYPE = np.dtype([("Le", np.float32, 3), ("n_lobes", np.uint32), ("lobes", LOBE_DTYPE, 8)])


class RenderConfig(C.Structure):
    _fields_ = [("spp", C.c_uint32), ("max_depth", C.c_uint32), ("seed", C.c_uint64),
                ("wavefront_size", C.c_uint32), ("rr_min_depth", C.c_uint32), ("block_size", C.c_uint32),
                ("flags", C.c_uint32)]


class Camera(C.Structure):
    _fields_ = [("eye", C.c_float * 3), ("lookat", C.c_float * 3), ("up", C.c_float * 3),
                ("fov_deg", C.c_float), ("near_clip", C.c_float), ("far_clip", C.c_float), ("flip", C.c_int32)]


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        l = C.CDLL(path)
        sig = {
            "kzo_bvh_build": (_P, [_P, C.c_uint32]),
            "kzo_bvh_free": (None, [_P]),
            "kzo_closest": (None, [_P, _P, C.c_uint64, C.c_int, _P, _P, _P, _P]),
            "kzo_any": (None, [_P, _P, C.c_uint64, C.c_int, _P]),
            "kzo_closest_brute": (None, [_P, C.c_uint32, _P, C.c_uint64, _P, _P]),
            "kzo_closure_eval": (None, [_P, _P, _P, C.c_uint64, C.c_int, _P, _P]),
            "kzo_closure_sample": (None, [_P, _P, _P, C.c_uint64, _P, _P, _P, _P]),
            "kzo_furnace_weak": (C.c_double, [C.c_int, C.c_float, C.c_float]),
            "kzo_furnace_fixed_beckmann": (C.c_double, [C.c_float, C.c_float]),
            "kzo_scene_create": (_P, [_P, C.c_uint32, _P, _P, _P, C.c_uint32, _P, C.c_uint32]),
            "kzo_scene_free": (None, [_P]),
            "kzo_scene_set_textures": (None, [_P, _P, C.c_uint32, _P, _P, C.c_int32]),
            "kzo_scene_add_point_light": (None, [_P, _P, _P]),
            "kzo_scene_set_normals": (None, [_P, _P, _P]),
            "kzo_render": (None, [_P, C.POINTER(Camera), C.c_uint32, C.c_uint32, C.POINTER(RenderConfig), C.c_int,
                                  C.c_uint32, C.c_uint32, _P, _P]),
            "kzo_camera_rays": (None, [C.POINTER(Camera), C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64, _P]),
            "kzo_li": (None, [_P, _P, C.c_uint64, C.POINTER(RenderConfig), C.c_int, _P, _P]),
            "kzo_pcg32_outputs": (None, [C.c_uint64, C.c_uint64, _P, C.c_int]),
            "kzo_mdf_terms": (None, [C.c_int, _P, C.c_uint64, _P]),
            "kzo_mt_intersect": (None, [_P, C.c_uint32, _P, C.c_uint64, C.c_int, _P, _P, _P, _P]),
            "kzo_render_compat": (None, [_P, C.POINTER(Camera), C.c_uint32, C.c_uint32, C.POINTER(RenderConfig),
                                         C.c_int, C.c_uint32, C.c_uint32, C.c_uint32, _P, _P]),
            "kzo_fresnel_terms": (None, [_P, C.c_uint64, _P]),
            "kzo_refract": (None, [_P, C.c_uint64, _P]),
            "kzo_frame": (None, [_P, C.c_uint64, _P]),
            "kzo_warps": (None, [_P, C.c_uint64, _P]),
        }
        for name, (res, args) in sig.items():
            f = getattr(l, name)
            f.restype = res
            f.argtypes = args
        _lib = l
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Bvh:
    """The restatement's own BVH (object-median binary) over a world-space soup."""

    def __init__(self, tri_verts):
        self.tv = np.ascontiguousarray(tri_verts, np.float32).reshape(-1, 9)
        self.h = lib().kzo_bvh_build(_p(self.tv), len(self.tv))

    def __del__(self):
        if getattr(self, "h", None):
            lib().kzo_bvh_free(self.h)
            self.h = None

    def closest(self, rays, nthreads=0):
        r = np.ascontiguousarray(rays, RAY_DTYPE)
        n = len(r)
        t = np.empty(n, np.float32)
        prim = np.empty(n, np.uint32)
        u = np.empty(n, np.float32)
        v = np.empty(n, np.float32)
        lib().kzo_closest(self.h, _p(r), n, nthreads, _p(t), _p(prim), _p(u), _p(v))
        return {"t": t, "prim": prim, "u": u, "v": v}

    def any(self, rays, nthreads=0):
        r = np.ascontiguousarray(rays, RAY_DTYPE)
        occ = np.empty(len(r), np.uint8)
        lib().kzo_any(self.h, _p(r), len(r), nthreads, _p(occ))
        return occ.astype(bool)


def closest_brute(tri_verts, rays):
    tv = np.ascontiguousarray(tri_verts, np.float32).reshape(-1, 9)
    r = np.ascontiguousarray(rays, RAY_DTYPE)
    t = np.empty(len(r), np.float32)
    prim = np.empty(len(r), np.uint32)
    lib().kzo_closest_brute(_p(tv), len(tv), _p(r), len(r), _p(t), _p(prim))
    return {"t": t, "prim": prim}


def closure_eval(lobes, wi, wo, convention=0):
    lb = np.ascontiguousarray(lobes, LOBE_DTYPE).reshape(-1)
    a = np.ascontiguousarray(wi, np.float32).reshape(-1, 3)
    b = np.ascontiguousarray(wo, np.float32).reshape(-1, 3)
    f = np.empty((len(lb), 3), np.float32)
    pdf = np.empty(len(lb), np.float32)
    lib().kzo_closure_eval(_p(lb), _p(a), _p(b), len(lb), convention, _p(f), _p(pdf))
    return f, pdf


def closure_sample(lobes, wi, u):
    lb = np.ascontiguousarray(lobes, LOBE_DTYPE).reshape(-1)
    a = np.ascontiguousarray(wi, np.float32).reshape(-1, 3)
    uu = np.ascontiguousarray(u, np.float32).reshape(-1, 3)
    n = len(lb)
    wo = np.empty((n, 3), np.float32)
    w = np.empty((n, 3), np.float32)
    pdf = np.empty(n, np.float32)
    fl = np.empty(n, np.uint8)
    lib().kzo_closure_sample(_p(lb), _p(a), _p(uu), n, _p(wo), _p(w), _p(pdf), _p(fl))
    return wo, w, pdf, fl


def furnace_weak(dist, theta_deg, alpha):
    return lib().kzo_furnace_weak(dist, theta_deg, alpha)


def furnace_fixed_beckmann(alpha, theta):
    return lib().kzo_furnace_fixed_beckmann(alpha, theta)


def pcg32(initstate, initseq, n=16):
    out = np.empty(n, np.uint32)
    lib().kzo_pcg32_outputs(initstate, initseq, _p(out), n)
    return out


def make_camera(eye, lookat, up, fov, flip=False):
    c = Camera()
    c.eye[:] = [float(x) for x in eye]
    c.lookat[:] = [float(x) for x in lookat]
    c.up[:] = [float(x) for x in up]
    c.fov_deg = fov
    c.near_clip = 1e-3
    c.far_clip = 1e4
    c.flip = 1 if flip else 0
    return c


def make_config(spp, max_depth, seed=0, rr_min_depth=3, flags=0):
    c = RenderConfig()
    c.spp = spp
    c.max_depth = max_depth
    c.seed = seed
    c.rr_min_depth = rr_min_depth
    c.flags = flags
    return c


class Scene:
    """Render scene: world-space triangles in global order + per-mesh data + materials."""

    def __init__(self, tri_verts, tri_geom, geom_material, geom_is_light, materials):
        self.tv = np.ascontiguousarray(tri_verts, np.float32).reshape(-1, 9)
        self.tg = np.ascontiguousarray(tri_geom, np.uint32)
        self.gm = np.ascontiguousarray(geom_material, np.int32)
        self.gl = np.ascontiguousarray(geom_is_light, np.int32)
        self.mats = np.ascontiguousarray(materials, MATERIAL_DTYPE).reshape(-1)
        self.h = lib().kzo_scene_create(_p(self.tv), len(self.tv), _p(self.tg), _p(self.gm), _p(self.gl),
                                        len(self.gm), _p(self.mats), len(self.mats))

    @classmethod
    def from_desc(cls, desc):
        tv, tg, gm, gl = desc.flatten()
        sc = cls(tv, tg, gm, gl, desc.material_array())
        nrm = desc.tri_normals() if hasattr(desc, "tri_normals") else None
        if nrm is not None:
            sc._nrm = np.ascontiguousarray(nrm[0], np.float32)
            sc._has = np.ascontiguousarray(nrm[1], np.uint8)
            lib().kzo_scene_set_normals(sc.h, _p(sc._nrm), _p(sc._has))
        for pos, rad in getattr(desc, "point_lights", []):
            lib().kzo_scene_add_point_light(sc.h, _p(np.ascontiguousarray(pos, np.float32)),
                                            _p(np.ascontiguousarray(rad, np.float32)))
        textures = getattr(desc, "textures", [])
        env = np.ascontiguousarray(getattr(desc, "env", (0, 0, 0)), np.float32)
        if textures or env.any():
            recs = [t.to_c() for t in textures]
            sc._keep = [k for _, k in recs]
            arr = (type(recs[0][0]) * len(recs))(*[r for r, _ in recs]) if recs else None
            uv = desc.tri_uvs()
            sc._uv = None if uv is None else np.ascontiguousarray(uv, np.float32)
            sc._env = env
            lib().kzo_scene_set_textures(sc.h, C.cast(arr, C.c_void_p) if arr is not None else None, len(recs),
                                         _p(sc._uv), _p(env), int(getattr(desc, "env_texture", -1)))
        return sc

    def __del__(self):
        if getattr(self, "h", None):
            lib().kzo_scene_free(self.h)
            self.h = None

    def render(self, camera, W, H, spp, max_depth, seed=0, rr_min_depth=3, nthreads=0, rows=None, flags=0):
        cfg = make_config(spp, max_depth, seed, rr_min_depth, flags)
        out = np.zeros((H, W, 3), np.float64)
        stats = np.zeros(2, np.uint64)
        r0, r1 = rows if rows is not None else (0, H)
        lib().kzo_render(self.h, C.byref(camera), W, H, C.byref(cfg), nthreads, r0, r1, _p(out), _p(stats))
        return out, {"path_bounces": int(stats[0]), "shadow_rays": int(stats[1])}

    def render_compat(self, camera, W, H, spp, max_depth, compat, seed=0, rr_min_depth=3, nthreads=0):
        """The frame with the path loop as the reference writes it, per COMPAT_* bit."""
        cfg = make_config(spp, max_depth, seed, rr_min_depth)
        out = np.zeros((H, W, 3), np.float64)
        stats = np.zeros(2, np.uint64)
        lib().kzo_render_compat(self.h, C.byref(camera), W, H, C.byref(cfg), nthreads, 0, H, compat, _p(out),
                                _p(stats))
        return out, {"path_bounces": int(stats[0]), "shadow_rays": int(stats[1])}

    def li(self, rays, max_depth, seed=0, rr_min_depth=3, nthreads=0):
        r = np.ascontiguousarray(rays, RAY_DTYPE)
        cfg = make_config(1, max_depth, seed, rr_min_depth)
        out = np.zeros((len(r), 3), np.float64)
        stats = np.zeros(2, np.uint64)
        lib().kzo_li(self.h, _p(r), len(r), C.byref(cfg), nthreads, _p(out), _p(stats))
        return out, {"path_bounces": int(stats[0]), "shadow_rays": int(stats[1])}


# reference-as-written modes of the path loop (kz_oracle.cpp, COMPAT_*)
COMPAT_NEE, COMPAT_BSDF, COMPAT_EMISSION, COMPAT_DEPTH = 1, 2, 4, 8
COMPAT_ALL = 15


def mt_intersect(tri_verts, rays, first_hit=False):
    """The reference's single-sided Moller-Trumbore over a triangle list:
    the closest accepted hit, or (first_hit) the first accepted triangle in
    index order as TriangleMesh::intersect returns it."""
    tv = np.ascontiguousarray(tri_verts, np.float32).reshape(-1, 9)
    r = np.ascontiguousarray(rays, RAY_DTYPE)
    n = len(r)
    out = {"t": np.empty(n, np.float32), "prim": np.empty(n, np.uint32), "u": np.empty(n, np.float32),
           "v": np.empty(n, np.float32)}
    lib().kzo_mt_intersect(_p(tv), len(tv), _p(r), n, 1 if first_hit else 0, _p(out["t"]), _p(out["prim"]),
                           _p(out["u"]), _p(out["v"]))
    return out


def camera_rays(camera, W, H, spp, seed):
    rays = np.zeros(W * H * spp, RAY_DTYPE)
    lib().kzo_camera_rays(C.byref(camera), W, H, spp, seed, _p(rays))
    return rays


def scalar_terms(name, inp, n_out, dist=None):
    """The restatement's scalar building blocks over rows of inputs (see
    kzo_mdf_terms / kzo_fresnel_terms / kzo_refract / kzo_frame / kzo_warps)."""
    a = np.ascontiguousarray(inp, np.float32)
    out = np.empty((len(a), n_out), np.float32)
    f = getattr(lib(), "kzo_" + name)
    if dist is None:
        f(_p(a), len(a), _p(out))
    else:
        f(dist, _p(a), len(a), _p(out))
    return out
