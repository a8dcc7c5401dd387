"""Python host API over the C ABI, mirroring kazen_proto's hot-path interfaces.

Reference interfaces mirrored (paths within kazen_proto):
  * Scene.add_mesh / build_bvh ........ src/core/scene.h:144-164, src/binding/api.cpp:121-170
  * Scene.intersect / occluded ........ HitableInterface, src/core/hitable.h:10-37
  * PathIntegrator.setup / Li .......... src/core/integrator.h:23-39, src/core/integrator.cpp:362-561
  * Renderer(spp).render ............... src/core/renderer.cpp:18-90
  * closure lobes ...................... ClosureID / *Params, src/shading/bsdf.h:16-75, src/shading/bsdfs.h:18-119

Arrays may be numpy arrays (host memory; the library stages the copies) or
CUDA torch tensors (device memory, used in place). Every call goes to the
CUDA library; a missing library or GPU raises.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _native as N
from ._native import check, lib

try:  # torch is optional plumbing for device buffers
    import torch
except Exception:  # pragma: no cover
    torch = None


def _is_cuda_tensor(x) -> bool:
    return torch is not None and isinstance(x, torch.Tensor) and x.is_cuda


def _ptr(x):
    if x is None:
        return None
    if _is_cuda_tensor(x):
        return C.c_void_p(x.data_ptr())
    return x.ctypes.data_as(C.c_void_p)


def _host_ptr(x, count, dtype):
    """Pointer to a caller's host buffer of `count` C-contiguous elements of
    `dtype`: a numpy array or a CPU tensor (pinned or not)."""
    if hasattr(x, "data_ptr"):  # a torch tensor
        if x.is_cuda or not x.is_contiguous() or x.numel() != count or x.element_size() != np.dtype(dtype).itemsize:
            raise ValueError("out must be a contiguous CPU tensor of %d %s" % (count, np.dtype(dtype).name))
        return C.c_void_p(x.data_ptr())
    if (not isinstance(x, np.ndarray) or x.dtype != dtype or x.size != count or not x.flags["C_CONTIGUOUS"]
            or not x.flags["WRITEABLE"]):
        raise ValueError("out must be a writable C-contiguous %s array of %d elements" % (np.dtype(dtype).name, count))
    return x.ctypes.data_as(C.c_void_p)


# ---------------------------------------------------------------- closures / materials
def lobe(closure_id: int, weight=(1.0, 1.0, 1.0), params=()) -> np.ndarray:
    rec = np.zeros((), dtype=N.LOBE_DTYPE)
    rec["closure_id"] = closure_id
    rec["weight"] = np.asarray(weight, np.float32)
    p = np.zeros(12, np.float32)
    p[: len(params)] = np.asarray(params, np.float32)
    rec["params"] = p
    return rec


def diffuse(albedo=(1.0, 1.0, 1.0), N_local=(0.0, 1.0, 0.0)):
    """`Cs * diffuse(N)`: Diffuse lobe (bsdfs.cpp:27-41)."""
    return lobe(N.KZ_CLOSURE_DIFFUSE, albedo, N_local)


def mirror(weight=(1.0, 1.0, 1.0)):
    """`Cs * kp_mirror()` (bsdfs.cpp:254-266)."""
    return lobe(N.KZ_CLOSURE_KP_MIRROR, weight)


def dielectric(int_ior=1.5046, ext_ior=1.000277, weight=(1.0, 1.0, 1.0)):
    """`Cs * kp_dielectric(int_ior, ext_ior)` (bsdfs.cpp:268-298)."""
    return lobe(N.KZ_CLOSURE_KP_DIELECTRIC, weight, (int_ior, ext_ior))


def microfacet(dist="ggx", xalpha=0.2, yalpha=None, eta=1.5, refract=0, weight=(1.0, 1.0, 1.0)):
    """`microfacet(dist, N, U, xalpha, yalpha, eta, refract)` lowered as the
    reference's process_closure does (bsdf.cpp:227-254): refract 0 -> KpGloss,
    1 or 2 -> KpGlass."""
    d = N.KZ_DIST_BECKMANN if dist == "beckmann" or dist == "default" else N.KZ_DIST_GGX
    ya = xalpha if yalpha is None else yalpha
    cid = N.KZ_CLOSURE_KP_GLOSS if refract == 0 else N.KZ_CLOSURE_KP_GLASS
    return lobe(cid, weight, (d, 0, 1, 0, 1, 0, 0, xalpha, ya, eta, refract))


def conductor_ggx(F0=(0.95, 0.64, 0.54), alpha=0.2, weight=(1.0, 1.0, 1.0)):
    """GGX conductor with RGB Schlick F0 (not a reference lobe; built from the
    reference GGX terms and fresnel_schlick(F0), fresnel.h:185-187)."""
    return lobe(N.KZ_CLOSURE_CONDUCTOR_GGX, weight, (F0[0], F0[1], F0[2], alpha, alpha))


def principle_specular(F0=(0.04, 0.04, 0.04), alpha=0.2, eta=1.5, metallic=0.0, weight=(1.0, 1.0, 1.0), yalpha=None):
    """`kp_principle_specular_reflection(F0, N, xalpha, yalpha, eta, metallic)` (bsdfs.cpp:688-730)."""
    ya = alpha if yalpha is None else yalpha
    return lobe(N.KZ_CLOSURE_KP_PRINCIPLE_SPECULAR_REFL, weight,
                (F0[0], F0[1], F0[2], 0, 1, 0, alpha, ya, eta, metallic))


def phong(exponent=20.0, weight=(1.0, 1.0, 1.0), N_local=(0.0, 1.0, 0.0)):
    """`phong(N, exponent)` (bsdfs.cpp:43-81)."""
    return lobe(N.KZ_CLOSURE_PHONG, weight, (*N_local, exponent))


def ward(xalpha=0.1, yalpha=None, weight=(1.0, 1.0, 1.0), N_local=(0.0, 1.0, 0.0), T_local=(1.0, 0.0, 0.0)):
    """`ward(N, T, xalpha, yalpha)` (bsdfs.cpp:92-148); anisotropy along the
    local x (tangent) and z axes."""
    ya = xalpha if yalpha is None else yalpha
    return lobe(N.KZ_CLOSURE_WARD, weight, (*N_local, *T_local, xalpha, ya))


def reflection(eta=1.5, weight=(1.0, 1.0, 1.0), N_local=(0.0, 1.0, 0.0)):
    """`reflection(N, eta)`: a perfect mirror without a Fresnel factor (bsdfs.cpp:150-167)."""
    return lobe(N.KZ_CLOSURE_REFLECTION, weight, (*N_local, eta))


def refraction(eta=1.5, weight=(1.0, 1.0, 1.0), N_local=(0.0, 1.0, 0.0)):
    """`refraction(N, eta)`: Snell transmission, eta = inside / outside (bsdfs.cpp:169-203)."""
    return lobe(N.KZ_CLOSURE_REFRACTION, weight, (*N_local, eta))


def transparent(weight=(1.0, 1.0, 1.0)):
    """`transparent()`: straight through (bsdfs.cpp:205-217)."""
    return lobe(N.KZ_CLOSURE_TRANSPARENT, weight)


def translucent(weight=(1.0, 1.0, 1.0)):
    """`translucent()`: Lambertian transmission (bsdfs.cpp:219-230)."""
    return lobe(N.KZ_CLOSURE_TRANSLUCENT, weight)


def kp_microfacet(alpha=0.1, int_ior=1.5046, ext_ior=1.000277, kd=0.5, weight=(1.0, 1.0, 1.0)):
    """`kp_microfacet(alpha, int_ior, ext_ior, kd)`: Beckmann Cook-Torrance over a
    diffuse base (bsdfs.cpp:300-336)."""
    return lobe(N.KZ_CLOSURE_KP_MICROFACET, weight, (alpha, int_ior, ext_ior, kd))


def principle_diffuse(weight=(1.0, 1.0, 1.0), N_local=(0.0, 1.0, 0.0)):
    """`kp_principle_diffuse(N)` (bsdfs.cpp:563-584)."""
    return lobe(N.KZ_CLOSURE_KP_PRINCIPLE_DIFFUSE, weight, N_local)


def principle_retro(roughness=0.5, weight=(1.0, 1.0, 1.0), N_local=(0.0, 1.0, 0.0)):
    """`kp_principle_retro(N, roughness)` (bsdfs.cpp:586-612)."""
    return lobe(N.KZ_CLOSURE_KP_PRINCIPLE_RETRO, weight, (*N_local, roughness))


def principle_fakess(roughness=0.5, weight=(1.0, 1.0, 1.0)):
    """`kp_principle_fakess(roughness)` (bsdfs.cpp:614-647)."""
    return lobe(N.KZ_CLOSURE_KP_PRINCIPLE_FAKESS, weight, (roughness,))


def principle_sheen(sheen=1.0, weight=(1.0, 1.0, 1.0), N_local=(0.0, 1.0, 0.0)):
    """`kp_principle_sheen(N)` (bsdfs.cpp:649-673). OSL registers only N for
    this closure, so the reference's `sheen` field is never written by a
    shader; lowered shaders carry the sheen amount in the weight and use 1."""
    return lobe(N.KZ_CLOSURE_KP_PRINCIPLE_SHEEN, weight, (*N_local, sheen))


def principle_clearcoat(roughness=0.1, weight=(1.0, 1.0, 1.0), N_local=(0.0, 1.0, 0.0)):
    """`kp_principle_clearcoat(N, roughness)`: GTR1 alpha in (0, 1) (bsdfs.cpp:736-800)."""
    return lobe(N.KZ_CLOSURE_KP_PRINCIPLE_CLEARCOAT, weight, (*N_local, roughness))


@dataclass
class Texture:
    """A lobe-weight or environment texture (kz_texture): the OSL checkerboard
    shader's pattern, or an (H, W, 3) float image (row 0 at t = 0)."""
    kind: int = N.KZ_TEX_CHECKER
    image: np.ndarray = None
    scale_s: float = 4.0
    scale_t: float = 4.0
    Ca: tuple = (1.0, 1.0, 1.0)
    Cb: tuple = (0.0, 0.0, 0.0)

    def to_c(self):
        t = N.KzTexture()
        t.kind = self.kind
        keep = None
        if self.kind == N.KZ_TEX_IMAGE:
            keep = np.ascontiguousarray(self.image, np.float32)
            if keep.ndim != 3 or keep.shape[2] != 3:
                raise ValueError(f"image texture must be (H, W, 3), got {keep.shape}")
            t.height, t.width = keep.shape[0], keep.shape[1]
            t.rgb = keep.ctypes.data_as(C.c_void_p)
        t.scale_s, t.scale_t = self.scale_s, self.scale_t
        t.Ca[:] = [float(x) for x in self.Ca]
        t.Cb[:] = [float(x) for x in self.Cb]
        return t, keep


def checker_texture(scale_s=4.0, scale_t=4.0, Ca=(1.0, 1.0, 1.0), Cb=(0.0, 0.0, 0.0)) -> Texture:
    """The OSL checkerboard shader (resource/scene/textured_cornell_box/checkerboard.osl)."""
    return Texture(N.KZ_TEX_CHECKER, None, scale_s, scale_t, tuple(Ca), tuple(Cb))


def image_texture(rgb) -> Texture:
    """An (H, W, 3) float image, bilinear with periodic wrap (OSL texture(filename, s, t))."""
    return Texture(N.KZ_TEX_IMAGE, np.ascontiguousarray(rgb, np.float32))


def textured(lobe_rec, texture_index: int) -> np.ndarray:
    """The lobe with its weight multiplied by texture `texture_index` of the scene."""
    rec = np.array(lobe_rec, dtype=N.LOBE_DTYPE)
    rec["params"][N.KZ_LOBE_TEXTURE_PARAM] = texture_index + 1
    return rec


def material(lobes=(), Le=(0.0, 0.0, 0.0)) -> np.ndarray:
    """A lowered surface shader: Le plus up to 8 lobes (ShadingResult, bsdf.h:217-229).
    An emitter shader `Cs * kp_emitter(a)` lowers to Le = Cs with no lobe."""
    if len(lobes) > N.KZ_MAX_LOBES:
        raise ValueError("at most 8 lobes")
    m = np.zeros((), dtype=N.MATERIAL_DTYPE)
    m["Le"] = np.asarray(Le, np.float32)
    m["n_lobes"] = len(lobes)
    for i, l in enumerate(lobes):
        m["lobes"][i] = l
    return m


# ---------------------------------------------------------------- rays
def make_rays(o, d, tmin=1e-4, tmax=np.inf) -> np.ndarray:
    """Ray records (32 B). Directions are normalised here, once, in FP32."""
    o = np.asarray(o, np.float32).reshape(-1, 3)
    d = np.asarray(d, np.float32).reshape(-1, 3)
    n = max(len(o), len(d))
    o = np.broadcast_to(o, (n, 3))
    d = np.broadcast_to(d, (n, 3))
    ln = np.sqrt((d * d).sum(axis=1, dtype=np.float32), dtype=np.float32)
    dn = (d / ln[:, None]).astype(np.float32)
    r = np.zeros(n, dtype=N.RAY_DTYPE)
    r["ox"], r["oy"], r["oz"] = o[:, 0], o[:, 1], o[:, 2]
    r["dx"], r["dy"], r["dz"] = dn[:, 0], dn[:, 1], dn[:, 2]
    r["tmin"] = np.float32(tmin)
    r["tmax"] = np.float32(tmax)
    return r


@dataclass
class Camera:
    """Camera(position, lookat, up, near, far, fov, flip) (camera.h:31-48); fov is horizontal, degrees."""
    eye: tuple = (0.0, 0.0, 0.0)
    lookat: tuple = (0.0, 0.0, -1.0)
    up: tuple = (0.0, 1.0, 0.0)
    fov: float = 40.0
    near: float = 1e-3
    far: float = 1e4
    flip: bool = False

    def to_c(self) -> N.KzCamera:
        c = N.KzCamera()
        c.eye[:] = [float(v) for v in self.eye]
        c.lookat[:] = [float(v) for v in self.lookat]
        c.up[:] = [float(v) for v in self.up]
        c.fov_deg = self.fov
        c.near_clip = self.near
        c.far_clip = self.far
        c.flip = 1 if self.flip else 0
        return c


def render_config(spp=16, max_depth=5, seed=0, wavefront_size=0, rr_min_depth=3, block_size=0,
                  flags=0) -> N.KzRenderConfig:
    c = N.KzRenderConfig()
    c.spp = spp
    c.max_depth = max_depth
    c.seed = seed
    c.wavefront_size = wavefront_size
    c.rr_min_depth = rr_min_depth
    c.block_size = block_size
    c.flags = flags
    return c


# ---------------------------------------------------------------- scene
class Scene:
    """Scene handle: meshes + lowered materials + BVH on the GPU."""

    def __init__(self):
        h = C.c_void_p()
        check(lib().kz_scene_create(C.byref(h)))
        self._h = h
        self._materials = None

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            lib().kz_scene_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_mesh(self, verts, indices, material_id=0, is_light=False, xform=None) -> int:
        """Scene::add_mesh(world, verts, ..., idx, name, shader, is_light) (scene.h:144-160)."""
        v = np.ascontiguousarray(verts, np.float32).reshape(-1, 3)
        i = np.ascontiguousarray(indices, np.uint32).reshape(-1, 3)
        x = None if xform is None else np.ascontiguousarray(xform, np.float32).reshape(12)
        gid = C.c_int32(-1)
        check(lib().kz_scene_add_mesh(self._h, _ptr(v), len(v), _ptr(i), len(i), _ptr(x), int(material_id),
                                      1 if is_light else 0, C.byref(gid)))
        return gid.value

    def set_materials(self, materials) -> None:
        m = np.ascontiguousarray(np.asarray(materials, dtype=N.MATERIAL_DTYPE).reshape(-1))
        self._materials = m
        check(lib().kz_scene_set_materials(self._h, _ptr(m), len(m)))

    def set_textures(self, textures) -> None:
        """Textures that lobes (params[11] = index + 1) and the environment reference."""
        recs = [t.to_c() for t in textures]
        arr = (N.KzTexture * max(1, len(recs)))(*[r for r, _ in recs])
        check(lib().kz_scene_set_textures(self._h, C.cast(arr, C.c_void_p), len(recs)))

    def set_mesh_uvs(self, geom_id: int, uv) -> None:
        """Per-vertex texture coordinates (nverts, 2) of a mesh."""
        a = np.ascontiguousarray(uv, np.float32).reshape(-1, 2)
        check(lib().kz_scene_set_mesh_uvs(self._h, int(geom_id), _ptr(a), len(a)))

    def add_point_light(self, position, radiance) -> int:
        """PointLight(position, radiance) (light.cpp:18-36): radiance / (0.1 |d|^2) at distance d."""
        p = np.ascontiguousarray(position, np.float32).reshape(3)
        r = np.ascontiguousarray(radiance, np.float32).reshape(3)
        lid = C.c_int32(-1)
        check(lib().kz_scene_add_point_light(self._h, _ptr(p), _ptr(r), C.byref(lid)))
        return lid.value

    def set_mesh_normals(self, geom_id: int, normals) -> None:
        """Per-vertex normals (nverts, 3) of a mesh, in the space its vertices were given in."""
        a = np.ascontiguousarray(normals, np.float32).reshape(-1, 3)
        check(lib().kz_scene_set_mesh_normals(self._h, int(geom_id), _ptr(a), len(a)))

    def set_environment(self, rgb=(0.0, 0.0, 0.0), texture: int = -1) -> None:
        """Radiance of rays that leave the scene: rgb times a lat-long texture (-1: none)."""
        a = np.ascontiguousarray(rgb, np.float32).reshape(3)
        check(lib().kz_scene_set_environment(self._h, _ptr(a), int(texture)))

    def build_bvh(self) -> None:
        """Scene::build_bvh / Accelerator::build (accel.h:22-32)."""
        check(lib().kz_scene_build(self._h))

    build = build_bvh

    def info(self) -> dict:
        inf = N.KzSceneInfo()
        check(lib().kz_scene_get_info(self._h, C.byref(inf)))
        return {k: getattr(inf, k) for k, _ in N.KzSceneInfo._fields_}

    def set_stream(self, stream) -> None:
        """Run on an external CUDA stream (torch.cuda.Stream or raw handle). None, or a
        handle of 0 (torch's legacy default stream), selects the library's own stream."""
        raw = None
        if stream is not None:
            raw = stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)
        check(lib().kz_scene_set_stream(self._h, C.c_void_p(raw) if raw else None))

    def synchronize(self) -> None:
        check(lib().kz_scene_synchronize(self._h))

    def release_scratch(self) -> None:
        """Free cached render scratch (wavefront buffers); the scene stays built."""
        check(lib().kz_scene_release_scratch(self._h))

    # -- intersector ------------------------------------------------------
    def intersect(self, rays, want_uv=True, out=None):
        """Closest hits. numpy ray records -> numpy outputs; a CUDA float32
        tensor (n, 8) -> CUDA tensors (asynchronous; call synchronize())."""
        if _is_cuda_tensor(rays):
            n = rays.shape[0]
            dev = rays.device
            if out is None:
                out = {"t": torch.empty(n, dtype=torch.float32, device=dev),
                       "prim_id": torch.empty(n, dtype=torch.int32, device=dev),
                       "geom_id": torch.empty(n, dtype=torch.int32, device=dev)}
                if want_uv:
                    out["u"] = torch.empty(n, dtype=torch.float32, device=dev)
                    out["v"] = torch.empty(n, dtype=torch.float32, device=dev)
            hits = N.KzHits(out["t"].data_ptr(), out["prim_id"].data_ptr(),
                            out["geom_id"].data_ptr() if "geom_id" in out else None,
                            out["u"].data_ptr() if "u" in out else None, out["v"].data_ptr() if "v" in out else None)
            check(lib().kz_intersect_closest(self._h, C.c_void_p(rays.data_ptr()), n, hits, N.KZ_MEM_DEVICE))
            return out
        r = np.ascontiguousarray(rays, dtype=N.RAY_DTYPE)
        n = len(r)
        res = {"t": np.empty(n, np.float32), "prim_id": np.empty(n, np.uint32), "geom_id": np.empty(n, np.uint32)}
        if want_uv:
            res["u"] = np.empty(n, np.float32)
            res["v"] = np.empty(n, np.float32)
        hits = N.KzHits(res["t"].ctypes.data, res["prim_id"].ctypes.data, res["geom_id"].ctypes.data,
                        res["u"].ctypes.data if want_uv else None, res["v"].ctypes.data if want_uv else None)
        check(lib().kz_intersect_closest(self._h, _ptr(r), n, hits, N.KZ_MEM_HOST))
        return res

    def occluded(self, rays, out=None):
        """Any hit in (tmin, tmax] per ray (HitableInterface::occluded, hitable.h:15-33)."""
        if _is_cuda_tensor(rays):
            n = rays.shape[0]
            if out is None:
                out = torch.empty(n, dtype=torch.uint8, device=rays.device)
            check(lib().kz_intersect_any(self._h, C.c_void_p(rays.data_ptr()), n, C.c_void_p(out.data_ptr()),
                                         N.KZ_MEM_DEVICE))
            return out
        r = np.ascontiguousarray(rays, dtype=N.RAY_DTYPE)
        occ = np.empty(len(r), np.uint8)
        check(lib().kz_intersect_any(self._h, _ptr(r), len(r), _ptr(occ), N.KZ_MEM_HOST))
        return occ.astype(bool)

    def intersect_stats(self, rays):
        """(BVH node fetches, triangle fetches) summed over the closest-hit traversal of `rays`."""
        a, b = C.c_uint64(), C.c_uint64()
        if _is_cuda_tensor(rays):
            check(lib().kz_intersect_stats(self._h, C.c_void_p(rays.data_ptr()), rays.shape[0], N.KZ_MEM_DEVICE,
                                           C.byref(a), C.byref(b)))
        else:
            r = np.ascontiguousarray(rays, dtype=N.RAY_DTYPE)
            check(lib().kz_intersect_stats(self._h, _ptr(r), len(r), N.KZ_MEM_HOST, C.byref(a), C.byref(b)))
        return a.value, b.value


# ---------------------------------------------------------------- integrator / renderer
class PathIntegrator:
    """PathIntegrator (integrator.cpp:362-561): NEE + power-heuristic MIS + roulette, batched."""

    def __init__(self, max_depth=5, rr_min_depth=3, seed=0, wavefront_size=0, block_size=0):
        self.cfg = render_config(1, max_depth, seed, wavefront_size, rr_min_depth, block_size)
        self.scene = None
        self.last_stats = None

    def setup(self, scene: Scene) -> None:
        """Integrator::setup(Scene*) (integrator.cpp:20-23)."""
        self.scene = scene

    def Li(self, rays):
        """Radiance of each camera ray; ray i uses PCG32 stream (seed, i)."""
        st = N.KzRenderStats()
        if _is_cuda_tensor(rays):
            n = rays.shape[0]
            out = torch.empty((n, 3), dtype=torch.float32, device=rays.device)
            check(lib().kz_li_batch(self.scene.handle, C.c_void_p(rays.data_ptr()), n, C.byref(self.cfg),
                                    C.c_void_p(out.data_ptr()), N.KZ_MEM_DEVICE, C.byref(st)))
        else:
            r = np.ascontiguousarray(rays, dtype=N.RAY_DTYPE)
            out = np.empty((len(r), 3), np.float32)
            check(lib().kz_li_batch(self.scene.handle, _ptr(r), len(r), C.byref(self.cfg), _ptr(out), N.KZ_MEM_HOST,
                                    C.byref(st)))
        self.last_stats = {k: getattr(st, k) for k, _ in N.KzRenderStats._fields_}
        return out


class Renderer:
    """Renderer(spp).render(scene): per-pixel spp average (renderer.cpp:18-90)."""

    def __init__(self, spp=16, max_depth=5, seed=0, wavefront_size=0, rr_min_depth=3, block_size=0, flags=0):
        self.cfg = render_config(spp, max_depth, seed, wavefront_size, rr_min_depth, block_size, flags)
        self.last_stats = None

    def render(self, scene: Scene, camera: Camera, width: int, height: int, fp64: bool = False, device_out=None,
               out=None):
        """Returns an (H, W, 3) float32 image (and the FP64 accumulation when fp64).
        out: an optional host buffer of H*W*3 float32 to write the image into
        (a C-contiguous numpy array or CPU tensor, e.g. pinned memory reused
        across frames); it is returned as the image."""
        film = N.KzFilmDesc(width, height)
        cam = camera.to_c()
        st = N.KzRenderStats()
        if device_out is not None:
            rgb, rgb64 = device_out
            check(lib().kz_render(scene.handle, C.byref(cam), C.byref(film), C.byref(self.cfg),
                                  C.c_void_p(rgb.data_ptr()), C.c_void_p(rgb64.data_ptr()) if rgb64 is not None else None,
                                  N.KZ_MEM_DEVICE, C.byref(st)))
            self.last_stats = {k: getattr(st, k) for k, _ in N.KzRenderStats._fields_}
            return rgb, rgb64
        if out is None:
            img = np.empty((height, width, 3), np.float32)
            img_ptr = _ptr(img)
        else:
            img = out
            img_ptr = _host_ptr(out, height * width * 3, np.float32)
        img64 = np.empty((height, width, 3), np.float64) if fp64 else None
        check(lib().kz_render(scene.handle, C.byref(cam), C.byref(film), C.byref(self.cfg), img_ptr, _ptr(img64),
                              N.KZ_MEM_HOST, C.byref(st)))
        self.last_stats = {k: getattr(st, k) for k, _ in N.KzRenderStats._fields_}
        return (img, img64) if fp64 else img


# ---------------------------------------------------------------- closure batches
def closure_eval(lobes, wi, wo, convention=N.KZ_CONVENTION_REFERENCE):
    lb = np.ascontiguousarray(lobes, dtype=N.LOBE_DTYPE).reshape(-1)
    a = np.ascontiguousarray(wi, np.float32).reshape(-1, 3)
    b = np.ascontiguousarray(wo, np.float32).reshape(-1, 3)
    n = len(lb)
    f = np.empty((n, 3), np.float32)
    pdf = np.empty(n, np.float32)
    check(lib().kz_closure_eval_batch(_ptr(lb), _ptr(a), _ptr(b), n, convention, _ptr(f), _ptr(pdf), N.KZ_MEM_HOST))
    return f, pdf


def closure_sample(lobes, wi, u):
    lb = np.ascontiguousarray(lobes, dtype=N.LOBE_DTYPE).reshape(-1)
    a = np.ascontiguousarray(wi, np.float32).reshape(-1, 3)
    uu = np.ascontiguousarray(u, np.float32).reshape(-1, 3)
    n = len(lb)
    wo = np.empty((n, 3), np.float32)
    w = np.empty((n, 3), np.float32)
    pdf = np.empty(n, np.float32)
    fl = np.empty(n, np.uint8)
    check(lib().kz_closure_sample_batch(_ptr(lb), _ptr(a), _ptr(uu), n, _ptr(wo), _ptr(w), _ptr(pdf), _ptr(fl),
                                        N.KZ_MEM_HOST))
    return wo, w, pdf, fl


# ---------------------------------------------------------------- learned path guiding
class Guide:
    """The guiding network (51 -> 64 -> 64 -> 64 -> 40, 8 vMF lobes) on the GPU."""

    n_params = N.KZ_GUIDE_PARAMS

    def __init__(self, seed=1):
        h = C.c_void_p()
        check(lib().kz_guide_create(C.byref(h), seed))
        self._h = h

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            lib().kz_guide_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        out = np.empty(N.KZ_GUIDE_PARAMS, np.float32)
        check(lib().kz_guide_get_params(self._h, _ptr(out)))
        return out

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == N.KZ_GUIDE_PARAMS
        check(lib().kz_guide_set_params(self._h, _ptr(p)))

    def state(self):
        """(weights, Adam first moments, Adam second moments) and the step count."""
        st = np.empty(3 * N.KZ_GUIDE_PARAMS, np.float32)
        step = C.c_uint32()
        check(lib().kz_guide_get_state(self._h, _ptr(st), C.byref(step)))
        p = N.KZ_GUIDE_PARAMS
        return (st[:p], st[p:2 * p], st[2 * p:]), step.value

    def set_state(self, params, m, v, step) -> None:
        st = np.ascontiguousarray(np.concatenate([params, m, v]), np.float32)
        check(lib().kz_guide_set_state(self._h, _ptr(st), int(step)))

    def forward(self, p01, nrm) -> np.ndarray:
        """Raw network outputs (n, 40) for points in the unit scene box with normals."""
        p01 = np.asarray(p01, np.float32).reshape(-1, 3)
        nrm = np.asarray(nrm, np.float32).reshape(-1, 3)
        pts = np.zeros((len(p01), 8), np.float32)
        pts[:, 0:3] = p01
        pts[:, 4:7] = nrm
        out = np.empty((len(p01), 40), np.float32)
        check(lib().kz_guide_forward(self._h, _ptr(pts), len(p01), _ptr(out), N.KZ_MEM_HOST))
        return out

    def train_step(self, p01, nrm, dirs, weights, lr=1e-3, apply=True, want_grad=False):
        n = len(p01)
        smp = np.zeros((n, 12), np.float32)
        smp[:, 0:3] = p01
        smp[:, 3] = weights
        smp[:, 4:7] = nrm
        smp[:, 8:11] = dirs
        loss = C.c_float()
        grad = np.empty(N.KZ_GUIDE_PARAMS, np.float32) if want_grad else None
        check(lib().kz_guide_train_step(self._h, _ptr(smp), n, lr, 1 if apply else 0, C.byref(loss), _ptr(grad),
                                        N.KZ_MEM_HOST))
        return (loss.value, grad) if want_grad else loss.value


def guide_config(alpha=0.5, learning_rate=1e-2, spp_per_pass=1, train=True, max_train_samples=1 << 18,
                 steps_per_pass=1, time_budget_ms=0.0, max_train_steps=0) -> N.KzGuideConfig:
    c = N.KzGuideConfig()
    c.alpha = alpha
    c.learning_rate = learning_rate
    c.spp_per_pass = spp_per_pass
    c.train = 1 if train else 0
    c.max_train_samples = max_train_samples
    c.steps_per_pass = steps_per_pass
    c.max_train_steps = max_train_steps
    c.time_budget_ms = time_budget_ms
    return c


def render_guided(scene: Scene, guide: Guide, camera: Camera, width: int, height: int, spp: int, max_depth: int,
                  seed=0, gcfg=None, fp64=False, wavefront_size=0, flags=0):
    """Guided render; returns (image, fp64 image or None, render stats, guide stats)."""
    cfg = render_config(spp, max_depth, seed, wavefront_size, flags=flags)
    gcfg = gcfg or guide_config()
    film = N.KzFilmDesc(width, height)
    cam = camera.to_c()
    st, gst = N.KzRenderStats(), N.KzGuideStats()
    img = np.empty((height, width, 3), np.float32)
    img64 = np.empty((height, width, 3), np.float64) if fp64 else None
    check(lib().kz_render_guided(scene.handle, guide.handle, C.byref(cam), C.byref(film), C.byref(cfg), C.byref(gcfg),
                                 _ptr(img), _ptr(img64), N.KZ_MEM_HOST, C.byref(st), C.byref(gst)))
    return (img, img64, {k: getattr(st, k) for k, _ in N.KzRenderStats._fields_},
            {k: getattr(gst, k) for k, _ in N.KzGuideStats._fields_})


# ---------------------------------------------------------------- batched rendering
BATCH_WAVEFRONT = 0
BATCH_MEGAKERNEL = 1
BATCH_PERSISTENT = 2


def batch_config(block_size=0, ctas_per_sm=0, refill_period=0, use_graph=True, mode=BATCH_WAVEFRONT,
                 wavefront_size=0) -> N.KzBatchConfig:
    c = N.KzBatchConfig()
    c.block_size = block_size
    c.ctas_per_sm = ctas_per_sm
    c.refill_period = refill_period
    c.use_graph = 1 if use_graph else 0
    c.mode = mode
    c.wavefront_size = wavefront_size
    return c


def render_batch(jobs, cfg=None):
    """jobs: list of dicts {scene, camera, width, height, spp, max_depth, seed[, rr_min_depth]}.
    Returns (list of (H, W, 3) images, stats). All jobs in one wavefront: stage
    kernels per iteration (BATCH_WAVEFRONT) or the whole loop in one cooperative
    launch (BATCH_PERSISTENT); or one persistent megakernel launch
    (BATCH_MEGAKERNEL)."""
    arr = (N.KzBatchJob * len(jobs))()
    outs = []
    for k, j in enumerate(jobs):
        img = np.empty((j["height"], j["width"], 3), np.float32)
        outs.append(img)
        a = arr[k]
        a.scene = j["scene"].handle
        a.camera = j["camera"].to_c()
        a.width, a.height = j["width"], j["height"]
        a.spp, a.max_depth = j["spp"], j["max_depth"]
        a.rr_min_depth = j.get("rr_min_depth", 3)
        a.seed = j.get("seed", 0)
        a.out_rgb = img.ctypes.data
    st = N.KzBatchStats()
    check(lib().kz_render_batch(arr, len(jobs), C.byref(cfg or batch_config()), N.KZ_MEM_HOST, C.byref(st)))
    return outs, {k: getattr(st, k) for k, _ in N.KzBatchStats._fields_}
