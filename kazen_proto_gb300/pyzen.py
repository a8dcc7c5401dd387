"""pyzen-compatible Python interface over the GPU path.

Mirrors the names and argument meanings of kazen_proto's pybind11 module
(src/binding/api.cpp:84-232, src/binding/base_types.cpp:363-392), so that a
pyzen caller (the Blender add-on drives a scene this way) can switch to the
GPU renderer:

    api.Scene: parse_from_file, set_film, set_camera, set_accelerator,
        set_integrator, add_sphere, add_triangle, add_quad, add_mesh,
        build_bvh, set_shader_search_path, begin_shader_group,
        load_oso_shader, set_shader_param_*, end_shader_group
    api.Renderer(sample_count, nthreads, callback).render(scene | file, output)
    api.RenderCallback.on_tile_end(film, tile_id)
    api.AcceleratorType, api.IntegratorType
    concepts.Film (tiles, generate_tiles, write_tiles, ...), concepts.Tile

Differences, each stated where it happens: shaders are lowered from their
OSL source (load_oso_shader looks for name.osl, not the compiled .oso; shader
networks and texture lookups lower as scene_xml lowers them, texture files
relative to the working directory); spheres are
tessellated (with the reference's parametric uv); PathEmsIntegrator and
PathMatIntegrator render with the NEE-only and BSDF-only estimators, every
other integrator type with the path integrator; the frame renders in one GPU call and on_tile_end then runs for
each tile in tile order; tiles cover the film exactly (the reference's
generate_tiles, film.cpp:66-78, gives the last row and column the nominal
size and the others the remainder, which overlaps tiles and leaves pixels
uncovered when the size does not divide evenly); Renderer.render writes no
file (neither does the reference's), Film.write_tiles writes one by
extension (film_io).
"""
from __future__ import annotations

import enum
import os
import types

import numpy as np

from . import api as _api
from . import film_io, scene_xml
from .scenes import SceneDesc


class AcceleratorType(enum.Enum):
    BVH = 0
    Embree = 1


class IntegratorType(enum.Enum):
    NormalIntegrator = 0
    AmbientOcclusionIntegrator = 1
    WhittedIntegrator = 2
    PathMatIntegrator = 3
    PathEmsIntegrator = 4
    PathIntegrator = 5


# the integrators the GPU path renders as such (render-config flags)
_ESTIMATOR_FLAGS = {IntegratorType.PathIntegrator: 0,
                    IntegratorType.PathEmsIntegrator: _api.N.KZ_RENDER_FLAG_NEE_ONLY,
                    IntegratorType.PathMatIntegrator: _api.N.KZ_RENDER_FLAG_BSDF_ONLY}


# ---------------------------------------------------------------- concepts
class Tile:
    """A rectangle of the film; get_data() is its RGB floats, row by row."""

    def __init__(self, x: int, y: int, width: int, height: int):
        self.x, self.y, self.width, self.height = int(x), int(y), int(width), int(height)
        self._rgb = np.zeros((self.height, self.width, 3), np.float32)

    def set_pixel_color(self, i: int, j: int, rgb) -> None:
        self._rgb[j, i] = rgb

    def set_tile_color(self, rgb) -> None:
        self._rgb[...] = rgb

    def get_data(self) -> list:
        return self._rgb.reshape(-1).tolist()


class Film:
    def __init__(self, width: int = 800, height: int = 600, tile_res_x: int = 1, tile_res_y: int = 1,
                 filename: str = "./test.png"):
        if width <= 0 or height <= 0 or tile_res_x <= 0 or tile_res_y <= 0:
            raise ValueError("film size and tile counts must be positive")
        self.width, self.height = int(width), int(height)
        self.tile_res_x, self.tile_res_y = int(tile_res_x), int(tile_res_y)
        self.filename = filename
        self.tiles: list[Tile] = []

    def generate_tiles(self) -> None:
        self.tile_width = self.width // self.tile_res_x
        self.tile_height = self.height // self.tile_res_y
        self.tiles = []
        for j in range(self.tile_res_y):
            th = self.height - self.tile_height * j if j == self.tile_res_y - 1 else self.tile_height
            for i in range(self.tile_res_x):
                tw = self.width - self.tile_width * i if i == self.tile_res_x - 1 else self.tile_width
                self.tiles.append(Tile(i * self.tile_width, j * self.tile_height, tw, th))

    def get_tile_count(self) -> int:
        return len(self.tiles)

    def set_film_color(self, rgb) -> None:
        for t in self.tiles:
            t.set_tile_color(rgb)

    def set_tile_color(self, rgb, xidx: int, yidx: int) -> None:
        self.tiles[self.tile_res_x * yidx + xidx].set_tile_color(rgb)

    def image(self) -> np.ndarray:
        img = np.zeros((self.height, self.width, 3), np.float32)
        for t in self.tiles:
            img[t.y:t.y + t.height, t.x:t.x + t.width] = t._rgb
        return img

    def write_tiles(self) -> bool:
        film_io.write_image(self.filename, self.image())
        return True


concepts = types.SimpleNamespace(Film=Film, Tile=Tile)


# ---------------------------------------------------------------- api
def _world(world) -> np.ndarray:
    """3x4 affine part of a 4x4 world matrix (row-major, translation in the
    last column), or the identity."""
    if world is None:
        return scene_xml.mesh_transform()
    m = np.asarray(world, np.float64)
    if m.shape != (4, 4):
        raise ValueError("world must be a 4x4 matrix")
    return m[:3, :4]


class Scene:
    def __init__(self):
        self.desc = SceneDesc()
        self.film = Film()
        self.film.generate_tiles()
        self.integrator = IntegratorType.PathIntegrator
        self.warnings: list[str] = []
        self._search = []
        self._groups: dict[str, int] = {}
        self._group = None          # [name, [(shader, layer, params, source path)], connections]
        self._tex = scene_xml.TextureTable(os.getcwd())
        self._built = None          # the GPU scene after build_bvh
        self._mirror_x = False

    # -- scene file
    def parse_from_file(self, path: str) -> None:
        L = scene_xml.load(path)
        self.desc = L.desc
        self._groups = {n: i for i, n in enumerate(L.material_names)}
        self._mirror_x = L.mirror_x
        self.warnings += L.warnings
        self.integrator = {"PathEmsIntegrator": IntegratorType.PathEmsIntegrator,
                           "PathMatsIntegrator": IntegratorType.PathMatIntegrator}.get(L.integrator,
                                                                                       IntegratorType.PathIntegrator)
        self.film = Film(L.desc.width, L.desc.height, 1, 1)
        self.film.generate_tiles()
        self._built = None  # built by build_bvh or the first render, as the reference defers it

    # -- film and camera
    def set_film(self, w: int, h: int, xres: int, yres: int, filename: str) -> None:
        self.film = Film(w, h, xres, yres, filename)
        self.film.generate_tiles()
        self.desc.width, self.desc.height = int(w), int(h)

    def set_camera(self, p, l, u, near_plane: float = 1.0, far_plane: float = 1000.0, fov: float = 60.0) -> None:
        """Camera(p, l, u, near, far, fov, film, flip = true), as the reference's set_camera builds it."""
        self.desc.camera = _api.Camera(eye=tuple(map(float, p)), lookat=tuple(map(float, l)),
                                       up=tuple(map(float, u)), fov=float(fov), near=float(near_plane),
                                       far=float(far_plane), flip=True)

    def set_accelerator(self, kind: AcceleratorType) -> None:
        pass  # one accelerator: the 8-wide GPU BVH

    def set_integrator(self, kind: IntegratorType) -> None:
        self.integrator = kind
        if kind not in _ESTIMATOR_FLAGS:
            self.warnings.append(f"{kind.name} renders with the path integrator")

    # -- shaders
    def set_shader_search_path(self, path: str) -> None:
        self._search = [p for p in path.split(":") if p]

    def begin_shader_group(self, name: str) -> None:
        self._group = [name, [], []]
        self._pending = {}

    def load_oso_shader(self, kind: str, name: str, layer: str, lib_path: str) -> bool:
        if self._group is None:
            raise RuntimeError("load_oso_shader outside a shader group")
        for d in [lib_path] + self._search:
            src = os.path.join(d, name + ".osl")
            if os.path.exists(src):
                self._group[1].append((name, layer, self._pending, src))
                self._pending = {}
                return True
        raise FileNotFoundError(f"no OSL source {name}.osl in {[lib_path] + self._search} (needed to lower it)")

    def _param(self, name, value):
        """A parameter of the next shader loaded in the group, as OSL's
        Parameter() calls precede their Shader() (scene.cpp:631, 316);
        parameters set after the group's last shader apply to that shader."""
        if self._group is None:
            raise RuntimeError("shader parameter outside a shader group")
        self._pending[name] = value

    def set_shader_param_bool(self, name, value): self._param(name, bool(value))
    def set_shader_param_int(self, name, value): self._param(name, int(value))
    def set_shader_param_float(self, name, value): self._param(name, float(value))
    def set_shader_param_vec3f(self, name, value): self._param(name, np.asarray(value, np.float64).reshape(3))
    def set_shader_param_vec4f(self, name, value): self._param(name, np.asarray(value, np.float64).reshape(4))
    def set_shader_param_str(self, name, value): self._param(name, str(value))
    def set_shader_param_ustr(self, name, value): self._param(name, str(value))

    def connect_shader(self, src_layer, src_param, dst_layer, dst_param):
        if self._group is None:
            raise RuntimeError("connect_shader outside a shader group")
        self._group[2].append((src_layer, src_param, dst_layer, dst_param))

    def end_shader_group(self) -> None:
        name, shaders, conns = self._group
        if not shaders:
            raise RuntimeError(f"shader group {name!r} has no shader")
        shaders[-1][2].update(self._pending)
        self._pending = {}
        paths = {sname: src for sname, _, _, src in shaders}

        def source(sname):
            with open(paths[sname]) as f:
                return f.read()
        r = scene_xml.lower_group("", [(a, b, c) for a, b, c, _ in shaders], conns, source)
        self.warnings += [f"shader group {name!r}: {w}" for w in r.warnings]
        self.desc.materials.append(self._tex.material(r))
        self.desc.textures = self._tex.textures
        self._groups[name] = len(self.desc.materials) - 1
        self._group = None

    def _material(self, shader_name: str) -> int:
        if shader_name not in self._groups:
            raise KeyError(f"unknown shader group {shader_name!r}")
        return self._groups[shader_name]

    # -- geometry
    def add_mesh(self, world, vs, ns, ts, idx, name: str, shader_name: str, is_light: bool = False) -> None:
        """ns: per-vertex normals (shading normals; None / empty: the geometric
        normal); ts: per-vertex texture coordinates (None / empty: uv = barycentrics)."""
        M = _world(world)
        v = scene_xml.apply_transform(M, np.asarray(vs, np.float64).reshape(-1, 3))
        uv = None if ts is None or len(ts) == 0 else np.asarray(ts, np.float32).reshape(-1, 2)
        nr = None if ns is None or len(ns) == 0 else scene_xml.apply_normal_transform(
            M, np.asarray(ns, np.float64).reshape(-1, 3))
        self.desc.add(v, np.asarray(idx, np.uint32).reshape(-1, 3), self._material(shader_name), bool(is_light),
                      uv=uv, normals=nr)

    def add_triangle(self, world, a, b, c, name: str, shader_name: str, is_light: bool = False) -> None:
        self.add_mesh(world, [a, b, c], None, None, [[0, 1, 2]], name, shader_name, is_light)

    def add_quad(self, world, c, d, u, w: float, h: float, name: str, shader_name: str,
                 is_light: bool = False) -> None:
        n, up = np.asarray(d, np.float64), np.asarray(u, np.float64)
        hv = np.cross(up, n)
        hv /= np.linalg.norm(hv)
        c = np.asarray(c, np.float64)
        q = [c - hv * w - up * h, c + hv * w - up * h, c + hv * w + up * h, c - hv * w + up * h]
        self.add_mesh(world, q, None, [[0, 0], [1, 0], [1, 1], [0, 1]], [[0, 1, 2], [0, 2, 3]], name, shader_name,
                      is_light)

    def add_sphere(self, world, p, r: float, name: str, shader_name: str, is_light: bool = False) -> None:
        v, f, uv = scene_xml.sphere_mesh(np.asarray(p, np.float64), float(r))
        self.add_mesh(world, v, v - np.asarray(p, np.float32), uv, f, name, shader_name, is_light)
        self.warnings.append(f"sphere {name!r} tessellated to {len(f)} triangles")

    def add_point_light(self, radiance, position, shader_name) -> None:
        """A PointLight at `position` (shader_name is not used by the reference's point light either)."""
        self.desc.point_lights.append((tuple(map(float, position)), tuple(map(float, radiance))))

    def build_bvh(self, names=None) -> None:
        if self._built is not None:
            self._built.close()
        self._built = self.desc.build()


class RenderCallback:
    """Subclass and override on_tile_end(film, tile_id)."""

    def on_tile_end(self, film: Film, tile_id: int) -> None:
        pass


class Renderer:
    """Renderer(sample_count, nthreads, callback). nthreads is accepted for
    API parity (the GPU renders the frame); max_depth follows the reference's
    PathIntegrator (8)."""

    def __init__(self, sample_count: int = 16, nthreads: int = 0, callback: RenderCallback | None = None,
                 max_depth: int = 8, seed: int = 0):
        self.sample_count, self.nthreads, self.callback = int(sample_count), int(nthreads), callback
        self.max_depth, self.seed = int(max_depth), int(seed)

    def render(self, scene, output: str = "./test.png") -> bool:
        if isinstance(scene, str):
            path = scene
            scene = Scene()
            scene.parse_from_file(path)
        if scene._built is None:
            scene.build_bvh()
        if scene.desc.camera is None:
            raise RuntimeError("camera not set")
        film = scene.film
        r = _api.Renderer(spp=self.sample_count, max_depth=self.max_depth, seed=self.seed,
                          flags=_ESTIMATOR_FLAGS.get(scene.integrator, 0))
        img = r.render(scene._built, scene.desc.camera, film.width, film.height)
        if scene._mirror_x:
            img = img[:, ::-1]
        for t_id, t in enumerate(film.tiles):
            t._rgb[...] = img[t.y:t.y + t.height, t.x:t.x + t.width]
            if self.callback is not None:
                self.callback.on_tile_end(film, t_id)
        film.filename = output
        self.last_stats = r.last_stats
        return True


api = types.SimpleNamespace(Scene=Scene, Renderer=Renderer, RenderCallback=RenderCallback,
                            AcceleratorType=AcceleratorType, IntegratorType=IntegratorType)
