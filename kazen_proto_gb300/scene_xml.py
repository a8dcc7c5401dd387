"""Scene ingestion: kazen_proto's XML scene files and OBJ meshes -> SceneDesc.

Replaces Scene::parse_from_file (src/core/scene.cpp:319-712 in kazen_proto)
and load_triangle_mesh (src/core/shape.cpp:767-790, Assimp) for the parts
the GPU path renders:

* <Film width height>, <Camera position lookat up fov [near far] [scale]>
  (the scale multiplies the camera axes as Camera::scale does,
  src/core/camera.h:101-105: -1 on x mirrors the image horizontally, -1 on
  y is the vertical flip; the reference's x axis, up x (position - lookat),
  points right, so scenes written for a left-pointing camera x, like the
  cbox scenes and their scale -1, come out mirrored as the reference's own
  camera makes them);
* <Materials> of <ShaderGroupBegin name> / <Shader name layer> /
  <Parameter ...> / <ShaderGroupEnd>: each group's shader is lowered from
  its OSL source (name.osl next to the scene file) by evaluating its body
  over constant inputs (kazen_proto_gb300.osl_lower): the closures the
  reference registers (diffuse, ward, reflection, refraction, microfacet,
  kp_mirror, kp_dielectric, kp_microfacet, the kp_principle_* family) become
  lobes; kp_emitter and emission add their weight to Le; a closure weighted
  by texture(filename, u, v) or by a connected checkerboard layer
  (<ConnectShaders>) becomes a textured lobe (kz_texture: image files via
  texture_io, the checkerboard as a procedural texture);
* <EnvironmentBegin> / <Shader> / <EnvironmentEnd>: the background shader,
  `color(environment(filename, I)) * background()`, becomes the scene
  environment (constant or latitude-longitude image; an empty file name is
  black, as OIIO returns for it);
* <Objects>: <Mesh filename shader_name [is_light] [translate] [rotate]
  [scale]> from OBJ files (positions, texture coordinates and faces;
  polygons fan-triangulated, negative indices resolved), <Triangle verta
  vertb vertc> (uv = barycentrics), <Quad center dir vertical_vec half_width
  half_height> (uv over the quad, as Quad::intersect), <Sphere> (tessellated
  to an icosphere of 5,120 triangles with the reference's parametric uv);
  transforms compose as the reference's do, world = T * R * S * local,
  rotate = (axis xyz, degrees);
* integrator tags are recorded: PathEmsIntegrator and PathMatsIntegrator map to
  the NEE-only and BSDF-only estimators (`LoadedScene.render_flags`), every
  other integrator renders with the path integrator (with a warning).

Shader files are looked up next to the scene, then in the reference's shader
library directory (../../shader/src relative to the scene).

<PointLight position radiance> becomes a point light (kz_scene_add_point_light).

OBJ vertex normals (and the tessellated spheres' radial normals) become shading
normals (kz_scene_set_mesh_normals).

Not supported (reported in `LoadedScene.warnings` or raised, never silently
changed): BSSRDF closures, bump mapping and shaders whose
closure weights depend on the shading point other than through the texture
lookups above. The reference's own parser sets is_light for any `is_light`
attribute whatever its value (scene.cpp:540); this loader honours the value.
"""
from __future__ import annotations

import math
import os
import re
import xml.etree.ElementTree as ET
from dataclasses import dataclass, field

import numpy as np

from . import _native as N
from . import api, osl_lower, texture_io
from .scenes import SceneDesc, icosphere


# ---------------------------------------------------------------- typed attribute values
_NUM = re.compile(r"^[-+]?(\d+\.?\d*|\.\d+)([eE][-+]?\d+)?")


def _number(tok: str) -> float:
    """The leading number of a token, as std::stof reads it (the reference's
    parser, scene.cpp:118-128, so '0,' reads as 0)."""
    m = _NUM.match(tok)
    if not m:
        raise ValueError(f"not a number: {tok!r}")
    return float(m.group(0))


def parse_value(text: str):
    """'float3 1 2 3' -> np.array, 'float 0.5' -> float, 'int 3', 'bool true',
    'string x', 'func_translate ...' / 'func_scale ...' -> np.array."""
    parts = text.split()
    if not parts:
        return ""  # an untyped empty value, e.g. filename="" of the environment shader
    kind, vals = parts[0], parts[1:]
    if kind == "bool":
        return vals[0] == "true"
    if kind == "int":
        return int(_number(vals[0]))
    if kind == "float":
        return _number(vals[0])
    if kind in ("float3", "float4", "func_translate", "func_scale"):
        n = 4 if kind == "float4" else 3
        if len(vals) != n:
            raise ValueError(f"{kind} needs {n} numbers: {text!r}")
        return np.array([_number(v) for v in vals], np.float64)
    if kind in ("string", "ustring"):
        return vals[0] if vals else ""
    raise ValueError(f"unknown attribute type {kind!r}")


# ---------------------------------------------------------------- OBJ
def load_obj(path: str, with_uv: bool = False):
    """Vertices (n, 3) float32 and triangles (m, 3) uint32 of an OBJ file;
    with_uv also returns (n, 2) texture coordinates (None when the file has
    no `vt`), vertices split where one position carries several uvs."""
    v, t, uv, _ = load_obj_attributes(path, normals=False)
    return (v, t, uv) if with_uv else (v, t)


def load_obj_attributes(path: str, normals: bool = True):
    """(vertices (n, 3), triangles (m, 3), uvs (n, 2) or None, normals (n, 3)
    or None) of an OBJ file: a vertex per distinct (position, texcoord,
    normal) triple the faces use, polygons fan-triangulated."""
    verts, uvs, nrms, corners = [], [], [], []
    with open(path) as f:
        for line in f:
            line = line.split("#", 1)[0].strip()
            if not line:
                continue
            tok = line.split()
            if tok[0] == "v":
                verts.append([float(tok[1]), float(tok[2]), float(tok[3])])
            elif tok[0] == "vt":
                uvs.append([float(tok[1]), float(tok[2]) if len(tok) > 2 else 0.0])
            elif tok[0] == "vn":
                nrms.append([float(tok[1]), float(tok[2]), float(tok[3])])
            elif tok[0] == "f":
                idx = []
                for t in tok[1:]:
                    parts = t.split("/")
                    i = int(parts[0])
                    vi = i - 1 if i > 0 else len(verts) + i
                    ti = ni = -1
                    if len(parts) > 1 and parts[1]:
                        j = int(parts[1])
                        ti = j - 1 if j > 0 else len(uvs) + j
                    if len(parts) > 2 and parts[2]:
                        j = int(parts[2])
                        ni = j - 1 if j > 0 else len(nrms) + j
                    idx.append((vi, ti, ni))
                if len(idx) < 3:
                    raise ValueError(f"{path}: face with {len(idx)} vertices")
                for k in range(1, len(idx) - 1):  # fan
                    corners.append([idx[0], idx[k], idx[k + 1]])
    v = np.asarray(verts, np.float32).reshape(-1, 3)
    c = np.asarray(corners, np.int64).reshape(-1, 3, 3)
    if c.size and (c[..., 0].min() < 0 or c[..., 0].max() >= len(v)):
        raise ValueError(f"{path}: face index out of range")
    use_uv = bool(uvs) and (c[..., 1] >= 0).any()
    use_n = normals and bool(nrms) and (c[..., 2] >= 0).any()
    if use_uv and ((c[..., 1] < 0).any() or c[..., 1].max() >= len(uvs)):
        raise ValueError(f"{path}: texture coordinate index missing or out of range")
    if use_n and ((c[..., 2] < 0).any() or c[..., 2].max() >= len(nrms)):
        raise ValueError(f"{path}: normal index missing or out of range")
    if not use_uv and not use_n:
        return v, c[..., 0].astype(np.uint32), None, None
    keys = c[..., [0] + ([1] if use_uv else []) + ([2] if use_n else [])].reshape(len(c) * 3, -1)
    uniq, inv = np.unique(keys, axis=0, return_inverse=True)
    uv = np.asarray(uvs, np.float32)[uniq[:, 1]] if use_uv else None
    nr = np.asarray(nrms, np.float32)[uniq[:, -1]] if use_n else None
    return v[uniq[:, 0]], inv.reshape(-1, 3).astype(np.uint32), uv, nr


# ---------------------------------------------------------------- transforms
def _rotation(axis, degrees):
    a = np.asarray(axis, np.float64)
    n = np.linalg.norm(a)
    if n == 0.0 or degrees == 0.0:
        return np.eye(3)
    x, y, z = a / n
    t = math.radians(degrees)
    c, s = math.cos(t), math.sin(t)
    C = 1.0 - c
    return np.array([[c + x * x * C, x * y * C - z * s, x * z * C + y * s],
                     [y * x * C + z * s, c + y * y * C, y * z * C - x * s],
                     [z * x * C - y * s, z * y * C + x * s, c + z * z * C]])


def mesh_transform(translate=None, rotate=None, scale=None):
    """3x4 world matrix T * R * S (the reference applies translate, then
    rotate, then scale to local_to_world by right-multiplication)."""
    S = np.diag(np.asarray(scale if scale is not None else (1.0, 1.0, 1.0), np.float64))
    R = _rotation(rotate[:3], rotate[3]) if rotate is not None else np.eye(3)
    M = np.zeros((3, 4))
    M[:, :3] = R @ S
    M[:, 3] = np.asarray(translate if translate is not None else (0.0, 0.0, 0.0), np.float64)
    return M


def apply_transform(M, v):
    v = np.asarray(v, np.float64)
    return (v @ M[:, :3].T + M[:, 3]).astype(np.float32)


def apply_normal_transform(M, n):
    """Normals under the 3x4 world matrix M: its inverse transpose, renormalised."""
    n = np.asarray(n, np.float64) @ np.linalg.inv(M[:, :3])
    return (n / np.linalg.norm(n, axis=1, keepdims=True)).astype(np.float32)


# ---------------------------------------------------------------- OSL lowering
def lower_shader(src: str, params: dict, warnings: list | None = None):
    """kz_material record of a surface shader: OSL source + group parameters
    (evaluated by osl_lower over constant inputs)."""
    r = osl_lower.lower(src, params)
    if warnings is not None:
        warnings.extend(r.warnings)
    return api.material(r.lobes, Le=tuple(float(x) for x in r.Le))


def _find(paths, what):
    for p in paths:
        if os.path.exists(p):
            return p
    raise FileNotFoundError(f"{what} not found (looked in: {', '.join(paths)})")


def shader_source(base: str, name: str) -> str:
    """An .osl file next to the scene, else in the shader library two levels
    up (resource/shader/src beside resource/scene/<name>/ in kazen_proto)."""
    path = _find([os.path.join(base, name + ".osl"),
                  os.path.join(base, "..", "..", "shader", "src", name + ".osl")], f"shader {name}.osl")
    with open(path) as f:
        return f.read()


def lower_group(base: str, shaders, connections, source=None):
    """Evaluate a shader group: each layer (shader name, layer name, params)
    in order, connections (src layer, src param, dst layer, dst param) feeding
    an upstream output parameter into a downstream input; the last layer's
    closures are the group's (OSL's group semantics). `source(name)` returns
    a shader's OSL text (default: shader_source beside `base`). Returns
    osl_lower.Lowered."""
    outputs, last = {}, None
    for sname, layer, params in shaders:
        ov = dict(params)
        for sl, sp, dl, dp in connections:
            if dl == layer:
                if sl not in outputs or sp not in outputs[sl]:
                    raise ValueError(f"connection from {sl}.{sp}: no such earlier layer output")
                ov[dp] = outputs[sl][sp]
        src = source(sname) if source else shader_source(base, sname)
        if sname == "checkerboard":
            _, p = osl_lower.shader_params(src, ov)
            outputs[layer] = {"Cout": osl_lower.checkerboard_output(p)}
            last = None
        else:
            last = osl_lower.lower(src, ov)
            outputs[layer] = last.outputs
    if last is None:
        raise ValueError("the last layer of a shader group must be a surface shader")
    return last


class TextureTable:
    """Scene-wide texture list built from the lowered shaders' references."""

    def __init__(self, base: str):
        self.base = base
        self.specs, self.textures = [], []

    def index(self, spec) -> int:
        if spec in self.specs:
            return self.specs.index(spec)
        if spec[0] == "checker":
            _, ss, st, ca, cb = spec
            tex = api.checker_texture(ss, st, ca, cb)
        else:
            fname = spec[1]
            path = _find([fname if os.path.isabs(fname) else os.path.join(self.base, fname),
                          os.path.join(self.base, os.path.basename(fname))], f"texture {fname}")
            tex = api.image_texture(texture_io.read_image(path))
        self.specs.append(spec)
        self.textures.append(tex)
        return len(self.specs) - 1

    def material(self, r):
        lobes = []
        for lb in r.lobes:
            k = int(lb["params"][N.KZ_LOBE_TEXTURE_PARAM])
            if k:
                lb = api.textured(lb, self.index(r.textures[k - 1]))
            lobes.append(lb)
        return api.material(lobes, Le=tuple(float(x) for x in r.Le))


def sphere_mesh(center, radius, level=4):
    """Icosphere with the reference's parametric uv (Sphere::intersect,
    src/core/shape.cpp:81-86: u = phi / 2 pi of atan2(z, x), v = theta / pi
    + 0.5); triangles keep their own vertices so the seam does not wrap."""
    sv, sf = icosphere(level)
    v = (sv[sf].reshape(-1, 3)).astype(np.float64)
    phi = np.arctan2(v[:, 2], v[:, 0])
    phi = np.where(phi < 0, phi + 2 * np.pi, phi)
    u = (phi / (2 * np.pi)).reshape(-1, 3)
    pole = (np.hypot(v[:, 0], v[:, 2]) < 1e-6).reshape(-1, 3)
    span = np.where(pole, 0.0, u).max(axis=1, keepdims=True) - np.where(pole, 1.0, u).min(axis=1, keepdims=True)
    u = np.where((span > 0.5) & (u < 0.5), u + 1.0, u)
    # a pole has no azimuth: give it the mean of its triangle's other corners
    other = np.where(pole, 0.0, u).sum(axis=1, keepdims=True) / np.maximum(1, (~pole).sum(axis=1, keepdims=True))
    u = np.where(pole, other, u).reshape(-1)
    t = np.arccos(np.clip(v[:, 1], -1.0, 1.0)) / np.pi + 0.5
    uv = np.stack([u, t], -1).astype(np.float32)
    return (v * radius + center).astype(np.float32), np.arange(len(v), dtype=np.uint32).reshape(-1, 3), uv


# ---------------------------------------------------------------- scene
# integrator tags the GPU path renders as such: render-config flags
ESTIMATOR_FLAGS = {"PathIntegrator": 0, "PathEmsIntegrator": N.KZ_RENDER_FLAG_NEE_ONLY,
                   "PathMatsIntegrator": N.KZ_RENDER_FLAG_BSDF_ONLY}


@dataclass
class LoadedScene:
    desc: SceneDesc
    mirror_x: bool = False          # camera scale -1 on x: flip rendered images left-right
    integrator: str = "PathIntegrator"
    material_names: list = field(default_factory=list)
    warnings: list = field(default_factory=list)

    @property
    def render_flags(self) -> int:
        """kz_render_config.flags of the scene's integrator (the path integrator's for the others)."""
        return ESTIMATOR_FLAGS.get(self.integrator, 0)

    def postprocess(self, img):
        """Apply the camera's horizontal mirror to a rendered (H, W, 3) image."""
        return img[:, ::-1] if self.mirror_x else img


def load(path: str, spp: int = 16, max_depth: int = 5) -> LoadedScene:
    path = os.path.abspath(path)
    base = os.path.dirname(path)
    root = ET.parse(path).getroot()
    if root.tag != "Scene":
        raise ValueError(f"{path}: root element is <{root.tag}>, not <Scene>")
    d = SceneDesc(spp=spp, max_depth=max_depth)
    out = LoadedScene(desc=d)
    groups = {}

    def attrs(node):
        return {k: parse_value(v) for k, v in node.attrib.items() if k != "name" and k != "layer"}

    for node in root.iter():
        tag = node.tag
        if tag == "Film":
            a = attrs(node)
            d.width, d.height = int(a.get("width", 256)), int(a.get("height", 256))
        elif tag == "Camera":
            a = attrs(node)
            scale = a.get("scale", np.ones(3))
            if scale[2] < 0:
                raise ValueError("camera scale with a negative z is not supported")
            out.mirror_x = bool(scale[0] < 0)
            d.camera = api.Camera(eye=tuple(a["position"]), lookat=tuple(a["lookat"]), up=tuple(a["up"]),
                                  fov=float(a.get("fov", 30.0)), near=float(a.get("near", 1e-3)),
                                  far=float(a.get("far", 1e4)), flip=bool(scale[1] < 0))
        elif tag == "ShaderGroupBegin":
            pass  # handled with its Shader siblings below
        elif tag.endswith("Integrator"):
            out.integrator = tag
            if tag not in ESTIMATOR_FLAGS:
                out.warnings.append(f"<{tag}> rendered with the path integrator")
        elif tag == "PointLight":
            # PointLight defaults: position (0, 5, 0) (light.h:53-56), radiance 0 unless given
            a = attrs(node)
            d.point_lights.append((tuple(float(x) for x in a.get("position", (0.0, 5.0, 0.0))),
                                   tuple(float(x) for x in a.get("radiance", (0.0, 0.0, 0.0)))))

    # materials: a ShaderGroupBegin starts a group, its Shader and
    # ConnectShaders siblings follow; the environment is a group between
    # EnvironmentBegin and EnvironmentEnd at the top level
    def shader_node(node):
        params = {}
        for p in node.iter("Parameter"):
            for k, v in p.attrib.items():
                params[k] = parse_value(v)
        return node.attrib["name"], node.attrib.get("layer", ""), params

    def connection(node):
        a = node.attrib
        return a["srclayer"], a["srcparam"], a["dstlayer"], a["dstparam"]

    env_group = None
    for parent in [root] + list(root.iter("Materials")):
        current = None
        for node in list(parent):
            if node.tag in ("ShaderGroupBegin", "EnvironmentBegin"):
                current = node.attrib.get("name", "env") if node.tag == "ShaderGroupBegin" else "<environment>"
                if node.tag == "EnvironmentBegin":
                    env_group = ([], [])
                else:
                    groups[current] = ([], [])
            elif node.tag in ("ShaderGroupEnd", "EnvironmentEnd"):
                current = None
            elif node.tag in ("Shader", "ConnectShaders"):
                if current is None:
                    raise ValueError(f"<{node.tag}> outside a shader group")
                g = env_group if current == "<environment>" else groups[current]
                if node.tag == "Shader":
                    g[0].append(shader_node(node))
                else:
                    g[1].append(connection(node))
    tex = TextureTable(base)
    for name, (shaders, conns) in groups.items():
        r = lower_group(base, shaders, conns)
        d.materials.append(tex.material(r))
        out.warnings.extend(f"shader group {name!r}: {x}" for x in r.warnings)
        out.material_names.append(name)
    if env_group is not None and env_group[0]:
        try:
            r = lower_group(base, *env_group)
        except FileNotFoundError as e:
            out.warnings.append(f"environment: {e}; the background stays black")
        else:
            d.env = tuple(float(x) for x in r.background)
            if r.background_texture is not None:
                d.env_texture = tex.index(("image", r.background_texture[1]))
    d.textures = tex.textures
    mat_id = {n: i for i, n in enumerate(out.material_names)}

    def shader_of(node):
        v = node.attrib.get("shader_name")
        if v is None:
            raise ValueError(f"<{node.tag}> has no shader_name")
        name = parse_value(v) if " " in v else v
        if name not in mat_id:
            raise ValueError(f"unknown shader group {name!r}")
        return mat_id[name]

    for objs in root.iter("Objects"):
        for node in list(objs):
            a = {k: parse_value(v) for k, v in node.attrib.items() if k not in ("shader_name",)}
            light = bool(a.get("is_light", False))
            M = mesh_transform(a.get("translate"), a.get("rotate"), a.get("scale"))
            if node.tag == "Mesh":
                v, t, uv, nr = load_obj_attributes(os.path.join(base, a["filename"]))
                d.add(apply_transform(M, v), t, shader_of(node), light, uv=uv,
                      normals=None if nr is None else apply_normal_transform(M, nr))
            elif node.tag == "Triangle":
                v = np.stack([a["verta"], a["vertb"], a["vertc"]])
                d.add(apply_transform(M, v), np.array([[0, 1, 2]], np.uint32), shader_of(node), light)
            elif node.tag == "Quad":
                n = np.asarray(a["dir"], np.float64)
                up = np.asarray(a["vertical_vec"], np.float64)
                h = np.cross(up, n)
                h /= np.linalg.norm(h)
                c, hw, hh = np.asarray(a["center"]), float(a["half_width"]), float(a["half_height"])
                q = np.stack([c - h * hw - up * hh, c + h * hw - up * hh, c + h * hw + up * hh, c - h * hw + up * hh])
                # uv of Quad::intersect (shape.cpp:335-345): P = c + h hw (u - 1/2) + up hh (v - 1/2)
                d.add(apply_transform(M, q), np.array([[0, 1, 2], [0, 2, 3]], np.uint32), shader_of(node), light,
                      uv=np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32))
            elif node.tag == "Sphere":
                cr = a["center_n_radius"]
                v, sf, uv = sphere_mesh(cr[:3], cr[3])
                d.add(apply_transform(M, v), sf, shader_of(node), light, uv=uv,
                      normals=apply_normal_transform(M, v - np.asarray(cr[:3], np.float32)))
                out.warnings.append("<Sphere> tessellated to an icosphere of %d triangles" % len(sf))
            elif node.tag != "PointLight":  # read with the lights above
                out.warnings.append(f"<{node.tag}> in <Objects> is not supported and was skipped")
    if d.camera is None:
        raise ValueError(f"{path}: no <Camera>")
    return out
