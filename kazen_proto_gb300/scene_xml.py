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
  lobes; kp_emitter and emission add their weight to Le;
* <Objects>: <Mesh filename shader_name [is_light] [translate] [rotate]
  [scale]> from OBJ files (positions and faces; polygons fan-triangulated,
  negative indices resolved), <Triangle verta vertb vertc>, <Quad center dir
  vertical_vec half_width half_height>; transforms compose as the
  reference's do, world = T * R * S * local, rotate = (axis xyz, degrees);
* integrator tags are recorded; rendering always uses the path integrator.

Not supported (reported in `LoadedScene.warnings`, never silently changed):
analytic <Sphere> (tessellated to an icosphere of 5,120 triangles), point
lights, textures and shader networks (<ConnectShaders>), the environment
shader (a miss contributes nothing). Shading uses geometric normals (OBJ
vertex normals are not read). The reference's own parser sets is_light for
any `is_light` attribute whatever its value (scene.cpp:540); this loader
honours the value.
"""
from __future__ import annotations

import math
import os
import re
import xml.etree.ElementTree as ET
from dataclasses import dataclass, field

import numpy as np

from . import api, osl_lower
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
        raise ValueError("empty attribute value")
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
def load_obj(path: str):
    """Vertices (n, 3) float32 and triangles (m, 3) uint32 of an OBJ file."""
    verts, tris = [], []
    with open(path) as f:
        for line in f:
            line = line.split("#", 1)[0].strip()
            if not line:
                continue
            tok = line.split()
            if tok[0] == "v":
                verts.append([float(tok[1]), float(tok[2]), float(tok[3])])
            elif tok[0] == "f":
                idx = []
                for t in tok[1:]:
                    i = int(t.split("/")[0])
                    idx.append(i - 1 if i > 0 else len(verts) + i)
                if len(idx) < 3:
                    raise ValueError(f"{path}: face with {len(idx)} vertices")
                for k in range(1, len(idx) - 1):  # fan
                    tris.append([idx[0], idx[k], idx[k + 1]])
    v = np.asarray(verts, np.float32).reshape(-1, 3)
    t = np.asarray(tris, np.int64).reshape(-1, 3)
    if t.size and (t.min() < 0 or t.max() >= len(v)):
        raise ValueError(f"{path}: face index out of range")
    return v, t.astype(np.uint32)


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


# ---------------------------------------------------------------- OSL lowering
def lower_shader(src: str, params: dict, warnings: list | None = None):
    """kz_material record of a surface shader: OSL source + group parameters
    (evaluated by osl_lower over constant inputs)."""
    r = osl_lower.lower(src, params)
    if warnings is not None:
        warnings.extend(r.warnings)
    return api.material(r.lobes, Le=tuple(float(x) for x in r.Le))


# ---------------------------------------------------------------- scene
@dataclass
class LoadedScene:
    desc: SceneDesc
    mirror_x: bool = False          # camera scale -1 on x: flip rendered images left-right
    integrator: str = "PathIntegrator"
    material_names: list = field(default_factory=list)
    warnings: list = field(default_factory=list)

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
            if tag != "PathIntegrator":
                out.warnings.append(f"<{tag}> rendered with the path integrator")
        elif tag in ("PointLight", "ConnectShaders"):
            out.warnings.append(f"<{tag}> is not supported and was skipped")

    # materials: a ShaderGroupBegin starts a group, its Shader siblings follow
    for mats in root.iter("Materials"):
        current = None
        for node in list(mats):
            if node.tag == "ShaderGroupBegin":
                current = node.attrib["name"]
                groups[current] = []
            elif node.tag == "ShaderGroupEnd":
                current = None
            elif node.tag == "Shader":
                if current is None:
                    raise ValueError("<Shader> outside a shader group")
                params = {}
                for p in node.iter("Parameter"):
                    for k, v in p.attrib.items():
                        params[k] = parse_value(v)
                groups[current].append((node.attrib["name"], params))
    for name, shaders in groups.items():
        if len(shaders) != 1:
            raise ValueError(f"shader group {name!r} has {len(shaders)} shaders; networks are not lowered")
        sname, params = shaders[0]
        osl = os.path.join(base, sname + ".osl")
        with open(osl) as f:
            w = []
            d.materials.append(lower_shader(f.read(), params, w))
        out.warnings.extend(f"shader group {name!r}: {x}" for x in w)
        out.material_names.append(name)
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
                v, t = load_obj(os.path.join(base, a["filename"]))
                d.add(apply_transform(M, v), t, shader_of(node), light)
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
                d.add(apply_transform(M, q), np.array([[0, 1, 2], [0, 2, 3]], np.uint32), shader_of(node), light)
            elif node.tag == "Sphere":
                cr = a["center_n_radius"]
                sv, sf = icosphere(4)
                v = sv * cr[3] + cr[:3]
                d.add(apply_transform(M, v), sf, shader_of(node), light)
                out.warnings.append("<Sphere> tessellated to an icosphere of %d triangles" % len(sf))
            elif node.tag != "PointLight":  # reported with the other unsupported tags
                out.warnings.append(f"<{node.tag}> in <Objects> is not supported and was skipped")
    if d.camera is None:
        raise ValueError(f"{path}: no <Camera>")
    return out
