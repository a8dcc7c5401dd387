"""kazen_proto_gb300 — GB300-native (sm_103a) rendering hot path of kazen_proto.

BVH traversal, closure sample/eval/pdf, area-light NEE with MIS and the path
integrator loop, run as hand-written CUDA kernels behind the C ABI in
include/kazen_gb300.h. The Python layer (api.py) mirrors the reference's
Scene / intersector / PathIntegrator / Renderer interfaces over that ABI.
"""
from . import _native
from .api import (Camera, PathIntegrator, Renderer, Scene, closure_eval, closure_sample, conductor_ggx, dielectric,
                  diffuse, make_rays, material, microfacet, mirror, principle_specular, render_config)

__all__ = ["Camera", "PathIntegrator", "Renderer", "Scene", "closure_eval", "closure_sample", "conductor_ggx",
           "dielectric", "diffuse", "make_rays", "material", "microfacet", "mirror", "principle_specular",
           "render_config", "_native"]
