"""A scene read from kazen_proto's XML format (the box_room fixture: OBJ
meshes with transforms, Triangle and Quad elements, lowered OSL shaders,
an area light, a mirrored camera) renders on the GPU as the CPU
restatement renders the same description: relMSE <= 1e-3 against the
restatement's FP64 image, the bound of the other image tests."""
import os

import numpy as np
import pytest

from kazen_proto_gb300 import api
from kazen_proto_gb300 import scene_xml as X

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "scenes", "box_room", "scene.xml")
TEXTURED = os.path.join(HERE, "golden", "scenes", "textured_room", "scene.xml")


def rel_mse(img, ref, eps=1e-2):
    img = np.asarray(img, np.float64)
    ref = np.asarray(ref, np.float64)
    return float(np.mean((img - ref) ** 2 / (ref ** 2 + eps)))


def test_xml_scene_matches_restatement(gpu, oracle_mod):
    L = X.load(FIXTURE, spp=16, max_depth=5)
    d = L.desc
    s = d.build()
    W, H, spp = d.width, d.height, 16
    img = L.postprocess(api.Renderer(spp=spp, max_depth=5, seed=3).render(s, d.camera, W, H))
    cam = d.camera
    ocam = oracle_mod.make_camera(cam.eye, cam.lookat, cam.up, cam.fov, cam.flip)
    ref, _ = oracle_mod.Scene.from_desc(d).render(ocam, W, H, spp, 5, seed=3)
    ref = L.postprocess(ref)
    assert ref.mean() > 1e-3  # the light reaches the camera
    assert rel_mse(img, ref) <= 1e-3
    s.close()


def test_textured_xml_scene_matches_restatement(gpu, oracle_mod):
    """The textured_room fixture: a checkerboard shader network, PNG textures
    at sphere and OBJ uvs, a PFM environment map."""
    L = X.load(TEXTURED, spp=16, max_depth=5)
    d = L.desc
    assert len(d.textures) == 3 and d.env_texture == 2
    s = d.build()
    W, H, spp = d.width, d.height, 16
    img = api.Renderer(spp=spp, max_depth=5, seed=5).render(s, d.camera, W, H)
    cam = d.camera
    ocam = oracle_mod.make_camera(cam.eye, cam.lookat, cam.up, cam.fov, cam.flip)
    ref, _ = oracle_mod.Scene.from_desc(d).render(ocam, W, H, spp, 5, seed=5)
    assert ref.mean() > 1e-2
    assert rel_mse(img, ref) <= 1e-3
    s.close()
