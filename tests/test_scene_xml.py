"""CPU tests of the scene loader (kazen_proto_gb300.scene_xml): typed
attribute values, OBJ parsing (fan triangulation, negative indices), the
reference's transform order (world = T * R * S * local), lowering of OSL
surface shaders to closure records, and loading the box_room fixture
(tests/golden/scenes, written by tests/golden/make_scene_fixtures.py)."""
import os

import numpy as np
import pytest

from kazen_proto_gb300 import _native as N
from kazen_proto_gb300 import scene_xml as X

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "scenes", "box_room", "scene.xml")


def test_parse_value():
    assert X.parse_value("int 7") == 7
    assert X.parse_value("float 0.25") == 0.25
    assert X.parse_value("bool true") is True and X.parse_value("bool false") is False
    assert X.parse_value("string meshes/a.obj") == "meshes/a.obj"
    assert np.array_equal(X.parse_value("float3 1 2 3"), [1, 2, 3])
    assert np.array_equal(X.parse_value("func_scale 0.5 0.5 2"), [0.5, 0.5, 2])
    assert np.array_equal(X.parse_value("float4 0 1 0 90"), [0, 1, 0, 90])
    # numbers are read as std::stof reads them: the leading number of a token
    assert np.array_equal(X.parse_value("float3 0, 3 -2e1"), [0, 3, -20])
    with pytest.raises(ValueError):
        X.parse_value("float3 1 2")
    with pytest.raises(ValueError):
        X.parse_value("matrix 1")


def test_obj_fan_triangulation_and_negative_indices(tmp_path):
    p = tmp_path / "m.obj"
    p.write_text("# quad and pentagon\nv 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvn 0 0 1\n"
                 "f 1//1 2//1 3//1 4//1\nv 2 0 0\nv 3 0 0\nv 3 1 0\nv 2.5 2 0\nv 2 1 0\n"
                 "f -5/1 -4/2 -3/3 -2/4 -1/5\n")
    v, t = X.load_obj(str(p))
    assert v.shape == (9, 3) and v.dtype == np.float32
    assert t.tolist() == [[0, 1, 2], [0, 2, 3], [4, 5, 6], [4, 6, 7], [4, 7, 8]]


def test_obj_rejects_bad_faces(tmp_path):
    p = tmp_path / "bad.obj"
    p.write_text("v 0 0 0\nv 1 0 0\nf 1 2 3\n")
    with pytest.raises(ValueError):
        X.load_obj(str(p))
    p.write_text("v 0 0 0\nv 1 0 0\nf 1 2\n")
    with pytest.raises(ValueError):
        X.load_obj(str(p))


def test_transform_order_is_translate_rotate_scale():
    M = X.mesh_transform(translate=(1, 2, 3), rotate=(0, 1, 0, 90), scale=(2, 1, 1))
    # scale first: (1,0,0) -> (2,0,0); rotate +90 deg about y: -> (0,0,-2); translate
    p = X.apply_transform(M, [[1, 0, 0]])[0]
    assert np.allclose(p, [1, 2, 1], atol=1e-6)
    assert np.allclose(X.apply_transform(X.mesh_transform(), [[4, 5, 6]]), [[4, 5, 6]])


def lobes(m):
    return [(int(l["closure_id"]), np.round(np.asarray(l["weight"], np.float64), 6).tolist())
            for l in m["lobes"][:m["n_lobes"]]]


def test_shader_lowering():
    src = '''surface s ( color Cs = 0.7, float alpha = 0.3, float eta = 1.5 )
    {
        // Ci = Cs * kp_mirror();
        Ci = 0.5 * Cs * diffuse(N) + 0.1 * Cs * microfacet("beckmann", N, alpha, eta, 0);
    }'''
    m = X.lower_shader(src, {"Cs": np.array([1.0, 0.5, 0.25]), "alpha": 0.2})
    assert lobes(m) == [(N.KZ_CLOSURE_DIFFUSE, [0.5, 0.25, 0.125]), (N.KZ_CLOSURE_KP_GLOSS, [0.1, 0.05, 0.025])]
    gloss = m["lobes"][1]["params"]
    assert gloss[0] == N.KZ_DIST_BECKMANN and np.isclose(gloss[7], 0.2) and np.isclose(gloss[9], 1.5)
    e = X.lower_shader("surface e ( color Cs = 1 ) { Ci = Cs * emission(); }", {"Cs": np.array([3.0, 2, 1])})
    assert e["n_lobes"] == 0 and np.allclose(e["Le"], [3, 2, 1])
    d = X.lower_shader("surface d ( color Cs = 1 ) { Ci = Cs * kp_dielectric(1.5046, 1.000277); }", {})
    assert lobes(d) == [(N.KZ_CLOSURE_KP_DIELECTRIC, [1.0, 1.0, 1.0])]
    with pytest.raises(ValueError):
        X.lower_shader("surface w ( color Cs = 1 ) { Ci = Cs * ward(N, 0.1, 0.2); }", {})
    with pytest.raises(ValueError):
        X.lower_shader("surface u ( color Cs = 1 ) { Ci = kd * diffuse(N); }", {})


def test_load_fixture_scene():
    L = X.load(FIXTURE)
    d = L.desc
    assert (d.width, d.height) == (64, 48) and L.mirror_x and L.integrator == "PathIntegrator"
    assert L.material_names == ["white", "red", "green", "coated", "mirror", "glass", "light"]
    assert L.warnings == []
    assert [m[2] for m in d.meshes] == [0, 1, 2, 4, 3, 5, 6]
    assert [m[3] for m in d.meshes] == [False] * 6 + [True]
    assert d.n_triangles() == 6 + 2 + 2 + 12 + 320 + 1 + 2
    assert np.allclose(d.materials[6]["Le"], [17, 12, 4]) and d.materials[6]["n_lobes"] == 0
    # every wall faces into the room, the light faces down
    for k, want in ((1, (1, 0, 0)), (2, (-1, 0, 0)), (6, (0, -1, 0))):
        v, i = d.meshes[k][0], d.meshes[k][1]
        n = np.cross(v[i[:, 1]] - v[i[:, 0]], v[i[:, 2]] - v[i[:, 0]])
        n /= np.linalg.norm(n, axis=1, keepdims=True)
        assert np.allclose(n, want, atol=1e-6)
    # the mirrored camera flips images left-right
    img = np.arange(2 * 3 * 3, dtype=np.float32).reshape(2, 3, 3)
    assert np.array_equal(L.postprocess(img), img[:, ::-1])


def test_loader_errors(tmp_path):
    osl = "surface matte ( color Cs = 0.5 ) { Ci = Cs * diffuse(N); }"
    (tmp_path / "matte.osl").write_text(osl)
    (tmp_path / "t.obj").write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n")
    cam = '<Camera position="float3 0 0 5" lookat="float3 0 0 0" up="float3 0 1 0" fov="float 30"/>'
    group = ('<Materials><ShaderGroupBegin name="m"/><Shader name="matte" layer="a"/>'
             '<ShaderGroupEnd/></Materials>')

    def scene(body):
        p = tmp_path / "s.xml"
        p.write_text("<Scene>" + body + "</Scene>")
        return str(p)

    with pytest.raises(ValueError):  # unknown shader group
        X.load(scene(cam + group + '<Objects><Mesh filename="string t.obj" shader_name="x"/></Objects>'))
    with pytest.raises(ValueError):  # no camera
        X.load(scene(group + '<Objects><Mesh filename="string t.obj" shader_name="m"/></Objects>'))
    two = ('<Materials><ShaderGroupBegin name="m"/><Shader name="matte" layer="a"/>'
           '<Shader name="matte" layer="b"/><ShaderGroupEnd/></Materials>')
    with pytest.raises(ValueError):  # shader networks are not lowered
        X.load(scene(cam + two))
    L = X.load(scene(cam + group + '<Objects><Mesh filename="string t.obj" shader_name="m" is_light="bool false"/>'
                     '<PointLight/></Objects><WhittedIntegrator/>'))
    assert L.desc.meshes[0][3] is False and len(L.warnings) == 2
