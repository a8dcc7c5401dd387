"""CPU tests of the scene loader (kazen_proto_gb300.scene_xml): typed
attribute values, OBJ parsing (fan triangulation, negative indices), the
reference's transform order (world = T * R * S * local), lowering of OSL
surface shaders to closure records, and loading the box_room fixture
(tests/golden/scenes, written by tests/golden/make_scene_fixtures.py)."""
import os

import numpy as np
import pytest

from kazen_proto_gb300 import _native as N
from kazen_proto_gb300 import film_io
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
    bad_link = ('<Materials><ShaderGroupBegin name="m"/><Shader name="matte" layer="a"/>'
                '<ConnectShaders srclayer="z" srcparam="Cout" dstlayer="a" dstparam="Cs"/>'
                '<ShaderGroupEnd/></Materials>')
    with pytest.raises(ValueError):  # a connection from a layer that does not exist
        X.load(scene(cam + bad_link))
    L = X.load(scene(cam + group + '<Objects><Mesh filename="string t.obj" shader_name="m" is_light="bool false"/>'
                     '</Objects><Lights><PointLight radiance="float3 1 2 3" position="float3 0 4 0"/></Lights>'
                     '<WhittedIntegrator/>'))
    assert L.desc.meshes[0][3] is False and len(L.warnings) == 1
    assert L.desc.point_lights == [((0.0, 4.0, 0.0), (1.0, 2.0, 3.0))]
    assert L.render_flags == 0  # Whitted renders with the path integrator (the warning)
    L = X.load(scene(cam + group + '<Objects><Mesh filename="string t.obj" shader_name="m"/></Objects>'
                     '<PathEmsIntegrator/>'))
    assert L.render_flags == N.KZ_RENDER_FLAG_NEE_ONLY and not L.warnings
    L = X.load(scene(cam + group + '<Objects><Mesh filename="string t.obj" shader_name="m"/></Objects>'
                     '<PathMatsIntegrator/>'))
    assert L.render_flags == N.KZ_RENDER_FLAG_BSDF_ONLY and not L.warnings


CHECKER_OSL = """shader checkerboard (
    float s = u, float t = v, float scale_s = 4, float scale_t = 4,
    color Ca = color(1, 1, 1), color Cb = color(0, 0, 0),
    output color Cout = 0)
{
    // the parity rule of OSL's checkerboard example
    float cs = fmod(s * scale_s, 2);
    float ct = fmod(t * scale_t, 2);
    if ((int(cs) ^ int(ct)) == 0) Cout = Ca; else Cout = Cb;
}
"""


def _scene_dir(tmp_path, shaders, materials, objects, extra=""):
    for name, src in shaders.items():
        (tmp_path / (name + ".osl")).write_text(src)
    (tmp_path / "s.xml").write_text(
        '<Scene><Camera position="float3 0 0 5" lookat="float3 0 0 0" up="float3 0 1 0" fov="float 30"/>'
        + extra + "<Materials>" + materials + "</Materials><Objects>" + objects + "</Objects></Scene>")
    return str(tmp_path / "s.xml")


def test_checkerboard_network_becomes_a_texture(tmp_path):
    mats = ('<ShaderGroupBegin name="c"/><Shader name="checkerboard" layer="l0">'
            '<Parameter scale_s="float 20"/><Parameter Ca="float3 0.1 0.1 0.1"/></Shader>'
            '<Shader name="matte" layer="l1"><Parameter Cs="float3 0.6 0.6 0.6"/></Shader>'
            '<ConnectShaders srclayer="l0" srcparam="Cout" dstlayer="l1" dstparam="Cs"/><ShaderGroupEnd/>')
    p = _scene_dir(tmp_path, {"checkerboard": CHECKER_OSL,
                              "matte": "surface matte ( color Cs = 1 ) { Ci = 0.5 * Cs * diffuse(N); }"},
                   mats, '<Triangle verta="float3 0 0 0" vertb="float3 1 0 0" vertc="float3 0 1 0" shader_name="c"/>')
    L = X.load(p)
    t = L.desc.textures
    assert len(t) == 1 and t[0].kind == N.KZ_TEX_CHECKER and (t[0].scale_s, t[0].scale_t) == (20.0, 4.0)
    assert np.allclose(t[0].Ca, 0.1) and np.allclose(t[0].Cb, 0.0)
    lb = L.desc.materials[0]["lobes"][0]
    assert lb["closure_id"] == N.KZ_CLOSURE_DIFFUSE and np.allclose(lb["weight"], 0.5)
    assert lb["params"][N.KZ_LOBE_TEXTURE_PARAM] == 1


def test_image_texture_uvs_and_environment(tmp_path):
    rng = np.random.default_rng(3)
    img = rng.random((5, 7, 3)).astype(np.float32)
    film_io.write_pfm(str(tmp_path / "tex.pfm"), img)
    film_io.write_pfm(str(tmp_path / "sky.pfm"), img[::-1])
    (tmp_path / "m.obj").write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nv 1 1 0\nvt 0 0\nvt 1 0\nvt 0 1\nvt 1 1\nvt 0.5 0.5\n"
                                    "f 1/1 2/2 3/3\nf 2/5 4/4 3/3\n")
    shaders = {"tm": 'surface tm ( string filename = "tex.pfm" ) { color c = texture(filename, u, v); '
                     'Ci = c * diffuse(N) + 0.2 * kp_mirror(); }',
               "env": 'shader env ( string filename = "" ) { Ci = 2 * color(environment(filename, I)) * background(); }'}
    mats = '<ShaderGroupBegin name="t"/><Shader name="tm" layer="a"/><ShaderGroupEnd/>'
    env = '<EnvironmentBegin/><Shader name="env" layer="e"><Parameter filename="string sky.pfm"/></Shader><EnvironmentEnd/>'
    L = X.load(_scene_dir(tmp_path, shaders, mats, '<Mesh filename="string m.obj" shader_name="t"/>'
                          '<Quad center="float3 0 0 0" dir="float3 0 0 1" vertical_vec="float3 0 1 0" half_width="float 1"'
                          ' half_height="float 1" shader_name="t"/>', env))
    d = L.desc
    assert [t.kind for t in d.textures] == [N.KZ_TEX_IMAGE, N.KZ_TEX_IMAGE]
    assert np.array_equal(d.textures[0].image, img) and np.array_equal(d.textures[1].image, img[::-1])
    assert d.env == (2.0, 2.0, 2.0) and d.env_texture == 1
    m = d.materials[0]["lobes"]
    assert m[0]["params"][N.KZ_LOBE_TEXTURE_PARAM] == 1 and m[1]["params"][N.KZ_LOBE_TEXTURE_PARAM] == 0
    # the OBJ vertex 2 carries two uvs, so it is split: 5 (position, uv) pairs
    v, t = d.meshes[0][0], d.meshes[0][1]
    uv = d.uvs[0]
    assert len(v) == 5 and len(uv) == 5
    corner = {tuple(np.round(v[i], 3)) + tuple(np.round(uv[i], 3)) for i in t.reshape(-1)}
    assert (1.0, 0.0, 0.0, 0.5, 0.5) in corner and (1.0, 0.0, 0.0, 1.0, 0.0) in corner
    assert np.allclose(d.uvs[1], [[0, 0], [1, 0], [1, 1], [0, 1]])
    # an empty environment file name is black
    env0 = '<EnvironmentBegin/><Shader name="env" layer="e"><Parameter filename=""/></Shader><EnvironmentEnd/>'
    L0 = X.load(_scene_dir(tmp_path, shaders, mats, '<Mesh filename="string m.obj" shader_name="t"/>', env0))
    assert L0.desc.env == (0.0, 0.0, 0.0) and L0.desc.env_texture == -1


def test_sphere_uv_has_no_wrapped_triangles():
    v, f, uv = X.sphere_mesh(np.zeros(3), 1.0, level=3)
    span = uv[f][:, :, 0].max(1) - uv[f][:, :, 0].min(1)
    assert span.max() < 0.5 and len(v) == 3 * len(f)
    assert uv[:, 1].min() >= 0.5 and uv[:, 1].max() <= 1.5


def test_textured_fixture():
    L = X.load(os.path.join(os.path.dirname(FIXTURE), "..", "textured_room", "scene.xml"))
    d = L.desc
    assert [t.kind for t in d.textures] == [N.KZ_TEX_CHECKER, N.KZ_TEX_IMAGE, N.KZ_TEX_IMAGE]
    assert d.env_texture == 2 and d.env == (1.0, 1.0, 1.0)
    assert d.textures[1].image.shape == (24, 32, 3) and d.textures[2].image.shape == (8, 16, 3)
    ids = [(int(l["closure_id"]), int(l["params"][N.KZ_LOBE_TEXTURE_PARAM]))
           for m in d.materials for l in m["lobes"][:m["n_lobes"]]]
    # the painted group's lobes reference paint.png (texture 1 of the scene);
    # the environment map (sky.pfm) joins the table after the materials'
    assert ids == [(N.KZ_CLOSURE_DIFFUSE, 1), (N.KZ_CLOSURE_KP_PRINCIPLE_DIFFUSE, 2),
                   (N.KZ_CLOSURE_KP_PRINCIPLE_CLEARCOAT, 0)]
    assert sorted(d.uvs) == [0, 1, 2, 3]


def test_obj_normals_split_and_transform(tmp_path):
    (tmp_path / "n.obj").write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nv 1 1 0\nvn 0 0 1\nvn 0 0.6 0.8\n"
                                    "f 1//1 2//1 3//1\nf 2//2 4//2 3//1\n")
    v, t, uv, n = X.load_obj_attributes(str(tmp_path / "n.obj"))
    assert uv is None and len(v) == 5 and n.shape == (5, 3)  # vertex 2 carries two normals
    corners = {tuple(np.round(np.concatenate([v[i], n[i]]).astype(np.float64), 3)) for i in t.reshape(-1)}
    assert (1.0, 0.0, 0.0, 0.0, 0.6, 0.8) in corners and (1.0, 0.0, 0.0, 0.0, 0.0, 1.0) in corners
    # a mirroring, non-uniform scale: normals follow the inverse transpose
    M = X.mesh_transform(scale=np.array([-1.0, 2.0, 1.0]))
    nn = X.apply_normal_transform(M, np.array([[0.0, 0.6, 0.8]]))
    want = np.array([0.0, 0.3, 0.8]) / np.linalg.norm([0.0, 0.3, 0.8])
    assert np.allclose(nn[0], want, atol=1e-6)


def test_sphere_objects_carry_normals(tmp_path):
    mats = '<ShaderGroupBegin name="m"/><Shader name="matte" layer="a"/><ShaderGroupEnd/>'
    p = _scene_dir(tmp_path, {"matte": "surface matte ( color Cs = 1 ) { Ci = Cs * diffuse(N); }"}, mats,
                   '<Sphere center_n_radius="float4 1 2 3 0.5" shader_name="m"/>')
    d = X.load(p).desc
    v, n = d.meshes[0][0], d.normals[0]
    assert np.allclose(np.linalg.norm(n, axis=1), 1, atol=1e-6)
    assert np.allclose((v - [1, 2, 3]) / 0.5, n, atol=1e-5)
