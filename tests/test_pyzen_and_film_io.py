"""CPU tests of the pyzen-compatible layer (kazen_proto_gb300.pyzen) and
the film writers (kazen_proto_gb300.film_io): film tiling covers every
pixel once, the scene-building calls produce the expected description,
unsupported features raise, and the written PNG / PPM / PFM / EXR files
decode to the image."""
import os
import struct
import zlib

import numpy as np
import pytest

from kazen_proto_gb300 import _native as N
from kazen_proto_gb300 import film_io, pyzen

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE_DIR = os.path.join(HERE, "golden", "scenes", "box_room")


@pytest.mark.parametrize("w,h,xr,yr", [(800, 600, 7, 7), (64, 48, 1, 1), (33, 17, 4, 3), (5, 5, 5, 5)])
def test_film_tiles_cover_each_pixel_once(w, h, xr, yr):
    f = pyzen.concepts.Film(w, h, xr, yr, "x.png")
    f.generate_tiles()
    assert f.get_tile_count() == xr * yr
    cover = np.zeros((h, w), np.int32)
    for t in f.tiles:
        cover[t.y:t.y + t.height, t.x:t.x + t.width] += 1
        assert len(t.get_data()) == t.width * t.height * 3
    assert (cover == 1).all()


def test_film_colors_and_image():
    f = pyzen.concepts.Film(6, 4, 2, 2, "x.png")
    f.generate_tiles()
    f.set_film_color((0.1, 0.2, 0.3))
    f.set_tile_color((1, 0, 0), 1, 0)
    f.tiles[2].set_pixel_color(0, 1, (0, 0, 5))
    img = f.image()
    assert np.allclose(img[0, 0], [0.1, 0.2, 0.3]) and np.allclose(img[0, 3], [1, 0, 0])
    assert np.allclose(img[3, 0], [0, 0, 5])
    assert f.tiles[1].get_data()[:3] == [1.0, 0.0, 0.0]


def build_scene():
    s = pyzen.api.Scene()
    s.set_film(64, 48, 2, 2, "out.png")
    s.set_camera((0.5, 0.5, 2.4), (0.5, 0.45, 0.5), (0, 1, 0), 0.01, 100.0, 40.0)
    s.set_shader_search_path(FIXTURE_DIR)
    for name, shader, params in (("white", "matte", {"Cs": (0.72, 0.71, 0.68)}),
                                 ("coated", "glossy", {"Cs": (0.8, 0.6, 0.3), "alpha": 0.25}),
                                 ("light", "lamp", {"Cs": (17, 12, 4)})):
        s.begin_shader_group(name)
        assert s.load_oso_shader("surface", shader, "layer_" + name, "/nonexistent")
        for k, v in params.items():
            (s.set_shader_param_vec3f if isinstance(v, tuple) else s.set_shader_param_float)(k, v)
        s.end_shader_group()
    floor = [(0, 0, 0), (1, 0, 0), (1, 0, 1), (0, 0, 1)]
    s.add_mesh(None, floor, [], [], [(0, 3, 2), (0, 2, 1)], "floor", "white")
    world = np.eye(4)
    world[:3, 3] = (0, 1, 0)  # the ceiling: the floor moved up and turned over
    s.add_mesh(world, floor, [], [], [(0, 1, 2), (0, 2, 3)], "ceiling", "white")
    s.add_triangle(None, (0, 0, 0), (1, 0, 0), (0, 1, 0), "back", "white")
    s.add_quad(None, (0.5, 0.999, 0.5), (0, -1, 0), (0, 0, 1), 0.12, 0.12, "lamp", "light", True)
    s.add_sphere(None, (0.6, 0.15, 0.5), 0.15, "ball", "coated")
    return s


def test_scene_building_calls():
    s = build_scene()
    d = s.desc
    assert (d.width, d.height) == (64, 48) and d.camera.flip and d.camera.fov == 40.0
    assert len(d.materials) == 3 and [m[2] for m in d.meshes] == [0, 0, 0, 2, 1]
    assert d.meshes[3][3] is True and d.materials[2]["n_lobes"] == 0 and np.allclose(d.materials[2]["Le"], [17, 12, 4])
    assert [int(l["closure_id"]) for l in d.materials[1]["lobes"][:2]] == [N.KZ_CLOSURE_DIFFUSE, N.KZ_CLOSURE_KP_GLOSS]
    assert np.allclose(d.meshes[1][0][:, 1], 1.0)  # world matrix applied
    assert any("tessellated" in w for w in s.warnings)
    s.set_integrator(pyzen.api.IntegratorType.WhittedIntegrator)
    assert any("WhittedIntegrator" in w for w in s.warnings)


def test_unsupported_calls_raise():
    s = pyzen.api.Scene()
    with pytest.raises(RuntimeError):
        s.load_oso_shader("surface", "matte", "l", FIXTURE_DIR)  # outside a group
    s.begin_shader_group("g")
    with pytest.raises(FileNotFoundError):
        s.load_oso_shader("surface", "no_such_shader", "l", FIXTURE_DIR)
    s.load_oso_shader("surface", "matte", "l", FIXTURE_DIR)
    s.connect_shader("z", "Cout", "l", "Cs")  # from a layer that does not exist
    with pytest.raises(ValueError):
        s.end_shader_group()
    s.add_point_light((1, 2, 3), (0, 5, 0), "g")
    assert s.desc.point_lights == [((0.0, 5.0, 0.0), (1.0, 2.0, 3.0))]
    with pytest.raises(KeyError):
        s.add_mesh(None, [(0, 0, 0), (1, 0, 0), (0, 1, 0)], [], [], [(0, 1, 2)], "m", "unknown")


def test_parse_from_file_defers_the_build():
    s = pyzen.api.Scene()
    s.parse_from_file(os.path.join(FIXTURE_DIR, "scene.xml"))
    assert (s.film.width, s.film.height) == (64, 48) and s.film.get_tile_count() == 1
    assert len(s.desc.meshes) == 7 and s._built is None


def test_image_writers(tmp_path):
    rng = np.random.default_rng(3)
    img = rng.random((5, 7, 3)).astype(np.float32) * 1.2
    img[0, 0] = (-1.0, 0.5, 3.0)
    q = np.round(np.clip(img, 0, 1) * 255).astype(np.uint8)

    p = tmp_path / "a.png"
    film_io.write_image(str(p), img)
    data = p.read_bytes()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    w, h = struct.unpack(">II", data[16:24])
    assert (w, h) == (7, 5)
    idat = data.index(b"IDAT")
    n = struct.unpack(">I", data[idat - 4:idat])[0]
    raw = zlib.decompress(data[idat + 4:idat + 4 + n])
    rows = np.frombuffer(raw, np.uint8).reshape(5, 1 + 21)
    assert (rows[:, 0] == 0).all() and np.array_equal(rows[:, 1:].reshape(5, 7, 3), q)

    p = tmp_path / "a.ppm"
    film_io.write_image(str(p), img)
    d = p.read_bytes()
    assert d.startswith(b"P6\n7 5\n255\n") and np.array_equal(np.frombuffer(d[11:], np.uint8).reshape(5, 7, 3), q)

    p = tmp_path / "a.pfm"
    film_io.write_image(str(p), img)
    d = p.read_bytes()
    assert d.startswith(b"PF\n7 5\n-1.0\n")
    back = np.frombuffer(d[len(b"PF\n7 5\n-1.0\n"):], "<f4").reshape(5, 7, 3)[::-1]
    assert np.array_equal(back, img)

    p = tmp_path / "a.exr"
    film_io.write_image(str(p), img)
    d = p.read_bytes()
    assert struct.unpack("<ii", d[:8]) == (20000630, 2)
    hdr_end = d.index(b"screenWindowWidth\0float\0") + len(b"screenWindowWidth\0float\0") + 4 + 4 + 1
    offsets = struct.unpack("<5Q", d[hdr_end:hdr_end + 40])
    for y, off in enumerate(offsets):
        yy, size = struct.unpack("<ii", d[off:off + 8])
        assert yy == y and size == 7 * 3 * 4
        planes = np.frombuffer(d[off + 8:off + 8 + size], "<f4").reshape(3, 7)  # B, G, R
        assert np.array_equal(planes[::-1].T, img[y])

    with pytest.raises(ValueError):
        film_io.write_image(str(tmp_path / "a.jpg"), img)


def test_shader_network_and_uvs(tmp_path):
    """A checkerboard layer connected into a matte layer (parameters before
    their shader, as OSL orders them), texcoords on add_mesh, the sphere's
    parametric uv."""
    (tmp_path / "checkerboard.osl").write_text(
        "shader checkerboard ( float s = u, float t = v, float scale_s = 4, float scale_t = 4,"
        " color Ca = 1, color Cb = 0, output color Cout = 0 ) { Cout = Ca; }")
    (tmp_path / "matte.osl").write_text("surface matte ( color Cs = 1 ) { Ci = Cs * diffuse(N); }")
    s = pyzen.api.Scene()
    s.set_shader_search_path(str(tmp_path))
    s.begin_shader_group("checker")
    s.set_shader_param_float("scale_s", 10.0)
    assert s.load_oso_shader("shader", "checkerboard", "tex", "")
    assert s.load_oso_shader("surface", "matte", "m", "")
    s.connect_shader("tex", "Cout", "m", "Cs")
    s.end_shader_group()
    d = s.desc
    assert len(d.textures) == 1 and d.textures[0].kind == N.KZ_TEX_CHECKER and d.textures[0].scale_s == 10.0
    assert d.materials[0]["lobes"][0]["params"][N.KZ_LOBE_TEXTURE_PARAM] == 1
    s.add_mesh(None, [(0, 0, 0), (1, 0, 0), (0, 1, 0)], [], [(0, 0), (2, 0), (0, 2)], [(0, 1, 2)], "t", "checker")
    s.add_sphere(None, (0, 0, 0), 1.0, "ball", "checker")
    assert np.allclose(d.uvs[0], [[0, 0], [2, 0], [0, 2]]) and len(d.uvs[1]) == len(d.meshes[1][0])
