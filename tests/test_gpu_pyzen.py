"""The pyzen-compatible layer on the GPU: Renderer(spp, nthreads, callback)
renders a scene built through the pyzen calls, calls on_tile_end once per
tile in tile order, and the tiles hold the image the C-ABI render of the
same description gives (up to the order of FP32 film atomics); a scene file renders through the same call
and the film writes to disk."""
import os

import numpy as np
import pytest

from kazen_proto_gb300 import api, pyzen

from test_pyzen_and_film_io import FIXTURE_DIR, build_scene

pytestmark = pytest.mark.gpu


class Recorder(pyzen.api.RenderCallback):
    def __init__(self):
        self.seen = []

    def on_tile_end(self, film, tile_id):
        t = film.tiles[tile_id]
        self.seen.append((tile_id, t.x, t.y, len(t.get_data())))


def test_tiled_render_matches_direct_render(gpu):
    s = build_scene()
    cb = Recorder()
    r = pyzen.api.Renderer(8, 0, cb, max_depth=6, seed=5)
    assert r.render(s, "ignored.png")
    assert [x[0] for x in cb.seen] == list(range(s.film.get_tile_count()))
    assert all(n == t.width * t.height * 3 for (_, _, _, n), t in zip(cb.seen, s.film.tiles))
    direct = api.Renderer(spp=8, max_depth=6, seed=5).render(s._built, s.desc.camera, 64, 48)
    # the same paths; only the order of the film's FP32 atomic additions differs
    img = s.film.image().astype(np.float64)
    assert float(np.mean((img - direct) ** 2 / (direct.astype(np.float64) ** 2 + 1e-2))) < 1e-10
    assert direct.mean() > 1e-3
    assert s.film.filename == "ignored.png"


def test_scene_file_render_and_write(gpu, tmp_path):
    r = pyzen.api.Renderer(4, 0, None)
    s = pyzen.api.Scene()
    s.parse_from_file(os.path.join(FIXTURE_DIR, "scene.xml"))
    assert r.render(s, str(tmp_path / "frame.exr"))
    assert s.film.write_tiles() and (tmp_path / "frame.exr").stat().st_size > 64 * 48 * 12
    assert r.render(os.path.join(FIXTURE_DIR, "scene.xml"))  # a path renders too
