"""Seeded synthetic workloads of the kazen hot path (numpy, float32).

* box_scene ......... closed unit box (5 inward quads), a tall Lambert box, a
                      GGX-conductor box and a 0.25 x 0.25 ceiling emitter;
                      256 x 256, pinhole fov 40 deg, 16 spp, max depth 5.
* triangle_soup ..... 1,048,576 triangles, centroids U[0,1]^3, vertices
                      centroid + U(-0.01, 0.01)^3.
* soup_rays ......... incoherent rays: origins uniform on the sphere of
                      radius 2, directions toward U[0,1]^3 points.
* terrain_scene ..... 1024 x 1024-cell fBm heightfield (2,097,152 triangles,
                      amplitude 0.1) + 64 icospheres (subdivision 3, 1,280
                      triangles each: an icosphere has 20*4^s faces, so 2,560
                      is not reachable), 4 quad lights; 1920 x 1080, 64 spp,
                      max depth 8.

None of these exist in the reference (it ships no benchmark scenes); the
reference renders Cornell-box variants from XML (resource/scene/cbox/*.xml).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import api


@dataclass
class SceneDesc:
    meshes: list = field(default_factory=list)   # (verts (n,3) f32, idx (m,3) u32, material_id, is_light)
    materials: list = field(default_factory=list)
    camera: api.Camera = None
    width: int = 256
    height: int = 256
    spp: int = 16
    max_depth: int = 5
    textures: list = field(default_factory=list)   # api.Texture
    uvs: dict = field(default_factory=dict)         # mesh index -> (nverts, 2) f32
    env: tuple = (0.0, 0.0, 0.0)
    env_texture: int = -1
    point_lights: list = field(default_factory=list)   # (position, radiance)
    normals: dict = field(default_factory=dict)        # mesh index -> (nverts, 3) f32 unit normals

    def add(self, verts, idx, material_id, is_light=False, uv=None, normals=None) -> int:
        self.meshes.append((np.asarray(verts, np.float32).reshape(-1, 3), np.asarray(idx, np.uint32).reshape(-1, 3),
                            int(material_id), bool(is_light)))
        g = len(self.meshes) - 1
        if uv is not None:
            self.uvs[g] = np.asarray(uv, np.float32).reshape(-1, 2)
        if normals is not None:
            n = np.asarray(normals, np.float64).reshape(-1, 3)
            self.normals[g] = (n / np.linalg.norm(n, axis=1, keepdims=True)).astype(np.float32)
        return g

    def material_array(self):
        arr = np.zeros(len(self.materials), dtype=api.N.MATERIAL_DTYPE)
        for i, m in enumerate(self.materials):
            arr[i] = m
        return arr

    def n_triangles(self):
        return sum(len(m[1]) for m in self.meshes)

    def build(self) -> api.Scene:
        s = api.Scene()
        for g, (v, i, mat, light) in enumerate(self.meshes):
            s.add_mesh(v, i, mat, light)
            if g in self.uvs:
                s.set_mesh_uvs(g, self.uvs[g])
            if g in self.normals:
                s.set_mesh_normals(g, self.normals[g])
        s.set_materials(self.material_array())
        for pos, rad in self.point_lights:
            s.add_point_light(pos, rad)
        if self.textures:
            s.set_textures(self.textures)
        if any(self.env) or self.env_texture >= 0:
            s.set_environment(self.env, self.env_texture)
        s.build_bvh()
        return s

    def tri_normals(self):
        """((N, 9) per-triangle vertex normals, (N,) has-normals flags) in global order, or None.
        The normals are renormalised in FP32 as the library does."""
        if not self.normals:
            return None
        nrm, has = [], []
        for g, (v, i, _, _) in enumerate(self.meshes):
            if g in self.normals:
                n = self.normals[g].astype(np.float32)
                ln = np.sqrt((n * n).sum(axis=1, dtype=np.float32), dtype=np.float32)
                n = (n / ln[:, None]).astype(np.float32)
                nrm.append(n[i].reshape(-1, 9))
                has.append(np.ones(len(i), np.uint8))
            else:
                nrm.append(np.zeros((len(i), 9), np.float32))
                has.append(np.zeros(len(i), np.uint8))
        return np.concatenate(nrm).astype(np.float32), np.concatenate(has)

    def tri_uvs(self):
        """(N, 6) per-triangle vertex uvs in global order (barycentric defaults), or None."""
        if not self.uvs:
            return None
        out = []
        for g, (v, i, _, _) in enumerate(self.meshes):
            if g in self.uvs:
                out.append(self.uvs[g][i].reshape(-1, 6))
            else:
                out.append(np.tile(np.array([0, 0, 1, 0, 0, 1], np.float32), (len(i), 1)))
        return np.concatenate(out).astype(np.float32)

    def flatten(self):
        """World-space triangle soup in global (mesh) order for the CPU restatement:
        (tri_verts (N,9) f32, tri_geom (N,) u32, geom_material (G,) i32, geom_is_light (G,) i32)."""
        tv, tg = [], []
        for g, (v, i, _, _) in enumerate(self.meshes):
            tv.append(v[i].reshape(-1, 9))
            tg.append(np.full(len(i), g, np.uint32))
        tv = np.concatenate(tv).astype(np.float32) if tv else np.zeros((0, 9), np.float32)
        tg = np.concatenate(tg) if tg else np.zeros(0, np.uint32)
        gm = np.array([m[2] for m in self.meshes], np.int32)
        gl = np.array([1 if m[3] else 0 for m in self.meshes], np.int32)
        return tv, tg, gm, gl


def quad(p0, e1, e2):
    """Two triangles with geometric normal normalize(cross(e1, e2))."""
    p0, e1, e2 = (np.asarray(x, np.float32) for x in (p0, e1, e2))
    v = np.stack([p0, p0 + e1, p0 + e1 + e2, p0 + e2]).astype(np.float32)
    return v, np.array([[0, 1, 2], [0, 2, 3]], np.uint32)


def box(lo, hi):
    """Axis-aligned box, 12 triangles, outward normals."""
    lo = np.asarray(lo, np.float32)
    hi = np.asarray(hi, np.float32)
    dx, dy, dz = hi - lo
    X, Y, Z = np.array([dx, 0, 0], np.float32), np.array([0, dy, 0], np.float32), np.array([0, 0, dz], np.float32)
    faces = [
        (lo, Z, Y),                               # -x
        (np.array([hi[0], lo[1], lo[2]]), Y, Z),  # +x
        (lo, X, Z),                               # -y
        (np.array([lo[0], hi[1], lo[2]]), Z, X),  # +y
        (lo, Y, X),                               # -z
        (np.array([lo[0], lo[1], hi[2]]), X, Y),  # +z
    ]
    vs, ids = [], []
    for k, (p0, a, b) in enumerate(faces):
        v, i = quad(p0, a, b)
        vs.append(v)
        ids.append(i + 4 * k)
    return np.concatenate(vs), np.concatenate(ids)


def box_scene(width=256, height=256, spp=16, max_depth=5) -> SceneDesc:
    """Small box scene (36 triangles): the reference CPU-path workload."""
    d = SceneDesc(width=width, height=height, spp=spp, max_depth=max_depth)
    red = api.material([api.diffuse((0.63, 0.065, 0.05))])
    green = api.material([api.diffuse((0.14, 0.45, 0.09))])
    white = api.material([api.diffuse((0.725, 0.71, 0.68))])
    metal = api.material([api.conductor_ggx((0.95, 0.64, 0.54), 0.2)])
    light = api.material([], Le=(17.0, 12.0, 4.0))
    d.materials = [red, green, white, metal, light]
    RED, GREEN, WHITE, METAL, LIGHT = range(5)
    walls = [
        ((0, 0, 0), (0, 0, 1), (1, 0, 0), WHITE),  # floor, +y
        ((0, 1, 0), (1, 0, 0), (0, 0, 1), WHITE),  # ceiling, -y
        ((0, 0, 1), (0, 1, 0), (1, 0, 0), WHITE),  # back, -z
        ((0, 0, 0), (0, 1, 0), (0, 0, 1), RED),    # left, +x
        ((1, 0, 0), (0, 0, 1), (0, 1, 0), GREEN),  # right, -x
    ]
    for p0, e1, e2, m in walls:
        v, i = quad(p0, e1, e2)
        d.add(v, i, m)
    v, i = box((0.15, 0.0, 0.5), (0.45, 0.6, 0.8))
    d.add(v, i, WHITE)
    v, i = box((0.55, 0.0, 0.2), (0.85, 0.3, 0.5))
    d.add(v, i, METAL)
    v, i = quad((0.375, 0.999, 0.375), (0.25, 0, 0), (0, 0, 0.25))  # faces -y
    d.add(v, i, LIGHT, is_light=True)
    d.camera = api.Camera(eye=(0.5, 0.5, -1.4), lookat=(0.5, 0.5, 0.5), up=(0, 1, 0), fov=40.0)
    return d


def triangle_soup(n_tris=1 << 20, seed=1) -> np.ndarray:
    """(n, 9) float32 triangle soup of the traversal microbenchmark."""
    rng = np.random.default_rng(seed)
    c = rng.random((n_tris, 1, 3), dtype=np.float32)
    off = rng.uniform(-0.01, 0.01, size=(n_tris, 3, 3)).astype(np.float32)
    return (c + off).astype(np.float32).reshape(n_tris, 9)


def soup_rays(n_rays=1 << 24, seed=2, chunk=1 << 22) -> np.ndarray:
    """Incoherent rays: origin 2*normalize(gaussian), direction toward U[0,1]^3."""
    rng = np.random.default_rng(seed)
    out = np.zeros(n_rays, dtype=api.N.RAY_DTYPE)
    for s in range(0, n_rays, chunk):
        m = min(chunk, n_rays - s)
        g = rng.standard_normal((m, 3), dtype=np.float32)
        g /= np.sqrt((g * g).sum(1, dtype=np.float32))[:, None]
        o = (np.float32(2.0) * g).astype(np.float32)
        tgt = rng.random((m, 3), dtype=np.float32)
        dv = (tgt - o).astype(np.float32)
        dn = (dv / np.sqrt((dv * dv).sum(1, dtype=np.float32))[:, None]).astype(np.float32)
        blk = out[s:s + m]
        blk["ox"], blk["oy"], blk["oz"] = o[:, 0], o[:, 1], o[:, 2]
        blk["dx"], blk["dy"], blk["dz"] = dn[:, 0], dn[:, 1], dn[:, 2]
    out["tmin"] = np.float32(1e-4)
    out["tmax"] = np.float32(np.inf)
    return out


def soup_desc(tris: np.ndarray) -> SceneDesc:
    d = SceneDesc()
    d.materials = [api.material([api.diffuse((0.5, 0.5, 0.5))])]
    n = len(tris)
    d.add(tris.reshape(-1, 3), np.arange(3 * n, dtype=np.uint32).reshape(n, 3), 0)
    return d


def icosphere(subdiv=3):
    t = (1.0 + 5 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
         (8, 6, 7), (9, 8, 1)]
    verts = [np.array(p, np.float64) / np.linalg.norm(p) for p in v]
    faces = list(f)
    for _ in range(subdiv):
        cache = {}

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    return np.array(verts, np.float32), np.array(faces, np.uint32)


def fbm_heightfield(n=1024, amplitude=0.1, octaves=6, seed=3):
    """(n+1)^2 heights: sum of bilinearly interpolated value-noise octaves."""
    rng = np.random.default_rng(seed)
    xs = np.linspace(0.0, 1.0, n + 1)
    h = np.zeros((n + 1, n + 1))
    amp, freq, norm = 1.0, 4, 0.0
    for _ in range(octaves):
        g = rng.random((freq + 2, freq + 2)) * 2.0 - 1.0
        p = xs * freq
        i0 = np.floor(p).astype(int)
        f = p - i0
        f = f * f * (3 - 2 * f)
        a = g[np.ix_(i0, i0)] * (1 - f)[:, None] * (1 - f)[None, :]
        a += g[np.ix_(i0 + 1, i0)] * f[:, None] * (1 - f)[None, :]
        a += g[np.ix_(i0, i0 + 1)] * (1 - f)[:, None] * f[None, :]
        a += g[np.ix_(i0 + 1, i0 + 1)] * f[:, None] * f[None, :]
        h += amp * a
        norm += amp
        amp *= 0.5
        freq *= 2
    return (amplitude * h / norm).astype(np.float32)


def terrain_scene(width=1920, height=1080, spp=64, max_depth=8, cells=1024, n_spheres=64, subdiv=3,
                  seed=7) -> SceneDesc:
    rng = np.random.default_rng(seed)
    d = SceneDesc(width=width, height=height, spp=spp, max_depth=max_depth)
    d.materials = [api.material([api.diffuse((0.5, 0.5, 0.5))])]  # terrain
    hgt = fbm_heightfield(cells, 0.1, seed=seed + 1)
    xs = np.linspace(0.0, 1.0, cells + 1, dtype=np.float32)
    X, Z = np.meshgrid(xs, xs, indexing="ij")
    verts = np.stack([X, hgt, Z], axis=-1).reshape(-1, 3).astype(np.float32)
    i = np.arange(cells)
    a = (i[:, None] * (cells + 1) + i[None, :]).reshape(-1)
    b = a + (cells + 1)
    c = a + 1
    e = b + 1
    # upward normals: cross(v1-v0, v2-v0) with v = (x, h, z) grid, x along i
    t0 = np.stack([a, c, b], -1)
    t1 = np.stack([b, c, e], -1)
    idx = np.concatenate([t0, t1]).astype(np.uint32)
    d.add(verts, idx, 0)
    sv, sf = icosphere(subdiv)
    for k in range(n_spheres):
        r = rng.uniform(0.02, 0.1)
        pos = np.array([rng.uniform(0.05, 0.95), rng.uniform(0.15, 0.4), rng.uniform(0.05, 0.95)], np.float32)
        kind = rng.integers(0, 3)
        if kind == 0:
            m = api.material([api.diffuse(tuple(rng.uniform(0.2, 0.8, 3)))])
        elif kind == 1:
            m = api.material([api.conductor_ggx(tuple(rng.uniform(0.5, 1.0, 3)), float(rng.uniform(0.05, 0.8)))])
        else:
            m = api.material([api.dielectric(1.5, 1.0)])
        d.materials.append(m)
        d.add((sv * np.float32(r) + pos).astype(np.float32), sf, len(d.materials) - 1)
    d.materials.append(api.material([], Le=(12.0, 12.0, 12.0)))
    L = len(d.materials) - 1
    for (x, z) in [(0.25, 0.25), (0.75, 0.25), (0.25, 0.75), (0.75, 0.75)]:
        v, q = quad((x - 0.1, 1.2, z - 0.1), (0.2, 0, 0), (0, 0, 0.2))  # faces -y
        d.add(v, q, L, is_light=True)
    d.camera = api.Camera(eye=(0.5, 0.9, -0.6), lookat=(0.5, 0.05, 0.55), up=(0, 1, 0), fov=60.0)
    return d


def slit_room_scene(width=1024, height=1024, spp=16, max_depth=10, n_spheres=32, seed=11, light_size=4.0,
                    light_dist=2.0) -> SceneDesc:
    """Narrow-aperture guiding scene: a closed unit room of 24 inward Lambert
    quads (five walls split 2 x 2, and the +x wall made of the 4 quads that
    frame a 0.05 x 0.5 slit), an exterior quad light of radiance 200 facing
    the slit (4 x 4, 2 units outside the wall: only a sliver of it is visible
    through the slit from inside), and 32 GGX-conductor icospheres (alpha
    U[0.1, 0.5])."""
    rng = np.random.default_rng(seed)
    d = SceneDesc(width=width, height=height, spp=spp, max_depth=max_depth)
    d.materials = [api.material([api.diffuse((0.7, 0.7, 0.7))])]
    WALL = 0

    def split(p0, e1, e2):
        p0, e1, e2 = (np.asarray(x, np.float32) for x in (p0, e1, e2))
        for a in range(2):
            for b in range(2):
                v, i = quad(p0 + e1 * (0.5 * a) + e2 * (0.5 * b), e1 * 0.5, e2 * 0.5)
                d.add(v, i, WALL)

    split((0, 0, 0), (0, 0, 1), (1, 0, 0))   # floor, +y
    split((0, 1, 0), (1, 0, 0), (0, 0, 1))   # ceiling, -y
    split((0, 0, 1), (0, 1, 0), (1, 0, 0))   # back, -z
    split((0, 0, 0), (1, 0, 0), (0, 1, 0))   # front, +z
    split((0, 0, 0), (0, 1, 0), (0, 0, 1))   # left, +x
    # right wall (x = 1, facing -x) with a vertical slit: z in [0.475, 0.525], y in [0.25, 0.75]
    z0, z1, y0, y1 = 0.475, 0.525, 0.25, 0.75
    for (za, zb, ya, yb) in [(0, 1, 0, y0), (0, 1, y1, 1), (0, z0, y0, y1), (z1, 1, y0, y1)]:
        v, i = quad((1, ya, za), (0, 0, zb - za), (0, yb - ya, 0))
        d.add(v, i, WALL)
    light = api.material([], Le=(200.0, 200.0, 200.0))
    d.materials.append(light)
    h = 0.5 * light_size  # centred on the slit, light_dist outside the wall, facing -x
    v, i = quad((1.0 + light_dist, 0.5 - h, 0.5 - h), (0, 0, light_size), (0, light_size, 0))
    d.add(v, i, len(d.materials) - 1, is_light=True)
    sv, sf = icosphere(2)
    for _ in range(n_spheres):
        r = rng.uniform(0.03, 0.07)
        pos = np.array([rng.uniform(0.1, 0.9), rng.uniform(0.05, 0.6), rng.uniform(0.1, 0.9)], np.float32)
        d.materials.append(api.material([api.conductor_ggx(tuple(rng.uniform(0.6, 0.95, 3)),
                                                            float(rng.uniform(0.1, 0.5)))]))
        d.add((sv * np.float32(r) + pos).astype(np.float32), sf, len(d.materials) - 1)
    d.camera = api.Camera(eye=(0.08, 0.55, 0.08), lookat=(0.75, 0.35, 0.8), up=(0, 1, 0), fov=75.0)
    return d


def soup_render_scene(n_tris, seed, albedo=0.6) -> SceneDesc:
    """A render job over the traversal workload's generator: an n_tris
    triangle soup in the unit cube (Lambert), a 1 x 1 quad light above it."""
    d = SceneDesc()
    d.materials = [api.material([api.diffuse((albedo, albedo, albedo))]), api.material([], Le=(6.0, 6.0, 6.0))]
    tv = triangle_soup(n_tris, seed)
    d.add(tv.reshape(-1, 3), np.arange(3 * n_tris, dtype=np.uint32).reshape(n_tris, 3), 0)
    v, i = quad((0.0, 1.6, 0.0), (1.0, 0, 0), (0, 0, 1.0))  # faces -y
    d.add(v, i, 1, is_light=True)
    d.camera = api.Camera(eye=(1.9, 1.3, -1.3), lookat=(0.5, 0.45, 0.5), up=(0, 1, 0), fov=45.0)
    return d


def batch_jobs(n_jobs=256, seed=5, tri_range=(50_000, 500_000), resolutions=(64, 128, 256, 512), spps=(4, 16, 64),
               depths=(4, 8)):
    """Uneven batch: seeded soup scenes with tri_range triangles, resolution,
    spp and max depth drawn uniformly from the given sets."""
    rng = np.random.default_rng(seed)
    jobs = []
    for k in range(n_jobs):
        n = int(rng.integers(tri_range[0], tri_range[1] + 1))
        r = int(rng.choice(resolutions))
        jobs.append({"desc_args": (n, int(rng.integers(1 << 30))), "width": r, "height": r,
                     "spp": int(rng.choice(spps)), "max_depth": int(rng.choice(depths)), "seed": 1000 + k})
    return jobs


def build_batch_scenes(jobs, workers=8):
    """Generate and build every job's scene (BVH builds run in parallel; the
    C ABI releases the GIL). Adds 'scene' and 'camera' to each job."""
    import concurrent.futures as cf

    def one(j):
        d = soup_render_scene(*j["desc_args"])
        return d.build(), d.camera

    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        for j, (sc, cam) in zip(jobs, ex.map(one, jobs)):
            j["scene"], j["camera"] = sc, cam
    return jobs
