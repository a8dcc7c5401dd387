"""Writes the scene fixtures under tests/golden/scenes/: small scenes in
kazen_proto's XML scene format with OBJ meshes and OSL surface shaders,
written here from scratch (the reference's own scene files are not copied).
They exercise what kazen_proto_gb300.scene_xml reads: Film, Camera with a
mirroring scale, shader groups with parameters, Mesh with translate / rotate
/ scale, Triangle and Quad elements, an area light, and the lowering of
diffuse, mirror, dielectric, microfacet mixture and emitter shaders
(box_room); a shader network, image textures, OBJ texture coordinates, a
Sphere and an environment map (textured_room).

Run: python tests/golden/make_scene_fixtures.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from kazen_proto_gb300 import film_io  # noqa: E402
from kazen_proto_gb300.scenes import icosphere  # noqa: E402

OUT = os.path.join(HERE, "scenes", "box_room")

SHADERS = {
    "matte": '''surface matte
(
    color Cs = 0.5
)
{
    Ci = Cs * diffuse(N);
}
''',
    "glossy": '''surface glossy
(
    color Cs = 0.7,
    float alpha = 0.3,
    float eta = 1.5
)
{
    // a diffuse base under a Beckmann coat
    Ci = 0.5 * Cs * diffuse(N) + 0.1 * Cs * microfacet("beckmann", N, alpha, eta, 0);
}
''',
    "chrome": '''surface chrome
(
    color Cs = 1
)
{
    Ci = Cs * kp_mirror();
}
''',
    "glass": '''surface glass
(
    color Cs = 1
)
{
    Ci = Cs * kp_dielectric(1.5, 1.0);
}
''',
    "lamp": '''surface lamp
(
    color Cs = 1
)
{
    Ci = Cs * kp_emitter(0.5);
}
''',
}

SCENE = '''<Scene>
    <Film width="int 64" height="int 48"/>
    <Camera position="float3 0.5 0.5 2.4" lookat="float3 0.5 0.45 0.5" up="float3 0 1 0" fov="float 40" scale="float3 -1 1 1"/>
    <Materials>
        <ShaderGroupBegin name="white"/>
            <Shader name="matte" layer="l0">
                <Parameter Cs="float3 0.72 0.71 0.68"/>
            </Shader>
        <ShaderGroupEnd/>
        <ShaderGroupBegin name="red"/>
            <Shader name="matte" layer="l1">
                <Parameter Cs="float3 0.63 0.065 0.05"/>
            </Shader>
        <ShaderGroupEnd/>
        <ShaderGroupBegin name="green"/>
            <Shader name="matte" layer="l2">
                <Parameter Cs="float3 0.14 0.45 0.09"/>
            </Shader>
        <ShaderGroupEnd/>
        <ShaderGroupBegin name="coated"/>
            <Shader name="glossy" layer="l3">
                <Parameter Cs="float3 0.8 0.6 0.3"/>
                <Parameter alpha="float 0.25"/>
            </Shader>
        <ShaderGroupEnd/>
        <ShaderGroupBegin name="mirror"/>
            <Shader name="chrome" layer="l4"/>
        <ShaderGroupEnd/>
        <ShaderGroupBegin name="glass"/>
            <Shader name="glass" layer="l5"/>
        <ShaderGroupEnd/>
        <ShaderGroupBegin name="light"/>
            <Shader name="lamp" layer="l6">
                <Parameter Cs="float3 17 12 4"/>
            </Shader>
        <ShaderGroupEnd/>
    </Materials>
    <Objects>
        <Mesh filename="string meshes/room.obj" shader_name="white"/>
        <Mesh filename="string meshes/wall.obj" shader_name="red"/>
        <Mesh filename="string meshes/wall.obj" shader_name="green" translate="func_translate 1 0 1" rotate="float4 0 1 0 180"/>
        <Mesh filename="string meshes/cube.obj" shader_name="mirror" translate="func_translate 0.32 0 0.45" rotate="float4 0 1 0 25" scale="func_scale 0.15 0.3 0.15"/>
        <Mesh filename="string meshes/ball.obj" shader_name="coated" translate="func_translate 0.68 0.14 0.55" scale="func_scale 0.14 0.14 0.14"/>
        <Triangle verta="float3 0.15 0.001 0.9" vertb="float3 0.35 0.001 0.9" vertc="float3 0.25 0.001 0.7" shader_name="string glass"/>
        <Quad center="float3 0.5 0.999 0.5" dir="float3 0 -1 0" vertical_vec="float3 0 0 1" half_width="float 0.12" half_height="float 0.12" shader_name="string light" is_light="bool true"/>
    </Objects>
    <EmbreeAccelerator/>
    <PathIntegrator/>
</Scene>
'''


TEX_SHADERS = {
    "checkerboard": """shader checkerboard (
    float s = u, float t = v, float scale_s = 4, float scale_t = 4,
    color Ca = color(1, 1, 1), color Cb = color(0, 0, 0),
    output color Cout = 0)
{
    // alternate Ca and Cb over the (s, t) grid
    float cs = fmod(s * scale_s, 2);
    float ct = fmod(t * scale_t, 2);
    if ((int(cs) ^ int(ct)) == 0) Cout = Ca; else Cout = Cb;
}
""",
    "matte": """surface matte ( color Cs = 0.5 )
{
    Ci = Cs * diffuse(N);
}
""",
    "painted": """surface painted ( string filename = "paint.png", float gloss = 0.2 )
{
    color c = texture(filename, u, v);
    Ci = 0.8 * c * kp_principle_diffuse(N) + gloss * kp_principle_clearcoat(N, 0.1);
}
""",
    "lamp": SHADERS["lamp"],
    "env": """shader env ( string filename = "" )
{
    Ci = color(environment(filename, I)) * background();
}
""",
}

TEX_SCENE = '''<Scene>
    <Film width="int 64" height="int 48"/>
    <Camera position="float3 0.5 0.45 2.2" lookat="float3 0.5 0.3 0.5" up="float3 0 1 0" fov="float 45"/>
    <EnvironmentBegin/>
        <Shader name="env" layer="e0">
            <Parameter filename="string sky.pfm"/>
        </Shader>
    <EnvironmentEnd/>
    <Materials>
        <ShaderGroupBegin name="checker_floor"/>
            <Shader name="checkerboard" layer="l0">
                <Parameter scale_s="float 8"/>
                <Parameter scale_t="float 8"/>
                <Parameter Ca="float3 0.8 0.8 0.75"/>
                <Parameter Cb="float3 0.15 0.15 0.2"/>
            </Shader>
            <Shader name="matte" layer="l1"/>
            <ConnectShaders srclayer="l0" srcparam="Cout" dstlayer="l1" dstparam="Cs"/>
        <ShaderGroupEnd/>
        <ShaderGroupBegin name="painted"/>
            <Shader name="painted" layer="l2"/>
        <ShaderGroupEnd/>
        <ShaderGroupBegin name="light"/>
            <Shader name="lamp" layer="l3">
                <Parameter Cs="float3 6 5 4"/>
            </Shader>
        <ShaderGroupEnd/>
    </Materials>
    <Objects>
        <Quad center="float3 0.5 0 0.5" dir="float3 0 1 0" vertical_vec="float3 0 0 1" half_width="float 0.8" half_height="float 0.8" shader_name="string checker_floor"/>
        <Sphere center_n_radius="float4 0.5 0.25 0.5 0.25" shader_name="string painted"/>
        <Mesh filename="string meshes/panel.obj" shader_name="painted" translate="func_translate 0.1 0 0.2"/>
        <Quad center="float3 0.5 1.2 0.5" dir="float3 0 -1 0" vertical_vec="float3 0 0 1" half_width="float 0.2" half_height="float 0.2" shader_name="string light" is_light="bool true"/>
    </Objects>
    <PathIntegrator/>
</Scene>
'''


def write_obj(path, verts, faces, comment):
    with open(path, "w") as f:
        f.write(f"# {comment}\n")
        for v in verts:
            f.write("v %.6f %.6f %.6f\n" % tuple(v))
        for fc in faces:
            f.write("f " + " ".join(str(i) for i in fc) + "\n")


def main():
    os.makedirs(os.path.join(OUT, "meshes"), exist_ok=True)
    for name, src in SHADERS.items():
        with open(os.path.join(OUT, name + ".osl"), "w") as f:
            f.write(src)
    with open(os.path.join(OUT, "scene.xml"), "w") as f:
        f.write(SCENE)
    # floor, ceiling and back wall of the unit room (quads, 1-based, inward)
    write_obj(os.path.join(OUT, "meshes", "room.obj"),
              [(0, 0, 0), (1, 0, 0), (1, 0, 1), (0, 0, 1), (0, 1, 0), (1, 1, 0), (1, 1, 1), (0, 1, 1)],
              [(1, 4, 3, 2), (5, 6, 7, 8), (1, 2, 6, 5)], "floor, ceiling, back wall")
    # the x = 0 wall facing +x, given with negative (relative) indices
    write_obj(os.path.join(OUT, "meshes", "wall.obj"),
              [(0, 0, 0), (0, 1, 0), (0, 1, 1), (0, 0, 1)], [(-4, -3, -2, -1)], "side wall")
    cube_v = [(x, y, z) for x in (-1, 1) for y in (0, 1) for z in (-1, 1)]
    idx = {v: i + 1 for i, v in enumerate(cube_v)}
    cube_f = [(idx[(-1, 0, -1)], idx[(1, 0, -1)], idx[(1, 0, 1)], idx[(-1, 0, 1)]),
              (idx[(-1, 1, -1)], idx[(-1, 1, 1)], idx[(1, 1, 1)], idx[(1, 1, -1)]),
              (idx[(-1, 0, -1)], idx[(-1, 1, -1)], idx[(1, 1, -1)], idx[(1, 0, -1)]),
              (idx[(-1, 0, 1)], idx[(1, 0, 1)], idx[(1, 1, 1)], idx[(-1, 1, 1)]),
              (idx[(-1, 0, -1)], idx[(-1, 0, 1)], idx[(-1, 1, 1)], idx[(-1, 1, -1)]),
              (idx[(1, 0, -1)], idx[(1, 1, -1)], idx[(1, 1, 1)], idx[(1, 0, 1)])]
    write_obj(os.path.join(OUT, "meshes", "cube.obj"), cube_v, cube_f, "unit cube, base at y = 0")
    sv, sf = icosphere(2)
    write_obj(os.path.join(OUT, "meshes", "ball.obj"), sv, (np.asarray(sf) + 1).tolist(), "icosphere, 320 faces")
    print("wrote", OUT)
    write_textured_room()


def write_textured_room():
    """A textured room: a checkerboard shader network on the floor, an image
    texture on a sphere and on an OBJ panel with its own texture coordinates,
    and an environment map seen where the room is open."""
    out = os.path.join(HERE, "scenes", "textured_room")
    os.makedirs(os.path.join(out, "meshes"), exist_ok=True)
    for name, src in TEX_SHADERS.items():
        with open(os.path.join(out, name + ".osl"), "w") as f:
            f.write(src)
    with open(os.path.join(out, "scene.xml"), "w") as f:
        f.write(TEX_SCENE)
    # paint.png: 32 x 24 stripes and a gradient; sky.pfm: 16 x 8 sky with a bright band
    y, x = np.mgrid[0:24, 0:32]
    paint = np.stack([(x % 8 < 4) * 0.8 + 0.1, y / 23.0, 0.5 + 0.4 * np.sin(x / 5.0)], -1)
    film_io.write_png(os.path.join(out, "paint.png"), paint)
    sy, sx = np.mgrid[0:8, 0:16]
    sky = np.stack([0.3 + 0.1 * sx / 15, 0.4 + 0.05 * sy, 1.2 - 0.1 * sy], -1) * (1 + 4 * (sy == 2))[:, :, None]
    film_io.write_pfm(os.path.join(out, "sky.pfm"), sky.astype(np.float32))
    with open(os.path.join(out, "meshes", "panel.obj"), "w") as f:
        f.write("# upright panel with texture coordinates (vertex 2 carries two)\n")
        for v in [(0, 0, 0), (0.3, 0, 0), (0.3, 0.5, 0), (0, 0.5, 0)]:
            f.write("v %g %g %g\n" % v)
        for t in [(0, 0), (2, 0), (2, 3), (0, 3), (1, 1)]:
            f.write("vt %g %g\n" % t)
        f.write("f 1/1 2/2 3/3\nf 1/1 3/5 4/4\n")
    print("wrote", out)


if __name__ == "__main__":
    main()
