"""Writes the scene fixtures under tests/golden/scenes/: small scenes in
kazen_proto's XML scene format with OBJ meshes and OSL surface shaders,
written here from scratch (the reference's own scene files are not copied).
They exercise what kazen_proto_gb300.scene_xml reads: Film, Camera with a
mirroring scale, shader groups with parameters, Mesh with translate / rotate
/ scale, Triangle and Quad elements, an area light, and the lowering of
diffuse, mirror, dielectric, microfacet mixture and emitter shaders.

Run: python tests/golden/make_scene_fixtures.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

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


if __name__ == "__main__":
    main()
