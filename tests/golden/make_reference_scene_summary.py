"""Loads the reference's own scene files with kazen_proto_gb300.scene_xml
and records what came out (film, meshes, triangles, lights, the closures
each shader group lowered to, the loader's warnings) in
tests/golden/reference_scenes_summary.json. It reads the scenes where the
reference checkout lies; nothing else reads them.

Run: python tests/golden/make_reference_scene_summary.py [reference root]
     (root: first argument or KAZEN_PROTO_ROOT)
"""
import glob
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from kazen_proto_gb300 import _native as N  # noqa: E402
from kazen_proto_gb300 import scene_xml as X  # noqa: E402

CLOSURES = {v: k[len("KZ_CLOSURE_"):] for k, v in vars(N).items() if k.startswith("KZ_CLOSURE_")}


def reference_root():
    """The kazen_proto checkout to read: the first command-line argument, else
    the KAZEN_PROTO_ROOT environment variable."""
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("KAZEN_PROTO_ROOT")
    if not root:
        sys.exit("usage: %s <kazen_proto checkout>  (or set KAZEN_PROTO_ROOT)" % os.path.basename(sys.argv[0]))
    return root


def main():
    root = reference_root()
    scenes = sorted(glob.glob(os.path.join(root, "resource", "scene", "*", "*.xml")))
    out = {}
    for path in scenes:
        rel = os.path.relpath(path, root)
        try:
            L = X.load(path)
        except Exception as e:  # recorded, not hidden
            msg = str(e).replace(os.path.join(root, ""), "")  # paths relative to the reference root
            out[rel] = {"loaded": False, "error": f"{type(e).__name__}: {msg}"}
            continue
        d = L.desc
        mats = {}
        for name, m in zip(L.material_names, d.materials):
            mats[name] = {"Le": [round(float(x), 6) for x in m["Le"]],
                          "lobes": [CLOSURES.get(int(l["closure_id"]), int(l["closure_id"]))
                                    + (f"@texture{int(l['params'][N.KZ_LOBE_TEXTURE_PARAM]) - 1}"
                                       if l["params"][N.KZ_LOBE_TEXTURE_PARAM] else "")
                                    for l in m["lobes"][:int(m["n_lobes"])]]}
        out[rel] = {"loaded": True, "film": [d.width, d.height], "mirror_x": L.mirror_x,
                    "integrator": L.integrator, "meshes": len(d.meshes), "triangles": int(d.n_triangles()),
                    "lights": int(sum(1 for m in d.meshes if m[3])), "materials": mats, "warnings": L.warnings,
                    "textures": [("checker" if t.kind == N.KZ_TEX_CHECKER else "image %dx%d" % t.image.shape[1::-1])
                                 for t in d.textures],
                    "environment": {"rgb": [round(float(x), 6) for x in d.env], "texture": d.env_texture},
                    "meshes_with_uv": len(d.uvs), "meshes_with_normals": len(d.normals),
                    "point_lights": len(d.point_lights)}
    dst = os.path.join(HERE, "reference_scenes_summary.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print("wrote", dst, "-", sum(v["loaded"] for v in out.values()), "of", len(out), "scenes loaded")


if __name__ == "__main__":
    main()
