"""Lowers the reference's own shader library (resource/shader/src/*.osl in
kazen_proto) with kazen_proto_gb300.osl_lower at the shaders' default
parameters and records the result -- lobes (closure id, weight, params),
Le, warnings, or the reason a shader is not lowered -- in
tests/golden/reference_shaders_lowered.json. It reads the shaders where the
reference checkout lies; nothing else reads them.

Run: python tests/golden/make_reference_shader_summary.py [reference root]
     (root: first argument or KAZEN_PROTO_ROOT)
"""
import glob
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from kazen_proto_gb300 import osl_lower  # noqa: E402


def reference_root():
    """The kazen_proto checkout to read: the first command-line argument, else
    the KAZEN_PROTO_ROOT environment variable."""
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("KAZEN_PROTO_ROOT")
    if not root:
        sys.exit("usage: %s <kazen_proto checkout>  (or set KAZEN_PROTO_ROOT)" % os.path.basename(sys.argv[0]))
    return root


def main():
    root = reference_root()
    out = {}
    for path in sorted(glob.glob(os.path.join(root, "resource", "shader", "src", "*.osl"))):
        rel = os.path.relpath(path, root)
        with open(path) as f:
            src = f.read()
        try:
            r = osl_lower.lower(src)
        except Exception as e:  # recorded, not hidden
            out[rel] = {"lowered": False, "error": f"{type(e).__name__}: {e}"}
            continue
        out[rel] = {"lowered": True, "Le": [round(float(x), 7) for x in r.Le], "warnings": r.warnings,
                    "lobes": [{"closure_id": int(l["closure_id"]),
                               "weight": [round(float(x), 7) for x in l["weight"]],
                               "params": [round(float(x), 7) for x in l["params"]]} for l in r.lobes]}
    dst = os.path.join(HERE, "reference_shaders_lowered.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print("wrote", dst, "-", sum(v["lowered"] for v in out.values()), "of", len(out), "shaders lowered")


if __name__ == "__main__":
    main()
