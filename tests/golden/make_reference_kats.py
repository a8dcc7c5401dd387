"""Regenerate tests/golden/reference_kats.json from the reference's own tests.

Reads, as text, the known-answer tests kazen_proto ships for this path:
  * tests/render_tests/microfacet_tests.cpp  (white-furnace integrals)
  * tests/libusage_tests/embree_tests.cpp   (single-triangle hit)
and records them with their file:line. The PCG32 vector is the published
output of the PCG reference implementation for pcg32_srandom(42, 54): pcg32
is a third-party header the reference includes (src/core/sampler.h, not
vendored), so its own test vector pins the generator.

Usage: python tests/golden/make_reference_kats.py [path-to-kazen_proto]
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def reference_root():
    """The kazen_proto checkout to read: the first command-line argument, else
    the KAZEN_PROTO_ROOT environment variable."""
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("KAZEN_PROTO_ROOT")
    if not root:
        sys.exit("usage: %s <kazen_proto checkout>  (or set KAZEN_PROTO_ROOT)" % os.path.basename(sys.argv[0]))
    return root


def main(ref):
    mf = os.path.join(ref, "tests/render_tests/microfacet_tests.cpp")
    em = os.path.join(ref, "tests/libusage_tests/embree_tests.cpp")
    mtxt = open(mf).read().splitlines()
    etxt = open(em).read()

    def line_of(lines, pat):
        for i, l in enumerate(lines, 1):
            if re.search(pat, l):
                return i
        raise RuntimeError(pat)

    fixed = re.search(r"fixed_beckmann_white_furnace_test\(([\d.]+)f,", "\n".join(mtxt))
    eps = re.findall(r"epsilon\(([\d.e-]+)\)", "\n".join(mtxt))
    furnace = [
        {"name": "fixed_beckmann", "alpha": float(fixed.group(1)), "theta_rad": "pi/4", "expected": 1.0,
         "rel_tol": float(eps[0]), "source": "tests/render_tests/microfacet_tests.cpp:%d-%d" % (
             line_of(mtxt, "fixed_beckmann_white_furnace_test"), line_of(mtxt, "fixed_beckmann_white_furnace_test") + 1)},
        {"name": "weak_beckmann", "theta_deg": 45.0, "alpha": 1.0, "expected": 1.0, "rel_tol": float(eps[1]),
         "source": "tests/render_tests/microfacet_tests.cpp:%d-%d" % (
             line_of(mtxt, "theta_o = 45"), line_of(mtxt, "interface_beckmann\\);") + 1)},
        {"name": "weak_ggx", "theta_deg": 45.0, "alpha": 1.0, "expected": 1.0, "rel_tol": float(eps[2]),
         "source": "tests/render_tests/microfacet_tests.cpp:%d-%d" % (
             line_of(mtxt, "interface_ggx ="), line_of(mtxt, "interface_ggx\\);") + 1)},
    ]
    verts = re.search(r"verts = \{([^}]*)\}", etxt).group(1)
    verts = [float(x) for x in re.findall(r"-?\d+(?:\.\d+)?", verts)]
    org = [float(re.search(r"org_%s = (-?\d+)" % a, etxt).group(1)) for a in "xyz"]
    dr = [float(re.search(r"dir_%s = (-?\d+)" % a, etxt).group(1)) for a in "xyz"]
    elines = etxt.splitlines()
    kats = {
        "furnace": furnace,
        "embree_single_triangle": {
            "verts": verts, "ray_o": org, "ray_d": dr, "tnear": 0.0, "tfar": "FLT_MAX",
            "expect_hit": True, "expect_prim": 0,
            "source": "tests/libusage_tests/embree_tests.cpp:%d-%d" % (line_of(elines, "std::array<float, 9> verts"),
                                                                          line_of(elines, "REQUIRE\\(rayhit.hit.geomID ==")),
        },
        "pcg32": {"initstate": 42, "initseq": 54,
                  "outputs": [0xa15c02b7, 0x7b47f409, 0xba1d3330, 0x83d2f293, 0xbfa4784b, 0xcbed606e],
                  "source": "PCG reference implementation (pcg32_srandom_r(42, 54)); pcg32.h is included by "
                            "src/core/sampler.h and not vendored"},
    }
    with open(os.path.join(HERE, "reference_kats.json"), "w") as f:
        json.dump(kats, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    main(reference_root())
