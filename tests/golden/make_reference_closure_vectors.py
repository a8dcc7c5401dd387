"""Regenerate tests/golden/reference_closure_vectors.npz by running the
reference's own closure math (oracle/ref_harness.cpp built by
oracle/ref_build.py from a kazen_proto checkout's headers).

Tables (float32, one row per case; columns as the harness prints them):
  mdf_ggx, mdf_beckmann  wi wo m ax ay -> D(m) lambda(wi) lambda(wo) G1(wi) G1(wo) G(wo) pdf(m)
  kpgloss                dist wi wo ax ay eta -> f pdf   (KpGloss::eval, bsdfs.cpp:359-392)
  principle_specular     wi wo ax ay eta F0 -> f(rgb) pdf (bsdfs.cpp:688-717)
  diffuse                wo -> value = pdf                (bsdfs.cpp:27-33)
  fresnel                cos eta ext int -> fresnel_dielectric fresnel_refl_dielectric
                         fresnel_trans_dielectric fresnel(utils) fresnel_schlick schlick_weight
  refract                wi n eta -> refract(wi, n, eta)
  frame                  n v -> Frame(n).s .t to_local(v)
  warps                  u1 u2 a b -> to_cosine_hemisphere(u) to_uniform_disk(u)
                         sample_hemisphere(u) power_heuristic(1, a, 1, b)

Usage: python tests/golden/make_reference_closure_vectors.py <kazen_proto checkout>
       (or set KAZEN_PROTO_ROOT)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def main():
    from oracle import ref_build
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("KAZEN_PROTO_ROOT")
    if not root:
        sys.exit("usage: %s <kazen_proto checkout>  (or set KAZEN_PROTO_ROOT)" % os.path.basename(sys.argv[0]))
    tables = ref_build.run(root)
    out = os.path.join(HERE, "reference_closure_vectors.npz")
    np.savez_compressed(out, **tables)
    print(out, {k: v.shape for k, v in tables.items()})


if __name__ == "__main__":
    main()
