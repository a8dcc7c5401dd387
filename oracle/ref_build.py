"""Recipe: compile the reference's own header-only closure math into oracle/_ref.

TEST INFRASTRUCTURE. oracle/ref_harness.cpp includes kazen_proto's headers
where they lie in a kazen_proto checkout (src/shading/microfacet.h,
src/shading/fresnel.h, src/base/utils.h, src/core/sampling.h, src/base/vec.h),
with the stand-ins in oracle/ref_shim for their third-party includes (OSL's
Imath vector types, boost's math constants, the CMake-written config.h), and
g++ builds it into oracle/_ref/ref_harness. No reference source is copied.

The checkout is the first argument, else KAZEN_PROTO_ROOT, else
/root/reference. Without a checkout nothing is built (the fixture made from
the harness's output, tests/golden/reference_closure_vectors.npz, is
committed).

  python oracle/ref_build.py [kazen_proto checkout]
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "ref_harness.cpp")
SHIM = os.path.join(HERE, "ref_shim")
OUT_DIR = os.path.join(HERE, "_ref")
EXE = os.path.join(OUT_DIR, "ref_harness")
HEADERS = ["src/shading/microfacet.h", "src/shading/fresnel.h", "src/base/utils.h", "src/core/sampling.h",
           "src/base/vec.h"]


def reference_root(arg: str | None = None) -> str | None:
    root = arg or os.environ.get("KAZEN_PROTO_ROOT") or "/root/reference"
    return root if os.path.exists(os.path.join(root, "src", "shading", "microfacet.h")) else None


def build(root: str | None = None, force: bool = False) -> str | None:
    """Build the harness; returns its path, or None when no checkout is present."""
    root = reference_root(root)
    if root is None:
        return None
    os.makedirs(OUT_DIR, exist_ok=True)
    deps = [SRC] + [os.path.join(root, h) for h in HEADERS]
    for dp, _, fs in os.walk(SHIM):
        deps += [os.path.join(dp, f) for f in fs]
    if not force and os.path.exists(EXE) and os.path.getmtime(EXE) >= max(os.path.getmtime(d) for d in deps):
        return EXE
    tmp = EXE + ".tmp"
    cmd = ["g++", "-std=c++20", "-O2", "-ffp-contract=off", "-fno-fast-math", "-I", SHIM, "-I",
           os.path.join(root, "src"), SRC, "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        raise RuntimeError("reference harness build failed")
    os.replace(tmp, EXE)
    return EXE


def run(root: str | None = None) -> dict:
    """Run the harness; returns {table name: (rows, cols) float32 array}."""
    import numpy as np
    exe = build(root)
    if exe is None:
        raise RuntimeError("no kazen_proto checkout: pass its path or set KAZEN_PROTO_ROOT")
    txt = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    tables, name, rows = {}, None, []
    for line in txt.splitlines():
        if line.startswith("#"):
            if name:
                tables[name] = np.array(rows, np.float32)
            name, rows = line.split()[1], []
        elif line.strip():
            rows.append([float(x) for x in line.split()])
    if name:
        tables[name] = np.array(rows, np.float32)
    return tables


if __name__ == "__main__":
    p = build(sys.argv[1] if len(sys.argv) > 1 else None, force="-f" in sys.argv)
    print(p if p else "no kazen_proto checkout found: nothing built")
