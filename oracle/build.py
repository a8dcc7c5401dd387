"""Compile oracle/kz_oracle.cpp into oracle/_build/libkz_oracle.so (g++, -O3, no FP contraction).

Test infrastructure: the CPU restatement used as parity checker and CPU baseline.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "kz_oracle.cpp")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libkz_oracle.so")
HDR = os.path.join(HERE, "..", "include", "kazen_gb300.h")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC), os.path.getmtime(HDR)):
        return LIB
    tmp = LIB + ".tmp"
    cmd = ["g++", "-O3", "-std=c++20", "-ffp-contract=off", "-fno-fast-math", "-shared", "-fPIC", "-pthread",
           SRC, "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        raise RuntimeError("oracle build failed")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="-f" in sys.argv))
