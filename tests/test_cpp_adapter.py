"""The header-only C++ adapter (include/kazen_gb300.hpp) compiles and links
against the library on any machine, and runs the reference's single-triangle
case on a GPU."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "adapter_demo.cpp")
OUT = os.path.join(ROOT, "kazen_proto_gb300", "_build", "adapter_demo")


def build_demo(native_lib):
    libdir = os.path.join(ROOT, "kazen_proto_gb300", "_build")
    subprocess.run(["g++", "-std=c++17", "-O1", SRC, "-o", OUT, "-L" + libdir, "-lkazen_gb300",
                    "-Wl,-rpath," + libdir], check=True)
    return OUT


def test_adapter_compiles_and_links(native_lib):
    assert os.path.exists(build_demo(native_lib))


@pytest.mark.gpu
def test_adapter_runs_reference_case(gpu):
    exe = build_demo(gpu)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "hit=1 geom=0 prim=0 t=1.000000 occluded=1" in r.stdout
