"""Build libkazen_gb300.so (sm_103a) in-tree with nvcc.

Translation units compile in parallel, then link into
kazen_proto_gb300/_build/libkazen_gb300.so. The whole library is compiled
with --fmad=false so FP32 expressions round as written (the traversal's
bit-exact hit ids depend on it) and with IEEE division / square root
(no fast-math anywhere).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libkazen_gb300.so")

SOURCES = ["kz_api.cu", "kz_trace.cu", "kz_kernels.cu", "kz_shade_guided.cu", "kz_batch.cu", "kz_megakernel.cu",
           "kz_closures.cu", "kz_mlp.cu", "kz_mlp_tc.cu", "kz_guide_tc.cu",
           "kz_bvh.cpp"]
DEPS = ["kz_device.cuh", "kz_traverse.cuh", "kz_guide.cuh", "kz_stages.cuh", "kz_internal.h", "kz_bvh.h", "kz_tc.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    p = shutil.which("nvcc")
    if p:
        return p
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def common_flags() -> list[str]:
    return [
        "-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-prec-div=true", "-prec-sqrt=true",
        "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
        "-I", os.path.join(HERE, "..", "include"),
    ] + ARCH


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def extra_flags() -> list[str]:
    """Extra nvcc flags from KZ_NVCC_FLAGS (tuning builds, e.g. -DKZ_TRACE_REFILL=12)."""
    return os.environ.get("KZ_NVCC_FLAGS", "").split()


# Test builds: the library compiled with extra defines into its own folder
# (kazen_proto_gb300/_build_<name>/), loaded by tests in a separate process
# through KZ_LIBRARY. "stack2": a two-entry traversal stack, which makes the
# traversal kernels take their stack-overflow path (KZ_ERR_STACK).
TEST_VARIANTS = {"stack2": ["-DKZ_WIDE_STACK=2", "-DKZ_SMEM_STACK=0"]}


def build(verbose: bool = False, ptxas_verbose: bool = False, force: bool = False, variant: str | None = None) -> str:
    out_dir = BUILD if variant is None else os.path.join(HERE, "_build_" + variant)
    lib_path = LIB if variant is None else os.path.join(out_dir, "libkazen_gb300.so")
    os.makedirs(out_dir, exist_ok=True)
    nvcc = nvcc_path()
    flags = extra_flags() if variant is None else TEST_VARIANTS[variant]
    # a change of the extra flags rebuilds everything
    stamp = os.path.join(out_dir, "flags.txt")
    flags_now = " ".join(flags)
    if not os.path.exists(stamp) or open(stamp).read() != flags_now:
        force = True
        with open(stamp, "w") as f:
            f.write(flags_now)
    hdrs = [os.path.join(CSRC, d) for d in DEPS] + [os.path.join(HERE, "..", "include", "kazen_gb300.h")]
    objs = []
    jobs = []
    for src in SOURCES:
        sp = os.path.join(CSRC, src)
        obj = os.path.join(out_dir, src + ".o")
        objs.append(obj)
        if not force and _newer(obj, [sp] + hdrs):
            continue
        cmd = [nvcc, "-c", sp, "-o", obj] + common_flags() + flags
        if ptxas_verbose and src.endswith(".cu"):
            cmd += ["-Xptxas", "-v"]
        jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or ptxas_verbose or r.returncode != 0:
                sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed for {cmd[2]}")
    if force or jobs or not _newer(lib_path, objs):
        tmp = lib_path + ".tmp"
        cmd = [nvcc, "-shared", "-o", tmp] + objs + ARCH + ["-Xcompiler", "-fPIC", "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            raise RuntimeError("link failed")
        os.replace(tmp, lib_path)
    return lib_path


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, ptxas_verbose="--ptxas" in sys.argv, force="-f" in sys.argv)
    print(LIB)
