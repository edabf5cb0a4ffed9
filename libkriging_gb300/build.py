"""Build the GB300 shared library (libkriging_gb300/_build/liblkgpu.so) in-tree with nvcc for sm_103a.

Every translation unit is compiled as CUDA C++ (``-x cu``) in parallel, then linked into one shared object whose
``extern "C"`` symbols are declared in ``include/libkriging_gb300.h``.  Usage::

    python -m libkriging_gb300.build          # or: from libkriging_gb300.build import build; build()
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
SO = BUILD / "liblkgpu.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code is built without floating-point contraction (-ffp-contract=off): GCC contracts a * b + c into one fused
# operation by default where the target has one (the Arm hosts do), which would change host-side sums that must
# round like the reference's
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-O2", "-Xcompiler", "-ffp-contract=off", "-Xptxas", "-O3"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the GB300 library needs the CUDA 13 toolkit")


def sources():
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _needs_rebuild(objs, srcs) -> bool:
    if not SO.exists():
        return True
    t = SO.stat().st_mtime
    deps = srcs + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.hpp")) + [PKG.parent / "include" / "libkriging_gb300.h",
                                                                         Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps if p.exists())


def build(force: bool = False, verbose: bool = False, jobs: int | None = None) -> Path:
    srcs = sources()
    BUILD.mkdir(exist_ok=True)
    objs = [BUILD / (s.name + ".o") for s in srcs]
    if not force and not _needs_rebuild(objs, srcs):
        return SO
    nvcc = _nvcc()

    def compile_one(pair):
        src, obj = pair
        cmd = [nvcc, "-x", "cu", *ARCH, *NVCC_FLAGS, "-I", str(CSRC), "-I", str(PKG.parent / "include"), "-c",
               str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed on %s:\n%s%s" % (src.name, r.stdout, r.stderr))
        return r.stdout + r.stderr

    with ThreadPoolExecutor(max_workers=jobs or min(len(srcs), os.cpu_count() or 4)) as ex:
        for out in ex.map(compile_one, list(zip(srcs, objs))):
            if verbose and out.strip():
                print(out)
    tmp = SO.with_suffix(".so.tmp%d" % os.getpid())
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, SO)
    return SO


if __name__ == "__main__":
    p = build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(p)
