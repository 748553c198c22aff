"""Build recipe of libbemgpu.so (sm_103a) -- compiles every translation unit in parallel.

Usage: ``python build.py`` (or ``__graft_entry__.build()``).  Output:
``bemgpu/libbemgpu.so`` beside the Python host package; objects in ``_build/``.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
OUT = os.path.join(HERE, "bemgpu", "libbemgpu.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fPIC,-ffp-contract=off", f"-I{INCLUDE}"] + ARCH
CXX_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", f"-I{INCLUDE}"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libbemgpu")


def _stale(obj: str, src: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + deps)


def _compile(cmd: list[str]) -> tuple[list[str], int, str]:
    r = subprocess.run(cmd, capture_output=True, text=True)
    return cmd, r.returncode, r.stdout + r.stderr


def build(verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    deps = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))
    cmds, objs = [], []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, src, deps):
            cmds.append([nvcc] + NVCC_FLAGS + ["-c", src, "-o", obj])
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cpp"))):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, src, deps):
            cmds.append(["g++"] + CXX_FLAGS + ["-c", src, "-o", obj])
    jobs = jobs or min(len(cmds), os.cpu_count() or 4) or 1
    errors = []
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        for cmd, rc, log in ex.map(_compile, cmds):
            if verbose or rc:
                sys.stderr.write(" ".join(cmd) + "\n" + log)
            if rc:
                errors.append(cmd[-3])
    if errors:
        raise RuntimeError(f"compilation failed: {errors}")
    if cmds or not os.path.exists(OUT) or any(os.path.getmtime(o) > os.path.getmtime(OUT)
                                              for o in objs):
        link = [nvcc, "-shared"] + ARCH + ["-o", OUT] + objs + ["-lpthread"]
        r = subprocess.run(link, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(" ".join(link) + "\n" + r.stdout + r.stderr)
            raise RuntimeError("link failed")
    return OUT


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
