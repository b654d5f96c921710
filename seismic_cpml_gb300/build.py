"""Build libcpml.so (the C-ABI library) in-tree with nvcc for sm_103a.

Each translation unit is compiled in parallel; the shared library lands in
seismic_cpml_gb300/_build/libcpml.so. No CMake, no torch extension machinery:
the product is a plain C-ABI shared library.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libcpml.so")
PROGRAM = os.path.join(OUT, "cpml_program")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["api.cu", "kernels2d.cu", "kernels2d_ext.cu", "kernels3d.cu", "fused3d.cu", "support.cu",
           "noalloc.cu", "batch2d.cu", "cluster2d.cu", "surrogate.cu", "host.cpp"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    deps = [path] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    deps.append(os.path.join(HERE, "..", "include", "cpml.h"))
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-Wall", "-c", path, "-o", obj, *extra]
    if src.endswith(".cpp"):
        cmd = [nvcc(), "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, extra: list[str] | None = None) -> str:
    os.makedirs(OUT, exist_ok=True)
    extra = extra or []
    with ThreadPoolExecutor(max_workers=min(8, len(SOURCES))) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        tmp = LIB + ".tmp"
        cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    drv = os.path.join(CSRC, "driver.cpp")
    if not os.path.exists(PROGRAM) or os.path.getmtime(PROGRAM) < max(os.path.getmtime(drv), os.path.getmtime(LIB)):
        cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", drv, "-o", PROGRAM + ".tmp",
               "-L" + OUT, "-lcpml", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"driver link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(PROGRAM + ".tmp", PROGRAM)
    if verbose:
        print("built", LIB, "and", PROGRAM)
    return LIB


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
