"""In-tree build of the native libraries (no cmake, one -gencode, parallel compiles).

Outputs, git-ignored:
  _lib/libgrt.so            the C-ABI traversal library (include/grt.h)
  _lib/libgrt_workloads.so  the seeded scene / ray generators
Objects go to _build/. Host code is compiled with -ffp-contract=off everywhere: the BVH builder
and the workload generators must round every float operation as written on x86-64 and
aarch64 alike.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "_lib")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found (set CUDA_HOME)")


def _run(cmd: list[str]) -> str:
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + p.stdout)
    return p.stdout


def _newer(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def build(verbose: bool = False, ptxas_info: bool = False) -> dict:
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".hpp", ".cuh", ".h"))]
    headers.append(os.path.join(HERE, "..", "include", "grt.h"))
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = ["api.cpp", "api_pt.cpp", "api_multi.cpp", "api_gpu_build.cpp", "api_direct.cpp", "bvh_builder.cpp", "bvh_cache.cpp"]
    hostflags = ["-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-Wall", "-Wno-unused-function"]
    jobs = []
    for f in cu:
        o = os.path.join(OBJ, f + ".o")
        cmd = [nvcc, ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
               "-c", os.path.join(CSRC, f), "-o", o]
        if ptxas_info:
            cmd.insert(1, "-Xptxas=-v")
        jobs.append((o, [os.path.join(CSRC, f)] + headers, cmd))
    for f in cpp:
        o = os.path.join(OBJ, f + ".o")
        cmd = ["g++", *hostflags, "-I" + os.path.join(cuda, "include"), "-c", os.path.join(CSRC, f), "-o", o]
        jobs.append((o, [os.path.join(CSRC, f)] + headers, cmd))
    wl_src = os.path.join(CSRC, "workloads.cpp")
    wl_lib = os.path.join(LIB, "libgrt_workloads.so")
    jobs.append((wl_lib, [wl_src, os.path.join(CSRC, "pmath.hpp")],
                 ["g++", *hostflags, "-shared", wl_src, "-o", wl_lib]))
    logs = {}
    todo = [j for j in jobs if ptxas_info or not _newer(j[0], j[1])]
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(todo), os.cpu_count() or 4))) as ex:
        for (o, _, cmd), out in zip(todo, ex.map(lambda j: _run(j[2]), todo)):
            logs[os.path.basename(o)] = out
            if verbose:
                print(" ".join(cmd))
    grt_lib = os.path.join(LIB, "libgrt.so")
    objs = [os.path.join(OBJ, f + ".o") for f in cu + cpp]
    if todo or not os.path.exists(grt_lib):
        logs["link"] = _run([nvcc, ARCH, "-shared", "-o", grt_lib, *objs, "-Xcompiler", "-fPIC"])
    return logs


if __name__ == "__main__":
    info = "--ptxas" in sys.argv
    logs = build(verbose="-v" in sys.argv, ptxas_info=info)
    if info:
        for k, v in logs.items():
            if v.strip():
                print(f"== {k}\n{v}")
    print("built", os.path.join(LIB, "libgrt.so"))
