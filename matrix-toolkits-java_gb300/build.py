"""Builds the native libraries of the package in-tree.

  lib/libmtjg.so            the CUDA library behind include/mtjg.h (sm_103a only)
  lib/libmtjg_workloads.so  host-only generators of the synthetic systems

Translation units compile in parallel; the whole build takes well under a
minute.  Run as ``python build.py`` or through ``build()``.

MTJG_BUILD_DEFINES (environment) adds -D flags to every translation unit,
for the build-time tuning knobs of csrc/internal.h and csrc/spmv.cuh, e.g.
``MTJG_BUILD_DEFINES="-DMTJG_TILE_ROWS=512 -DMTJG_TILE_NNZ=2304"``; objects
built with other defines are rebuilt.
"""
from __future__ import annotations

import os
import platform
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "lib")
OBJ = os.path.join(LIB, "_obj")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["spmv.cu", "precond.cu", "solver.cu", "server.cu", "noalloc.cu", "convert.cu", "batch.cu"]
CPP_SOURCES = ["abi.cpp", "icc_host.cpp", "ilut_host.cpp", "mmio.cpp"]


def _cuda_home() -> str:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "bin", "nvcc")):
            return cand
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + proc.stdout)


def _newer(out: str, inputs: list[str]) -> bool:
    if not os.path.exists(out):
        return False
    t = os.path.getmtime(out)
    return all(os.path.getmtime(i) <= t for i in inputs)


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(OBJ, exist_ok=True)
    # objects built on another host architecture are never reused
    stamp = os.path.join(OBJ, "ARCH")
    defines = os.environ.get("MTJG_BUILD_DEFINES", "").split()
    if any(not d.startswith("-D") for d in defines):
        raise RuntimeError("MTJG_BUILD_DEFINES takes -D flags only")
    arch = " ".join([platform.machine()] + defines)
    if not os.path.exists(stamp) or open(stamp).read().strip() != arch:
        for f in os.listdir(OBJ):
            os.remove(os.path.join(OBJ, f))
        for f in ("libmtjg.so", "libmtjg_workloads.so"):
            if os.path.exists(os.path.join(LIB, f)):
                os.remove(os.path.join(LIB, f))
        with open(stamp, "w") as fh:
            fh.write(arch)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(INCLUDE, "mtjg.h"))
    jobs = []
    objs = []
    for src in CU_SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(OBJ, src + ".o")
        objs.append(obj)
        if _newer(obj, [path] + headers):
            continue
        cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
               "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr",
               *defines, "-I", CSRC, "-I", INCLUDE, "-c", path, "-o", obj]
        if ptxas_info:
            cmd.insert(1, "-Xptxas=-v")
        jobs.append(cmd)
    for src in CPP_SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(OBJ, src + ".o")
        objs.append(obj)
        if _newer(obj, [path] + headers):
            continue
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fvisibility=hidden", *defines,
                     "-I", os.path.join(cuda, "include"), "-I", CSRC, "-I", INCLUDE,
                     "-c", path, "-o", obj])
    with ThreadPoolExecutor(max_workers=max(1, min(8, len(jobs)))) as ex:
        for _ in ex.map(_run, jobs):
            pass
    so = os.path.join(LIB, "libmtjg.so")
    if not _newer(so, objs):
        _run([nvcc, *ARCH, "-shared", "-Xcompiler", "-fPIC", "-o", so, *objs, "-lpthread"])
    wl_src = os.path.join(CSRC, "workloads.c")
    wl_so = os.path.join(LIB, "libmtjg_workloads.so")
    if not _newer(wl_so, [wl_src]):
        _run(["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fvisibility=hidden",
              "-o", wl_so, wl_src, "-lm"])
    if verbose:
        print("built", so, wl_so)
    return so


if __name__ == "__main__":
    build(verbose=True, ptxas_info="--ptxas" in sys.argv)
