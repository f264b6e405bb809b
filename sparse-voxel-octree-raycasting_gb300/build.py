"""Builds libsvo_gb300.so in this directory for sm_103a.

Two translation units compiled in parallel: csrc/svo_device.cu (nvcc, all
kernels and the device runtime) and csrc/svo_host.cpp (g++, octree builder,
scenes, cameras), linked into one shared library with the CUDA runtime
statically linked. Float arithmetic is strict IEEE binary32 on both sides
(-fmad=false / -ffp-contract=off, IEEE division and square root) because the
traversal is bit-exact against the CPU oracle.
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libsvo_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
    "-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
]
CXX_FLAGS = ["-std=c++17", "-O3", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-Wall", "-pthread"]

SOURCES_CU = ["svo_device.cu"]
SOURCES_CPP = ["svo_host.cpp"]
HEADERS = ["svo_trace.cuh", "svo_kernels.cuh", "svo_net.cuh", "svo_net_train.cuh"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cxx() -> str:
    return os.environ.get("CXX", "g++")


def _mtime(p: str) -> float:
    return os.path.getmtime(p) if os.path.exists(p) else 0.0


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compiles (if stale) and returns the path of libsvo_gb300.so."""
    os.makedirs(OBJ, exist_ok=True)
    deps = [os.path.join(CSRC, f) for f in SOURCES_CU + SOURCES_CPP + HEADERS]
    deps += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h", ".hpp"))]
    deps.append(os.path.join(INCLUDE, "svo_gb300.h"))
    deps.append(os.path.abspath(__file__))
    newest = max(_mtime(d) for d in deps)
    if not force and _mtime(LIB) > newest:
        return LIB
    nvcc = _nvcc()
    jobs = []
    for src in SOURCES_CU:
        obj = os.path.join(OBJ, src + ".o")
        jobs.append([nvcc] + NVCC_FLAGS + ["-I", INCLUDE, "-c", os.path.join(CSRC, src), "-o", obj])
    for src in SOURCES_CPP:
        obj = os.path.join(OBJ, src + ".o")
        jobs.append([_cxx()] + CXX_FLAGS + ["-I", INCLUDE, "-c", os.path.join(CSRC, src), "-o", obj])
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        for f in [ex.submit(_run, j) for j in jobs]:
            f.result()
    objs = [os.path.join(OBJ, s + ".o") for s in SOURCES_CU + SOURCES_CPP]
    tmp = LIB + ".tmp"
    _run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread"])
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
