"""Build libhdg.so in-tree with nvcc for sm_103a (GB300).

Translation units are compiled in parallel; host C++ is built without floating-point
contraction so that x86_64 and aarch64 produce the same mesh coordinates and tables.
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
LIB = os.path.join(HERE, "libhdg.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU = ["element.cu", "trace.cu", "cg.cu", "recover.cu", "noalloc.cu", "amg.cu", "lagrange.cu", "refine.cu"]
CPP = ["capi.cpp", "mesh.cpp", "tables.cpp", "assembler.cpp", "serve.cpp", "dofhandler.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libhdg")


def _sources():
    return [os.path.join(CSRC, f) for f in CU + CPP]


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(HERE, "..", "include", "hdg.h"))
    return hs


def needs_build() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in _sources() + _headers() + [__file__])


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not needs_build():
        return LIB
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "-I", os.path.join(HERE, "..", "include")]
    jobs = []
    for f in CU:
        obj = os.path.join(BUILD, f + ".o")
        jobs.append([nvcc, *ARCH, "-lineinfo", *common, "-c", os.path.join(CSRC, f), "-o", obj])
    for f in CPP:
        obj = os.path.join(BUILD, f + ".o")
        jobs.append([nvcc, *common, "-x", "c++", "-c", os.path.join(CSRC, f), "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)
        return cmd[-1]

    with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        objs = list(ex.map(run, jobs))
    tmp = LIB + ".tmp"
    run([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
