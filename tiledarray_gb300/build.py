"""Build recipe for libtagpu.so (in-tree, sm_103a only, no cmake).

Each .cu is compiled by nvcc with `-gencode arch=compute_103a,code=sm_103a`,
the host library by g++ with -ffp-contract=off; all translation units are
compiled in parallel and linked into tiledarray_gb300/libtagpu.so.
Object files go to tiledarray_gb300/_build/ (git-ignored).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
ROOT = os.path.dirname(HERE)
LIB = os.path.join(HERE, "libtagpu.so")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["k_shape.cu", "k_permute.cu", "k_add.cu", "k_copy.cu", "k_gen.cu", "k_dmma.cu", "k_ozaki.cu",
              "k_noalloc.cu", "k_peak.cu"]
CPP_SOURCES = ["tagpu.cpp"]


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(ROOT, "include", "tagpu.h"))
    return files


def _newest(paths):
    return max(os.path.getmtime(p) for p in paths if os.path.exists(p))


def _compile(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(force: bool = False, verbose: bool = False, extra_nvcc=()) -> str:
    if (not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _newest(_deps())):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
    jobs = []
    objs = []
    for f in CU_SOURCES:
        o = os.path.join(BUILD, f + ".o")
        objs.append(o)
        jobs.append([NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr",
                     *extra_nvcc, *inc, "-c", os.path.join(CSRC, f), "-o", o])
    for f in CPP_SOURCES:
        o = os.path.join(BUILD, f + ".o")
        objs.append(o)
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
                     "-Wall", "-Wno-unused-function", *inc,
                     "-I" + os.path.join(CUDA_HOME, "include"), "-c", os.path.join(CSRC, f),
                     "-o", o])
    with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        outs = list(ex.map(_compile, jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    tmp = LIB + ".tmp"
    _compile([NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart", "-lcuda",
              "-Xcompiler", "-pthread"])
    os.replace(tmp, LIB)
    return LIB


def clean():
    if os.path.isdir(BUILD):
        shutil.rmtree(BUILD)
    if os.path.exists(LIB):
        os.remove(LIB)


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True))
