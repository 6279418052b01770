"""Build the sm_103a shared library ``solver_cpp_gb300/_build/libdgx.so`` (in tree).

Each CUDA translation unit is compiled by nvcc in parallel for
``-gencode arch=compute_103a,code=sm_103a`` and linked into one C-ABI library
(declared in include/dgx.h).  No CMake; one nvcc per source file.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libdgx.so")
SOURCES = ["constitutive.cu", "spectral.cu", "solver.cu", "peak.cu", "noalloc.cu", "batch.cu", "results.cu"]
HOST_SOURCES = ["ref_stiffness.cpp", "server.cpp", "vti.cpp"]
HEADERS = ["dgx_internal.cuh", "spectral.cuh", "rve.cuh", "h5lite.hpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _flags(verbose_ptxas=False):
    # host code keeps the reference's FP64 rounding (no FMA contraction); device code is unaffected
    f = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
         "-I", os.path.join(ROOT, "include")] + ARCH
    if verbose_ptxas:
        f += ["-Xptxas", "-v"]
    return f


def _compile(src, verbose_ptxas=False):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    if src.endswith(".cpp"):
        cuda_inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc()))), "include")
        cmd = ["g++", "-c", os.path.join(CSRC, src), "-o", obj, "-O2", "-std=c++17", "-fPIC", "-pthread",
               "-ffp-contract=off", "-I", cuda_inc]
    else:
        cmd = [nvcc(), "-c", os.path.join(CSRC, src), "-o", obj] + _flags(verbose_ptxas)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    deps = [os.path.join(CSRC, s) for s in SOURCES + HOST_SOURCES + HEADERS] + [os.path.join(ROOT, "include", "dgx.h"),
                                                                   os.path.abspath(__file__)]
    if not force and not verbose_ptxas and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in deps):
            return LIB
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES) + len(HOST_SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose_ptxas), SOURCES + HOST_SOURCES))
    if verbose_ptxas:
        for _, log in results:
            sys.stderr.write(log)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-shared", "-o", tmp] + objs + ARCH + ["-lcudart", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
