"""Build recipe for the CPU oracle (test infrastructure only).

Compiles the plain-C restatement in this directory into ``oracle/_build/libdgo.so``.
Only the tests, the smoke check and the CPU-baseline leg of ``bench.py`` load it.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
SOURCES = ["dgo_const.c", "dgo_cons.c", "dgo_spec.c", "dgo_solver.c"]
LIB = os.path.join(BUILD, "libdgo.so")


def build(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(HERE, s) for s in SOURCES] + [os.path.join(HERE, "dgo.h")]
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(s) <= t for s in srcs):
            return LIB
    cmd = ["gcc", "-O3", "-std=gnu11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-Wall", "-Wno-unused-function", "-o", LIB + ".tmp"]
    cmd += [os.path.join(HERE, s) for s in SOURCES] + ["-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
