"""Extract the reference's Fortran DAMASK_grid trace into tests/golden/fortran_trace_tensionX_3x3x3.json.

The reference ships the standard output of one Fortran DAMASK_grid run (``output_damask_f.sh``:
``DAMASK_grid -g mytest.vti -l tensionX.yaml -m material.yaml``, default numerics): a
3 x 3 x 3 grid with 20 Voronoi grains (``make_grid.py``; the geometry file itself is not
in the tree), the example material (``examples/grid/material.yaml``, 20 orientations)
and uniaxial tension in x at 1e-3/s over 10 increments of 0.5 s.  This script keeps, per
converged increment, the last volume-averaged first Piola-Kirchhoff stress the run
printed (MPa, as printed) and the number of iterations it took, plus the 20 example
orientations (w, x, y, z) in the order of the material list.  Run in a checkout that
has the reference tree:

    python tests/golden/make_trace_fixture.py /path/to/reference
"""
import json
import os
import re
import sys


def trace_records(path):
    lines = open(path, encoding="utf-8", errors="replace").read().splitlines()
    recs, last_P, iters = [], None, 0
    i = 0
    while i < len(lines):
        ln = lines[i]
        if "Piola--Kirchhoff stress" in ln and "MPa" in ln:
            last_P = [[float(v) for v in lines[i + k].split()] for k in (1, 2, 3)]
            i += 4
            continue
        m = re.search(r"Increment (\d+)/\d+-\d+/\d+ @ Iteration \d+\S(\d+)\S\d+", ln)
        if m:
            iters = max(iters, int(m.group(2)))
        m = re.match(r"\s*increment (\d+) converged", ln)
        if m:
            recs.append({"increment": int(m.group(1)), "P_av_MPa": last_P, "iterations": iters})
            iters = 0
        i += 1
    return recs


def orientations(path):
    q = []
    for ln in open(path, encoding="utf-8"):
        m = re.match(r"\s*O:\s*\[([^\]]+)\]", ln)
        if m:
            q.append([float(v) for v in m.group(1).split(",")])
    return q


def main(ref):
    recs = trace_records(os.path.join(ref, "output_damask_f.sh"))
    q = orientations(os.path.join(ref, "examples", "grid", "material.yaml"))
    out = {"source": "output_damask_f.sh (Fortran DAMASK_grid v3.0.0-alpha8, -g mytest.vti -l tensionX.yaml "
                     "-m material.yaml); orientations from examples/grid/material.yaml",
           "cells": [3, 3, 3], "size": [1e-5, 1e-5, 1e-5], "grains": 20,
           "load": {"kind": "tensionX", "rate": 1e-3, "t": 5.0, "N": 10},
           "increments": recs, "orientations": q}
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "fortran_trace_tensionX_3x3x3.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=1)
    print(f"{len(recs)} increments, {len(q)} orientations -> {dst}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_trace_fixture.py /path/to/reference")
    main(sys.argv[1])
