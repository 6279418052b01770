"""Command line of a DAMASK_grid job on the GPU: ``python -m solver_cpp_gb300``.

Mirrors ``DAMASK_grid -g GEOMETRY -l LOADCASE -m MATERIAL [-n NUMERICS] [-j JOBNAME]
[-w WORKINGDIRECTORY]`` (src/grid/main.cpp:36-49; the Fortran CLI.f90:142-148): the job
name defaults to the stems of the geometry, load-case, material and numerics files
joined by underscores, as the reference names its result file (e.g.
``mytest_tensionX_material.hdf5``); the DADF5 results go to ``<jobname>.hdf5`` in the
working directory.  One JSON line per increment is printed (time, iterations, residual
evaluations, err_div, err_BC, P_av in Pa, wall seconds).  Additions: ``--precision
mixed`` selects the mixed-precision form, ``--restart-every K`` writes
``<jobname>_restart.hdf5`` every K increments.
"""
import argparse
import json
import os
import sys


def job_name(geometry, load, material, numerics=None):
    """<geometry>_<load>_<material>[_<numerics>] from the files' stems."""
    parts = [geometry, load, material] + ([numerics] if numerics else [])
    return "_".join(os.path.splitext(os.path.basename(p))[0] for p in parts)


def parse_args(argv=None):
    p = argparse.ArgumentParser(prog="python -m solver_cpp_gb300",
                                description="DAMASK_grid spectral-basic job on one GPU")
    p.add_argument("-g", "--geom", "--geometry", dest="geometry", required=True, help="VTI geometry file")
    p.add_argument("-l", "--load", "--loadcase", dest="load", required=True, help="load case YAML file")
    p.add_argument("-m", "--material", "--materialconfig", dest="material", required=True,
                   help="material YAML file")
    p.add_argument("-n", "--numerics", "--numericsconfig", dest="numerics", default=None,
                   help="numerics YAML file")
    p.add_argument("-j", "--job", "--jobname", dest="job", default=None, help="job name (result file stem)")
    p.add_argument("-w", "--wd", "--workingdir", "--workingdirectory", dest="workdir", default=None,
                   help="working directory of the relative input paths and of the results")
    p.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    p.add_argument("--restart-every", type=int, default=0, help="restart file every K increments (0: none)")
    return p.parse_args(argv)


def main(argv=None, run=None):
    """Run the job; returns the per-increment records.  ``run`` replaces the solve
    (``inputs.grid_job``) for tests of the command line itself."""
    a = parse_args(argv)
    wd = os.path.abspath(a.workdir) if a.workdir else os.getcwd()

    def path(p):
        return p if os.path.isabs(p) else os.path.join(wd, p)

    files = {"geometry": path(a.geometry), "load": path(a.load), "material": path(a.material)}
    if a.numerics:
        files["numerics"] = path(a.numerics)
    for what, f in files.items():
        if not os.path.isfile(f):
            raise SystemExit(f"{what} file not found: {f}")
    name = a.job or job_name(a.geometry, a.load, a.material, a.numerics)
    result = os.path.join(wd, name + ".hdf5")
    restart = os.path.join(wd, name + "_restart.hdf5") if a.restart_every > 0 else None
    if run is None:
        from .inputs import grid_job as run
    rve, recs = run(files["geometry"], files["material"], files["load"], numerics=files.get("numerics"),
                    result=result, restart=restart, restart_every=a.restart_every, precision=a.precision)
    for i, r in enumerate(recs, 1):
        print(json.dumps({"increment": i, "t": r["t"], "iterations": r["iterations"],
                          "evaluations": r["evaluations"], "err_div": r["err_div"], "err_BC": r["err_BC"],
                          "P_av": [[float(x) for x in row] for row in r["P_av"]], "seconds": r["seconds"]}),
              flush=True)
    if rve is not None and hasattr(rve, "close"):
        rve.close()
    print(json.dumps({"job": name, "result": result, "restart": restart, "increments": len(recs)}), flush=True)
    return recs


if __name__ == "__main__":
    main(sys.argv[1:])
