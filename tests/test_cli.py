"""The job command line (python -m solver_cpp_gb300), CPU only: DAMASK_grid's options
(-g -l -m -n -j -w), the reference's job name (stems joined by underscores, e.g.
mytest_tensionX_material), the result and restart paths handed to the solve, one JSON
line per increment, and refusal of missing input files.  The solve itself (grid_job)
is replaced by a recorder here; tests/test_gpu_output.py runs it on the GPU."""
import json

import numpy as np
import pytest


def test_job_name_is_the_references():
    from solver_cpp_gb300.__main__ import job_name
    assert job_name("mytest.vti", "tensionX.yaml", "material.yaml") == "mytest_tensionX_material"
    assert job_name("a/2x2x2.vti", "b/tensionX.yaml", "material.yaml", "numerics.yaml") == \
        "2x2x2_tensionX_material_numerics"


def test_command_line_hands_the_job_to_the_solver(tmp_path, capsys):
    from solver_cpp_gb300.__main__ import main
    for n in ("grid.vti", "tensionX.yaml", "material.yaml", "numerics.yaml"):
        (tmp_path / n).write_text("x")
    seen = {}

    def fake_run(geometry, material, load, numerics=None, result=None, restart=None, restart_every=0,
                 precision="fp64"):
        seen.update(geometry=geometry, material=material, load=load, numerics=numerics, result=result,
                    restart=restart, restart_every=restart_every, precision=precision)
        rec = dict(t=0.5, iterations=3, evaluations=5, err_div=0.1, err_BC=0.2, P_av=np.eye(3) * 1e6, seconds=0.01)
        return None, [rec, dict(rec, t=1.0)]

    recs = main(["-g", "grid.vti", "-l", "tensionX.yaml", "-m", "material.yaml", "-n", "numerics.yaml",
                 "-w", str(tmp_path), "--precision", "mixed", "--restart-every", "2"], run=fake_run)
    assert len(recs) == 2
    assert seen["geometry"] == str(tmp_path / "grid.vti") and seen["load"] == str(tmp_path / "tensionX.yaml")
    assert seen["numerics"] == str(tmp_path / "numerics.yaml") and seen["precision"] == "mixed"
    assert seen["result"] == str(tmp_path / "grid_tensionX_material_numerics.hdf5")
    assert seen["restart"] == str(tmp_path / "grid_tensionX_material_numerics_restart.hdf5")
    assert seen["restart_every"] == 2
    lines = [json.loads(x) for x in capsys.readouterr().out.strip().splitlines()]
    assert [x["increment"] for x in lines[:2]] == [1, 2] and lines[1]["t"] == 1.0
    assert lines[0]["P_av"][0][0] == 1e6 and lines[-1]["increments"] == 2


def test_command_line_refuses_missing_inputs(tmp_path):
    from solver_cpp_gb300.__main__ import main
    (tmp_path / "grid.vti").write_text("x")
    with pytest.raises(SystemExit, match="load file not found"):
        main(["-g", "grid.vti", "-l", "nope.yaml", "-m", "material.yaml", "-w", str(tmp_path)],
             run=lambda *a, **k: (None, []))
    with pytest.raises(SystemExit):
        main(["-g", "grid.vti"])                      # -l and -m are required
