"""Results (DADF5 layout), coordinates and restart through the C ABI.

The DADF5 file of the 6-grain tensionY run is read back with the project's HDF5
reader and compared with the Fortran DAMASK result shipped with the reference
(same layout of an increment group; F, P, F_p, u_p, u_n, O within 1e-8 relative;
t/s attributes); restart: a load case continued from a restart file is bitwise
identical to the uninterrupted run."""
import os
import sys

import numpy as np
import pytest

from oracle import dgo
from tests import cases

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
from hdf5lite import HDF5File  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def knowns():
    import json
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_knowns.json")) as f:
        return json.load(f)


@pytest.fixture(scope="module")
def gpu():
    import solver_cpp_gb300 as g
    from solver_cpp_gb300 import build
    build.build()
    return g


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


def test_dadf5_result_vs_damask(gpu, tmp_path):
    fx = cases.damask_6grains()
    rve = gpu.RVE(fx["cells"], fx["size"], fx["material_at"], fx["orientations"])
    path = tmp_path / "6grains_tensionY.hdf5"
    rve.loop_over_loadcase([gpu.load_step("tensionY", t=20.0, N=40, f_out=4)], result=path, phase="pheno_fcc",
                           homogenization="SX", setup={"tensionY.yaml": "loadstep: tensionY\n"})
    f = HDF5File(str(path))
    assert sorted(f.keys("/")) == sorted(fx["layout_root"].tolist())
    layout = []
    for g in ("geometry", "phase/pheno_fcc/mechanical", "homogenization/SX/mechanical"):
        layout += [f"{g}/{k}" for k in f.keys(f"/increment_40/{g}")]
    assert sorted(layout) == sorted(fx["layout_increment"].tolist())
    assert float(f.attrs("/increment_4")["t/s"]) == pytest.approx(2.0, rel=1e-14)
    assert list(f.attrs("/geometry")["cells"]) == list(fx["cells"])
    rec = f.read("/cell_to/phase")
    assert rec.shape == (rve.N, 1) and rec["label"][0, 0] == b"pheno_fcc"
    ph = "/phase/pheno_fcc/mechanical/"
    for inc in (20, 40):
        for name in ("F", "P", "F_p", "F_e"):
            assert rel(f.read(f"/increment_{inc}{ph}{name}"), fx[f"{name}_{inc}"]) < 1e-8, (inc, name)
        assert np.abs(f.read(f"/increment_{inc}{ph}O") - fx[f"O_{inc}"]).max() < 1e-8
        assert rel(f.read(f"/increment_{inc}/geometry/u_p"), fx[f"u_p_{inc}"]) < 1e-8
        assert rel(f.read(f"/increment_{inc}/geometry/u_n"), fx[f"u_n_{inc}"]) < 1e-8
    # coordinates of the final state against the oracle on the same F field
    un, up = rve.update_coords()
    un_o, up_o = dgo.update_coords(fx["cells"], fx["size"], dgo.fortran9(rve.get("F")))
    assert rel(up, up_o) < 1e-12 and rel(un, un_o) < 1e-12
    assert f.attrs(f"/increment_40{ph}O")["lattice"] == "cF"
    assert f.attrs(f"/increment_40{ph}P")["unit"] == "Pa"


def test_restart_continues_bitwise(gpu, tmp_path):
    cells, size, mat_at = cases.grains16()
    q = __import__("solver_cpp_gb300.synthetic", fromlist=["x"]).random_quaternions(20, 2024)
    step = gpu.load_step("tensionX", t=6.0, N=6)
    full = gpu.RVE(cells, size, mat_at, q)
    ref = full.loop_over_loadcase([step])
    first = gpu.RVE(cells, size, mat_at, q)
    rpath = tmp_path / "job_restart.hdf5"
    part = first.loop_over_loadcase([gpu.load_step("tensionX", t=6.0, N=6)], max_records=3, restart=rpath,
                                    restart_every=3)
    assert len(part) == 3
    # the file now holds the state after increment 6 (written every 3); rewrite it at 3 instead:
    again = gpu.RVE(cells, size, mat_at, q)
    again.init()
    for inc in range(3):
        again.run_increment(step, 0, inc)
    again.write_restart(rpath)
    cont = gpu.RVE(cells, size, mat_at, q)
    cont.read_restart(rpath)
    recs = [cont.run_increment(step, 0, inc) for inc in range(3, 6)]
    for a, b in zip(recs, ref[3:]):
        assert np.array_equal(a["P_av"], b["P_av"]) and np.array_equal(a["F_av"], b["F_av"])
        assert a["iterations"] == b["iterations"]
    for key in ("F", "P", "Fp", "xi"):
        assert np.array_equal(cont.get(key), full.get(key)), key


TENSION_Y = """solver:
  mechanical: spectral_basic
loadstep:
  - boundary_conditions:
      mechanical:
        dot_F: [[x, 0, 0], [0, 1.0e-3, 0], [0, 0, x]]
        P: [[0, x, x], [x, x, x], [x, x, 0]]
    discretization: {t: 20, N: 40}
    f_out: 4
"""


def test_grid_job_from_input_files(gpu, tmp_path, knowns):
    """DAMASK_grid-style job from the 6-grain geometry (VTI) and material.yaml of the
    Fortran run: averages equal the Fortran result; inputs stored under /setup."""
    from solver_cpp_gb300.inputs import grid_job
    fx = cases.damask_6grains()
    path = tmp_path / "job.hdf5"
    rve, recs = grid_job(knowns["vti_6grains"], knowns["material_yaml_6grains"], TENSION_Y, result=path)
    assert len(recs) == 40
    for k, inc in enumerate(fx["increments"]):
        if inc:
            assert rel(recs[inc - 1]["P_av"], fx["P_av"][k]) < 1e-9
    f = HDF5File(str(path))
    assert sorted(f.keys("/setup")) == ["geometry.vti", "load.yaml", "material.yaml"]
    assert f.read("/setup/load.yaml").item().rstrip(b"\0").decode() == TENSION_Y
