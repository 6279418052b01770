"""Pin the CPU oracle against a complete Fortran DAMASK_grid result.

Fixture: tests/golden/damask_6grains6x7x8_tensionY.npz, extracted by
make_damask_fixture.py from the reference's python/tests/resources/Result files
(6 grains, 6x7x8 cells, tensionY, 40 increments, default numerics).  The oracle
restates the full path (constitutive law, FFT/Gamma/div-RMS, PETSc NGMRES), so the
comparison is iterate-for-iterate: agreement is at FP64 rounding level.
"""
import os

import numpy as np
import pytest

from oracle import dgo

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def run():
    fx = np.load(os.path.join(HERE, "golden", "damask_6grains6x7x8_tensionY.npz"))
    s = dgo.Solver(fx["cells"], fx["size"], fx["material_at"], fx["orientations"])
    recs = s.run([dgo.loadstep("tensionY", t=20.0, N=40, f_out=4)])
    return fx, s, recs


def test_volume_averages_per_increment(run):
    fx, s, recs = run
    assert len(recs) == 40
    for k, inc in enumerate(fx["increments"]):
        if inc == 0:
            continue
        P = dgo.from_fortran9(recs[inc - 1]["P_av"])
        F = dgo.from_fortran9(recs[inc - 1]["F_av"])
        relP = np.abs(P - fx["P_av"][k]).max() / np.abs(fx["P_av"][k]).max()
        assert relP < 1e-10, (inc, relP)
        assert np.abs(F - fx["F_av"][k]).max() < 1e-12


def test_fields_final_increment(run):
    fx, s, recs = run
    for name, key in (("F", "F"), ("P", "P"), ("F_p", "Fp"), ("L_p", "Lp")):
        ref = fx[f"{name}_40"]
        got = dgo.from_fortran9(s.get(key))
        rel = np.abs(got - ref).max() / np.abs(ref).max()
        assert rel < 1e-9, (name, rel)
    xi = s.get("xi")
    assert np.abs(xi - fx["xi_sl_40"]).max() / fx["xi_sl_40"].max() < 1e-10


def test_oracle_coordinates_and_orientations_vs_damask():
    """Coordinate update (u_p, u_n) and orientation output (O) of the oracle against the
    Fortran DAMASK result, computed from that result's own F and F_e fields."""
    from tests import cases
    fx = cases.damask_6grains()
    for inc in (20, 40):
        un, up = dgo.update_coords(fx["cells"], fx["size"], dgo.fortran9(fx[f"F_{inc}"]))
        assert np.abs(up - fx[f"u_p_{inc}"]).max() < 1e-12 * np.abs(fx[f"u_p_{inc}"]).max()
        assert np.abs(un - fx[f"u_n_{inc}"]).max() < 1e-12 * np.abs(fx[f"u_n_{inc}"]).max()
        O = dgo.orientation_output(dgo.fortran9(fx[f"F_e_{inc}"]))
        assert np.abs(O - fx[f"O_{inc}"]).max() < 1e-13
