"""The oracle against the reference's Fortran DAMASK_grid trace (CPU only).

The reference ships the output of one Fortran run: a 3 x 3 x 3 grid of 20 random Voronoi
grains with the 20 orientations of the example material, uniaxial tension in x at
1e-3/s, 10 increments of 0.5 s (fixture `tests/golden/fortran_trace_tensionX_3x3x3.json`,
made by `make_trace_fixture.py`).  The run's grain arrangement is not in the tree, so the
oracle solves the same orientations on 16 seeded arrangements of the same grid and the
trace must look like one draw of them: the elastic first increment (which depends on
the orientations alone) within 1 % of the arrangements' mean, every increment's P_xx
within 2.5 standard deviations of that mean, the lateral stresses at their prescribed
zero, and a similar number of iterations per increment.
"""
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SEEDS = range(16)


def _fixture():
    with open(os.path.join(HERE, "golden", "fortran_trace_tensionX_3x3x3.json")) as f:
        return json.load(f)


def _runs(fx):
    from oracle import dgo
    from solver_cpp_gb300.synthetic import voronoi
    cells, size = tuple(fx["cells"]), tuple(fx["size"])
    q = np.asarray(fx["orientations"], dtype=float)
    ld = fx["load"]
    P, its = [], []
    for seed in SEEDS:
        mat = voronoi(cells, size, fx["grains"], seed)
        s = dgo.Solver(cells, size, mat, q)
        recs = s.run([dgo.loadstep(ld["kind"], t=ld["t"], N=ld["N"], rate=ld["rate"])])
        P.append([dgo.from_fortran9(r["P_av"]) / 1e6 for r in recs])
        its.append([r["iterations"] for r in recs])
    return np.asarray(P), np.asarray(its, dtype=float)


def test_oracle_reproduces_the_fortran_trace_statistically():
    fx = _fixture()
    ref = np.array([r["P_av_MPa"] for r in fx["increments"]])            # (10, 3, 3), MPa
    ref_its = np.array([r["iterations"] for r in fx["increments"]], dtype=float)
    P, its = _runs(fx)                                                   # (16, 10, 3, 3)
    assert P.shape[1] == ref.shape[0] == 10
    Pxx, ref_xx = P[:, :, 0, 0], ref[:, 0, 0]
    mean, sd = Pxx.mean(0), Pxx.std(0)
    # elastic first increment: set by the orientations, not by their arrangement
    assert abs(mean[0] - ref_xx[0]) / ref_xx[0] < 0.01, (mean[0], ref_xx[0])
    # every increment: the Fortran run is one draw of the arrangements' distribution
    assert np.all(np.abs(ref_xx - mean) <= 2.5 * sd + 1e-9), (ref_xx, mean, sd)
    # hardening towards saturation, as in the trace
    assert np.all(np.diff(mean) > 0.0) and (mean[-1] - mean[-2]) / mean[-1] < 0.005
    # the stress boundary condition P_yy = P_zz = 0 within the solver's stress tolerance
    assert np.abs(P[:, :, 1, 1]).max() < 0.1 and np.abs(P[:, :, 2, 2]).max() < 0.1
    # the same convergence behaviour of the spectral solver, increment by increment
    assert np.all(np.abs(its.mean(0) - ref_its) <= 2.0), (its.mean(0), ref_its)
