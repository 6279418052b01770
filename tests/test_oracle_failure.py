"""Failure detection of the oracle's constitutive response (CPU only), injected on the
host: a NaN in one cell's deformation gradient makes that cell's integration fail
(phase_mechanical.f90:504,544,637,651, then the cut-back driver gives up) and the
response reports the points terminally ill (homogenization.f90:246,260-263), while the
other cells keep the results of the same response without the NaN cell; an Lp Newton
allowed a single iteration fails a plastic step the same way."""
import numpy as np

from oracle import dgo


def _case():
    from solver_cpp_gb300.synthetic import microstructure
    mat_at, q = microstructure((4, 4, 4), 5, seed=11)
    F = np.tile(np.eye(3), (64, 1, 1))
    F[:, 0, 0] += 4e-3
    F[:, 1, 1] -= 2e-3
    F[:, 2, 2] -= 2e-3
    return q[mat_at], F


def test_nan_deformation_gradient_is_terminally_ill():
    qa, F = _case()
    clean = dgo.PointSet(dgo.material(), qa)
    assert not clean.response(dgo.fortran9(F), 1.0, False)
    Fn = F.copy()
    Fn[5, 0, 0] = np.nan
    ops = dgo.PointSet(dgo.material(), qa)
    assert ops.response(dgo.fortran9(Fn), 1.0, False)
    keep = np.arange(64) != 5
    assert np.array_equal(ops.field("P")[keep], clean.field("P")[keep])


def test_single_lp_iteration_is_terminally_ill():
    qa, F = _case()
    ops = dgo.PointSet(dgo.material(N_iter_Lp_max=1), qa)
    assert ops.response(dgo.fortran9(F), 1.0, False)
