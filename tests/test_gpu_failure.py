"""Failure detection, injected on the host (no GPU fault, trap or hang), through the C
ABI and against the oracle: an Lp Newton allowed too few iterations for a plastic step
makes the cells' integration fail (phase_mechanical.f90:544 and the cut-back driver's
give-up, :1046-1085); the response reports the RVE terminally ill
(homogenization.f90:246, 260-263), as the oracle does.  (The oracle's handling of a NaN
deformation gradient is tested on the CPU, tests/test_oracle_failure.py.)"""
import numpy as np
import pytest

from oracle import dgo

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    import solver_cpp_gb300 as g
    from solver_cpp_gb300 import build
    build.build()
    return g


def _setup(gpu, mat=None, omat=None):
    from solver_cpp_gb300.synthetic import microstructure
    cells = (4, 4, 4)
    mat_at, q = microstructure(cells, 5, seed=11)
    rve = gpu.RVE(cells, (1, 1, 1), mat_at, q, mat=mat)
    ops = dgo.PointSet(omat if omat is not None else dgo.material(), q[mat_at])
    F = np.tile(np.eye(3), (64, 1, 1))
    F[:, 0, 0] += 4e-3
    F[:, 1, 1] -= 2e-3
    F[:, 2, 2] -= 2e-3
    return rve, ops, F


def test_too_few_lp_iterations_is_terminally_ill(gpu):
    rve, ops, F = _setup(gpu, mat=gpu.material(N_iter_Lp_max=1), omat=dgo.material(N_iter_Lp_max=1))
    rve.constitutive_response(F, 1.0)
    ill_ref = bool(ops.response(dgo.fortran9(F), 1.0, False))
    assert rve.terminally_ill == ill_ref and ill_ref
    rve.close()
