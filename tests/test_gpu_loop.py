"""The load-case loop through the C ABI on the GPU (TestDamaskGridLoopOverLoadcase,
test_damask_grid.cpp): one increment of a 1 s step ends at t = 1 with the oracle's
iteration count, and with at most one iteration and no cut-back allowed the loop
returns DGX_ERR_NOT_CONVERGED (the reference throws) instead of a result."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

Q = [[1.0, 0.0, 0.0, 0.0], [0.7936696712125002, -0.28765777461664166, -0.3436487135089419, 0.4113964260949434]]


def test_loop_result_and_no_solution():
    import solver_cpp_gb300 as g
    from solver_cpp_gb300 import build
    from oracle import dgo
    build.build()
    cells, size, mat = (2, 1, 1), (2e-5, 1e-5, 1e-5), np.array([0, 1])
    rve = g.RVE(cells, size, mat, Q)
    recs = rve.loop_over_loadcase([g.load_step("tensionX", t=1.0, N=1)])
    ref = dgo.Solver(cells, size, mat, Q).run([dgo.loadstep("tensionX", t=1.0, N=1)])
    assert len(recs) == 1 and recs[0]["t"] == 1.0
    assert recs[0]["iterations"] == ref[0]["iterations"]
    rve.close()
    rve = g.RVE(cells, size, mat, Q, num=g.numerics(itmax=1, max_cut_back=0))
    with pytest.raises(g.DgxError, match=r"\(-5\)"):
        rve.loop_over_loadcase([g.load_step("tensionX", t=1.0, N=1)])
    rve.close()
