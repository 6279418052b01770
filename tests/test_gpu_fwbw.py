"""The forward/backward-difference derivative (numerics derivative FWBW_difference) on
the device against the oracle, through the C ABI.

xi_p = (e^(i t_p) - 1)(e^(i t_q) + 1)(e^(i t_r) + 1) / (4 h_p), t = 2 pi k / n, (q, r)
the next two axes (reference src/grid/spectral.cpp:115-124 states this operator; as
written there the expression ends in a comma operator and evaluates to zero, so the
oracle follows the forward/backward-difference formula it spells out).  xi is complex,
so K(xi) is Hermitian and Gamma uses the inverse of the real 6x6 form of
mech_base.cpp:164-205.  Tolerances: Gamma and divergence 1e-11 / 1e-12 (operator
level), full solves 1e-8 (the FP64 parity bound)."""
import numpy as np
import pytest

from oracle import dgo
from solver_cpp_gb300 import synthetic

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a); b = np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.fixture(scope="module")
def gpu():
    import solver_cpp_gb300 as g
    from solver_cpp_gb300 import build
    build.build()
    return g


@pytest.mark.parametrize("cells,size", [((8, 6, 5), (1.0, 0.75, 0.625)), ((7, 4, 9), (0.7, 0.4, 0.9))])
def test_fwbw_gamma_and_divergence_vs_oracle(gpu, cells, size):
    n = int(np.prod(cells))
    mat_at, q = synthetic.microstructure(cells, 4, seed=2)
    num = gpu.numerics(derivative="FWBW_difference")
    rve = gpu.RVE(cells, size, mat_at, q, num=num)
    rve.init()
    C_ref = rve.get("C_ref").ravel(order="F")
    rng = np.random.default_rng(4)
    P = 1e7 * rng.standard_normal((n, 3, 3))
    aim = 1e-4 * rng.standard_normal((3, 3))
    out = rve.gamma_convolution(P, aim)
    x1, _ = dgo.xi(cells, size, 2)
    ref = dgo.gamma_convolution(cells, x1, C_ref, dgo.fortran9(aim[None])[0], dgo.fortran9(P))
    assert rel(out, dgo.from_fortran9(ref.reshape(n, 9))) < 1e-11
    sg = dgo.scaled_geom(cells, size, "size+grid")
    r_or = dgo.divergence_rms(cells, size, sg, x1, dgo.fortran9(P))
    assert rve.calculate_divergence_rms(P) == pytest.approx(r_or, rel=1e-12)
    rve.close()


def test_fwbw_solve_and_coordinates_vs_oracle(gpu):
    cells, size = (8, 6, 5), (1.0, 0.75, 0.625)
    mat_at, q = synthetic.microstructure(cells, 5, seed=8)
    rve = gpu.RVE(cells, size, mat_at, q, num=gpu.numerics(derivative="FWBW_difference"))
    recs = rve.loop_over_loadcase([gpu.load_step("tensionX", t=3.0, N=3)])
    s = dgo.Solver(cells, size, mat_at, q, num=dgo.numerics(derivative="FWBW_difference"))
    ro = s.run([dgo.loadstep("tensionX", t=3.0, N=3)])
    assert len(recs) == len(ro) == 3
    for rg, r0 in zip(recs, ro):
        assert rel(rg["P_av"], dgo.from_fortran9(r0["P_av"])) < 1e-8
        assert rel(rg["F_av"], dgo.from_fortran9(r0["F_av"])) < 1e-8
        assert rg["iterations"] == r0["iterations"]
    for key in ("F", "P", "Fp"):
        assert rel(rve.get(key), dgo.from_fortran9(s.get(key))) < 1e-8, key
    un, up = rve.update_coords()
    un_o, up_o = dgo.update_coords(cells, size, s.get("F").reshape(-1), 2)
    assert rel(up, np.asarray(up_o).reshape(-1, 3)) < 1e-10
    assert rel(un, np.asarray(un_o).reshape(-1, 3)) < 1e-10
    rve.close()


def test_fwbw_mixed_precision_within_bound(gpu):
    cells = (8, 8, 8)
    mat_at, q = synthetic.microstructure(cells, 6, seed=12)
    steps = [gpu.load_step("tensionX", t=3.0, N=3)]
    a = gpu.RVE(cells, (1, 1, 1), mat_at, q, num=gpu.numerics(derivative="FWBW_difference")).loop_over_loadcase(steps)
    b = gpu.RVE(cells, (1, 1, 1), mat_at, q,
                num=gpu.numerics(derivative="FWBW_difference", precision="mixed")).loop_over_loadcase(steps)
    for ra, rb in zip(a, b):
        assert rel(rb["P_av"], ra["P_av"]) < 1e-5
