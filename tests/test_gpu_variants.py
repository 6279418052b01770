"""GPU parity (through the C ABI) on the load-case and numerics variants of the
reference's grid solver, against the CPU oracle with the same inputs: fixed-point
solver, rotated boundary-condition frame (R), geometric time stepping (r), F / L
deformation targets, stress-rate (dot_P) targets, divergence corrections, central
difference derivative, Gamma update, non-lazy tangent, multi-step load cases with
rate estimation, and the sub-step cut-back driver (a step too large to converge).

Tolerance: 1e-8 relative (FP64 plain form) on volume-averaged P and F per increment,
identical iteration and cut-back counts, and the final F and P fields.
"""
import numpy as np
import pytest

from oracle import dgo
from solver_cpp_gb300 import loadcase, synthetic

pytestmark = pytest.mark.gpu

TOL = 1e-8
CELLS = (8, 6, 4)


@pytest.fixture(scope="module")
def gpu():
    import solver_cpp_gb300 as g
    from solver_cpp_gb300 import build
    build.build()
    return g


def rel(a, b):
    a = np.asarray(a); b = np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def to_oracle(step):
    ls = dgo.LoadStep()
    for f, _ in dgo.LoadStep._fields_:
        v = getattr(step, f)
        if hasattr(v, "__len__"):
            for i in range(len(v)):
                getattr(ls, f)[i] = v[i]
        else:
            setattr(ls, f, v)
    return ls


def tension(rate=1e-3, t=3.0, N=3, **kw):
    return loadcase.make_step("dot_F", np.diag([rate, 0, 0]), np.diag([0, 1, 1]), "P", np.zeros((3, 3)),
                              1 - np.diag([0, 1, 1]), t, N, **kw)


def run_both(g, steps, num_kw=None, gpu_only_kw=None, grains=5, seed=77, tol=TOL, fields=True):
    mat, q = synthetic.microstructure(CELLS, grains, seed)
    num_kw = num_kw or {}
    rve = g.RVE(CELLS, (1.0, 1.0, 1.0), mat, q, num=g.numerics(**num_kw, **(gpu_only_kw or {})))
    rg = rve.loop_over_loadcase(steps)
    so = dgo.Solver(CELLS, (1.0, 1.0, 1.0), mat, q, num=dgo.numerics(**num_kw))
    ro = so.run([to_oracle(s) for s in steps])
    assert len(rg) == len(ro)
    for a, b in zip(rg, ro):
        assert a["iterations"] == b["iterations"] and a["cutbacks"] == b["cutbacks"]
        assert rel(a["P_av"], dgo.from_fortran9(b["P_av"])) < tol
        assert rel(a["F_av"], dgo.from_fortran9(b["F_av"])) < tol
    for key in ("F", "P") if fields else ():
        assert rel(rve.get(key), dgo.from_fortran9(so.get(key))) < tol, key
    return rg


def test_fixed_point_solver(gpu):
    run_both(gpu, [tension(N=2, t=2.0)], num_kw={"solver": 1})


def test_rotated_boundary_frame(gpu):
    c, s = np.cos(np.pi / 12), np.sin(np.pi / 12)
    run_both(gpu, [tension(rot=(c, 0.0, 0.0, s))])


def test_geometric_time_steps(gpu):
    recs = run_both(gpu, [tension(t=4.0, N=4, r=1.5)])
    dts = [r["dt"] for r in recs]
    assert dts[1] / dts[0] == pytest.approx(1.5)


def test_deformation_gradient_and_velocity_gradient_targets(gpu):
    F_target = np.eye(3); F_target[0, 0] = 1.004
    sF = loadcase.make_step("F", F_target, np.diag([0, 1, 1]), "P", np.zeros((3, 3)), 1 - np.diag([0, 1, 1]), 4.0, 4)
    L = np.zeros((3, 3)); L[0, 0] = 1e-3; L[0, 1] = 2e-4
    mask = np.zeros((3, 3), int); mask[1, 1] = mask[2, 2] = 1
    sL = loadcase.make_step("L", L, mask, "P", np.zeros((3, 3)), 1 - mask, 3.0, 3)
    run_both(gpu, [sF, sL])


def test_stress_rate_target(gpu):
    dm = np.diag([0, 1, 1])
    sv = np.zeros((3, 3)); sv[1, 1] = 2e5
    s = loadcase.make_step("dot_F", np.diag([1e-3, 0, 0]), dm, "dot_P", sv, 1 - dm, 3.0, 3)
    run_both(gpu, [s])


@pytest.mark.parametrize("divcorr,deriv", [("none", "continuous"), ("size", "continuous"),
                                           ("size+grid", "central_difference")])
def test_divergence_correction_and_derivative(gpu, divcorr, deriv):
    run_both(gpu, [tension(N=2, t=2.0)], num_kw={"divergence_correction": divcorr, "derivative": deriv})


def test_gamma_update(gpu):
    run_both(gpu, [tension(N=3, t=3.0)], num_kw={"update_gamma": 1})


def test_non_lazy_tangent(gpu):
    run_both(gpu, [tension(N=2, t=2.0)], gpu_only_kw={"lazy_tangent": 0})


def test_two_steps_with_rate_estimate(gpu):
    shear = loadcase.make_step("dot_F", np.array([[0, 1e-3, 0], [0, 0, 0], [0, 0, 0]]), np.zeros((3, 3), int), "P",
                               np.zeros((3, 3)), np.ones((3, 3), int), 2.0, 2)
    run_both(gpu, [tension(N=2, t=2.0), shear])


def test_cutback_driver(gpu):
    """An iteration limit of 8: increments that need more are cut back (3 and 2 times)
    and re-solved in sub-steps."""
    recs = run_both(gpu, [tension(rate=4e-3, t=2.0, N=2)], num_kw={"itmax": 8})
    assert [r["cutbacks"] for r in recs] == [3, 2]


def test_cutback_large_step(gpu):
    """5 % strain in one increment: two cut-backs and 218 NGMRES iterations.  The GPU and
    the oracle sum in different orders, and over that many iterations of a strongly
    nonlinear step the rounding differences grow to ~1e-8 in the averages (bound 1e-7
    here, same iteration and cut-back counts); the fields are compared in the milder
    cut-back case above."""
    recs = run_both(gpu, [tension(rate=5e-2, t=1.0, N=1)], tol=1e-7, fields=False)
    assert recs[0]["cutbacks"] == 2


def test_mixed_form_through_cutbacks(gpu):
    """The mixed form (FP32 spectra and Newton Jacobian, warm starts within a step)
    through the cut-back driver (iteration limit 8): the same cut-backs as the FP64 form
    and volume averages within 1e-5 of it; warm starts restart cold after every cut-back."""
    mat, q = synthetic.microstructure(CELLS, 5, 77)
    steps = [tension(rate=4e-3, t=2.0, N=2)]
    recs = {}
    for prec in ("fp64", "mixed"):
        rve = gpu.RVE(CELLS, (1.0, 1.0, 1.0), mat, q, num=gpu.numerics(itmax=8, precision=prec))
        recs[prec] = rve.loop_over_loadcase(steps)
    assert len(recs["fp64"]) == len(recs["mixed"]) == 2
    for a, b in zip(recs["fp64"], recs["mixed"]):
        assert a["cutbacks"] == b["cutbacks"]
        assert rel(b["P_av"], a["P_av"]) < 1e-5
        assert rel(b["F_av"], a["F_av"]) < 1e-5
