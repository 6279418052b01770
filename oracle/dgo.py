"""ctypes view of the CPU oracle (test infrastructure only).

The oracle is a plain-C FP64 restatement of the reference path; this module loads
``oracle/_build/libdgo.so`` (built by ``oracle/build.py``) and exposes numpy-facing
helpers.  Product code never imports it.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None

DERIV = {"continuous": 0, "central_difference": 1, "FWBW_difference": 2}
DIVCORR = {"none": 0, "size": 1, "size+grid": 2, "grid+size": 2}


class Material(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("C11", "C12", "C44", "xi_0", "xi_inf", "h_0", "n",
                                          "dot_gamma_0", "a", "c_1", "c_2")] + [
        ("h_sl_sl", C.c_double * 7), ("atol_xi", C.c_double), ("atol_gamma", C.c_double),
        ("r_cutback_min", C.c_double), ("r_cutback", C.c_double), ("r_increase", C.c_double),
        ("eps_rel_state", C.c_double), ("N_iter_state_max", C.c_int), ("N_iter_Lp_max", C.c_int),
        ("r_linesearch_Lp", C.c_double), ("eps_rel_Lp", C.c_double), ("eps_abs_Lp", C.c_double),
        ("f_update_jacobi_Lp", C.c_int)]


class Consts(C.Structure):
    _fields_ = [("P_sl", C.c_double * 108), ("h", C.c_double * 144), ("C66", C.c_double * 36),
                ("C", C.c_double * 81)]


class Points(C.Structure):
    _fields_ = [("n", C.c_int64)] + [(n, C.POINTER(C.c_double)) for n in (
        "F", "F0", "Fp", "Fp0", "Fi", "Fi0", "Fe", "Lp", "Lp0", "Li", "Li0", "S", "S0", "P",
        "xi", "xi0", "gamma", "gamma0", "dPdF")] + [("status", C.POINTER(C.c_int32))]


class Numerics(C.Structure):
    _fields_ = [("itmin", C.c_int), ("itmax", C.c_int), ("update_gamma", C.c_int),
                ("eps_abs_div", C.c_double), ("eps_rel_div", C.c_double), ("eps_abs_P", C.c_double),
                ("eps_rel_P", C.c_double), ("divergence_correction", C.c_int), ("derivative", C.c_int),
                ("stag_iter_max", C.c_int), ("max_cut_back", C.c_int), ("solver", C.c_int),
                ("ngmres_m", C.c_int), ("snes_max_it", C.c_int)]


class LoadStep(C.Structure):
    _fields_ = [("def_type", C.c_int), ("def_values", C.c_double * 9), ("def_mask", C.c_int * 9),
                ("stress_type", C.c_int), ("stress_values", C.c_double * 9), ("stress_mask", C.c_int * 9),
                ("rot_q", C.c_double * 4), ("t", C.c_double), ("N", C.c_int), ("r", C.c_double),
                ("estimate_rate", C.c_int), ("f_out", C.c_int)]


class IncRecord(C.Structure):
    _fields_ = [("t", C.c_double), ("dt", C.c_double), ("P_av", C.c_double * 9), ("F_aim", C.c_double * 9),
                ("F_av", C.c_double * 9), ("iterations", C.c_int), ("evaluations", C.c_int),
                ("converged", C.c_int), ("cutbacks", C.c_int), ("err_div", C.c_double), ("err_BC", C.c_double),
                ("seconds", C.c_double)]


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int)
        L.dgo_material_default.argtypes = [C.POINTER(Material)]
        L.dgo_consts_build.argtypes = [C.POINTER(Material), C.POINTER(Consts)]
        L.dgo_points_alloc.argtypes = [C.POINTER(Points), C.c_int64]
        L.dgo_points_free.argtypes = [C.POINTER(Points)]
        L.dgo_points_init.argtypes = [C.POINTER(Material), C.POINTER(Points), dp]
        L.dgo_points_commit.argtypes = [C.POINTER(Points)]
        L.dgo_constitutive_response.argtypes = [C.POINTER(Material), C.POINTER(Consts), C.POINTER(Points),
                                                dp, C.c_double, C.c_int, C.c_int]
        L.dgo_averages.argtypes = [C.c_int64, dp, dp, dp, dp, dp]
        L.dgo_qu2om.argtypes = [dp, dp]
        L.dgo_invert.argtypes = [C.c_int, dp, dp]
        L.dgo_rotate2.argtypes = [dp, dp, dp, C.c_int]
        L.dgo_rotate4.argtypes = [dp, dp, dp, C.c_int]
        L.dgo_fft_r2c.argtypes = [ip, C.c_int, dp, dp]
        L.dgo_fft_c2r.argtypes = [ip, C.c_int, dp, dp]
        L.dgo_xi.argtypes = [ip, dp, C.c_int, dp, dp]
        L.dgo_scaled_geom.argtypes = [ip, dp, C.c_int, dp]
        L.dgo_update_coords.argtypes = [ip, dp, C.c_int, dp, dp, dp]
        L.dgo_rotational_part.argtypes = [dp, dp]
        L.dgo_om2qu.argtypes = [dp, dp]
        L.dgo_orientation_output.argtypes = [dp, dp]
        L.dgo_divergence_rms_spec.argtypes = [ip, dp, dp, dp, dp]
        L.dgo_divergence_rms_spec.restype = C.c_double
        L.dgo_divergence_rms.argtypes = [ip, dp, dp, dp, dp]
        L.dgo_divergence_rms.restype = C.c_double
        L.dgo_gamma_convolution.argtypes = [ip, dp, dp, dp, dp]
        L.dgo_forward_field.argtypes = [C.c_int64, C.c_double, dp, dp, dp, dp]
        L.dgo_calculate_rate.argtypes = [C.c_int64, C.c_int, dp, dp, C.c_double, dp, dp]
        L.dgo_masked_compliance.argtypes = [dp, dp, ip, dp]
        L.dgo_mul3333xx33.argtypes = [dp, dp, dp]
        L.dgo_numerics_default.argtypes = [C.POINTER(Numerics)]
        L.dgo_solver_create.restype = vp
        L.dgo_solver_create.argtypes = [ip, dp, C.POINTER(C.c_int32), C.c_int, dp, C.POINTER(Material),
                                        C.POINTER(Numerics), C.c_int]
        L.dgo_solver_free.argtypes = [vp]
        L.dgo_solver_run.argtypes = [vp, C.c_int, C.POINTER(LoadStep), C.POINTER(IncRecord), C.c_int]
        L.dgo_solver_get.argtypes = [vp, C.c_char_p, dp]
        L.dgo_solver_total_evaluations.argtypes = [vp]
        L.dgo_solver_total_evaluations.restype = C.c_int64
        L.dgo_solver_init_state.argtypes = [vp]
        L.dgo_solver_forward.argtypes = [vp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                         C.POINTER(LoadStep)]
        L.dgo_solver_solve.argtypes = [vp, ip, ip]
        L.dgo_form_residual_bc.argtypes = [dp, dp, dp, ip, dp, dp, dp]
        L.dgo_form_residual_bc.restype = C.c_double
        L.dgo_counters.argtypes = [C.POINTER(C.c_int64)]
        L.dgo_counters_reset.argtypes = []
        _lib = L
    return _lib


def f64(a, shape=None):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
    return a if shape is None else a.reshape(shape)


def fortran9(a):
    """(..., 3, 3) numpy row-major matrices -> column-major flat 9-vectors."""
    a = np.asarray(a, dtype=np.float64)
    return np.ascontiguousarray(np.swapaxes(a, -1, -2).reshape(a.shape[:-2] + (9,)))


def from_fortran9(v):
    v = np.asarray(v)
    return np.swapaxes(v.reshape(v.shape[:-1] + (3, 3)), -1, -2)


def material(**kw):
    m = Material()
    lib().dgo_material_default(C.byref(m))
    for k, v in kw.items():
        if k == "h_sl_sl":
            for i, x in enumerate(v):
                m.h_sl_sl[i] = x
        else:
            setattr(m, k, v)
    return m


def numerics(**kw):
    n = Numerics()
    lib().dgo_numerics_default(C.byref(n))
    for k, v in kw.items():
        if k == "divergence_correction" and isinstance(v, str):
            v = DIVCORR[v]
        if k == "derivative" and isinstance(v, str):
            v = DERIV[v]
        setattr(n, k, v)
    return n


def consts(mat):
    c = Consts()
    lib().dgo_consts_build(C.byref(mat), C.byref(c))
    return c


class PointSet:
    """Material-point state held by the oracle (reference AoS layout)."""

    def __init__(self, mat, quats):
        q = f64(quats).reshape(-1, 4)
        self.mat = mat
        self.consts = consts(mat)
        self.pts = Points()
        lib().dgo_points_alloc(C.byref(self.pts), q.shape[0])
        lib().dgo_points_init(C.byref(mat), C.byref(self.pts), _p(q))
        self.n = q.shape[0]

    def __del__(self):
        try:
            lib().dgo_points_free(C.byref(self.pts))
        except Exception:
            pass

    def field(self, name, width=9):
        ptr = getattr(self.pts, name)
        return np.ctypeslib.as_array(ptr, shape=(self.n * width,)).reshape(self.n, width).copy()

    def set_field(self, name, values, width=9):
        ptr = getattr(self.pts, name)
        np.ctypeslib.as_array(ptr, shape=(self.n * width,))[:] = f64(values).ravel()

    def commit(self):
        lib().dgo_points_commit(C.byref(self.pts))

    def response(self, F9, dt, want_dPdF=True, nthreads=0):
        F9 = f64(F9).reshape(self.n, 9)
        ill = lib().dgo_constitutive_response(C.byref(self.mat), C.byref(self.consts), C.byref(self.pts),
                                              _p(F9), dt, int(want_dPdF), nthreads)
        return ill


def averages(P9, dPdF81):
    P9 = f64(P9)
    n = P9.size // 9
    P_av = np.zeros(9); Cv = np.zeros(81); Cm = np.zeros(81)
    d = f64(dPdF81) if dPdF81 is not None else None
    lib().dgo_averages(n, _p(P9), _p(d) if d is not None else None, _p(P_av), _p(Cv), _p(Cm))
    return P_av, Cv, Cm


def _cells(cells):
    return (C.c_int * 3)(*[int(c) for c in cells])


def fft_r2c(cells, field9):
    N0, N1, N2 = cells
    out = np.zeros((N1, N2, N0 // 2 + 1, 9), dtype=np.complex128)
    lib().dgo_fft_r2c(_cells(cells), 9, _p(f64(field9)), out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def fft_c2r(cells, spec):
    N0, N1, N2 = cells
    spec = np.ascontiguousarray(spec, dtype=np.complex128)
    out = np.zeros(9 * N0 * N1 * N2)
    lib().dgo_fft_c2r(_cells(cells), 9, spec.ctypes.data_as(C.POINTER(C.c_double)), _p(out))
    return out


def xi(cells, geom, derivative=0):
    N0, N1, N2 = cells
    x1 = np.zeros((N1, N2, N0 // 2 + 1, 3), dtype=np.complex128)
    x2 = np.zeros_like(x1)
    lib().dgo_xi(_cells(cells), _p(f64(geom)), int(derivative),
                 x1.ctypes.data_as(C.POINTER(C.c_double)), x2.ctypes.data_as(C.POINTER(C.c_double)))
    return x1, x2


def update_coords(cells, geom, F9, derivative=0):
    """(u_n (nodes, 3), u_p (cells, 3)) of the F field (N, 9 column-major)."""
    N0, N1, N2 = cells
    un = np.zeros(((N0 + 1) * (N1 + 1) * (N2 + 1), 3))
    up = np.zeros((N0 * N1 * N2, 3))
    F9 = np.ascontiguousarray(F9, dtype=np.float64)
    lib().dgo_update_coords(_cells(cells), _p(f64(geom)), int(derivative), _p(F9), _p(un), _p(up))
    return un, up


def orientation_output(Fe9):
    """Quaternions (N, 4) written as the crystal orientation O for elastic deformation gradients (N, 9)."""
    Fe9 = np.ascontiguousarray(np.asarray(Fe9, dtype=np.float64).reshape(-1, 9))
    out = np.zeros((Fe9.shape[0], 4))
    for k in range(Fe9.shape[0]):
        lib().dgo_orientation_output(_p(Fe9[k]), _p(out[k]))
    return out


def scaled_geom(cells, geom, divcorr):
    out = np.zeros(3)
    if isinstance(divcorr, str):
        divcorr = DIVCORR[divcorr]
    lib().dgo_scaled_geom(_cells(cells), _p(f64(geom)), int(divcorr), _p(out))
    return out


def divergence_rms(cells, geom, scaled, xi1st, P9):
    xi1st = np.ascontiguousarray(xi1st, dtype=np.complex128)
    return lib().dgo_divergence_rms(_cells(cells), _p(f64(geom)), _p(f64(scaled)),
                                    xi1st.ctypes.data_as(C.POINTER(C.c_double)), _p(f64(P9)))


def gamma_convolution(cells, xi1st, C_ref81, aim9, field9):
    xi1st = np.ascontiguousarray(xi1st, dtype=np.complex128)
    f = f64(field9).copy()
    lib().dgo_gamma_convolution(_cells(cells), xi1st.ctypes.data_as(C.POINTER(C.c_double)),
                                _p(f64(C_ref81)), _p(f64(aim9)), _p(f))
    return f


def forward_field(dt, last9, rate9, aim9=None):
    last9 = f64(last9); out = np.zeros_like(last9)
    lib().dgo_forward_field(last9.size // 9, dt, _p(last9), _p(f64(rate9)),
                            _p(f64(aim9)) if aim9 is not None else None, _p(out))
    return out


def calculate_rate(heterogeneous, field0, field, dt, avRate9):
    field = f64(field); out = np.zeros_like(field)
    lib().dgo_calculate_rate(field.size // 9, int(heterogeneous), _p(f64(field0)), _p(field), dt,
                             _p(f64(avRate9)), _p(out))
    return out


def masked_compliance(C81, q, mask9):
    out = np.zeros(81)
    m = (C.c_int * 9)(*[int(x) for x in mask9])
    lib().dgo_masked_compliance(_p(f64(C81)), _p(f64(q)), m, _p(out))
    return out


def form_residual_bc(S81, P_av9, P_aim9, mask9, q, F_aim9):
    F_aim = f64(F_aim9).copy(); rot = np.zeros(9)
    m = (C.c_int * 9)(*[int(x) for x in mask9])
    err = lib().dgo_form_residual_bc(_p(f64(S81)), _p(f64(P_av9)), _p(f64(P_aim9)), m, _p(f64(q)),
                                     _p(F_aim), _p(rot))
    return err, F_aim, rot


def qu2om(q):
    out = np.zeros(9)
    lib().dgo_qu2om(_p(f64(q)), _p(out))
    return out


def loadstep(kind="tensionX", t=20.0, N=20, rate=1e-3, f_out=1, r=1.0, estimate_rate=1, rot=(1, 0, 0, 0)):
    """Build a load step: 'tensionX|Y|Z' (uniaxial, other normal P = 0) or 'shearXY'."""
    ls = LoadStep()
    ls.def_type = 1
    ls.stress_type = 0
    ax = {"tensionX": 0, "tensionY": 1, "tensionZ": 2}
    defv = np.zeros((3, 3)); defm = np.zeros((3, 3), dtype=int)
    strv = np.zeros((3, 3)); strm = np.ones((3, 3), dtype=int)
    if kind in ax:
        a = ax[kind]
        defv[a, a] = rate
        for i in range(3):
            for j in range(3):
                if i == j and i != a:
                    defm[i, j] = 1          # 'x': free
                    strm[i, j] = 0          # P prescribed 0
    elif kind == "shearXY":
        defv[0, 1] = rate
    else:
        raise ValueError(kind)
    for k, (i, j) in enumerate([(i, j) for j in range(3) for i in range(3)]):
        ls.def_values[k] = defv[i, j]; ls.def_mask[k] = int(defm[i, j])
        ls.stress_values[k] = strv[i, j]; ls.stress_mask[k] = int(strm[i, j])
    for k in range(4):
        ls.rot_q[k] = rot[k]
    ls.t = t; ls.N = N; ls.r = r; ls.estimate_rate = estimate_rate; ls.f_out = f_out
    return ls


class Solver:
    """Whole-solver oracle run (DamaskGrid::loop_over_loadcase)."""

    def __init__(self, cells, geom, material_at, orientations, mat=None, num=None, nthreads=0):
        self.cells = tuple(int(c) for c in cells)
        self.mat = mat if mat is not None else material()
        self.num = num if num is not None else numerics()
        ma = np.ascontiguousarray(np.asarray(material_at, dtype=np.int32).ravel())
        q = f64(orientations).reshape(-1, 4)
        self._keep = (ma, q)
        self.h = lib().dgo_solver_create(_cells(cells), _p(f64(geom)), ma.ctypes.data_as(C.POINTER(C.c_int32)),
                                         q.shape[0], _p(q), C.byref(self.mat), C.byref(self.num), nthreads)
        self.N = int(np.prod(self.cells))

    def __del__(self):
        try:
            lib().dgo_solver_free(self.h)
        except Exception:
            pass

    def run(self, steps, max_records=10000):
        arr = (LoadStep * len(steps))(*steps)
        recs = (IncRecord * max_records)()
        n = lib().dgo_solver_run(self.h, len(steps), arr, recs, max_records)
        if n < 0:
            raise RuntimeError(f"oracle: no solution found at increment {-n}")
        out = []
        for r in recs[:n]:
            out.append(dict(t=r.t, dt=r.dt, P_av=np.array(r.P_av[:]), F_aim=np.array(r.F_aim[:]),
                            F_av=np.array(r.F_av[:]), iterations=r.iterations, evaluations=r.evaluations,
                            cutbacks=r.cutbacks, err_div=r.err_div, err_BC=r.err_BC, seconds=r.seconds))
        return out

    def get(self, name):
        width = {"xi": 12, "gamma": 12, "dPdF": 81, "P_av": 9, "F_aim": 9, "C_volAvg": 81,
                 "C_minMaxAvg": 81, "C_ref": 81, "S_compliance": 81}.get(name, 9)
        per_point = name not in ("P_av", "F_aim", "C_volAvg", "C_minMaxAvg", "C_ref", "S_compliance")
        out = np.zeros(width * (self.N if per_point else 1))
        lib().dgo_solver_get(self.h, name.encode(), _p(out))
        return out.reshape(self.N, width) if per_point else out

    @property
    def evaluations(self):
        return lib().dgo_solver_total_evaluations(self.h)


def counters():
    a = (C.c_int64 * 4)()
    lib().dgo_counters(a)
    return dict(evaluations=a[0], state_iterations=a[1], lp_iterations=a[2], tangents=a[3])


def counters_reset():
    lib().dgo_counters_reset()
