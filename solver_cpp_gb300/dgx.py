"""ctypes binding of the C ABI in include/dgx.h (libdgx.so, built in tree).

The library is the product: there is no CPU fallback.  If the shared library is
missing or no CUDA device is present, the calls raise.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libdgx.so")

_lib = None


class Material(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("C11", "C12", "C44", "xi_0", "xi_inf", "h_0", "n",
                                          "dot_gamma_0", "a", "c_1", "c_2")] + [
        ("h_sl_sl", C.c_double * 7), ("atol_xi", C.c_double), ("atol_gamma", C.c_double),
        ("r_cutback_min", C.c_double), ("r_cutback", C.c_double), ("r_increase", C.c_double),
        ("eps_rel_state", C.c_double), ("N_iter_state_max", C.c_int32), ("N_iter_Lp_max", C.c_int32),
        ("r_linesearch_Lp", C.c_double), ("eps_rel_Lp", C.c_double), ("eps_abs_Lp", C.c_double),
        ("f_update_jacobi_Lp", C.c_int32)]


class Numerics(C.Structure):
    _fields_ = [("itmin", C.c_int32), ("itmax", C.c_int32), ("update_gamma", C.c_int32),
                ("eps_abs_div", C.c_double), ("eps_rel_div", C.c_double), ("eps_abs_P", C.c_double),
                ("eps_rel_P", C.c_double), ("divergence_correction", C.c_int32), ("derivative", C.c_int32),
                ("stag_iter_max", C.c_int32), ("max_cut_back", C.c_int32), ("solver", C.c_int32),
                ("ngmres_m", C.c_int32), ("snes_max_it", C.c_int32), ("precision", C.c_int32),
                ("lazy_tangent", C.c_int32)]


class LoadStep(C.Structure):
    _fields_ = [("def_type", C.c_int32), ("def_values", C.c_double * 9), ("def_mask", C.c_int32 * 9),
                ("stress_type", C.c_int32), ("stress_values", C.c_double * 9), ("stress_mask", C.c_int32 * 9),
                ("rot_q", C.c_double * 4), ("t", C.c_double), ("N", C.c_int32), ("r", C.c_double),
                ("estimate_rate", C.c_int32), ("f_out", C.c_int32)]


class IncRecord(C.Structure):
    _fields_ = [("t", C.c_double), ("dt", C.c_double), ("P_av", C.c_double * 9), ("F_aim", C.c_double * 9),
                ("F_av", C.c_double * 9), ("iterations", C.c_int32), ("evaluations", C.c_int32),
                ("converged", C.c_int32), ("cutbacks", C.c_int32), ("err_div", C.c_double),
                ("err_BC", C.c_double), ("seconds", C.c_double)]


class Request(C.Structure):
    _fields_ = [("cells", C.c_int32 * 3), ("size", C.c_double * 3), ("material_at", C.POINTER(C.c_int32)),
                ("n_materials", C.c_int32), ("orientations", C.POINTER(C.c_double)), ("material", Material),
                ("numerics", Numerics), ("nsteps", C.c_int32), ("steps", C.POINTER(LoadStep))]


class RequestStatus(C.Structure):
    _fields_ = [("state", C.c_int32), ("status", C.c_int32), ("n_records", C.c_int32), ("t_submit", C.c_double),
                ("t_admit", C.c_double), ("t_done", C.c_double), ("device_bytes", C.c_int64),
                ("points", C.c_int64), ("error", C.c_char * 160)]


class ServerInfo(C.Structure):
    _fields_ = [("queued", C.c_int32), ("running", C.c_int32), ("completed", C.c_int64), ("failed", C.c_int64),
                ("rounds", C.c_int64), ("budget_bytes", C.c_int64), ("used_bytes", C.c_int64), ("now", C.c_double),
                ("status", C.c_int32)]


SYMBOLS = ["dgx_material_default", "dgx_numerics_default", "dgx_rve_create", "dgx_rve_destroy", "dgx_last_error",
           "dgx_rve_points", "dgx_rve_device_bytes", "dgx_constitutive_response", "dgx_averages",
           "dgx_commit_increment", "dgx_divergence_rms", "dgx_gamma_convolution", "dgx_update_gamma",
           "dgx_fft_forward", "dgx_solver_init", "dgx_solver_forward", "dgx_solver_solve", "dgx_run_loadcase",
           "dgx_run_increment", "dgx_get", "dgx_counters", "dgx_timers", "dgx_rve_stream",
           "dgx_measure_fp64_peak", "dgx_divergence_rms_static", "dgx_batch_create", "dgx_batch_destroy",
           "dgx_batch_add", "dgx_batch_step", "dgx_batch_run", "dgx_batch_member", "dgx_batch_remove",
           "dgx_batch_stats", "dgx_batch_stream", "dgx_rve_footprint", "dgx_server_create", "dgx_server_destroy",
           "dgx_server_submit", "dgx_server_poll", "dgx_server_release", "dgx_server_stats",
           "dgx_update_coords", "dgx_result_open", "dgx_result_add_setup", "dgx_result_write_increment",
           "dgx_result_close", "dgx_restart_write", "dgx_restart_read", "dgx_run_loadcase_output", "dgx_batch_tuning", "dgx_flop_model", "dgx_flop_model_mixed",
           "dgx_batch_set_round_points",
           "dgx_server_set_round_points", "dgx_device_math", "dgx_fields", "dgx_constitutive_response_fields",
           "dgx_vti_read_cells_size_origin", "dgx_vti_read_dataset_int", "dgx_batch_host_times"]


class FieldPtrs(C.Structure):
    _fields_ = [("n", C.c_int64), ("F0", C.c_void_p), ("F", C.c_void_p), ("P", C.c_void_p), ("dPdF", C.c_void_p),
                ("terminally_ill", C.c_void_p), ("stream", C.c_void_p)]


class DgxError(RuntimeError):
    pass


def lib():
    """Load libdgx.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise DgxError(f"{LIB_PATH} is missing: run solver_cpp_gb300.build.build() first")
    L = C.CDLL(LIB_PATH)
    dp, ip, i64p = C.POINTER(C.c_double), C.POINTER(C.c_int32), C.POINTER(C.c_int64)
    vp = C.c_void_p
    L.dgx_material_default.argtypes = [C.POINTER(Material)]
    L.dgx_material_default.restype = None
    L.dgx_numerics_default.argtypes = [C.POINTER(Numerics)]
    L.dgx_numerics_default.restype = None
    L.dgx_rve_create.argtypes = [ip, dp, ip, C.c_int32, dp, C.POINTER(Material), C.POINTER(Numerics), C.POINTER(vp)]
    L.dgx_rve_destroy.argtypes = [vp]
    L.dgx_rve_destroy.restype = None
    L.dgx_last_error.restype = C.c_char_p
    L.dgx_rve_points.argtypes = [vp]
    L.dgx_rve_points.restype = C.c_int64
    L.dgx_rve_device_bytes.argtypes = [vp]
    L.dgx_rve_device_bytes.restype = C.c_int64
    L.dgx_constitutive_response.argtypes = [vp, dp, C.c_double, C.c_int32, C.c_int32, dp, dp, ip]
    L.dgx_averages.argtypes = [vp, dp, dp, dp]
    L.dgx_commit_increment.argtypes = [vp]
    L.dgx_divergence_rms.argtypes = [vp, dp, dp]
    L.dgx_gamma_convolution.argtypes = [vp, dp, dp]
    L.dgx_update_gamma.argtypes = [vp, dp]
    L.dgx_fft_forward.argtypes = [vp, dp, dp]
    L.dgx_solver_init.argtypes = [vp]
    L.dgx_solver_forward.argtypes = [vp, C.c_int32, C.c_int32, C.c_double, C.c_double, C.c_double, C.POINTER(LoadStep)]
    L.dgx_solver_solve.argtypes = [vp, ip, ip, ip]
    L.dgx_run_loadcase.argtypes = [vp, C.c_int32, C.POINTER(LoadStep), C.POINTER(IncRecord), C.c_int32, ip]
    L.dgx_run_increment.argtypes = [vp, C.POINTER(LoadStep), C.c_int32, C.c_int32, C.POINTER(IncRecord)]
    L.dgx_get.argtypes = [vp, C.c_char_p, dp]
    L.dgx_counters.argtypes = [vp, i64p]
    L.dgx_timers.argtypes = [vp, dp, i64p]
    L.dgx_rve_stream.argtypes = [vp]
    L.dgx_rve_stream.restype = vp
    L.dgx_measure_fp64_peak.argtypes = [dp, dp]
    L.dgx_device_math.argtypes = [C.c_int32, C.c_int64, dp, dp]
    L.dgx_batch_create.argtypes = [C.c_int32, C.c_int32, C.POINTER(vp)]
    L.dgx_batch_destroy.argtypes = [vp]
    L.dgx_batch_destroy.restype = None
    L.dgx_batch_add.argtypes = [vp, vp, C.c_int32, C.POINTER(LoadStep), C.POINTER(IncRecord), C.c_int32, ip]
    L.dgx_batch_step.argtypes = [vp, ip]
    L.dgx_batch_run.argtypes = [vp]
    L.dgx_batch_member.argtypes = [vp, C.c_int32, ip, ip, ip]
    L.dgx_batch_remove.argtypes = [vp, C.c_int32]
    L.dgx_batch_stats.argtypes = [vp, dp, C.POINTER(C.c_int64)]
    L.dgx_batch_stream.argtypes = [vp]
    L.dgx_batch_stream.restype = vp
    L.dgx_update_coords.argtypes = [vp, dp, dp]
    L.dgx_batch_tuning.argtypes = [vp, ip]
    L.dgx_flop_model.argtypes = [dp]
    L.dgx_batch_set_round_points.argtypes = [vp, C.c_int64]
    L.dgx_server_set_round_points.argtypes = [vp, C.c_int64]
    L.dgx_flop_model.restype = None
    L.dgx_flop_model_mixed.argtypes = [dp, dp]
    L.dgx_result_open.argtypes = [C.c_char_p, vp, C.c_char_p, C.c_char_p, C.POINTER(vp)]
    L.dgx_result_add_setup.argtypes = [vp, C.c_char_p, C.c_char_p, C.c_int64]
    L.dgx_result_write_increment.argtypes = [vp, vp, C.c_int32, C.c_double]
    L.dgx_result_close.argtypes = [vp]
    L.dgx_restart_write.argtypes = [vp, C.c_char_p]
    L.dgx_restart_read.argtypes = [vp, C.c_char_p]
    L.dgx_run_loadcase_output.argtypes = [vp, C.c_int32, C.POINTER(LoadStep), C.POINTER(IncRecord), C.c_int32, ip, vp,
                                          C.c_char_p, C.c_int32]
    L.dgx_rve_footprint.argtypes = [ip, C.POINTER(Numerics), C.c_int32, i64p]
    L.dgx_server_create.argtypes = [C.c_int64, C.c_int32, C.c_int32, C.POINTER(vp)]
    L.dgx_server_destroy.argtypes = [vp]
    L.dgx_server_destroy.restype = None
    L.dgx_server_submit.argtypes = [vp, C.POINTER(Request), i64p]
    L.dgx_server_poll.argtypes = [vp, C.c_int64, C.c_double, C.POINTER(RequestStatus), C.POINTER(IncRecord),
                                  C.c_int32]
    L.dgx_server_release.argtypes = [vp, C.c_int64]
    L.dgx_server_stats.argtypes = [vp, C.POINTER(ServerInfo)]
    L.dgx_divergence_rms_static.argtypes = [ip, dp, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]
    L.dgx_fields.argtypes = [vp, C.c_int32, C.POINTER(FieldPtrs)]
    L.dgx_batch_host_times.argtypes = [vp, dp]
    L.dgx_constitutive_response_fields.argtypes = [vp, C.c_double, C.c_int32, C.c_int32, C.c_int32]
    L.dgx_vti_read_cells_size_origin.argtypes = [C.c_char_p, C.c_int64, ip, dp, dp]
    L.dgx_vti_read_dataset_int.argtypes = [C.c_char_p, C.c_int64, C.c_char_p, C.c_int32, ip, i64p]
    for name in SYMBOLS:
        f = getattr(L, name)
        if name not in ("dgx_material_default", "dgx_numerics_default", "dgx_rve_destroy", "dgx_last_error",
                        "dgx_rve_points", "dgx_rve_device_bytes", "dgx_rve_stream", "dgx_batch_destroy",
                        "dgx_batch_stream", "dgx_server_destroy", "dgx_flop_model", "dgx_flop_model_mixed"):
            f.restype = C.c_int32
    _lib = L
    return L


def check(status, what=""):
    if status != 0:
        msg = lib().dgx_last_error().decode(errors="replace")
        raise DgxError(f"{what} failed ({status}): {msg}")


def dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))
