"""GB300-native DAMASK_grid spectral-basic solver (phenopowerlaw cF) -- host API.

Thin Python view of the C ABI (include/dgx.h, libdgx.so).  Method names follow
the reference's operator surface: ``Spectral::constitutive_response``,
``MechBase::calculate_divergence_rms`` / ``gamma_convolution`` / ``update_gamma``,
``MechSolverBasic::init`` / ``forward`` / ``calculate_solution`` and
``DamaskGrid::loop_over_loadcase`` (reference src/grid/*.cpp).  All tensors use
the reference layout: (N, 3, 3) per cell with numpy row/column meaning [i][j],
cells ordered x fastest.
"""
import ctypes as C

import numpy as np

from . import dgx as _d
from .dgx import DgxError  # noqa: F401
from .loadcase import load_step, parse_load_yaml, parse_numerics_yaml  # noqa: F401

__all__ = ["RVE", "Batch", "Server", "footprint", "material", "numerics", "load_step", "vti_read", "DgxError"]


def material(**kw):
    m = _d.Material()
    _d.lib().dgx_material_default(C.byref(m))
    for k, v in kw.items():
        if k == "h_sl_sl":
            for i, x in enumerate(v):
                m.h_sl_sl[i] = float(x)
        else:
            setattr(m, k, v)
    return m


def numerics(**kw):
    n = _d.Numerics()
    _d.lib().dgx_numerics_default(C.byref(n))
    names = {"none": 0, "size": 1, "size+grid": 2, "grid+size": 2,
             "continuous": 0, "central_difference": 1, "FWBW_difference": 2,
             "ngmres": 0, "fixed_point": 1, "fp64": 0, "mixed": 1}
    for k, v in kw.items():
        if isinstance(v, str):
            v = names[v]
        setattr(n, k, v)
    return n


def _f9(a):
    """(N,3,3) numpy -> reference (3,3,N) column-major flat array."""
    a = np.asarray(a, dtype=np.float64)
    return np.ascontiguousarray(np.swapaxes(a, -1, -2)).reshape(-1)


def _unf9(v, n):
    return np.swapaxes(np.asarray(v).reshape(n, 3, 3), -1, -2)


class RVE:
    """One representative volume element resident on the current CUDA device."""

    def __init__(self, cells, size, material_at, orientations, mat=None, num=None):
        L = _d.lib()
        self.cells = tuple(int(c) for c in cells)
        self.N = int(np.prod(self.cells))
        ma = np.ascontiguousarray(np.asarray(material_at, dtype=np.int32).ravel())
        if ma.size != self.N:
            raise ValueError("material_at must have N0*N1*N2 entries")
        q = np.ascontiguousarray(np.asarray(orientations, dtype=np.float64).reshape(-1, 4))
        self.mat = mat if mat is not None else material()
        self.num = num if num is not None else numerics()
        h = C.c_void_p()
        cells_c = (C.c_int32 * 3)(*self.cells)
        size_c = (C.c_double * 3)(*[float(s) for s in size])
        _d.check(L.dgx_rve_create(cells_c, size_c, ma.ctypes.data_as(C.POINTER(C.c_int32)), q.shape[0],
                                  _d.dptr(q), C.byref(self.mat), C.byref(self.num), C.byref(h)), "dgx_rve_create")
        self.h = h
        self.size = tuple(float(s) for s in size)

    def close(self):
        if getattr(self, "h", None):
            _d.lib().dgx_rve_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def device_bytes(self):
        return int(_d.lib().dgx_rve_device_bytes(self.h))

    # ------------------------------------------------------------ reference operators
    def constitutive_response(self, F, dt, want_dPdF=False):
        """Spectral::constitutive_response for F (N,3,3): returns P (N,3,3) [, dPdF (N,3,3,3,3)]."""
        F9 = _f9(F)
        P = np.zeros(9 * self.N)
        dP = np.zeros(81 * self.N) if want_dPdF else None
        ill = C.c_int32(0)
        _d.check(_d.lib().dgx_constitutive_response(self.h, _d.dptr(F9), float(dt), 0, self.N, _d.dptr(P),
                                                    _d.dptr(dP) if dP is not None else None, C.byref(ill)),
                 "dgx_constitutive_response")
        self.terminally_ill = bool(ill.value)
        Pn = _unf9(P, self.N)
        if want_dPdF:
            d = dP.reshape(self.N, 3, 3, 3, 3, order="C")
            # flat index i + 3j + 9k + 27l per cell -> array [cell][l][k][j][i]
            return Pn, np.transpose(d, (0, 4, 3, 2, 1))
        return Pn

    def fields(self, with_dPdF=False):
        """Library-owned device fields in the reference layout (dgx_fields): dict of
        device pointers F0, F, P, dPdF (0 if not requested), terminally_ill, the stream
        and the cell count n."""
        fp = _d.FieldPtrs()
        _d.check(_d.lib().dgx_fields(self.h, int(bool(with_dPdF)), C.byref(fp)), "dgx_fields")
        return dict(n=fp.n, F0=fp.F0 or 0, F=fp.F or 0, P=fp.P or 0, dPdF=fp.dPdF or 0,
                    terminally_ill=fp.terminally_ill or 0, stream=fp.stream or 0)

    def constitutive_response_fields(self, dt, want_dPdF=False):
        """Constitutive response of the exported device field F in place
        (dgx_constitutive_response_fields); results in the exported P / dPdF."""
        _d.check(_d.lib().dgx_constitutive_response_fields(self.h, float(dt), 0, self.N, int(bool(want_dPdF))),
                 "dgx_constitutive_response_fields")

    def averages(self):
        P = np.zeros(9); Cv = np.zeros(81); Cm = np.zeros(81)
        _d.check(_d.lib().dgx_averages(self.h, _d.dptr(P), _d.dptr(Cv), _d.dptr(Cm)), "dgx_averages")
        return (_unf9(P, 1)[0], Cv.reshape(3, 3, 3, 3, order="F"), Cm.reshape(3, 3, 3, 3, order="F"))

    def commit(self):
        _d.check(_d.lib().dgx_commit_increment(self.h), "dgx_commit_increment")

    def calculate_divergence_rms(self, P):
        r = C.c_double(0.0)
        P9 = _f9(P)
        _d.check(_d.lib().dgx_divergence_rms(self.h, _d.dptr(P9), C.byref(r)), "dgx_divergence_rms")
        return r.value

    def update_gamma(self, C4):
        c = np.ascontiguousarray(np.asarray(C4, dtype=np.float64).reshape(3, 3, 3, 3).ravel(order="F"))
        _d.check(_d.lib().dgx_update_gamma(self.h, _d.dptr(c)), "dgx_update_gamma")

    def gamma_convolution(self, field, aim):
        f = _f9(field).copy()
        a = _f9(np.asarray(aim).reshape(1, 3, 3))
        _d.check(_d.lib().dgx_gamma_convolution(self.h, _d.dptr(f), _d.dptr(a)), "dgx_gamma_convolution")
        return _unf9(f, self.N)

    def fft_forward(self, field):
        """FFT<5>::forward: (N,3,3) -> complex (N1, N2, N0//2+1, 3, 3) in the transposed-out order."""
        N0, N1, N2 = self.cells
        out = np.zeros(2 * 9 * (N0 // 2 + 1) * N1 * N2)
        f = _f9(field)
        _d.check(_d.lib().dgx_fft_forward(self.h, _d.dptr(f), _d.dptr(out)), "dgx_fft_forward")
        z = out[0::2] + 1j * out[1::2]
        z = z.reshape(N1, N2, N0 // 2 + 1, 9)
        return np.swapaxes(z.reshape(N1, N2, N0 // 2 + 1, 3, 3), -1, -2)

    def init(self):
        """MechSolverBasic::init: F = I, constitutive response at dt = 0, C_ref."""
        _d.check(_d.lib().dgx_solver_init(self.h), "dgx_solver_init")

    def forward(self, cutback, guess, dt, dt_old, t_remaining, step):
        _d.check(_d.lib().dgx_solver_forward(self.h, int(cutback), int(guess), float(dt), float(dt_old),
                                             float(t_remaining), C.byref(step)), "dgx_solver_forward")

    def calculate_solution(self):
        conv = C.c_int32(0); it = C.c_int32(0); ill = C.c_int32(0)
        _d.check(_d.lib().dgx_solver_solve(self.h, C.byref(conv), C.byref(it), C.byref(ill)), "dgx_solver_solve")
        return dict(converged=bool(conv.value), required_iterations=it.value, terminally_ill=bool(ill.value))

    def loop_over_loadcase(self, steps, max_records=100000, result=None, restart=None, restart_every=0,
                           phase="phase", homogenization="SX", setup=None):
        """DamaskGrid::loop_over_loadcase from solver init.  result: DADF5 file written
        at increment 0 and every f_out-th increment; restart: restart file rewritten
        every restart_every increments; setup: {name: text} stored under /setup."""
        arr = (_d.LoadStep * len(steps))(*steps)
        nrec = sum(int(s.N) for s in steps)
        recs = (_d.IncRecord * max(1, min(nrec, max_records)))()
        n = C.c_int32(0)
        L = _d.lib()
        if result is None and restart is None:
            _d.check(L.dgx_run_loadcase(self.h, len(steps), arr, recs, len(recs), C.byref(n)), "dgx_run_loadcase")
            return [_record(r) for r in recs[:n.value]]
        res = C.c_void_p()
        if result is not None:
            _d.check(L.dgx_result_open(str(result).encode(), self.h, phase.encode(), homogenization.encode(),
                                       C.byref(res)), "dgx_result_open")
            for name, text in (setup or {}).items():
                t = text.encode()
                _d.check(L.dgx_result_add_setup(res, name.encode(), t, len(t)), "dgx_result_add_setup")
        try:
            _d.check(L.dgx_run_loadcase_output(self.h, len(steps), arr, recs, len(recs), C.byref(n), res,
                                               str(restart).encode() if restart else None, int(restart_every)),
                     "dgx_run_loadcase_output")
        finally:
            if res:
                _d.check(L.dgx_result_close(res), "dgx_result_close")
        return [_record(r) for r in recs[:n.value]]

    def write_restart(self, path):
        _d.check(_d.lib().dgx_restart_write(self.h, str(path).encode()), "dgx_restart_write")

    def read_restart(self, path):
        """Continue from a restart file written by an RVE created with the same inputs."""
        _d.check(_d.lib().dgx_restart_read(self.h, str(path).encode()), "dgx_restart_read")

    def run_increment(self, step, step_index, inc):
        rec = _d.IncRecord()
        _d.check(_d.lib().dgx_run_increment(self.h, C.byref(step), int(step_index), int(inc), C.byref(rec)),
                 "dgx_run_increment")
        return _record(rec)

    def update_coords(self):
        """MechSolverBasic::update_coords: (u_n (nodes, 3), u_p (cells, 3)) displacements."""
        N0, N1, N2 = self.cells
        un = np.zeros(3 * (N0 + 1) * (N1 + 1) * (N2 + 1))
        up = np.zeros(3 * self.N)
        _d.check(_d.lib().dgx_update_coords(self.h, _d.dptr(un), _d.dptr(up)), "dgx_update_coords")
        return un.reshape(-1, 3), up.reshape(-1, 3)

    def get(self, name, out=None):
        """A field (N, 3, 3) / (N, 12) or a volume quantity.  `out`: optional host buffer
        of the field's size (float64, C-contiguous; e.g. pinned memory) to read into."""
        width = {"xi": 12, "gamma": 12}.get(name, 9)
        scalars = {"P_av": 9, "F_aim": 9, "C_volAvg": 81, "C_minMaxAvg": 81, "C_ref": 81, "S_compliance": 81}
        if name in scalars:
            out = np.zeros(scalars[name])
            _d.check(_d.lib().dgx_get(self.h, name.encode(), _d.dptr(out)), "dgx_get")
            return _unf9(out, 1)[0] if scalars[name] == 9 else out.reshape(3, 3, 3, 3, order="F")
        if out is None:
            out = np.empty(width * self.N)
        else:
            out = out.reshape(-1)
            if out.dtype != np.float64 or out.size != width * self.N or not out.flags.c_contiguous:
                raise ValueError(f"dgx_get {name}: out must be {width * self.N} contiguous float64")
        _d.check(_d.lib().dgx_get(self.h, name.encode(), _d.dptr(out)), "dgx_get")
        return _unf9(out, self.N) if width == 9 else out.reshape(self.N, width)

    def counters(self):
        a = (C.c_int64 * 10)()
        _d.check(_d.lib().dgx_counters(self.h, a), "dgx_counters")
        return dict(evaluations=a[0], state_iterations=a[1], lp_iterations=a[2], tangents=a[3], launches=a[4],
                    jacobians=a[5], h2d_bytes=a[6], d2h_bytes=a[7], fpi_iterations=a[8], graph_rounds=a[9])

    def timers(self):
        ms = (C.c_double * 3)(); n = (C.c_int64 * 3)()
        _d.check(_d.lib().dgx_timers(self.h, ms, n), "dgx_timers")
        return dict(constitutive_ms=ms[0], spectral_ms=ms[1], tangent_ms=ms[2], constitutive_launches=n[0],
                    spectral_launches=n[1], tangent_launches=n[2])

    @property
    def stream(self):
        """cudaStream_t of this RVE (as an int), e.g. for torch.cuda.ExternalStream."""
        return int(_d.lib().dgx_rve_stream(self.h) or 0)


def _record(r):
    return dict(t=r.t, dt=r.dt, P_av=_unf9(np.array(r.P_av[:]), 1)[0], F_aim=_unf9(np.array(r.F_aim[:]), 1)[0],
                F_av=_unf9(np.array(r.F_av[:]), 1)[0], iterations=r.iterations, evaluations=r.evaluations,
                cutbacks=r.cutbacks, err_div=r.err_div, err_BC=r.err_BC, seconds=r.seconds)


class Batch:
    """Many RVEs advanced together on one stream (dgx_batch_*).

    ``add(rve, steps)`` makes the RVE run the load case from solver init, like
    ``RVE.loop_over_loadcase``; ``step()`` runs one round (every member's pending
    residual evaluation or reduction in batched launches); ``run()`` rounds until
    all members are done.  Members can be added between rounds.
    """

    def __init__(self, capacity, cons_block=0):
        h = C.c_void_p()
        _d.check(_d.lib().dgx_batch_create(int(capacity), int(cons_block), C.byref(h)), "dgx_batch_create")
        self.h = h
        self._keep = {}          # slot -> (rve, steps array, records array)

    def close(self):
        if getattr(self, "h", None):
            _d.lib().dgx_batch_destroy(self.h)
            self.h = None
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, rve, steps, max_records=None):
        arr = (_d.LoadStep * len(steps))(*steps)
        nrec = sum(int(s.N) for s in steps)
        recs = (_d.IncRecord * max(1, nrec if max_records is None else min(nrec, max_records)))()
        slot = C.c_int32(0)
        _d.check(_d.lib().dgx_batch_add(self.h, rve.h, len(steps), arr, recs, len(recs), C.byref(slot)),
                 "dgx_batch_add")
        self._keep[slot.value] = (rve, arr, recs)
        return slot.value

    def step(self):
        n = C.c_int32(0)
        _d.check(_d.lib().dgx_batch_step(self.h, C.byref(n)), "dgx_batch_step")
        return n.value

    def run(self):
        _d.check(_d.lib().dgx_batch_run(self.h), "dgx_batch_run")

    def member(self, slot):
        done = C.c_int32(0); n = C.c_int32(0); st = C.c_int32(0)
        _d.check(_d.lib().dgx_batch_member(self.h, int(slot), C.byref(done), C.byref(n), C.byref(st)),
                 "dgx_batch_member")
        return dict(done=bool(done.value), n_records=n.value, status=st.value)

    def records(self, slot):
        m = self.member(slot)
        recs = self._keep[slot][2]
        return [_record(r) for r in recs[:m["n_records"]]]

    def remove(self, slot):
        _d.check(_d.lib().dgx_batch_remove(self.h, int(slot)), "dgx_batch_remove")
        self._keep.pop(slot, None)

    def stats(self):
        ms = (C.c_double * 3)(); a = (C.c_int64 * 10)()
        _d.check(_d.lib().dgx_batch_stats(self.h, ms, a), "dgx_batch_stats")
        return dict(constitutive_ms=ms[0], spectral_ms=ms[1], round_device_ms=ms[2], point_evaluations=a[0],
                    state_iterations=a[1], lp_iterations=a[2], rounds=a[3], launches=a[4], jacobians=a[5],
                    h2d_bytes=a[6], d2h_bytes=a[7], fpi_iterations=a[8], graph_rounds=a[9])

    def host_times(self):
        """Host wall time of the rounds (dgx_batch_host_times): plan / wait / results / advance, ms."""
        ms = (C.c_double * 4)()
        _d.check(_d.lib().dgx_batch_host_times(self.h, ms), "dgx_batch_host_times")
        return dict(plan_issue=ms[0], wait=ms[1], results=ms[2], advance=ms[3])

    def set_round_points(self, points):
        """Cap the residual evaluations per round (cells); 0 serves every request."""
        _d.check(_d.lib().dgx_batch_set_round_points(self.h, int(points)), "dgx_batch_set_round_points")

    def tuning(self):
        a = (C.c_int32 * 4)()
        _d.check(_d.lib().dgx_batch_tuning(self.h, a), "dgx_batch_tuning")
        return dict(cons_block=a[0], tuned_grids=a[1], blocks_per_sm=a[2], tuning_block=a[0] == 0,
                    tuning_tiles=bool(a[3]))

    @property
    def stream(self):
        return int(_d.lib().dgx_batch_stream(self.h) or 0)


def vti_read(content, label="material"):
    """(cells, size, origin, dataset) of VTI content through the library's reader
    (dgx_vti_read_cells_size_origin / dgx_vti_read_dataset_int; host only)."""
    b = content.encode() if isinstance(content, str) else bytes(content)
    cells = (C.c_int32 * 3)(); size = (C.c_double * 3)(); origin = (C.c_double * 3)()
    _d.check(_d.lib().dgx_vti_read_cells_size_origin(b, len(b), cells, size, origin), "dgx_vti_read_cells_size_origin")
    n = C.c_int64(cells[0] * cells[1] * cells[2])
    data = np.zeros(n.value, dtype=np.int32)
    lb = label.encode()
    _d.check(_d.lib().dgx_vti_read_dataset_int(b, len(b), lb, len(lb), data.ctypes.data_as(C.POINTER(C.c_int32)),
                                               C.byref(n)), "dgx_vti_read_dataset_int")
    return np.array(cells[:]), np.array(size[:]), np.array(origin[:]), data[:n.value]


def flop_model():
    """FP64 flops per counted unit of the constitutive kernel (dgx_flop_model)."""
    a = (C.c_double * 4)()
    _d.lib().dgx_flop_model(a)
    return dict(lp=a[0], jacobian=a[1], state=a[2], fpi=a[3])


def flop_model_mixed():
    """FP64 and FP32 flops per counted unit of the mixed-precision constitutive form
    (dgx_flop_model_mixed): ({lp, jacobian, state, fpi} FP64, the same FP32)."""
    a = (C.c_double * 4)()
    b = (C.c_double * 4)()
    _d.lib().dgx_flop_model_mixed(a, b)
    keys = ("lp", "jacobian", "state", "fpi")
    return dict(zip(keys, a)), dict(zip(keys, b))


def footprint(cells, num=None, n_materials=1):
    """Device bytes an RVE of this grid and numerics holds (dgx_rve_footprint)."""
    b = C.c_int64(0)
    num = num if num is not None else numerics()
    _d.check(_d.lib().dgx_rve_footprint((C.c_int32 * 3)(*[int(c) for c in cells]), C.byref(num), int(n_materials),
                                        C.byref(b)), "dgx_rve_footprint")
    return int(b.value)


class Server:
    """Continuous-batching service of RVE solves (dgx_server_*).

    ``submit`` queues a solve (inputs are copied) and returns its id; the worker
    thread admits requests in arrival order as batch slots and HBM budget free up,
    runs them together and frees each one's memory when it is done.  ``result``
    waits for a request and returns its status and per-increment records.
    """

    STATES = ("queued", "running", "done", "failed")

    def __init__(self, hbm_budget_bytes=0, max_active=64, cons_block=0, round_points=None):
        h = C.c_void_p()
        _d.check(_d.lib().dgx_server_create(int(hbm_budget_bytes), int(max_active), int(cons_block), C.byref(h)),
                 "dgx_server_create")
        self.h = h
        if round_points is not None:
            _d.check(_d.lib().dgx_server_set_round_points(h, int(round_points)), "dgx_server_set_round_points")

    def close(self):
        if getattr(self, "h", None):
            _d.lib().dgx_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, cells, size, material_at, orientations, steps, mat=None, num=None):
        ma = np.ascontiguousarray(np.asarray(material_at, dtype=np.int32).ravel())
        q = np.ascontiguousarray(np.asarray(orientations, dtype=np.float64).reshape(-1, 4))
        arr = (_d.LoadStep * len(steps))(*steps)
        req = _d.Request()
        for i in range(3):
            req.cells[i] = int(cells[i]); req.size[i] = float(size[i])
        req.material_at = ma.ctypes.data_as(C.POINTER(C.c_int32))
        req.n_materials = q.shape[0]
        req.orientations = _d.dptr(q)
        req.material = mat if mat is not None else material()
        req.numerics = num if num is not None else numerics()
        req.nsteps = len(steps)
        req.steps = arr
        rid = C.c_int64(0)
        _d.check(_d.lib().dgx_server_submit(self.h, C.byref(req), C.byref(rid)), "dgx_server_submit")
        return int(rid.value)

    def status(self, rid, wait=0.0, max_records=0):
        st = _d.RequestStatus()
        recs = (_d.IncRecord * max(1, max_records))()
        _d.check(_d.lib().dgx_server_poll(self.h, int(rid), float(wait), C.byref(st), recs, int(max_records)),
                 "dgx_server_poll")
        out = dict(state=self.STATES[st.state], status=st.status, n_records=st.n_records, t_submit=st.t_submit,
                   t_admit=st.t_admit, t_done=st.t_done, device_bytes=st.device_bytes, points=st.points,
                   error=st.error.decode(errors="replace"))
        if max_records and st.state == 2:
            out["records"] = [_record(r) for r in recs[:min(st.n_records, max_records)]]
        return out

    def result(self, rid, timeout=3600.0, max_records=100000):
        """Wait for the request; its status with the records."""
        st = self.status(rid, wait=timeout, max_records=max_records)
        if st["state"] not in ("done", "failed"):
            raise TimeoutError(f"request {rid} not finished after {timeout} s")
        return st

    def release(self, rid):
        _d.check(_d.lib().dgx_server_release(self.h, int(rid)), "dgx_server_release")

    def stats(self):
        i = _d.ServerInfo()
        _d.check(_d.lib().dgx_server_stats(self.h, C.byref(i)), "dgx_server_stats")
        return dict(queued=i.queued, running=i.running, completed=i.completed, failed=i.failed, rounds=i.rounds,
                    budget_bytes=i.budget_bytes, used_bytes=i.used_bytes, now=i.now, status=i.status)
