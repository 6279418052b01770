#!/usr/bin/env python
"""Point-updates/s of the DAMASK_grid spectral-basic solver (phenopowerlaw cF) on GB300.

Workload (the plain-FP64 GPU configuration of the benchmark definition): 64^3 cells,
200 grains from a seeded periodic Voronoi tessellation with uniformly random
orientations, single-phase cF phenopowerlaw (C11 106.75 GPa, C12 60.41 GPa,
C44 28.34 GPa, xi_0 31 MPa, xi_inf 63 MPa, h_0 75 MPa, n 20, dot_gamma_0 1e-3/s,
a 2.25, h_sl-sl [1,1,1.4,1.4,1.4,1.4,1.4]), uniaxial tension in x (dot_F_xx =
1e-3/s, P_yy = P_zz = 0), 40 increments over 40 s, FP64 end to end.

One "step" is one load increment (a full NGMRES solve of the increment).
The point-update is one material point's constitutive evaluation plus its share
of one residual evaluation (FFT -> div-RMS/Gamma -> iFFT, reductions, NGMRES
vector work): value = N_cells x (residual evaluations) / time.

  value  : K increments, state resident in HBM, timed with CUDA events on the
           solver's stream (state + NGMRES history ~1.3 GB >> 129 MB L2).
  e2e    : the same through the public C ABI with every increment's result
           fields (P and F, 2 x 9N doubles) copied to host memory inside the
           timed region; byte counts are the library's own copy counters.
  --impl reference : the CPU oracle (plain-C restatement of the reference path,
           all host threads) on the same workload; the reference itself cannot
           be built on this image (Fortran/PETSc/FFTW toolchain absent).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "point-updates/s, mixed vs FP64 GPU at ≤1e-5 rel. P error; p50/p99 RVE latency"
UNIT = "point-updates/s"
SEED = 42

# DRAM traffic of one constitutive launch per cell, from an ncu capture of this
# workload (dram__bytes_read.sum + dram__bytes_write.sum of the 41st launch / 262,144
# cells: 0.152 + 0.249 GB = 0.401 GB; profiles/constitutive_64cube.md)
TRAFFIC_BYTES_PER_CELL = 1530.0


def args_():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--cells", type=int, default=64)
    p.add_argument("--grains", type=int, default=200)
    p.add_argument("--increments", type=int, default=40)
    p.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    p.add_argument("--no-extras", action="store_true", help="skip e2e / mixed / CPU-baseline legs")
    p.add_argument("--cpu-sample-increments", type=int, default=2,
                   help="increments of the CPU oracle sample (also the mixed form's error against the oracle)")
    p.add_argument("--batch-rves", type=int, default=256, help="RVEs of the batched leg (0: skip)")
    p.add_argument("--batch-seconds", type=float, default=300.0,
                   help="safety bound of each batched run (runs end when every member is done)")
    p.add_argument("--batch-compare", type=int, default=64, help="RVEs of the batched-vs-one-at-a-time comparison")
    p.add_argument("--no-mixed-large", action="store_true",
                   help="skip the 128^3 / 1000-grain tension-then-shear configuration (both forms, ~1 min)")
    p.add_argument("--serve-requests", type=int, default=12, help="requests of each serving leg (0: skip)")
    p.add_argument("--serve-rates", default="5,20,50,200", help="Poisson arrival rates of the sweep (requests/s)")
    p.add_argument("--serve-seconds", type=float, default=60.0, help="time bound of each serving leg")
    return p.parse_args()


def workload(a):
    from solver_cpp_gb300.synthetic import microstructure
    cells = (a.cells, a.cells, a.cells)
    mat_at, q = microstructure(cells, a.grains, SEED)
    return cells, (1.0, 1.0, 1.0), mat_at, q


def config(a):
    return {"workload": f"{a.cells}^3 cells, {a.grains} Voronoi grains (seed {SEED}), phenopowerlaw cF, "
                        f"tension x 1e-3/s, {a.increments} increments over {float(a.increments):g} s",
            "cells": a.cells, "grains": a.grains, "increments": a.increments, "step": "one load increment",
            "precision": a.precision, "solver": "NGMRES (PETSc SNESNGMRES defaults)",
            "l2": "inputs larger than L2 (resident state + NGMRES history > 1 GB)"}


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))


def max_over_ranks(ms, device):
    """The timed region's milliseconds, maximum over all ranks: N independent replicas
    finish when the slowest does, so the job's value is all ranks' units over this."""
    import torch
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------- CPU oracle timing
def oracle_increments(a, count, threads):
    """Run `count` increments of the workload on the CPU oracle (load case restarted
    from a fresh solve every `a.increments` increments); per-increment records."""
    from oracle import dgo
    cells, size, mat_at, q = workload(a)
    recs = []
    while len(recs) < count:
        take = min(a.increments, count - len(recs))
        s = dgo.Solver(cells, size, mat_at, q, nthreads=threads)
        recs += s.run([dgo.loadstep("tensionX", t=float(take), N=take)])
    return recs


def cpu_oracle_sample(a, increments, threads):
    cells, _, _, _ = workload(a)
    n = cells[0] * cells[1] * cells[2]
    recs = oracle_increments(a, increments, threads)
    dt = sum(r["seconds"] for r in recs)
    ev = sum(r["evaluations"] for r in recs)
    return n * ev / dt, dt, ev, recs


def from_fortran9(v):
    """reference (3,3) column-major 9 values -> 3x3 numpy [i][j]"""
    import numpy as np
    return np.asarray(v).reshape(3, 3).T


def cpu_one_core_sample(a):
    """One residual evaluation of the workload on one host core with the CPU oracle:
    the constitutive response of every cell at the first iteration's deformation
    (F = I + dot_F dt), the divergence RMS and the Gamma convolution (each with its own
    forward FFT, as the reference does).  Point-updates/s = cells / time."""
    import numpy as np
    from oracle import dgo
    cells, size, mat_at, q = workload(a)
    n = cells[0] * cells[1] * cells[2]
    mat = dgo.material()
    ps = dgo.PointSet(mat, np.asarray(q)[np.asarray(mat_at)])
    F = np.tile(np.eye(3).ravel(order="F"), (n, 1))
    F[:, 0] += 1e-3
    x1, _ = dgo.xi(cells, size)
    sc = dgo.scaled_geom(cells, size, 0)
    C11, C12, C44 = mat.C11, mat.C12, mat.C44
    Cref = np.zeros(81)
    for i in range(3):
        for j in range(3):
            for k in range(3):
                for l in range(3):
                    v = C12 * (i == j) * (k == l) + C44 * ((i == k) * (j == l) + (i == l) * (j == k))
                    v += (C11 - C12 - 2 * C44) * (i == j == k == l)
                    Cref[i + 3 * j + 9 * k + 27 * l] = v
    t0 = time.perf_counter()
    ps.response(F, 1.0, want_dPdF=False, nthreads=1)
    P = ps.field("P")
    dgo.divergence_rms(cells, size, sc, x1, P)
    dgo.gamma_convolution(cells, x1, Cref, np.zeros(9), P)
    dt = time.perf_counter() - t0
    return n / dt, dt


def reference_arm(a):
    rank, world = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    cells, _, _, _ = workload(a)
    n = cells[0] * cells[1] * cells[2]
    recs = oracle_increments(a, a.warmup + a.steps, threads)
    timed = recs[a.warmup:]
    total_t = sum(r["seconds"] for r in timed)
    total_ev = sum(r["evaluations"] for r in timed)
    value = n * total_ev / total_t if total_t > 0 else 0.0
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": a.gpus,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * total_t / max(1, a.steps),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Voronoi + uniform SO(3) orientations)", "config": config(a),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{a.steps} increments of the {a.cells}^3 workload after {a.warmup} warm-up "
                                       "increments (CPU oracle, OpenMP over cells; reference not buildable here)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- clocks sampling
class Clocks:
    def __init__(self):
        self.samples = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0],
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        sm = [float(s[0]) for s in self.samples if s and s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if len(s) > 1 and s[1].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            for k, nm in enumerate(names):
                if len(s) > 4 + k and s[4 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


# ---------------------------------------------------------------- GPU arm
BATCH_KINDS = ("tensionX", "tensionY", "tensionZ", "shearXY")   # as solver_cpp_gb300.synthetic


def batch_population(count, seed=1000):
    """RVEs of the batched configuration: grid uniform in {8,16,32,48}^3, 8-200
    grains, load case uniform in tension x/y/z and shear xy (1e-3/s), per-RVE seeds."""
    from solver_cpp_gb300 import synthetic
    return synthetic.batch_population(count, seed)


def _pct(v, p):
    import numpy as np
    return float(np.percentile(v, p)) if len(v) else None


def _run_batch(g, torch, pop, precision, increments, seconds):
    """One batch over the population in the given form, run until every member is done
    (or `seconds` pass): CUDA-event time on the batch's stream, per-member completion
    times (wall clock from the first round) and per-increment latencies."""
    num = g.numerics(precision=precision)
    steps = {k: [g.load_step(k, t=float(increments), N=increments)] for k in BATCH_KINDS}
    batch = g.Batch(len(pop))
    rves = []
    for cells, ng, kind, mat, q in pop:
        r = g.RVE(cells, (1.0, 1.0, 1.0), mat, q, num=num)
        rves.append((r, batch.add(r, steps[kind])))
    st = torch.cuda.ExternalStream(batch.stream)
    s0 = batch.stats()
    e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(st)
    t_start = time.perf_counter()
    pending = {slot for _, slot in rves}
    done_at = {}
    active = 1
    t_in_step = 0.0
    while active and time.perf_counter() - t_start < seconds:
        ts = time.perf_counter()
        active = batch.step()
        t_in_step += time.perf_counter() - ts
        now = time.perf_counter() - t_start
        for slot in list(pending):
            if batch.member(slot)["done"]:
                done_at[slot] = now
                pending.discard(slot)
    e1.record(st)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    s1 = batch.stats()
    inc_lat, recs = [], {}
    for r, slot in rves:
        recs[slot] = batch.records(slot)
        inc_lat += [x["seconds"] for x in recs[slot]]
    comp = sorted(done_at.values())
    out = {"value": (s1["point_evaluations"] - s0["point_evaluations"]) / (ms * 1e-3), "unit": UNIT,
           "precision": precision, "rves": len(pop), "points": int(sum(r.N for r, _ in rves)),
           "increments": increments, "rounds": s1["rounds"] - s0["rounds"], "seconds": ms * 1e-3,
           "all_done": not active, "completed": len(comp),
           "p50_rve_completion_s": _pct(comp, 50), "p99_rve_completion_s": _pct(comp, 99),
           "p50_increment_ms": 1e3 * _pct(inc_lat, 50) if inc_lat else None,
           "p99_increment_ms": 1e3 * _pct(inc_lat, 99) if inc_lat else None,
           "constitutive_share": (s1["constitutive_ms"] - s0["constitutive_ms"]) / ms,
           "spectral_share": (s1["spectral_ms"] - s0["spectral_ms"]) / ms,
           "round_device_share": (s1["round_device_ms"] - s0["round_device_ms"]) / ms,
           "graph_rounds": s1["graph_rounds"] - s0["graph_rounds"],
           "host_ms": batch.host_times(), "wall_in_step_s": t_in_step,
           "launches": s1["launches"] - s0["launches"], "autotuned": batch.tuning()}
    batch.close()
    for r, _ in rves:
        r.close()
    return out, [recs[slot] for _, slot in rves]


def _max_err(recs_a, recs_b):
    err = 0.0
    for ra, rb in zip(recs_a, recs_b):
        for a_, b_ in zip(ra, rb):
            err = max(err, float(abs(a_["P_av"] - b_["P_av"]).max() / abs(b_["P_av"]).max()))
    return err


def batch_leg(g, torch, n_rves, increments, seconds, compare):
    """The batched configuration to completion in the mixed form and in FP64 (equal work:
    the same population, load cases and increments), and the first `compare` RVEs solved
    one at a time in plain FP64 (the drop-in's use) against the same RVEs batched mixed,
    both timed with CUDA events."""
    pop = batch_population(n_rves)
    mixed, recs_m = _run_batch(g, torch, pop, "mixed", increments, seconds)
    fp64, recs_f = _run_batch(g, torch, pop, "fp64", increments, seconds)
    out = {"mixed": mixed, "fp64": fp64, "value": mixed["value"], "unit": UNIT,
           "mixed_vs_fp64_batched": mixed["value"] / fp64["value"] if fp64["value"] else None,
           "max_rel_P_av_error_mixed_vs_fp64": _max_err(recs_m, recs_f)}
    if compare:
        sub = pop[:compare]
        plain = g.numerics(precision="fp64")
        steps = {k: g.load_step(k, t=float(increments), N=increments) for k in BATCH_KINDS}
        ref_recs, ms_seq, pts_seq = [], 0.0, 0
        e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
        for cells, ng, kind, mat, q in sub:
            r = g.RVE(cells, (1.0, 1.0, 1.0), mat, q, num=plain)
            st = torch.cuda.ExternalStream(r.stream)
            r.init()
            c0 = r.counters()
            torch.cuda.synchronize()
            e0.record(st)
            recs = [r.run_increment(steps[kind], 0, i) for i in range(increments)]
            e1.record(st)
            torch.cuda.synchronize()
            ms_seq += e0.elapsed_time(e1)
            pts_seq += r.N * (r.counters()["evaluations"] - c0["evaluations"])
            ref_recs.append(recs)
            r.close()
        bm, recs_b = _run_batch(g, torch, sub, "mixed", increments, seconds)
        seq = pts_seq / (ms_seq * 1e-3)
        out["vs_plain_fp64_one_at_a_time"] = {
            "rves": compare, "increments": increments, "plain_fp64_one_at_a_time": seq,
            "batched_mixed": bm["value"], "speedup": bm["value"] / seq,
            "max_rel_P_av_error_vs_fp64": _max_err(recs_b, ref_recs),
            "timing": "CUDA events on each solver's stream (one at a time: sum over the RVEs' solves)"}
    return out


def mixed_large_leg(g, torch, cells=128, grains=1000, inc_each=30):
    """The mixed-precision configuration: 128^3 cells, 1000 grains, tension x then
    shear xy (1e-3/s, 30 increments each).  The same load case in plain FP64 on the GPU
    is the reference for the per-increment error of the volume-averaged P."""
    from solver_cpp_gb300.synthetic import microstructure
    c3 = (cells, cells, cells)
    mat_at, q = microstructure(c3, grains, SEED + 1)
    steps = [g.load_step("tensionX", t=float(inc_each), N=inc_each),
             g.load_step("shearXY", t=float(inc_each), N=inc_each)]
    out = {"workload": f"{cells}^3 cells, {grains} grains (seed {SEED + 1}), tension x then shear xy, "
                       f"{inc_each} + {inc_each} increments"}
    recs = {}
    for prec in ("mixed", "fp64"):       # FP64 last: its converged field gives the divergence noise floor
        rve = g.RVE(c3, (1.0, 1.0, 1.0), mat_at, q, num=g.numerics(precision=prec))
        st = torch.cuda.ExternalStream(rve.stream)
        e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(st)
        recs[prec] = rve.loop_over_loadcase(steps)
        e1.record(st)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        ev = rve.counters()["evaluations"]
        lat = [x["seconds"] for x in recs[prec]]
        out[prec] = {"value": rve.N * ev / (ms * 1e-3), "unit": UNIT, "seconds": ms * 1e-3, "evaluations": ev,
                     "p50_increment_ms": 1e3 * _pct(lat, 50), "p99_increment_ms": 1e3 * _pct(lat, 99)}
        if prec == "fp64":
            # FP32-spectrum noise floor of the divergence test: the divergence RMS of the
            # converged FP64 stress field with FP64 and with FP32 spectra, against divTol
            P = rve.get("P")
            rms64 = rve.calculate_divergence_rms(P)
            rve.close()
            r32 = g.RVE(c3, (1.0, 1.0, 1.0), mat_at, q, num=g.numerics(precision="mixed"))
            rms32 = r32.calculate_divergence_rms(P)
            r32.close()
            num = g.numerics()
            div_tol = max(float(abs(recs[prec][-1]["P_av"]).max()) * num.eps_rel_div, num.eps_abs_div)
            out["divergence_fp32_noise_over_divTol"] = abs(rms32 - rms64) / div_tol
            out["err_div_over_divTol_at_convergence"] = {
                p_: max(float(r["err_div"]) / max(float(abs(r["P_av"]).max()) * num.eps_rel_div, num.eps_abs_div)
                        for r in recs[p_]) for p_ in recs}
        else:
            rve.close()
    errs = [float(abs(a["P_av"] - b["P_av"]).max() / abs(b["P_av"]).max()) for a, b in zip(recs["mixed"], recs["fp64"])]
    out["max_rel_P_av_error_vs_fp64"] = max(errs)
    out["per_increment_error"] = errs
    out["error_reference"] = ("the GPU FP64 form of the same load case (itself within 1e-8 of the CPU oracle in the "
                              "parity tests at 16^3 and 64^3; the oracle needs minutes per 128^3 increment)")
    return out


SERVE_SIZES = (16, 32, 64, 96)


def serve_leg(g, precision, rate, n_requests, seconds, seed=5000):
    """Poisson arrivals (rate req/s) of RVE solve requests: grid uniform in
    {16,32,64,96}^3, 10-500 grains, load case uniform in tension x/y/z and shear xy
    (1e-3/s), 10-40 increments.  Requests are submitted at their arrival times from
    this thread while the server's worker runs; reports per-increment and
    per-request latency and the aggregate point-updates/s of the window."""
    import numpy as np
    from solver_cpp_gb300 import synthetic
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, n_requests)
    reqs = []
    for k in range(n_requests):
        c = int(SERVE_SIZES[rng.integers(len(SERVE_SIZES))])
        ng = int(rng.integers(10, 501))
        kind = BATCH_KINDS[rng.integers(len(BATCH_KINDS))]
        n_inc = int(rng.integers(10, 41))
        mat, q = synthetic.microstructure((c, c, c), ng, seed + k)
        reqs.append(((c, c, c), mat, q, [g.load_step(kind, t=float(n_inc), N=n_inc)]))
    num = g.numerics(precision=precision)
    srv = g.Server(max_active=64)
    ids, t0 = [], time.perf_counter()
    due = t0
    for gap, (cells, mat, q, steps) in zip(gaps, reqs):
        due += gap
        d = due - time.perf_counter()
        if d > 0:
            time.sleep(d)
        ids.append(srv.submit(cells, (1.0, 1.0, 1.0), mat, q, steps, num=num))
    deadline = t0 + seconds
    done, inc_lat, req_lat, evals = [], [], [], 0
    for rid, (cells, _, _, _) in zip(ids, reqs):
        st = srv.status(rid, wait=max(0.0, deadline - time.perf_counter()), max_records=64)
        if st["state"] != "done":
            continue
        done.append(rid)
        req_lat.append(st["t_done"] - st["t_submit"])
        for r in st["records"]:
            inc_lat.append(r["seconds"])
            evals += r["evaluations"] * cells[0] * cells[1] * cells[2]
    window = time.perf_counter() - t0
    info = srv.stats()
    srv.close()

    def pct(v, p):
        return float(np.percentile(v, p)) if v else None
    return {"precision": precision, "rate_req_per_s": rate, "requests": n_requests, "completed": len(done),
            "window_s": window, "value": evals / window, "unit": UNIT,
            "p50_increment_ms": 1e3 * pct(inc_lat, 50) if inc_lat else None,
            "p99_increment_ms": 1e3 * pct(inc_lat, 99) if inc_lat else None,
            "p50_request_s": pct(req_lat, 50), "p99_request_s": pct(req_lat, 99), "rounds": info["rounds"],
            "note": "value counts the completed requests' point-updates over the whole window (wall clock)"}


def spectral_roofline(cells, precision, ms, fp64_peak):
    """FFT / Gamma / div-RMS chain of one residual evaluation against both ceilings.
    bytes: read P and write R (9N FP64 each) plus the spectrum traffic between the five
    passes (x out, y in/out, z in/out, y in/out, x in: 8 x 9 Nh complex of the spectral
    precision).  flops: 5 n log2 n per complex line FFT (forward and inverse; along x
    two real lines share one complex FFT), ~230 per frequency for Gamma and the
    divergence sum, ~8 per frequency to separate and join the packed x lines."""
    import math
    N0, N1, N2 = cells
    N, N0r = N0 * N1 * N2, N0 // 2 + 1
    Nh = N0r * N1 * N2
    cs = 16 if precision == "fp64" else 8
    bytes_ = 2 * 9 * N * 8 + 8 * 9 * Nh * cs
    fl = 2 * 5 * 9 * (N1 * N2 * N0 * math.log2(N0) / 2 + N0r * N2 * N1 * math.log2(N1) + N0r * N1 * N2 * math.log2(N2))
    fl += 230 * Nh + 8 * 9 * Nh
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    gbs = bytes_ / (ms * 1e-3) / 1e9
    tfs = fl / (ms * 1e-3) / 1e12
    return {"bound": "fp64" if precision == "fp64" else "hbm", "bytes_per_residual": bytes_,
            "achieved_gbs": gbs, "peak_gbs": hbm, "frac_hbm": gbs / hbm,
            "peak_source_hbm": "measured (MEASURED_PEAKS.json)" if "hbm_gbs" in peaks else "fallback",
            "flops_per_residual": fl, "achieved_tflops": tfs,
            "frac_fp64": tfs / fp64_peak if fp64_peak else None}


def run_increments(rve, step, start, count, n_inc, read_back=None, records=None):
    """Run `count` increments starting at global index `start` (load case cycled);
    read_back: host buffers (P, F) the fields are copied into after every increment."""
    lat = []
    for i in range(start, start + count):
        inc = i % n_inc
        if inc == 0:
            rve.init()
        t0 = time.perf_counter()
        rec = rve.run_increment(step, 0, inc)
        if records is not None:
            records.append(rec)
        if read_back is not None:
            rve.get("P", out=read_back[0]); rve.get("F", out=read_back[1])
        lat.append(time.perf_counter() - t0)
    return lat


def gpu_arm(a):
    import torch
    rank, world = dist_env()
    if world > 1:
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import ctypes as C
    import solver_cpp_gb300 as g
    from solver_cpp_gb300 import build, dgx
    build.build()
    cells, size, mat_at, q = workload(a)
    n = cells[0] * cells[1] * cells[2]
    num = g.numerics(precision=a.precision)
    step = g.load_step("tensionX", t=float(a.increments), N=a.increments)

    peak = C.c_double(0.0)
    dgx.check(dgx.lib().dgx_measure_fp64_peak(C.byref(peak), None), "fp64 peak")

    rve = g.RVE(cells, size, mat_at, q, num=num)
    stream = torch.cuda.ExternalStream(rve.stream)
    run_increments(rve, step, 0, a.warmup, a.increments)
    c0, t0 = rve.counters(), rve.timers()
    e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
    clocks = Clocks(); clocks.start()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    e0.record(stream)
    lat = run_increments(rve, step, a.warmup, a.steps, a.increments)
    e1.record(stream)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ck = clocks.stop()
    ms = e0.elapsed_time(e1)
    c1, t1 = rve.counters(), rve.timers()
    if world > 1:
        ms = max_over_ranks(ms, "cuda")
    evals = c1["evaluations"] - c0["evaluations"]
    value = n * evals * world / (ms * 1e-3)
    # roofline of the dominant kernel (constitutive, FP64-bound)
    d_lp = c1["lp_iterations"] - c0["lp_iterations"]
    d_jac = c1["jacobians"] - c0["jacobians"]
    d_st = c1["state_iterations"] - c0["state_iterations"]
    launches = t1["constitutive_launches"] - t0["constitutive_launches"]
    kms = t1["constitutive_ms"] - t0["constitutive_ms"]
    d_fpi = c1["fpi_iterations"] - c0["fpi_iterations"]
    fm = g.flop_model()          # algorithmic FP64 flops per counted unit (FMA = 2), from the library
    flops = fm["lp"] * d_lp + fm["jacobian"] * d_jac + fm["state"] * d_st + fm["fpi"] * d_fpi
    achieved = flops / (kms * 1e-3) / 1e12 if kms > 0 else 0.0
    traffic = TRAFFIC_BYTES_PER_CELL * n if TRAFFIC_BYTES_PER_CELL else None
    spec_ms = t1["spectral_ms"] - t0["spectral_ms"]
    spec_n = t1["spectral_launches"] - t0["spectral_launches"]
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": ms / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if a.precision == "fp64" else "f64+f32", "data": "synthetic (seeded Voronoi + uniform "
            "SO(3) orientations; inputs generated in-process)", "config": config(a),
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak.value, "unit": "TFLOP/s",
                         "frac": achieved / peak.value if peak.value else None, "traffic": traffic,
                         "kernel": "k_constitutive", "flops_per_launch": flops / max(1, launches),
                         "units_per_evaluation": {k: v / max(1, evals * n) for k, v in
                                                  (("lp", d_lp), ("jacobian", d_jac), ("state", d_st),
                                                   ("fpi", d_fpi))},
                         "ms_per_launch": kms / max(1, launches),
                         "peak_source": "measured: dgx_measure_fp64_peak DFMA probe (MEASURED_PEAKS.json has no FP64)"},
            "kernel_time_share": {"constitutive": kms / ms, "spectral": spec_ms / ms,
                                  "tangent": (t1["tangent_ms"] - t0["tangent_ms"]) / ms,
                                  "spectral_ms_per_residual": spec_ms / max(1, spec_n),
                                  "tangent_ms_per_launch": (t1["tangent_ms"] - t0["tangent_ms"]) /
                                                           max(1, t1["tangent_launches"] - t0["tangent_launches"])},
            "roofline_spectral": spectral_roofline(cells, a.precision, spec_ms / max(1, spec_n), peak.value),
            "evaluations_per_increment": evals / a.steps,
            "latency": {"p50_increment_ms": 1e3 * statistics.median(lat),
                        "p99_increment_ms": 1e3 * sorted(lat)[min(len(lat) - 1, int(0.99 * len(lat)))]},
            "gpu_launches": c1["launches"] - c0["launches"], "clocks": ck}
    rve.close()
    if not a.no_extras and rank == 0:
        # e2e through the public API with results read back to host each increment
        rve2 = g.RVE(cells, size, mat_at, q, num=num)
        host = [torch.empty(9 * n, dtype=torch.float64, pin_memory=True).numpy() for _ in range(2)]
        run_increments(rve2, step, 0, a.warmup, a.increments, read_back=host)
        c0 = rve2.counters()
        t_e = time.perf_counter()
        run_increments(rve2, step, a.warmup, a.steps, a.increments, read_back=host)
        t_e = time.perf_counter() - t_e
        c1 = rve2.counters()
        rve2.close()
        line["e2e"] = {"value": n * (c1["evaluations"] - c0["evaluations"]) / t_e, "unit": UNIT,
                       "h2d_bytes_per_step": (c1["h2d_bytes"] - c0["h2d_bytes"]) / a.steps,
                       "d2h_bytes_per_step": (c1["d2h_bytes"] - c0["d2h_bytes"]) / a.steps,
                       "note": "public C-ABI increments, P and F fields copied every step into pinned host "
                               "buffers (AoS, transposed on the device)"}
        # both forms over the whole load case of the workload (solver init and all
        # increments, CUDA events on each solver's stream); P_av error of the mixed form
        # per increment against the FP64 run, and against the CPU oracle for the
        # increments of the oracle sample (below)
        recs = {}
        if a.precision == "fp64":
            vals, secs = {}, {}
            for prec in ("fp64", "mixed"):
                r2 = g.RVE(cells, size, mat_at, q, num=g.numerics(precision=prec))
                st2 = torch.cuda.ExternalStream(r2.stream)
                torch.cuda.synchronize()
                c0, tm0 = r2.counters(), r2.timers()
                e0.record(st2)
                out = []
                run_increments(r2, step, 0, a.increments, a.increments, records=out)
                e1.record(st2)
                torch.cuda.synchronize()
                c1, tm1 = r2.counters(), r2.timers()
                ms2 = e0.elapsed_time(e1)
                vals[prec] = n * (c1["evaluations"] - c0["evaluations"]) / (ms2 * 1e-3)
                secs[prec] = ms2 * 1e-3
                recs[prec] = out
                if prec == "mixed":
                    kms_m = tm1["constitutive_ms"] - tm0["constitutive_ms"]
                    nl_m = max(1, tm1["constitutive_launches"] - tm0["constitutive_launches"])
                    f64, f32 = g.flop_model_mixed()
                    units = {"lp": c1["lp_iterations"] - c0["lp_iterations"],
                             "jacobian": c1["jacobians"] - c0["jacobians"],
                             "state": c1["state_iterations"] - c0["state_iterations"],
                             "fpi": c1["fpi_iterations"] - c0["fpi_iterations"]}
                    fl64 = sum(f64[k] * v for k, v in units.items())
                    fl32 = sum(f32[k] * v for k, v in units.items())
                    ach = fl64 / (kms_m * 1e-3) / 1e12 if kms_m > 0 else 0.0
                    mixed_roof = {"bound": "fp64", "kernel": "k_constitutive (mixed form)",
                                  "ms_per_launch": kms_m / nl_m, "achieved": ach, "peak": peak.value,
                                  "unit": "TFLOP/s", "frac": ach / peak.value if peak.value else None,
                                  "fp64_flops_per_launch": fl64 / nl_m, "fp32_flops_per_launch": fl32 / nl_m,
                                  "units_per_evaluation": {k: v / max(1, n * (c1["evaluations"] - c0["evaluations"]))
                                                           for k, v in units.items()},
                                  "kernel_time_share": kms_m / ms2,
                                  "spectral_ms_per_residual": (tm1["spectral_ms"] - tm0["spectral_ms"]) /
                                  max(1, tm1["spectral_launches"] - tm0["spectral_launches"])}
                r2.close()
            errs = [float(abs(b["P_av"] - a_["P_av"]).max() / abs(a_["P_av"]).max())
                    for a_, b in zip(recs["fp64"], recs["mixed"])]
            line["mixed"] = {"value": vals["mixed"], "unit": UNIT, "fp64_same_run": vals["fp64"],
                             "increments": a.increments, "seconds": secs,
                             "timed": "whole load case (solver init and every increment) in each form",
                             "max_rel_P_av_error_vs_fp64": max(errs),
                             "per_increment_error_vs_fp64": errs, "roofline": mixed_roof,
                             "note": "FP32 FFT / Gamma with FP64 accumulation; Lp Newton Jacobian and hardening rate in FP32 (residual, update, convergence tests, tangent FP64)"}
        if a.batch_rves > 0:
            line["batched"] = batch_leg(g, torch, a.batch_rves, 20, a.batch_seconds, a.batch_compare)
        if not a.no_mixed_large:
            line["mixed_128"] = mixed_large_leg(g, torch)
        if a.serve_requests > 0:
            line["serving"] = [serve_leg(g, p, float(rate), a.serve_requests, a.serve_seconds)
                               for rate in a.serve_rates.split(",") for p in ("fp64", "mixed")]
        if rank == 0:
            threads = os.cpu_count() or 1
            try:
                v, dt, ev, orecs = cpu_oracle_sample(a, a.cpu_sample_increments, threads)
                if "mixed" in line:
                    k = min(len(orecs), len(recs.get("mixed", [])))
                    ev_or = [float(abs(recs[pr][i]["P_av"] - from_fortran9(orecs[i]["P_av"])).max() /
                                   abs(from_fortran9(orecs[i]["P_av"])).max()) for pr in ("mixed", "fp64")
                             for i in range(k)]
                    line["mixed"]["max_rel_P_av_error_vs_oracle"] = max(ev_or[:k]) if k else None
                    line["mixed"]["fp64_max_rel_P_av_error_vs_oracle"] = max(ev_or[k:]) if k else None
                    line["mixed"]["oracle_increments"] = k
                line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                                        "sample": f"solver init + first {a.cpu_sample_increments} increment(s) of the "
                                                  f"{a.cells}^3 workload ({ev} residual evaluations, {dt:.1f} s), "
                                                  "CPU oracle with OpenMP over cells"}
                v1, dt1 = cpu_one_core_sample(a)
                line["cpu_baseline"]["one_core"] = {
                    "value": v1, "unit": UNIT, "cores": 1,
                    "sample": f"one residual evaluation of the {a.cells}^3 workload at its first iteration "
                              f"(constitutive response of every cell, divergence RMS, Gamma convolution; {dt1:.1f} s), "
                              "CPU oracle on one thread (the reference's per-rank serial loop)"}
            except Exception as ex:  # the baseline is reported, never required
                line["cpu_baseline"] = {"value": None, "unit": UNIT, "cores": threads, "kind": "port",
                                        "sample": f"failed: {ex}"}
    if rank == 0:
        ratios = mixed_vs_fp64_ratios(line)
        if ratios:
            line["mixed_vs_fp64_ratios"] = ratios
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def mixed_vs_fp64_ratios(line):
    """The mixed form against the plain FP64 form, from the legs of this run that
    measured both on equal work: the 64^3 workload's whole load case, the 128^3
    configuration, the batched population in both forms, the batched population's
    first RVEs batched mixed against one at a time in FP64, and the served mix at each
    arrival rate in both forms.  A summary of values already in the line."""
    r = {}
    try:
        m = line.get("mixed")
        if m and m.get("fp64_same_run"):
            r["mixed_vs_fp64_same_workload"] = m["value"] / m["fp64_same_run"]
        m128 = line.get("mixed_128")
        if m128 and m128.get("fp64", {}).get("value"):
            r["mixed_vs_fp64_128cube"] = m128["mixed"]["value"] / m128["fp64"]["value"]
        b = line.get("batched") or {}
        if b.get("mixed_vs_fp64_batched"):
            r["batched_mixed_vs_batched_fp64"] = b["mixed_vs_fp64_batched"]
        seq = b.get("vs_plain_fp64_one_at_a_time")
        if seq:
            r["batched_mixed_vs_fp64_one_at_a_time"] = seq["speedup"]
        sv = {}
        for x in line.get("serving") or []:
            if x.get("value"):
                sv.setdefault(x["rate_req_per_s"], {})[x["precision"]] = x["value"]
        for rate, v in sorted(sv.items()):
            if "mixed" in v and "fp64" in v:
                r[f"served_mixed_vs_served_fp64_{rate:g}_req_s"] = v["mixed"] / v["fp64"]
        if "value" in line and b.get("value"):
            r["batched_mixed_vs_plain_fp64_value"] = b["value"] / line["value"]
    except (KeyError, TypeError, ZeroDivisionError):
        pass
    return r


def main():
    a = args_()
    if a.impl == "reference":
        from oracle import build as ob
        ob.build()
        reference_arm(a)
        return
    gpu_arm(a)


if __name__ == "__main__":
    main()
