"""Batched execution (dgx_batch_*) through the C ABI.

A member of a batch of uneven RVEs (different grids, grain counts, load cases and
spectral precision) must compute exactly what the same RVE computes alone: the
batched kernels run the same per-point arithmetic, the same reduction partitions
and the same summation orders, so the comparison is bitwise (tolerance 0).
"""
import numpy as np
import pytest

from solver_cpp_gb300 import synthetic

pytestmark = pytest.mark.gpu

# (cells, grains, seed, load case, spectral precision)
CASES = [((8, 8, 8), 5, 11, "tensionX", "fp64"),
         ((16, 16, 16), 12, 12, "shearXY", "fp64"),
         ((12, 10, 8), 7, 13, "tensionY", "mixed"),
         ((8, 8, 8), 9, 14, "tensionZ", "mixed"),
         ((16, 16, 16), 20, 15, "tensionX", "fp64")]


@pytest.fixture(scope="module")
def gpu():
    import solver_cpp_gb300 as g
    from solver_cpp_gb300 import build
    build.build()
    return g


def _make(g, case, N=4):
    cells, ng, seed, kind, prec = case
    mat, q = synthetic.microstructure(cells, ng, seed)
    rve = g.RVE(cells, (1.0, 1.0, 1.0), mat, q, num=g.numerics(precision=prec))
    return rve, [g.load_step(kind, t=float(N), N=N)]


def _same(recs_a, recs_b):
    assert len(recs_a) == len(recs_b)
    for a, b in zip(recs_a, recs_b):
        assert np.array_equal(a["P_av"], b["P_av"])
        assert np.array_equal(a["F_av"], b["F_av"])
        assert a["iterations"] == b["iterations"] and a["evaluations"] == b["evaluations"]


def test_batch_members_equal_solo_runs(gpu):
    solo = []
    for c in CASES:
        rve, steps = _make(gpu, c)
        solo.append((rve, rve.loop_over_loadcase(steps)))
    batch = gpu.Batch(8)
    members = [_make(gpu, c) for c in CASES]
    slots = [batch.add(r, s) for r, s in members]
    batch.run()
    st = batch.stats()
    assert st["rounds"] > 0 and st["point_evaluations"] > 0
    for slot, (rve, steps), (srve, srecs) in zip(slots, members, solo):
        m = batch.member(slot)
        assert m["done"] and m["status"] == 0
        _same(batch.records(slot), srecs)
        batch.remove(slot)
        for key in ("F", "P", "Fp"):
            assert np.array_equal(rve.get(key), srve.get(key)), key
    batch.close()


def test_member_added_between_rounds(gpu):
    """Continuous batching: a member that joins while others are mid-solve."""
    late_case = CASES[2]
    srve, steps = _make(gpu, late_case, N=3)
    srecs = srve.loop_over_loadcase(steps)
    batch = gpu.Batch(4)
    a, sa = _make(gpu, CASES[0], N=3)
    b, sb = _make(gpu, CASES[1], N=3)
    batch.add(a, sa)
    batch.add(b, sb)
    for _ in range(7):
        batch.step()
    late, lsteps = _make(gpu, late_case, N=3)
    slot = batch.add(late, lsteps)
    batch.run()
    _same(batch.records(slot), srecs)
    batch.close()


def test_batch_capacity_and_state_errors(gpu):
    batch = gpu.Batch(1)
    a, sa = _make(gpu, CASES[0], N=1)
    b, sb = _make(gpu, CASES[3], N=1)
    batch.add(a, sa)
    with pytest.raises(gpu.DgxError):
        batch.add(b, sb)                     # full
    with pytest.raises(gpu.DgxError):
        a.loop_over_loadcase(sa)             # driven by the batch
    batch.run()
    batch.remove(0)
    a.loop_over_loadcase(sa)                 # back on its own stream
    batch.close()


def test_autotuned_tiles_and_blocks_do_not_change_results(gpu, monkeypatch):
    """The autotuner picks points per block and FFT tiles; results are identical to
    a fixed configuration (DGX_AUTOTUNE=0, 64 points per block)."""
    monkeypatch.setenv("DGX_AUTOTUNE", "0")
    monkeypatch.setenv("DGX_CONS_BLOCK", "64")
    fixed, steps = _make(gpu, CASES[1], N=6)
    ref = fixed.loop_over_loadcase(steps)
    monkeypatch.delenv("DGX_AUTOTUNE")
    monkeypatch.delenv("DGX_CONS_BLOCK")
    batch = gpu.Batch(2)
    tuned, steps2 = _make(gpu, CASES[1], N=6)
    slot = batch.add(tuned, steps2)
    batch.run()
    t = batch.tuning()
    assert t["tuned_grids"] >= 1 and not t["tuning_block"] and t["cons_block"] in (32, 64, 128, 256)
    _same(batch.records(slot), ref)
    batch.close()


def test_round_point_budget_keeps_results(gpu):
    """With a per-round point cap the smallest remaining work goes first; every member
    still computes exactly its solo result."""
    solo = []
    for c in CASES[:4]:
        rve, steps = _make(gpu, c, N=3)
        solo.append(rve.loop_over_loadcase(steps))
    batch = gpu.Batch(8)
    batch.set_round_points(5000)        # below the sum of the members' cells
    slots = [batch.add(*_make(gpu, c, N=3)) for c in CASES[:4]]
    batch.run()
    for slot, ref in zip(slots, solo):
        _same(batch.records(slot), ref)
    batch.close()


def test_graph_replay_is_bitwise_identical(gpu, monkeypatch):
    """Rounds whose launch parameters repeat are replayed as captured CUDA graphs; the
    records equal those of a batch that launches every round directly (DGX_GRAPHS=0)."""
    monkeypatch.setenv("DGX_GRAPHS", "0")
    direct = gpu.Batch(4)
    m0 = [_make(gpu, c, N=4) for c in CASES[:3]]
    s0 = [direct.add(r, s) for r, s in m0]
    direct.run()
    assert direct.stats()["graph_rounds"] == 0
    monkeypatch.delenv("DGX_GRAPHS")
    graphed = gpu.Batch(4)
    m1 = [_make(gpu, c, N=4) for c in CASES[:3]]
    s1 = [graphed.add(r, s) for r, s in m1]
    graphed.run()
    st = graphed.stats()
    assert st["graph_rounds"] > st["rounds"] // 4
    for a, b, (ra, _), (rb, _) in zip(s0, s1, m0, m1):
        _same(direct.records(a), graphed.records(b))
        direct.remove(a); graphed.remove(b)
        assert np.array_equal(ra.get("P"), rb.get("P"))
    direct.close()
    graphed.close()


def test_single_rve_uses_graphs(gpu):
    """A single-RVE load case is a batch of one: its repeated rounds replay graphs too."""
    rve, steps = _make(gpu, CASES[0], N=3)
    rve.loop_over_loadcase(steps)
    assert rve.counters()["graph_rounds"] > 0


def test_batch_of_derivatives_and_prime_grids_equals_solo(gpu):
    """Members with the forward/backward-difference and central-difference derivatives
    and grid lengths with prime factors above 16 (two FWBW members of one grid share a
    size group: the complex-xi z pass, each member's own Gamma table), next to a
    continuous-derivative member: each bitwise equal to its solo run."""
    cases = [((17, 6, 5), 5, 21, "tensionX", "fp64", "FWBW_difference"),
             ((17, 6, 5), 4, 22, "shearXY", "fp64", "FWBW_difference"),
             ((12, 10, 9), 6, 23, "tensionY", "fp64", "central_difference"),
             ((19, 4, 6), 3, 24, "tensionZ", "mixed", "continuous"),
             ((8, 8, 8), 5, 25, "tensionX", "mixed", "FWBW_difference")]

    def make(c):
        cells, ng, seed, kind, prec, deriv = c
        mat, q = synthetic.microstructure(cells, ng, seed)
        size = tuple(n / max(cells) for n in cells)
        rve = gpu.RVE(cells, size, mat, q, num=gpu.numerics(precision=prec, derivative=deriv))
        return rve, [gpu.load_step(kind, t=3.0, N=3)]

    solo = [r.loop_over_loadcase(s) for r, s in (make(c) for c in cases)]
    batch = gpu.Batch(len(cases))
    members = [make(c) for c in cases]
    slots = [batch.add(r, s) for r, s in members]
    batch.run()
    ht = batch.host_times()
    assert min(ht.values()) >= 0.0 and ht["wait"] > 0.0 and ht["advance"] > 0.0
    for slot, srecs in zip(slots, solo):
        m = batch.member(slot)
        assert m["done"] and m["status"] == 0
        _same(batch.records(slot), srecs)
