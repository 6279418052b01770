"""Serving (dgx_server_*) through the C ABI: requests that arrive while others run
are admitted by HBM footprint, overlap on the device, and each result is the same
as the same solve run alone (bitwise: batch members compute what they compute alone)."""
import time

import numpy as np
import pytest

from solver_cpp_gb300 import synthetic

pytestmark = pytest.mark.gpu

CASES = [((8, 8, 8), 6, 21, "tensionX", "fp64", 3),
         ((16, 16, 16), 15, 22, "shearXY", "mixed", 2),
         ((12, 8, 10), 8, 23, "tensionZ", "fp64", 3),
         ((16, 16, 16), 30, 24, "tensionY", "fp64", 2),
         ((8, 8, 8), 10, 25, "tensionY", "mixed", 4)]


@pytest.fixture(scope="module")
def gpu():
    import solver_cpp_gb300 as g
    from solver_cpp_gb300 import build
    build.build()
    return g


def _inputs(g, case):
    cells, ng, seed, kind, prec, n = case
    mat, q = synthetic.microstructure(cells, ng, seed)
    return cells, mat, q, [g.load_step(kind, t=float(n), N=n)], g.numerics(precision=prec)


def _solo(g, case):
    cells, mat, q, steps, num = _inputs(g, case)
    rve = g.RVE(cells, (1.0, 1.0, 1.0), mat, q, num=num)
    recs = rve.loop_over_loadcase(steps)
    rve.close()
    return recs


def test_requests_in_a_mix_equal_solo(gpu):
    solo = [_solo(gpu, c) for c in CASES]
    srv = gpu.Server(max_active=8)
    ids = []
    for k, c in enumerate(CASES):
        cells, mat, q, steps, num = _inputs(gpu, c)
        ids.append(srv.submit(cells, (1.0, 1.0, 1.0), mat, q, steps, num=num))
        if k == 1:
            time.sleep(0.05)          # later requests arrive while the first ones run
    for rid, ref in zip(ids, solo):
        st = srv.result(rid, timeout=600)
        assert st["state"] == "done", st
        assert len(st["records"]) == len(ref)
        for a, b in zip(st["records"], ref):
            assert np.array_equal(a["P_av"], b["P_av"]) and np.array_equal(a["F_av"], b["F_av"])
            assert a["iterations"] == b["iterations"]
        assert st["t_submit"] <= st["t_admit"] <= st["t_done"]
    info = srv.stats()
    assert info["completed"] == len(CASES) and info["used_bytes"] == 0 and info["status"] == 0
    srv.close()


def test_admission_by_footprint(gpu):
    big = CASES[3]
    fp = gpu.footprint(big[0], gpu.numerics(precision=big[4]), big[1])
    srv = gpu.Server(hbm_budget_bytes=int(2.5 * fp), max_active=16)
    ids = []
    for s in range(5):
        cells, mat, q, steps, num = _inputs(gpu, big[:2] + (30 + s,) + big[3:])
        ids.append(srv.submit(cells, (1.0, 1.0, 1.0), mat, q, steps, num=num))
    peak = 0
    while srv.stats()["completed"] < 5:
        i = srv.stats()
        peak = max(peak, i["running"])
        assert i["used_bytes"] <= i["budget_bytes"]
        time.sleep(0.002)
    assert peak <= 2
    for rid in ids:
        assert srv.result(rid)["state"] == "done"
    # a request that can never fit is refused at submission
    cells, mat, q, steps, num = _inputs(gpu, big)
    tiny = gpu.Server(hbm_budget_bytes=fp // 2, max_active=2)
    with pytest.raises(gpu.DgxError):
        tiny.submit(cells, (1.0, 1.0, 1.0), mat, q, steps, num=num)
    tiny.close()
    srv.close()


def test_footprint_matches_allocation(gpu):
    for c in CASES[:3]:
        cells, mat, q, steps, num = _inputs(gpu, c)
        rve = gpu.RVE(cells, (1.0, 1.0, 1.0), mat, q, num=num)
        assert gpu.footprint(cells, num, q.shape[0]) == rve.device_bytes
        rve.close()
