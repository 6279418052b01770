"""The bench line's mixed-vs-FP64 summary (CPU only): every ratio comes from the legs
that measured both forms on equal work, with the keys the bench line carries."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def test_mixed_vs_fp64_ratios_from_the_legs():
    import bench
    line = {"value": 6.0e7,
            "mixed": {"value": 1.2e8, "fp64_same_run": 6.0e7},
            "mixed_128": {"mixed": {"value": 1.5e8}, "fp64": {"value": 6.0e7}},
            "batched": {"value": 1.3e8, "mixed_vs_fp64_batched": 2.2,
                        "vs_plain_fp64_one_at_a_time": {"speedup": 3.5}},
            "serving": [{"precision": "fp64", "rate_req_per_s": 20.0, "value": 5.0e7},
                        {"precision": "mixed", "rate_req_per_s": 20.0, "value": 1.2e8},
                        {"precision": "mixed", "rate_req_per_s": 50.0, "value": 1.2e8}]}
    r = bench.mixed_vs_fp64_ratios(line)
    assert r["mixed_vs_fp64_same_workload"] == 2.0
    assert r["mixed_vs_fp64_128cube"] == 2.5
    assert r["batched_mixed_vs_batched_fp64"] == 2.2
    assert r["batched_mixed_vs_fp64_one_at_a_time"] == 3.5
    assert r["served_mixed_vs_served_fp64_20_req_s"] == 2.4
    assert "served_mixed_vs_served_fp64_50_req_s" not in r      # no FP64 leg at that rate
    assert abs(r["batched_mixed_vs_plain_fp64_value"] - 1.3e8 / 6.0e7) < 1e-12


def test_mixed_vs_fp64_ratios_tolerates_missing_legs():
    import bench
    assert bench.mixed_vs_fp64_ratios({"value": 1.0}) == {}
