"""The C-ABI library builds for sm_103a, loads without a GPU and exports every
entry point declared in include/dgx.h; calls fail loudly without a device."""
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    src = open(os.path.join(ROOT, "include", "dgx.h")).read()
    return sorted(set(re.findall(r"\b(dgx_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_all_declared_symbols():
    from solver_cpp_gb300 import build
    lib = build.build()
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (dgx_\w+)", out))
    missing = [s for s in declared() if s not in exported]
    assert not missing, missing
    from solver_cpp_gb300 import dgx
    L = dgx.lib()
    for s in declared():
        assert hasattr(L, s)


def test_no_silent_fallback_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    import solver_cpp_gb300 as g
    with pytest.raises(g.DgxError):
        g.RVE((4, 4, 4), (1, 1, 1), np.zeros(64, int), [[1, 0, 0, 0]])


def test_flop_models_are_consistent():
    """The mixed form's flop model moves work from FP64 to FP32 and never adds FP64:
    the Lp iteration is unchanged, the Jacobian's FP64 and FP32 parts add up to the
    plain count, and every FP64 part is at most the plain one (host-only calls)."""
    import solver_cpp_gb300 as g
    plain = g.flop_model()
    f64, f32 = g.flop_model_mixed()
    assert f64["lp"] == plain["lp"] and f32["lp"] == 0.0
    assert f64["jacobian"] + f32["jacobian"] == plain["jacobian"]
    for k in plain:
        assert 0.0 <= f64[k] <= plain[k] and f32[k] >= 0.0
