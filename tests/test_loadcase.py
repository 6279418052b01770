"""Host-side input parsing (load case and numerics YAML of the reference)."""
import numpy as np

def _examples():
    import json
    import os
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_knowns.json")) as f:
        return json.load(f)["examples_grid"]


TENSION_X = _examples()["tensionX.yaml"]
NUMERICS = _examples()["numerics.yaml"]


def test_parse_load_yaml_tensionX():
    from solver_cpp_gb300 import parse_load_yaml, load_step
    (s,) = parse_load_yaml(TENSION_X)
    assert s.def_type == 1 and s.stress_type == 0
    assert s.t == 5 and s.N == 10 and s.f_out == 4
    dv = np.array(s.def_values[:]).reshape(3, 3, order="F")
    dm = np.array(s.def_mask[:]).reshape(3, 3, order="F")
    sm = np.array(s.stress_mask[:]).reshape(3, 3, order="F")
    assert dv[0, 0] == 1e-3 and dm[1, 1] == 1 and dm[2, 2] == 1 and dm[0, 0] == 0
    assert sm[1, 1] == 0 and sm[2, 2] == 0 and sm[0, 0] == 1 and sm[0, 1] == 1
    ref = load_step("tensionX", t=5, N=10, f_out=4)
    assert list(ref.def_mask) == list(s.def_mask) and list(ref.stress_mask) == list(s.stress_mask)


def test_parse_numerics_yaml():
    from solver_cpp_gb300 import parse_numerics_yaml
    n = parse_numerics_yaml(NUMERICS)
    assert n.itmin == 4 and n.itmax == 40
    assert n.eps_rel_div == 5e-4 and n.divergence_correction == 2


def _config_yaml():
    import json
    import os
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_knowns.json")) as f:
        return json.load(f)["config_yaml"]


def test_numerics_yaml_read_success():
    """NumYamlSetup.TestYamlReadSuccess (test_config.cpp): every grid key the solver reads."""
    from solver_cpp_gb300 import parse_numerics_yaml
    n = parse_numerics_yaml(_config_yaml()["numerics"])
    assert n.stag_iter_max == 10 and n.max_cut_back == 3
    assert n.itmin == 1 and n.itmax == 100
    assert n.eps_abs_div == 1.0e-4 and n.eps_rel_div == 5.0e-4
    assert n.eps_abs_P == 1.0e3 and n.eps_rel_P == 1.0e-3
    assert n.update_gamma == 0
    assert n.divergence_correction == 2 and n.derivative == 0


def test_load_yaml_read_basic():
    """LoadYamlSetup.TestYamlReadBasic (test_config.cpp): r, t, N, estimate_rate, R,
    f_out and the deformation values and mask of one load step.  (f_restart is not a
    field of the load step here: the restart cadence is an argument of the run.)"""
    from solver_cpp_gb300 import parse_load_yaml
    (s,) = parse_load_yaml(_config_yaml()["load"])
    assert s.r == 2 and s.t == 60 and s.N == 120 and s.estimate_rate == 0
    assert list(s.rot_q) == [1.0, 2.0, 3.0, 4.0] and s.f_out == 4
    assert s.def_type == 1 and s.stress_type == 0
    dv = np.array(s.def_values[:]).reshape(3, 3, order="F")
    dm = np.array(s.def_mask[:]).reshape(3, 3, order="F")
    assert np.array_equal(dv, [[0.001, 1, 0], [0, 0, 0], [2, 0, 0]])
    assert np.array_equal(dm, [[0, 0, 0], [0, 1, 0], [0, 0, 1]])


def test_load_yaml_errors():
    """The parser's refusals (test_config.cpp / config.cpp): two deformation
    specifications, a rotation that is not a quaternion, a string other than x in a
    matrix, and a solver other than spectral_basic."""
    import pytest
    from solver_cpp_gb300 import parse_load_yaml
    base = _config_yaml()["load"]
    with pytest.raises(ValueError):
        parse_load_yaml(base.replace("        R: [1, 2, 3, 4]", "        R: [1, 2, 3]"))
    with pytest.raises(ValueError):
        parse_load_yaml(base.replace("        R: [1, 2, 3, 4]", "        F: [[1, 0, 0], [0, 1, 0], [0, 0, 1]]"))
    with pytest.raises(ValueError):
        parse_load_yaml(base.replace("[0,      x, 0]", "[0,      y, 0]"))
    with pytest.raises(ValueError):
        parse_load_yaml(base.replace("spectral_basic", "FEM"))
