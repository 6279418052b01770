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
