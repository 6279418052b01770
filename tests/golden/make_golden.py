"""Extract the reference's known-answer vectors into tests/golden/reference_knowns.json.

Also stored as text: the example inputs of examples/grid (load cases, material.yaml,
numerics.yaml) and the geometry and material.yaml of the 6-grain result in
python/tests/resources/Result, used as input-format test cases.

Reads the reference's own GoogleTest sources as text (the Eigen ``setValues`` literals and
scalar expectations) and writes them out as JSON, keeping each value exactly as printed.
Run in a checkout that has the reference tree:

    python tests/golden/make_golden.py /path/to/reference

Arrays are written in the nested order of the Eigen initialiser (first index outermost);
``numpy.array(v).ravel(order="F")`` gives the reference's column-major storage.
"""
import ast
import json
import os
import re
import sys


def _literal(text):
    # complex literals c( re , im ) -> [re, im]
    text = re.sub(r"c\(\s*([^,()]+?)\s*,\s*([^,()]+?)\s*\)", r"[\1, \2]", text)
    text = text.replace("{", "[").replace("}", "]")
    return ast.literal_eval(text)


def set_values(src, name, occurrence=0):
    """Return the nested list passed to ``name.setValues(...)`` (n-th occurrence)."""
    starts = [m.end() for m in re.finditer(r"(?<![\w.])" + re.escape(name) + r"\.setValues\(", src)]
    start = starts[occurrence]
    depth, i = 0, start
    while True:
        ch = src[i]
        if ch == "(":
            depth += 1
        elif ch == ")":
            if depth == 0:
                break
            depth -= 1
        i += 1
    return _literal(src[start:i])


def stream_matrix(src, lhs, occurrence=0):
    """Eigen comma initialiser ``lhs << a, b, ...;`` (row-major 3x3)."""
    m = [mm for mm in re.finditer(re.escape(lhs) + r"\s*<<([^;]+);", src)][occurrence]
    toks = [t.strip() for t in m.group(1).replace("\n", " ").split(",")]
    vals = []
    for t in toks:
        vals.append({"true": 1, "false": 0}.get(t, None) if t in ("true", "false") else float(t))
    return [vals[0:3], vals[3:6], vals[6:9]]


def main(ref):
    tdir = os.path.join(ref, "src", "grid", "test")
    rd = lambda f: open(os.path.join(tdir, f)).read()
    sp, mb, ms, dg = rd("test_spectral.cpp"), rd("test_mech_base.cpp"), rd("test_mech_solver_basic.cpp"), \
        rd("test_discretization_grid.cpp")
    out = {"source": "reference src/grid/test/*.cpp (GoogleTest known answers)"}
    out["spectral_init_2x1x1"] = {
        "cells": [2, 1, 1], "geom": [2e-5, 1e-5, 1e-5],
        "xi1st": set_values(sp, "expected_xi1st"), "xi2nd": set_values(sp, "expected_xi2nd")}
    out["constitutive_response_2x1x1"] = {
        "F": set_values(sp, "F"), "P": set_values(sp, "mech2_homogenization_P_result"),
        "dPdF": set_values(sp, "mech2_homogenization_dPdF_result"),
        "P_av": set_values(sp, "expected_P_av"), "C_volAvg": set_values(sp, "expected_C_vol_avg"),
        "C_minMaxAvg": set_values(sp, "expected_C_minmax_avg")}
    out["divergence_correction"] = {"cells": [2, 1, 1], "geom": [3, 4, 5],
                                    "size": [0.75, 1, 1.25], "size+grid": [0.6, 0.8, 1]}
    out["update_coords_2x1x1_identity"] = {
        "x_n": set_values(mb, "expected_x_n"), "x_p": set_values(mb, "expected_x_p")}
    out["forward_field"] = {
        "field_last_inc": set_values(mb, "field_last_inc"), "rate": set_values(mb, "rate"),
        "aim": set_values(mb, "aim"), "wgt": 0.5, "delta_t": 1.0,
        "expected": set_values(mb, "expected_forwarded_field")}
    mask = stream_matrix(mb, "mask_stress")
    out["masked_compliance"] = {"C": set_values(mb, "C"), "mask_stress": mask,
                                "expected": set_values(mb, "expected_masked_compliance")}
    rms = float(re.search(r"ASSERT_EQ\(rms,\s*([0-9.eE+-]+)\)", mb).group(1))
    out["divergence_rms_4x1x1"] = {"cells": [4, 1, 1], "geom": [4e-5, 1e-5, 1e-5], "wgt": 0.25,
                                   "field": set_values(mb, "tensor_field"),
                                   "xi1st": set_values(mb, "spectral.xi1st", 1), "rms": rms,
                                   "rms_text": re.search(r"ASSERT_EQ\(rms,\s*([0-9.eE+-]+)\)", mb).group(1)}
    out["gamma_convolution_2x1x1"] = {
        "field_aim": set_values(mb, "field_aim"), "C_ref": set_values(mb, "mech_base.C_ref"),
        "field": set_values(mb, "field"), "expected": set_values(mb, "expected_gamma_field")}
    out["calculate_rate"] = {"field": set_values(mb, "field", 1), "field_0": set_values(mb, "field_0"),
                             "avRate": set_values(mb, "avRate"), "dt": 100.2,
                             "expected": set_values(mb, "expected_rate")}
    out["form_residual"] = {
        "S": set_values(ms, "mech_basic.S"), "P_av": set_values(ms, "mech_basic.P_av"),
        "F_aim": stream_matrix(ms, "mech_basic.F_aim"),
        "stress_mask": stream_matrix(ms, "mech_basic.params.stress_mask"),
        "expected_rotated": set_values(ms, "expected_rotated"),
        "expected_F_aim": set_values(ms, "expected_F_aim"),
        "expected_err_BC": float(re.search(r"EXPECT_EQ\(mech_basic\.err_BC,\s*([0-9.eE+-]+)\)", ms).group(1))}
    out["basic_forward"] = {
        "deformation_values": stream_matrix(ms, "deformation_bc.values"),
        "deformation_mask": stream_matrix(ms, "deformation_bc.mask"),
        "stress_mask": stream_matrix(ms, "stress_bc.mask"),
        "delta_t": 100.2, "delta_t_old": 1.0, "t_remaining": 1002.0,
        "expected_field_last_inc": set_values(ms, "expected_field_last_inc"),
        "expected_aim": set_values(ms, "expected_aim")}
    out["ip_node_coords_2x1x1"] = {"cells": [2, 1, 1], "geom": [2e-5, 1e-5, 1e-5],
                                   "ip": set_values(dg, "expected_ip_coords0"),
                                   "node": set_values(dg, "expected_node_coords0")}
    m = re.search(r'vti_file_content = \(R""""\((.*?)\)""""\);', dg, re.S)
    out["vti_16x16x16"] = {"content": m.group(1), "cells": [16, 16, 16], "size": [1, 1, 1],
                           "origin": [0, 0, 0]}
    cf = rd("test_config.cpp")
    raw = re.findall(r'write_to_file\(R""""\((.*?)\)""""\);', cf, re.S)
    out["config_yaml"] = {"numerics": raw[0], "load": raw[1]}
    ex = os.path.join(ref, "examples", "grid")
    out["examples_grid"] = {n: open(os.path.join(ex, n)).read()
                            for n in ("tensionX.yaml", "shearXY.yaml", "shearZX.yaml", "material.yaml", "numerics.yaml")}
    res = os.path.join(ref, "python", "tests", "resources", "Result")
    out["material_yaml_6grains"] = open(os.path.join(res, "6grains6x7x8_single_phase.material.yaml")).read()
    out["vti_6grains"] = open(os.path.join(res, "6grains6x7x8_single_phase.vti")).read()
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_knowns.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", dst)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {os.path.basename(__file__)} <path of the reference checkout>")
    main(sys.argv[1])
