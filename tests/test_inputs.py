"""Geometry / material / load / numerics inputs in the reference's formats (CPU only).

Known answers: the reference's VTI test (src/grid/test/test_discretization_grid.cpp:
16^3 cells, size 1, origin 0), the 6-grain DAMASK result's geometry and material
files (material map and orientations of the Fortran run) and the example inputs of
examples/grid, all extracted as text by tests/golden/make_golden.py."""
import base64
import json
import os
import struct
import zlib

import numpy as np
import pytest

from tests import cases

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def knowns():
    with open(os.path.join(HERE, "golden", "reference_knowns.json")) as f:
        return json.load(f)


def test_read_vti_reference_known_answer(knowns):
    from solver_cpp_gb300.inputs import read_vti
    k = knowns["vti_16x16x16"]
    cells, size, origin, mat = read_vti(k["content"])
    assert list(cells) == k["cells"] and list(size) == k["size"] and list(origin) == k["origin"]
    c2, s2, m2 = cases.vti_material(k["content"])
    assert np.array_equal(mat, m2) and mat.size == 16 ** 3


def test_read_vti_6grains_matches_damask_run(knowns):
    from solver_cpp_gb300.inputs import read_vti
    fx = cases.damask_6grains()
    cells, size, origin, mat = read_vti(knowns["vti_6grains"])
    assert list(cells) == list(fx["cells"]) and np.allclose(size, fx["size"], rtol=1e-15)
    assert np.array_equal(mat, fx["material_at"])


@pytest.mark.parametrize("fmt", ["ascii", "raw32", "raw64", "zlib64"])
def test_read_vti_encodings(fmt):
    from solver_cpp_gb300.inputs import read_vti
    cells = (3, 2, 4)
    data = np.arange(24, dtype=np.int64)[::-1].copy()
    header = "UInt64" if fmt.endswith("64") else "UInt32"
    hf = "<Q" if header == "UInt64" else "<I"
    extra = ' compressor="vtkZLibDataCompressor"' if fmt.startswith("zlib") else ""
    if fmt == "ascii":
        body, f = " ".join(str(v) for v in data), "ascii"
    elif fmt.startswith("raw"):
        raw = data.tobytes()
        body, f = base64.b64encode(struct.pack(hf, len(raw)) + raw).decode(), "binary"
    else:
        raw = data.tobytes()
        blocks = [raw[:100], raw[100:]]
        comp = [zlib.compress(b) for b in blocks]
        hdr = struct.pack("<3Q", 2, 100, len(blocks[1])) + struct.pack("<2Q", *[len(c) for c in comp])
        body, f = base64.b64encode(hdr).decode() + base64.b64encode(b"".join(comp)).decode(), "binary"
    text = (f'<?xml version="1.0"?>\n<VTKFile type="ImageData" version="0.1" byte_order="LittleEndian" '
            f'header_type="{header}"{extra}>\n<ImageData WholeExtent="0 3 0 2 0 4" Origin="1 2 3" '
            f'Spacing="0.5 0.25 2">\n<Piece Extent="0 3 0 2 0 4">\n<CellData>\n'
            f'<DataArray type="Int64" Name="material" format="{f}">\n{body}\n</DataArray>\n'
            f'</CellData>\n</Piece>\n</ImageData>\n</VTKFile>\n')
    c, s, o, m = read_vti(text)
    assert list(c) == list(cells) and list(s) == [1.5, 0.5, 8.0] and list(o) == [1, 2, 3]
    assert np.array_equal(m, data)


def test_read_material_yaml_examples(knowns):
    from solver_cpp_gb300.inputs import read_material_yaml
    mat, q, ph, ho = read_material_yaml(knowns["examples_grid"]["material.yaml"])
    assert (mat.C11, mat.C12, mat.C44) == (106.75e9, 60.41e9, 28.34e9)
    assert (mat.xi_0, mat.xi_inf, mat.h_0, mat.n, mat.dot_gamma_0, mat.a) == (31e6, 63e6, 75e6, 20, 1e-3, 2.25)
    assert list(mat.h_sl_sl) == [1, 1, 1.4, 1.4, 1.4, 1.4, 1.4]
    assert ph == "Aluminum" and ho == "SX" and q.shape[1] == 4 and list(q[0]) == [1, 0, 0, 0]
    fx = cases.damask_6grains()
    mat, q, ph, ho = read_material_yaml(knowns["material_yaml_6grains"])
    assert ph == "pheno_fcc" and np.array_equal(q, fx["orientations"])


def test_read_material_yaml_rejects_unsupported(knowns):
    from solver_cpp_gb300.inputs import read_material_yaml
    text = knowns["examples_grid"]["material.yaml"]
    with pytest.raises(ValueError):
        read_material_yaml(text.replace("lattice: cF", "lattice: cI"))
    with pytest.raises(ValueError):
        read_material_yaml(text.replace("type: phenopowerlaw", "type: isotropic"))


def test_example_load_cases_and_numerics(knowns):
    from solver_cpp_gb300 import material, numerics, parse_load_yaml, parse_numerics_yaml
    from solver_cpp_gb300.inputs import apply_phase_numerics
    ex = knowns["examples_grid"]
    (sx,) = parse_load_yaml(ex["shearXY.yaml"])
    (sz,) = parse_load_yaml(ex["shearZX.yaml"])
    assert sz.N == 120 and sz.t == 60 and sz.f_out == 20 and list(sz.stress_mask) == [1] * 9
    assert sz.def_values[6] == 1e-3 and sx.def_type == 1
    n = parse_numerics_yaml(ex["numerics.yaml"], numerics())
    assert n.itmin == 4 and n.itmax == 40
    m = apply_phase_numerics("phase:\n  mechanical:\n    r_cutback: 0.5\n    plastic:\n      N_iter_Lp_max: 33\n",
                             material())
    assert m.r_cutback == 0.5 and m.N_iter_Lp_max == 33
