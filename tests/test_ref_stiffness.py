"""The reference stiffness C_minMaxAvg at F = I is an argmax/argmin over cells whose
norms tie to FP64 rounding; the library's host evaluation (ref_stiffness.cpp) must
pick exactly what the reference's operation order picks (the oracle reproduces the
Fortran result bit for bit on the 6-grain fixture).  CPU-only: no device needed."""
import ctypes as C

import numpy as np
import pytest

from oracle import dgo
from tests import cases


def _lib_fn():
    from solver_cpp_gb300 import build, dgx
    build.build()
    f = dgx.lib().dgx_reference_stiffness
    f.argtypes = [C.c_double] * 3 + [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_int32), C.c_int64,
                                     C.POINTER(C.c_double)]
    return f


def _cases():
    from solver_cpp_gb300.synthetic import microstructure, random_quaternions
    fx = cases.damask_6grains()
    yield fx["cells"], fx["size"], fx["material_at"], fx["orientations"]
    c, s, m = cases.grains16()
    yield c, s, m, random_quaternions(20, 2024)
    for cells, ng, seed in [((8, 8, 8), 6, 1), ((16, 16, 16), 50, 3), ((12, 10, 9), 17, 8)]:
        m, q = microstructure(cells, ng, seed)
        yield cells, (1, 1, 1), m, q


@pytest.mark.parametrize("k", range(5))
def test_reference_stiffness_bitwise(k):
    cells, size, mat, q = list(_cases())[k]
    f = _lib_fn()
    out = np.zeros(81)
    qq = np.ascontiguousarray(q, dtype=float)
    mm = np.ascontiguousarray(mat, dtype=np.int32)
    assert f(106.75e9, 60.41e9, 28.34e9, len(qq), qq.ctypes.data_as(C.POINTER(C.c_double)),
             mm.ctypes.data_as(C.POINTER(C.c_int32)), len(mm), out.ctypes.data_as(C.POINTER(C.c_double))) == 0
    s = dgo.Solver(cells, size, mat, q)
    dgo.lib().dgo_solver_init_state(s.h)
    assert np.array_equal(out, s.get("C_minMaxAvg"))
