"""Allocation-free divergence RMS (dgx_divergence_rms_static) against the regular
entry point (dgx_divergence_rms), through the C ABI.

The static entry point serves callers that cannot call cudaMalloc: their device
memory is owned by their own pool or budget, or allocation is not allowed in
their loop.  It works in a fixed file-scope device array, so this file runs last
(pytest collects it after the other tests) and checks two calls in a row for
every divergence correction (none, size, size+grid) and both derivatives
(continuous, central difference), on grids with an odd and a size-1 axis.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12          # the divergence-RMS tolerance of the other parity tests

GRIDS = [((6, 7, 8), (0.75, 0.875, 1.0)), ((5, 1, 9), (0.5, 0.1, 0.9)), ((32, 32, 32), (1.0, 1.0, 1.0))]


def _static_rms(lib, cells, size, corr, deriv, P_dev, out_dev, stream):
    c = (C.c_int32 * 3)(*cells)
    s = (C.c_double * 3)(*size)
    return lib.dgx_divergence_rms_static(c, s, corr, deriv, C.c_void_p(P_dev), C.c_void_p(out_dev), C.c_void_p(stream))


@pytest.mark.parametrize("deriv", [0, 1])
@pytest.mark.parametrize("corr", [0, 1, 2])
def test_static_divergence_rms_matches_regular_entry_point(corr, deriv):
    import torch
    import solver_cpp_gb300 as g
    from solver_cpp_gb300 import build, dgx
    build.build()
    lib = dgx.lib()
    rng = np.random.default_rng(123 + 10 * corr + deriv)
    for cells, size in GRIDS:
        n = int(np.prod(cells))
        num = g.numerics(divergence_correction=corr, derivative=deriv)
        rve = g.RVE(cells, size, np.zeros(n, int), [[1, 0, 0, 0]], num=num)
        stream = torch.cuda.current_stream().cuda_stream
        out = torch.zeros(1, dtype=torch.float64, device="cuda")
        for call in range(2):                                   # two calls in a row
            P = 1e7 * rng.standard_normal((n, 3, 3)) + 3e7 * np.eye(3)
            ref = rve.calculate_divergence_rms(P)
            flat = np.ascontiguousarray(np.swapaxes(P, -1, -2)).reshape(-1)   # (3,3,N) reference layout
            P_dev = torch.from_numpy(flat).cuda()
            torch.cuda.synchronize()
            st = _static_rms(lib, cells, size, corr, deriv, P_dev.data_ptr(), out.data_ptr(), stream)
            assert st == 0, lib.dgx_last_error()
            torch.cuda.synchronize()
            got = float(out.item())
            assert got == pytest.approx(ref, rel=TOL), (cells, corr, deriv, call, got, ref)
        rve.close()


def test_static_divergence_rms_rejects_bad_arguments():
    import torch
    from solver_cpp_gb300 import build, dgx
    build.build()
    lib = dgx.lib()
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    P = torch.zeros(9 * 64, dtype=torch.float64, device="cuda")
    # beyond the 32768-cell scratch
    assert _static_rms(lib, (64, 32, 32), (1.0, 1.0, 1.0), 2, 0, P.data_ptr(), out.data_ptr(), 0) == -1
    # divergence correction outside none / size / size+grid
    assert _static_rms(lib, (4, 4, 4), (1.0, 1.0, 1.0), 3, 0, P.data_ptr(), out.data_ptr(), 0) == -1
    assert _static_rms(lib, (4, 4, 4), (1.0, 1.0, 1.0), -1, 0, P.data_ptr(), out.data_ptr(), 0) == -1
    # unknown derivative; the forward/backward difference is not offered here
    assert _static_rms(lib, (4, 4, 4), (1.0, 1.0, 1.0), 2, 7, P.data_ptr(), out.data_ptr(), 0) == -1
    assert _static_rms(lib, (4, 4, 4), (1.0, 1.0, 1.0), 2, 2, P.data_ptr(), out.data_ptr(), 0) == -4
