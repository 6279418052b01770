"""The device-resident drop-in boundary, exercised by a C++ caller of the C ABI
(tests/native/fields_check.cpp): VTI geometry read through the library
(f_VTI_readCellsSizeOrigin / f_VTI_readDataset_int, src/grid/discretization_grid.h:19-22),
library-owned device fields (f_homogenization_fetch_tensor_pointers, src/grid/spectral.h:17-19)
and the in-place constitutive response (f_homogenization_mechanical_response + _response2),
bitwise equal to the host-copy entry point on the same inputs."""
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _cuda_home():
    nv = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(os.path.realpath(nv)))


def test_native_caller_device_fields_and_vti(tmp_path, knowns):
    from solver_cpp_gb300 import build
    lib = build.build()
    cuda = _cuda_home()
    libdirs = [d for d in (os.path.join(cuda, "lib64"), os.path.join(cuda, "targets", "sbsa-linux", "lib"),
                           os.path.join(cuda, "targets", "x86_64-linux", "lib")) if os.path.isdir(d)]
    exe = str(tmp_path / "fields_check")
    cmd = ["g++", "-O1", "-std=c++17", os.path.join(HERE, "native", "fields_check.cpp"), "-o", exe,
           "-I", os.path.join(cuda, "include"), lib, "-Wl,-rpath," + os.path.dirname(lib)]
    for d in libdirs:
        cmd += ["-L", d, "-Wl,-rpath," + d]
    cmd += ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    vti = tmp_path / "grid.vti"
    vti.write_text(knowns["vti_16x16x16"]["content"])
    r = subprocess.run([exe, str(vti)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("ok 16 16 16"), r.stdout + r.stderr
