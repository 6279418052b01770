"""The HDF5 writer/reader used for DADF5 results and restarts (solver_cpp_gb300/csrc/h5lite.hpp),
built into a small host program and checked three ways: the C++ reader reads back what
was written, the independent Python reader (tests/golden/hdf5lite.py) sees the same
tree, values and attributes, and the file uses the structures of the HDF5 library's
own files (symbol-table groups, local heaps with a free block)."""
import os
import subprocess
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
from hdf5lite import HDF5File  # noqa: E402


@pytest.fixture(scope="module")
def h5file(tmp_path_factory):
    d = tmp_path_factory.mktemp("h5")
    exe = str(d / "h5lite_check")
    r = subprocess.run(["g++", "-O1", "-std=c++17", os.path.join(HERE, "native", "h5lite_check.cpp"), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    path = str(d / "check.hdf5")
    r = subprocess.run([exe, path], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "ok", (r.returncode, r.stdout, r.stderr)
    return path


def test_python_reader_sees_the_tree(h5file):
    f = HDF5File(h5file)
    assert f.keys("/") == ["cell_to", "geometry", "increment_0", "many", "setup", "solver"]
    assert len(f.keys("/many")) == 70
    F = f.read("/increment_0/phase/alpha/mechanical/F")
    assert F.shape == (2, 3, 3) and np.array_equal(F.ravel(), 0.5 * np.arange(18) - 1.0)
    assert np.array_equal(f.read("/solver/ints"), [7, -8, 9])
    assert f.read("/many/d42")[0] == 42.0
    assert f.keys("/increment_0/homogenization/SX/mechanical") == []


def test_attributes_strings_and_records(h5file):
    f = HDF5File(h5file)
    a = f.attrs("/")
    assert int(a["DADF5_version_major"]) == 1 and a["creator"] == "check"
    assert list(f.attrs("/geometry")["cells"]) == [2, 3, 4]
    assert float(f.attrs("/increment_0")["t/s"]) == 2.5
    assert f.attrs("/increment_0/phase/alpha/mechanical/F")["unit"] == "1"
    assert f.read("/setup/load.yaml").item().rstrip(b"\0") == b"line one\nline two"
    rec = f.read("/cell_to/phase")
    assert rec.shape == (3, 1) and list(rec["entry"][:, 0]) == [0, 1, 2]
    assert all(x == b"alpha" for x in rec["label"][:, 0])


def test_heap_layout_like_the_hdf5_library(h5file):
    import struct
    b = open(h5file, "rb").read()
    i = b.find(b"HEAP")
    size, free, addr = struct.unpack_from("<QQQ", b, i + 8)
    assert free < size                               # free list points at a block in the segment
    nxt, fsz = struct.unpack_from("<QQ", b, addr + free)
    assert nxt == 1 and fsz == 16                    # 1 = end of the free list
