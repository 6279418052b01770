"""Shared inputs for the parity tests (fixtures committed under tests/golden/)."""
import base64
import json
import os
import re
import struct
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def damask_6grains():
    return np.load(os.path.join(HERE, "golden", "damask_6grains6x7x8_tensionY.npz"))


def vti_material(text):
    """cells, size, material_at of a VTK ImageData file with a zlib-compressed Int64 'material'."""
    ext = [int(x) for x in re.search(r'WholeExtent="([^"]+)"', text).group(1).split()]
    cells = [ext[1] - ext[0], ext[3] - ext[2], ext[5] - ext[4]]
    sp = [float(x) for x in re.search(r'Spacing="([^"]+)"', text).group(1).split()]
    da = re.search(r'<DataArray type="(\w+)" Name="material" format="binary"[^>]*>\s*([^<]+?)\s*</DataArray>', text)
    data = da.group(2).strip()
    nb = struct.unpack("<I", base64.b64decode(data[:8])[:4])[0]
    hb64 = ((4 * (3 + nb) + 2) // 3) * 4
    hdr = base64.b64decode(data[:hb64])
    sizes = struct.unpack("<%dI" % nb, hdr[12:12 + 4 * nb])
    raw = base64.b64decode(data[hb64:])
    out, off = b"", 0
    for s in sizes:
        out += zlib.decompress(raw[off:off + s]); off += s
    return cells, [sp[i] * cells[i] for i in range(3)], np.frombuffer(out, dtype="<i8").astype(np.int32)


def grains16():
    """The reference's 16x16x16, 20-grain VTI (src/grid/test/test_discretization_grid.cpp)."""
    with open(os.path.join(HERE, "golden", "reference_knowns.json")) as f:
        k = json.load(f)
    return vti_material(k["vti_16x16x16"]["content"])


def random_F(n, seed, amp=1e-3):
    rng = np.random.default_rng(seed)
    return np.eye(3)[None] + amp * rng.standard_normal((n, 3, 3))
