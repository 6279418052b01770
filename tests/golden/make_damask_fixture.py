"""Extract the reference's complete Fortran DAMASK result into a small fixture.

Source (reference tree, read-only): python/tests/resources/Result/
  6grains6x7x8_single_phase.vti, 6grains6x7x8_single_phase.material.yaml,
  6grains6x7x8_single_phase_tensionY.hdf5  (DAMASK_grid 3.0.0-alpha7-366, tensionY.yaml:
  dot_F_yy = 1e-3/s, P_xx = P_zz = 0, t = 20 s, N = 40, f_out = 4, default numerics)
Writes tests/golden/damask_6grains6x7x8_tensionY.npz with the material map,
orientations, volume averages of F and P at every written increment and the
fields F, P, F_e, F_p, L_p, xi_sl, O (orientation quaternion) and the displacements
u_p (cell centres) and u_n (nodes) at increments 20 and 40 (HDF5 C order:
[cell][i][j]), and the list of datasets of one increment group (DADF5 layout).

    python tests/golden/make_damask_fixture.py /path/to/reference
"""
import base64
import os
import re
import struct
import sys
import zlib

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from hdf5lite import HDF5File  # noqa: E402


def read_vti_material(text):
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


def main(ref):
    R = os.path.join(ref, "python", "tests", "resources", "Result")
    cells, size, mat = read_vti_material(open(os.path.join(R, "6grains6x7x8_single_phase.vti")).read())
    y = open(os.path.join(R, "6grains6x7x8_single_phase.material.yaml")).read()
    O = np.array([[float(x) for x in m.split(",")] for m in re.findall(r"O: \[([^\]]+)\]", y)])
    f = HDF5File(os.path.join(R, "6grains6x7x8_single_phase_tensionY.hdf5"))
    ph = "/phase/pheno_fcc/mechanical/"
    incs = list(range(0, 41, 4))
    P_av = np.array([f.read(f"/increment_{i}{ph}P").mean(0) for i in incs])
    F_av = np.array([f.read(f"/increment_{i}{ph}F").mean(0) for i in incs])
    out = dict(cells=np.array(cells), size=np.array(size), material_at=mat, orientations=O,
               increments=np.array(incs), P_av=P_av, F_av=F_av)
    for inc in (20, 40):
        for name in ("F", "P", "F_e", "F_p", "L_p", "xi_sl", "O"):
            out[f"{name}_{inc}"] = f.read(f"/increment_{inc}{ph}{name}")
        for name in ("u_p", "u_n"):
            out[f"{name}_{inc}"] = f.read(f"/increment_{inc}/geometry/{name}")
    layout = []
    for g in ("geometry", "phase/pheno_fcc/mechanical", "homogenization/SX/mechanical"):
        for k in f.keys(f"/increment_40/{g}"):
            layout.append(f"{g}/{k}")
    out["layout_increment"] = np.array(sorted(layout))
    out["layout_root"] = np.array(sorted(f.keys("/")))
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "damask_6grains6x7x8_tensionY.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst, os.path.getsize(dst), "bytes")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {os.path.basename(__file__)} <path of the reference checkout>")
    main(sys.argv[1])
