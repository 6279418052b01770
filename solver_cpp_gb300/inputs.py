"""Geometry and material inputs in the reference's formats, and a DAMASK_grid-style job.

* ``read_vti``: VTK ImageData geometry (f_VTI_readCellsSizeOrigin /
  f_VTI_readDataset_int, reference src/grid/discretization_grid.h:19-21,
  discretization_grid.cpp): cells from WholeExtent, size = cells x Spacing, origin;
  the cell data array (default "material") in ascii or base64 binary, raw or
  vtkZLibDataCompressor blocks, UInt32 or UInt64 headers, any integer type.
* ``read_material_yaml``: material.yaml (reference examples/grid/material.yaml,
  src/material.f90, phase_mechanical_plastic_phenopowerlaw.f90:75-200): one
  single-constituent homogenization, one cF phase with Hooke elasticity and
  phenopowerlaw plasticity on the 12 {111}<110> systems; per material the
  orientation O (w, x, y, z).
* ``apply_phase_numerics``: the phase.mechanical section of numerics.yaml
  (phase_mechanical.f90:277-294: cut-back, state and Lp iteration controls).
* ``grid_job``: the inputs of ``DAMASK_grid -g -m -l -n`` to a finished run with
  DADF5 results (input files stored under /setup) and optional restarts.
"""
import base64
import os
import re
import struct
import zlib

import numpy as np

from .loadcase import parse_load_yaml, parse_numerics_yaml, yaml_load

_INT_TYPES = {"Int8": "<i1", "UInt8": "<u1", "Int16": "<i2", "UInt16": "<u2", "Int32": "<i4", "UInt32": "<u4",
              "Int64": "<i8", "UInt64": "<u8", "Float32": "<f4", "Float64": "<f8"}


def _text(src):
    if isinstance(src, bytes):
        return src.decode()
    if "\n" not in src and os.path.exists(src):
        with open(src) as f:
            return f.read()
    return src


def _decode_binary(data, header_type, compressed, dtype):
    hsz = 4 if header_type == "UInt32" else 8
    hfmt = "<I" if hsz == 4 else "<Q"
    data = re.sub(r"\s+", "", data)
    if not compressed:
        # the byte-count header and the data are base64-encoded either as one stream or
        # each on its own (then the header's encoding ends in '=' padding)
        hchars = ((hsz + 2) // 3) * 4
        n = struct.unpack(hfmt, base64.b64decode(data[:hchars])[:hsz])[0]
        if "=" in data[:hchars]:
            raw = base64.b64decode(data[hchars:])[:n]
        else:
            raw = base64.b64decode(data)[hsz:hsz + n]
        return np.frombuffer(raw, dtype=dtype)
    nb = struct.unpack(hfmt, base64.b64decode(data[:((hsz + 2) // 3) * 4])[:hsz])[0]
    hlen = hsz * (3 + nb)
    hb64 = ((hlen + 2) // 3) * 4
    hdr = base64.b64decode(data[:hb64])
    sizes = struct.unpack("<%d%s" % (nb, hfmt[1]), hdr[3 * hsz:3 * hsz + hsz * nb])
    raw = base64.b64decode(data[hb64:])
    out, off = [], 0
    for s in sizes:
        out.append(zlib.decompress(raw[off:off + s]))
        off += s
    return np.frombuffer(b"".join(out), dtype=dtype)


def read_vti(src, label="material"):
    """(cells, size, origin, data) of a VTK ImageData file; data flattened x fastest."""
    text = _text(src)
    head = re.search(r"<VTKFile([^>]*)>", text)
    if not head or 'type="ImageData"' not in head.group(1):
        raise ValueError("not a VTK ImageData file")
    attrs = dict(re.findall(r'(\w+)="([^"]*)"', head.group(1)))
    if attrs.get("byte_order", "LittleEndian") != "LittleEndian":
        raise ValueError("only LittleEndian VTI files are supported")
    header_type = attrs.get("header_type", "UInt32")
    compressed = "compressor" in attrs
    if compressed and attrs["compressor"] != "vtkZLibDataCompressor":
        raise ValueError(f"unsupported compressor {attrs['compressor']}")
    img = re.search(r"<ImageData([^>]*)>", text)
    ia = dict(re.findall(r'(\w+)="([^"]*)"', img.group(1)))
    ext = [int(x) for x in ia["WholeExtent"].split()]
    cells = np.array([ext[1] - ext[0], ext[3] - ext[2], ext[5] - ext[4]])
    spacing = np.array([float(x) for x in ia["Spacing"].split()])
    origin = np.array([float(x) for x in ia.get("Origin", "0 0 0").split()])
    if np.any(cells < 1) or np.any(spacing <= 0.0):
        raise ValueError("invalid cells or spacing")
    cd = re.search(r"<CellData[^>]*>(.*?)</CellData>", text, re.S)
    if not cd:
        raise ValueError("no CellData")
    for m in re.finditer(r"<DataArray([^>]*)>(.*?)</DataArray>", cd.group(1), re.S):
        da = dict(re.findall(r'(\w+)="([^"]*)"', m.group(1)))
        if da.get("Name") != label:
            continue
        dtype = np.dtype(_INT_TYPES[da["type"]])
        fmt = da.get("format", "ascii")
        if fmt == "ascii":
            data = np.array(m.group(2).split(), dtype=dtype)
        elif fmt == "binary":
            data = _decode_binary(m.group(2), header_type, compressed, dtype)
        else:
            raise ValueError(f"unsupported DataArray format {fmt}")
        if data.size != int(np.prod(cells)):
            raise ValueError(f"{label}: {data.size} values for {int(np.prod(cells))} cells")
        return cells, cells * spacing, origin, data
    raise ValueError(f"no cell data array named {label}")


def _first(v):
    return v[0] if isinstance(v, (list, tuple)) else v


def read_material_yaml(src):
    """(dgx material, orientations (n_materials, 4), phase name, homogenization name)."""
    from . import material as _material
    doc = yaml_load(_text(src)) or {}
    phases = doc.get("phase") or {}
    homogs = doc.get("homogenization") or {}
    mats = doc.get("material") or []
    if not mats:
        raise ValueError("material.yaml: no material entries")
    used_ph, used_ho, q = set(), set(), []
    for m in mats:
        cons = m.get("constituents") or []
        if len(cons) != 1:
            raise ValueError("only single-constituent materials are supported")
        c = cons[0]
        used_ph.add(c["phase"]); used_ho.add(m["homogenization"])
        q.append([float(x) for x in c.get("O", [1.0, 0.0, 0.0, 0.0])])
    if len(used_ph) != 1 or len(used_ho) != 1:
        raise ValueError("only one phase and one homogenization are supported")
    ph_name, ho_name = used_ph.pop(), used_ho.pop()
    ho = homogs.get(ho_name) or {}
    if int(ho.get("N_constituents", 1)) != 1:
        raise ValueError("homogenization must have one constituent")
    ph = phases[ph_name]
    if ph.get("lattice") != "cF":
        raise ValueError("only the cF lattice is supported")
    mech = ph.get("mechanical") or {}
    el, pl = mech.get("elastic") or {}, mech.get("plastic") or {}
    if el.get("type") != "Hooke" or pl.get("type") != "phenopowerlaw":
        raise ValueError("only Hooke elasticity with phenopowerlaw plasticity is supported")
    if [int(x) for x in pl.get("N_sl", [12])] != [12]:
        raise ValueError("phenopowerlaw cF: N_sl must be [12]")
    if pl.get("N_tw") and any(int(x) for x in pl["N_tw"]):
        raise ValueError("twinning is not supported")
    mat = _material(C11=float(el["C_11"]), C12=float(el["C_12"]), C44=float(el["C_44"]),
                    xi_0=float(_first(pl["xi_0_sl"])), xi_inf=float(_first(pl["xi_inf_sl"])),
                    h_0=float(_first(pl["h_0_sl-sl"])), n=float(_first(pl["n_sl"])),
                    dot_gamma_0=float(_first(pl["dot_gamma_0_sl"])), a=float(_first(pl["a_sl"])))
    h = [float(x) for x in pl["h_sl-sl"]]
    if len(h) < 7:
        raise ValueError("h_sl-sl needs the 7 cF interaction values")
    for i in range(7):
        mat.h_sl_sl[i] = h[i]
    if "atol_xi" in pl:
        mat.atol_xi = float(pl["atol_xi"])
    if "c_1" in pl:
        mat.c_1 = float(pl["c_1"])
    if "c_2" in pl:
        mat.c_2 = float(pl["c_2"])
    return mat, np.array(q), ph_name, ho_name


def apply_phase_numerics(text, mat):
    """phase.mechanical (and .plastic) keys of numerics.yaml into the material's integration controls."""
    doc = yaml_load(_text(text)) or {}
    mech = ((doc.get("phase") or {}).get("mechanical")) or {}
    plast = mech.get("plastic") or {}
    for key, attr, conv in (("r_cutback_min", "r_cutback_min", float), ("r_cutback", "r_cutback", float),
                            ("r_increase", "r_increase", float), ("eps_rel_state", "eps_rel_state", float),
                            ("N_iter_state_max", "N_iter_state_max", int)):
        if key in mech:
            setattr(mat, attr, conv(mech[key]))
    for key, attr, conv in (("N_iter_Lp_max", "N_iter_Lp_max", int), ("r_linesearch_Lp", "r_linesearch_Lp", float),
                            ("eps_rel_Lp", "eps_rel_Lp", float), ("eps_abs_Lp", "eps_abs_Lp", float),
                            ("f_update_jacobi_Lp", "f_update_jacobi_Lp", int)):
        if key in plast:
            setattr(mat, attr, conv(plast[key]))
    return mat


def grid_job(geometry, material, load, numerics=None, result=None, restart=None, restart_every=0, precision="fp64"):
    """Run a DAMASK_grid job from its input files (paths or text).  Returns
    (RVE, per-increment records); the RVE stays alive for further queries."""
    from . import RVE, numerics as _numerics
    gtext, mtext, ltext = _text(geometry), _text(material), _text(load)
    cells, size, origin, mat_at = read_vti(gtext)
    mat, q, ph, ho = read_material_yaml(mtext)
    if mat_at.min() < 0 or mat_at.max() >= len(q):
        raise ValueError("geometry refers to materials not in material.yaml")
    num = _numerics(precision=precision)
    if numerics is not None:
        ntext = _text(numerics)
        num = parse_numerics_yaml(ntext, num)
        mat = apply_phase_numerics(ntext, mat)
    steps = parse_load_yaml(ltext)
    rve = RVE(cells, size, mat_at.astype(np.int32), q, mat=mat, num=num)
    setup = {"geometry.vti": gtext, "material.yaml": mtext, "load.yaml": ltext}
    if numerics is not None:
        setup["numerics.yaml"] = _text(numerics)
    recs = rve.loop_over_loadcase(steps, result=result, restart=restart, restart_every=restart_every, phase=ph,
                                  homogenization=ho, setup=setup if result is not None else None)
    return rve, recs
