"""Load-case and numerics inputs in the reference's YAML formats.

``parse_load_yaml`` reads the load file of ``DAMASK_grid -l`` (reference
src/grid/config.cpp:247-358: solver.mechanical, loadstep list with
boundary_conditions.mechanical {dot_F|F|L} and {P|dot_P} 3x3 matrices where 'x'
marks an unprescribed component (a step without P / dot_P prescribes no stress, as
in the reference's examples/grid/shearZX.yaml), optional R quaternion, discretization {t, N, r},
f_out, estimate_rate) and returns dgx_loadstep structures.  ``parse_numerics_yaml``
reads solver.grid (config.cpp:360-464).  The YAML subset understood here is
block mappings/sequences plus flow sequences and flow mappings -- what the
reference's example inputs use.
"""
import re

import numpy as np

from . import dgx as _d


# ---------------------------------------------------------------- minimal YAML subset
def _scalar(tok):
    tok = tok.strip()
    if tok == "":
        return None
    if tok[0] in "\"'" and tok[-1] == tok[0]:
        return tok[1:-1]
    low = tok.lower()
    if low in ("true", "yes", "on"):
        return True
    if low in ("false", "no", "off"):
        return False
    try:
        if re.fullmatch(r"[+-]?\d+", tok):
            return int(tok)
        return float(tok)
    except ValueError:
        return tok


def _flow(text):
    """Parse a flow collection ([...] or {...}) into python objects."""
    pos = 0

    def skip():
        nonlocal pos
        while pos < len(text) and text[pos] in " \t\r\n":
            pos += 1

    def value():
        nonlocal pos
        skip()
        if text[pos] == "[":
            pos += 1
            out = []
            skip()
            if text[pos] == "]":
                pos += 1
                return out
            while True:
                out.append(value())
                skip()
                if text[pos] == ",":
                    pos += 1
                    continue
                if text[pos] == "]":
                    pos += 1
                    return out
                raise ValueError("bad flow sequence")
        if text[pos] == "{":
            pos += 1
            out = {}
            skip()
            if text[pos] == "}":
                pos += 1
                return out
            while True:
                skip()
                m = re.compile(r"([^:,{}\[\]]+):").match(text, pos)
                if not m:
                    raise ValueError("bad flow mapping")
                key = m.group(1).strip()
                pos = m.end()
                out[key] = value()
                skip()
                if text[pos] == ",":
                    pos += 1
                    continue
                if text[pos] == "}":
                    pos += 1
                    return out
                raise ValueError("bad flow mapping")
        m = re.compile(r"[^,\]}]+").match(text, pos)
        pos = m.end()
        return _scalar(m.group(0))

    v = value()
    return v


def yaml_load(text):
    lines = []
    for raw in text.splitlines():
        s = raw.split("#", 1)[0].rstrip() if "#" in raw else raw.rstrip()
        if s.strip() in ("", "---", "..."):
            continue
        lines.append(s)
    # join multi-line flow collections
    joined, buf, depth = [], "", 0
    for s in lines:
        if depth > 0:
            buf += " " + s.strip()
        else:
            buf = s
        depth += s.count("[") + s.count("{") - s.count("]") - s.count("}")
        if depth <= 0:
            joined.append(buf)
            depth = 0
    items = [(len(s) - len(s.lstrip(" ")), s.strip()) for s in joined]
    pos = 0

    def parse_block(indent):
        nonlocal pos
        if pos >= len(items):
            return None
        if items[pos][1].startswith("- ") or items[pos][1] == "-":
            out = []
            while pos < len(items) and items[pos][0] == indent and (items[pos][1].startswith("-")):
                ind, s = items[pos]
                rest = s[1:].strip()
                if rest == "":
                    pos += 1
                    out.append(parse_block(items[pos][0]))
                    continue
                # "- key: value" starts a mapping whose further keys are indented to the key column
                col = ind + (len(s) - len(rest))
                items[pos] = (col, rest)
                if re.match(r"^[^\[\]{}]+:(\s|$)", rest):
                    out.append(parse_block(col))
                else:
                    pos += 1
                    out.append(_flow(rest) if rest[0] in "[{" else _scalar(rest))
            return out
        out = {}
        while pos < len(items) and items[pos][0] == indent:
            s = items[pos][1]
            m = re.match(r"^([^:]+?):(\s+(.*))?$", s)
            if not m:
                raise ValueError(f"cannot parse line: {s}")
            key, val = m.group(1).strip(), (m.group(3) or "").strip()
            pos += 1
            if val == "":
                if pos < len(items) and items[pos][0] > indent:
                    out[key] = parse_block(items[pos][0])
                elif pos < len(items) and items[pos][0] == indent and items[pos][1].startswith("-"):
                    out[key] = parse_block(indent)
                else:
                    out[key] = None
            elif val[0] in "[{":
                out[key] = _flow(val)
            else:
                out[key] = _scalar(val)
        return out

    return parse_block(items[0][0]) if items else {}


# ---------------------------------------------------------------- load steps
def _matrix(rows):
    vals = np.zeros((3, 3)); mask = np.zeros((3, 3), dtype=int)
    if len(rows) != 3 or any(len(r) != 3 for r in rows):
        raise ValueError("expected a 3x3 matrix")
    for i in range(3):
        for j in range(3):
            v = rows[i][j]
            if isinstance(v, str):
                if v != "x":
                    raise ValueError("invalid string value in matrix: expected 'x'")
                mask[i, j] = 1
            else:
                vals[i, j] = float(v)
    return vals, mask


def _fill(step, prefix, vals, mask):
    for i in range(3):
        for j in range(3):
            getattr(step, prefix + "_values")[i + 3 * j] = vals[i, j]
            getattr(step, prefix + "_mask")[i + 3 * j] = int(mask[i, j])


def make_step(def_type, def_values, def_mask, stress_type, stress_values, stress_mask, t, N, r=1.0, f_out=1,
              estimate_rate=True, rot=(1.0, 0.0, 0.0, 0.0)):
    s = _d.LoadStep()
    s.def_type = {"F": 0, "dot_F": 1, "L": 2}[def_type] if isinstance(def_type, str) else int(def_type)
    s.stress_type = {"P": 0, "dot_P": 1}[stress_type] if isinstance(stress_type, str) else int(stress_type)
    _fill(s, "def", np.asarray(def_values, float), np.asarray(def_mask, int))
    _fill(s, "stress", np.asarray(stress_values, float), np.asarray(stress_mask, int))
    for k in range(4):
        s.rot_q[k] = float(rot[k])
    s.t = float(t); s.N = int(N); s.r = float(r); s.f_out = int(f_out); s.estimate_rate = int(bool(estimate_rate))
    return s


def load_step(kind="tensionX", t=20.0, N=20, rate=1e-3, f_out=1, r=1.0, estimate_rate=True):
    """Standard load steps: 'tensionX|Y|Z' (dot_F on the axis, the other normal
    P components 0, the remaining components free) and 'shearXY' (dot_F_xy)."""
    dv = np.zeros((3, 3)); dm = np.zeros((3, 3), int)
    sv = np.zeros((3, 3)); sm = np.ones((3, 3), int)
    axes = {"tensionX": 0, "tensionY": 1, "tensionZ": 2}
    if kind in axes:
        a = axes[kind]
        dv[a, a] = rate
        for i in range(3):
            if i != a:
                dm[i, i] = 1
                sm[i, i] = 0
    elif kind == "shearXY":
        dv[0, 1] = rate
    else:
        raise ValueError(kind)
    return make_step("dot_F", dv, dm, "P", sv, sm, t, N, r=r, f_out=f_out, estimate_rate=estimate_rate)


def parse_load_yaml(text):
    doc = yaml_load(text)
    solver = doc.get("solver")
    if not isinstance(solver, dict) or solver.get("mechanical") != "spectral_basic":
        raise ValueError("load case needs solver.mechanical: spectral_basic")
    steps = []
    for item in doc.get("loadstep") or []:
        bc = item["boundary_conditions"]["mechanical"]
        defs = [k for k in ("F", "dot_F", "L") if k in bc]
        strs = [k for k in ("P", "dot_P") if k in bc]
        if len(defs) != 1 or len(strs) > 1:
            raise ValueError("exactly one deformation and at most one stress specification per load step")
        dv, dm = _matrix(bc[defs[0]])
        if strs:
            sv, sm = _matrix(bc[strs[0]])
        else:                  # no stress specification: no stress component prescribed
            strs = ["P"]
            sv, sm = np.zeros((3, 3)), np.ones((3, 3), dtype=int)
        disc = item["discretization"]
        rot = bc.get("R", (1.0, 0.0, 0.0, 0.0))
        if not isinstance(rot, (list, tuple)) or len(rot) != 4:
            raise ValueError("R of a load step must have exactly 4 elements (quaternion w, x, y, z)")
        steps.append(make_step(defs[0], dv, dm, strs[0], sv, sm, disc["t"], disc["N"], r=disc.get("r", 1.0),
                               f_out=item.get("f_out", 1), estimate_rate=item.get("estimate_rate", True), rot=rot))
    return steps


def parse_numerics_yaml(text, num=None):
    from . import numerics as _numerics
    n = num if num is not None else _numerics()
    doc = yaml_load(text) or {}
    grid = ((doc.get("solver") or {}).get("grid")) or {}
    if "N_staggered_iter_max" in grid:
        n.stag_iter_max = int(grid["N_staggered_iter_max"])
    if "N_cutback_max" in grid:
        n.max_cut_back = int(grid["N_cutback_max"])
    mech = grid.get("mechanical") or {}
    for key, attr in (("N_iter_min", "itmin"), ("N_iter_max", "itmax")):
        if key in mech:
            setattr(n, attr, int(mech[key]))
    for key, attr in (("eps_abs_div(P)", "eps_abs_div"), ("eps_rel_div(P)", "eps_rel_div"),
                      ("eps_abs_P", "eps_abs_P"), ("eps_rel_P", "eps_rel_P")):
        if key in mech:
            setattr(n, attr, float(mech[key]))
    if "update_gamma" in mech:
        n.update_gamma = int(bool(mech["update_gamma"]))
    fft = grid.get("FFT") or {}
    if "divergence_correction" in fft:
        n.divergence_correction = {"none": 0, "size": 1, "size+grid": 2, "grid+size": 2}[fft["divergence_correction"]]
    if "derivative" in fft:
        n.derivative = {"continuous": 0, "central_difference": 1, "FWBW_difference": 2}[fft["derivative"]]
    return n
