"""polymlp.yaml and legacy polymlp.lammps model files.

`save_mlp_yaml` writes a fitted model (params dict, coefficients and feature
scales) in the text layout of the reference's writer
(src/pypolymlp/core/io_polymlp_yaml.py:17-94): the file the reference's C++
parser (cxx/src/polymlp/polymlp_parse_potential.cpp:214-257) and LAMMPS read,
coefficients written as c / s with 15 decimals of mantissa.  `save_mlp_lammps`
writes the legacy line format that io_polymlp_legacy.py:23-161 and
polymlp_parse_potential_legacy.cpp read (one value list per line, "# tag"
comments, elements line tagged "# element").  `load_mlp_yaml`,
`load_mlp_lammps` and `load_mlp` (dispatch on the legacy tag,
io_polymlp.py:59-76, 142-156) read both back as a params dict of the form
`make_params_dict` builds and the coefficients divided by the scales.  The
invariant tables of a gtinv model are screened from the reference's basis
for the file's gtinv order, l_max and version (`gtinv.Readgtinv`).
"""

from __future__ import annotations

import ast
import os
from typing import Optional, Sequence

import numpy as np

from pypolymlp_gb300.params import expand_spins, load_gtinv

# Standard atomic weights (IUPAC, abridged) for the mass entry of the files.
ATOMIC_MASS = {
    "H": 1.008, "He": 4.003, "Li": 6.94, "Be": 9.012, "B": 10.81, "C": 12.011, "N": 14.007, "O": 15.999,
    "F": 18.998, "Ne": 20.18, "Na": 22.99, "Mg": 24.305, "Al": 26.982, "Si": 28.085, "P": 30.974, "S": 32.06,
    "Cl": 35.45, "Ar": 39.95, "K": 39.098, "Ca": 40.078, "Sc": 44.956, "Ti": 47.867, "V": 50.942, "Cr": 51.996,
    "Mn": 54.938, "Fe": 55.845, "Co": 58.933, "Ni": 58.693, "Cu": 63.546, "Zn": 65.38, "Ga": 69.723,
    "Ge": 72.63, "As": 74.922, "Se": 78.971, "Br": 79.904, "Kr": 83.798, "Rb": 85.468, "Sr": 87.62,
    "Y": 88.906, "Zr": 91.224, "Nb": 92.906, "Mo": 95.95, "Tc": 98.0, "Ru": 101.07, "Rh": 102.906,
    "Pd": 106.42, "Ag": 107.868, "Cd": 112.414, "In": 114.818, "Sn": 118.71, "Sb": 121.76, "Te": 127.6,
    "I": 126.904, "Xe": 131.293, "Cs": 132.905, "Ba": 137.327, "La": 138.905, "Ce": 140.116, "Pr": 140.908,
    "Nd": 144.242, "Pm": 145.0, "Sm": 150.36, "Eu": 151.964, "Gd": 157.25, "Tb": 158.925, "Dy": 162.5,
    "Ho": 164.93, "Er": 167.259, "Tm": 168.934, "Yb": 173.045, "Lu": 174.967, "Hf": 178.49, "Ta": 180.948,
    "W": 183.84, "Re": 186.207, "Os": 190.23, "Ir": 192.217, "Pt": 195.084, "Au": 196.967, "Hg": 200.592,
    "Tl": 204.38, "Pb": 207.2, "Bi": 208.98, "Th": 232.038, "U": 238.029,
}


def _masses(elements: Sequence[str], mass: Optional[Sequence[float]]):
    if mass is not None:
        if len(mass) != len(elements):
            raise ValueError("one mass per element")
        return [float(m) for m in mass]
    return [ATOMIC_MASS.get(str(e), 0.0) for e in elements]


def _model_parts(params_dict: dict):
    """(model, n_type, elements, type pairs with radial ids), element-level: for a
    model with spins (params.expand_spins) the elements before the split, each
    element pair taking the radial ids of its first types."""
    m = params_dict["model"]
    sp = params_dict.get("spin_elements")
    if sp:
        elements = list(sp["elements"])
        n_type = len(elements)
        first = [int(t[0]) for t in sp["types"]]
    else:
        n_type = int(params_dict["n_type"])
        elements = list(params_dict.get("elements") or [f"E{i}" for i in range(n_type)])
        first = list(range(n_type))
    cond = m.get("pair_params_conditional") or {}
    pairs = []
    for i in range(n_type):
        for j in range(i, n_type):
            a, b = first[i], first[j]
            ids = cond.get((a, b), cond.get(f"{a},{b}"))
            if ids is None:
                ids = list(range(len(m["pair_params"])))
            pairs.append(((i, j), [int(v) for v in ids]))
    return m, n_type, elements, pairs


def _fmt_list(values) -> str:
    return "[" + ", ".join(repr(v) for v in values) + "]"


def save_mlp_yaml(params_dict: dict, coeffs, scales, filename: str = "polymlp.yaml",
                  mass: Optional[Sequence[float]] = None) -> None:
    """Write polymlp.yaml; the stored coefficients are coeffs / scales."""
    m, n_type, elements, pairs = _model_parts(params_dict)
    c = np.asarray(coeffs, dtype=np.float64) / np.asarray(scales, dtype=np.float64)
    gt = m.get("gtinv") or {}
    sp = params_dict.get("spin_elements")
    spins = [int(bool(v)) for v in sp["enable_spins"]] if sp else [0] * n_type
    type_elements = list(params_dict["elements"]) if sp else elements
    lines = [
        f"elements:      [{', '.join(str(e) for e in elements)}]",
        f"enable_spins:  {_fmt_list(spins)}",
        f"cutoff:        {float(m['cutoff'])!r}",
        f"pair_type:     {m.get('pair_type', 'gaussian')}",
        f"feature_type:  {m['feature_type']}",
        f"model_type:    {int(m['model_type'])}",
        f"max_p:         {int(m['max_p'])}",
        f"max_l:         {int(m['max_l'])}",
        "",
    ]
    if m["feature_type"] == "gtinv":
        maxl = [int(v) for v in gt["max_l"]]
        lines += [
            f"gtinv_order:   {int(gt['order'])}",
            f"gtinv_maxl:    {_fmt_list(maxl)}",
            f"gtinv_sym:     {_fmt_list([0] * len(maxl))}",
            f"gtinv_version: {int(gt.get('version', 1))}",
            "",
        ]
    lines += [
        "electrostatic: 0",
        f"mass:          {_fmt_list(_masses(type_elements, mass))}",
        "",
        f"n_pair_params: {len(m['pair_params'])}",
        "pair_params:",
    ]
    lines += [f"- {_fmt_list([float(a) for a in p])}" for p in m["pair_params"]]
    lines += ["", f"n_type_pairs: {len(pairs)}", "type_pairs:"]
    for (i, j), ids in pairs:
        lines += [f"- atom_type_pair:      {_fmt_list([i, j])}", f"  pair_params_indices: {_fmt_list(ids)}"]
    tfull = 1 if params_dict.get("type_full", True) in (True, 1, None) else 0
    tidx = [int(v) for v in params_dict.get("type_indices", list(range(n_type)))]
    lines += ["", f"type_full:    {tfull}", f"type_indices: {_fmt_list(tidx)}", "",
              f"n_coeffs: {len(c)}", "coeffs: [" + ", ".join(f"{v:.15e}" for v in c) + "]"]
    with open(filename, "w") as f:
        f.write("\n".join(lines) + "\n")


def save_mlp_lammps(params_dict: dict, coeffs, scales, filename: str = "polymlp.lammps",
                    mass: Optional[Sequence[float]] = None) -> None:
    """Write the legacy polymlp.lammps format (coefficients and scales on separate lines)."""
    if params_dict.get("spin_elements"):
        raise ValueError("the legacy polymlp.lammps format has no spin entries: use save_mlp_yaml")
    m, n_type, elements, pairs = _model_parts(params_dict)
    c = np.asarray(coeffs, dtype=np.float64)
    s = np.asarray(scales, dtype=np.float64)
    gt = m.get("gtinv") or {}
    gtinv = m["feature_type"] == "gtinv"
    lines = [" ".join(str(e) for e in elements) + " # element",
             f"{float(m['cutoff'])!r} # cutoff", f"{m.get('pair_type', 'gaussian')} # pair_type",
             f"{m['feature_type']} # feature_type", f"{int(m['model_type'])} # model_type",
             f"{int(m['max_p'])} # max power", f"{int(m['max_l'])} # max l"]
    if gtinv:
        maxl = [int(v) for v in gt["max_l"]][: int(gt["order"]) - 1]
        lines += [f"{int(gt['order'])} # gtinv_order", " ".join(map(str, maxl)) + " # gtinv_maxl",
                  " ".join("0" for _ in maxl) + " # gtinv_sym"]
    lines += [f"{len(c)} # n_coeffs", " ".join(repr(float(v)) for v in c) + " # reg. coeffs",
              " ".join(repr(float(v)) for v in s) + " # scales", f"{len(m['pair_params'])} # n_params"]
    lines += [f"{float(p[0])!r} {float(p[1])!r} # pair params" for p in m["pair_params"]]
    lines += [" ".join(repr(v) for v in _masses(elements, mass)) + " # mass", "0 # electrostatic"]
    if gtinv:
        lines += [f"{int(gt.get('version', 1))} # gtinv_version"]
    lines += [f"{len(pairs)} # n_type_pairs"]
    for (i, j), ids in pairs:
        lines += [f"{i} {j} {len(ids)} # atom type pair", " ".join(map(str, ids)) + " # pair params indices"]
    tfull = 1 if params_dict.get("type_full", True) in (True, 1, None) else 0
    tidx = [int(v) for v in params_dict.get("type_indices", list(range(n_type)))]
    lines += [f"{tfull} # type_full", " ".join(map(str, tidx)) + " # type_indices"]
    with open(filename, "w") as f:
        f.write("\n".join(lines) + "\n")


def _scalar(text: str):
    for conv in (int, float):
        try:
            return conv(text)
        except ValueError:
            pass
    return text


def _value(text: str):
    text = text.strip()
    if text.startswith("["):
        try:
            return ast.literal_eval(text)
        except (ValueError, SyntaxError):
            inner = text[1:-1].strip()
            return [_scalar(t.strip()) for t in inner.split(",")] if inner else []
    return _scalar(text)


def _parse_yaml(text: str) -> dict:
    """The flat YAML subset of polymlp.yaml: `key: value`, block lists of
    `- value` and of `- atom_type_pair: ...` / `  pair_params_indices: ...`."""
    out, block = {}, None
    for raw in text.splitlines():
        line = raw.split("#", 1)[0].rstrip()
        if not line.strip():
            continue
        if line.startswith("- ") or line.startswith("  "):
            body = line[2:]
            if block is None:
                raise ValueError(f"list item outside a list: {raw!r}")
            if ":" in body and not body.lstrip().startswith("["):
                k, _, v = body.partition(":")
                if line.startswith("- "):
                    out[block].append({})
                out[block][-1][k.strip()] = _value(v)
            else:
                out[block].append(_value(body))
            continue
        key, _, rest = line.partition(":")
        if rest.strip():
            out[key.strip()] = _value(rest)
            block = None
        else:
            block = key.strip()
            out[block] = []
    return out


def params_from_model(n_type: int, elements, cutoff: float, model_type: int, max_p: int, max_l: int,
                      feature_type: str, pair_params, cond: dict, gtinv_order: int = 0,
                      gtinv_maxl: Sequence[int] = (), gtinv_version: int = 1, pair_type: str = "gaussian") -> dict:
    """A params dict (the `make_params_dict` form) from explicit model settings."""
    if feature_type == "gtinv":
        l_comb, lm_seq, lm_coeffs = load_gtinv(gtinv_order, gtinv_maxl, gtinv_version)
        gtinv = {"order": int(gtinv_order), "max_l": [int(v) for v in gtinv_maxl], "n_type": n_type,
                 "lm_seq": lm_seq, "l_comb": l_comb, "lm_coeffs": lm_coeffs, "version": int(gtinv_version)}
    else:
        gtinv = {"order": 0, "max_l": [], "n_type": n_type, "lm_seq": [], "l_comb": [], "lm_coeffs": [],
                 "version": 1}
        max_l = 0
    return {
        "n_type": int(n_type),
        "elements": [str(e) for e in elements],
        "model": {
            "cutoff": float(cutoff), "model_type": int(model_type), "max_p": int(max_p), "max_l": int(max_l),
            "feature_type": feature_type, "gtinv": gtinv, "pair_type": pair_type, "pair_conditional": True,
            "pair_params": [[float(a), float(b)] for a, b in pair_params],
            "pair_params_conditional": {tuple(int(v) for v in k): [int(i) for i in ids] for k, ids in cond.items()},
        },
        "include_force": True,
        "include_stress": True,
        "print_memory": False,
        "alphas": None,
    }


def load_mlp_yaml(filename: str = "polymlp.yaml"):
    """(params dict, coefficients) of a polymlp.yaml file."""
    with open(filename) as f:
        y = _parse_yaml(f.read())
    elements = y["elements"]
    cond = {tuple(tp["atom_type_pair"]): tp["pair_params_indices"] for tp in y.get("type_pairs", [])}
    gt = y["feature_type"] == "gtinv"
    p = params_from_model(len(elements), elements, y["cutoff"], y["model_type"], y["max_p"], y["max_l"],
                          y["feature_type"], y["pair_params"], cond,
                          gtinv_order=y.get("gtinv_order", 0) if gt else 0,
                          gtinv_maxl=y.get("gtinv_maxl", []) if gt else [],
                          gtinv_version=y.get("gtinv_version", 1) if gt else 1, pair_type=y.get("pair_type", "gaussian"))
    p["mass"] = [float(v) for v in y.get("mass", [])]
    p["type_full"] = bool(y.get("type_full", 1))
    p["type_indices"] = [int(v) for v in y.get("type_indices", list(range(len(elements))))]
    # spin-enabled elements become two atom types each (io_polymlp_yaml.py:111-116, 146-150)
    expand_spins(p, y.get("enable_spins"))
    return p, np.asarray(y["coeffs"], dtype=np.float64)


def load_mlp_lammps(filename: str = "polymlp.lammps"):
    """(params dict, coefficients / scales) of a legacy polymlp.lammps file."""
    with open(filename) as f:
        lines = [ln for ln in f.read().splitlines()]
    pos = [0]

    def values(conv=_scalar):
        line = lines[pos[0]]
        pos[0] += 1
        return [conv(t) for t in line.split("#", 1)[0].split()]

    def tagged(tag):
        return pos[0] < len(lines) and tag in lines[pos[0]]

    elements = values(str)
    n_type = len(elements)
    cutoff, = values(float)
    pair_type, = values(str)
    feature_type, = values(str)
    model_type, = values(int)
    max_p, = values(int)
    max_l, = values(int)
    gtinv_order, gtinv_maxl = 0, []
    if feature_type == "gtinv":
        gtinv_order, = values(int)
        gtinv_maxl = values(int)
        values()  # gtinv_sym
    values()  # n_coeffs
    coeffs = np.asarray(values(float), dtype=np.float64)
    scales = np.asarray(values(float), dtype=np.float64)
    n_params, = values(int)
    pair_params = [values(float)[:2] for _ in range(n_params)]
    mass = values(float)
    values()  # electrostatic
    version = 1
    if feature_type == "gtinv" and tagged("gtinv_version"):
        version, = values(int)
    cond = {}
    if tagged("n_type_pairs"):
        n_pairs, = values(int)
        for _ in range(n_pairs):
            i, j = values(int)[:2]
            cond[(i, j)] = values(int)
    else:
        for i in range(n_type):
            for j in range(i, n_type):
                cond[(i, j)] = list(range(n_params))
    type_full, type_indices = True, list(range(n_type))
    if tagged("type_full"):
        type_full = values(lambda t: t.lower() in ("1", "true", "t", "yes", "y", "on"))[0]
        type_indices = values(int)
    p = params_from_model(n_type, elements, cutoff, model_type, max_p, max_l, feature_type, pair_params, cond,
                          gtinv_order=gtinv_order, gtinv_maxl=gtinv_maxl, gtinv_version=version,
                          pair_type=pair_type)
    p["mass"] = [float(v) for v in mass]
    p["type_full"] = type_full
    p["type_indices"] = type_indices
    return p, coeffs / scales


def is_legacy(filename: str) -> bool:
    with open(filename) as f:
        return "# ele" in f.readline()


def load_mlp(filename: str):
    """(params dict, coefficients) of either format."""
    return load_mlp_lammps(filename) if is_legacy(filename) else load_mlp_yaml(filename)


def convert_to_yaml(lammps_file: str, yaml_file: str = "polymlp.yaml") -> bool:
    """Rewrite a legacy file as polymlp.yaml (False if it is not legacy)."""
    if not is_legacy(lammps_file):
        return False
    p, c = load_mlp_lammps(lammps_file)
    save_mlp_yaml(p, c, np.ones(len(c)), yaml_file, mass=p.get("mass") or None)
    return True


def find_mlps(path: str):
    """polymlp.yaml* files of a directory, else polymlp.lammps*, sorted (None if neither)."""
    names = sorted(os.listdir(path)) if os.path.isdir(path) else []
    for prefix in ("polymlp.yaml", "polymlp.lammps"):
        hits = [os.path.join(path, n) for n in names if n.startswith(prefix)]
        if hits:
            return hits
    return None
