"""Model-parameter dictionaries in the reference's FFI format.

`make_params_dict` builds the dictionary that ``PolymlpParamsSingle.as_dict()``
produces (src/pypolymlp/core/data_format.py:268) for the settings of
``set_all_params`` (src/pypolymlp/core/params_utils.py:141): Gaussian radial
parameters as ``set_gaussian_params`` makes them (product of two linspaces,
plus the constant (0, 0) function appended at the end, params_utils.py:69-93),
and every radial function active for every type pair.  The gtinv tables
(l_comb, lm_seq, lm_coeffs) are the reference's invariant tables for the
chosen order and l_max, screened from the reference's basis by
`gtinv.Readgtinv` (src/pypolymlp/cxx/src/polymlp/polymlp_read_gtinv.cpp:12).
"""

from __future__ import annotations

import itertools
import json
from typing import Optional, Sequence

import numpy as np

from pypolymlp_gb300.gtinv import get_gtinv_attrs


def load_gtinv(order: int, maxl: Sequence[int], version: int = 1):
    """(l_comb, lm_seq, lm_coeffs) of the invariants up to `order` (gtinv.Readgtinv)."""
    return get_gtinv_attrs(order, maxl, version)


def gaussian_params(params1=(1.0, 1.0, 1), params2=(0.0, 5.0, 7), n_gaussians: Optional[int] = None,
                    cutoff: Optional[float] = None):
    """(beta, mu) of the Gaussian radial functions, the constant (0, 0) last
    (params_utils.py:69-93): the product of two linspaces, or with n_gaussians
    n-1 centres spread over [0, cutoff - 1] with width max(1, spacing)."""
    if n_gaussians is None:
        g1 = np.linspace(float(params1[0]), float(params1[1]), int(params1[2]))
        g2 = np.linspace(float(params2[0]), float(params2[1]), int(params2[2]))
        pp = [[float(a), float(b)] for a, b in itertools.product(g1, g2)]
    else:
        if cutoff is None:
            raise RuntimeError("Cutoff required for automatic setting of Gaussians.")
        if int(n_gaussians) < 3:
            raise ValueError("n_gaussians must be at least 3 (two Gaussians set the width)")
        mu = np.linspace(0.0, 1.0, int(n_gaussians) - 1) * (float(cutoff) - 1.0)
        width = max(1.0, float(mu[1] - mu[0]))
        pp = [[width, float(m)] for m in mu]
    pp.append([0.0, 0.0])
    return pp


def active_gaussian_params(pair_params, elements: Sequence[str], distance: Optional[dict] = None):
    """Radial ids per type pair (i <= j) and whether they are conditional
    (params_utils.py:96-140): without `distance` every function for every pair;
    for an element pair given typical distances, the constant function and each
    Gaussian whose centre lies within 1/beta of one of them."""
    elements = list(elements)
    given = {}
    for pair, dis in (distance or {}).items():
        if len(pair) != 2:
            raise RuntimeError("Keys of distance must be element pair.")
        if not isinstance(dis, (list, tuple, np.ndarray)):
            raise RuntimeError("Values of distance must be array-type.")
        given[tuple(sorted(pair, key=elements.index))] = list(dis)
    cond = {}
    for i, j in itertools.combinations_with_replacement(range(len(elements)), 2):
        key = (elements[i], elements[j])
        if key not in given:
            cond[(i, j)] = list(range(len(pair_params)))
            continue
        match = {len(pair_params) - 1}
        for d in given[key]:
            for k, (beta, mu) in enumerate(pair_params[:-1]):
                if mu - 1.0 / beta < d < mu + 1.0 / beta:
                    match.add(k)
        cond[(i, j)] = sorted(match)
    return cond, distance is not None


def make_params_dict(
    n_type: int,
    cutoff: float,
    model_type: int,
    max_p: int,
    feature_type: str = "gtinv",
    gaussian_params1=(1.0, 1.0, 1),
    gaussian_params2=(0.0, 5.0, 7),
    gtinv_order: int = 3,
    gtinv_maxl: Sequence[int] = (4, 4, 2, 1, 1),
    gtinv_tables: Optional[tuple] = None,
    gtinv_version: int = 1,
    elements: Optional[Sequence[str]] = None,
    include_force: bool = True,
    include_stress: bool = True,
    alphas: Optional[Sequence[float]] = None,
    enable_spins: Optional[Sequence[bool]] = None,
    n_gaussians: Optional[int] = None,
    distance: Optional[dict] = None,
) -> dict:
    pair_params = gaussian_params(gaussian_params1, gaussian_params2, n_gaussians, cutoff)
    if elements is None:
        elements = [f"E{i}" for i in range(n_type)]
    cond, pair_conditional = active_gaussian_params(pair_params, elements, distance)
    if feature_type == "gtinv":
        if gtinv_tables is None:
            gtinv_tables = load_gtinv(gtinv_order, gtinv_maxl, gtinv_version)
        l_comb, lm_seq, lm_coeffs = gtinv_tables
        max_l = int(max(gtinv_maxl[: max(gtinv_order - 1, 1)])) if gtinv_order > 1 else 0
        gtinv = {
            "order": gtinv_order,
            "max_l": list(gtinv_maxl),
            "n_type": n_type,
            "lm_seq": lm_seq,
            "l_comb": l_comb,
            "lm_coeffs": lm_coeffs,
            "version": gtinv_version,
        }
    else:
        max_l = 0
        gtinv = {"order": 0, "max_l": [], "n_type": n_type, "lm_seq": [], "l_comb": [],
                 "lm_coeffs": [], "version": 1}
    return expand_spins({
        "n_type": n_type,
        "elements": list(elements),
        "model": {
            "cutoff": float(cutoff),
            "model_type": int(model_type),
            "max_p": int(max_p),
            "max_l": max_l,
            "feature_type": feature_type,
            "gtinv": gtinv,
            "pair_type": "gaussian",
            "pair_conditional": pair_conditional,
            "pair_params": pair_params,
            "pair_params_conditional": cond,
        },
        "include_force": include_force,
        "include_stress": include_stress,
        "print_memory": False,
        "alphas": list(alphas) if alphas is not None else None,
    }, enable_spins)


def expand_spins(params_dict: dict, enable_spins: Optional[Sequence[bool]]) -> dict:
    """Split every element with its spin enabled into two atom types (spin up and
    down), as PolymlpParamsSingle._set_params_spins and
    PolymlpModelParams.revise_params do (src/pypolymlp/core/data_format.py:291-320,
    192-201): types are renumbered element by element, an enabled element taking two
    consecutive types; elements are repeated; each element pair's radial ids go to
    every pair of their types.  params_dict["n_type"] and ["elements"] are
    element-level on entry.  The element-level settings are kept under
    "spin_elements" (elements, enable_spins, per-element types) for the model
    writers.  Without an enabled spin the dict is returned with
    "enable_spins": None."""
    if enable_spins is None or not any(bool(v) for v in enable_spins):
        params_dict["enable_spins"] = None
        return params_dict
    elements = list(params_dict["elements"])
    if len(enable_spins) != len(elements) or int(params_dict["n_type"]) != len(elements):
        raise ValueError("enable_spins needs one flag per element")
    map_types, new_elements, flags = [], [], []
    for ele, spin in zip(elements, enable_spins):
        types = [len(new_elements)] + ([len(new_elements) + 1] if spin else [])
        map_types.append(types)
        new_elements += [ele] * len(types)
        flags += [bool(spin)] * len(types)
    model = params_dict["model"]
    cond = model.get("pair_params_conditional") or {}
    revised = {}
    for (a, b), ids in cond.items():
        for t1 in map_types[a]:
            for t2 in map_types[b]:
                revised[tuple(sorted((t1, t2)))] = list(ids)
    model["pair_params_conditional"] = revised
    params_dict["spin_elements"] = {"elements": elements, "enable_spins": [bool(v) for v in enable_spins],
                                    "types": map_types}
    params_dict["n_type"] = len(new_elements)
    params_dict["elements"] = new_elements
    params_dict["enable_spins"] = flags
    return params_dict


def to_json(params_dict: dict) -> str:
    """JSON form (tuple keys become "i,j")."""
    d = dict(params_dict)
    d["model"] = dict(params_dict["model"])
    cond = d["model"].get("pair_params_conditional") or {}
    d["model"]["pair_params_conditional"] = {
        (f"{k[0]},{k[1]}" if isinstance(k, tuple) else str(k)): [int(a) for a in v] for k, v in cond.items()
    }
    return json.dumps(d, default=lambda o: o.tolist() if hasattr(o, "tolist") else str(o))


def from_json(text: str) -> dict:
    d = json.loads(text)
    cond = d["model"].get("pair_params_conditional") or {}
    d["model"]["pair_params_conditional"] = {
        tuple(int(a) for a in k.split(",")): v for k, v in cond.items()
    }
    return d
