"""Calculator facade: structures from files, properties and features.

`PypolymlpCalc` mirrors the evaluation and feature parts of the reference's
facade of the same name (src/pypolymlp/api/pypolymlp_calc.py:24-214, 666-750):
structures are loaded from POSCAR or vasprun.xml files (`load_poscars`,
`load_vaspruns`, `load_structures_from_files`) or set directly; `eval` returns
energies (eV per cell), forces [(3, n_atom)] and stresses (n_str, 6) from
`calculator.Properties`; `run_features` returns the rows of X of one model for
the structures (compute_features.py:28-123: atom types from the model's element
order, energy rows only, or with features_force the energy, stress and force
rows of PotentialModel's layout), from a model file, a params dict, or the
model settings of a polymlp.in file (`parse_polymlp_in`).  The property
applications of the reference facade (elastic constants, EOS, phonons, QHA,
geometry optimisation, force constants, formation energies) are not part of
this module.
"""

from __future__ import annotations

from typing import Optional, Sequence, Union

import numpy as np

from pypolymlp_gb300 import _ffi
from pypolymlp_gb300.calculator import PolymlpStructure, Properties, load_poscar, replace_types


def parse_polymlp_in(filename: str) -> dict:
    """Params dict from the model settings of a polymlp.in file (one "key values"
    per line, "#" comments): n_type, elements, feature_type, cutoff, model_type,
    max_p, gtinv_order, gtinv_maxl, gtinv_version, gaussian_params1/2,
    n_gaussians, reg_alpha_params, include_force, include_stress; dataset keys are
    ignored (core/parser_polymlp_params.py reads the same keys)."""
    from pypolymlp_gb300.params import make_params_dict

    kv = {}
    with open(filename) as f:
        for line in f:
            tok = line.split("#", 1)[0].split()
            if tok:
                kv[tok[0]] = tok[1:]
    elements = kv.get("elements")
    n_type = int(kv["n_type"][0]) if "n_type" in kv else len(elements)
    kw = dict(n_type=n_type, cutoff=float(kv.get("cutoff", [6.0])[0]),
              model_type=int(kv.get("model_type", [4])[0]), max_p=int(kv.get("max_p", [2])[0]),
              feature_type=kv.get("feature_type", ["gtinv"])[0], elements=elements)
    if "gaussian_params1" in kv:
        a, b, n = kv["gaussian_params1"][:3]
        kw["gaussian_params1"] = (float(a), float(b), int(n))
    if "gaussian_params2" in kv:
        a, b, n = kv["gaussian_params2"][:3]
        kw["gaussian_params2"] = (float(a), float(b), int(n))
    if "n_gaussians" in kv:
        kw["n_gaussians"] = int(kv["n_gaussians"][0])
    if kw["feature_type"] == "gtinv":
        kw["gtinv_order"] = int(kv.get("gtinv_order", [3])[0])
        kw["gtinv_maxl"] = tuple(int(v) for v in kv.get("gtinv_maxl", [4, 4, 2, 1, 1]))
        kw["gtinv_version"] = int(kv.get("gtinv_version", [1])[0])
    if "reg_alpha_params" in kv:
        a, b, n = kv["reg_alpha_params"][:3]
        kw["alphas"] = [10.0 ** x for x in np.linspace(float(a), float(b), round(float(n)))]
    for key in ("include_force", "include_stress"):
        if key in kv:
            kw[key] = kv[key][0].lower() in ("true", "1", "yes")
    return make_params_dict(**kw)


def _features_x(params: dict, structures, e_row, f_row, s_row, n_rows: int, precision: int):
    """X rows of a batch on the GPU (pg_features_x)."""
    return _ffi.Model(params).features_x(structures, e_row, f_row, s_row, n_rows, precision=precision)


class PypolymlpCalc:
    def __init__(self, pot: Optional[Union[str, Sequence[str]]] = None, params=None, coeffs=None,
                 properties: Optional[Properties] = None, verbose: bool = False, require_mlp: bool = True,
                 precision: int = _ffi.PG_FP64):
        self._prop = None
        if properties is not None:
            self._prop = properties
        elif pot is not None or params is not None:
            if pot is None and coeffs is None:
                raise RuntimeError("Coefficients not provided.")
            self._prop = Properties(pot=pot, params=params, coeffs=coeffs, precision=precision)
        elif require_mlp:
            raise RuntimeError("Polymlp not provided.")
        self._verbose = verbose
        self._precision = precision
        self._structures = None
        self._features = None

    # -- structures -----------------------------------------------------------------
    def load_poscars(self, poscars: Union[str, Sequence[str]]):
        self.structures = load_poscar(poscars) if isinstance(poscars, str) else [load_poscar(p) for p in poscars]
        return self.structures

    def load_vaspruns(self, vaspruns: Union[str, Sequence[str]]):
        from pypolymlp_gb300.io_vasp import Vasprun

        self.structures = (Vasprun(vaspruns).structure if isinstance(vaspruns, str)
                           else [Vasprun(v).structure for v in vaspruns])
        return self.structures

    def load_structures_from_files(self, poscars=None, vaspruns=None):
        if poscars is None and vaspruns is None:
            raise RuntimeError("Structure files not found.")
        return self.load_poscars(poscars) if poscars is not None else self.load_vaspruns(vaspruns)

    @property
    def structures(self) -> list:
        return self._structures

    @structures.setter
    def structures(self, structures):
        if isinstance(structures, PolymlpStructure):
            self._structures = [structures]
        elif isinstance(structures, list):
            self._structures = structures
        else:
            raise RuntimeError("Invalid structure type.")

    @property
    def first_structure(self) -> PolymlpStructure:
        return self._structures[0]

    # -- properties -----------------------------------------------------------------
    def eval(self, structures=None):
        """(energies (n_str,), forces [(3, n_atom)], stresses (n_str, 6))."""
        if structures is not None:
            self.structures = structures
        if self._prop is None:
            raise RuntimeError("Polymlp not provided.")
        return self._prop.eval_multiple(self.structures)

    def eval_multiple(self, structures=None):
        return self.eval(structures)

    def save_properties(self):
        self._prop.save(verbose=self._verbose)
        return self

    def print_properties(self):
        self._prop.print_single()
        return self

    @property
    def instance_properties(self) -> Properties:
        return self._prop

    @property
    def params(self):
        return None if self._prop is None else self._prop.params

    @property
    def energies(self):
        return self._prop.energies

    @property
    def forces(self):
        return self._prop.forces

    @property
    def stresses(self):
        return self._prop.stresses

    @property
    def stresses_gpa(self):
        return self._prop.stresses_gpa

    # -- features -------------------------------------------------------------------
    def run_features(self, structures=None, develop_infile: Optional[str] = None, features_force: bool = False,
                     features_stress: bool = False) -> np.ndarray:
        """X of the structures: (n_str, n_features) without forces; with
        features_force the energy rows, then 6 stress rows per structure, then
        3 n_atom force rows per structure (the stress rows come with the force
        rows, as in the reference, whatever features_stress says)."""
        from pypolymlp_gb300.abi import Structures, row_layout

        if structures is not None:
            self.structures = structures
        if develop_infile is not None:
            params = parse_polymlp_in(develop_infile)
        else:
            params = self.params
            if params is None:
                raise RuntimeError("Polymlp file or parameters not found.")
            if isinstance(params, list):
                raise NotImplementedError("Only single polymlp file is available.")
        elements = list(params["elements"])
        sts = self.structures
        st = Structures([s.axis for s in sts], [(s.axis @ s.positions).T for s in sts],
                        [replace_types(s, elements) for s in sts])
        e, f, s, n = row_layout(st.n_atoms, [bool(features_force)] * st.n_st)
        self._features = _features_x(params, st, e, f, s, n, self._precision)
        return self._features

    def save_features(self):
        np.save("features.npy", self._features)
        return self

    @property
    def features(self):
        return self._features
