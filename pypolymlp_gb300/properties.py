"""Energies, forces and stress tensors from a fitted polynomial MLP on the GPU.

`PotentialPropertiesFast` mirrors libmlpcpp.PotentialPropertiesFast
(src/pypolymlp/cxx/src/compute/py_properties_fast.cpp:10-84, bound in
python/pybind11_mlp.cpp:51-67): constructed from the params dict and the
coefficients (already divided by the feature scales), `eval` takes one
structure, `eval_multiple` a list, and the getters return energies in eV per
cell, forces as (n_atom, 3) in eV/angstrom and stresses (xx, yy, zz, xy, yz, zx)
in eV per cell.  `PropertiesSingle` mirrors the Python wrapper of
calculator/properties_single.py:48-130 (forces returned as (3, n_atom)).
"""

from __future__ import annotations

from typing import Sequence

import numpy as np

from pypolymlp_gb300 import _ffi
from pypolymlp_gb300.abi import Structures


class PotentialPropertiesFast:
    """GPU drop-in for libmlpcpp.PotentialPropertiesFast(params_dict, coeffs)."""

    def __init__(self, params_dict: dict, coeffs, precision: int = _ffi.PG_FP64):
        self._ev = _ffi.Evaluator(params_dict, coeffs, precision)
        self._e = 0.0
        self._f = np.zeros((0, 3))
        self._s = np.zeros(6)
        self._e_array = np.zeros(0)
        self._f_array: list = []
        self._s_array = np.zeros((0, 6))

    def eval(self, axis, positions_c, types, use_openmp: bool = True):
        """One structure; positions_c is (3, n_atom) Cartesian."""
        st = Structures.from_columns([axis], [positions_c], [types])
        e, f, s = self._ev.run(st)
        self._e, self._f, self._s = float(e[0]), f, s[0]

    def eval_multiple(self, axis_array: Sequence, positions_c_array: Sequence, types_array: Sequence):
        st = Structures.from_columns(axis_array, positions_c_array, types_array)
        e, f, s = self._ev.run(st)
        offs = st.atom_offsets
        self._e_array = e
        self._f_array = [f[offs[i]:offs[i + 1]] for i in range(st.n_st)]
        self._s_array = s

    def get_e(self):
        return self._e

    def get_f(self):
        return self._f

    def get_s(self):
        return self._s

    def get_e_array(self):
        return self._e_array

    def get_f_array(self):
        return self._f_array

    def get_s_array(self):
        return self._s_array


class PropertiesSingle:
    """eval / eval_multiple on structures with `axis` (3x3, lattice vectors as
    columns), fractional `positions` (3, n_atom) and integer `types`."""

    def __init__(self, params: dict, coeffs, precision: int = _ffi.PG_FP64):
        self._obj = PotentialPropertiesFast(params, coeffs, precision)

    def eval(self, st, use_openmp: bool = True):
        axis = np.asarray(st.axis, dtype=np.float64)
        self._obj.eval(axis, axis @ np.asarray(st.positions, dtype=np.float64), st.types)
        return self._obj.get_e(), np.array(self._obj.get_f()).T, np.array(self._obj.get_s())

    def eval_multiple(self, structures: Sequence):
        axis = [np.asarray(st.axis, dtype=np.float64) for st in structures]
        pos_c = [a @ np.asarray(st.positions, dtype=np.float64) for a, st in zip(axis, structures)]
        self._obj.eval_multiple(axis, pos_c, [st.types for st in structures])
        energies = np.array(self._obj.get_e_array())
        forces = [np.array(f).T for f in self._obj.get_f_array()]
        stresses = np.array(self._obj.get_s_array()).reshape(-1, 6)
        return energies, forces, stresses
