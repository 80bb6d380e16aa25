"""Hybrid models: several polynomial MLPs, each on all or on a subset of the
atom types, summed.

`PropertiesHybrid` mirrors calculator/properties_hybrid.py:13-60 with the
per-model atom selection of properties_single.py:52-140: a model whose params
dict has type_full false sees only the atoms whose type is one of its
type_indices, with the types renumbered in that order; its forces are placed
back on those atoms, structures without such atoms get zeros; energies,
forces and stresses of the models are added.

`PotentialHybridModel` mirrors libmlpcpp.PotentialHybridModel
(cxx/src/compute/py_hybrid_model.cpp:11-100): the columns of X are the models'
columns side by side (get_cumulative_n_features), each model's rows computed
on its active atoms (the GPU X rows, `pg_features_x`) and placed in the
dataset's row layout: the energy and stress rows of the structure, the force
rows 3 a + c of its active atoms a.
"""

from __future__ import annotations

from typing import Sequence

import numpy as np

from pypolymlp_gb300 import _ffi
from pypolymlp_gb300.abi import Structures, row_layout, row_layout_datasets


def active_atoms(types, params_dict: dict):
    """(indices of the atoms the model sees, their types in the model's numbering)."""
    types = np.asarray(types, dtype=np.int64)
    if params_dict.get("type_full", True) in (True, 1, None):
        return np.arange(len(types)), types
    if params_dict.get("spin_elements"):
        # the reference has no partial models with spins (properties_utils.py:14-16)
        raise RuntimeError("Not available for system with spin configurations.")
    order = [int(t) for t in params_dict["type_indices"]]
    lookup = {t: k for k, t in enumerate(order)}
    idx = np.array([a for a, t in enumerate(types) if int(t) in lookup], dtype=np.int64)
    return idx, np.array([lookup[int(types[a])] for a in idx], dtype=np.int64)


class PropertiesHybrid:
    """E/F/S of the sum of models (params dicts, coefficients divided by the scales)."""

    def __init__(self, params_list: Sequence[dict], coeffs_list: Sequence, precision: int = _ffi.PG_FP64):
        if len(params_list) != len(coeffs_list) or not params_list:
            raise ValueError("one coefficient vector per model")
        self._params = list(params_list)
        self._ev = [_ffi.Evaluator(p, c, precision) for p, c in zip(params_list, coeffs_list)]

    def eval_multiple(self, axis_array, positions_c_array, types_array):
        """Structures as the reference FFI takes them (positions_c (3, N)):
        energies (n_st,), forces [(N, 3)], stresses (n_st, 6)."""
        n_st = len(types_array)
        energies = np.zeros(n_st)
        forces = [np.zeros((len(t), 3)) for t in types_array]
        stresses = np.zeros((n_st, 6))
        for p, ev in zip(self._params, self._ev):
            sel = [active_atoms(t, p) for t in types_array]
            keep = [s for s in range(n_st) if len(sel[s][0]) > 0]
            if not keep:
                continue
            st = Structures([axis_array[s] for s in keep],
                            [np.asarray(positions_c_array[s], dtype=np.float64).T[sel[s][0]] for s in keep],
                            [sel[s][1] for s in keep])
            e, f, s6 = ev.run(st)
            offs = st.atom_offsets
            for q, s in enumerate(keep):
                energies[s] += e[q]
                forces[s][sel[s][0]] += f[offs[q]:offs[q + 1]]
                stresses[s] += s6[q]
        return energies, forces, stresses

    def eval(self, axis, positions_c, types):
        e, f, s = self.eval_multiple([axis], [positions_c], [types])
        return float(e[0]), f[0], s[0]


def hybrid_features_x(params_list: Sequence[dict], st: Structures, e_row, f_row, s_row, n_rows: int,
                      precision: int = _ffi.PG_FP64):
    """X (n_rows x sum of the models' columns, Fortran order) of a hybrid model
    in the given row layout, and the cumulative column counts."""
    models = [_ffi.Model(p) for p in params_list]
    cum = np.cumsum([m.n_features for m in models]).tolist()
    x = np.zeros((n_rows, cum[-1]), order="F")
    offs = st.atom_offsets
    pos = [st.positions[offs[s]:offs[s + 1]] for s in range(st.n_st)]
    types = [st.types[offs[s]:offs[s + 1]] for s in range(st.n_st)]
    for m, p, c1 in zip(models, params_list, cum):
        c0 = c1 - m.n_features
        sel = [active_atoms(t, p) for t in types]
        keep = [s for s in range(st.n_st) if len(sel[s][0]) > 0]
        if not keep:
            continue
        sub = Structures([st.axis[s] for s in keep], [pos[s][sel[s][0]] for s in keep], [sel[s][1] for s in keep])
        force = [f_row[s] >= 0 for s in keep]
        e, f, s6, n = row_layout(sub.n_atoms, force)
        xs = m.features_x(sub, e, f, s6, n, precision=precision)
        for q, s in enumerate(keep):
            x[e_row[s], c0:c1] = xs[e[q]]
            if f_row[s] >= 0:
                if s_row[s] >= 0:
                    x[s_row[s]:s_row[s] + 6, c0:c1] = xs[s6[q]:s6[q] + 6]
                rows = f_row[s] + (3 * sel[s][0][:, None] + np.arange(3)[None, :]).reshape(-1)
                x[rows, c0:c1] = xs[f[q]:f[q] + 3 * len(sel[s][0])]
    return x, cum


class PotentialHybridModel:
    """Drop-in for libmlpcpp.PotentialHybridModel(params_dict_array, axis,
    positions_c, types, n_st_dataset, force_dataset, n_atoms)."""

    def __init__(self, params_dict_array, axis, positions_c, types, n_st_dataset, force_dataset, n_atoms,
                 precision: int = _ffi.PG_FP64):
        st = Structures.from_columns(axis, positions_c, types)
        e, f, s, n_rows, self._fbegin, self._sbegin, self._n_data = row_layout_datasets(
            n_st_dataset, force_dataset, n_atoms)
        self._x, self._cum = hybrid_features_x(params_dict_array, st, e, f, s, n_rows, precision)

    def get_x(self):
        return self._x

    def get_fbegin(self):
        return self._fbegin

    def get_sbegin(self):
        return self._sbegin

    def get_cumulative_n_features(self):
        return self._cum

    def get_n_data(self):
        return self._n_data
