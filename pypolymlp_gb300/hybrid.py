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

from typing import Optional, Sequence

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


def hybrid_normal_equations(params_list: Sequence[dict], datasets, precision: int = _ffi.PG_FP64,
                            weight_stress: float = 0.1, min_energy: Optional[float] = None, scales=None,
                            batch_size: int = 500):
    """Scaled normal equations of a hybrid model (regression.DataXY), as the
    reference's calc_xtx_xty forms them for PotentialHybridModel's X
    (mlp_dev/core/data_sequential.py:95-160): per batch of structures the rows of X
    on the GPU (`hybrid_features_x`), the column sums of the unweighted energy
    rows, the reference's weights and targets, and the Gram of the weighted rows
    on the device (`_ffi.gram_xtx`); then the feature scales and zero columns of
    `regression.compute_scales`."""
    from pypolymlp_gb300 import regression as rg

    min_energy = rg.get_min_energy(datasets) if min_energy is None else min_energy
    xtx = xty = xe_sum = xe_sq = None
    yty, n_total = 0.0, 0
    for d in datasets:
        for b in range(0, len(d), batch_size):
            sub = d.slice(b, min(len(d), b + batch_size))
            e_row, f_row, s_row, n_rows, w, y = rg.weights_and_targets(sub, min_energy, weight_stress)
            st = Structures(sub.axis, sub.positions, sub.types)
            x, cum = hybrid_features_x(params_list, st, e_row, f_row, s_row, n_rows, precision)
            xe = x[np.asarray(e_row)]
            xw = np.asfortranarray(x * np.asarray(w)[:, None])
            g, r = _ffi.gram_xtx(xw, precision), xw.T @ np.asarray(y)
            if xtx is None:
                xtx, xty, xe_sum, xe_sq = g, r, xe.sum(axis=0), np.square(xe).sum(axis=0)
            else:
                xtx, xty = xtx + g, xty + r
                xe_sum, xe_sq = xe_sum + xe.sum(axis=0), xe_sq + np.square(xe).sum(axis=0)
            yty += float(np.asarray(y) @ np.asarray(y))
            n_total += int(n_rows)
    n_data = sum(len(d.energies) for d in datasets)
    scales, zero_ids = rg.compute_scales(scales, xe_sum, xe_sq, n_data, any(d.include_force for d in datasets))
    xtx = np.array(xtx, dtype=np.float64)
    xtx[zero_ids] = 0.0
    xtx[:, zero_ids] = 0.0
    xty = np.array(xty, dtype=np.float64)
    xty[zero_ids] = 0.0
    xtx /= scales[:, None]
    xtx /= scales[None, :]
    xty /= scales
    return rg.DataXY(xtx, xty, yty, n_total, scales, zero_ids, min_energy, xe_sum, xe_sq), cum


def fit_hybrid(params_list: Sequence[dict], train, test, alphas: Sequence[float], precision: int = _ffi.PG_FP64,
               weight_stress: float = 0.1):
    """Ridge fit of a hybrid model (the reference's fit over PotentialHybridModel,
    mlp_dev/standard/fit.py:12-60): the training normal equations, posv per
    alpha on the device, the test normal equations with the training scales and
    reference energy, the alpha of the smallest test RMSE (compute_rmse_seq).
    Returns (regression.FitResult, cumulative feature counts of the models)."""
    from pypolymlp_gb300 import regression as rg

    alphas = np.asarray(alphas, dtype=np.float64)
    xy, cum = hybrid_normal_equations(params_list, train, precision, weight_stress)
    coefs, info = rg.solver_ridge(xy.xtx, xy.xty, alphas)
    txy, _ = hybrid_normal_equations(params_list, test, precision, weight_stress, min_energy=xy.min_energy,
                                     scales=xy.scales)
    rmse_train = np.asarray(rg.compute_rmse_seq(coefs, xy))
    rmse_test = np.asarray(rg.compute_rmse_seq(coefs, txy))
    idx = int(np.argmin(rmse_test))
    res = rg.FitResult(coefs[:, idx], xy.scales, float(alphas[idx]), float(rmse_train[idx]),
                       float(rmse_test[idx]), coefs, rmse_train, rmse_test, info)
    return res, cum
