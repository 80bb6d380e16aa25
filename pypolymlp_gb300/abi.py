"""ctypes mirrors of the C ABI structs in include/polymlp_gb300.h.

`FeatureParams.from_params_dict` takes the dictionary that the reference passes
across its FFI boundary (``params.as_dict()``, read on the C++ side by
``convert_params_dict_to_feature_params`` in
src/pypolymlp/cxx/src/compute/py_params.cpp:11-60) and packs it into the flat
``pg_feature_params`` struct.  `Structures.pack` packs a list of structures
(axis 3x3 with lattice vectors as columns, Cartesian positions) into
``pg_structures``.  Both keep the numpy buffers alive for as long as the
struct is used.
"""

from __future__ import annotations

import ctypes as C
from typing import Any, Sequence

import numpy as np

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class pg_feature_params(C.Structure):
    _fields_ = [
        ("n_type", C.c_int),
        ("feature_type", C.c_int),
        ("model_type", C.c_int),
        ("max_p", C.c_int),
        ("max_l", C.c_int),
        ("cutoff", C.c_double),
        ("n_fn", C.c_int),
        ("pair_params", _dp),
        ("cond_offsets", _ip),
        ("cond_values", _ip),
        ("n_lcomb", C.c_int),
        ("lcomb_offsets", _ip),
        ("lcomb_values", _ip),
        ("lmseq_offsets", _ip),
        ("lmseq_values", _ip),
        ("lm_coeffs", _dp),
    ]


class pg_structures(C.Structure):
    _fields_ = [
        ("n_st", C.c_int),
        ("n_atoms", _ip),
        ("axis", _dp),
        ("positions", _dp),
        ("types", _ip),
    ]


def _iarr(x) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(x, dtype=np.int32).reshape(-1))


def _darr(x) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(x, dtype=np.float64).reshape(-1))


def _ip_of(a: np.ndarray):
    return a.ctypes.data_as(_ip)


def _dp_of(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def _cond_lookup(cond: Any, i: int, j: int):
    """pair_params_conditional entry for type pair (i, j), i <= j.

    The reference keys the dict by tuples (j, i) with j <= i (py_params.cpp:41-49);
    JSON fixtures store the key as the string "i,j".
    """
    for key in ((i, j), f"{i},{j}", str((i, j)), f"({i}, {j})"):
        if key in cond:
            return cond[key]
    raise KeyError(f"pair_params_conditional has no entry for type pair ({i}, {j})")


class FeatureParams:
    """Owner of a packed pg_feature_params and its buffers."""

    def __init__(self, params_dict: dict):
        model = params_dict["model"]
        n_type = int(params_dict["n_type"])
        feature_type = model["feature_type"]
        if feature_type not in ("pair", "gtinv"):
            raise ValueError(f"unknown feature_type {feature_type!r}")
        if model.get("pair_type", "gaussian") != "gaussian":
            raise ValueError("only pair_type 'gaussian' is evaluated by the reference")
        pair_params = np.asarray(model["pair_params"], dtype=np.float64).reshape(-1, 2)
        cond = model.get("pair_params_conditional")
        offs, vals = [0], []
        for i in range(n_type):
            for j in range(n_type):
                if j >= i:
                    if cond is None:
                        v = list(range(len(pair_params)))
                    else:
                        v = list(_cond_lookup(cond, i, j))
                    vals.extend(int(a) for a in v)
                offs.append(len(vals))
        gt = model.get("gtinv") or {}
        l_comb = gt.get("l_comb") or []
        lm_seq = gt.get("lm_seq") or []
        lm_coeffs = gt.get("lm_coeffs") or []
        if feature_type == "pair":
            l_comb, lm_seq, lm_coeffs = [], [], []
        lc_offs, lc_vals, lm_offs, lm_vals, coeffs = [0], [], [0], [], []
        for lc, seq, cf in zip(l_comb, lm_seq, lm_coeffs):
            lc_vals.extend(int(v) for v in lc)
            lc_offs.append(len(lc_vals))
            for mc, c in zip(seq, cf):
                if len(mc) != len(lc):
                    raise ValueError("lm_seq entry does not match its l combination")
                lm_vals.extend(int(v) for v in mc)
                coeffs.append(float(c))
            lm_offs.append(len(coeffs))

        self.params_dict = params_dict
        self._pair = _darr(pair_params)
        self._cond_offs = _iarr(offs)
        self._cond_vals = _iarr(vals if vals else [0])
        self._lc_offs = _iarr(lc_offs)
        self._lc_vals = _iarr(lc_vals if lc_vals else [0])
        self._lm_offs = _iarr(lm_offs)
        self._lm_vals = _iarr(lm_vals if lm_vals else [0])
        self._coeffs = _darr(coeffs if coeffs else [0.0])
        s = pg_feature_params()
        s.n_type = n_type
        s.feature_type = 1 if feature_type == "gtinv" else 0
        s.model_type = int(model["model_type"])
        s.max_p = int(model["max_p"])
        s.max_l = int(model.get("max_l", 0) or 0)
        s.cutoff = float(model["cutoff"])
        s.n_fn = len(pair_params)
        s.pair_params = _dp_of(self._pair)
        s.cond_offsets = _ip_of(self._cond_offs)
        s.cond_values = _ip_of(self._cond_vals)
        s.n_lcomb = len(lc_offs) - 1
        s.lcomb_offsets = _ip_of(self._lc_offs)
        s.lcomb_values = _ip_of(self._lc_vals)
        s.lmseq_offsets = _ip_of(self._lm_offs)
        s.lmseq_values = _ip_of(self._lm_vals)
        s.lm_coeffs = _dp_of(self._coeffs)
        # the struct keeps its buffers alive even if this owner is dropped
        s._keep = (self._pair, self._cond_offs, self._cond_vals, self._lc_offs, self._lc_vals,
                   self._lm_offs, self._lm_vals, self._coeffs)
        self.struct = s
        self.n_type = n_type
        self.cutoff = s.cutoff

    def ref(self):
        return C.byref(self.struct)


class Structures:
    """Owner of a packed pg_structures.

    axis: (n_st, 3, 3) with lattice vectors as columns; positions: list of
    (N_s, 3) Cartesian arrays (or one (sum N, 3) array with n_atoms given);
    types: list of (N_s,) integer arrays.
    """

    def __init__(self, axis, positions_list: Sequence, types_list: Sequence):
        axis = np.ascontiguousarray(np.asarray(axis, dtype=np.float64).reshape(-1, 3, 3))
        n_atoms = np.array([len(t) for t in types_list], dtype=np.int32)
        if len(positions_list) != len(types_list) or len(axis) != len(types_list):
            raise ValueError("axis, positions and types must describe the same structures")
        pos = [np.asarray(p, dtype=np.float64).reshape(-1, 3) for p in positions_list]
        for p, n in zip(pos, n_atoms):
            if len(p) != n:
                raise ValueError("positions and types disagree on the number of atoms")
        self.axis = axis
        self.n_atoms = n_atoms
        self.positions = (
            np.ascontiguousarray(np.concatenate(pos, axis=0)) if len(pos) else np.zeros((0, 3))
        )
        self.types = (
            np.ascontiguousarray(np.concatenate([np.asarray(t, dtype=np.int32) for t in types_list]))
            if len(types_list)
            else np.zeros(0, dtype=np.int32)
        )
        if not np.all(np.isfinite(self.positions)) or not np.all(np.isfinite(self.axis)):
            raise ValueError("structures contain non-finite coordinates")
        s = pg_structures()
        s.n_st = len(n_atoms)
        s.n_atoms = _ip_of(self.n_atoms)
        s.axis = _dp_of(self.axis)
        s.positions = _dp_of(self.positions)
        s.types = _ip_of(self.types)
        s._keep = (self.n_atoms, self.axis, self.positions, self.types)
        self.struct = s

    @classmethod
    def from_columns(cls, axis_list, positions_c_list, types_list):
        """Reference FFI layout: positions_c as (3, N) per structure."""
        return cls(axis_list, [np.asarray(p).T for p in positions_c_list], types_list)

    @property
    def n_st(self) -> int:
        return int(len(self.n_atoms))

    @property
    def atom_offsets(self) -> np.ndarray:
        return np.concatenate([[0], np.cumsum(self.n_atoms, dtype=np.int64)])

    def ref(self):
        return C.byref(self.struct)


def row_layout(n_atoms: Sequence[int], force: Sequence[bool]):
    """Row offsets of X as PyModel::set_index lays them out
    (src/pypolymlp/cxx/src/compute/py_model.cpp:58-106) for one dataset:
    energies [0, n_st), then 6 stress rows per force structure, then 3N force
    rows per force structure.  Returns (e_row, f_row, s_row, n_rows)."""
    n_st = len(n_atoms)
    e_row = np.arange(n_st, dtype=np.int64)
    f_row = np.full(n_st, -1, dtype=np.int64)
    s_row = np.full(n_st, -1, dtype=np.int64)
    r = n_st
    for s in range(n_st):
        if force[s]:
            s_row[s] = r
            r += 6
    for s in range(n_st):
        if force[s]:
            f_row[s] = r
            r += 3 * int(n_atoms[s])
    return e_row, f_row, s_row, r


def row_layout_datasets(n_st_dataset, force_dataset, n_atoms):
    """Multi-dataset row layout of PyModel::set_index; also returns the per-dataset
    first force/stress rows (get_fbegin / get_sbegin, -1 if absent) and
    n_data = [n_e, n_f, n_s]."""
    n_st = int(sum(n_st_dataset))
    e_row = np.arange(n_st, dtype=np.int64)
    f_row = np.full(n_st, -1, dtype=np.int64)
    s_row = np.full(n_st, -1, dtype=np.int64)
    fbegin = [-1] * len(n_st_dataset)
    sbegin = [-1] * len(n_st_dataset)
    n_data = [n_st, 0, 0]
    st = 0
    r = n_st
    for d, n in enumerate(n_st_dataset):
        if force_dataset[d]:
            sbegin[d] = r
            n_data[2] += 6 * n
        for _ in range(n):
            if force_dataset[d]:
                s_row[st] = r
                r += 6
            st += 1
    st = 0
    for d, n in enumerate(n_st_dataset):
        if force_dataset[d]:
            fbegin[d] = r
        for _ in range(n):
            if force_dataset[d]:
                f_row[st] = r
                r += 3 * int(n_atoms[st])
                n_data[1] += 3 * int(n_atoms[st])
            st += 1
    return e_row, f_row, s_row, r, fbegin, sbegin, n_data
