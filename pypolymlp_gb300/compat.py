"""Drop-ins for the reference's pybind11 module `libmlpcpp` on this path.

The reference's Python reaches its C++ hot path through
`from pypolymlp.cxx.lib import libmlpcpp` (src/pypolymlp/cxx/src/python/
pybind11_mlp.cpp:10-268).  This module offers the same classes with the same
constructor arguments and getters, backed by libpolymlp_gb300.so, so that a
caller can write `from pypolymlp_gb300 import compat as libmlpcpp`:

* `PotentialModel` (pybind11_mlp.cpp:12-29; compute/py_model.cpp:10-106): X of
  a list of structures in the reference's row layout;
* `PotentialHybridModel`, `PotentialPropertiesFast`, `FeaturesAttr` and
  `Readgtinv`: the classes of the same names in `hybrid`, `properties`,
  `features_attr` and `gtinv`.
"""

from __future__ import annotations

from typing import Sequence

import numpy as np

from . import _ffi
from .abi import Structures, row_layout_datasets
from .features_attr import FeaturesAttr  # noqa: F401
from .gtinv import Readgtinv  # noqa: F401
from .hybrid import PotentialHybridModel  # noqa: F401
from .properties import PotentialPropertiesFast  # noqa: F401


class PotentialModel:
    """X (n_data x F, float64, Fortran order) of structures, as
    libmlpcpp.PotentialModel builds it (py_model.cpp:10-56) and
    mlp_dev/core/features.py:120 constructs it:

    PotentialModel(params_dict, axis, positions_c, types, n_st_dataset,
                   force_dataset, n_atoms)

    axis: per structure a 3 x 3 array (lattice vectors as columns);
    positions_c: per structure a 3 x N Cartesian array; types: per structure
    N type indices; n_st_dataset: structures per dataset (in order);
    force_dataset: per dataset whether its force and stress rows are built;
    n_atoms: atoms per structure.  Rows: the energies of all structures, then
    six stress rows per structure of a force dataset, then 3 N force rows
    (atom-major x, y, z) per such structure (PyModel::set_index,
    py_model.cpp:58-106).  X is computed on the GPU in FP64 and returned by
    `get_x()` as a writable Fortran-ordered array that the caller may scale
    in place, as the reference's reference_internal Eigen view allows
    (data_standard.py:48-49, utils_weights.py:76-92).  Invalid parameters
    raise GB300Error (the reference exits)."""

    def __init__(self, params_dict: dict, axis: Sequence, positions_c: Sequence, types: Sequence,
                 n_st_dataset: Sequence[int], force_dataset: Sequence[bool], n_atoms: Sequence[int]):
        n_st = int(sum(int(n) for n in n_st_dataset))
        if len(axis) != n_st or len(positions_c) != n_st or len(types) != n_st or len(n_atoms) != n_st:
            raise ValueError("axis, positions_c, types and n_atoms must list sum(n_st_dataset) structures")
        if len(force_dataset) != len(n_st_dataset):
            raise ValueError("one force flag per dataset")
        for k in range(n_st):
            if np.asarray(positions_c[k]).shape != (3, int(n_atoms[k])) or len(types[k]) != int(n_atoms[k]):
                raise ValueError(f"structure {k}: positions_c must be 3 x n_atoms and types n_atoms long")
        st = Structures.from_columns([np.asarray(a, dtype=np.float64) for a in axis],
                                     [np.asarray(p, dtype=np.float64) for p in positions_c],
                                     [np.asarray(t, dtype=np.int32) for t in types])
        e, f, s, n_rows, self._fbegin, self._sbegin, self._n_data = row_layout_datasets(
            [int(n) for n in n_st_dataset], [bool(b) for b in force_dataset], [int(n) for n in n_atoms])
        model = _ffi.Model(params_dict)
        self._x = model.features_x(st, e, f, s, n_rows, precision=_ffi.PG_FP64)

    def get_x(self) -> np.ndarray:
        return self._x

    def get_fbegin(self) -> list:
        return list(self._fbegin)

    def get_sbegin(self) -> list:
        return list(self._sbegin)

    def get_n_data(self) -> list:
        return list(self._n_data)
