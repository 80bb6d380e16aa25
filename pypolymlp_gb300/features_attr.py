"""Feature attributes of a model: what each column of X is.

`FeaturesAttr` mirrors the reference's pybind class of the same name
(src/pypolymlp/cxx/src/compute/py_features_attr.cpp:11-60), computed on the
host by `pg_feature_attrs` from the same model tables the GPU kernels use (no
device needed).  Per linear feature: its radial function id, its invariant id
(gtinv models; the index into gtinv.l_comb) and its type combination (type-pair
ids); then the polynomial columns as lists of linear-feature ids.
`get_features_attr` and `get_num_features` follow
src/pypolymlp/mlp_dev/core/features_attr.py:12-48, on params dictionaries.
"""

from __future__ import annotations

import ctypes as C
from collections import defaultdict
from typing import Sequence, Union

import numpy as np

from pypolymlp_gb300 import _ffi
from pypolymlp_gb300.abi import FeatureParams


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


class FeaturesAttr:
    def __init__(self, params_dict: dict):
        L = _ffi.lib()
        fp = FeatureParams(params_dict)
        h = C.cast(fp.ref(), C.c_void_p)
        nl, ntv, npoly, npv = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        null = C.POINTER(C.c_int)()
        _ffi.check(L.pg_feature_attrs(h, C.byref(nl), null, null, C.byref(ntv), null, null, C.byref(npoly),
                                      C.byref(npv), null, null, null))
        n_type = int(params_dict["n_type"])
        rad = np.zeros(max(nl.value, 1), np.int32)
        gt = np.zeros(max(nl.value, 1), np.int32)
        tco = np.zeros(nl.value + 1, np.int32)
        tcv = np.zeros(max(ntv.value, 1), np.int32)
        po = np.zeros(npoly.value + 1, np.int32)
        pv = np.zeros(max(npv.value, 1), np.int32)
        tps = np.zeros(n_type * n_type, np.int32)
        _ffi.check(L.pg_feature_attrs(h, C.byref(nl), _p(rad), _p(gt), C.byref(ntv), _p(tco), _p(tcv),
                                      C.byref(npoly), C.byref(npv), _p(po), _p(pv), _p(tps)))
        n = nl.value
        self._radial = rad[:n].tolist()
        self._gtinv = gt[:n].tolist() if params_dict["model"]["feature_type"] == "gtinv" else []
        self._tcomb = [tcv[tco[i]:tco[i + 1]].tolist() for i in range(n)]
        self._poly = [pv[po[i]:po[i + 1]].tolist() for i in range(npoly.value)]
        self._type_pairs = tps.reshape(n_type, n_type).tolist()

    def get_radial_ids(self) -> list:
        return self._radial

    def get_gtinv_ids(self) -> list:
        return self._gtinv

    def get_tcomb_ids(self) -> list:
        return self._tcomb

    def get_polynomial_ids(self) -> list:
        return self._poly

    def get_type_pairs(self) -> list:
        return self._type_pairs


def get_features_attr(params_dict: dict):
    """(features_attr, polynomial_attr, atomtype_pair_dict): per linear feature
    (radial id, type combination) for pair models or (radial id, gtinv id, type
    combination) for gtinv models; polynomial columns; type pair -> [[t1, t2], ...]."""
    obj = FeaturesAttr(params_dict)
    atomtype_pair_dict = defaultdict(list)
    for type1, tps in enumerate(obj.get_type_pairs()):
        for type2, tp in enumerate(tps):
            atomtype_pair_dict[tp].append([type1, type2])
    if params_dict["model"]["feature_type"] == "pair":
        features_attr = list(zip(obj.get_radial_ids(), obj.get_tcomb_ids()))
    else:
        features_attr = list(zip(obj.get_radial_ids(), obj.get_gtinv_ids(), obj.get_tcomb_ids()))
    return features_attr, obj.get_polynomial_ids(), atomtype_pair_dict


def get_num_features(params: Union[dict, Sequence[dict]]) -> int:
    """Number of columns of X of one model, or summed over the models of a hybrid."""
    total = 0
    for p in ([params] if isinstance(params, dict) else params):
        features_attr, polynomial_attr, _ = get_features_attr(p)
        total += len(features_attr) + len(polynomial_attr)
    return total
