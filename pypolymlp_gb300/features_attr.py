"""Feature attributes of a model: what each column of X is.

`FeaturesAttr` mirrors the reference's pybind class of the same name
(src/pypolymlp/cxx/src/compute/py_features_attr.cpp:11-60), computed on the
host by `pg_feature_attrs` from the same model tables the GPU kernels use (no
device needed).  Per linear feature: its radial function id, its invariant id
(gtinv models; the index into gtinv.l_comb) and its type combination (type-pair
ids); then the polynomial columns as lists of linear-feature ids.
`get_features_attr`, `get_num_features` and `write_polymlp_params_yaml`
follow src/pypolymlp/mlp_dev/core/features_attr.py:12-133, on params
dictionaries.
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


def _write_params_yaml(params_dict: dict, filename: str) -> int:
    features_attr, polynomial_attr, atomtype_pair_dict = get_features_attr(params_dict)
    model = params_dict["model"]
    elements = list(params_dict["elements"])
    with open(filename, "w") as f:
        print("radial_params:", file=f)
        for i, p in enumerate(model["pair_params"]):
            print("- radial_id: ", i, file=f)
            print("  params:    ", [float(v) for v in p], file=f)
            print("", file=f)
        print("", file=f)
        print("atomtype_pairs:", file=f)
        for k, v in atomtype_pair_dict.items():
            print("- pair_id:       ", k, file=f)
            print("  pair_elements: ", file=f)
            for t1, t2 in v:
                print("  - ", [elements[t1], elements[t2]], file=f)
            print("", file=f)
        print("", file=f)
        print("features:", file=f)
        seq_id = 0
        for i, attr in enumerate(features_attr):
            print("- id:               ", seq_id, file=f)
            print("  feature_id:       ", i, file=f)
            print("  radial_id:        ", attr[0], file=f)
            if model["feature_type"] == "gtinv":
                print("  gtinv_id:         ", attr[1], file=f)
                print("  l_combination:    ", list(model["gtinv"]["l_comb"][attr[1]]), file=f)
            print("  atomtype_pair_ids:", attr[-1], file=f)
            print("", file=f)
            seq_id += 1
        print("", file=f)
        if polynomial_attr:
            print("polynomial_features:", file=f)
            for attr in polynomial_attr:
                print("- id:          ", seq_id, file=f)
                print("  feature_ids: ", attr, file=f)
                print("", file=f)
                seq_id += 1
    return seq_id


def write_polymlp_params_yaml(params: Union[dict, Sequence[dict]], filename: str = "polymlp_params.yaml") -> int:
    """Write the column attributes of X as polymlp_params.yaml, in the layout of
    src/pypolymlp/mlp_dev/core/features_attr.py:51-133: radial parameters, the
    element pairs of each type pair, one entry per linear feature (radial id,
    invariant id and l combination for gtinv models, type-pair ids), then the
    polynomial columns; ids run over all columns.  A hybrid (list of params
    dicts) writes polymlp_params1.yaml, polymlp_params2.yaml, ...  Returns the
    number of columns."""
    if isinstance(params, dict):
        return _write_params_yaml(params, filename)
    return sum(_write_params_yaml(p, f"polymlp_params{i + 1}.yaml") for i, p in enumerate(params))
