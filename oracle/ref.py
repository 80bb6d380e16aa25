"""ctypes access to the reference's own C++ build (oracle/_ref/libpolymlp_ref.so).

Test infrastructure only.  The library exists only where the reference
sources were available to compile it (`make -C oracle ref`); callers must
check `available()` and skip otherwise.
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

from pypolymlp_gb300.abi import FeatureParams, Structures

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_ref", "libpolymlp_ref.so")
_lib = None


def available() -> bool:
    if not os.path.exists(LIB_PATH):
        return False
    try:
        _load()
    except OSError:
        return False
    return True


def _load():
    global _lib
    if _lib is None:
        _lib = C.CDLL(LIB_PATH)
    return _lib


def _check(rc: int):
    if rc != 0:
        buf = C.create_string_buffer(1024)
        _load().ref_last_error(buf, 1024)
        raise RuntimeError(buf.value.decode())


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def readgtinv(order: int, maxl, version: int = 1):
    """(l_comb, lm_seq, lm_coeffs) exactly as Readgtinv returns them."""
    lib = _load()
    maxl = np.ascontiguousarray(np.asarray(list(maxl), dtype=np.int32))
    sizes = np.zeros(4, dtype=np.int32)
    null = C.POINTER(C.c_int)()
    _check(lib.ref_readgtinv(order, _p(maxl, C.c_int), len(maxl), version, _p(sizes, C.c_int),
                             null, null, null, null, C.POINTER(C.c_double)()))
    nl, nlv, nm, nmv = (int(v) for v in sizes)
    lco = np.zeros(nl + 1, np.int32)
    lcv = np.zeros(max(nlv, 1), np.int32)
    lmo = np.zeros(nl + 1, np.int32)
    lmv = np.zeros(max(nmv, 1), np.int32)
    cf = np.zeros(max(nm, 1), np.float64)
    _check(lib.ref_readgtinv(order, _p(maxl, C.c_int), len(maxl), version, _p(sizes, C.c_int),
                             _p(lco, C.c_int), _p(lcv, C.c_int), _p(lmo, C.c_int), _p(lmv, C.c_int),
                             _p(cf, C.c_double)))
    l_comb, lm_seq, lm_coeffs = [], [], []
    mpos = 0
    for c in range(nl):
        lc = [int(v) for v in lcv[lco[c]:lco[c + 1]]]
        order_c = len(lc)
        seq = []
        for q in range(lmo[c], lmo[c + 1]):
            seq.append([int(v) for v in lmv[mpos:mpos + order_c]])
            mpos += order_c
        l_comb.append(lc)
        lm_seq.append(seq)
        lm_coeffs.append([float(v) for v in cf[lmo[c]:lmo[c + 1]]])
    return l_comb, lm_seq, lm_coeffs


def n_features(params_dict) -> int:
    fp = FeatureParams(params_dict)
    n = C.c_int()
    _check(_load().ref_n_features(fp.ref(), C.byref(n)))
    return n.value


def features_x(params_dict, st: Structures, e_row, f_row, s_row, n_rows: int):
    fp = FeatureParams(params_dict)
    nf = n_features(params_dict)
    x = np.zeros((n_rows, nf), dtype=np.float64, order="F")
    e_row = np.ascontiguousarray(e_row, dtype=np.int64)
    f_row = np.ascontiguousarray(f_row, dtype=np.int64)
    s_row = np.ascontiguousarray(s_row, dtype=np.int64)
    _check(_load().ref_features_x(fp.ref(), st.ref(), _p(e_row, C.c_int64), _p(f_row, C.c_int64),
                                  _p(s_row, C.c_int64), _p(x, C.c_double), C.c_int64(n_rows)))
    return x


def evaluate(params_dict, coeffs, st: Structures):
    fp = FeatureParams(params_dict)
    coeffs = np.ascontiguousarray(coeffs, dtype=np.float64)
    e = np.zeros(st.n_st)
    f = np.zeros((int(st.n_atoms.sum()), 3))
    s = np.zeros((st.n_st, 6))
    _check(_load().ref_eval(fp.ref(), _p(coeffs, C.c_double), len(coeffs), st.ref(), _p(e, C.c_double),
                            _p(f, C.c_double), _p(s, C.c_double)))
    return e, f, s


def neighbor_list(st: Structures, s: int, cutoff: float, half: bool):
    lib = _load()
    n = C.c_int64()
    null_i = C.POINTER(C.c_int)()
    _check(lib.ref_neighbor_list(st.ref(), s, C.c_double(cutoff), int(half), C.byref(n), null_i, null_i,
                                 C.POINTER(C.c_double)()))
    na = int(st.n_atoms[s])
    offs = np.zeros(na + 1, np.int32)
    nb = np.zeros(max(n.value, 1), np.int32)
    d = np.zeros((max(n.value, 1), 3))
    _check(lib.ref_neighbor_list(st.ref(), s, C.c_double(cutoff), int(half), C.byref(n), _p(offs, C.c_int),
                                 _p(nb, C.c_int), _p(d, C.c_double)))
    return offs, nb[:n.value], d[:n.value]


def translations(st: Structures, s: int, cutoff: float):
    lib = _load()
    nt = C.c_int()
    _check(lib.ref_translations(st.ref(), s, C.c_double(cutoff), C.byref(nt), C.POINTER(C.c_double)(),
                                C.POINTER(C.c_double)()))
    t = np.zeros((nt.value, 3))
    pr = np.zeros((int(st.n_atoms[s]), 3))
    _check(lib.ref_translations(st.ref(), s, C.c_double(cutoff), C.byref(nt), _p(t, C.c_double),
                                _p(pr, C.c_double)))
    return t, pr


def feature_attrs(params_dict):
    lib = _load()
    fp = FeatureParams(params_dict)
    nl, ntv, npoly, npv = C.c_int(), C.c_int(), C.c_int(), C.c_int()
    null = C.POINTER(C.c_int)()
    _check(lib.ref_feature_attrs(fp.ref(), C.byref(nl), null, null, C.byref(ntv), null, null,
                                 C.byref(npoly), C.byref(npv), null, null))
    rad = np.zeros(max(nl.value, 1), np.int32)
    gt = np.zeros(max(nl.value, 1), np.int32)
    tco = np.zeros(nl.value + 1, np.int32)
    tcv = np.zeros(max(ntv.value, 1), np.int32)
    po = np.zeros(npoly.value + 1, np.int32)
    pv = np.zeros(max(npv.value, 1), np.int32)
    _check(lib.ref_feature_attrs(fp.ref(), C.byref(nl), _p(rad, C.c_int), _p(gt, C.c_int), C.byref(ntv),
                                 _p(tco, C.c_int), _p(tcv, C.c_int), C.byref(npoly), C.byref(npv),
                                 _p(po, C.c_int), _p(pv, C.c_int)))
    tcomb = [list(tcv[tco[i]:tco[i + 1]]) for i in range(nl.value)]
    poly = [list(pv[po[i]:po[i + 1]]) for i in range(npoly.value)]
    return rad[:nl.value].tolist(), gt[:nl.value].tolist(), tcomb, poly


def type_pairs(params_dict):
    """FeaturesAttr::get_type_pairs: [t1][t2] -> type-pair id."""
    lib = _load()
    n = int(params_dict["n_type"])
    out = np.zeros(n * n, np.int32)
    _check(lib.ref_type_pairs(FeatureParams(params_dict).ref(), _p(out, C.c_int)))
    return out.reshape(n, n).tolist()


def parse_potential(path: str, legacy: bool = False) -> dict:
    """A model file read by the reference's own C++ parsers (ref_parse_potential):
    {elements, cutoff, pair_type, feature_type, model_type, max_p, max_l,
    n_l_comb, params (n x 2), cond {(i, j): ids}, coeffs (2 x the file's), mass}."""
    lib = _load()
    buf = C.create_string_buffer(1 << 24)
    _check(lib.ref_parse_potential(path.encode(), 1 if legacy else 0, buf, C.c_size_t(1 << 24)))
    out = {"cond": {}}
    for line in buf.value.decode().splitlines():
        key, *vals = line.split()
        if key == "cond":
            out["cond"][(int(vals[0]), int(vals[1]))] = [int(v) for v in vals[2:]]
        elif key == "elements":
            out[key] = vals
        elif key in ("pair_type", "feature_type"):
            out[key] = vals[0]
        elif key in ("model_type", "max_p", "max_l", "n_l_comb"):
            out[key] = int(vals[0])
        elif key == "cutoff":
            out[key] = float(vals[0])
        elif key == "params":
            out[key] = np.array([float(v) for v in vals]).reshape(-1, 2)
        else:
            out[key] = np.array([float(v) for v in vals])
    return out


def api_sum_of_prod(path: str, elements, type1: int, anlmtp):
    """PolymlpAPI::parse_polymlp_file + compute_sum_of_prod_anlmtp of the reference
    build: (prod_sum_e, prod_sum_f), complex."""
    a = np.ascontiguousarray(np.asarray(anlmtp, dtype=np.complex128))
    k = len(a)
    pe, pf = np.zeros(2 * k), np.zeros(2 * k)
    n = C.c_int()
    _check(_load().ref_api_sum_of_prod(path.encode(), elements[0].encode(), elements[1].encode(), type1,
                                       _p(a.view(np.float64), C.c_double), k, _p(pe, C.c_double),
                                       _p(pf, C.c_double), C.byref(n)))
    return pe.view(np.complex128)[:n.value], pf.view(np.complex128)[:n.value]
