"""ctypes access to the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the checker or the timed CPU baseline.  The
product never imports this module.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from pypolymlp_gb300.abi import FeatureParams, Structures

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with make (a few seconds)."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", _HERE, "oracle"], check=True)
    return LIB_PATH


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = C.CDLL(LIB_PATH)
    return _lib


def _check(rc: int):
    if rc != 0:
        buf = C.create_string_buffer(2048)
        _load().or_last_error(buf, 2048)
        raise RuntimeError(buf.value.decode())


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def n_features(params_dict) -> int:
    fp = FeatureParams(params_dict)
    n = C.c_int()
    _check(_load().or_n_features(fp.ref(), C.byref(n)))
    return n.value


def features_x(params_dict, st: Structures, e_row, f_row, s_row, n_rows: int, n_threads: int = 0):
    fp = FeatureParams(params_dict)
    nf = n_features(params_dict)
    x = np.zeros((n_rows, nf), dtype=np.float64, order="F")
    e_row = np.ascontiguousarray(e_row, dtype=np.int64)
    f_row = np.ascontiguousarray(f_row, dtype=np.int64)
    s_row = np.ascontiguousarray(s_row, dtype=np.int64)
    _check(_load().or_features_x(fp.ref(), st.ref(), _p(e_row, C.c_int64), _p(f_row, C.c_int64),
                                 _p(s_row, C.c_int64), _p(x, C.c_double), C.c_int64(n_rows), int(n_threads)))
    return x


def evaluate(params_dict, coeffs, st: Structures, n_threads: int = 0):
    fp = FeatureParams(params_dict)
    coeffs = np.ascontiguousarray(coeffs, dtype=np.float64)
    e = np.zeros(st.n_st)
    f = np.zeros((int(st.n_atoms.sum()), 3))
    s = np.zeros((st.n_st, 6))
    _check(_load().or_eval(fp.ref(), _p(coeffs, C.c_double), len(coeffs), st.ref(), _p(e, C.c_double),
                           _p(f, C.c_double), _p(s, C.c_double), int(n_threads)))
    return e, f, s


def neighbor_list(st: Structures, s: int, cutoff: float, half: bool):
    lib = _load()
    n = C.c_int64()
    null_i = C.POINTER(C.c_int)()
    _check(lib.or_neighbor_list(st.ref(), s, C.c_double(cutoff), int(half), C.byref(n), null_i, null_i,
                                C.POINTER(C.c_double)()))
    na = int(st.n_atoms[s])
    offs = np.zeros(na + 1, np.int32)
    nb = np.zeros(max(n.value, 1), np.int32)
    d = np.zeros((max(n.value, 1), 3))
    _check(lib.or_neighbor_list(st.ref(), s, C.c_double(cutoff), int(half), C.byref(n), _p(offs, C.c_int),
                                _p(nb, C.c_int), _p(d, C.c_double)))
    return offs, nb[:n.value], d[:n.value]


def translations(st: Structures, s: int, cutoff: float):
    lib = _load()
    nt = C.c_int()
    _check(lib.or_translations(st.ref(), s, C.c_double(cutoff), C.byref(nt), C.POINTER(C.c_double)(),
                               C.POINTER(C.c_double)()))
    t = np.zeros((nt.value, 3))
    pr = np.zeros((int(st.n_atoms[s]), 3))
    _check(lib.or_translations(st.ref(), s, C.c_double(cutoff), C.byref(nt), _p(t, C.c_double),
                               _p(pr, C.c_double)))
    return t, pr


def fn(dis: float, cutoff: float, pair_params):
    pp = np.ascontiguousarray(np.asarray(pair_params, dtype=np.float64).reshape(-1, 2))
    f = np.zeros(len(pp))
    fd = np.zeros(len(pp))
    _check(_load().or_fn(C.c_double(dis), C.c_double(cutoff), len(pp), _p(pp, C.c_double), _p(f, C.c_double),
                         _p(fd, C.c_double)))
    return f, fd


def ylm(r: float, x: float, y: float, z: float, lmax: int):
    n = (lmax + 1) * (lmax + 2) // 2
    arrs = [np.zeros(2 * n) for _ in range(4)]
    _check(_load().or_ylm(C.c_double(r), C.c_double(x), C.c_double(y), C.c_double(z), lmax,
                          *[_p(a, C.c_double) for a in arrs]))
    return [a[0::2] + 1j * a[1::2] for a in arrs]


class PolymlpAPI:
    """The per-type PolymlpAPI steps of the reference (polymlp_api.cpp:62-190) on
    given order parameters: conjugate completion, features, feature derivatives
    and the adjoint sums (coefficients as the reference's parser returns them)."""

    def __init__(self, params_dict, coeffs=None):
        self._fp = FeatureParams(params_dict)
        self._gtinv = params_dict["model"]["feature_type"] == "gtinv"
        self._c = None if coeffs is None else np.ascontiguousarray(coeffs, dtype=np.float64)

    def sizes(self, t):
        s = np.zeros(5, np.int32)
        _check(_load().or_api_sizes(self._fp.ref(), t, _p(s, C.c_int)))
        return [int(v) for v in s]

    @staticmethod
    def _cplx(a):
        a = np.ascontiguousarray(np.asarray(a, dtype=np.complex128))
        return a.view(np.float64)

    def compute_anlmtp_conjugate(self, re, im, t):
        k, k0 = self.sizes(t)[:2]
        re = np.ascontiguousarray(np.asarray(re, dtype=np.float64)[:k0])
        im = np.ascontiguousarray(np.asarray(im, dtype=np.float64)[:k0])
        out = np.zeros(k, np.complex128)
        _check(_load().or_api_conjugate(self._fp.ref(), t, _p(re, C.c_double), _p(im, C.c_double),
                                        _p(out.view(np.float64), C.c_double)))
        return out

    def compute_features(self, a, t):
        out = np.zeros(self.sizes(t)[3])
        src = self._cplx(a) if self._gtinv else np.ascontiguousarray(np.asarray(a, dtype=np.float64))
        _check(_load().or_api_features(self._fp.ref(), t, _p(src, C.c_double), _p(out, C.c_double)))
        return out

    def compute_features_deriv(self, a, dfx, dfy, dfz, ds, t):
        nl = self.sizes(t)[3]
        n_col = np.asarray(dfx).shape[1]
        outs = [np.zeros((nl, n_col)), np.zeros((nl, n_col)), np.zeros((nl, n_col)), np.zeros((nl, 6))]
        ins = [self._cplx(v) for v in (a, dfx, dfy, dfz, ds)]
        _check(_load().or_api_features_deriv(self._fp.ref(), t, *[_p(v, C.c_double) for v in ins], n_col,
                                             *[_p(o, C.c_double) for o in outs]))
        return outs

    def compute_sum_of_prod(self, a, t):
        n = self.sizes(t)[4]
        if self._gtinv:
            src, pe, pf = self._cplx(a), np.zeros(n, np.complex128), np.zeros(n, np.complex128)
            pe_p, pf_p = pe.view(np.float64), pf.view(np.float64)
        else:
            src, pe, pf = np.ascontiguousarray(np.asarray(a, dtype=np.float64)), np.zeros(n), np.zeros(n)
            pe_p, pf_p = pe, pf
        _check(_load().or_api_sum_of_prod(self._fp.ref(), _p(self._c, C.c_double), len(self._c), t,
                                          _p(src, C.c_double), _p(pe_p, C.c_double), _p(pf_p, C.c_double)))
        return pe, pf
