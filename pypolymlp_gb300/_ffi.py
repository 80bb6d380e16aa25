"""ctypes binding of libpolymlp_gb300.so (include/polymlp_gb300.h).

The library is built in-tree by `pypolymlp_gb300.build.build()`.  There is no
CPU fallback: if the library or a CUDA device is missing, every entry point
raises.
"""

from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

from .abi import FeatureParams, Structures

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "lib", "libpolymlp_gb300.so")
_lib = None
_lock = threading.Lock()

PG_FP64 = 0
PG_MIXED = 1

_i64p = C.POINTER(C.c_int64)
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_vp = C.c_void_p


class GB300Error(RuntimeError):
    pass


def lib():
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise GB300Error(
                    f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                    "(there is no CPU fallback)"
                )
            L = C.CDLL(LIB_PATH)
            L.pg_last_error.argtypes = [C.c_char_p, C.c_size_t]
            L.pg_device_count.argtypes = [_ip]
            L.pg_set_stream.argtypes = [_vp]
            L.pg_get_stream.argtypes = [C.POINTER(_vp)]
            L.pg_model_create.argtypes = [_vp, C.POINTER(_vp)]
            L.pg_model_destroy.argtypes = [_vp]
            L.pg_model_n_features.argtypes = [_vp, _ip]
            L.pg_model_feature_attrs.argtypes = [_vp, _ip, _ip, _ip, _ip, _ip, _ip, _ip, _ip, _ip, _ip]
            L.pg_feature_attrs.argtypes = [_vp, _ip, _ip, _ip, _ip, _ip, _ip, _ip, _ip, _ip, _ip, _ip]
            L.pg_features_x.argtypes = [_vp, _vp, _i64p, _i64p, _i64p, _dp, C.c_int64, C.c_int]
            L.pg_neighbor_list.argtypes = [_vp, C.c_int, C.c_double, C.c_int, _i64p, _ip, _ip, _dp]
            for name, args in [
                ("pg_gram_create", [_vp, C.c_int, C.POINTER(_vp)]),
                ("pg_gram_destroy", [_vp]),
                ("pg_gram_accumulate", [_vp, _vp, _i64p, _i64p, _i64p, C.c_int64, _dp, _dp]),
                ("pg_gram_result", [_vp, _dp, _dp, _dp, _dp, _dp, _i64p]),
                ("pg_gram_reset", [_vp]),
                ("pg_batch_create", [_vp, _vp, _i64p, _i64p, _i64p, C.c_int64, _dp, _dp, C.c_int, C.POINTER(_vp)]),
                ("pg_batch_destroy", [_vp]),
                ("pg_gram_accumulate_batch", [_vp, _vp]),
                ("pg_batch_residual", [_vp, _vp, _dp, C.c_int, _dp, _dp, _i64p]),
                ("pg_gram_xtx", [_dp, C.c_int64, C.c_int, C.c_int64, C.c_int, _dp]),
                ("pg_profile_enable", [C.c_int]),
                ("pg_profile_read", [C.c_char_p, C.c_size_t, _dp, _ip, C.c_int, _ip]),
                ("pg_solve_ridge", [C.c_int, _dp, _dp, _dp, C.c_int, _dp, _ip]),
                ("pg_solve_ridge_rhs", [C.c_int, _dp, _dp, _dp, C.c_int, _dp, _ip]),
                ("pg_model_work", [_vp, _ip, _ip, _ip, _ip, _i64p]),
                ("pg_model_xrow_work", [_vp, _ip, _ip]),
                ("pg_batch_pair_counts", [_vp, C.c_int, _i64p]),
                ("pg_solve_ridge_noalloc", [C.c_int, _vp, _vp, C.c_double, _vp, _ip]),
                ("pg_eval_create", [_vp, _dp, C.c_int, C.c_int, C.POINTER(_vp)]),
                ("pg_eval_destroy", [_vp]),
                ("pg_eval_run", [_vp, _vp, _dp, _dp, _dp]),
                ("pg_eval_bind", [_vp, _vp, C.c_double]),
                ("pg_eval_update", [_vp, _dp, _ip]),
                ("pg_eval_bound_energy", [_vp, _dp]),
                ("pg_eval_bound_run", [_vp, _dp, _dp, _dp]),
                ("pg_eval_workspace_bytes", [_vp, _i64p]),
            ]:
                if hasattr(L, name):
                    getattr(L, name).argtypes = args
            _lib = L
    return _lib


def check(rc: int):
    if rc != 0:
        buf = C.create_string_buffer(4096)
        lib().pg_last_error(buf, 4096)
        raise GB300Error(buf.value.decode(errors="replace"))


def device_count() -> int:
    n = C.c_int()
    check(lib().pg_device_count(C.byref(n)))
    return n.value


def set_stream(stream=None):
    """Issue the calling thread's later library calls on `stream`: a
    torch.cuda.Stream, a raw cudaStream_t handle (int), or None for the legacy
    default stream (pg_set_stream).  Every call still returns with its results
    on the host; the stream orders its device work against the caller's."""
    h = 0 if stream is None else int(getattr(stream, "cuda_stream", stream))
    check(lib().pg_set_stream(_vp(h)))


def get_stream() -> int:
    """The raw cudaStream_t handle of the calling thread (0: legacy default)."""
    h = _vp()
    check(lib().pg_get_stream(C.byref(h)))
    return int(h.value or 0)


class on_stream:
    """Context manager: library calls of this thread on `stream`, then back."""

    def __init__(self, stream):
        self.stream = stream

    def __enter__(self):
        self.prev = get_stream()
        set_stream(self.stream)
        return self

    def __exit__(self, *exc):
        set_stream(self.prev)


def require_device():
    if device_count() < 1:
        raise GB300Error("no CUDA device is visible: the GB300 hot path has no CPU fallback")


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


class Model:
    """Handle of pg_model (model tables uploaded to the device)."""

    def __init__(self, params_dict: dict):
        require_device()
        self.fp = FeatureParams(params_dict)
        self.params_dict = params_dict
        h = _vp()
        check(lib().pg_model_create(C.cast(self.fp.ref(), _vp), C.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and _lib is not None:
            _lib.pg_model_destroy(h)
            self._h = None

    @property
    def n_features(self) -> int:
        n = C.c_int()
        check(lib().pg_model_n_features(self._h, C.byref(n)))
        return n.value

    def features_x(self, st: Structures, e_row, f_row, s_row, n_rows: int, precision: int = PG_FP64, out=None):
        nf = self.n_features
        if out is None:
            out = np.zeros((n_rows, nf), dtype=np.float64, order="F")
        if out.dtype != np.float64 or not out.flags["F_CONTIGUOUS"] or out.shape[1] != nf:
            raise ValueError("out must be a Fortran-ordered float64 array with n_features columns")
        e_row = np.ascontiguousarray(e_row, dtype=np.int64)
        f_row = np.ascontiguousarray(f_row, dtype=np.int64)
        s_row = np.ascontiguousarray(s_row, dtype=np.int64)
        check(lib().pg_features_x(self._h, C.cast(st.ref(), _vp), _p(e_row, C.c_int64), _p(f_row, C.c_int64),
                                  _p(s_row, C.c_int64), _p(out, C.c_double), C.c_int64(out.shape[0]),
                                  int(precision)))
        return out

    def work(self):
        """{n_type, max_l, n_radial, k0_pair (n_type x n_type heads), n_terms (per type)}."""
        L = lib()
        nt, ml, nr = C.c_int(), C.c_int(), C.c_int()
        check(L.pg_model_work(self._h, C.byref(nt), C.byref(ml), C.byref(nr), C.POINTER(C.c_int)(),
                              C.POINTER(C.c_int64)()))
        k0 = np.zeros(nt.value * nt.value, np.int32)
        terms = np.zeros(nt.value, np.int64)
        check(L.pg_model_work(self._h, C.byref(nt), C.byref(ml), C.byref(nr), _p(k0, C.c_int),
                              _p(terms, C.c_int64)))
        return {"n_type": nt.value, "max_l": ml.value, "n_radial": nr.value,
                "k0_pair": k0.reshape(nt.value, nt.value), "n_terms": terms}

    def xrow_work(self):
        """{n_entries, n_positions}: per (centre type, neighbour type) the adjoint
        entries and the linear features with entries of that type pair."""
        n = self.work()["n_type"]
        ne = np.zeros(n * n, np.int32)
        npos = np.zeros(n * n, np.int32)
        check(lib().pg_model_xrow_work(self._h, _p(ne, C.c_int), _p(npos, C.c_int)))
        return {"n_entries": ne.reshape(n, n), "n_positions": npos.reshape(n, n)}

    def feature_attrs(self):
        L = lib()
        nl, ntv, npoly, npv = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        null = C.POINTER(C.c_int)()
        check(L.pg_model_feature_attrs(self._h, C.byref(nl), null, null, C.byref(ntv), null, null, C.byref(npoly),
                                       C.byref(npv), null, null))
        rad = np.zeros(max(nl.value, 1), np.int32)
        gt = np.zeros(max(nl.value, 1), np.int32)
        tco = np.zeros(nl.value + 1, np.int32)
        tcv = np.zeros(max(ntv.value, 1), np.int32)
        po = np.zeros(npoly.value + 1, np.int32)
        pv = np.zeros(max(npv.value, 1), np.int32)
        check(L.pg_model_feature_attrs(self._h, C.byref(nl), _p(rad, C.c_int), _p(gt, C.c_int), C.byref(ntv),
                                       _p(tco, C.c_int), _p(tcv, C.c_int), C.byref(npoly), C.byref(npv),
                                       _p(po, C.c_int), _p(pv, C.c_int)))
        tcomb = [tcv[tco[i]:tco[i + 1]].tolist() for i in range(nl.value)]
        poly = [pv[po[i]:po[i + 1]].tolist() for i in range(npoly.value)]
        return rad[:nl.value].tolist(), gt[:nl.value].tolist(), tcomb, poly


def neighbor_list(st: Structures, s: int, cutoff: float):
    L = lib()
    n = C.c_int64()
    null_i = C.POINTER(C.c_int)()
    check(L.pg_neighbor_list(C.cast(st.ref(), _vp), s, cutoff, 0, C.byref(n), null_i, null_i,
                             C.POINTER(C.c_double)()))
    na = int(st.n_atoms[s])
    offs = np.zeros(na + 1, np.int32)
    nb = np.zeros(max(n.value, 1), np.int32)
    d = np.zeros((max(n.value, 1), 3))
    check(L.pg_neighbor_list(C.cast(st.ref(), _vp), s, cutoff, 0, C.byref(n), _p(offs, C.c_int), _p(nb, C.c_int),
                             _p(d, C.c_double)))
    return offs, nb[:n.value], d[:n.value]


def gram_xtx(x: np.ndarray, precision: int = PG_MIXED) -> np.ndarray:
    """X^T X of a host block on the device (pg_gram_xtx)."""
    require_device()
    x = np.asfortranarray(x, dtype=np.float64)
    n, F = x.shape
    out = np.zeros((F, F), order="F")
    check(lib().pg_gram_xtx(_p(x, C.c_double), n, F, max(n, 1), int(precision), _p(out, C.c_double)))
    return out


def profile_enable(on: bool = True):
    check(lib().pg_profile_enable(1 if on else 0))


def profile_read():
    """{kernel name: (total ms, launches)} since the previous read."""
    names = C.create_string_buffer(8192)
    ms = np.zeros(64)
    launches = np.zeros(64, dtype=np.int32)
    n = C.c_int()
    check(lib().pg_profile_read(names, 8192, _p(ms, C.c_double), _p(launches, C.c_int), 64, C.byref(n)))
    out = {}
    raw = names.raw
    pos = 0
    for k in range(n.value):
        end = raw.index(b"\0", pos)
        out[raw[pos:end].decode()] = (float(ms[k]), int(launches[k]))
        pos = end + 1
    return out


class Evaluator:
    """Handle of pg_eval: energies, forces and stresses of structures on the GPU."""

    def __init__(self, params_dict: dict, coeffs, precision: int = PG_FP64):
        require_device()
        self.fp = FeatureParams(params_dict)
        self.coeffs = np.ascontiguousarray(coeffs, dtype=np.float64).reshape(-1)
        h = _vp()
        check(lib().pg_eval_create(C.cast(self.fp.ref(), _vp), _p(self.coeffs, C.c_double), len(self.coeffs),
                                   int(precision), C.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and _lib is not None:
            _lib.pg_eval_destroy(h)
            self._h = None

    def run(self, st: Structures):
        """(energy (n_st,), forces (sum N, 3) atom-major, stress (n_st, 6))."""
        e = np.zeros(st.n_st)
        f = np.zeros((int(st.n_atoms.sum()), 3))
        s = np.zeros((st.n_st, 6))
        check(lib().pg_eval_run(self._h, C.cast(st.ref(), _vp), _p(e, C.c_double), _p(f, C.c_double),
                                _p(s, C.c_double)))
        return e, f, s

    # -- bound structures: neighbour lists kept across position updates --------
    def bind(self, st: Structures, skin: float = 0.5):
        """Stage `st` for repeated evaluation with lists built at cutoff + skin."""
        check(lib().pg_eval_bind(self._h, C.cast(st.ref(), _vp), float(skin)))
        self._bound = (st.n_st, int(st.n_atoms.sum()), st)

    def update(self, positions) -> bool:
        """New Cartesian positions (sum N x 3) of the bound atoms; True if the
        neighbour lists were rebuilt."""
        pos = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
        if pos.shape[0] != self._bound[1]:
            raise ValueError("positions do not match the bound atoms")
        r = C.c_int()
        check(lib().pg_eval_update(self._h, _p(pos, C.c_double), C.byref(r)))
        return bool(r.value)

    def bound_energy(self):
        e = np.zeros(self._bound[0])
        check(lib().pg_eval_bound_energy(self._h, _p(e, C.c_double)))
        return e

    def bound_run(self):
        n_st, n_at, _ = self._bound
        e, f, s = np.zeros(n_st), np.zeros((n_at, 3)), np.zeros((n_st, 6))
        check(lib().pg_eval_bound_run(self._h, _p(e, C.c_double), _p(f, C.c_double), _p(s, C.c_double)))
        return e, f, s

    def workspace_bytes(self) -> int:
        n = C.c_int64()
        check(lib().pg_eval_workspace_bytes(self._h, C.byref(n)))
        return int(n.value)
