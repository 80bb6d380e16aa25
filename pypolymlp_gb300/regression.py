"""Regression on the GPU: X^T X assembly, ridge solve and model selection.

The data preparation restates the reference's semantics exactly, since it
decides the targets and weights that the GPU Gram consumes:

* minimum energy per atom over all datasets (get_min_energy,
  src/pypolymlp/mlp_dev/core/utils.py:10-21),
* row weights and weighted targets (apply_weights,
  src/pypolymlp/mlp_dev/core/utils_weights.py:10-98),
* column scales from the unweighted energy rows and zeroed columns
  (compute_scales / round_scales, src/pypolymlp/mlp_dev/core/utils_scales.py:6-40;
  data_sequential.py:76-90),
* ridge solve for every alpha (solver_ridge, standard/solvers.py:48-84),
* RMSE from Gram quantities and selection by test RMSE
  (compute_rmse_seq / get_best_model, mlp_dev/core/utils_model_selection.py:37-117).

X never leaves the device: pg_gram_accumulate generates the rows of a batch
of structures, weights them and adds X^T X, X^T y, y^T y and the energy-row
column sums in one call.
"""

from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

from . import _ffi
from .abi import Structures, row_layout


@dataclass
class Dataset:
    """Structures with DFT energies, forces (N, 3 per structure) and stresses
    (n_st x 6, xx yy zz xy yz zx, eV per cell), as the reference's Dataset
    holds them after _set_properties (src/pypolymlp/core/dataset_utils.py:200-250)."""

    axis: List[np.ndarray]
    positions: List[np.ndarray]
    types: List[np.ndarray]
    energies: np.ndarray
    forces: Optional[List[np.ndarray]] = None
    stresses: Optional[np.ndarray] = None
    include_force: bool = True
    include_stress: bool = True
    weight: float = 1.0
    name: str = "data"

    @classmethod
    def from_structure_set(cls, sset, include_force=True, include_stress=True, weight=1.0, name="data"):
        return cls(list(sset.axis), list(sset.positions), list(sset.types), np.asarray(sset.energies),
                   sset.forces, sset.stresses, include_force, include_stress, weight, name)

    def __len__(self):
        return len(self.types)

    @property
    def total_n_atoms(self):
        return np.array([len(t) for t in self.types], dtype=np.int64)

    def slice(self, b, e):
        return Dataset(self.axis[b:e], self.positions[b:e], self.types[b:e], self.energies[b:e],
                       None if self.forces is None else self.forces[b:e],
                       None if self.stresses is None else self.stresses[b:e],
                       self.include_force, self.include_stress, self.weight, self.name)


def get_min_energy(datasets: Sequence[Dataset]) -> float:
    min_e = 1e10
    for d in datasets:
        if len(d.energies) == 0:
            raise RuntimeError("Empty energy data.")
        m = float(np.min(d.energies / d.total_n_atoms))
        min_e = min(min_e, m)
    return min_e


def _weight_energy(energy, n_atoms, min_e):
    e_per_atom = energy / n_atoms
    e_th1, e_th2 = min_e * 0.75, min_e * 0.50
    w = np.ones(len(energy))
    w[e_per_atom > e_th1] = 0.5
    w[e_per_atom > e_th2] = 0.3
    w[e_per_atom > 0.0] = 0.1
    return w


def _weight_force(forces, tol=1e-12):
    w = np.abs(forces)
    w[w < tol] = tol
    w = np.reciprocal(w)
    w[w > 1.0] = 1.0
    return w


def _weight_stress(stress, weight_stress, tol=1e-12):
    nonzero = np.abs(stress) > tol
    log1 = np.ones(len(stress)) * np.log10(tol)
    log1[nonzero] = np.log10(np.abs(stress)[nonzero])
    w = np.power(5, -log1)
    w[w > 1.0] = 1.0
    return w * weight_stress


def weights_and_targets(d: Dataset, min_e: float, weight_stress: float = 0.1):
    """Row layout (energies, stresses, forces) of a dataset with its weights w
    and weighted targets y (apply_weights)."""
    n_atoms = d.total_n_atoms
    force = [d.include_force] * len(d)
    e_row, f_row, s_row, n_rows = row_layout(n_atoms, force)
    w = np.ones(n_rows)
    y = np.zeros(n_rows)
    we = _weight_energy(np.asarray(d.energies, float), n_atoms, min_e) * d.weight
    w[e_row] = we
    y[e_row] = we * d.energies
    if d.include_force:
        fvec = np.concatenate([np.asarray(f, float).reshape(-1) for f in d.forces])
        svec = np.asarray(d.stresses, float).reshape(-1)
        f0 = int(f_row[0])
        s0 = int(s_row[0])
        wf = _weight_force(fvec) * d.weight
        w[f0:f0 + len(fvec)] = wf
        y[f0:f0 + len(fvec)] = wf * fvec
        if d.include_stress:
            ws = _weight_stress(svec, weight_stress * d.weight)
            w[s0:s0 + len(svec)] = ws
            y[s0:s0 + len(svec)] = ws * svec
        else:
            # stress rows are zeroed when forces are present without stresses
            w[s0:s0 + len(svec)] = 0.0
            y[s0:s0 + len(svec)] = 0.0
    return e_row, f_row, s_row, n_rows, w, y


class GramAccumulator:
    """Owner of a pg_gram handle."""

    def __init__(self, model: _ffi.Model, precision: int):
        self.model = model
        h = _ffi._vp()
        _ffi.check(_ffi.lib().pg_gram_create(model.handle, int(precision), C.byref(h)))
        self._h = h
        self.F = model.n_features

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and _ffi._lib is not None:
            _ffi._lib.pg_gram_destroy(h)
            self._h = None

    def accumulate(self, st: Structures, e_row, f_row, s_row, n_rows, w, y):
        e_row = np.ascontiguousarray(e_row, dtype=np.int64)
        f_row = np.ascontiguousarray(f_row, dtype=np.int64)
        s_row = np.ascontiguousarray(s_row, dtype=np.int64)
        w = np.ascontiguousarray(w, dtype=np.float64)
        y = np.ascontiguousarray(y, dtype=np.float64)
        p = _ffi._p
        _ffi.check(_ffi.lib().pg_gram_accumulate(self._h, C.cast(st.ref(), _ffi._vp), p(e_row, C.c_int64),
                                                 p(f_row, C.c_int64), p(s_row, C.c_int64), C.c_int64(n_rows),
                                                 p(w, C.c_double), p(y, C.c_double)))

    def reset(self):
        _ffi.check(_ffi.lib().pg_gram_reset(self._h))

    def accumulate_batch(self, batch: "DeviceBatch"):
        _ffi.check(_ffi.lib().pg_gram_accumulate_batch(self._h, batch.handle))

    def result(self):
        F = self.F
        xtx = np.zeros((F, F), order="F")
        xty = np.zeros(F)
        xe_sum = np.zeros(F)
        xe_sq = np.zeros(F)
        yty = C.c_double()
        n = C.c_int64()
        p = _ffi._p
        _ffi.check(_ffi.lib().pg_gram_result(self._h, p(xtx, C.c_double), p(xty, C.c_double), C.byref(yty),
                                             p(xe_sum, C.c_double), p(xe_sq, C.c_double), C.byref(n)))
        return xtx, xty, yty.value, xe_sum, xe_sq, n.value


class DeviceBatch:
    """A dataset staged in HBM (pg_batch): structures, row layout, weights and
    weighted targets, ready for repeated pg_gram_accumulate_batch calls."""

    def __init__(self, model: _ffi.Model, d: Dataset, min_energy: float, precision: int,
                 weight_stress: float = 0.1):
        e_row, f_row, s_row, n_rows, w, y = weights_and_targets(d, min_energy, weight_stress)
        st = Structures(d.axis, d.positions, d.types)
        self.n_rows = int(n_rows)
        p = _ffi._p
        e_row = np.ascontiguousarray(e_row, dtype=np.int64)
        f_row = np.ascontiguousarray(f_row, dtype=np.int64)
        s_row = np.ascontiguousarray(s_row, dtype=np.int64)
        w = np.ascontiguousarray(w)
        y = np.ascontiguousarray(y)
        h = _ffi._vp()
        _ffi.check(_ffi.lib().pg_batch_create(model.handle, C.cast(st.ref(), _ffi._vp), p(e_row, C.c_int64),
                                              p(f_row, C.c_int64), p(s_row, C.c_int64), C.c_int64(n_rows),
                                              p(w, C.c_double), p(y, C.c_double), int(precision), C.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def pair_counts(self, n_type: int) -> np.ndarray:
        """Neighbour pairs of the force structures by (centre type, neighbour
        type), from the lists of the last accumulation (zeros before)."""
        out = np.zeros(n_type * n_type, np.int64)
        _ffi.check(_ffi.lib().pg_batch_pair_counts(self._h, int(n_type), _ffi._p(out, C.c_int64)))
        return out.reshape(n_type, n_type)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and _ffi._lib is not None:
            _ffi._lib.pg_batch_destroy(h)
            self._h = None


@dataclass
class DataXY:
    xtx: np.ndarray
    xty: np.ndarray
    y_sq_norm: float
    total_n_data: int
    scales: np.ndarray
    zero_ids: np.ndarray
    min_energy: float
    xe_sum: Optional[np.ndarray] = None
    xe_sq_sum: Optional[np.ndarray] = None


def compute_scales(scales, xe_sum, xe_sq_sum, n_data, include_force=True, threshold=1e-10):
    if scales is None:
        variance = xe_sq_sum / n_data - np.square(xe_sum / n_data)
        variance[variance < 0.0] = 1.0
        scales = np.sqrt(variance)
    scales = np.array(scales, dtype=float)
    if include_force:
        zero_ids = np.abs(scales) < threshold
    else:
        zero_ids = np.abs(scales) < threshold * threshold
    scales[zero_ids] = 1.0
    return scales, zero_ids


def calc_xtx_xty(model: _ffi.Model, datasets: Sequence[Dataset], precision: int = _ffi.PG_MIXED,
                 scales=None, min_energy=None, weight_stress: float = 0.1, batch_size: int = 2000,
                 scale_threshold: float = 1e-10) -> DataXY:
    """GPU counterpart of calc_xtx_xty (data_sequential.py:25-94)."""
    if min_energy is None:
        min_energy = get_min_energy(datasets)
    acc = GramAccumulator(model, precision)
    for d in datasets:
        for b in range(0, len(d), batch_size):
            sub = d.slice(b, min(len(d), b + batch_size))
            e_row, f_row, s_row, n_rows, w, y = weights_and_targets(sub, min_energy, weight_stress)
            st = Structures(sub.axis, sub.positions, sub.types)
            acc.accumulate(st, e_row, f_row, s_row, n_rows, w, y)
    xtx, xty, yty, xe_sum, xe_sq, n_rows_total = acc.result()
    n_data = sum(len(d.energies) for d in datasets)
    include_force = any(d.include_force for d in datasets)
    scales, zero_ids = compute_scales(scales, xe_sum, xe_sq, n_data, include_force, scale_threshold)
    xtx[zero_ids] = 0.0
    xtx[:, zero_ids] = 0.0
    xty[zero_ids] = 0.0
    xtx /= scales[:, np.newaxis]
    xtx /= scales[np.newaxis, :]
    xty /= scales
    return DataXY(xtx, xty, yty, int(n_rows_total), scales, zero_ids, min_energy, xe_sum, xe_sq)


def solver_ridge(xtx: np.ndarray, xty: np.ndarray, alphas: Sequence[float]) -> np.ndarray:
    """Coefficients (F x n_alpha) of (xtx + alpha I) c = xty for every alpha,
    all alphas factored together on the device; a failed factorisation gives
    a column of 1e30.  xty may also be F x n_alpha: one right-hand side per
    alpha (the corrections of iterative refinement)."""
    F = xtx.shape[0]
    a = np.ascontiguousarray(np.asarray(alphas, dtype=np.float64))
    # xtx is symmetric: a row-major FP64 array is passed as its (equal)
    # transpose, without a column-major copy (3.9 GB at F = 21,945)
    if xtx.dtype == np.float64 and xtx.flags.c_contiguous:
        A = xtx.T
    else:
        A = np.asfortranarray(xtx, dtype=np.float64)
    b = np.asfortranarray(xty, dtype=np.float64)
    coefs = np.zeros((F, len(a)), order="F")
    info = np.zeros(len(a), dtype=np.int32)
    p = _ffi._p
    if b.ndim == 1:
        _ffi.check(_ffi.lib().pg_solve_ridge(F, p(A, C.c_double), p(b, C.c_double), p(a, C.c_double), len(a),
                                             p(coefs, C.c_double), p(info, C.c_int)))
    else:
        if b.shape != (F, len(a)):
            raise ValueError("xty must be F or F x n_alpha")
        _ffi.check(_ffi.lib().pg_solve_ridge_rhs(F, p(A, C.c_double), p(b, C.c_double), p(a, C.c_double), len(a),
                                                 p(coefs, C.c_double), p(info, C.c_int)))
    return np.asarray(coefs), info


def compute_rmse_seq(coefs_array, data_xy: DataXY, check_singular=False, error_threshold=1e6):
    out = []
    for c in coefs_array.T:
        mse = (c @ (data_xy.xtx @ c) - 2 * c @ data_xy.xty + data_xy.y_sq_norm) / data_xy.total_n_data
        out.append(np.sqrt(mse) if mse >= 0 else 1e10)
    out = np.array(out)
    if check_singular and np.all(out > error_threshold):
        raise RuntimeError("Matrix (X.T @ X + alpha * I) may be singular. "
                           "This singularity issue might be reduced by increasing "
                           "the value of alpha (the magnitude of the penalty term).")
    return out


def batch_residual(gram: GramAccumulator, batches: Sequence["DeviceBatch"], coefs: np.ndarray):
    """X^T R (F x k) and per-kind sums of squared weighted residuals (3 x k:
    energy, force, stress) for coefficient columns in X's own scaling."""
    coefs = np.asfortranarray(np.atleast_2d(np.asarray(coefs, dtype=np.float64).T).T)
    F, k = coefs.shape
    xtr_tot = np.zeros((F, k), order="F")
    sq_tot = np.zeros((3, k))
    n_tot = 0
    p = _ffi._p
    for b in batches:
        xtr = np.zeros((F, k), order="F")
        sq = np.zeros((3, k))
        n = C.c_int64()
        _ffi.check(_ffi.lib().pg_batch_residual(gram._h, b.handle, p(coefs, C.c_double), k, p(xtr, C.c_double),
                                                p(sq, C.c_double), C.byref(n)))
        xtr_tot += xtr
        sq_tot += sq
        n_tot += n.value
    return xtr_tot, sq_tot, n_tot


@dataclass
class FitResult:
    coeffs: np.ndarray          # coefficients of the best alpha in the scaled basis
    scales: np.ndarray
    alpha: float
    rmse_train: float
    rmse_test: float
    coefs_array: np.ndarray = field(repr=False, default=None)
    rmse_train_array: np.ndarray = field(repr=False, default=None)
    rmse_test_array: np.ndarray = field(repr=False, default=None)
    info: np.ndarray = field(repr=False, default=None)
    cg_iterations: int = 0                 # conjugate-gradient iterations (fit_cg)
    refine_sweeps: int = 0                 # iterative-refinement sweeps (fit)
    timings: dict = field(repr=False, default=None)  # fit: wall seconds of its phases, training rows

    @property
    def scaled_coeffs(self):
        """Coefficients divided by the scales (the polymlp.yaml convention)."""
        return self.coeffs / self.scales


def _assemble(model: _ffi.Model, train: Sequence[Dataset], precision: int, weight_stress: float,
              scales=None, min_energy=None, zero_ids=None):
    """Training batches on the device, their Gram (one pass) and the scaled
    normal equations: (batches, gram, DataXY)."""
    min_e = get_min_energy(train) if min_energy is None else min_energy
    tb = [DeviceBatch(model, d, min_e, precision, weight_stress) for d in train]
    gram = GramAccumulator(model, precision)
    for b in tb:
        gram.accumulate_batch(b)
    xtx, xty, yty, xe_sum, xe_sq, n_rows = gram.result()
    n_data = sum(len(d.energies) for d in train)
    scales, zids = compute_scales(scales, xe_sum, xe_sq, n_data, any(d.include_force for d in train))
    zero_ids = zids if zero_ids is None else zero_ids
    xtx[zero_ids] = 0.0
    xtx[:, zero_ids] = 0.0
    xty[zero_ids] = 0.0
    xtx /= scales[:, None]
    xtx /= scales[None, :]
    xty /= scales
    return tb, gram, DataXY(xtx, xty, yty, int(n_rows), scales, zero_ids, min_e, xe_sum, xe_sq)


def _select(model, gram, xy: DataXY, test, coefs, alphas, precision, weight_stress, info, n_iter=0, sweeps=0):
    """Training RMSEs from the Gram (compute_rmse_seq, with the reference's
    singularity check), test RMSEs from residuals over the test rows, and the
    alpha of the smallest test RMSE (get_best_model): a FitResult."""
    rmse_train = compute_rmse_seq(coefs, xy, check_singular=True)
    vb = [DeviceBatch(model, d, xy.min_energy, precision, weight_stress) for d in test]
    _, sq, n_te = batch_residual(gram, vb, coefs / xy.scales[:, None])
    rmse_test = np.sqrt(sq.sum(axis=0) / n_te)
    idx = int(np.argmin(rmse_test))
    return FitResult(coefs[:, idx], xy.scales, float(alphas[idx]), float(rmse_train[idx]), float(rmse_test[idx]),
                     coefs, rmse_train, rmse_test, info, n_iter, sweeps)


def solver_cg(xtx: np.ndarray, xty: np.ndarray, alpha: float = 1e-3, coef0: Optional[np.ndarray] = None,
              gtol: float = 1e-2, max_iter: int = 10000):
    """Conjugate gradients on (X^T X + alpha I) c = X^T y as solvers_cg.py:33-100
    runs them: start at coef0 (or 0), stop after more than 100 iterations once
    |r| / sqrt(F) < gtol, or after max_iter.  Returns (c, iterations); c is the
    last iterate, which is what the reference returns (its kept "best" array is
    the running iterate itself, updated in place)."""
    F = xtx.shape[1]
    c = np.zeros(F) if coef0 is None else np.array(coef0, dtype=np.float64)
    r = xty - (xtx @ c + alpha * c)
    d = r.copy()
    rn = float(np.linalg.norm(r))
    it = 0
    for it in range(max_iter):
        if it > 100 and rn / np.sqrt(F) < gtol:
            break
        t = xtx @ d + alpha * d
        lr = rn * rn / float(t @ d)
        c += lr * d
        r -= lr * t
        rn_new = float(np.linalg.norm(r))
        d = r + (rn_new * rn_new) / (rn * rn) * d
        rn = rn_new
    return c, it


def fit_cg(params_dict: dict, train: Sequence[Dataset], test: Sequence[Dataset], alphas: Sequence[float],
           gtol: float = 1e-2, max_iter: Optional[int] = None, precision: int = _ffi.PG_FP64,
           model: Optional[_ffi.Model] = None, weight_stress: float = 0.1) -> FitResult:
    """GPU counterpart of fit_cg (src/pypolymlp/mlp_dev/gradient/fit_cg.py:23-80):
    the Gram from the GPU, then conjugate gradients (`solver_cg`) for the alphas
    from the largest down, each started at the previous solution; model
    selection as `fit`."""
    model = model or _ffi.Model(params_dict)
    alphas = np.asarray(alphas, dtype=np.float64)
    tb, gram, xy = _assemble(model, train, precision, weight_stress)
    if max_iter is None:
        max_iter = max(model.n_features * 3, 50000)
    coefs, c0, n_iter = np.zeros((len(xy.xty), len(alphas))), None, 0
    for k in reversed(range(len(alphas))):
        c0, it = solver_cg(xy.xtx, xy.xty, float(alphas[k]), c0, gtol, max_iter)
        coefs[:, k] = c0
        n_iter += it
    return _select(model, gram, xy, test, coefs, alphas, precision, weight_stress,
                   np.zeros(len(alphas), dtype=np.int32), n_iter=n_iter)


def fit_learning_curve(params_dict: dict, train: Sequence[Dataset], test: Sequence[Dataset],
                       alphas: Sequence[float], precision: int = _ffi.PG_FP64, weight_stress: float = 0.1):
    """GPU counterpart of fit_learning_curve (src/pypolymlp/mlp_dev/standard/fit.py:115-179):
    ridge fits on the first n structures of the single training dataset, n =
    n_train // 10, 2 n_train // 10, ..., with the scales and the reference
    energy of the whole training set; after each, the best model's errors on
    every test dataset (`accuracy.PolymlpEvalAccuracy`).  Returns
    [[n, error dict], ...] in that order."""
    from pypolymlp_gb300.accuracy import PolymlpEvalAccuracy

    if len(train) != 1:
        raise RuntimeError("Number of training datasets must be one for learning curve.")
    model = _ffi.Model(params_dict)
    full = train[0]
    _, _, full_xy = _assemble(model, [full], precision, weight_stress)
    n_train = len(full)
    step = max(n_train // 10, 1)
    log = []
    for n in range(step, n_train + 1, step):
        sub = full.slice(0, n)
        tb, gram, xy = _assemble(model, [sub], precision, weight_stress, scales=full_xy.scales,
                                 min_energy=full_xy.min_energy, zero_ids=full_xy.zero_ids)
        coefs, info = solver_ridge(xy.xtx, xy.xty, alphas)
        best = _select(model, gram, xy, test, coefs, np.asarray(alphas, dtype=np.float64), precision,
                       weight_stress, info)
        acc = PolymlpEvalAccuracy(params_dict, best.scaled_coeffs, precision=precision)
        for d in test:
            log.append([n, acc.compute_error_single(d, log_energy=False)])
    return log


def fit(params_dict: dict, train: Sequence[Dataset], test: Sequence[Dataset], alphas: Sequence[float],
        precision: int = _ffi.PG_MIXED, model: Optional[_ffi.Model] = None, refine: int = 0,
        weight_stress: float = 0.1) -> FitResult:
    """GPU counterpart of fit() (src/pypolymlp/mlp_dev/standard/fit.py:12-60).

    One pass over the training rows assembles the Gram (PG_MIXED: FP32 rows
    and the tensor-core Gram of those rows, accurate to ~1e-12; PG_FP64: FP64
    rows and an FP64 Gram), then the ridge systems of all alphas are solved
    directly on the device (Cholesky, as posv).  `refine` > 0 adds that many
    iterative-refinement sweeps c += (A + alpha I)^-1 (X^T (y - X c) - alpha c),
    each with the residual from a fresh pass over the training rows (the rows
    at the same precision; the direct solve already matches them, so the
    default is none).  Training RMSEs come from the Gram and test RMSEs from
    residuals over the test rows; the best alpha has the smallest test RMSE."""
    model = model or _ffi.Model(params_dict)
    alphas = np.asarray(alphas, dtype=np.float64)
    t0 = time.perf_counter()
    tb, gram, xy = _assemble(model, train, precision, weight_stress)
    t1 = time.perf_counter()
    coefs, info = solver_ridge(xy.xtx, xy.xty, alphas)
    t2 = time.perf_counter()
    for _ in range(int(refine)):
        xtr, _, _ = batch_residual(gram, tb, coefs / xy.scales[:, None])
        r = xtr / xy.scales[:, None] - coefs * alphas[None, :]
        r[xy.zero_ids] = 0.0
        dc, info = solver_ridge(xy.xtx, np.asfortranarray(r), alphas)
        coefs = np.where(info[None, :] == 0, coefs + dc, 1e30)
    t3 = time.perf_counter()
    res = _select(model, gram, xy, test, coefs, alphas, precision, weight_stress, info, sweeps=int(refine))
    res.timings = {"assemble_s": t1 - t0, "solve_s": t2 - t1, "refine_s": t3 - t2,
                   "select_s": time.perf_counter() - t3, "train_rows": xy.total_n_data}
    return res
