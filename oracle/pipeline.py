"""CPU regression pipeline of the reference, for tests and the CPU baseline.

TEST INFRASTRUCTURE ONLY.  X rows come from the CPU oracle (the reference's
algorithm), X^T X and X^T y from numpy BLAS, and the ridge solve from LAPACK
posv through SciPy, exactly as the reference's calc_xtx_xty
(src/pypolymlp/mlp_dev/core/data_sequential.py:25-152) and solver_ridge
(src/pypolymlp/mlp_dev/standard/solvers.py:9-84) do.
"""

from __future__ import annotations

import numpy as np
from scipy.linalg.lapack import get_lapack_funcs

from oracle import oracle
from pypolymlp_gb300.abi import Structures
from pypolymlp_gb300.regression import DataXY, compute_scales, get_min_energy, weights_and_targets


def calc_xtx_xty_cpu(params, datasets, scales=None, min_energy=None, weight_stress=0.1, batch_size=2000,
                     n_threads=0, scale_threshold=1e-10):
    if min_energy is None:
        min_energy = get_min_energy(datasets)
    xtx = xty = xe_sum = xe_sq = None
    yty = 0.0
    n_total = 0
    for d in datasets:
        for b in range(0, len(d), batch_size):
            sub = d.slice(b, min(len(d), b + batch_size))
            e_row, f_row, s_row, n_rows, w, y = weights_and_targets(sub, min_energy, weight_stress)
            st = Structures(sub.axis, sub.positions, sub.types)
            x = oracle.features_x(params, st, e_row, f_row, s_row, n_rows, n_threads=n_threads)
            xe = x[e_row]
            s1, s2 = xe.sum(axis=0), np.square(xe).sum(axis=0)
            xe_sum = s1 if xe_sum is None else xe_sum + s1
            xe_sq = s2 if xe_sq is None else xe_sq + s2
            x *= w[:, None]
            g = x.T @ x
            xtx = g if xtx is None else xtx + g
            v = x.T @ y
            xty = v if xty is None else xty + v
            yty += float(y @ y)
            n_total += n_rows
    n_data = sum(len(d.energies) for d in datasets)
    include_force = any(d.include_force for d in datasets)
    scales, zero_ids = compute_scales(scales, xe_sum, xe_sq, n_data, include_force, scale_threshold)
    xtx[zero_ids] = 0.0
    xtx[:, zero_ids] = 0.0
    xty[zero_ids] = 0.0
    xtx /= scales[:, None]
    xtx /= scales[None, :]
    xty /= scales
    return DataXY(xtx, xty, yty, n_total, scales, zero_ids, min_energy, xe_sum, xe_sq)


def solver_ridge_cpu(xtx, xty, alphas):
    """LAPACK posv (upper) per alpha in ascending order, 1e30 on failure."""
    (posv,) = get_lapack_funcs(("posv",), (xtx, xty))
    F = xtx.shape[0]
    A = np.array(xtx, copy=True)
    out = np.zeros((F, len(alphas)))
    prev = 0.0
    for i, a in enumerate(alphas):
        A.flat[:: F + 1] += a - prev
        _, x, info = posv(A, xty, lower=False, overwrite_a=False, overwrite_b=False)
        out[:, i] = x if info == 0 else 1e30
        prev = a
    return out
