"""GPU regression assembly and ridge solve against the CPU pipeline
(oracle X + numpy X^T X + LAPACK posv).

Tolerances: FP64 Gram 1e-12 relative to max|X^T X|; mixed (FP32 rows, their
Gram from fixed-point BF16 slices) 1e-4 relative, the FP32 rounding of the
rows; ridge coefficients 1e-8 relative to max|c| for every alpha (all alphas
factored together); the fitted energy and force RMSEs of the mixed path
within 0.05 meV/atom and 1 meV/A of the FP64 fit.
"""

import numpy as np
import pytest

from oracle.pipeline import calc_xtx_xty_cpu, solver_ridge_cpu
from pypolymlp_gb300 import synthetic as syn
from pypolymlp_gb300.params import make_params_dict

pytestmark = pytest.mark.gpu


def _datasets(n=24, seed=5):
    ss = syn.fcc_set(n, seed=seed)
    syn.morse_labels(ss, syn.morse_D(1))
    from pypolymlp_gb300.regression import Dataset

    k = int(0.8 * n)
    return [Dataset.from_structure_set(ss.subset(range(k)), name="train")], \
           [Dataset.from_structure_set(ss.subset(range(k, n)), name="test")]


def _params():
    return make_params_dict(n_type=1, cutoff=6.0, model_type=2, max_p=2, gaussian_params2=(0, 5, 8),
                            gtinv_order=2, gtinv_maxl=(4,))


def test_gram_fp64_and_mixed_match_cpu():
    from pypolymlp_gb300 import _ffi
    from pypolymlp_gb300.regression import calc_xtx_xty

    p = _params()
    train, _ = _datasets()
    ref = calc_xtx_xty_cpu(p, train, batch_size=7)
    m = _ffi.Model(p)
    g64 = calc_xtx_xty(m, train, precision=_ffi.PG_FP64, batch_size=7)
    scale = np.abs(ref.xtx).max()
    assert np.abs(g64.xtx - ref.xtx).max() / scale < 1e-12
    assert np.abs(g64.xty - ref.xty).max() / np.abs(ref.xty).max() < 1e-12
    # scales come from E[x^2] - E[x]^2, which cancels: compare loosely
    np.testing.assert_allclose(g64.scales, ref.scales, rtol=1e-8)
    assert abs(g64.y_sq_norm - ref.y_sq_norm) <= 1e-12 * ref.y_sq_norm
    assert g64.total_n_data == ref.total_n_data
    g32 = calc_xtx_xty(m, train, precision=_ffi.PG_MIXED, batch_size=7)
    # the FP32 rounding of the (cancelling) force-row sums; the Gram of those rows is exact to ~1e-12
    assert np.abs(g32.xtx - ref.xtx).max() / scale < 1e-4
    # symmetric up to the rounding of the two-sided column scaling
    assert np.abs(g64.xtx - g64.xtx.T).max() <= 1e-14 * scale


def test_ridge_solve_matches_posv():
    from pypolymlp_gb300.regression import solver_ridge

    rng = np.random.default_rng(0)
    for F, n_alpha in ((5, 3), (64, 3), (130, 3), (300, 8), (1100, 8)):
        B = rng.normal(size=(F + 20, F))
        A = B.T @ B
        b = rng.normal(size=F)
        alphas = list(10.0 ** np.linspace(-4, 0, n_alpha))
        ref = solver_ridge_cpu(A, b, alphas)
        got, info = solver_ridge(A, b, alphas)
        assert (info == 0).all()
        for k in range(n_alpha):
            assert np.abs(got[:, k] - ref[:, k]).max() / np.abs(ref[:, k]).max() < 1e-8, (F, k)


def test_ridge_solve_blocked_triangular_matches_posv():
    """Above F = 4,096 the triangular solves run blocked over many blocks:
    against posv for two alphas, and a third alpha that makes the shifted
    matrix indefinite gives 1e30 while the others stay intact."""
    from pypolymlp_gb300.regression import solver_ridge

    rng = np.random.default_rng(3)
    F = 4500
    B = rng.normal(size=(F + 400, F))
    A = B.T @ B
    b = rng.normal(size=F)
    alphas = [1e-2, 1.0]
    ref = solver_ridge_cpu(A, b, alphas)
    got, info = solver_ridge(A, b, alphas + [-1e9])
    assert info[0] == 0 and info[1] == 0 and info[2] != 0
    for k in range(2):
        assert np.abs(got[:, k] - ref[:, k]).max() / np.abs(ref[:, k]).max() < 1e-8, k
    assert np.all(got[:, 2] == 1e30)


def test_ridge_solve_per_alpha_rhs_and_failures():
    """One right-hand side per alpha (pg_solve_ridge_rhs), and a failed
    factorisation of one alpha leaves the others intact."""
    from pypolymlp_gb300.regression import solver_ridge

    rng = np.random.default_rng(1)
    F = 200
    B = rng.normal(size=(F + 5, F))
    A = B.T @ B - 30.0 * np.eye(F)          # indefinite until alpha exceeds ~30 - lambda_min
    rhs = np.asfortranarray(rng.normal(size=(F, 3)))
    alphas = [1e-3, 100.0, 1000.0]
    got, info = solver_ridge(A, rhs, alphas)
    assert info[0] != 0 and np.all(got[:, 0] == 1e30)
    for k in (1, 2):
        assert info[k] == 0
        want = np.linalg.solve(A + alphas[k] * np.eye(F), rhs[:, k])
        assert np.abs(got[:, k] - want).max() <= 1e-9 * np.abs(want).max()


def test_ridge_singular_gives_1e30():
    from pypolymlp_gb300.regression import solver_ridge

    A = -np.eye(8)
    got, info = solver_ridge(A, np.ones(8), [1e-3])
    assert info[0] != 0
    assert np.all(got == 1e30)


def _energy_force_rmse(params, coefs_unscaled, datasets):
    """Energy RMSE per atom (eV/atom) and force RMSE (eV/A) of a model, with
    predictions from the CPU oracle's FP64 X rows."""
    from oracle import oracle
    from pypolymlp_gb300.abi import Structures, row_layout

    de, df = [], []
    for d in datasets:
        st = Structures(d.axis, d.positions, d.types)
        e, f, s, n = row_layout(st.n_atoms, [True] * st.n_st)
        x = oracle.features_x(params, st, e, f, s, n)
        pred = x @ coefs_unscaled
        de.append((pred[e] - d.energies) / st.n_atoms)
        fr = np.concatenate([pred[f[k]:f[k] + 3 * st.n_atoms[k]] for k in range(st.n_st)])
        df.append(fr - np.concatenate([np.asarray(v).reshape(-1) for v in d.forces]))
    de, df = np.concatenate(de), np.concatenate(df)
    return float(np.sqrt(np.mean(de ** 2))), float(np.sqrt(np.mean(df ** 2)))


def test_fit_mixed_vs_fp64_rmse():
    """End-to-end fit.  FP64 GPU path: test RMSEs of every alpha equal the CPU
    pipeline's (Gram formula, LAPACK posv) to 1e-6.  Mixed path (FP32 rows,
    tensor-core Gram, direct solve): the selected model's energy RMSE within
    0.05 meV/atom and force RMSE within 1 meV/A of the FP64 fit, with and
    without one iterative-refinement sweep."""
    from pypolymlp_gb300 import _ffi
    from pypolymlp_gb300.regression import compute_rmse_seq, fit

    p = _params()
    train, test = _datasets(40, seed=8)
    alphas = [1e-4, 1e-3, 1e-2, 1e-1]
    ref_train = calc_xtx_xty_cpu(p, train)
    coefs = solver_ridge_cpu(ref_train.xtx, ref_train.xty, alphas)
    ref_test = calc_xtx_xty_cpu(p, test, scales=ref_train.scales, min_energy=ref_train.min_energy)
    rmse_ref = compute_rmse_seq(coefs, ref_test)
    r64 = fit(p, train, test, alphas, precision=_ffi.PG_FP64)
    np.testing.assert_allclose(r64.rmse_test_array, rmse_ref, rtol=1e-6)
    e64, f64 = _energy_force_rmse(p, r64.scaled_coeffs, test)
    print(f"fp64: alpha {r64.alpha} rmse_test {r64.rmse_test_array}; E {e64 * 1e3:.4f} meV/atom F {f64 * 1e3:.3f} meV/A")
    for refine in (0, 1):
        r32 = fit(p, train, test, alphas, precision=_ffi.PG_MIXED, refine=refine)
        e32, f32 = _energy_force_rmse(p, r32.scaled_coeffs, test)
        print(f"mixed (refine {refine}): alpha {r32.alpha} rmse_test {r32.rmse_test_array}; "
              f"E {e32 * 1e3:.4f} meV/atom F {f32 * 1e3:.3f} meV/A")
        assert abs(e32 - e64) < 0.05e-3, (refine, e32, e64)
        assert abs(f32 - f64) < 1e-3, (refine, f32, f64)


def test_fit_cg_matches_direct_solve():
    """fit_cg (GPU Gram, conjugate gradients from the largest alpha down, warm
    started) reaches the direct FP64 ridge solution: test RMSEs to 1e-4 (the
    solver stops on an absolute residual, so the smallest alpha, the worst
    conditioned, is the least exact: 5e-6 relative at gtol 1e-9)."""
    from pypolymlp_gb300 import _ffi
    from pypolymlp_gb300.regression import fit, fit_cg

    p = _params()
    train, test = _datasets(30, seed=9)
    alphas = [1e-3, 1e-2, 1e-1]
    direct = fit(p, train, test, alphas, precision=_ffi.PG_FP64)
    cg = fit_cg(p, train, test, alphas, gtol=1e-9, max_iter=20000, precision=_ffi.PG_FP64)
    np.testing.assert_allclose(cg.rmse_test_array, direct.rmse_test_array, rtol=1e-4)
    assert cg.alpha == direct.alpha and cg.cg_iterations > 0


def test_learning_curve():
    """fit_learning_curve: ten fits on growing prefixes of the training set, the
    test errors of each from the GPU evaluator."""
    from pypolymlp_gb300.regression import fit_learning_curve

    p = _params()
    train, test = _datasets(25, seed=10)
    log = fit_learning_curve(p, train, test, [1e-3, 1e-2])
    assert [n for n, _ in log] == list(range(2, 21, 2))
    for _, err in log:
        assert np.isfinite(err["energy"]) and np.isfinite(err["force"]) and err["energy"] < 1.0
