"""CPU tests of the host-side solvers of pypolymlp_gb300.regression."""

import numpy as np

from pypolymlp_gb300.regression import solver_cg


def test_solver_cg_solves_the_ridge_system():
    rng = np.random.default_rng(0)
    a = rng.normal(size=(120, 40))
    xtx, xty = a.T @ a, a.T @ rng.normal(size=120)
    for alpha in (1e-3, 1e-1):
        c, it = solver_cg(xtx, xty, alpha, gtol=1e-12, max_iter=2000)
        want = np.linalg.solve(xtx + alpha * np.eye(40), xty)
        np.testing.assert_allclose(c, want, rtol=1e-8, atol=1e-10 * np.abs(want).max())
        assert 100 < it < 2000


def test_solver_cg_warm_start_and_cap():
    rng = np.random.default_rng(1)
    a = rng.normal(size=(60, 20))
    xtx, xty = a.T @ a, a.T @ rng.normal(size=60)
    c0, _ = solver_cg(xtx, xty, 1e-2, gtol=1e-12, max_iter=500)
    c1, it = solver_cg(xtx, xty, 1e-2, coef0=c0, gtol=1e-12, max_iter=500)
    np.testing.assert_allclose(c1, c0, rtol=1e-9, atol=1e-12)
    _, it = solver_cg(xtx, xty, 1e-2, gtol=0.0, max_iter=7)
    assert it == 6


class _NpFactor:
    """Host Cholesky stand-in for the device preconditioner factor."""

    def __init__(self, a, shift):
        try:
            self.L = np.linalg.cholesky(a + shift * np.eye(len(a)))
            self.info = 0
        except np.linalg.LinAlgError:
            self.info = 1

    def solve(self, r):
        from scipy.linalg import cho_solve

        return cho_solve((self.L, True), r)


def _ridge_pcg(a_exact, a_mixed, b, alphas, max_iter):
    from pypolymlp_gb300.regression import ridge_pcg

    return ridge_pcg(a_mixed, b, np.asarray(alphas), lambda v: a_exact @ v, np.zeros(len(b), bool),
                     max_iter=max_iter, factor=_NpFactor, return_residuals=True)


def test_ridge_pcg_converges_with_an_accurate_preconditioner():
    rng = np.random.default_rng(2)
    x = rng.normal(size=(200, 30))
    a, b = x.T @ x, x.T @ rng.normal(size=200)
    mixed = a * (1 + 1e-7 * rng.uniform(-1, 1, a.shape))
    mixed = (mixed + mixed.T) / 2
    alphas = [1e-3, 1e-1]
    c, it, taus, resid = _ridge_pcg(a, mixed, b, alphas, 60)
    assert np.all(resid <= 1e-10) and it < 60
    for k, al in enumerate(alphas):
        np.testing.assert_allclose(c[:, k], np.linalg.solve(a + al * np.eye(30), b), rtol=1e-8)


def test_ridge_pcg_reports_an_unconverged_small_alpha():
    """Singular values spread over five decades and a 1.5e-5 relative error in
    the mixed matrix: the preconditioner needs a large shift, the smallest
    alpha is not solved in 60 iterations, and the residual says so (the fit then
    falls back to FP64)."""
    rng = np.random.default_rng(3)
    u, _ = np.linalg.qr(rng.normal(size=(400, 50)))
    v, _ = np.linalg.qr(rng.normal(size=(50, 50)))
    x = (u * np.logspace(0, -5, 50)) @ v.T * 100.0
    a, b = x.T @ x, x.T @ rng.normal(size=400)
    e = rng.uniform(-1, 1, a.shape)
    mixed = a + (e + e.T) / 2 * 1.5e-5 * (np.abs(x).T @ np.abs(x))
    c, it, taus, resid = _ridge_pcg(a, mixed, b, [1e-6, 1.0], 60)
    assert resid[0] > 1e-8 and taus[0] > 0
    assert resid[1] <= 1e-10
