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
