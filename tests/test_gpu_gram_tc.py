"""Tensor-core Gram (tcgen05, BF16x3) against an FP64 numpy X^T X.

Bound: the BF16x3 products drop the lo x lo term (2^-16 of |x_i x_j|) and X is
rounded to FP32, so |G - X^T X| <= 3e-5 (|X|^T |X|) elementwise.  Shapes cover
F not a multiple of the 128-wide tile, rows not a multiple of the 64-row stage,
fewer rows than one stage, several FP32 segments (4,096 rows) and row splits.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("rows,F", [(5, 3), (63, 130), (200, 128), (4097, 257), (20000, 300), (70000, 140)])
def test_gram_tc_matches_fp64(rows, F):
    from pypolymlp_gb300 import _ffi

    rng = np.random.default_rng(rows + F)
    x = rng.normal(size=(rows, F)) * rng.uniform(0.1, 10.0, size=F)[None, :]
    ref = x.T @ x
    got = _ffi.gram_xtx(x, _ffi.PG_MIXED)
    bound = 3e-5 * (np.abs(x).T @ np.abs(x)) + 1e-300
    assert np.all(np.abs(got - ref) <= bound), float(np.max(np.abs(got - ref) / bound))
    np.testing.assert_array_equal(got, got.T)


def test_gram_fp64_entry_point():
    from pypolymlp_gb300 import _ffi

    rng = np.random.default_rng(7)
    x = rng.normal(size=(300, 70))
    np.testing.assert_allclose(_ffi.gram_xtx(x, _ffi.PG_FP64), x.T @ x, rtol=1e-12, atol=1e-12)


def test_gram_tc_deterministic():
    from pypolymlp_gb300 import _ffi

    x = np.random.default_rng(3).normal(size=(30000, 200))
    np.testing.assert_array_equal(_ffi.gram_xtx(x, _ffi.PG_MIXED), _ffi.gram_xtx(x, _ffi.PG_MIXED))
