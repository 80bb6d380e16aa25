"""Tensor-core Gram (tcgen05, fixed-point BF16 slices) against numpy.

Two bounds per case:
* against tests/gram_slices.py, the FP64 restatement of the slice arithmetic:
  |G - G_slices| <= 3e-11 (|X|^T |X|) elementwise (A1, A2 exact; A3, ~2^-15 of
  |x_a x_b|, rounds at 2^-24 of itself in each of its MMAs, a random walk of
  2^-39 steps; A4 and the float-float segment sums round far below that);
* against the FP64 Gram of the same FP32 rows: each element is quantised to
  2^-28 of its segment's column maximum m, so |G - X^T X| <= 2^-26 (m_seg^T |X|
  + |X|^T m_seg) summed over segments, plus the above.
Shapes cover F not a multiple of the 128-wide tile, rows not a multiple of
the 32-row stage or of the 1,024-row segment, fewer rows than one stage,
several segments and row splits, columns of very different magnitudes,
columns with a wide range inside a segment and all-zero columns.
"""

import numpy as np
import pytest

from gram_slices import SEG, gram_slices

pytestmark = pytest.mark.gpu


def _x(rows, F, seed):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(rows, F)) * rng.uniform(0.1, 10.0, size=F)[None, :]
    if F > 4:
        x[:, 1] *= 1e-12                                        # small column
        x[:, 2] = 0.0                                           # zero column
        x[:, 3] *= np.exp(rng.uniform(-20, 5, size=rows))       # wide range inside a column
    return x.astype(np.float32).astype(np.float64)


def _quant_bound(x):
    ax = np.abs(x)
    B = np.zeros((x.shape[1],) * 2)
    for b in range(0, x.shape[0], SEG):
        xs = ax[b:b + SEG]
        m = np.broadcast_to(xs.max(axis=0), xs.shape)
        B += m.T @ xs + xs.T @ m
    return 2.0 ** -26 * B


@pytest.mark.parametrize("rows,F", [(5, 3), (63, 130), (200, 128), (1025, 257), (4100, 300), (70000, 140)])
def test_gram_tc_matches_slices_and_fp64(rows, F):
    from pypolymlp_gb300 import _ffi

    x = _x(rows, F, rows + F)
    got = _ffi.gram_xtx(x, _ffi.PG_MIXED)
    mag = np.abs(x).T @ np.abs(x) + 1e-300
    ref_sl = gram_slices(x)
    err = np.abs(got - ref_sl) / mag
    assert err.max() <= 3e-11, float(err.max())
    ref = x.T @ x
    bound = _quant_bound(x) + 3e-11 * mag
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
