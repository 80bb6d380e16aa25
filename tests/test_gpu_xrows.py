"""GPU X rows (pg_features_x through the C ABI) against the oracle and the
reference's golden signatures.

Tolerances: FP64 path 1e-10 relative to the column magnitude (the bar for
features and derivatives); mixed path (FP32 features, FP64 neighbour sums)
1e-4 relative to the column magnitude.  Per element, over the elements of at
least 1e-3 of their column's magnitude, these bound the error relative to the
element itself by 1e-7 (FP64) and 0.1 (mixed); the oracle comparison prints
the measured per-element figures.
"""

import numpy as np
import pytest

from conftest import assert_signature, load_golden
from oracle import oracle
from pypolymlp_gb300 import synthetic as syn
from pypolymlp_gb300.abi import Structures, row_layout
from pypolymlp_gb300.params import make_params_dict

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-10
MIXED_RTOL = 1e-4


def _model(p):
    from pypolymlp_gb300 import _ffi

    return _ffi.Model(p)


def _colrel(x, ref):
    """Max error relative to the column magnitude, with a floor of 1e-4 of the
    largest |X| (columns that vanish up to rounding carry only noise)."""
    colmax = np.abs(ref).max(axis=0)
    scale = np.maximum(colmax, 1e-4 * max(colmax.max(), 1e-300))
    return float((np.abs(x - ref) / scale).max())


ELEM_FRAC = 1e-3


def _elemrel(x, ref):
    """Max error relative to the element itself, over the elements of at least
    ELEM_FRAC of their column's scale (the scale of _colrel): a column-relative
    error below e bounds it by e / ELEM_FRAC."""
    colmax = np.abs(ref).max(axis=0)
    scale = np.maximum(colmax, 1e-4 * max(colmax.max(), 1e-300))
    big = np.abs(ref) >= ELEM_FRAC * scale
    if not big.any():
        return 0.0
    return float((np.abs(x - ref)[big] / np.abs(ref)[big]).max())


@pytest.mark.parametrize("name", ["x_cfg1.npz", "x_cfg2.npz", "x_cfg3.npz", "x_cfg5p.npz", "x_pair_mt2_p3.npz"])
def test_fp64_rows_match_reference_signature(name):
    from pypolymlp_gb300 import _ffi

    params, st, gold = load_golden(name)
    e, f, s, n = row_layout(st.n_atoms, [True] * st.n_st)
    x = _model(params).features_x(st, e, f, s, n, precision=_ffi.PG_FP64)
    assert_signature(x, gold, rtol=FP64_RTOL)


CASES = {
    "binary_mt3": (dict(n_type=2, cutoff=7.0, model_type=3, max_p=2, gaussian_params2=(0, 5, 10), gtinv_order=3,
                        gtinv_maxl=(8, 4)), lambda: syn.binary_set(3, seed=31)),
    "ternary_mt4_p2": (dict(n_type=3, cutoff=5.0, model_type=4, max_p=2, gaussian_params2=(0, 4, 3), gtinv_order=3,
                            gtinv_maxl=(4, 2)), lambda: syn.ternary_set(3, seed=32, n_range=(8, 70))),
    "binary_mt2_p3": (dict(n_type=2, cutoff=5.0, model_type=2, max_p=3, gaussian_params2=(0, 4, 2), gtinv_order=2,
                           gtinv_maxl=(2,)), lambda: syn.binary_set(2, seed=35, n_min=16, n_max=40)),
    "unary_order4": (dict(n_type=1, cutoff=6.0, model_type=2, max_p=2, gaussian_params2=(0, 5, 5), gtinv_order=4,
                          gtinv_maxl=(8, 8, 2)), lambda: syn.fcc_set(2, seed=33)),
    # the order-4 ternary model of the large fit (F = 21,945, rc 8 A)
    "ternary_order4_rc8": (dict(n_type=3, cutoff=8.0, model_type=3, max_p=2, gaussian_params2=(0, 5, 4),
                                gtinv_order=4, gtinv_maxl=(8, 8, 2)),
                           lambda: syn.ternary_set(2, seed=36, n_range=(24, 40))),
    "pair_mt2_p3": (dict(n_type=2, cutoff=6.0, model_type=2, max_p=3, feature_type="pair",
                         gaussian_params2=(0, 5, 6)), lambda: syn.binary_set(2, seed=34, n_min=16, n_max=40)),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_rows_match_oracle(case):
    from pypolymlp_gb300 import _ffi

    kw, gen = CASES[case]
    p = make_params_dict(**kw)
    ss = gen()
    st = Structures(ss.axis, ss.positions, ss.types)
    force = [i % 3 != 1 for i in range(st.n_st)]  # mix energy-only structures in
    e, f, s, n = row_layout(st.n_atoms, force)
    ref = oracle.features_x(p, st, e, f, s, n)
    m = _model(p)
    x64 = m.features_x(st, e, f, s, n, precision=_ffi.PG_FP64)
    assert _colrel(x64, ref) < FP64_RTOL
    x32 = m.features_x(st, e, f, s, n, precision=_ffi.PG_MIXED)
    assert _colrel(x32, ref) < MIXED_RTOL
    # per element (the elements of at least 1e-3 of their column's scale):
    # bounded by the column-relative figures above, measured and printed
    r64, r32 = _elemrel(x64, ref), _elemrel(x32, ref)
    print(f"{case}: per-element relative error FP64 {r64:.2e}, mixed {r32:.2e}")
    assert r64 <= 1.001 * FP64_RTOL / ELEM_FRAC and r32 <= 1.001 * MIXED_RTOL / ELEM_FRAC


def test_rows_deterministic():
    from pypolymlp_gb300 import _ffi

    kw, gen = CASES["binary_mt3"]
    p = make_params_dict(**kw)
    ss = gen()
    st = Structures(ss.axis, ss.positions, ss.types)
    e, f, s, n = row_layout(st.n_atoms, [True] * st.n_st)
    m = _model(p)
    a = m.features_x(st, e, f, s, n, precision=_ffi.PG_FP64)
    b = m.features_x(st, e, f, s, n, precision=_ffi.PG_FP64)
    np.testing.assert_array_equal(a, b)


def test_neighbor_list_bit_exact():
    from pypolymlp_gb300 import _ffi

    ss = syn.ternary_set(8, seed=41)
    st = Structures(ss.axis, ss.positions, ss.types)
    for s in range(st.n_st):
        go, gj, gd = _ffi.neighbor_list(st, s, 6.0)
        oo, oj, od = oracle.neighbor_list(st, s, 6.0, half=False)
        np.testing.assert_array_equal(go, oo)
        np.testing.assert_array_equal(gj, oj)
        np.testing.assert_array_equal(gd, od)


def test_empty_and_single_atom_structures():
    """A one-atom cell (self images only) and a structure without force rows."""
    from pypolymlp_gb300 import _ffi

    kw, _ = CASES["binary_mt3"]
    p = make_params_dict(**kw)
    axis = [np.eye(3) * 3.1, np.eye(3) * 8.0]
    pos = [np.zeros((1, 3)), np.array([[0.0, 0.0, 0.0], [1.9, 0.3, 0.2]])]
    types = [np.array([0]), np.array([0, 1])]
    st = Structures(axis, pos, types)
    e, f, s, n = row_layout(st.n_atoms, [True, True])
    ref = oracle.features_x(p, st, e, f, s, n)
    x = _model(p).features_x(st, e, f, s, n, precision=_ffi.PG_FP64)
    assert _colrel(x, ref) < FP64_RTOL


def test_neighbor_list_bit_exact_cell_list():
    """Structures of 1,024+ atoms search a cell list and re-order their
    candidates; the list must still equal the reference's (j, translation)
    order bit for bit: a bcc 8x8x8 cell (1,024 atoms) and a sheared triclinic
    cell of 1,200 atoms."""
    from pypolymlp_gb300 import _ffi

    ss = syn.bcc_supercell(8, a=3.2, sigma=0.1, seed=6)
    rng = np.random.default_rng(8)
    ax = np.array([[21.0, 3.0, -2.0], [0.0, 19.0, 4.0], [0.0, 0.0, 18.0]])
    frac = rng.random((1200, 3))
    axis = [ss.axis[0], ax]
    pos = [ss.positions[0], frac @ ax.T]
    types = [ss.types[0], rng.integers(0, 2, 1200).astype(np.int32)]
    st = Structures(axis, pos, types)
    for s in range(st.n_st):
        go, gj, gd = _ffi.neighbor_list(st, s, 7.0)
        oo, oj, od = oracle.neighbor_list(st, s, 7.0, half=False)
        np.testing.assert_array_equal(go, oo)
        np.testing.assert_array_equal(gj, oj)
        np.testing.assert_array_equal(gd, od)


def test_xrow_work_and_pair_counts():
    """The roofline inputs of the bench: adjoint entries and positions per
    (centre type, neighbour type) of the binary l_max (8, 4) model (4,345
    entries and 957 features with entries for every type pair), and a staged
    batch's pair counts by type pair, which add up to its neighbour lists."""
    from pypolymlp_gb300 import _ffi
    from pypolymlp_gb300.regression import DeviceBatch, GramAccumulator, Dataset, get_min_energy

    p = make_params_dict(n_type=2, cutoff=7.0, model_type=3, max_p=2, gaussian_params2=(0.0, 5.0, 10),
                         gtinv_order=3, gtinv_maxl=(8, 4))
    m = _model(p)
    w = m.xrow_work()
    assert (w["n_entries"] == 4345).all() and (w["n_positions"] == 957).all()
    ss = syn.binary_set(6, seed=3)
    syn.morse_labels(ss, syn.morse_D(2), rc=7.0)
    d = Dataset.from_structure_set(ss)
    b = DeviceBatch(m, d, get_min_energy([d]), _ffi.PG_MIXED)
    assert b.pair_counts(2).sum() == 0  # no lists before an accumulation
    g = GramAccumulator(m, _ffi.PG_MIXED)
    g.accumulate_batch(b)
    pc = b.pair_counts(2)
    st = Structures(ss.axis, ss.positions, ss.types)
    want = np.zeros((2, 2), np.int64)
    for s in range(st.n_st):
        offs, nb, _ = _ffi.neighbor_list(st, s, 7.0)
        t = np.asarray(ss.types[s])
        np.add.at(want, (np.repeat(t, np.diff(offs)), t[nb]), 1)
    np.testing.assert_array_equal(pc, want)
