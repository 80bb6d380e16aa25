"""The CPU oracle against the reference's own outputs.

Golden signatures in tests/golden/ were produced by the reference C++ itself
(compiled from its sources; tests/golden/make_golden.py).  Where that build is
present (oracle/_ref), the oracle is also compared element by element.
"""

import numpy as np
import pytest

from conftest import assert_signature, load_golden
from oracle import oracle, ref
from pypolymlp_gb300.abi import row_layout

X_CASES = ["x_cfg1.npz", "x_cfg2.npz", "x_cfg3.npz", "x_cfg5p.npz", "x_pair_mt2_p3.npz"]


@pytest.mark.parametrize("name", X_CASES)
def test_oracle_x_matches_reference_signature(name):
    params, st, gold = load_golden(name)
    e, f, s, n = row_layout(st.n_atoms, [True] * st.n_st)
    x = oracle.features_x(params, st, e, f, s, n)
    # the oracle restates the reference with the same operation order: ~1e-15
    assert_signature(x, gold, rtol=1e-12)


@pytest.mark.parametrize("name", ["eval_cfg2.npz", "eval_pair.npz"])
def test_oracle_eval_matches_reference(name):
    params, st, gold = load_golden(name)
    e, f, s = oracle.evaluate(params, gold["coeffs"], st)
    np.testing.assert_allclose(e, gold["energy"], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(f, gold["forces"], rtol=0, atol=1e-10 * max(1.0, np.abs(gold["forces"]).max()))
    np.testing.assert_allclose(s, gold["stress"], rtol=0, atol=1e-10 * max(1.0, np.abs(gold["stress"]).max()))


def test_oracle_n_features_pins():
    """Feature counts of the benchmark configs, as the reference reports them."""
    from pypolymlp_gb300.params import make_params_dict

    cases = [
        (dict(n_type=1, cutoff=6.0, model_type=2, max_p=2, gaussian_params2=(0, 5, 8), gtinv_order=2,
              gtinv_maxl=(4,)), 1539),
        (dict(n_type=2, cutoff=7.0, model_type=3, max_p=2, gaussian_params2=(0, 5, 10), gtinv_order=3,
              gtinv_maxl=(8, 4)), 2618),
        (dict(n_type=3, cutoff=6.0, model_type=3, max_p=2, gaussian_params2=(0, 5, 8), gtinv_order=3,
              gtinv_maxl=(6, 4)), 8262),
    ]
    for kw, nf in cases:
        assert oracle.n_features(make_params_dict(**kw)) == nf


needs_ref = pytest.mark.skipif(not ref.available(), reason="reference build (oracle/_ref) not present")


@needs_ref
def test_oracle_neighbors_and_translations_bit_exact():
    from pypolymlp_gb300 import synthetic as syn
    from pypolymlp_gb300.abi import Structures

    ss = syn.ternary_set(12, seed=21)
    st = Structures(ss.axis, ss.positions, ss.types)
    for s in range(st.n_st):
        t1, p1 = ref.translations(st, s, 6.0)
        t2, p2 = oracle.translations(st, s, 6.0)
        np.testing.assert_array_equal(t1, t2)
        np.testing.assert_array_equal(p1, p2)
        for half in (False, True):
            for a, b in zip(ref.neighbor_list(st, s, 6.0, half), oracle.neighbor_list(st, s, 6.0, half)):
                np.testing.assert_array_equal(a, b)


@needs_ref
def test_oracle_x_elementwise_vs_reference():
    from pypolymlp_gb300 import synthetic as syn
    from pypolymlp_gb300.abi import Structures
    from pypolymlp_gb300.params import make_params_dict

    p = make_params_dict(n_type=2, cutoff=5.0, model_type=4, max_p=3, gaussian_params2=(0, 4, 3), gtinv_order=3,
                         gtinv_maxl=(4, 2))
    ss = syn.ternary_set(3, seed=5, n_range=(6, 20), n_types=2)
    st = Structures(ss.axis, ss.positions, ss.types)
    force = [True, False, True]
    e, f, s, n = row_layout(st.n_atoms, force)
    xr = ref.features_x(p, st, e, f, s, n)
    xo = oracle.features_x(p, st, e, f, s, n)
    colmax = np.abs(xr).max(axis=0)
    scale = np.maximum(colmax, 1e-4 * colmax.max())
    assert (np.abs(xr - xo) / scale).max() < 1e-12
