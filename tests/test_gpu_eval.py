"""GPU energies, forces and stresses (pg_eval_* through the C ABI) against the
reference's golden values and the oracle.

Tolerances: FP64 path 1e-10 relative to the largest magnitude of each
quantity; mixed path (FP32 features and adjoint, FP64 neighbour sums and
reductions) 1e-4 relative to the largest magnitude.
"""

import numpy as np
import pytest

from conftest import load_golden
from oracle import oracle
from pypolymlp_gb300 import synthetic as syn
from pypolymlp_gb300.abi import Structures
from pypolymlp_gb300.params import make_params_dict

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-10
MIXED_RTOL = 1e-4


def _rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300))


def _coeffs(p, seed):
    n = oracle.n_features(p)
    return np.random.default_rng(seed).normal(size=n) * 1e-3


@pytest.mark.parametrize("name", ["eval_cfg2.npz", "eval_pair.npz"])
def test_fp64_eval_matches_reference(name):
    from pypolymlp_gb300 import _ffi

    params, st, gold = load_golden(name)
    e, f, s = _ffi.Evaluator(params, gold["coeffs"], _ffi.PG_FP64).run(st)
    assert _rel(e, gold["energy"]) < FP64_RTOL
    assert _rel(f, gold["forces"]) < FP64_RTOL
    assert _rel(s, gold["stress"]) < FP64_RTOL


EVAL_CASES = {
    "binary_mt3": (dict(n_type=2, cutoff=7.0, model_type=3, max_p=2, gaussian_params2=(0, 5, 10), gtinv_order=3,
                        gtinv_maxl=(8, 4)), lambda: syn.binary_set(3, seed=51)),
    "ternary_mt4_p2": (dict(n_type=3, cutoff=5.0, model_type=4, max_p=2, gaussian_params2=(0, 4, 3), gtinv_order=3,
                            gtinv_maxl=(4, 2)), lambda: syn.ternary_set(3, seed=52, n_range=(8, 70))),
    "binary_mt2_p3": (dict(n_type=2, cutoff=5.0, model_type=2, max_p=3, gaussian_params2=(0, 4, 2), gtinv_order=2,
                           gtinv_maxl=(2,)), lambda: syn.binary_set(2, seed=55, n_min=16, n_max=40)),
    "unary_order4": (dict(n_type=1, cutoff=6.0, model_type=2, max_p=2, gaussian_params2=(0, 5, 5), gtinv_order=4,
                          gtinv_maxl=(8, 8, 2)), lambda: syn.fcc_set(2, seed=53)),
    "pair_mt2_p3": (dict(n_type=2, cutoff=6.0, model_type=2, max_p=3, feature_type="pair",
                         gaussian_params2=(0, 5, 6)), lambda: syn.binary_set(2, seed=54, n_min=16, n_max=40)),
}


@pytest.mark.parametrize("case", sorted(EVAL_CASES))
def test_eval_matches_oracle(case):
    from pypolymlp_gb300 import _ffi

    kw, gen = EVAL_CASES[case]
    p = make_params_dict(**kw)
    ss = gen()
    st = Structures(ss.axis, ss.positions, ss.types)
    c = _coeffs(p, 7)
    ref = oracle.evaluate(p, c, st)
    got = _ffi.Evaluator(p, c, _ffi.PG_FP64).run(st)
    for g, r in zip(got, ref):
        assert _rel(g, r) < FP64_RTOL
    got32 = _ffi.Evaluator(p, c, _ffi.PG_MIXED).run(st)
    for g, r in zip(got32, ref):
        assert _rel(g, r) < MIXED_RTOL


def test_forces_are_energy_gradient_and_sum_to_zero():
    """Central differences of the energy (h = 1e-5 angstrom) give the forces;
    the forces of a periodic cell sum to zero."""
    from pypolymlp_gb300 import _ffi

    kw, _ = EVAL_CASES["binary_mt3"]
    p = make_params_dict(**kw)
    ss = syn.binary_set(1, seed=56, n_min=8, n_max=12)
    c = _coeffs(p, 8)
    ev = _ffi.Evaluator(p, c, _ffi.PG_FP64)
    pos = np.asarray(ss.positions[0], dtype=np.float64)
    e0, f0, s0 = ev.run(Structures(ss.axis, [pos], ss.types))
    assert np.abs(f0.sum(axis=0)).max() < 1e-9 * max(1.0, np.abs(f0).max())
    h = 1e-5
    for atom, comp in [(0, 0), (1, 2), (len(pos) - 1, 1)]:
        pp, pm = pos.copy(), pos.copy()
        pp[atom, comp] += h
        pm[atom, comp] -= h
        ep = ev.run(Structures(ss.axis, [pp], ss.types))[0][0]
        em = ev.run(Structures(ss.axis, [pm], ss.types))[0][0]
        fd = -(ep - em) / (2 * h)
        assert abs(fd - f0[atom, comp]) < 1e-6 * max(1.0, np.abs(f0).max())


def test_eval_deterministic_and_edge_structures():
    """Two runs agree bit for bit; a one-atom cell and a dimer in a large box."""
    from pypolymlp_gb300 import _ffi

    kw, _ = EVAL_CASES["binary_mt3"]
    p = make_params_dict(**kw)
    axis = [np.eye(3) * 3.1, np.eye(3) * 8.0, np.eye(3) * 20.0]
    pos = [np.zeros((1, 3)), np.array([[0.0, 0.0, 0.0], [1.9, 0.3, 0.2]]), np.array([[0.0, 0.0, 0.0]])]
    types = [np.array([0]), np.array([0, 1]), np.array([1])]
    st = Structures(axis, pos, types)
    c = _coeffs(p, 9)
    ref = oracle.evaluate(p, c, st)
    ev = _ffi.Evaluator(p, c, _ffi.PG_FP64)
    a = ev.run(st)
    b = ev.run(st)
    for x, y, r in zip(a, b, ref):
        np.testing.assert_array_equal(x, y)
        assert _rel(x, r) < FP64_RTOL or np.abs(x - r).max() < 1e-12


def test_properties_api_matches_oracle():
    """PotentialPropertiesFast / PropertiesSingle shapes and values."""
    from pypolymlp_gb300.properties import PotentialPropertiesFast, PropertiesSingle

    kw, gen = EVAL_CASES["ternary_mt4_p2"]
    p = make_params_dict(**kw)
    ss = gen()
    st = Structures(ss.axis, ss.positions, ss.types)
    c = _coeffs(p, 10)
    e_ref, f_ref, s_ref = oracle.evaluate(p, c, st)
    prop = PotentialPropertiesFast(p, c)
    prop.eval(ss.axis[0], np.asarray(ss.positions[0]).T, ss.types[0])
    n0 = len(ss.types[0])
    assert abs(prop.get_e() - e_ref[0]) <= FP64_RTOL * abs(e_ref).max()
    assert prop.get_f().shape == (n0, 3)
    assert np.abs(prop.get_f() - f_ref[:n0]).max() < FP64_RTOL * np.abs(f_ref).max()

    class S:
        def __init__(self, axis, pos_c, types):
            self.axis = np.asarray(axis)
            self.positions = np.linalg.solve(self.axis, np.asarray(pos_c).T)
            self.types = types

    structs = [S(a, x, t) for a, x, t in zip(ss.axis, ss.positions, ss.types)]
    energies, forces, stresses = PropertiesSingle(p, c).eval_multiple(structs)
    assert energies.shape == (st.n_st,) and stresses.shape == (st.n_st, 6)
    assert forces[0].shape == (3, n0)
    # fractional round trip changes positions at the 1e-15 level
    assert _rel(energies, e_ref) < 1e-8


def test_eval_large_cell_matches_oracle():
    """A 1,024-atom bcc cell (cell-list neighbour search) against the oracle."""
    from pypolymlp_gb300 import _ffi

    kw, _ = EVAL_CASES["binary_mt3"]
    p = make_params_dict(**kw)
    ss = syn.bcc_supercell(8, a=3.2, sigma=0.1, seed=7)
    st = Structures(ss.axis, ss.positions, ss.types)
    c = _coeffs(p, 11)
    ref = oracle.evaluate(p, c, st)
    got = _ffi.Evaluator(p, c, _ffi.PG_FP64).run(st)
    for g, r in zip(got, ref):
        assert _rel(g, r) < FP64_RTOL
