"""Known answers of the reference's PolymlpAPI unit tests
(tests/test_cxx/test_polymlp_api.py, test_polymlp_api_pair.py; asserted shapes
and sums and the potential files they load copied by
tests/golden/make_known_answers.py): per atom type, the conjugate completion of
a_nlm, the feature values and their derivatives from given a_nlm, and the
potential's adjoint sums, for a gtinv and a pair MgO model.  The oracle's
per-type steps (oracle.PolymlpAPI over the host model tables the GPU kernels
are built from) must reproduce them; the inputs are the tests' own (aranges,
constant derivative arrays with three entries changed)."""

import json
import os

import numpy as np
import pytest

from pypolymlp_gb300 import io_polymlp

KA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "known_answers")


def _cases():
    with open(os.path.join(KA, "known_api.json")) as f:
        return json.load(f)["cases"]


def _values(name):
    """The variables the reference test computes, by the same names."""
    from oracle.oracle import PolymlpAPI

    case = _cases()[name]
    p, c = io_polymlp.load_mlp(os.path.join(KA, case["potential"]))
    api = PolymlpAPI(p, 2.0 * c)  # the reference's parser returns twice the stored coefficients
    n = len(c)
    v = {}
    if p["model"]["feature_type"] == "pair":
        antp = np.arange(n, dtype=np.float64)
        v["dn0"], v["dn1"] = api.compute_features(antp, 0), api.compute_features(antp, 1)
        v["prod_e"], v["prod_f"] = api.compute_sum_of_prod(antp, 0)
        return case, v
    r = np.arange(n, dtype=np.float64)
    v["anlmtp0"] = api.compute_anlmtp_conjugate(r, r, 0)
    v["anlmtp1"] = api.compute_anlmtp_conjugate(r, r, 1)
    v["dn0"], v["dn1"] = api.compute_features(v["anlmtp0"], 0), api.compute_features(v["anlmtp1"], 1)
    k = len(v["anlmtp0"])
    dfx = np.ones((k, 8))
    dfy = -np.ones((k, 8)) * 2
    dfy[200, 3] = 0.02
    dfz = np.ones((k, 8)) * 0.5
    dfz[100, 3] = -0.05
    ds = -np.ones((k, 6))
    ds[300, 3] = 0.03
    v["dfx"], v["dfy"], v["dfz"], v["ds"] = api.compute_features_deriv(v["anlmtp0"], dfx, dfy, dfz, ds, 0)
    v["prod_e"], v["prod_f"] = api.compute_sum_of_prod(v["anlmtp0"], 0)
    return case, v


@pytest.mark.parametrize("name", sorted(_cases()))
def test_oracle_reproduces_polymlp_api_known_answers(name):
    case, v = _values(name)
    for var, kind, want in case["checks"]:
        if kind == "shape":
            assert list(np.shape(v[var])) == want, var
        else:
            got = complex(np.sum(v[var]))
            assert got == pytest.approx(complex(*want)), (var, got, want)


@pytest.mark.parametrize("type1", [0, 1])
def test_oracle_adjoint_sums_match_reference_build(type1):
    """On a_nlm with real m = 0 entries (as physical ones are), per head."""
    import ctypes as C

    from oracle import ref
    from oracle.oracle import PolymlpAPI, _check, _load, _p

    if not ref.available():
        pytest.skip("the reference build (oracle/_ref) is not present")
    path = os.path.join(KA, "api.polymlp.yaml.MgO")
    p, c = io_polymlp.load_mlp(path)
    api = PolymlpAPI(p, 2.0 * c)
    k0 = api.sizes(type1)[1]
    m = np.zeros(k0, np.int32)
    _check(_load().or_api_noconj_m(api._fp.ref(), type1, _p(m, C.c_int)))
    rng = np.random.default_rng(5 + type1)
    re, im = rng.normal(size=k0), rng.normal(size=k0)
    im[m == 0] = 0.0
    a = api.compute_anlmtp_conjugate(re, im, type1)
    pe, pf = api.compute_sum_of_prod(a, type1)
    re_e, re_f = ref.api_sum_of_prod(path, ["Mg", "O"], type1, a)
    np.testing.assert_allclose(pe, re_e, rtol=1e-12, atol=1e-12 * np.abs(re_e).max())
    np.testing.assert_allclose(pf, re_f, rtol=1e-12, atol=1e-12 * np.abs(re_f).max())
