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
