"""Invariant tables (gtinv.Readgtinv) and feature attributes
(features_attr.FeaturesAttr), on the CPU.

Readgtinv must return exactly what the reference's Readgtinv returns: the JSON
tables in tests/golden/gtinv were written from the reference build
(tests/golden/make_golden.py, make_known_answers.py), and where that build is
present (oracle/_ref) random (order, l_max, version) requests are compared
with it directly.  FeaturesAttr, computed by the library's host code from the
tables the kernels use, must list the same radial ids, invariant ids, type
combinations, polynomial columns and type pairs as the reference's
FeaturesAttr, for pair and gtinv models of orders 2-6 and model types 1-4."""

import glob
import json
import os
import random

import pytest

from pypolymlp_gb300.gtinv import Readgtinv, get_gtinv_attrs
from pypolymlp_gb300.params import make_params_dict

GTINV = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "gtinv")


def _ref():
    from oracle import ref

    if not ref.available():
        pytest.skip("the reference build (oracle/_ref) is not present")
    return ref


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GTINV, "*.json"))), ids=os.path.basename)
def test_readgtinv_reproduces_reference_tables(path):
    with open(path) as f:
        d = json.load(f)
    got = get_gtinv_attrs(d["order"], d["maxl"], d["version"])
    assert got == (d["l_comb"], d["lm_seq"], d["lm_coeffs"])


def test_readgtinv_matches_reference_build():
    ref = _ref()
    rng = random.Random(7)
    for version, top in ((1, 6), (2, 2)):
        for order in range(0, top + 1):
            for _ in range(6):
                maxl = [rng.randint(0, 22) for _ in range(max(order - 1, 0))]
                assert get_gtinv_attrs(order, maxl, version) == tuple(ref.readgtinv(order, maxl, version)), \
                    (version, order, maxl)


def test_readgtinv_screens_by_largest_l():
    """Each order keeps exactly the invariants whose largest l is within its l_max,
    lm indices are l*l + l + m with |m| <= l, and every m combination has a coefficient."""
    r = Readgtinv(4, [6, 4, 2])
    limits = {1: 0, 2: 6, 3: 4, 4: 2}
    for lc, seq, co in zip(r.get_l_comb(), r.get_lm_seq(), r.get_lm_coeffs()):
        assert lc == sorted(lc) and lc[-1] <= limits[len(lc)]
        assert len(seq) == len(co) > 0
        for lm in seq:
            assert [int((v) ** 0.5) for v in lm] == lc
    orders = [len(lc) for lc in r.get_l_comb()]
    assert orders == sorted(orders) and set(orders) == {1, 2, 3, 4}


def test_readgtinv_errors():
    with pytest.raises(ValueError):
        Readgtinv(7, [4] * 6)
    with pytest.raises(ValueError):
        Readgtinv(2, [4], version=3)
    with pytest.raises(RuntimeError):
        Readgtinv(3, [4, 4], version=2)
    with pytest.raises(ValueError):
        Readgtinv(3, [4])
    assert get_gtinv_attrs(0, []) == ([], [], [])


ATTR_CASES = {
    "pair_binary_mt1_p3": dict(n_type=2, feature_type="pair", model_type=1, max_p=3),
    "pair_ternary_mt2": dict(n_type=3, feature_type="pair", model_type=2, max_p=2),
    "gtinv_quaternary_o3_mt3": dict(n_type=4, model_type=3, max_p=2, gtinv_order=3, gtinv_maxl=(4, 4)),
    "gtinv_binary_o2_l20": dict(n_type=2, model_type=2, max_p=2, gtinv_order=2, gtinv_maxl=(20,)),
    "gtinv_ternary_o6_mt1": dict(n_type=3, model_type=1, max_p=1, gtinv_order=6, gtinv_maxl=(4, 4, 2, 1, 1)),
    "gtinv_ternary_o4_mt4": dict(n_type=3, model_type=4, max_p=2, gtinv_order=4, gtinv_maxl=(4, 4, 2)),
    "gtinv_unary_o4_mt4_p3": dict(n_type=1, model_type=4, max_p=3, gtinv_order=4, gtinv_maxl=(12, 6, 3)),
}
# (linear features, polynomial columns) the reference build's FeaturesAttr lists
ATTR_COUNTS = {
    "pair_binary_mt1_p3": (15, 0), "pair_ternary_mt2": (30, 315), "gtinv_quaternary_o3_mt3": (11440, 750),
    "gtinv_binary_o2_l20": (540, 99845), "gtinv_ternary_o6_mt1": (21270, 0), "gtinv_ternary_o4_mt4": (8685, 39690),
    "gtinv_unary_o4_mt4_p3": (385, 62125),
}


def _attr_params(name):
    return make_params_dict(cutoff=6.0, gaussian_params2=(0.0, 5.0, 4), **ATTR_CASES[name])


@pytest.mark.parametrize("name", sorted(ATTR_CASES))
def test_features_attr_counts(name):
    from pypolymlp_gb300.features_attr import get_features_attr, get_num_features

    lin, poly, tp_dict = get_features_attr(_attr_params(name))
    assert (len(lin), len(poly)) == ATTR_COUNTS[name]
    assert get_num_features(_attr_params(name)) == sum(ATTR_COUNTS[name])
    n = ATTR_CASES[name]["n_type"]
    assert sorted(tuple(v) for vs in tp_dict.values() for v in vs) == [(a, b) for a in range(n) for b in range(n)]


@pytest.mark.parametrize("name", sorted(ATTR_CASES))
def test_features_attr_matches_reference_build(name):
    from pypolymlp_gb300.features_attr import FeaturesAttr

    ref = _ref()
    p = _attr_params(name)
    a = FeaturesAttr(p)
    rad, gt, tc, poly = ref.feature_attrs(p)
    assert a.get_radial_ids() == rad
    assert a.get_gtinv_ids() == (gt if p["model"]["feature_type"] == "gtinv" else [])
    assert a.get_tcomb_ids() == [[int(v) for v in x] for x in tc]
    assert a.get_polynomial_ids() == [[int(v) for v in x] for x in poly]
    assert a.get_type_pairs() == ref.type_pairs(p)
    assert len(rad) + len(poly) == ref.n_features(p)


def test_features_attr_rejects_pair_model_type_3():
    """The reference exits (polymlp_model_params_polynomial.cpp:42-44); the library returns an error."""
    from pypolymlp_gb300 import _ffi
    from pypolymlp_gb300.features_attr import FeaturesAttr

    p = make_params_dict(n_type=2, cutoff=6.0, feature_type="pair", model_type=3, max_p=2)
    with pytest.raises(_ffi.GB300Error):
        FeaturesAttr(p)


def test_num_features_of_a_hybrid_sums_the_models():
    from pypolymlp_gb300.features_attr import get_num_features

    a, b = _attr_params("pair_binary_mt1_p3"), _attr_params("pair_ternary_mt2")
    assert get_num_features([a, b]) == get_num_features(a) + get_num_features(b)


@pytest.mark.parametrize("name", ["pair_binary_mt1_p3", "pair_ternary_mt2", "gtinv_quaternary_o3_mt3"])
def test_polymlp_params_yaml_lists_every_column(tmp_path, name, monkeypatch):
    """polymlp_params.yaml (features_attr.py:51-117 layout): one entry per column,
    ids consecutive, linear entries carrying FeaturesAttr's radial/gtinv/type-pair ids."""
    import ast

    from pypolymlp_gb300.features_attr import get_features_attr, write_polymlp_params_yaml

    p = _attr_params(name)
    out = str(tmp_path / "polymlp_params.yaml")
    n = write_polymlp_params_yaml(p, out)
    lin, poly, tp_dict = get_features_attr(p)
    assert n == len(lin) + len(poly)
    ids, radial, tps, feats = [], [], [], []
    for line in open(out).read().splitlines():
        key, _, val = line.strip().lstrip("- ").partition(":")
        if key == "id":
            ids.append(int(val))
        elif key == "radial_id" and line.startswith("  "):
            radial.append(int(val))
        elif key == "atomtype_pair_ids":
            tps.append(ast.literal_eval(val.strip()))
        elif key == "feature_ids":
            feats.append(ast.literal_eval(val.strip()))
    assert ids == list(range(n))
    assert radial == [a[0] for a in lin] and tps == [list(a[-1]) for a in lin] and feats == poly
    text = open(out).read()
    assert text.count("- pair_id:") == len(tp_dict) and text.count("- radial_id:") == len(p["model"]["pair_params"])
    # a hybrid writes one numbered file per model into the working directory
    monkeypatch.chdir(tmp_path)
    assert write_polymlp_params_yaml([p, p]) == 2 * n
    assert (tmp_path / "polymlp_params1.yaml").exists() and (tmp_path / "polymlp_params2.yaml").exists()


def _gtinv_known():
    with open(os.path.join(os.path.dirname(GTINV), "known_answers", "known_gtinv.json")) as f:
        return json.load(f)["cases"]


@pytest.mark.parametrize("name", sorted(_gtinv_known()))
def test_readgtinv_reproduces_reference_known_answers(name):
    """tests/test_cxx/test_gtinv.py: table sizes, l combinations, lm sequences and
    coefficients at given indices.  Its third case asks for a version-2 table of
    order 6, which the reference does not ship (its v2 tables stop at order 2): the
    reference's reader throws there, and so does this one."""
    case = _gtinv_known()[name]
    if case["version"] == 2 and case["order"] > 2:
        with pytest.raises(RuntimeError):
            get_gtinv_attrs(case["order"], case["lmax"], case["version"])
        return
    got = dict(zip(("l_combs", "lm_seq", "lm_coeffs"), get_gtinv_attrs(case["order"], case["lmax"], case["version"])))
    for c in case["checks"]:
        v = got[c["name"]]
        for k in c["idx"]:
            v = v[k]
        if c["kind"] == "len":
            v = len(v)
        elif c["kind"] == "tuple":
            v = list(v)
        assert v == (pytest.approx(c["expect"]) if c["approx"] else c["expect"]), (c, v)
