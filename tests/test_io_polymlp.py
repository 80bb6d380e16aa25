"""Model files (pypolymlp_gb300.io_polymlp): polymlp.yaml and legacy
polymlp.lammps round trips, the files read by the reference's own C++ parsers
(where the reference build exists), and a loaded model evaluating as the
original (CPU oracle)."""

import numpy as np
import pytest

from oracle import oracle
from oracle import ref as refb
from pypolymlp_gb300 import io_polymlp as io
from pypolymlp_gb300 import synthetic as syn
from pypolymlp_gb300.abi import Structures
from pypolymlp_gb300.params import make_params_dict

MODELS = {
    "gtinv_binary": dict(n_type=2, cutoff=7.0, model_type=3, max_p=2, gaussian_params2=(0.0, 5.0, 10),
                         gtinv_order=3, gtinv_maxl=(8, 4), elements=["Ag", "Au"]),
    "pair_binary": dict(n_type=2, cutoff=5.0, model_type=2, max_p=3, feature_type="pair",
                        gaussian_params2=(0.0, 4.0, 4), elements=["Al", "Cu"]),
}


def _model(name, seed=0):
    p = make_params_dict(**MODELS[name])
    n = oracle.n_features(p)
    rng = np.random.default_rng(seed)
    return p, rng.normal(size=n), rng.uniform(0.5, 2.0, size=n)


def _same_model(a, b):
    ma, mb = a["model"], b["model"]
    assert a["n_type"] == b["n_type"] and list(a["elements"]) == list(b["elements"])
    for k in ("cutoff", "model_type", "max_p", "feature_type"):
        assert ma[k] == mb[k], k
    if ma["feature_type"] == "gtinv":
        assert ma["max_l"] == mb["max_l"]
        for k in ("order", "l_comb", "lm_seq", "lm_coeffs"):
            assert ma["gtinv"][k] == mb["gtinv"][k], k
        assert list(ma["gtinv"]["max_l"])[: ma["gtinv"]["order"] - 1] == list(mb["gtinv"]["max_l"])[
            : mb["gtinv"]["order"] - 1]
    np.testing.assert_array_equal(np.asarray(ma["pair_params"]), np.asarray(mb["pair_params"]))
    ca = {tuple(k) if not isinstance(k, str) else tuple(map(int, k.split(","))): list(v)
          for k, v in ma["pair_params_conditional"].items()}
    cb = {tuple(k): list(v) for k, v in mb["pair_params_conditional"].items()}
    assert ca == cb


@pytest.mark.parametrize("name", sorted(MODELS))
@pytest.mark.parametrize("fmt", ["yaml", "lammps"])
def test_round_trip(tmp_path, name, fmt):
    p, c, s = _model(name)
    path = str(tmp_path / f"polymlp.{fmt}")
    (io.save_mlp_yaml if fmt == "yaml" else io.save_mlp_lammps)(p, c, s, path)
    assert io.is_legacy(path) == (fmt == "lammps")
    q, cq = io.load_mlp(path)
    _same_model(p, q)
    np.testing.assert_allclose(cq, c / s, rtol=1e-15, atol=0)
    assert q["mass"] == [io.ATOMIC_MASS[e] for e in p["elements"]]


@pytest.mark.skipif(not refb.available(), reason="the reference build (oracle/_ref) is not present")
@pytest.mark.parametrize("name", sorted(MODELS))
@pytest.mark.parametrize("fmt", ["yaml", "lammps"])
def test_reference_parsers_read_the_files(tmp_path, name, fmt):
    p, c, s = _model(name, seed=1)
    path = str(tmp_path / f"polymlp.{fmt}")
    (io.save_mlp_yaml if fmt == "yaml" else io.save_mlp_lammps)(p, c, s, path)
    r = refb.parse_potential(path, legacy=fmt == "lammps")
    m = p["model"]
    assert r["elements"] == p["elements"]
    assert r["cutoff"] == m["cutoff"] and r["model_type"] == m["model_type"] and r["max_p"] == m["max_p"]
    assert r["feature_type"] == m["feature_type"] and r["pair_type"] == "gaussian"
    if m["feature_type"] == "gtinv":
        assert r["max_l"] == m["max_l"] and r["n_l_comb"] == len(m["gtinv"]["l_comb"])
    np.testing.assert_array_equal(r["params"], np.asarray(m["pair_params"]))
    assert r["cond"] == {k: list(v) for k, v in m["pair_params_conditional"].items()}
    # the parsers return 2 x the stored coefficient (the reference's energy convention)
    np.testing.assert_allclose(r["coeffs"], 2 * c / s, rtol=1e-15, atol=0)
    np.testing.assert_array_equal(r["mass"], [io.ATOMIC_MASS[e] for e in p["elements"]])


def test_loaded_model_evaluates_as_the_original(tmp_path):
    p, c, s = _model("gtinv_binary", seed=2)
    c = c * 1e-3
    path = str(tmp_path / "polymlp.yaml")
    io.save_mlp_yaml(p, c, s, path)
    q, cq = io.load_mlp(path)
    ss = syn.binary_set(1, seed=9, n_min=8, n_max=12)
    st = Structures(ss.axis, ss.positions, ss.types)
    e0, f0, s0 = oracle.evaluate(p, c / s, st)
    e1, f1, s1 = oracle.evaluate(q, cq, st)
    for a, b in ((e0, e1), (f0, f1), (s0, s1)):
        np.testing.assert_allclose(b, a, rtol=1e-13, atol=1e-13 * max(1.0, float(np.abs(a).max())))


def test_convert_and_find(tmp_path):
    p, c, s = _model("pair_binary")
    leg = str(tmp_path / "polymlp.lammps")
    io.save_mlp_lammps(p, c, s, leg)
    assert io.find_mlps(str(tmp_path)) == [leg]
    out = str(tmp_path / "polymlp.yaml")
    assert io.convert_to_yaml(leg, out)
    assert not io.convert_to_yaml(out, str(tmp_path / "x.yaml"))
    assert io.find_mlps(str(tmp_path)) == [out]
    q, cq = io.load_mlp(out)
    _same_model(p, q)
    np.testing.assert_allclose(cq, c / s, rtol=1e-15)


def test_spin_expansion_follows_revise_params():
    """enable_spins splits an element into two consecutive types and gives every
    pair of their types the element pair's radial ids (data_format.py:192-201, 291-320)."""
    from pypolymlp_gb300.params import expand_spins

    p = make_params_dict(n_type=2, cutoff=5.0, model_type=2, max_p=2, feature_type="pair",
                         gaussian_params2=(0.0, 4.0, 4), elements=["Fe", "Co"])
    p["model"]["pair_params_conditional"] = {(0, 0): [0, 1], (0, 1): [2], (1, 1): [3, 4]}
    q = expand_spins(p, [True, False])
    assert q["n_type"] == 3 and q["elements"] == ["Fe", "Fe", "Co"]
    assert q["enable_spins"] == [True, True, False]
    assert q["spin_elements"] == {"elements": ["Fe", "Co"], "enable_spins": [True, False], "types": [[0, 1], [2]]}
    assert q["model"]["pair_params_conditional"] == {(0, 0): [0, 1], (0, 1): [0, 1], (1, 1): [0, 1],
                                                     (0, 2): [2], (1, 2): [2], (2, 2): [3, 4]}
    r = make_params_dict(n_type=2, cutoff=5.0, model_type=2, max_p=2, feature_type="pair",
                         gaussian_params2=(0.0, 4.0, 4), elements=["Fe", "Co"], enable_spins=[False, False])
    assert r["n_type"] == 2 and r["enable_spins"] is None and "spin_elements" not in r


def test_spin_model_round_trip(tmp_path):
    """A spin model is written element-level (elements, enable_spins, element-pair
    radial ids, one mass per atom type) as io_polymlp_yaml.py:17-94 writes it, and
    reads back as the same expanded model; the legacy format refuses it."""
    p = make_params_dict(n_type=2, cutoff=5.0, model_type=2, max_p=2, feature_type="pair",
                         gaussian_params2=(0.0, 4.0, 4), elements=["Fe", "Co"], enable_spins=[True, False])
    n = oracle.n_features(p)
    rng = np.random.default_rng(4)
    c, s = rng.normal(size=n), rng.uniform(0.5, 2.0, size=n)
    path = str(tmp_path / "polymlp.yaml")
    io.save_mlp_yaml(p, c, s, path)
    text = open(path).read()
    assert "elements:      [Fe, Co]" in text and "enable_spins:  [1, 0]" in text
    assert f"mass:          [{io.ATOMIC_MASS['Fe']!r}, {io.ATOMIC_MASS['Fe']!r}, {io.ATOMIC_MASS['Co']!r}]" in text
    assert "n_type_pairs: 3" in text and "type_indices: [0, 1]" in text
    q, cq = io.load_mlp(path)
    _same_model(p, q)
    assert q["spin_elements"] == p["spin_elements"] and q["enable_spins"] == [True, True, False]
    np.testing.assert_allclose(cq, c / s, rtol=1e-15, atol=0)
    with pytest.raises(ValueError):
        io.save_mlp_lammps(p, c, s, str(tmp_path / "polymlp.lammps"))
