"""The calculator facade (pypolymlp_gb300.api.PypolymlpCalc) on the reference's
facade tests: energies of the legacy Ti-Al potential on five POSCARs
(test_api_properties_legacy_Ti-Al.py), pair MgO on 25 re-shaped cells
(test_check_neighbors.py::test_eval_neighbors_MgO), and the energy rows of X of
two MgO cells from the pair and gtinv model files and from the gtinv polymlp.in
(test_api_features.py).  On the CPU the oracle stands in for the GPU evaluator
and X rows (test infrastructure); the `gpu` tests run the GPU."""

import json
import os

import numpy as np
import pytest

from pypolymlp_gb300 import api
from pypolymlp_gb300.calculator import PolymlpStructure

KA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "known_answers")


def _json(name):
    with open(os.path.join(KA, name)) as f:
        return json.load(f)["cases"]


@pytest.fixture
def on_oracle(monkeypatch):
    from test_calculator import _OracleEvaluator

    from oracle import oracle
    from pypolymlp_gb300 import properties

    monkeypatch.setattr(properties, "PotentialPropertiesFast", _OracleEvaluator)
    monkeypatch.setattr(api, "_features_x", lambda p, st, e, f, s, n, precision: oracle.features_x(p, st, e, f, s, n))


def _tial(calc):
    case = _json("known_energies.json")["TiAl_gtinv_legacy"]
    for cell in case["cells"]:
        calc.load_poscars(os.path.join(KA, cell["structure"]))
        energies, _, _ = calc.eval()
        yield energies[0], cell["energy"], cell["tol"]["rel"]


def _mgo_shapes():
    case = _json("known_energies.json")["MgO_pair_cell_shapes"]
    from pypolymlp_gb300.calculator import load_poscar

    unit = load_poscar(os.path.join(KA, case["cells"][0]["structure"]))
    out = []
    for cell in case["cells"]:
        axis = unit.axis @ np.array(cell["expansion"], dtype=np.float64).T
        frac = np.linalg.solve(axis, unit.axis @ unit.positions)
        out.append(PolymlpStructure(axis, frac, unit.n_atoms, unit.elements, unit.types))
    return os.path.join(KA, case["potential"]), out, case["cells"][0]["energy"]


def _check_x(x, name):
    case = _json("known_x.json")[name]
    assert list(x.shape) == case["shape"]
    assert float(np.sum(x)) == pytest.approx(case["sum"], **case["sum_tol"])
    assert float(np.sum(x[0] - x[1])) == pytest.approx(case["diff01"], **case["diff01_tol"])


POSCARS = ["POSCAR-00001.MgO", "POSCAR-00002.MgO"]


def test_eval_reproduces_reference_energies(on_oracle):
    calc = api.PypolymlpCalc(pot=os.path.join(KA, "polymlp.lammps.gtinv.Ti-Al"))
    for got, want, rel in _tial(calc):
        assert got == pytest.approx(want, rel=rel)
    pot, structures, energy = _mgo_shapes()
    energies, forces, stresses = api.PypolymlpCalc(pot=pot).eval(structures)
    np.testing.assert_allclose(energies, energy, rtol=0, atol=1e-12)
    assert forces[0].shape == (3, 8) and stresses.shape == (25, 6)


@pytest.mark.parametrize("name,pot", [("X_MgO_pair", "polymlp.yaml.pair.MgO"), ("X_MgO_gtinv", "polymlp.yaml.gtinv.MgO")])
def test_features_from_model_files(on_oracle, name, pot):
    calc = api.PypolymlpCalc(pot=os.path.join(KA, pot), require_mlp=True)
    calc.load_structures_from_files(poscars=[os.path.join(KA, p) for p in POSCARS])
    _check_x(calc.run_features(features_force=False, features_stress=False), name)


def test_features_from_input_file(on_oracle):
    calc = api.PypolymlpCalc(require_mlp=False)
    calc.load_structures_from_files(poscars=[os.path.join(KA, p) for p in POSCARS])
    _check_x(calc.run_features(develop_infile=os.path.join(KA, "polymlp.in.gtinv.MgO")), "X_MgO_gtinv")
    x = calc.run_features(develop_infile=os.path.join(KA, "polymlp.in.gtinv.MgO"), features_force=True)
    n = [len(s.types) for s in calc.structures]
    assert x.shape[0] == 2 + 6 * 2 + 3 * sum(n)


def test_parse_polymlp_in_gives_the_model_of_the_file():
    from pypolymlp_gb300.io_polymlp import load_mlp

    p = api.parse_polymlp_in(os.path.join(KA, "polymlp.in.gtinv.MgO"))
    q, _ = load_mlp(os.path.join(KA, "polymlp.yaml.gtinv.MgO"))
    assert p["elements"] == q["elements"] == ["Mg", "O"]
    for k in ("cutoff", "model_type", "max_p", "feature_type", "pair_params"):
        assert p["model"][k] == q["model"][k], k
    for k in ("order", "l_comb", "lm_seq", "lm_coeffs"):
        assert p["model"]["gtinv"][k] == q["model"]["gtinv"][k], k


def test_facade_needs_a_model_unless_told_otherwise():
    with pytest.raises(RuntimeError):
        api.PypolymlpCalc()
    calc = api.PypolymlpCalc(require_mlp=False)
    with pytest.raises(RuntimeError):
        calc.load_structures_from_files()


@pytest.mark.gpu
def test_gpu_facade_reproduces_reference_answers():
    calc = api.PypolymlpCalc(pot=os.path.join(KA, "polymlp.lammps.gtinv.Ti-Al"))
    for got, want, _ in _tial(calc):
        assert got == pytest.approx(want, rel=1e-10)
    calc = api.PypolymlpCalc(pot=os.path.join(KA, "polymlp.yaml.pair.MgO"))
    calc.load_structures_from_files(poscars=[os.path.join(KA, p) for p in POSCARS])
    _check_x(calc.run_features(), "X_MgO_pair")
