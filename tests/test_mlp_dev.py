"""The model-development front end (pypolymlp_gb300.mlp_dev.Pypolymlp).

The reference's pair MgO fit (test_mlp_devel_vasp.py::test_mlp_devel_pair; its
vasprun data in tests/golden/known_answers/fit_MgO.npz) is passed in as the
reference's users pass structures: PolymlpStructure objects with element names
(atoms shuffled against the element order), fractional positions, energies
with atomic energies added back, forces (3, n_atom) and 3x3 stress tensors.
On the CPU the GPU regression and evaluator are replaced by the oracle
pipeline (test infrastructure), so the front end's parameter and dataset
handling is checked against the reference's asserted train/test errors; the
`gpu` test runs the same through the GPU."""

import numpy as np
import pytest

from pypolymlp_gb300 import _ffi
from pypolymlp_gb300.calculator import PolymlpStructure
from pypolymlp_gb300.mlp_dev import Pypolymlp

ATOMIC_E = (-0.6, -1.7)


def _structures(z, tag, rng):
    n = z[f"{tag}_n_atoms"]
    offs = np.concatenate([[0], np.cumsum(n)])
    names = np.array(["Mg", "O"])
    sts, energies, forces, stresses = [], [], [], []
    for i in range(len(n)):
        sl = slice(offs[i], offs[i + 1])
        axis = z[f"{tag}_axis"][i]
        perm = rng.permutation(n[i])
        pos = z[f"{tag}_positions"][sl][perm]
        types = z[f"{tag}_types"][sl][perm]
        frac = np.linalg.solve(axis, pos.T)
        sts.append(PolymlpStructure(axis, frac, [int(np.sum(types == t)) for t in (0, 1)], list(names[types]),
                                    [5] * len(types)))
        energies.append(z[f"{tag}_energies"][i] + sum(ATOMIC_E[t] for t in types))
        forces.append(z[f"{tag}_forces"][sl][perm].T)
        xx, yy, zz, xy, yz, zx = z[f"{tag}_stresses"][i]
        stresses.append([[xx, xy, zx], [xy, yy, yz], [zx, yz, zz]])
    return sts, np.array(energies), forces, np.array(stresses)


def _front_end(precision=_ffi.PG_FP64):
    from test_known_fit import KA, _cases

    case = _cases()["pair_single"]
    st = case["settings"]
    z = np.load(f"{KA}/{case['data']}")
    rng = np.random.default_rng(3)
    tr = _structures(z, "train1", rng)
    te = _structures(z, "test1", rng)
    pm = Pypolymlp(precision=precision)
    pm.set_params(elements=st["elements"], cutoff=st["cutoff"], model_type=st["model_type"], max_p=st["max_p"],
                  feature_type=st["feature_type"], gaussian_params1=tuple(st["gaussian_params1"]),
                  gaussian_params2=tuple(st["gaussian_params2"]), reg_alpha_params=(-3, 1, 5),
                  atomic_energy=ATOMIC_E)
    pm.set_datasets_structures(tr[0], te[0], tr[1], te[1], tr[2], te[2], tr[3], te[3])
    return pm, case


@pytest.fixture
def on_oracle(monkeypatch):
    """The GPU fit and evaluator replaced by the oracle pipeline."""
    from test_calculator import _OracleEvaluator
    from test_known_fit import cpu_fit

    from pypolymlp_gb300 import properties, regression

    class _Result:
        def __init__(self, c, s):
            self.coeffs, self.scales = c, s

    def fake_fit(params, train, test, alphas, **kw):
        return _Result(*cpu_fit(params, train, test, alphas))

    monkeypatch.setattr(properties, "PotentialPropertiesFast", _OracleEvaluator)
    monkeypatch.setattr(regression, "fit", fake_fit)


def _check(pm, case):
    from test_known_fit import _check as check_errors

    train, test = pm.errors
    got = {"train1": train["data1"], "test1": test["data2"]}
    check_errors(got, case["errors"])


def test_front_end_datasets_match_the_reference_dataset(tmp_path):
    from test_known_fit import _datasets

    pm, case = _front_end()
    assert pm.n_features == case["settings"]["n_features"]
    ref_train, _ = _datasets(case)
    d, r = pm.train[0], ref_train[0]
    assert len(d) == len(r) and d.include_force and d.include_stress
    np.testing.assert_allclose(d.energies, r.energies, rtol=0, atol=1e-12)
    np.testing.assert_allclose(d.stresses, r.stresses, rtol=0, atol=0)
    for a, b in zip(d.types, r.types):
        assert sorted(a.tolist()) == sorted(b.tolist())
    # the reference's row order does not matter: per structure, the same atoms
    for a, b, fa, fb in zip(d.positions, r.positions, d.forces, r.forces):
        ka, kb = np.lexsort(np.round(a, 9).T), np.lexsort(np.round(b, 9).T)
        np.testing.assert_allclose(a[ka], b[kb], atol=1e-12)
        np.testing.assert_array_equal(fa[ka], fb[kb])


def test_front_end_reproduces_reference_fit_errors(on_oracle, tmp_path):
    pm, case = _front_end()
    pm.run()
    _check(pm, case)
    pm.save_mlp(str(tmp_path / "polymlp.yaml"))
    pm.save_errors(str(tmp_path / "polymlp_error.yaml"))
    pm.save_params(str(tmp_path / "polymlp_params.yaml"))
    text = open(tmp_path / "polymlp_error.yaml").read()
    assert text.count("- dataset:") == 2 and "rmse_stress:" in text
    back = Pypolymlp().load_mlp(str(tmp_path / "polymlp.yaml"))
    np.testing.assert_allclose(back.coeffs, pm.coeffs, rtol=1e-15)
    assert back.n_features == case["settings"]["n_features"]


def test_missing_forces_turn_off_force_and_stress_fitting():
    pm = Pypolymlp().set_params(elements=["Mg", "O"], feature_type="pair", model_type=2, max_p=2)
    st = PolymlpStructure(np.eye(3) * 4.0, np.array([[0.0, 0.5], [0.0, 0.5], [0.0, 0.5]]), [1, 1], ["Mg", "O"],
                          [0, 1])
    pm.set_datasets_structures([st], [st], [-1.0], [-1.0])
    assert not pm.train[0].include_force and not pm.train[0].include_stress and pm.train[0].forces is None
    pm = Pypolymlp().set_params(elements=["Mg", "O"], feature_type="pair", model_type=2, max_p=2,
                                atomic_energy=(-1.0, -0.5), atomic_energy_unit="Hartree")
    pm.set_datasets_structures([st], [st], [-1.0], [-1.0], [np.zeros((3, 2))], [np.zeros((3, 2))])
    assert pm.train[0].include_force and not pm.train[0].include_stress
    assert pm.train[0].energies[0] == pytest.approx(-1.0 + 1.5 * 27.211386245981)


@pytest.mark.gpu
def test_gpu_front_end_reproduces_reference_fit_errors():
    pm, case = _front_end()
    pm.run()
    _check(pm, case)


def _param_cases():
    import json
    import os

    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "known_answers", "known_params.json")
    with open(path) as f:
        return json.load(f)["cases"]


def test_gaussians_from_n_gaussians_match_reference():
    from pypolymlp_gb300.params import gaussian_params

    for c in _param_cases()["n_gaussians"]:
        got = gaussian_params(n_gaussians=c["n_gaussians"], cutoff=c["cutoff"])
        np.testing.assert_array_equal(np.array(got), np.array(c["pair_params"]))
    with pytest.raises(ValueError):
        gaussian_params(n_gaussians=2, cutoff=6.0)


def test_distance_conditioned_radial_functions_match_reference():
    from pypolymlp_gb300.params import active_gaussian_params, make_params_dict

    for c in _param_cases()["distance"]:
        dist = {tuple(k): v for k, v in c["distance"]}
        cond, flag = active_gaussian_params(c["pair_params"], c["elements"], dist)
        assert flag == c["conditional"]
        assert cond == {tuple(k): v for k, v in c["cond"]}
    c = _param_cases()["distance"][1]
    p = make_params_dict(n_type=2, cutoff=7.0, model_type=2, max_p=2, feature_type="pair", n_gaussians=8,
                         elements=c["elements"], distance={tuple(k): v for k, v in c["distance"]})
    assert p["model"]["pair_conditional"] and p["model"]["pair_params"] == c["pair_params"]
    assert p["model"]["pair_params_conditional"] == {tuple(k): v for k, v in c["cond"]}


@pytest.mark.parametrize("name", ["pair_single", "gtinv_single", "gtinv_multi"])
def test_load_parameter_file_reads_the_reference_input(name, tmp_path):
    """The reference's input files of the known fits (data locations absent here):
    the model (feature count), alphas, stress flag, and one dataset per data line
    named by its glob."""
    from test_known_fit import KA, _cases

    from pypolymlp_gb300.features_attr import get_num_features

    files = {"pair_single": "polymlp.in.vasp.pair.single.MgO", "gtinv_single": "polymlp.in.vasp.single.MgO",
             "gtinv_multi": "polymlp.in.vasp.multi.MgO"}
    st = _cases()[name]["settings"]
    pm = Pypolymlp().load_parameter_file(f"{KA}/{files[name]}", prefix=str(tmp_path))
    assert get_num_features(pm.parameters) == st["n_features"]
    np.testing.assert_allclose(pm._alphas, st["alphas"], rtol=1e-15)
    assert pm.parameters["include_stress"] == st["include_stress"]
    n_sets = 2 if name == "gtinv_multi" else 1
    assert len(pm.train) == len(pm.test) == n_sets
    assert all(d.name.startswith("data-vasp-MgO/vaspruns/") and len(d) == 0 for d in pm.train + pm.test)


def test_load_parameter_file_dataset_lines(tmp_path):
    """train_data / test_data / data lines: glob, include_force flag, weight."""
    from test_known_fit import KA

    text = "\n".join(["n_type 2", "elements Mg O", "feature_type pair", "cutoff 6.0", "model_type 2", "max_p 2",
                      "atomic_energy -0.5 -1.5", "distance Mg O 2.1", "",
                      "train_data vasprun-0000*-MgO.xml True 2.0",
                      "test_data vasprun-t*.xml.polymlp False",
                      "data vasprun-*.xml* True 0.5"])
    path = tmp_path / "polymlp.in"
    path.write_text(text + "\n")
    pm = Pypolymlp().load_parameter_file(str(path), train_ratio=0.75, prefix=KA)
    assert [len(d) for d in pm.train] == [2, 3] and [len(d) for d in pm.test] == [2, 1]
    a, b = pm.train[0], pm.test[0]
    assert a.include_force and a.include_stress and a.weight == 2.0 and a.name == "vasprun-0000*-MgO.xml"
    assert not b.include_force and not b.include_stress and b.weight == 1.0
    assert pm.train[1].weight == 0.5 and pm.parameters["model"]["pair_conditional"]


def test_hybrid_front_end_fits_saves_and_reloads(monkeypatch, tmp_path):
    """Two pair models over Mg and O fitted together (append_hybrid_params): the GPU
    X rows, Gram, posv and evaluator replaced by the oracle, numpy and LAPACK
    (checker only).  The saved polymlp.yaml.1 / .2, evaluated together, give the
    errors the fit reported."""
    from test_hybrid import _oracle_hybrid_x

    from oracle import oracle
    from oracle.pipeline import solver_ridge_cpu
    from pypolymlp_gb300 import hybrid, regression
    from pypolymlp_gb300.abi import Structures  # noqa: F401

    class _OracleRun:
        def __init__(self, p, c, precision=None):
            self._p, self._c = p, np.asarray(c, dtype=np.float64)

        def run(self, st):
            return oracle.evaluate(self._p, self._c, st)

    monkeypatch.setattr(hybrid, "hybrid_features_x", _oracle_hybrid_x)
    monkeypatch.setattr(_ffi, "gram_xtx", lambda x, precision=None: x.T @ x)
    monkeypatch.setattr(_ffi, "Evaluator", _OracleRun)
    monkeypatch.setattr(regression, "solver_ridge", lambda a, b, al: (solver_ridge_cpu(a, b, al), None))
    pm, case = _front_end()
    pm._train = [d.slice(0, 40) for d in pm._train]
    pm._test = [d.slice(0, 10) for d in pm._test]
    pm.append_hybrid_params(elements=["Mg", "O"], cutoff=5.0, model_type=2, max_p=2, feature_type="pair",
                            gaussian_params2=(0.0, 4.0, 4))
    pm.run()
    train_err, _ = pm.errors
    pm.save_mlp(str(tmp_path / "polymlp.yaml"))
    from pypolymlp_gb300.accuracy import prediction_errors
    from pypolymlp_gb300.io_polymlp import load_mlp

    models = [load_mlp(str(tmp_path / f"polymlp.yaml.{k}")) for k in (1, 2)]
    from pypolymlp_gb300.features_attr import get_num_features

    assert [len(c) for _, c in models] == [case["settings"]["n_features"], get_num_features(models[1][0])]
    assert pm.n_features == sum(len(c) for _, c in models)
    ph = hybrid.PropertiesHybrid([p for p, _ in models], [c for _, c in models])
    d = pm.train[0]
    e, f, s = ph.eval_multiple(d.axis, [np.asarray(x).T for x in d.positions], d.types)
    err, _ = prediction_errors(d, e, f, s)
    for k in ("energy", "force", "stress"):
        assert err[k] == pytest.approx(train_err["data1"][k], rel=1e-9)


def _md_front_end():
    """The reference's MD fit (test_mlp_devel_vasp.py::test_mlp_devel_md): Cu, 225
    features, one MD vasprun.xml whose steps the parameter file's data_md line
    splits into Train_ and Test_ datasets."""
    from test_known_fit import KA, _cases

    case = _cases()["md_Cu"]
    pm = Pypolymlp().load_parameter_file(f"{KA}/{case['input']}", prefix=KA)
    return pm, case


def _check_md(pm, case):
    from test_known_fit import _check as check_errors

    train, test = pm.errors
    name = case["md_file"]
    check_errors({"train": train["Train_" + name], "test": test["Test_" + name]}, case["errors"])


def test_front_end_md_fit_reproduces_reference_fit_errors(on_oracle):
    pm, case = _md_front_end()
    assert pm.n_features == case["settings"]["n_features"]
    assert [d.name for d in pm.train] == ["Train_" + case["md_file"]]
    pm.run()
    _check_md(pm, case)


@pytest.mark.gpu
def test_gpu_front_end_md_fit_reproduces_reference_fit_errors():
    pm, case = _md_front_end()
    pm.run()
    _check_md(pm, case)
