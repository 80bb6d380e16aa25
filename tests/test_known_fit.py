"""Known answers of the reference's end-to-end fit tests
(tests/test_mlp_dev_api/test_mlp_devel_vasp.py: a pair and a gtinv model of MgO
fitted to 270 vasprun structures and tested on 30, and the gtinv model fitted
to two datasets (270 + 630) and tested on two (30 + 70); data and asserted
errors copied by tests/golden/make_known_answers.py).  The regression pipeline restated
on the CPU (oracle X rows, numpy Gram, LAPACK posv, the reference's weights,
scales and alpha selection) and the GPU fit (FP64) must give the asserted
train/test errors: energy 1e-8 eV/atom, force 1e-6 eV/A, stress 1e-5 eV/atom
absolute, the reference test's tolerances.  The mixed-precision GPU fit (FP32
rows, tensor-core Gram) must give them within 0.05 meV/atom (energy) and
1 meV/A (force), the bounds it is built to."""

import json
import os

import numpy as np
import pytest

from pypolymlp_gb300.accuracy import prediction_errors
from pypolymlp_gb300.params import make_params_dict
from pypolymlp_gb300.regression import Dataset

KA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "known_answers")


def _cases():
    with open(os.path.join(KA, "known_fit.json")) as f:
        return json.load(f)["cases"]


def _datasets(case):
    """(training datasets, test datasets) of a case, named as in its error table.
    Automatic division ("auto"): each group's files in sorted order (testN, then
    trainN) form one dataset, split as the reference's split_train_test splits
    files, into trainN and testN."""
    z = np.load(os.path.join(KA, case["data"]))
    stress = case["settings"]["include_stress"]
    if "auto" in case:
        from pypolymlp_gb300.io_vasp import split_ids_train_test

        train, test = [], []
        for g, (tags, force) in enumerate(zip(case["auto"]["groups"], case["auto"]["force"]), start=1):
            parts = []
            for tag in tags:
                n = z[f"{tag}_n_atoms"]
                offs = np.concatenate([[0], np.cumsum(n)])
                for i in range(len(n)):
                    sl = slice(offs[i], offs[i + 1])
                    parts.append((z[f"{tag}_axis"][i], z[f"{tag}_positions"][sl], z[f"{tag}_types"][sl],
                                  z[f"{tag}_energies"][i], z[f"{tag}_forces"][sl], z[f"{tag}_stresses"][i]))
            tr, te = split_ids_train_test(len(parts), 0.9)
            for ids, name, out in ((tr, f"train{g}", train), (te, f"test{g}", test)):
                sel = [parts[i] for i in ids]
                out.append(Dataset([p[0] for p in sel], [p[1] for p in sel], [p[2] for p in sel],
                                   np.array([p[3] for p in sel]), [p[4] for p in sel], np.array([p[5] for p in sel]),
                                   include_force=force, include_stress=stress and force, name=name))
        return train, test

    def one(tag):
        n = z[f"{tag}_n_atoms"]
        offs = np.concatenate([[0], np.cumsum(n)])
        sl = [slice(offs[i], offs[i + 1]) for i in range(len(n))]
        return Dataset([a for a in z[f"{tag}_axis"]], [z[f"{tag}_positions"][s] for s in sl],
                       [z[f"{tag}_types"][s] for s in sl], z[f"{tag}_energies"],
                       [z[f"{tag}_forces"][s] for s in sl], z[f"{tag}_stresses"], include_stress=stress, name=tag)

    return [one(t) for t in case["train"]], [one(t) for t in case["test_sets"]]


def _params(st):
    kw = dict(n_type=st["n_type"], cutoff=st["cutoff"], model_type=st["model_type"], max_p=st["max_p"],
              feature_type=st["feature_type"], gaussian_params1=tuple(st["gaussian_params1"]),
              gaussian_params2=tuple(st["gaussian_params2"]), elements=st["elements"])
    if st["feature_type"] == "gtinv":
        kw.update(gtinv_order=st["gtinv_order"], gtinv_maxl=tuple(st["gtinv_maxl"]))
    return make_params_dict(**kw)


def _check(errors, known):
    for tag, got in errors.items():
        for key, want in known[tag].items():
            assert got[key] == pytest.approx(want["value"], abs=want["abs"]), (tag, key, got[key], want["value"])


def cpu_fit(p, train, test, alphas):
    """(coefficients of the best alpha in the scaled basis, scales): oracle X rows,
    numpy Gram, LAPACK posv, the reference's selection by test RMSE."""
    from oracle.pipeline import calc_xtx_xty_cpu, solver_ridge_cpu
    from pypolymlp_gb300.regression import compute_rmse_seq

    xy = calc_xtx_xty_cpu(p, train)
    coefs = solver_ridge_cpu(xy.xtx, xy.xty, alphas)
    txy = calc_xtx_xty_cpu(p, test, scales=xy.scales, min_energy=xy.min_energy)
    return coefs[:, int(np.argmin(compute_rmse_seq(coefs, txy)))], xy.scales


def cpu_errors(p, coeffs, datasets):
    """Prediction errors per dataset with the oracle's E/F/S."""
    from oracle import oracle
    from pypolymlp_gb300.abi import Structures

    errors = {}
    for d in datasets:
        e, f, s = oracle.evaluate(p, coeffs, Structures(d.axis, d.positions, d.types))
        offs = np.concatenate([[0], np.cumsum(d.total_n_atoms)])
        errors[d.name], _ = prediction_errors(d, e, [f[offs[i]:offs[i + 1]] for i in range(len(d))], s)
    return errors


def _single_cases(slow_auto=False):
    """One-model fits from the npz data; with slow_auto the automatic-division
    cases carry the slow mark (minutes on the CPU)."""
    out = []
    for k, c in sorted(_cases().items()):
        if "models" in c or "md_file" in c:
            continue
        out.append(pytest.param(k, marks=pytest.mark.slow) if slow_auto and "auto" in c else k)
    return out


def _hybrid_cases():
    return sorted(k for k, c in _cases().items() if "models" in c)


@pytest.mark.parametrize("name", _single_cases(slow_auto=True))
def test_cpu_pipeline_reproduces_reference_fit_errors(name):
    from oracle import oracle

    case = _cases()[name]
    p = _params(case["settings"])
    assert oracle.n_features(p) == case["settings"]["n_features"]
    train, test = _datasets(case)
    c, scales = cpu_fit(p, train, test, case["settings"]["alphas"])
    _check(cpu_errors(p, c / scales, train + test), case["errors"])


def _gpu_fit_errors(name, precision):
    from pypolymlp_gb300.accuracy import PolymlpEvalAccuracy
    from pypolymlp_gb300.regression import fit

    case = _cases()[name]
    p = _params(case["settings"])
    train, test = _datasets(case)
    res = fit(p, train, test, case["settings"]["alphas"], precision=precision)
    acc = PolymlpEvalAccuracy(p, res.scaled_coeffs)
    return {d.name: acc.compute_error_single(d, log_energy=False) for d in train + test}, case, res


@pytest.mark.gpu
@pytest.mark.parametrize("name", _single_cases())
def test_gpu_fit_reproduces_reference_fit_errors(name):
    from pypolymlp_gb300 import _ffi

    errors, case, _ = _gpu_fit_errors(name, _ffi.PG_FP64)
    _check(errors, case["errors"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", _single_cases())
def test_gpu_mixed_fit_reproduces_reference_fit_errors(name):
    """FP32 rows and the tensor-core Gram, solved directly: every asserted
    energy and force error within 0.05 meV/atom and 1 meV/A, stresses within
    the reference's own tolerance scaled the same way (1e-5 eV/atom -> 0.05 meV/atom)."""
    from pypolymlp_gb300 import _ffi

    errors, case, res = _gpu_fit_errors(name, _ffi.PG_MIXED)
    bounds = {"energy": 0.05e-3, "force": 1e-3, "stress": 0.05e-3}
    worst = {}
    for tag, got in errors.items():
        for key, want in case["errors"][tag].items():
            d = abs(got[key] - want["value"])
            worst[key] = max(worst.get(key, 0.0), d)
            assert d < bounds[key], (tag, key, got[key], want["value"])
    print(f"{name}: alpha {res.alpha}, worst |delta| " + ", ".join(f"{k} {v:.3e}" for k, v in worst.items()))


def _hybrid_errors(params_list, coeffs, cum, datasets, evaluate):
    """Prediction errors of a hybrid (the sum of its models) per dataset."""
    bounds = [0] + list(cum)
    errors = {}
    for d in datasets:
        from pypolymlp_gb300.abi import Structures

        st = Structures(d.axis, d.positions, d.types)
        e = f = s = 0.0
        for k, p in enumerate(params_list):
            ek, fk, sk = evaluate(p, coeffs[bounds[k]:bounds[k + 1]], st)
            e, f, s = e + ek, f + fk, s + sk
        offs = np.concatenate([[0], np.cumsum(d.total_n_atoms)])
        errors[d.name], _ = prediction_errors(d, e, [f[offs[i]:offs[i + 1]] for i in range(len(d))], s)
    return errors


@pytest.mark.slow
@pytest.mark.parametrize("name", _hybrid_cases())
def test_cpu_hybrid_fit_reproduces_reference_fit_errors(name, monkeypatch):
    """test_mlp_devel_vasp.py::test_mlp_devel_hybrid_single_dataset: three gtinv
    models of MgO (infile-hybrid-MgO/polymlp{1,2,3}_hybrid.in, 5,736 features in
    all) fitted together (about two minutes on 8 cores: marked slow).  hybrid.fit_hybrid on the CPU with the oracle's X rows
    per model, numpy's Gram and LAPACK posv standing in for the device (checker
    only); the errors of the summed models from the oracle's E/F/S."""
    from test_hybrid import _oracle_hybrid_x

    from oracle import oracle
    from oracle.pipeline import solver_ridge_cpu
    from pypolymlp_gb300 import _ffi, hybrid, regression

    monkeypatch.setattr(hybrid, "hybrid_features_x", _oracle_hybrid_x)
    monkeypatch.setattr(_ffi, "gram_xtx", lambda x, precision=None: x.T @ x)
    monkeypatch.setattr(regression, "solver_ridge", lambda a, b, al: (solver_ridge_cpu(a, b, al), None))
    case = _cases()[name]
    ps = [_params(m) for m in case["models"]]
    assert sum(oracle.n_features(p) for p in ps) == case["settings"]["n_features"]
    train, test = _datasets(case)
    res, cum = hybrid.fit_hybrid(ps, train, test, case["settings"]["alphas"])
    assert cum[-1] == case["settings"]["n_features"]
    errors = _hybrid_errors(ps, res.coeffs / res.scales, cum, train + test, oracle.evaluate)
    _check(errors, case["errors"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", _hybrid_cases())
@pytest.mark.parametrize("mixed", [False, True])
def test_gpu_hybrid_fit_reproduces_reference_fit_errors(name, mixed):
    """The same hybrid fit on the GPU (hybrid X rows, device Gram, device
    Cholesky; errors from the GPU evaluator, FP64): at the reference's
    tolerances in FP64, within 0.05 meV/atom and 1 meV/A (stress 0.05 meV/atom)
    in mixed precision."""
    from pypolymlp_gb300 import _ffi, hybrid

    case = _cases()[name]
    ps = [_params(m) for m in case["models"]]
    train, test = _datasets(case)
    res, cum = hybrid.fit_hybrid(ps, train, test, case["settings"]["alphas"],
                                 precision=_ffi.PG_MIXED if mixed else _ffi.PG_FP64)
    assert cum[-1] == case["settings"]["n_features"]

    def evaluate(p, c, st):
        return _ffi.Evaluator(p, c, _ffi.PG_FP64).run(st)

    errors = _hybrid_errors(ps, res.coeffs / res.scales, cum, train + test, evaluate)
    if not mixed:
        _check(errors, case["errors"])
        return
    bounds = {"energy": 0.05e-3, "force": 1e-3, "stress": 0.05e-3}
    for tag, got in errors.items():
        for key, want in case["errors"][tag].items():
            assert abs(got[key] - want["value"]) < bounds[key], (tag, key, got[key], want["value"])
