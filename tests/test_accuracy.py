"""Prediction errors (pypolymlp_gb300.accuracy): the error arithmetic of
eval_accuracy.py:60-133 on given predictions (CPU), and PolymlpEvalAccuracy
through the GPU evaluator against the same arithmetic on the oracle's E/F/S."""

import numpy as np
import pytest

from pypolymlp_gb300 import synthetic as syn
from pypolymlp_gb300.accuracy import EV_TO_GPA, PolymlpEvalAccuracy, prediction_errors
from pypolymlp_gb300.regression import Dataset


def _labelled(n, seed):
    ss = syn.binary_set(n, seed=seed, n_min=8, n_max=16)
    syn.morse_labels(ss, syn.morse_D(2), rc=5.0)
    return Dataset.from_structure_set(ss, name="data/set.1")


def test_prediction_errors_arithmetic():
    d = _labelled(3, 71)
    rng = np.random.default_rng(1)
    e = d.energies + rng.normal(size=len(d)) * 0.01
    f = [x + rng.normal(size=x.shape) * 0.05 for x in d.forces]
    s = d.stresses + rng.normal(size=d.stresses.shape) * 0.1
    err, _ = prediction_errors(d, e, f, s, force_direction=True)
    n = d.total_n_atoms.astype(float)
    assert err["energy"] == pytest.approx(np.sqrt(np.mean(((d.energies - e) / n) ** 2)), rel=1e-12)
    assert err["energy_mae"] == pytest.approx(np.mean(np.abs((d.energies - e) / n)), rel=1e-12)
    tf, pf = np.concatenate([x.ravel() for x in d.forces]), np.concatenate([x.ravel() for x in f])
    assert err["force"] == pytest.approx(np.sqrt(np.mean((tf - pf) ** 2)), rel=1e-12)
    t3, p3 = tf.reshape(-1, 3), pf.reshape(-1, 3)
    cos = np.sum(t3 * p3, axis=1) / np.linalg.norm(t3, axis=1) / np.linalg.norm(p3, axis=1)
    assert err["force_direction"] == pytest.approx(np.degrees(np.arccos(np.mean(np.abs(cos)))), rel=1e-10)
    ns = np.repeat(n, 6)
    assert err["stress"] == pytest.approx(np.sqrt(np.mean(((d.stresses - s).ravel() / ns) ** 2)), rel=1e-12)
    err_gpa, _ = prediction_errors(d, e, f, s, stress_unit="GPa")
    vol = np.repeat([abs(np.linalg.det(a)) for a in d.axis], 6)
    want = np.sqrt(np.mean(((d.stresses - s).ravel() * EV_TO_GPA / vol) ** 2))
    assert err_gpa["stress"] == pytest.approx(want, rel=1e-12)
    d.forces, d.stresses = None, None
    err_e, _ = prediction_errors(d, e, f, s)
    assert err_e["force"] is None and err_e["stress"] is None


@pytest.mark.gpu
def test_eval_accuracy_on_gpu_matches_oracle(tmp_path):
    from oracle import oracle
    from pypolymlp_gb300.abi import Structures
    from pypolymlp_gb300.params import make_params_dict

    p = make_params_dict(n_type=2, cutoff=5.0, model_type=3, max_p=2, gaussian_params2=(0.0, 4.0, 4),
                         gtinv_order=3, gtinv_maxl=(4, 2))
    d = _labelled(4, 72)
    c = np.random.default_rng(3).normal(size=oracle.n_features(p)) * 1e-3
    acc = PolymlpEvalAccuracy(p, c)
    errs = acc.compute_error([d], stress_unit="GPa", log_energy=True, log_force=True, path_output=str(tmp_path))
    got = errs["data/set.1"]
    e, f, s = oracle.evaluate(p, c, Structures(d.axis, d.positions, d.types))
    offs = np.concatenate([[0], np.cumsum(d.total_n_atoms)])
    want, _ = prediction_errors(d, e, [f[offs[i]:offs[i + 1]] for i in range(len(d))], s, stress_unit="GPa")
    for k in ("energy", "force", "stress", "energy_mae", "force_mae", "stress_mae"):
        assert got[k] == pytest.approx(want[k], rel=1e-8, abs=1e-12), k
    assert (tmp_path / "predictions" / "energy.train-data-set-1.dat").exists()
    assert (tmp_path / "predictions" / "force.train-data-set-1.dat").exists()
