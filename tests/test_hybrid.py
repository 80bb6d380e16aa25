"""Hybrid models (pypolymlp_gb300.hybrid): atom selection on the CPU; E/F/S
(PropertiesHybrid) and X (PotentialHybridModel) on the GPU against the oracle
applied model by model to the atoms each model sees."""

import numpy as np
import pytest

from pypolymlp_gb300 import synthetic as syn
from pypolymlp_gb300.abi import Structures, row_layout
from pypolymlp_gb300.hybrid import active_atoms
from pypolymlp_gb300.params import make_params_dict


def test_active_atoms():
    t = np.array([0, 2, 1, 2, 0])
    idx, tt = active_atoms(t, {"type_full": False, "type_indices": [2, 0]})
    assert idx.tolist() == [0, 1, 3, 4] and tt.tolist() == [1, 0, 0, 1]
    idx, tt = active_atoms(t, {"type_full": True})
    assert idx.tolist() == [0, 1, 2, 3, 4] and tt.tolist() == t.tolist()
    idx, tt = active_atoms(t, {})
    assert idx.tolist() == [0, 1, 2, 3, 4]
    # a spin model sees every atom, or none is chosen (properties_utils.py:14-16)
    spin = {"type_full": False, "type_indices": [0], "spin_elements": {"elements": ["Fe"]}}
    with pytest.raises(RuntimeError):
        active_atoms(t, spin)
    assert active_atoms(t, dict(spin, type_full=True))[0].tolist() == [0, 1, 2, 3, 4]


def _hybrid():
    full = make_params_dict(n_type=2, cutoff=5.0, model_type=2, max_p=2, feature_type="pair",
                            gaussian_params2=(0.0, 4.0, 4))
    sub = make_params_dict(n_type=1, cutoff=5.0, model_type=3, max_p=2, gaussian_params2=(0.0, 4.0, 3),
                           gtinv_order=3, gtinv_maxl=(4, 2))
    sub["type_full"] = False
    sub["type_indices"] = [1]
    return full, sub


def _sub_structures(ss, p):
    sel = [active_atoms(t, p) for t in ss.types]
    keep = [s for s in range(len(ss.types)) if len(sel[s][0])]
    st = Structures([ss.axis[s] for s in keep], [np.asarray(ss.positions[s])[sel[s][0]] for s in keep],
                    [sel[s][1] for s in keep])
    return st, sel, keep


@pytest.mark.gpu
def test_properties_hybrid_matches_oracle_sum():
    from oracle import oracle
    from pypolymlp_gb300.hybrid import PropertiesHybrid

    full, sub = _hybrid()
    ss = syn.binary_set(3, seed=81, n_min=8, n_max=20)
    rng = np.random.default_rng(5)
    cf = rng.normal(size=oracle.n_features(full)) * 1e-3
    cs = rng.normal(size=oracle.n_features(sub)) * 1e-3
    hy = PropertiesHybrid([full, sub], [cf, cs])
    e, f, s = hy.eval_multiple(ss.axis, [np.asarray(p).T for p in ss.positions], ss.types)
    st = Structures(ss.axis, ss.positions, ss.types)
    e0, f0, s0 = oracle.evaluate(full, cf, st)
    offs = st.atom_offsets
    f_ref = [f0[offs[i]:offs[i + 1]].copy() for i in range(st.n_st)]
    sub_st, sel, keep = _sub_structures(ss, sub)
    e1, f1, s1 = oracle.evaluate(sub, cs, sub_st)
    o1 = sub_st.atom_offsets
    e_ref, s_ref = e0.copy(), s0.copy()
    for q, i in enumerate(keep):
        e_ref[i] += e1[q]
        s_ref[i] += s1[q]
        f_ref[i][sel[i][0]] += f1[o1[q]:o1[q + 1]]
    scale_e = np.abs(e_ref).max()
    assert np.abs(e - e_ref).max() < 1e-10 * scale_e
    fa, fr = np.concatenate(f), np.concatenate(f_ref)
    assert np.abs(fa - fr).max() < 1e-10 * np.abs(fr).max()
    assert np.abs(s - s_ref).max() < 1e-10 * np.abs(s_ref).max()


@pytest.mark.gpu
def test_hybrid_x_matches_oracle_per_model():
    from oracle import oracle
    from pypolymlp_gb300.hybrid import PotentialHybridModel

    full, sub = _hybrid()
    ss = syn.binary_set(3, seed=82, n_min=8, n_max=20)
    n_atoms = [len(t) for t in ss.types]
    hm = PotentialHybridModel([full, sub], ss.axis, [np.asarray(p).T for p in ss.positions], ss.types,
                              [len(n_atoms)], [True], n_atoms)
    x, cum = hm.get_x(), hm.get_cumulative_n_features()
    st = Structures(ss.axis, ss.positions, ss.types)
    e, f, s, n = row_layout(st.n_atoms, [True] * st.n_st)
    x0 = oracle.features_x(full, st, e, f, s, n)
    sub_st, sel, keep = _sub_structures(ss, sub)
    e1, f1, s1, n1 = row_layout(sub_st.n_atoms, [True] * sub_st.n_st)
    x1 = oracle.features_x(sub, sub_st, e1, f1, s1, n1)
    ref = np.zeros_like(x)
    ref[:, :cum[0]] = x0
    for q, i in enumerate(keep):
        ref[e[i], cum[0]:] = x1[e1[q]]
        ref[s[i]:s[i] + 6, cum[0]:] = x1[s1[q]:s1[q] + 6]
        rows = f[i] + (3 * sel[i][0][:, None] + np.arange(3)[None, :]).reshape(-1)
        ref[rows, cum[0]:] = x1[f1[q]:f1[q] + 3 * len(sel[i][0])]
    scale = np.maximum(np.abs(ref).max(axis=0), 1e-300)
    assert (np.abs(x - ref) / scale).max() < 1e-10
    assert cum == [x0.shape[1], x0.shape[1] + x1.shape[1]]


def _oracle_hybrid_x(params_list, st, e_row, f_row, s_row, n_rows, precision=None):
    """hybrid_features_x with the oracle's X per model (checker only)."""
    from oracle import oracle

    offs = st.atom_offsets
    cum, blocks = [], []
    for p in params_list:
        pos = [st.positions[offs[s]:offs[s + 1]] for s in range(st.n_st)]
        types = [st.types[offs[s]:offs[s + 1]] for s in range(st.n_st)]
        sel = [active_atoms(t, p) for t in types]
        sub = Structures(list(st.axis), [pos[s][sel[s][0]] for s in range(st.n_st)], [sel[s][1] for s in range(st.n_st)])
        e, f, s6, n = row_layout(sub.n_atoms, [f_row[s] >= 0 for s in range(st.n_st)])
        xs = oracle.features_x(p, sub, e, f, s6, n)
        x = np.zeros((n_rows, xs.shape[1]))
        for s in range(st.n_st):
            x[e_row[s]] = xs[e[s]]
            if f_row[s] >= 0:
                x[s_row[s]:s_row[s] + 6] = xs[s6[s]:s6[s] + 6]
                rows = f_row[s] + (3 * sel[s][0][:, None] + np.arange(3)[None, :]).reshape(-1)
                x[rows] = xs[f[s]:f[s] + 3 * len(sel[s][0])]
        blocks.append(x)
        cum.append(sum(b.shape[1] for b in blocks))
    return np.asfortranarray(np.hstack(blocks)), cum


def test_hybrid_fit_of_one_model_reproduces_reference_fit_errors(monkeypatch):
    """fit_hybrid with the pair MgO model alone, on the reference's MgO fit data, must
    give the reference's asserted errors (test_mlp_devel_vasp.py::test_mlp_devel_pair);
    the GPU X rows, device Gram and device posv are replaced by the oracle, numpy and
    LAPACK (checker only)."""
    from test_known_fit import _cases, _check, _datasets, _params, cpu_errors

    from oracle.pipeline import solver_ridge_cpu
    from pypolymlp_gb300 import _ffi, hybrid, regression

    monkeypatch.setattr(hybrid, "hybrid_features_x", _oracle_hybrid_x)
    monkeypatch.setattr(_ffi, "gram_xtx", lambda x, precision=None: x.T @ x)
    monkeypatch.setattr(regression, "solver_ridge", lambda a, b, al: (solver_ridge_cpu(a, b, al), None))
    case = _cases()["pair_single"]
    p = _params(case["settings"])
    train, test = _datasets(case)
    res, cum = hybrid.fit_hybrid([p], train, test, case["settings"]["alphas"])
    assert cum == [case["settings"]["n_features"]]
    _check(cpu_errors(p, res.coeffs / res.scales, train + test), case["errors"])
