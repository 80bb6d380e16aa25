"""vasprun.xml datasets (pypolymlp_gb300.io_vasp and Pypolymlp.set_datasets_vasp)
against the reference's own reading of the same files (core/interface_vasp.py,
run where the reference sources were present; values and files in
tests/golden/known_answers, written by make_known_answers.py)."""

import json
import os

import numpy as np
import pytest

from pypolymlp_gb300 import io_vasp

KA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "known_answers")


def _known():
    with open(os.path.join(KA, "known_vasp.json")) as f:
        return json.load(f)["cases"]


FILES = [k for k in _known() if not k.startswith("_")]


@pytest.mark.parametrize("name", FILES)
def test_vasprun_reads_what_the_reference_reads(name):
    want = _known()[name]
    v = io_vasp.Vasprun(os.path.join(KA, name))
    assert v.energy == want["energy"]
    np.testing.assert_array_equal(v.forces, want["forces"])
    np.testing.assert_array_equal(v.stress, want["stress_kbar"])
    st = v.structure
    np.testing.assert_array_equal(st.axis, want["axis"])
    np.testing.assert_array_equal(st.positions, want["positions"])
    assert list(st.n_atoms) == want["n_atoms"] and list(st.elements) == want["elements"]
    assert list(st.types) == want["types"] and st.volume == want["volume"]


def test_parse_properties_converts_stresses_to_ev_per_cell():
    want = _known()["_parsed"]
    sts, (e, f, s) = io_vasp.parse_properties_from_vaspruns([os.path.join(KA, n) for n in want["files"]])
    assert len(sts) == len(want["files"]) and len(f) == len(sts)
    np.testing.assert_array_equal(e, want["energies"])
    np.testing.assert_array_equal(s, want["stresses_ev"])


def test_split_follows_the_reference_rule():
    """core/utils.py:18-27: round(n * ratio) training structures, the test ones
    evenly spaced from the first to the last."""
    tr, te = io_vasp.split_ids_train_test(10, 0.9)
    assert te.tolist() == [0] and tr.tolist() == list(range(1, 10))
    tr, te = io_vasp.split_ids_train_test(20, 0.8)
    assert te.tolist() == [0, 6, 13, 19] and len(tr) == 16
    assert io_vasp.split_train_test(list("abcde"), 0.6) == (["b", "c", "d"], ["a", "e"])


def test_set_datasets_vasp_builds_the_reference_dataset():
    """Energies minus atomic energies, types by the model's element order,
    forces (N, 3), stresses (xx, yy, zz, xy, yz, zx) in eV per cell."""
    from pypolymlp_gb300.mlp_dev import Pypolymlp

    known = _known()
    files = [os.path.join(KA, n) for n in FILES]
    pm = Pypolymlp().set_params(elements=["Mg", "O"], feature_type="pair", model_type=2, max_p=2, cutoff=6.0,
                                atomic_energy=(-0.25, -0.75))
    pm.set_datasets_vasp(train_vaspruns=files[:3], test_vaspruns=files[3:])
    d = pm.train[0]
    assert d.name == "data1" and pm.test[0].name == "data2" and len(d) == 3 and len(pm.test[0]) == 1
    for k, name in enumerate(sorted(FILES[:3])):
        w = known[name]
        elements = w["elements"]
        types = [["Mg", "O"].index(e) for e in elements]
        assert d.types[k].tolist() == types
        assert d.energies[k] == pytest.approx(w["energy"] - sum((-0.25, -0.75)[t] for t in types), abs=1e-12)
        np.testing.assert_array_equal(d.forces[k], np.array(w["forces"]).T)
        axis = np.array(w["axis"])
        np.testing.assert_allclose(d.positions[k], (axis @ np.array(w["positions"])).T, rtol=0, atol=1e-12)
        sig = np.array(w["stress_kbar"]) * w["volume"] / io_vasp.EV_TO_KBAR
        np.testing.assert_array_equal(d.stresses[k], [sig[0, 0], sig[1, 1], sig[2, 2], sig[0, 1], sig[1, 2],
                                                      sig[2, 0]])
    pm.set_multiple_datasets_vasp([files[:2], files[2:3]], [files[3:]])
    assert [x.name for x in pm.train] == ["data1", "data2"] and [len(x) for x in pm.train] == [2, 1]
    pm.set_datasets_vasp(vaspruns=files, train_ratio=0.75)
    assert len(pm.train[0]) == 3 and len(pm.test[0]) == 1
