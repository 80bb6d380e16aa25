"""The Properties front end (pypolymlp_gb300.calculator): structures with element
names, models from files, type renumbering per model, partial and spin models,
hybrid sums, GPa stresses and the saved files.

On the CPU the GPU evaluator is replaced by the oracle (test infrastructure)
so that the front end's own logic is checked against the reference's known
answers (tests/golden/known_answers: the property tests' potentials, cells and
asserted values) and against test_calc/test_properties_attrs.py's checks; the
`gpu` tests run the same cases through the GPU evaluator."""

import json
import os

import numpy as np
import pytest

from pypolymlp_gb300 import calculator as calc
from pypolymlp_gb300.abi import Structures

KA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "known_answers")


class _OracleEvaluator:
    """PotentialPropertiesFast's interface over the CPU oracle (checker only)."""

    def __init__(self, params, coeffs, precision=None):
        self._p, self._c = params, coeffs

    def eval_multiple(self, axis_array, positions_c_array, types_array):
        from oracle import oracle

        st = Structures.from_columns(axis_array, positions_c_array, types_array)
        e, f, s = oracle.evaluate(self._p, self._c, st)
        offs = st.atom_offsets
        self._e, self._s = e, s
        self._f = [f[offs[i]:offs[i + 1]] for i in range(st.n_st)]

    def get_e_array(self):
        return self._e

    def get_f_array(self):
        return self._f

    def get_s_array(self):
        return self._s


@pytest.fixture
def on_oracle(monkeypatch):
    from pypolymlp_gb300 import properties

    monkeypatch.setattr(properties, "PotentialPropertiesFast", _OracleEvaluator)


def _cases():
    with open(os.path.join(KA, "known_answers.json")) as f:
        return json.load(f)["cases"]


def _structure(case):
    if "cell" in case:
        c = case["cell"]
        n = len(c["types"])
        return calc.PolymlpStructure(c["axis"], c["positions_frac"], [n], ["Fe"] * n, c["types"])
    return calc.load_poscar(os.path.join(KA, case["structure"]))


def _check(case, prop, gpu=False):
    st = _structure(case)
    e, f, s = prop.eval(st)
    assert f.shape == (3, len(st.types)) and s.shape == (6,)
    tol = dict(case["energy_tol"])
    if gpu and "abs" in tol:
        tol = {"rel": 1e-10}
    assert e == pytest.approx(case["energy"], **tol)
    if case["forces_kind"] == "f00":
        assert abs(f[0][0]) <= case["forces_atol"]
    elif case["forces_kind"] == "zero":
        np.testing.assert_allclose(f, 0.0, atol=case["forces_atol"])
    else:
        want = np.array(case["forces"])
        np.testing.assert_allclose(f.T, want, atol=case["forces_atol"], rtol=0)
    if "stresses" in case:
        got = prop.stresses_gpa[0] if case["stresses_unit"] == "GPa" else s
        np.testing.assert_allclose(got, case["stresses"], atol=case["stresses_atol"], rtol=0)


def _pots(case):
    return [os.path.join(KA, p) for p in case["potentials"]]


@pytest.mark.parametrize("name", sorted(_cases()))
def test_properties_reproduce_reference_known_answers(on_oracle, name):
    case = _cases()[name]
    pots = _pots(case)
    _check(case, calc.Properties(pot=pots if len(pots) > 1 else pots[0]))


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(_cases()))
def test_gpu_properties_reproduce_reference_known_answers(name):
    case = _cases()[name]
    pots = _pots(case)
    _check(case, calc.Properties(pot=pots if len(pots) > 1 else pots[0]), gpu=True)


def test_eval_multiple_hybrid_save_and_attributes(on_oracle, tmp_path, monkeypatch):
    """test_properties_attrs.py: one pair MgO model and the same model twice as a
    hybrid, on one cell and on a list of two; shapes, sums and the saved files."""
    case = _cases()["MgO_pair_yaml"]
    pot = _pots(case)[0]
    st = calc.load_poscar(os.path.join(KA, case["structure"]))
    prop = calc.Properties(pot=pot)
    energies, forces, stresses = prop.eval_multiple([st, st])
    np.testing.assert_allclose(energies, [case["energy"]] * 2, rtol=1e-8)
    assert np.array(prop.forces).shape == (2, 3, 8) and prop.stresses.shape == (2, 6)
    assert prop.params["n_type"] == 2 and prop.elements == ["Mg", "O"]
    monkeypatch.chdir(tmp_path)
    prop.save()
    for name in ("polymlp_energies.npy", "polymlp_forces.npy", "polymlp_stress_tensors.npy"):
        assert (tmp_path / name).exists()
    np.testing.assert_allclose(np.load(tmp_path / "polymlp_stress_tensors.npy"), prop.stresses_gpa)
    hy = calc.Properties(pot=[pot, pot])
    e, _, _ = hy.eval(st)
    assert e == pytest.approx(2 * case["energy"], rel=1e-8)
    energies, _, _ = hy.eval_multiple([st, st])
    np.testing.assert_allclose(energies, [2 * case["energy"]] * 2, rtol=1e-8)
    assert hy.stresses_gpa.shape == (2, 6)


def test_find_active_atoms():
    """properties_utils.py:9-44 (test_properties_attrs.py::test_find_active_atoms)."""
    st = calc.load_poscar(os.path.join(KA, "POSCAR.RS.MgO"))
    strs, atoms, kept = calc.find_active_atoms([st, st], ["Mg"])
    assert [len(s.elements) for s in strs] == [4, 4] and kept == [True, True]
    assert [a.tolist() for a in atoms] == [[0, 1, 2, 3]] * 2
    assert strs[0].types.tolist() == [0] * 4 and strs[0].positions.shape == (3, 4)
    assert calc.find_active_atoms([st], ["Al"]) == ([], [], [False])
    with pytest.raises(RuntimeError):
        calc.find_active_atoms([st], ["Fe", "Fe"])


def test_replace_types():
    """dataset_utils.py:11-46: by element order; repeated elements (spins) keep
    their atoms' given types apart, renumbered consecutively."""
    st = calc.PolymlpStructure(np.eye(3), np.zeros((3, 5)), [2, 3], ["O", "Mg", "O", "Mg", "Mg"], [9, 9, 9, 9, 9])
    assert calc.replace_types(st, ["Mg", "O"]).tolist() == [1, 0, 1, 0, 0]
    spin = calc.PolymlpStructure(np.eye(3), np.zeros((3, 5)), [5], ["Fe", "Fe", "Co", "Fe", "Co"], [3, 1, 0, 3, 7])
    assert calc.replace_types(spin, ["Fe", "Fe", "Co", "Co"]).tolist() == [1, 0, 2, 1, 3]
    with pytest.raises(RuntimeError):
        calc.replace_types(st, ["Mg"])


def test_load_poscar_matches_the_test_reader():
    from test_known_answers import read_poscar

    path = os.path.join(KA, "POSCAR.perovskite.SrTiO3")
    st = calc.load_poscar(path)
    axis, pos, types = read_poscar(path, ["Sr", "Ti", "O"])
    np.testing.assert_array_equal(st.axis, axis)
    np.testing.assert_allclose((st.axis @ st.positions).T, pos, rtol=0, atol=1e-15)
    assert st.types == types.tolist() and st.elements == ["Sr", "Ti", "O", "O", "O"]
    assert st.volume == pytest.approx(np.linalg.det(axis))


def test_properties_needs_a_model():
    with pytest.raises(RuntimeError):
        calc.Properties()


class _FakeAtoms:
    """The ASE Atoms accessors the calculator uses (ASE is not installed here)."""

    def __init__(self, st):
        self.cell = st.axis.T
        self._frac, self._symbols = st.positions.T, list(st.elements)

    def get_scaled_positions(self):
        return self._frac

    def get_chemical_symbols(self):
        return self._symbols

    def get_volume(self):
        return abs(np.linalg.det(self.cell))


def test_ase_calculator_reproduces_reference_known_answers(on_oracle):
    """calculator/utils/ase_calculator.py: energy, forces (n_atom, 3), stress in
    eV per cell (the reference's order), for atoms with interleaved elements."""
    from pypolymlp_gb300.ase_calculator import PolymlpASECalculator, ase_atoms_to_structure

    case = _cases()["MgO_pair_yaml"]
    st = calc.load_poscar(os.path.join(KA, case["structure"]))
    perm = np.array([0, 4, 1, 5, 2, 6, 3, 7])
    shuffled = calc.PolymlpStructure(st.axis, st.positions[:, perm], st.n_atoms, [st.elements[i] for i in perm],
                                     [st.types[i] for i in perm])
    atoms = _FakeAtoms(shuffled)
    assert ase_atoms_to_structure(atoms).elements == ["Mg", "O"] * 4
    # the per-call path (the GPU test covers the bound path that keeps neighbour lists)
    ase_calc = PolymlpASECalculator(pot=_pots(case)[0], reuse_neighbors=False)
    e = ase_calc.get_potential_energy(atoms)
    assert e == pytest.approx(case["energy"], **case["energy_tol"])
    f = ase_calc.get_forces(atoms)
    np.testing.assert_allclose(f, np.array(case["forces"])[perm], atol=case["forces_atol"], rtol=0)
    s = ase_calc.get_stress(atoms) * 160.21766208 / abs(np.linalg.det(st.axis))
    np.testing.assert_allclose(s, case["stresses"], atol=case["stresses_atol"], rtol=0)
    with pytest.raises(RuntimeError):
        PolymlpASECalculator()
