"""Known answers of the reference's own property tests
(tests/test_calc/test_properties_*.py: potentials shipped with its tests, in
polymlp.yaml and legacy polymlp.lammps form, pair and gtinv, with conditional
pair parameters, a spin-polarised Fe model (enable_spins: one element, two atom
types) and two hybrid models, on small cells; fixtures and asserted
values copied by tests/golden/make_known_answers.py).  The files are read by
pypolymlp_gb300.io_polymlp; the oracle (CPU) must reproduce every asserted value
at the reference test's tolerance, the GPU evaluator (FP64) too, with the
energy compared to 1e-10 relative where the reference asserts 1e-12 absolute
(its own summation order)."""

import json
import os

import numpy as np
import pytest

from pypolymlp_gb300 import io_polymlp
from pypolymlp_gb300.abi import Structures
from pypolymlp_gb300.hybrid import active_atoms

KA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "known_answers")
EV_TO_GPA = 160.21766208


def read_poscar(path, elements):
    """(axis with lattice vectors as columns, Cartesian positions (N, 3), types in `elements` order)."""
    lines = [ln.split() for ln in open(path).read().splitlines()]
    scale = float(lines[1][0])
    axis = np.array([[float(v) for v in lines[k]] for k in (2, 3, 4)]).T * scale
    names, counts = lines[5], [int(v) for v in lines[6]]
    kind = lines[7][0].lower()
    n = sum(counts)
    frac = np.array([[float(v) for v in lines[8 + i][:3]] for i in range(n)])
    pos = frac @ axis.T if kind.startswith("d") else frac * scale
    types = np.concatenate([[elements.index(e)] * c for e, c in zip(names, counts)])
    return axis, pos, types


def _cases():
    with open(os.path.join(KA, "known_answers.json")) as f:
        return json.load(f)["cases"]


def _load(case):
    models = [io_polymlp.load_mlp(os.path.join(KA, p)) for p in case["potentials"]]
    if "cell" in case:
        # a cell written in the test module: axis columns are the lattice vectors
        axis = np.array(case["cell"]["axis"], dtype=np.float64)
        pos = (axis @ np.array(case["cell"]["positions_frac"], dtype=np.float64)).T
        return models, axis, pos, np.array(case["cell"]["types"])
    axis, pos, types = read_poscar(os.path.join(KA, case["structure"]), models[0][0]["elements"])
    return models, axis, pos, types


def _check(case, e, f, s, axis, gpu=False):
    tol = dict(case["energy_tol"])
    if gpu and "abs" in tol:
        tol = {"rel": 1e-10}
    assert e == pytest.approx(case["energy"], **tol)
    if case["forces_kind"] == "f00":
        assert abs(f[0][0]) <= case["forces_atol"]
    elif case["forces_kind"] == "zero":
        np.testing.assert_allclose(f, 0.0, atol=case["forces_atol"])
    else:
        np.testing.assert_allclose(f, case["forces"], atol=case["forces_atol"], rtol=0)
    if "stresses" in case:
        s = np.asarray(s, dtype=np.float64)
        if case["stresses_unit"] == "GPa":
            s = s / abs(np.linalg.det(axis)) * EV_TO_GPA
        np.testing.assert_allclose(s, case["stresses"], atol=case["stresses_atol"], rtol=0)


@pytest.mark.parametrize("name", sorted(_cases()))
def test_oracle_reproduces_reference_known_answers(name):
    from oracle import oracle

    case = _cases()[name]
    models, axis, pos, types = _load(case)
    e, f, s = 0.0, np.zeros((len(types), 3)), np.zeros(6)
    for p, c in models:
        idx, t = active_atoms(types, p)
        if len(idx) == 0:
            continue
        em, fm, sm = oracle.evaluate(p, c, Structures([axis], [pos[idx]], [t]))
        e += float(em[0])
        f[idx] += fm
        s += sm[0]
    _check(case, e, f, s, axis)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(_cases()))
def test_gpu_evaluator_reproduces_reference_known_answers(name):
    from pypolymlp_gb300 import _ffi
    from pypolymlp_gb300.hybrid import PropertiesHybrid

    case = _cases()[name]
    models, axis, pos, types = _load(case)
    hy = PropertiesHybrid([p for p, _ in models], [c for _, c in models], _ffi.PG_FP64)
    e, f, s = hy.eval(axis, pos.T, types)
    _check(case, e, f, s, axis, gpu=True)


def _x_cases():
    with open(os.path.join(KA, "known_x.json")) as f:
        return json.load(f)["cases"]


def _x_inputs(case):
    from pypolymlp_gb300.abi import row_layout

    p, _ = io_polymlp.load_mlp(os.path.join(KA, case["potential"]))
    cells = [read_poscar(os.path.join(KA, n), p["elements"]) for n in case["structures"]]
    st = Structures([c[0] for c in cells], [c[1] for c in cells], [c[2] for c in cells])
    return p, st, row_layout(st.n_atoms, [False] * st.n_st)


def _check_x(case, x):
    assert list(x.shape) == case["shape"]
    assert float(np.sum(x)) == pytest.approx(case["sum"], **case["sum_tol"])
    assert float(np.sum(x[0] - x[1])) == pytest.approx(case["diff01"], **case["diff01_tol"])


@pytest.mark.parametrize("name", sorted(_x_cases()))
def test_oracle_x_reproduces_reference_known_answers(name):
    """Energy rows of X (test_compute_features.py: shape, sum, row difference)."""
    from oracle import oracle

    case = _x_cases()[name]
    p, st, (e, f, s, n) = _x_inputs(case)
    _check_x(case, oracle.features_x(p, st, e, f, s, n))


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(_x_cases()))
def test_gpu_x_reproduces_reference_known_answers(name):
    from pypolymlp_gb300 import _ffi

    case = _x_cases()[name]
    p, st, (e, f, s, n) = _x_inputs(case)
    m = _ffi.Model(p)
    _check_x(case, m.features_x(st, e, f, s, n, precision=_ffi.PG_FP64))
    # mixed (FP32 rows): the total to 1e-5; the row difference is a small
    # difference of large sums and below FP32 resolution at 1e-6
    x32 = m.features_x(st, e, f, s, n, precision=_ffi.PG_MIXED)
    assert float(np.sum(x32)) == pytest.approx(case["sum"], rel=1e-5)


def _fn_cases():
    with open(os.path.join(KA, "known_functions.json")) as f:
        return json.load(f)["cases"]


def test_oracle_radial_functions_reproduce_reference_known_answers():
    """f_n and df_n/dr of tests/test_cxx/test_functions.py::test_get_fn."""
    from oracle import oracle

    c = _fn_cases()["fn"]
    f, fd = oracle.fn(c["r"], c["cutoff"], c["params"])
    np.testing.assert_allclose(f, c["fn"], rtol=c["rtol"])
    np.testing.assert_allclose(fd, c["fn_d"], rtol=c["rtol"])


@pytest.mark.parametrize("name", ["test_get_ylm", "test_get_ylm_2"])
def test_oracle_ylm_reproduce_reference_known_answers(name):
    """Y_lm and its gradients (sums for l_max 10, tables for l_max 3)."""
    from oracle import oracle

    c = _fn_cases()[name]
    x, y, z = c["x"], c["y"], c["z"]
    got = oracle.ylm(float(np.sqrt(x * x + y * y + z * z)), x, y, z, c["lmax"])
    if "sums" in c:
        for g, (re, im) in zip(got, c["sums"]):
            assert complex(np.sum(g)) == pytest.approx(complex(re, im), rel=c["sums_rel"])
    if "tables" in c:
        for g, key in zip(got, ("ylm_true", "ylm_dx_true", "ylm_dy_true", "ylm_dz_true")):
            want = np.array([complex(a, b) for a, b in c["tables"][key]])
            np.testing.assert_allclose(g, want, atol=c["tables_atol"], rtol=0)


@pytest.mark.parametrize("name", ["MgO_pair_legacy", "SrTiO3_pair_cond_legacy"])
def test_legacy_file_converted_to_yaml_keeps_the_known_answers(tmp_path, name):
    """A shipped legacy file rewritten by convert_to_yaml evaluates to the same known answers."""
    from oracle import oracle

    case = _cases()[name]
    out = str(tmp_path / "polymlp.yaml")
    assert io_polymlp.convert_to_yaml(os.path.join(KA, case["potentials"][0]), out)
    p, c = io_polymlp.load_mlp(out)
    axis, pos, types = read_poscar(os.path.join(KA, case["structure"]), p["elements"])
    e, f, s = oracle.evaluate(p, c, Structures([axis], [pos], [types]))
    _check(case, float(e[0]), f, s[0], axis)


@pytest.mark.parametrize("name", ["polymlp.yaml.gtinv.MgO", "polymlp.lammps.pair.Ag"])
def test_rewritten_shipped_file_parses_like_the_original(tmp_path, name):
    """Load a shipped file, write it again as polymlp.yaml: the reference's C++ parser
    reads the same model and coefficients (to the 16 significant digits written)."""
    from oracle import ref as refb

    if not refb.available():
        pytest.skip("the reference build (oracle/_ref) is not present")
    src = os.path.join(KA, name)
    p, c = io_polymlp.load_mlp(src)
    out = str(tmp_path / "polymlp.yaml")
    io_polymlp.save_mlp_yaml(p, c, np.ones(len(c)), out, mass=p["mass"])
    a = refb.parse_potential(src, legacy=io_polymlp.is_legacy(src))
    b = refb.parse_potential(out, legacy=False)
    for k in ("elements", "cutoff", "pair_type", "feature_type", "model_type", "max_p", "cond"):
        assert a[k] == b[k], k
    np.testing.assert_array_equal(a["params"], b["params"])
    np.testing.assert_allclose(b["coeffs"], a["coeffs"], rtol=1e-15, atol=0)
    np.testing.assert_allclose(b["mass"], a["mass"], rtol=0, atol=0)


def _energy_cases():
    with open(os.path.join(KA, "known_energies.json")) as f:
        return json.load(f)["cases"]


def _energy_cells(case):
    """(params, coefficients, axes, Cartesian positions (N, 3) and types per cell,
    asserted energies, tolerances).
    An "expansion" H re-shapes the cell: lattice vectors become the rows of H times the
    unit cell's (H unimodular: the same crystal), positions stay where they are."""
    p, c = io_polymlp.load_mlp(os.path.join(KA, case["potential"]))
    axes, pos, types = [], [], []
    for cell in case["cells"]:
        axis, x, t = read_poscar(os.path.join(KA, cell["structure"]), p["elements"])
        if "expansion" in cell:
            h = np.array(cell["expansion"], dtype=np.float64)
            assert round(abs(np.linalg.det(h))) == 1
            axis = axis @ h.T
        axes.append(axis)
        pos.append(x)
        types.append(t)
    return p, c, axes, pos, types, [cell["energy"] for cell in case["cells"]], [cell["tol"] for cell in case["cells"]]


def _approx(want, tol):
    return pytest.approx(want, rel=tol.get("rel"), abs=tol.get("atol", tol.get("abs")))


@pytest.mark.parametrize("name", sorted(_energy_cases()))
def test_oracle_energies_reproduce_reference_known_answers(name):
    """Legacy gtinv Ti-Al on five cells (test_api_properties_legacy_Ti-Al.py) and pair
    MgO on 25 differently shaped cells of one crystal, down to lattice vectors ten
    times the cell edge (test_check_neighbors.py::test_eval_neighbors_MgO)."""
    from oracle import oracle

    p, c, axes, pos, types, want, tol = _energy_cells(_energy_cases()[name])
    e, _, _ = oracle.evaluate(p, c, Structures(axes, pos, types))
    for got, w, t in zip(e, want, tol):
        assert float(got) == _approx(w, t)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(_energy_cases()))
def test_gpu_energies_reproduce_reference_known_answers(name):
    """The same cells through PotentialPropertiesFast.eval_multiple (FP64), energies
    to 1e-10 relative (the reference asserts 1e-12: its own summation order)."""
    from pypolymlp_gb300 import _ffi
    from pypolymlp_gb300.properties import PotentialPropertiesFast

    p, c, axes, pos, types, want, _ = _energy_cells(_energy_cases()[name])
    prop = PotentialPropertiesFast(p, c, _ffi.PG_FP64)
    prop.eval_multiple(axes, [x.T for x in pos], types)
    np.testing.assert_allclose(prop.get_e_array(), want, rtol=1e-10, atol=0)
