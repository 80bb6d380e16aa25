"""Known-answer fixtures from the reference's own property tests.

Run where the reference tree is available ($PYPOLYMLP_REFERENCE, default
/root/reference):

    python tests/golden/make_known_answers.py

The reference's tests/test_calc/test_properties_*.py evaluate potentials
shipped with its tests on small cells and assert energies, forces and
stresses at fixed values.  For the cases listed in CASES this script copies
the potential files and POSCARs into tests/golden/known_answers/ and takes the
asserted values from the test source (literal assignments such as
`energy_true = ...`, or the literal of the energy's `pytest.approx(...)`, read
with `ast`, never executed) into known_answers.json, together with the
comparison each test makes (forces (N, 3) or only forces[0][0]; stresses in
GPa or eV per cell; tolerances); from test_compute_features.py it takes the
shape, sum and first-minus-second-row sum of the energy rows of X for two MgO
cells (known_x.json).  It also writes the invariant tables the gtinv
potentials need with the reference's Readgtinv (oracle/_ref), the radial
function and Y_lm values of tests/test_cxx/test_functions.py
(known_functions.json), the neighbour-list and cell-translation values of
tests/test_cxx/test_neighbor*.py (known_neighbors.json), the invariant-table
values of tests/test_cxx/test_gtinv.py (known_gtinv.json), the energies of
the Ti-Al legacy gtinv test and of the MgO cell-shape test
(known_energies.json), radial-function settings computed by the reference's
params_utils.py (known_params.json), the reference's reading of a few vasprun
files (known_vasp.json), the PolymlpAPI sums of tests/test_cxx/test_polymlp_api*.py
(known_api.json), and the MgO pair
and gtinv fits of
tests/test_mlp_dev_api/test_mlp_devel_vasp.py (their vasprun data as arrays,
fit_MgO.npz, and the asserted train/test errors, known_fit.json).
"""

import ast
import json
import os
import shutil
import sys

import numpy as np

REF_ROOT = os.environ.get("PYPOLYMLP_REFERENCE", "/root/reference")

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

REF = REF_ROOT + "/tests/test_calc"
OUT = os.path.join(HERE, "known_answers")

# id: (test file, function, potentials, POSCAR, forces layout, stress unit)
#   forces: "NxT" forces_true is (N, 3) (the test compares forces.T), "3xN" it is
#   (3, N), "f00" only forces[0][0] == 0 is asserted
CASES = {
    "MgO_pair_yaml": ("test_properties_MgO.py", "test_eval1", ["polymlp.yaml.pair.MgO"], "POSCAR.RS.MgO", "NxT", "GPa"),
    "MgO_gtinv_yaml": ("test_properties_MgO.py", "test_eval2", ["polymlp.yaml.gtinv.MgO"], "POSCAR.RS.MgO", "NxT",
                       "GPa"),
    "MgO_pair_legacy": ("test_properties_legacy_MgO.py", "test_eval1", ["polymlp.lammps.pair.MgO"], "POSCAR.RS.MgO",
                        "NxT", "GPa"),
    "Ag_pair_legacy": ("test_properties_legacy_Ag.py", "test_eval1", ["polymlp.lammps.pair.Ag"], "POSCAR.fcc.Ag",
                       "3xN", "eV"),
    "SrTiO3_pair_legacy": ("test_properties_legacy_SrTiO3.py", "test_eval1", ["polymlp.lammps.pair.SrTiO3"],
                           "POSCAR.perovskite.SrTiO3", "f00", "GPa"),
    "SrTiO3_pair_cond_legacy": ("test_properties_legacy_SrTiO3.py", "test_eval2_cond",
                                ["polymlp.lammps.pair.cond.SrTiO3"], "POSCAR.perovskite.SrTiO3", "f00", "GPa"),
    "SrTiO3_gtinv_cond_yaml": ("test_properties_SrTiO3.py", "test_eval_cond", ["polymlp.yaml.gtinv.cond.SrTiO3"],
                               "POSCAR.perovskite.SrTiO3", "f00", "GPa"),
    "SrTiO3_hybrid_yaml": ("test_properties_SrTiO3.py", "test_eval_flexible",
                           ["polymlp.yaml.flexible.1.SrTiO3", "polymlp.yaml.flexible.2.SrTiO3"],
                           "POSCAR.perovskite.SrTiO3", "f00", None),
    # spin-polarised Fe (enable_spins: one element, two atom types), the cell is
    # written in the test module; "zero": all forces are asserted to vanish
    "Fe_spin_pair_yaml": ("test_properties_Fe.py", "test_eval1", ["polymlp.yaml.1.Fe"], None, "zero", "GPa"),
    "Fe_spin_hybrid_yaml": ("test_properties_Fe.py", "test_eval2", ["polymlp.yaml.1.Fe", "polymlp.yaml.2.Fe"], None,
                            "zero", "GPa"),
}


def _module_cell(path):
    """axis (columns = lattice vectors), fractional positions (3, N) and types of
    a test module's `axis = np.eye(3) * a`, `positions = np.array([...]).T`,
    `types = [...]` assignments (read as syntax, not run)."""
    found = {}
    for node in ast.parse(open(path).read()).body:
        if isinstance(node, ast.Assign) and isinstance(node.targets[0], ast.Name):
            found[node.targets[0].id] = node.value
    ax = found["axis"]
    if not (isinstance(ax, ast.BinOp) and isinstance(ax.op, ast.Mult) and getattr(ax.left.func, "attr", "") == "eye"):
        raise ValueError("unexpected axis expression")
    axis = (np.eye(ast.literal_eval(ax.left.args[0])) * ast.literal_eval(ax.right)).tolist()
    pos = found["positions"]
    transpose = isinstance(pos, ast.Attribute) and pos.attr == "T"
    arr = np.array(ast.literal_eval((pos.value if transpose else pos).args[0]), dtype=float)
    frac = (arr.T if transpose else arr).tolist()
    return {"axis": axis, "positions_frac": frac, "types": ast.literal_eval(found["types"])}


def _function(path, name):
    tree = ast.parse(open(path).read())
    for fn in tree.body:
        if isinstance(fn, ast.FunctionDef) and fn.name == name:
            return fn
    raise KeyError(name)


def _assigned(fn, name):
    for node in ast.walk(fn):
        if isinstance(node, ast.Assign) and len(node.targets) == 1 and isinstance(node.targets[0], ast.Name) \
                and node.targets[0].id == name:
            return ast.literal_eval(node.value)
    return None


def _energy_approx(fn):
    """(value or None, tolerance kwargs) of `energy == pytest.approx(x, rel=.. | abs=..)`."""
    for node in ast.walk(fn):
        if isinstance(node, ast.Compare) and isinstance(node.left, ast.Name) and node.left.id == "energy":
            call = node.comparators[0]
            if isinstance(call, ast.Call) and getattr(call.func, "attr", "") == "approx":
                kw = {k.arg: ast.literal_eval(k.value) for k in call.keywords}
                try:
                    val = ast.literal_eval(call.args[0])
                except ValueError:
                    val = None
                return val, kw
    raise KeyError("energy approx")


# X known answers (test_compute_features.py): potential, the assert helper, POSCARs
X_CASES = {
    "X_MgO_pair": ("polymlp.yaml.pair.MgO", "_assert_pair_MgO"),
    "X_MgO_gtinv": ("polymlp.yaml.gtinv.MgO", "_assert_gtinv_MgO"),
}
X_POSCARS = ["POSCAR-00001.MgO", "POSCAR-00002.MgO"]


def _x_asserts(fn):
    """shape and the two pytest.approx literals (sum(x), sum(x[0] - x[1])) with their kwargs."""
    shape, approx = None, []
    for node in ast.walk(fn):
        if isinstance(node, ast.Compare) and isinstance(node.left, ast.Attribute) and node.left.attr == "shape":
            shape = list(ast.literal_eval(node.comparators[0]))
        if isinstance(node, ast.Call) and getattr(node.func, "attr", "") == "approx":
            approx.append((ast.literal_eval(node.args[0]), {k.arg: ast.literal_eval(k.value) for k in node.keywords}))
    return shape, approx


def function_answers():
    """Radial functions and Y_lm of tests/test_cxx/test_functions.py: the inputs and
    the asserted values (test_get_fn, test_get_ylm sums, test_get_ylm_2 tables)."""
    path = REF_ROOT + "/tests/test_cxx/test_functions.py"
    out = {}
    fn = _function(path, "test_get_fn")
    call = next(n for n in ast.walk(fn) if isinstance(n, ast.Call) and getattr(n.func, "id", "") == "get_fn")
    kw = {k.arg: k.value for k in call.keywords}
    expected = [ast.literal_eval(n.args[1]) for n in ast.walk(fn)
                if isinstance(n, ast.Call) and getattr(n.func, "attr", "") == "assert_allclose"]
    out["fn"] = {"r": ast.literal_eval(kw["r"]), "cutoff": ast.literal_eval(kw["cutoff"]),
                 "params": _assigned(fn, "params"), "fn": expected[0], "fn_d": expected[1], "rtol": 1e-7}
    for name in ("test_get_ylm", "test_get_ylm_2"):
        f = _function(path, name)
        call = next(n for n in ast.walk(f) if isinstance(n, ast.Call) and getattr(n.func, "id", "") == "get_ylm")
        lmax = ast.literal_eval({k.arg: k.value for k in call.keywords}["lmax"])
        case = {"x": _assigned(f, "x"), "y": _assigned(f, "y"), "z": _assigned(f, "z"), "lmax": lmax}
        sums = [ast.literal_eval(n.args[0]) for n in ast.walk(f)
                if isinstance(n, ast.Call) and getattr(n.func, "attr", "") == "approx"]
        if sums:
            case["sums"] = [[v.real, v.imag] for v in sums]
            case["sums_rel"] = 1e-6
        tables = {k: _assigned(f, k) for k in ("ylm_true", "ylm_dx_true", "ylm_dy_true", "ylm_dz_true")}
        if all(v is not None for v in tables.values()):
            case["tables"] = {k: [[complex(v).real, complex(v).imag] for v in t] for k, t in tables.items()}
            case["tables_atol"] = 1e-7
        out[name] = case
    return out


def gtinv_answers():
    """Invariant-table requests of tests/test_cxx/test_gtinv.py and their asserted
    values: (kind, index path, expected, approx) per assert."""
    tree = ast.parse(open(REF_ROOT + "/tests/test_cxx/test_gtinv.py").read())
    out = {}
    for fn in tree.body:
        if not isinstance(fn, ast.FunctionDef) or not fn.name.startswith("test_"):
            continue
        call = next(n for n in ast.walk(fn) if isinstance(n, ast.Call) and getattr(n.func, "id", "") == "get_gtinv_attrs")
        kw = {k.arg: ast.literal_eval(k.value) for k in call.keywords}
        checks = []
        for st in fn.body:
            if not (isinstance(st, ast.Assert) and isinstance(st.test, ast.Compare)):
                continue
            left, right = st.test.left, st.test.comparators[0]
            approx = isinstance(right, ast.Call)
            want = ast.literal_eval(right.args[0] if approx else right)
            if isinstance(left, ast.Call):   # len(x) or tuple(x[i]...)
                kind = left.func.id
                node = left.args[0]
            else:
                kind, node = "item", left
            idx = []
            while isinstance(node, ast.Subscript):
                idx.insert(0, ast.literal_eval(node.slice))
                node = node.value
            checks.append({"name": node.id, "kind": kind, "idx": idx,
                           "expect": list(want) if isinstance(want, tuple) else want, "approx": approx})
        out[fn.name] = {"order": kw["order"], "lmax": kw["lmax"], "version": kw["version"], "checks": checks}
    return out


def _load_poscars_sequence(fn):
    """[(POSCAR name, energy, tolerance kwargs)] of a test that alternates
    `polymlp.load_poscars(path_file + "poscars/X")` and
    `assert energies[0] == pytest.approx(v, rel=..)`."""
    out, current = [], None
    for st in fn.body:
        if isinstance(st, ast.Expr) and isinstance(st.value, ast.Call) and \
                getattr(st.value.func, "attr", "") == "load_poscars":
            current = ast.literal_eval(st.value.args[0].right).split("/")[-1]
        elif isinstance(st, ast.Assert) and isinstance(st.test.comparators[0], ast.Call):
            call = st.test.comparators[0]
            out.append((current, ast.literal_eval(call.args[0]),
                        {k.arg: ast.literal_eval(k.value) for k in call.keywords}))
    return out


def energy_answers():
    """Energies the reference asserts for several cells of one potential:
    tests/test_calc/test_api_properties_legacy_Ti-Al.py::test_eval1 (legacy gtinv
    Ti-Al on five cells) and test_check_neighbors.py::test_eval_neighbors_MgO (pair
    MgO on 25 unimodular re-shapings of one rocksalt cell, energies all equal)."""
    cases = {}
    fn = _function(os.path.join(REF, "test_api_properties_legacy_Ti-Al.py"), "test_eval1")
    cells = [{"structure": n, "energy": e, "tol": tol} for n, e, tol in _load_poscars_sequence(fn)]
    cases["TiAl_gtinv_legacy"] = {"test": "tests/test_calc/test_api_properties_legacy_Ti-Al.py::test_eval1",
                                  "potential": "polymlp.lammps.gtinv.Ti-Al", "cells": cells}
    fn = _function(os.path.join(REF, "test_check_neighbors.py"), "test_eval_neighbors_MgO")
    expansions = _assigned(fn, "expansions")
    poscar = next(ast.literal_eval(n.args[0].right).split("/")[-1] for n in ast.walk(fn)
                  if isinstance(n, ast.Call) and getattr(n.func, "id", "") == "Poscar")
    close = next(n for n in ast.walk(fn) if isinstance(n, ast.Call) and getattr(n.func, "attr", "") == "assert_allclose")
    energy = ast.literal_eval(close.args[1])
    tol = {k.arg: ast.literal_eval(k.value) for k in close.keywords}
    cases["MgO_pair_cell_shapes"] = {
        "test": "tests/test_calc/test_check_neighbors.py::test_eval_neighbors_MgO",
        "potential": "polymlp.yaml.pair.MgO",
        "cells": [{"structure": poscar, "expansion": h, "energy": energy, "tol": tol} for h in expansions]}
    for case in cases.values():
        shutil.copyfile(os.path.join(REF, "files", "mlps", case["potential"]), os.path.join(OUT, case["potential"]))
        for c in case["cells"]:
            shutil.copyfile(os.path.join(REF, "files", "poscars", c["structure"]), os.path.join(OUT, c["structure"]))
    return cases


def param_answers():
    """Radial-function settings computed by the reference's own Python
    (core/params_utils.py set_gaussian_params with n_gaussians, and
    set_active_gaussian_params with element-pair distances), imported from the
    reference sources with its compiled module stubbed out (not used by them)."""
    import types

    sys.path.insert(0, REF_ROOT + "/src")
    stub = types.ModuleType("pypolymlp.cxx.lib")
    stub.libmlpcpp = None
    sys.modules.setdefault("pypolymlp.cxx.lib", stub)
    from pypolymlp.core.params_utils import set_active_gaussian_params, set_gaussian_params

    out = {"n_gaussians": [], "distance": []}
    for n, rc in ((3, 5.0), (5, 6.0), (10, 8.0), (14, 7.5)):
        out["n_gaussians"].append({"n_gaussians": n, "cutoff": rc,
                                   "pair_params": [list(map(float, p)) for p in set_gaussian_params(
                                       n_gaussians=n, cutoff=rc)]})
    settings = [
        (["Sr", "Ti", "O"], {("Sr", "Sr"): [3.5, 4.8], ("Ti", "O"): [1.9, 3.4], ("O", "Sr"): [2.7]},
         dict(params1=(1.0, 1.0, 1), params2=(0.0, 6.0, 13))),
        (["Mg", "O"], {("O", "Mg"): [2.1, 4.4]}, dict(n_gaussians=8, cutoff=7.0)),
        (["Al", "Cu", "Zn"], {("Cu", "Cu"): [2.55], ("Zn", "Al"): [2.7, 3.9]},
         dict(params1=(0.5, 1.5, 3), params2=(0.0, 5.0, 6))),
    ]
    for elements, dist, g in settings:
        pp = set_gaussian_params(**g)
        cond, flag = set_active_gaussian_params(pp, elements, dist)
        out["distance"].append({"elements": elements, "distance": [[list(k), v] for k, v in dist.items()],
                                "pair_params": [list(map(float, p)) for p in pp], "conditional": flag,
                                "cond": [[list(k), v] for k, v in cond.items()]})
    return out


VASP_FILES = {
    "vasprun-00001-MgO.xml": REF_ROOT + "/tests/files/vasprun-00001-MgO.xml",
    "vasprun-00002-MgO.xml": REF_ROOT + "/tests/files/vasprun-00002-MgO.xml",
    "vasprun-train1-00001.xml.polymlp": "data-vasp-MgO/vaspruns/train1/vasprun-00001.xml.polymlp",
    "vasprun-test1-00010.xml.polymlp": "data-vasp-MgO/vaspruns/test1/vasprun-00010.xml.polymlp",
}


def vasp_answers():
    """The reference's own vasprun reading (core/interface_vasp.py Vasprun and
    parse_properties_from_vaspruns, imported from its sources with the compiled
    module stubbed out) of a few files, copied alongside."""
    import types

    sys.path.insert(0, REF_ROOT + "/src")
    stub = types.ModuleType("pypolymlp.cxx.lib")
    stub.libmlpcpp = None
    sys.modules.setdefault("pypolymlp.cxx.lib", stub)
    from pypolymlp.core.interface_vasp import Vasprun, parse_properties_from_vaspruns

    out = {}
    for name, src in VASP_FILES.items():
        src = src if src.startswith("/") else os.path.join(FIT_DIR, src)
        shutil.copyfile(src, os.path.join(OUT, name))
        v = Vasprun(src)
        st = v.structure
        out[name] = {"energy": v.energy, "forces": v.forces.tolist(), "stress_kbar": v.stress.tolist(),
                     "axis": st.axis.tolist(), "positions": st.positions.tolist(), "n_atoms": list(st.n_atoms),
                     "elements": list(st.elements), "types": list(st.types), "volume": st.volume}
    files = [os.path.join(OUT, n) for n in VASP_FILES]
    sts, (e, f, s) = parse_properties_from_vaspruns(files)
    out["_parsed"] = {"files": list(VASP_FILES), "energies": e.tolist(), "stresses_ev": s.tolist()}
    return out


API_TESTS = {"test_polymlp_api.py": "polymlp.yaml.MgO", "test_polymlp_api_pair.py": "polymlp.yaml.pair.MgO"}


def api_answers():
    """Shapes and sums asserted by tests/test_cxx/test_polymlp_api*.py (the
    PolymlpAPI steps on arange / constant order parameters), per test function:
    [variable, "shape" | "sum", expected]; the potential files they load are
    copied (as api.<name>)."""
    out = {}
    for fname, pot in API_TESTS.items():
        tree = ast.parse(open(os.path.join(REF_ROOT + "/tests/test_cxx", fname)).read())
        shutil.copyfile(os.path.join(REF_ROOT + "/tests/files", pot), os.path.join(OUT, "api." + pot))
        for fn in tree.body:
            if not isinstance(fn, ast.FunctionDef) or not fn.name.startswith("test_compute"):
                continue
            checks = []
            for st in ast.walk(fn):
                if not (isinstance(st, ast.Assert) and isinstance(st.test, ast.Compare)):
                    continue
                left, right = st.test.left, st.test.comparators[0]
                if isinstance(left, ast.Attribute) and left.attr == "shape":
                    checks.append([left.value.id, "shape", list(ast.literal_eval(right))])
                elif isinstance(left, ast.Call) and getattr(left.func, "attr", "") == "sum":
                    want = ast.literal_eval(right.args[0] if isinstance(right, ast.Call) else right)
                    want = [want.real, want.imag] if isinstance(want, complex) else [float(want), 0.0]
                    checks.append([left.args[0].id, "sum", want])
            out[f"{fname}::{fn.name}"] = {"potential": "api." + pot, "checks": checks}
    return out


FIT_DIR = REF_ROOT + "/tests/test_mlp_dev_api"
EV_TO_KBAR = 1602.1766208


def _read_input(path):
    """key -> list of tokens of a polymlp.in file."""
    out = {}
    for line in open(path).read().splitlines():
        tok = line.split("#")[0].split()
        if tok:
            out[tok[0]] = tok[1:]
    return out


def _vasprun(path, elements):
    """One single-point vasprun (.xml.polymlp): the reference's Vasprun reading
    (core/interface_vasp.py:108-220) of energy (e_wo_entrp), forces, stress (kbar
    -> eV per cell, interface_vasp.py:72) and the final structure, atoms in the
    parameter file's element order (dataset_utils.py:225-245)."""
    import xml.etree.ElementTree as ET

    root = ET.parse(path).getroot()
    arr = lambda v: np.array([[float(x) for x in e.text.split()] for e in v])  # noqa: E731
    energy = float(root.find("calculation").find("energy")[1].text)
    forces = arr(root.find(".//*[@name='forces']"))
    stress = arr(root.find(".//*[@name='stress']"))
    st = root.find(".//*[@name='finalpos']")
    basis = arr(st.find(".//*[@name='basis']"))
    frac = arr(st.find(".//*[@name='positions']"))
    volume = float(st.find(".//*[@name='volume']").text)
    names = [rc.findall("c")[0].text.strip() for rc in root.findall(".//*[@name='atoms']/set/rc")]
    types = np.array([elements.index(n) for n in names])
    order = np.argsort(types, kind="stable")
    axis = basis.T
    pos = (frac @ basis)[order]
    sigma = stress * volume / EV_TO_KBAR
    s6 = [sigma[0][0], sigma[1][1], sigma[2][2], sigma[0][1], sigma[1][2], sigma[2][0]]
    return axis, pos, types[order], energy, forces[order], s6


# end-to-end fits of tests/test_mlp_dev_api/test_mlp_devel_vasp.py on the MgO
# vasprun data: case -> (input file, test function, error-check helper, the
# helper's arguments in order (dataset names))
FIT_CASES = {
    "pair_single": ("polymlp.in.vasp.pair.single.MgO", "test_mlp_devel_pair", "_check_errors_pair_single_dataset_MgO",
                    ["train1", "test1"]),
    "gtinv_single": ("polymlp.in.vasp.single.MgO", "test_mlp_devel_single_dataset",
                     "_check_errors_single_dataset_MgO", ["train1", "test1"]),
    "gtinv_multi": ("polymlp.in.vasp.multi.MgO", "test_mlp_devel_multiple_datasets",
                    "_check_errors_multiple_datasets_MgO", ["train1", "train2", "test1", "test2"]),
    # a hybrid of three gtinv models fitted together (5,736 features); the datasets,
    # alphas and atomic energies come from the first input file
    "hybrid_single": (["infile-hybrid-MgO/polymlp1_hybrid.in", "infile-hybrid-MgO/polymlp2_hybrid.in",
                       "infile-hybrid-MgO/polymlp3_hybrid.in"], "test_mlp_devel_hybrid_single_dataset",
                      "_check_errors_hybrid_single_dataset_MgO", ["train1", "test1"]),
}
FIT_DATA = "data-vasp-MgO/vaspruns/{}/vasprun-*.xml.polymlp"

# fits whose `data` lines the reference splits itself ("automatic division": the
# sorted files of glob "*N", i.e. testN then trainN, split by split_train_test):
# case -> (input file, test function, error helper or None (asserts inline),
# helper argument names, the file groups in sorted order, force flag per group)
AUTO_CASES = {
    "gtinv_single_auto": ("polymlp.in.vasp.single.auto.MgO", "test_mlp_devel_single_dataset_autodiv",
                          "_check_errors_single_dataset_MgO_auto", ["train1", "test1"],
                          [["test1", "train1"]], [True]),
    "gtinv_multi_auto": ("polymlp.in.vasp.multi.auto.MgO", "test_mlp_devel_multiple_datasets_autodiv", None, None,
                         [["test1", "train1"], ["test2", "train2"]], [True, True]),
    "gtinv_multi_auto_selective": ("polymlp.in.vasp.multi.auto.selective.MgO",
                                   "test_mlp_devel_multiple_datasets_autodiv_selective", None, None,
                                   [["test1", "train1"], ["test2", "train2"]], [True, False]),
}
# one MD vasprun.xml split by step (data_md): case -> (input, test, helper, names, file)
MD_CASES = {"md_Cu": ("polymlp.in.vasp.md.Cu", "test_mlp_devel_md", "_check_errors_md_Cu", ["train", "test"],
                      "data-vasp-md-Cu/vasprun.xml")}


def _inline_errors(fn):
    """{tag: {quantity: {value, abs}}} of asserts `error_<tag>[q] == approx(v, abs=a)`
    written in a test function itself."""
    expected = {}
    for node in ast.walk(fn):
        if isinstance(node, ast.Assert) and isinstance(node.test, ast.Compare) and \
                isinstance(node.test.left, ast.Subscript) and isinstance(node.test.left.value, ast.Name):
            var = node.test.left.value.id
            if not var.startswith("error_"):
                continue
            call = node.test.comparators[0]
            expected.setdefault(var[len("error_"):], {})[ast.literal_eval(node.test.left.slice)] = {
                "value": ast.literal_eval(call.args[0]), **{k.arg: ast.literal_eval(k.value) for k in call.keywords}}
    return expected


def _fit_errors(fn, names):
    """{dataset name: {quantity: {value, abs}}} of an error-check helper whose
    arguments are the datasets' error dicts in `names` order; checks under
    `if use_stress:` are left out (the tests call them without stress)."""
    args = [a.arg for a in fn.args.args]
    expected = {}
    for node in fn.body:
        if isinstance(node, ast.Assert) and isinstance(node.test, ast.Compare) and \
                isinstance(node.test.left, ast.Subscript):
            cmp = node.test
            ds = names[args.index(cmp.left.value.id)]
            call = cmp.comparators[0]
            expected.setdefault(ds, {})[ast.literal_eval(cmp.left.slice)] = {
                "value": ast.literal_eval(call.args[0]), **{k.arg: ast.literal_eval(k.value) for k in call.keywords}}
    return expected


def fit_known_answers():
    """The MgO fits of tests/test_mlp_dev_api/test_mlp_devel_vasp.py (FIT_CASES): the
    settings of each input file, the vasprun data of every dataset they use
    (atomic energies subtracted, dataset.py:295-310) as arrays, and the errors
    each test asserts per dataset."""
    import glob

    cases, arrays = {}, {}
    test_src = os.path.join(FIT_DIR, "test_mlp_devel_vasp.py")
    for cid, (infiles, test_fn, helper, names) in FIT_CASES.items():
        infiles = [infiles] if isinstance(infiles, str) else infiles
        inps = [_read_input(os.path.join(FIT_DIR, f)) for f in infiles]
        for f in infiles:
            shutil.copyfile(os.path.join(FIT_DIR, f), os.path.join(OUT, os.path.basename(f)))
        inp = inps[0]
        elements = inp["elements"]
        atom_e = np.array([float(v) for v in inp["atomic_energy"]])
        for tag in names:
            if f"{tag}_n_atoms" in arrays:
                continue
            files = sorted(glob.glob(os.path.join(FIT_DIR, FIT_DATA.format(tag))))
            rows = [_vasprun(f, elements) for f in files]
            e = np.array([r[3] - np.bincount(r[2], minlength=len(elements)) @ atom_e for r in rows])
            arrays.update({f"{tag}_n_atoms": np.array([len(r[2]) for r in rows]),
                           f"{tag}_axis": np.array([r[0] for r in rows]),
                           f"{tag}_positions": np.concatenate([r[1] for r in rows]),
                           f"{tag}_types": np.concatenate([r[2] for r in rows]), f"{tag}_energies": e,
                           f"{tag}_forces": np.concatenate([r[4] for r in rows]),
                           f"{tag}_stresses": np.array([r[5] for r in rows])})
            print(tag, len(files), "structures")
        fit = _function(test_src, test_fn)
        n_features = next(ast.literal_eval(n.comparators[0]) for n in ast.walk(fit)
                          if isinstance(n, ast.Compare) and getattr(n.left, "attr", "") == "n_features")
        a0, a1, na = (float(v) for v in inp["reg_alpha_params"])

        def settings(one):
            st = {"n_type": int(one["n_type"][0]), "elements": one["elements"],
                  "feature_type": one["feature_type"][0], "cutoff": float(one["cutoff"][0]),
                  "model_type": int(one["model_type"][0]), "max_p": int(one["max_p"][0]),
                  "gaussian_params1": [float(v) for v in one["gaussian_params1"]],
                  "gaussian_params2": [float(v) for v in one["gaussian_params2"]],
                  "alphas": list(np.logspace(a0, a1, int(na))), "n_features": n_features,
                  "include_stress": inp.get("include_stress", ["True"])[0].lower() in ("true", "1")}
            if st["feature_type"] == "gtinv":
                st["gtinv_order"] = int(one["gtinv_order"][0])
                st["gtinv_maxl"] = [int(v) for v in one["gtinv_maxl"]]
            return st

        st = settings(inp)
        cases[cid] = {"test": f"tests/test_mlp_dev_api/test_mlp_devel_vasp.py::{test_fn}", "settings": st,
                      "train": [n for n in names if n.startswith("train")],
                      "test_sets": [n for n in names if n.startswith("test")],
                      "errors": _fit_errors(_function(test_src, helper), names), "data": "fit_MgO.npz"}
        if len(inps) > 1:
            cases[cid]["models"] = [settings(one) for one in inps]
        print(cid, cases[cid]["errors"])
    def plain_settings(inp, n_features):
        a0, a1, na = (float(v) for v in inp["reg_alpha_params"])
        st = {"n_type": int(inp["n_type"][0]), "elements": inp["elements"], "feature_type": inp["feature_type"][0],
              "cutoff": float(inp["cutoff"][0]), "model_type": int(inp["model_type"][0]),
              "max_p": int(inp["max_p"][0]), "gaussian_params1": [float(v) for v in inp["gaussian_params1"]],
              "gaussian_params2": [float(v) for v in inp["gaussian_params2"]],
              "alphas": list(np.logspace(a0, a1, int(na))), "n_features": n_features,
              "include_stress": inp.get("include_stress", ["True"])[0].lower() in ("true", "1"),
              "atomic_energy": [float(v) for v in inp["atomic_energy"]]}
        if st["feature_type"] == "gtinv":
            st["gtinv_order"] = int(inp["gtinv_order"][0])
            st["gtinv_maxl"] = [int(v) for v in inp["gtinv_maxl"]]
        return st

    def n_features_of(fit):
        return next(ast.literal_eval(n.comparators[0]) for n in ast.walk(fit)
                    if isinstance(n, ast.Compare) and getattr(n.left, "attr", "") == "n_features")

    for cid, (infile, test_fn, helper, names, groups, forces) in AUTO_CASES.items():
        inp = _read_input(os.path.join(FIT_DIR, infile))
        shutil.copyfile(os.path.join(FIT_DIR, infile), os.path.join(OUT, infile))
        fit = _function(test_src, test_fn)
        errors = _fit_errors(_function(test_src, helper), names) if helper else _inline_errors(fit)
        cases[cid] = {"test": f"tests/test_mlp_dev_api/test_mlp_devel_vasp.py::{test_fn}",
                      "settings": plain_settings(inp, n_features_of(fit)), "auto": {"groups": groups, "force": forces},
                      "errors": errors, "data": "fit_MgO.npz"}
        print(cid, cases[cid]["errors"])
    for cid, (infile, test_fn, helper, names, md_file) in MD_CASES.items():
        inp = _read_input(os.path.join(FIT_DIR, infile))
        shutil.copyfile(os.path.join(FIT_DIR, infile), os.path.join(OUT, infile))
        os.makedirs(os.path.join(OUT, os.path.dirname(md_file)), exist_ok=True)
        shutil.copyfile(os.path.join(FIT_DIR, md_file), os.path.join(OUT, md_file))
        fit = _function(test_src, test_fn)
        cases[cid] = {"test": f"tests/test_mlp_dev_api/test_mlp_devel_vasp.py::{test_fn}",
                      "settings": plain_settings(inp, n_features_of(fit)), "input": infile, "md_file": md_file,
                      "errors": _fit_errors(_function(test_src, helper), names)}
        print(cid, cases[cid]["errors"])
    np.savez_compressed(os.path.join(OUT, "fit_MgO.npz"), **arrays)
    with open(os.path.join(OUT, "known_fit.json"), "w") as f:
        json.dump({"cases": cases}, f, indent=1)


# neighbour-list known answers (tests/test_cxx/test_neighbor*.py)
# (types in the POSCAR's element order, as the reference's Poscar reader gives them)
NEIGHBOR_TESTS = {"test_neighbor.py": "POSCAR-rocksalt", "test_neighbor_variants.py": "POSCAR-BiGd2"}


def _neighbor_expr(node):
    """(variable, indices, op, arg) of the left side of a neighbour-test assert."""
    def chain(n):
        idx = []
        while isinstance(n, ast.Subscript):
            idx.insert(0, ast.literal_eval(n.slice))
            n = n.value
        return n.id, idx

    if isinstance(node, ast.Call):
        f = node.func
        name = f.id if isinstance(f, ast.Name) else f.attr
        arg = node.args[0]
        if name == "len":
            return (*chain(arg), "len", None)
        if name == "sum":
            if isinstance(arg, ast.Call) and getattr(arg.func, "attr", "") == "square":
                return (*chain(arg.args[0]), "sumsq", None)
            return (*chain(arg), "sum", None)
        if name == "count_nonzero":
            inner = arg
            return (*chain(inner.args[0]), "count_close", ast.literal_eval(inner.args[1]))
    if isinstance(node, ast.Attribute) and node.attr == "shape":
        return (*chain(node.value.args[0]), "shape", None)
    if isinstance(node, ast.Subscript):
        return (*chain(node), "item", None)
    return None


def neighbor_answers():
    out = {}
    for fname, poscar in NEIGHBOR_TESTS.items():
        tree = ast.parse(open(os.path.join(REF_ROOT + "/tests/test_cxx", fname)).read())
        for fn in tree.body:
            if not isinstance(fn, ast.FunctionDef) or not fn.name.startswith("test_"):
                continue
            ctor, cutoff, attrs, checks = None, None, {}, []
            for st in fn.body:
                if isinstance(st, ast.Assign) and isinstance(st.value, ast.Call) and \
                        getattr(st.value.func, "id", "").startswith("Neighbor"):
                    ctor = st.value.func.id
                    cutoff = ast.literal_eval({k.arg: k.value for k in st.value.keywords}["cutoff"])
                elif isinstance(st, ast.Assign) and isinstance(st.value, ast.Attribute) and \
                        getattr(st.value.value, "id", "") == "neigh":
                    attrs[st.targets[0].id] = st.value.attr
                elif isinstance(st, ast.Assert) and isinstance(st.test, ast.Compare):
                    e = _neighbor_expr(st.test.left)
                    if e is None or e[0] not in attrs:
                        continue
                    cmpv = st.test.comparators[0]
                    approx = isinstance(cmpv, ast.Call)
                    val = ast.literal_eval(cmpv.args[0] if approx else cmpv)
                    checks.append({"ctor": ctor, "cutoff": cutoff, "attr": attrs[e[0]], "idx": e[1], "op": e[2],
                                   "arg": e[3], "expect": list(val) if isinstance(val, tuple) else val,
                                   "approx": approx})
            if checks:
                out[f"{fname}::{fn.name}"] = {"structure": poscar, "checks": checks}
        shutil.copyfile(os.path.join(REF_ROOT + "/tests/files", poscar), os.path.join(OUT, poscar))
    return out


def gtinv_file(order, maxl, version=1):
    """Fixture path of the reference's Readgtinv output for (order, l_max per order)."""
    tag = "_".join(str(int(v)) for v in list(maxl)[: max(order - 1, 0)])
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "gtinv",
                        f"gtinv_v{version}_order{order}_maxl{tag}.json")


def gtinv_spec(path):
    """(order, maxl) of a gtinv potential file, None for a pair potential."""
    lines = open(path).read().splitlines()
    if "# ele" in lines[0]:
        vals = [ln.split("#")[0].split() for ln in lines]
        if vals[3][0] != "gtinv":
            return None
        order = int(vals[7][0])
        return order, tuple(int(v) for v in vals[8][: order - 1])
    kv = {ln.split(":", 1)[0].strip(): ln.split(":", 1)[1].strip() for ln in lines if ":" in ln and
          not ln.startswith(("-", " "))}
    if kv.get("feature_type") != "gtinv":
        return None
    order = int(kv["gtinv_order"])
    maxl = tuple(int(v) for v in kv["gtinv_maxl"].strip("[]").split(","))
    return order, maxl[: order - 1]


def main():
    from oracle import ref

    os.makedirs(OUT, exist_ok=True)
    cases, tables = {}, set()
    for cid, (test, fname, pots, poscar, forces_kind, s_unit) in CASES.items():
        fn = _function(os.path.join(REF, test), fname)
        e_val, e_tol = _energy_approx(fn)
        if e_val is None:
            e_val = _assigned(fn, "energy_true")
        case = {"test": f"tests/test_calc/{test}::{fname}", "potentials": pots, "structure": poscar,
                "energy": e_val, "energy_tol": e_tol, "forces_kind": forces_kind, "forces_atol": 1e-6}
        if poscar is None:
            case["cell"] = _module_cell(os.path.join(REF, test))
        if forces_kind in ("NxT", "3xN"):
            f = _assigned(fn, "forces_true")
            case["forces"] = [list(r) for r in zip(*f)] if forces_kind == "3xN" else f
        elif forces_kind == "f00":
            case["forces_atol"] = 1e-12
        s = _assigned(fn, "stresses_true")
        if s_unit is not None and s is not None:
            case.update({"stresses": s, "stresses_unit": s_unit, "stresses_atol": 1e-5})
        cases[cid] = case
        for name in pots + ([poscar] if poscar else []):
            src = os.path.join(REF, "files", "mlps" if name.startswith("polymlp") else "poscars", name)
            shutil.copyfile(src, os.path.join(OUT, name))
        for p in pots:
            spec = gtinv_spec(os.path.join(OUT, p))
            if spec:
                tables.add(spec)
        print(cid, case["energy"], case["energy_tol"])
    with open(os.path.join(OUT, "known_answers.json"), "w") as f:
        json.dump({"source": "tests/test_calc/test_properties_*.py", "cases": cases}, f, indent=1)
    xcases = {}
    for cid, (pot, helper) in X_CASES.items():
        shape, approx = _x_asserts(_function(os.path.join(REF, "test_compute_features.py"), helper))
        xcases[cid] = {"test": f"tests/test_calc/test_compute_features.py::{helper}", "potential": pot,
                       "structures": X_POSCARS, "rows": "energy", "shape": shape,
                       "sum": approx[0][0], "sum_tol": approx[0][1], "diff01": approx[1][0], "diff01_tol": approx[1][1]}
        print(cid, shape, approx)
    for name in X_POSCARS:
        shutil.copyfile(os.path.join(REF, "files", "poscars", name), os.path.join(OUT, name))
    # the input file of test_api_features.py::test_features_from_infile1 (same model as X_MgO_gtinv)
    shutil.copyfile(os.path.join(REF, "files", "mlps", "polymlp.in.gtinv.MgO"), os.path.join(OUT, "polymlp.in.gtinv.MgO"))
    with open(os.path.join(OUT, "known_x.json"), "w") as f:
        json.dump({"source": "tests/test_calc/test_compute_features.py", "cases": xcases}, f, indent=1)
    with open(os.path.join(OUT, "known_functions.json"), "w") as f:
        json.dump({"source": "tests/test_cxx/test_functions.py", "cases": function_answers()}, f, indent=1)
    print("wrote known_functions.json")
    with open(os.path.join(OUT, "known_energies.json"), "w") as f:
        json.dump({"source": "tests/test_calc/test_api_properties_legacy_Ti-Al.py, test_check_neighbors.py",
                   "cases": energy_answers()}, f, indent=1)
    print("wrote known_energies.json")
    with open(os.path.join(OUT, "known_params.json"), "w") as f:
        json.dump({"source": "src/pypolymlp/core/params_utils.py (run here)", "cases": param_answers()}, f,
                  indent=1)
    print("wrote known_params.json")
    with open(os.path.join(OUT, "known_vasp.json"), "w") as f:
        json.dump({"source": "src/pypolymlp/core/interface_vasp.py (run here)", "cases": vasp_answers()}, f,
                  indent=1)
    print("wrote known_vasp.json")
    with open(os.path.join(OUT, "known_api.json"), "w") as f:
        json.dump({"source": "tests/test_cxx/test_polymlp_api*.py", "cases": api_answers()}, f, indent=1)
    print("wrote known_api.json")
    with open(os.path.join(OUT, "known_gtinv.json"), "w") as f:
        json.dump({"source": "tests/test_cxx/test_gtinv.py", "cases": gtinv_answers()}, f, indent=1)
    print("wrote known_gtinv.json")
    nb = neighbor_answers()
    with open(os.path.join(OUT, "known_neighbors.json"), "w") as f:
        json.dump({"source": "tests/test_cxx/test_neighbor*.py", "cases": nb}, f, indent=1)
    print("wrote known_neighbors.json:", {k: len(v["checks"]) for k, v in nb.items()})
    fit_known_answers()
    for order, maxl in sorted(tables):
        l_comb, lm_seq, lm_coeffs = ref.readgtinv(order, maxl)
        with open(gtinv_file(order, maxl), "w") as f:
            json.dump({"order": order, "maxl": list(maxl), "version": 1, "l_comb": l_comb, "lm_seq": lm_seq,
                       "lm_coeffs": lm_coeffs}, f, separators=(",", ":"))
        print("wrote", gtinv_file(order, maxl))


if __name__ == "__main__":
    main()
