"""Known answers of the reference's own tests (test_calc/test_properties_MgO.py:
two shipped MgO potentials on a displaced rocksalt cell; fixtures and the
asserted values copied by tests/golden/make_known_answers.py).  The shipped
polymlp.yaml files are read by pypolymlp_gb300.io_polymlp; the oracle (CPU)
and the GPU evaluator must reproduce the asserted energy (1e-8 relative),
forces (1e-6 eV/A) and stresses (1e-5 GPa), the reference test's tolerances."""

import json
import os

import numpy as np
import pytest

from pypolymlp_gb300 import io_polymlp
from pypolymlp_gb300.abi import Structures

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


def _check(case, e, f, s, axis, force_atol=None, energy_rel=None, stress_atol=None):
    tol = case["tolerances"]
    assert e == pytest.approx(case["energy"], rel=energy_rel or tol["energy_rel"])
    np.testing.assert_allclose(f, case["forces"], atol=force_atol or tol["forces_abs"], rtol=0)
    s_gpa = np.asarray(s) / abs(np.linalg.det(axis)) * EV_TO_GPA
    np.testing.assert_allclose(s_gpa, case["stresses_gpa"], atol=stress_atol or tol["stresses_gpa_abs"], rtol=0)


def _load(case):
    p, c = io_polymlp.load_mlp(os.path.join(KA, case["potential"]))
    axis, pos, types = read_poscar(os.path.join(KA, case["structure"]), p["elements"])
    return p, c, Structures([axis], [pos], [types]), axis


@pytest.mark.parametrize("name", sorted(_cases()))
def test_oracle_reproduces_reference_known_answers(name):
    from oracle import oracle

    case = _cases()[name]
    p, c, st, axis = _load(case)
    e, f, s = oracle.evaluate(p, c, st)
    _check(case, float(e[0]), f, s[0], axis)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(_cases()))
def test_gpu_evaluator_reproduces_reference_known_answers(name):
    from pypolymlp_gb300 import _ffi

    case = _cases()[name]
    p, c, st, axis = _load(case)
    e, f, s = _ffi.Evaluator(p, c, _ffi.PG_FP64).run(st)
    _check(case, float(e[0]), f, s[0], axis)
    # mixed precision: FP32 features and adjoint (1e-6 relative energy, 1e-4 eV/A, 1e-3 GPa)
    e, f, s = _ffi.Evaluator(p, c, _ffi.PG_MIXED).run(st)
    _check(case, float(e[0]), f, s[0], axis, force_atol=1e-4, energy_rel=1e-6, stress_atol=1e-3)
