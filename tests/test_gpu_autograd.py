"""The torch.autograd energy function and the bound evaluator, on the GPU.

Model: the binary X^T X model (gtinv order 3, l_max (8, 4), rc 7 A,
F = 2,618) with seeded random coefficients; cell: bcc 8 x 8 x 8 x 2 = 1,024
atoms, a = 3.2 A, displacements N(0, 0.1 A), species 50/50 (the evaluator
workload's small cell).

* autograd forces (-dE/dr from the adjoint backward pass) equal
  pg_eval_run's forces to 1e-10 of max|F| (FP64) and the CPU oracle's
  (the reference algorithm) to 1e-9;
* central finite differences of the forward energy, h = 1e-4 A, on 50 seeded
  atoms (150 components): |F_fd - F| < 1e-6 eV/A;
* positions moved by less than skin / 2 reuse the neighbour lists (no
  rebuild) and give pg_eval_run's E/F/S on the moved positions to 1e-10;
  larger moves rebuild and agree as well;
* the evaluator's device workspace stays within the lists, a_nlm and the
  per-pair gradients: no per-atom derivative arrays;
* the mixed-precision (FP32) bound evaluator: forces within 1e-4 of max|F|;
* the ASE calculator's loop keeps its lists across small steps and matches
  the per-call evaluation.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PARAMS = dict(n_type=2, cutoff=7.0, model_type=3, max_p=2, gaussian_params2=(0.0, 5.0, 10), gtinv_order=3,
              gtinv_maxl=(8, 4))


@pytest.fixture(scope="module")
def case():
    from pypolymlp_gb300 import _ffi
    from pypolymlp_gb300 import synthetic as syn
    from pypolymlp_gb300.params import make_params_dict

    p = make_params_dict(**PARAMS)
    coefs = np.random.default_rng(4).normal(size=_ffi.Model(p).n_features) * 1e-3
    ss = syn.bcc_supercell(8, a=3.2, sigma=0.1, seed=4)
    return p, coefs, ss


def _run(p, coefs, axis, pos, types):
    from pypolymlp_gb300 import _ffi
    from pypolymlp_gb300.abi import Structures

    return _ffi.Evaluator(p, coefs, _ffi.PG_FP64).run(Structures([axis], [pos], [types]))


def test_autograd_forces_match_evaluator_and_oracle(case):
    import torch

    from oracle import oracle
    from pypolymlp_gb300.abi import Structures
    from pypolymlp_gb300.torch_potential import PolymlpPotential

    p, coefs, ss = case
    axis, pos, types = ss.axis[0], ss.positions[0], ss.types[0]
    pot = PolymlpPotential(p, coefs).bind(axis, pos, types)
    e_ref, f_ref, s_ref = _run(p, coefs, axis, pos, types)
    for device in ("cpu", "cuda"):
        r = torch.tensor(pos, dtype=torch.float64, device=device, requires_grad=True)
        e = pot.energy(r)
        (g,) = torch.autograd.grad(e.sum(), r)
        f_ad = -g.cpu().numpy()
        assert abs(float(e[0]) - e_ref[0]) <= 1e-10 * abs(e_ref[0])
        assert np.abs(f_ad - f_ref).max() <= 1e-10 * np.abs(f_ref).max()
        np.testing.assert_allclose(pot.last_stress[0], s_ref[0], rtol=0, atol=1e-10 * np.abs(s_ref).max())
    e_o, f_o, _ = oracle.evaluate(p, coefs, Structures([axis], [pos], [types]))
    assert np.abs(f_ad - f_o).max() <= 1e-9 * np.abs(f_o).max()
    assert abs(float(e[0]) - e_o[0]) <= 1e-10 * abs(e_o[0])


def test_autograd_forces_match_central_differences(case):
    import torch

    from pypolymlp_gb300.torch_potential import PolymlpPotential

    p, coefs, ss = case
    axis, pos, types = ss.axis[0], ss.positions[0], ss.types[0]
    pot = PolymlpPotential(p, coefs).bind(axis, pos, types)
    r = torch.tensor(pos, dtype=torch.float64, requires_grad=True)
    (g,) = torch.autograd.grad(pot.energy(r).sum(), r)
    f_ad = -g.numpy()
    h = 1e-4
    rng = np.random.default_rng(50)
    worst = 0.0
    for a in rng.choice(len(pos), 50, replace=False):
        for c in range(3):
            q = pos.copy()
            q[a, c] += h
            ep = float(pot.energy(torch.tensor(q))[0])
            q[a, c] -= 2 * h
            em = float(pot.energy(torch.tensor(q))[0])
            worst = max(worst, abs(-(ep - em) / (2 * h) - f_ad[a, c]))
    assert worst < 1e-6, worst
    assert pot.rebuilds == 0  # every displacement stayed inside skin / 2


def test_bound_lists_are_reused_and_rebuilt(case):
    from pypolymlp_gb300 import _ffi
    from pypolymlp_gb300.abi import Structures

    p, coefs, ss = case
    axis, pos, types = ss.axis[0], ss.positions[0], ss.types[0]
    ev = _ffi.Evaluator(p, coefs, _ffi.PG_FP64)
    ev.bind(Structures([axis], [pos], [types]), skin=0.5)
    rng = np.random.default_rng(7)
    for step, amp, rebuild in ((1, 0.05, False), (2, 0.05, False), (3, 0.6, True)):
        pos = pos + rng.normal(0.0, amp / 3, pos.shape).clip(-amp, amp)
        assert ev.update(pos) == rebuild, step
        e, f, s = ev.bound_run()
        e_ref, f_ref, s_ref = _run(p, coefs, axis, pos, types)
        assert abs(e[0] - e_ref[0]) <= 1e-10 * abs(e_ref[0]), step
        assert np.abs(f - f_ref).max() <= 1e-10 * np.abs(f_ref).max(), step
        assert np.abs(s - s_ref).max() <= 1e-10 * np.abs(s_ref).max(), step
        assert abs(ev.bound_energy()[0] - e[0]) <= 1e-12 * abs(e[0]), step
    # workspace: neighbour lists (int + 3 doubles + float4 + key per entry), a_nlm and
    # its adjoint (2 x K0 complex per atom), per-pair gradients and mirrors
    k0 = int(_ffi.Model(p).work()["k0_pair"].sum(axis=1).max())
    n_pairs = len(_ffi.neighbor_list(Structures([axis], [pos], [types]), 0, 7.5)[1])
    bound = n_pairs * (4 + 24 + 16 + 8 + 24 + 8 + 8) + len(pos) * (2 * 16 * k0 + 8 * 16) + (1 << 20)
    assert ev.workspace_bytes() <= 1.5 * bound, (ev.workspace_bytes(), bound)
    # mixed precision
    ev32 = _ffi.Evaluator(p, coefs, _ffi.PG_MIXED)
    ev32.bind(Structures([axis], [pos], [types]), skin=0.5)
    _, f32, _ = ev32.bound_run()
    _, f_ref, _ = _run(p, coefs, axis, pos, types)
    assert np.abs(f32 - f_ref).max() <= 1e-4 * np.abs(f_ref).max()


def test_ase_calculator_keeps_lists_across_steps(case):
    from pypolymlp_gb300.ase_calculator import PolymlpASECalculator

    p, coefs, ss = case
    axis, pos, types = ss.axis[0], ss.positions[0], ss.types[0]
    names = np.array(p["elements"])[types]

    class Atoms:
        def __init__(self, r):
            self.cell = axis.T
            self.r = r

        def get_positions(self):
            return self.r

        def get_scaled_positions(self):
            return np.linalg.solve(axis, self.r.T).T % 1.0

        def get_chemical_symbols(self):
            return list(names)

        def get_volume(self):
            return abs(np.linalg.det(axis))

    ase_calc = PolymlpASECalculator(params=p, coeffs=coefs)
    per_call = PolymlpASECalculator(params=p, coeffs=coefs, reuse_neighbors=False)
    rng = np.random.default_rng(9)
    r = pos.copy()
    for _ in range(4):
        r = r + rng.normal(0.0, 0.02, r.shape)
        atoms = Atoms(r)
        e = ase_calc.get_potential_energy(atoms)
        f = ase_calc.get_forces(atoms)
        e1 = per_call.get_potential_energy(atoms)
        f1 = per_call.get_forces(atoms)
        assert abs(e - e1) <= 1e-10 * abs(e1)
        assert np.abs(f - f1).max() <= 1e-10 * np.abs(f1).max()
    assert ase_calc._bound[0].rebuilds == 0
