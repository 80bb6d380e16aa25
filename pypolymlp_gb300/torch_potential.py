"""Energies as a differentiable torch function of the atomic positions.

E = sum_i c . F(features_i) is evaluated by the GPU evaluator, and its
gradient with respect to the positions comes from the evaluator's hand-written
adjoint kernels, not from autograd through the features:

* forward  : pg_eval_bound_energy - a_nlm, the features, the polynomial with
             the coefficients and E_i per atom (no pair gradients);
* backward : pg_eval_bound_run - a_nlm recomputed, the adjoint
             A_i = dE_i/da_nlm, the per-pair gradients g_p = Re(A_i . da/dd_p)
             and their gather into dE/dr (and the virial stress of the same
             pass), so that no derivative array per atom or pair is kept
             between the passes.

This is the reference's own evaluation order (PolymlpEval::eval_gtinv,
src/pypolymlp/cxx/src/compute/polymlp_eval.cpp:182-335: prod_sum = dE/da per
atom, then the pair loop), split into the two halves an autograd function
needs.  The structures are bound once (neighbour lists at cutoff + skin) and
later positions only refresh the lists' displacements (pg_eval_update), as a
molecular-dynamics caller such as calculator/utils/ase_calculator.py:63 needs.
"""

from __future__ import annotations

from typing import Optional, Sequence

import numpy as np

from . import _ffi
from .abi import Structures


def _torch():
    import torch

    return torch


class PolymlpPotential:
    """A polymlp (params dict, coefficients already divided by the scales, as
    in polymlp.yaml) bound to structures for repeated differentiable
    evaluation on the GPU.

    >>> pot = PolymlpPotential(params, coeffs)
    >>> pot.bind(axis, positions, types)          # (n_st, 3, 3), (sum N, 3), (sum N,)
    >>> r = torch.tensor(positions, requires_grad=True)
    >>> e = pot.energy(r)                          # (n_st,) float64
    >>> (f,) = torch.autograd.grad(-e.sum(), r)    # forces (sum N, 3)
    """

    def __init__(self, params_dict: dict, coeffs, precision: int = _ffi.PG_FP64, skin: float = 0.5):
        self.ev = _ffi.Evaluator(params_dict, coeffs, precision)
        self.skin = float(skin)
        self._n_atoms = None
        self._atom_st = None
        self.last_stress = None
        self.rebuilds = 0

    def bind(self, axis, positions, types, n_atoms: Optional[Sequence[int]] = None):
        """Bind structures: axis (n_st, 3, 3) with lattice vectors as columns,
        positions (sum N, 3) Cartesian, types (sum N,); n_atoms per structure
        (default: one structure)."""
        axis = np.asarray(axis, dtype=np.float64).reshape(-1, 3, 3)
        pos = np.asarray(positions, dtype=np.float64).reshape(-1, 3)
        types = np.asarray(types, dtype=np.int32).reshape(-1)
        n_atoms = [len(types)] if n_atoms is None else [int(n) for n in n_atoms]
        if sum(n_atoms) != len(types) or len(pos) != len(types) or len(axis) != len(n_atoms):
            raise ValueError("axis, positions, types and n_atoms disagree")
        offs = np.concatenate([[0], np.cumsum(n_atoms)])
        st = Structures(axis, [pos[offs[i]:offs[i + 1]] for i in range(len(n_atoms))],
                        [types[offs[i]:offs[i + 1]] for i in range(len(n_atoms))])
        self.ev.bind(st, self.skin)
        self._n_atoms = np.asarray(n_atoms)
        self._atom_st = np.repeat(np.arange(len(n_atoms)), n_atoms)
        self._pos = pos.copy()
        return self

    @property
    def n_structures(self) -> int:
        return len(self._n_atoms)

    def _set_positions(self, pos: np.ndarray):
        if self._n_atoms is None:
            raise RuntimeError("bind structures first")
        if not np.array_equal(pos, self._pos):
            if self.ev.update(pos):
                self.rebuilds += 1
            self._pos = pos.copy()

    def energy(self, positions):
        """E per structure (float64 tensor on the positions' device) as a
        differentiable function of positions (sum N x 3 tensor)."""
        return _EnergyFunction.apply(positions, self)

    def energy_forces_stress(self, positions=None):
        """(E (n_st,), forces (sum N, 3), stress (n_st, 6) in eV per cell, xx yy
        zz xy yz zx) as numpy arrays, in one pass."""
        if positions is not None:
            self._set_positions(np.asarray(positions, dtype=np.float64).reshape(-1, 3))
        return self.ev.bound_run()


class _EnergyFunction:
    """torch.autograd.Function over the evaluator (built lazily: torch is only
    needed by callers of PolymlpPotential.energy)."""

    _fn = None

    @classmethod
    def apply(cls, positions, pot):
        if cls._fn is None:
            torch = _torch()

            class Fn(torch.autograd.Function):
                @staticmethod
                def forward(ctx, r, pot_):
                    pos = r.detach().to("cpu", torch.float64).numpy().reshape(-1, 3)
                    pot_._set_positions(pos)
                    ctx.pot = pot_
                    ctx.pos = pos
                    ctx.shape, ctx.dtype = r.shape, r.dtype
                    return torch.as_tensor(pot_.ev.bound_energy(), dtype=torch.float64, device=r.device)

                @staticmethod
                def backward(ctx, grad_e):
                    pot_ = ctx.pot
                    pot_._set_positions(ctx.pos)
                    _, f, s = pot_.ev.bound_run()
                    pot_.last_stress = s
                    g = grad_e.detach().to("cpu", torch.float64).numpy()
                    # dE_s/dr_b = -F_b for the atoms b of structure s
                    grad_r = -f * g[pot_._atom_st][:, None]
                    return torch.as_tensor(grad_r.reshape(ctx.shape), dtype=ctx.dtype, device=grad_e.device), None

            cls._fn = Fn
        return cls._fn.apply(positions, pot)
