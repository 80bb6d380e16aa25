"""ASE calculator over the GPU evaluator.

`PolymlpASECalculator` mirrors the reference's calculator of the same name
(src/pypolymlp/calculator/utils/ase_calculator.py:13-75): each `calculate`
converts the atoms to a structure as `ase_atoms_to_structure` does
(calculator/utils/ase_utils.py:42-57: lattice vectors as columns, scaled
positions, element names per atom) and stores the model's energy (eV), forces
(n_atom, 3) in eV/angstrom and stress (xx, yy, zz, xy, yz, zx in eV per cell,
as the reference stores it) in `results`.  With ASE importable the class is an
`ase.calculators.calculator.Calculator`; without it (ASE is not installed in
every environment) it is a plain class with the same `calculate`, `results`
and `get_potential_energy` / `get_forces` / `get_stress` for any object that
offers ASE's Atoms accessors (`cell`, `get_scaled_positions`,
`get_chemical_symbols`, `get_volume`).

Repeated calls on the same atoms (a molecular-dynamics or relaxation loop)
keep the GPU evaluator's neighbour lists: for a single model over all atoms
the calculator binds the atoms once (lists built at cutoff + `skin`) and later
calls only move them (`torch_potential.PolymlpPotential`), rebuilding when
the cell, the elements or their order change or an atom has moved more than
skin / 2.  Hybrid and partial models take the per-call path.
"""

from __future__ import annotations

from collections import Counter
from typing import Optional

import numpy as np

from pypolymlp_gb300.calculator import PolymlpStructure, Properties, replace_types

try:  # ASE is optional
    from ase.calculators.calculator import Calculator as _Base
    from ase.calculators.calculator import all_changes as _all_changes

    ALL_CHANGES = tuple(_all_changes)
except ImportError:
    _Base = object
    ALL_CHANGES = ("positions", "numbers", "cell", "pbc")


def ase_atoms_to_structure(atoms) -> PolymlpStructure:
    elements = list(atoms.get_chemical_symbols())
    unique = sorted(set(elements), key=elements.index)
    counts = Counter(elements)
    n_atoms = [counts[e] for e in unique]
    types = [i for i, n in enumerate(n_atoms) for _ in range(n)]
    return PolymlpStructure(np.asarray(atoms.cell, dtype=np.float64).T,
                            np.asarray(atoms.get_scaled_positions(), dtype=np.float64).T, n_atoms, elements, types,
                            float(atoms.get_volume()))


class PolymlpASECalculator(_Base):
    implemented_properties = ("energy", "forces", "stress")

    def __init__(self, pot=None, params=None, coeffs=None, properties: Optional[Properties] = None,
                 require_mlp: bool = True, skin: float = 0.5, reuse_neighbors: bool = True, **kwargs):
        if _Base is not object:
            super().__init__(**kwargs)
        else:
            self.results = {}
            self.atoms = None
        self._prop = None
        self._skin = float(skin)
        self._reuse = bool(reuse_neighbors)
        self._bound = None      # (PolymlpPotential, key of the bound atoms)
        if properties is not None:
            self._prop = properties
        elif pot is not None or (params is not None and coeffs is not None):
            self._prop = Properties(pot=pot, params=params, coeffs=coeffs)
        elif require_mlp:
            raise RuntimeError("Polymlp not provided.")

    def set_calculator(self, pot=None, params=None, coeffs=None):
        self._prop = Properties(pot=pot, params=params, coeffs=coeffs)
        self._bound = None

    def _single_model(self):
        ms = getattr(self._prop, "_models", None)
        if not self._reuse or not ms or len(ms) != 1:
            return None
        m = ms[0]
        return m if m.params.get("type_full", True) in (True, 1, None) else None

    def _bound_eval(self, model, st: PolymlpStructure, atoms):
        """E, forces (3, n), stress (6,) through a bound PolymlpPotential."""
        from pypolymlp_gb300.torch_potential import PolymlpPotential

        cart = (np.asarray(atoms.get_positions(), dtype=np.float64) if hasattr(atoms, "get_positions")
                else (st.axis @ st.positions).T)
        key = (np.asarray(st.axis).tobytes(), tuple(st.elements))
        if self._bound is None or self._bound[1] != key:
            pot = PolymlpPotential(model.params, model.coeffs, model.precision, skin=self._skin)
            pot.bind(st.axis, cart, replace_types(st, list(model.params["elements"])))
            self._bound = (pot, key)
        e, f, s = self._bound[0].energy_forces_stress(cart)
        return float(e[0]), f.T, s[0]

    def calculate(self, atoms=None, properties=("energy", "forces", "stress"), system_changes=ALL_CHANGES):
        if _Base is not object:
            super().calculate(atoms, properties, system_changes)
        else:
            self.atoms = atoms
        if self._prop is None:
            raise RuntimeError("Polymlp not provided.")
        st = ase_atoms_to_structure(self.atoms)
        model = self._single_model()
        if model is not None:
            energy, forces, stress = self._bound_eval(model, st, self.atoms)
        else:
            energy, forces, stress = self._prop.eval(st)
        self.results["energy"] = energy
        self.results["forces"] = forces.T
        self.results["stress"] = stress

    if _Base is object:
        def get_potential_energy(self, atoms=None):
            self.calculate(atoms)
            return self.results["energy"]

        def get_forces(self, atoms=None):
            self.calculate(atoms)
            return self.results["forces"]

        def get_stress(self, atoms=None):
            self.calculate(atoms)
            return self.results["stress"]
