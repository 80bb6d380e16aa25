"""Property calculator front end: structures with element names in, E/F/S out.

`Properties` mirrors the reference's calculator class
(src/pypolymlp/calculator/properties.py:14-177) together with the two classes
it dispatches to (properties_single.py:18-157, properties_hybrid.py:13-78): it
is built from one or several model files (`pot`) or from params dicts and
coefficients, and for each model

  * a model over all its elements (type_full) renumbers the atom types of every
    structure by the model's element order (`replace_types`,
    src/pypolymlp/core/dataset_utils.py:11-46; for a spin model, whose element
    list repeats an element, the given types of that element's atoms are kept
    apart and renumbered consecutively);
  * a partial model sees only the atoms of its elements (`find_active_atoms`,
    calculator/utils/properties_utils.py:9-44); structures without such atoms
    contribute zero, forces of the other atoms are zero;

and the models' energies, forces and stresses are summed.  Forces are returned
as (3, n_atom) arrays, stresses (xx, yy, zz, xy, yz, zx) in eV per cell and,
through `stresses_gpa`, in GPa.  Every model is evaluated on the GPU by
`properties.PotentialPropertiesFast` (the adjoint evaluator); there is no CPU
path.  `load_poscar` reads a POSCAR as the reference's Poscar class does
(core/interface_vasp.py:371-430: coordinates taken as fractional).
"""

from __future__ import annotations

import re
from dataclasses import dataclass
from typing import Optional, Sequence, Union

import numpy as np

from pypolymlp_gb300 import _ffi
from pypolymlp_gb300 import properties as _properties
from pypolymlp_gb300.io_polymlp import load_mlp

EV_TO_GPA = 160.21766208


@dataclass
class PolymlpStructure:
    """axis (3, 3), lattice vectors as columns; positions (3, n_atom) fractional;
    n_atoms per element group; elements and types per atom."""

    axis: np.ndarray
    positions: np.ndarray
    n_atoms: Sequence[int]
    elements: Sequence[str]
    types: Sequence[int]
    volume: Optional[float] = None
    comment: Optional[str] = None
    name: Optional[str] = None

    def __post_init__(self):
        self.axis = np.asarray(self.axis, dtype=np.float64)
        self.positions = np.asarray(self.positions, dtype=np.float64)
        if self.volume is None:
            self.volume = float(np.linalg.det(self.axis))


def load_poscar(filename: str) -> PolymlpStructure:
    """POSCAR -> PolymlpStructure (types numbered by element group)."""
    with open(filename) as f:
        lines = f.read().splitlines()
    scale = float(lines[1].split()[0])
    axis = np.array([[float(v) for v in lines[k].split()[:3]] for k in (2, 3, 4)]).T * scale
    if re.search(r"[a-zA-Z]", lines[5]):
        names, n_atoms, row = lines[5].split(), [int(v) for v in lines[6].split()], 8
    else:
        names, n_atoms, row = list("ABCDEFGHIJKLMNOPQRSTUVWXYZ"), [int(v) for v in lines[5].split()], 7
    elements = [names[i] for i, n in enumerate(n_atoms) for _ in range(n)]
    types = [i for i, n in enumerate(n_atoms) for _ in range(n)]
    pos = np.array([[float(v) for v in lines[row + k].split()[:3]] for k in range(sum(n_atoms))]).T
    return PolymlpStructure(axis, pos.reshape(3, -1), n_atoms, elements, types, comment=lines[0], name=filename)


def replace_types(st: PolymlpStructure, element_order: Sequence[str]) -> np.ndarray:
    """Atom types of `st` in the numbering of a model with elements `element_order`."""
    elements = np.asarray(st.elements)
    given = np.asarray(st.types, dtype=np.int64)
    types = given.copy()
    count = 0
    if len(element_order) == len(set(element_order)):
        for t, ele in enumerate(element_order):
            match = elements == ele
            types[match] = t
            count += int(np.count_nonzero(match))
    else:
        # an element listed twice (spins): its atoms' given types map, in
        # increasing order, onto consecutive model types
        types = np.zeros_like(given)
        offset = 0
        for ele in dict.fromkeys(element_order):
            ids = np.nonzero(elements == ele)[0]
            count += len(ids)
            distinct = np.unique(given[ids])
            lookup = {int(v): offset + k for k, v in enumerate(distinct)}
            types[ids] = [lookup[int(v)] for v in given[ids]]
            offset += len(distinct)
    if count != len(elements):
        raise RuntimeError("Elements in structure not found in elements.")
    return types


def find_active_atoms(structures: Sequence[PolymlpStructure], element_order: Sequence[str]):
    """(structures of the atoms whose element is in `element_order`, typed in its
    order; their atom indices per kept structure; per structure, whether it kept any)."""
    if len(element_order) != len(set(element_order)):
        raise RuntimeError("Not available for system with spin configurations.")
    out, atoms_all, kept = [], [], []
    for st in structures:
        atoms = np.array([i for i, e in enumerate(st.elements) if e in element_order], dtype=np.int64)
        if len(atoms) == 0:
            kept.append(False)
            continue
        types = np.array([list(element_order).index(st.elements[i]) for i in atoms], dtype=np.int64)
        out.append(PolymlpStructure(st.axis, st.positions[:, atoms],
                                    [int(np.count_nonzero(types == t)) for t in range(len(element_order))],
                                    [st.elements[i] for i in atoms], types))
        atoms_all.append(atoms)
        kept.append(True)
    return out, atoms_all, kept


def convert_stresses_in_gpa(stresses, structures):
    """Stresses in eV per cell -> GPa (properties_utils.py:45-65)."""
    s = np.asarray(stresses, dtype=np.float64)
    if s.ndim == 1:
        vol = structures.volume if isinstance(structures, PolymlpStructure) else structures[0].volume
        return s * EV_TO_GPA / vol
    if s.ndim == 2:
        if len(structures) != s.shape[0]:
            raise ValueError("one structure per stress row")
        return s * EV_TO_GPA / np.array([st.volume for st in structures])[:, None]
    raise RuntimeError("Stress shape must be 1 or 2.")


class _Model:
    """One model's evaluator (PropertiesSingle of the reference)."""

    def __init__(self, params: dict, coeffs, precision: int):
        self.params = params
        self.coeffs = np.asarray(coeffs, dtype=np.float64)
        self.precision = precision
        self.prop = _properties.PotentialPropertiesFast(params, self.coeffs, precision)

    def eval_multiple(self, structures: Sequence[PolymlpStructure]):
        n_st = len(structures)
        energies = np.zeros(n_st)
        forces = [np.zeros((3, len(st.types))) for st in structures]
        stresses = np.zeros((n_st, 6))
        elements = list(self.params["elements"])
        if self.params.get("type_full", True) in (True, 1, None):
            calc = structures
            types = [replace_types(st, elements) for st in structures]
            atoms = [np.arange(len(st.types)) for st in structures]
            slots = list(range(n_st))
        else:
            calc, atoms, kept = find_active_atoms(structures, elements)
            types = [st.types for st in calc]
            slots = [s for s in range(n_st) if kept[s]]
        if not calc:
            return energies, forces, stresses
        self.prop.eval_multiple([st.axis for st in calc], [st.axis @ st.positions for st in calc], types)
        for q, s in enumerate(slots):
            energies[s] = self.prop.get_e_array()[q]
            forces[s][:, atoms[q]] = np.asarray(self.prop.get_f_array()[q]).T
            stresses[s] = self.prop.get_s_array()[q]
        return energies, forces, stresses


class Properties:
    """E/F/S of one model or the sum of several (a hybrid)."""

    def __init__(self, pot: Optional[Union[str, Sequence[str]]] = None,
                 params: Optional[Union[dict, Sequence[dict]]] = None, coeffs=None,
                 precision: int = _ffi.PG_FP64):
        if pot is not None:
            pots = [pot] if isinstance(pot, str) else list(pot)
            loaded = [load_mlp(p) for p in pots]
            self._pot = pot
        else:
            if params is None or coeffs is None:
                raise RuntimeError("Polymlp not provided.")
            if isinstance(params, dict):
                loaded = [(params, coeffs)]
            else:
                if len(params) != len(coeffs):
                    raise RuntimeError("Length of params and coeffs not consistent.")
                loaded = list(zip(params, coeffs))
            self._pot = "Coefficients"
        self._models = [_Model(p, c, precision) for p, c in loaded]
        self._e, self._f, self._s, self._structures = None, None, None, None

    def eval(self, st: PolymlpStructure, use_openmp: bool = True):
        """(energy, forces (3, n_atom), stress (6,)) of one structure."""
        e, f, s = self._sum([st])
        self._e, self._f, self._s = [float(e[0])], [f[0]], [s[0]]
        self._structures = [st]
        return float(e[0]), f[0], s[0]

    def eval_multiple(self, structures: Sequence[PolymlpStructure]):
        """(energies (n_st,), forces [(3, n_atom)], stresses (n_st, 6))."""
        self._e, self._f, self._s = self._sum(list(structures))
        self._structures = list(structures)
        return self._e, self._f, self._s

    def _sum(self, structures):
        energies, forces, stresses = self._models[0].eval_multiple(structures)
        for m in self._models[1:]:
            e, f, s = m.eval_multiple(structures)
            energies = energies + e
            forces = [a + b for a, b in zip(forces, f)]
            stresses = stresses + s
        return energies, forces, stresses

    def save(self, verbose: bool = False):
        """polymlp_energies.npy, polymlp_stress_tensors.npy (GPa) and
        polymlp_forces.npy (or one file per structure when their sizes differ)."""
        np.save("polymlp_energies.npy", self.energies)
        np.save("polymlp_stress_tensors.npy", self.stresses_gpa)
        if len({f.shape for f in self.forces}) == 1:
            np.save("polymlp_forces.npy", np.array(self.forces))
        else:
            for i, f in enumerate(self.forces):
                np.save("polymlp_forces_" + str(i + 1).zfill(5) + ".npy", f)
        if len(self.forces) == 1:
            np.savetxt("polymlp_energies.dat", self.energies, fmt="%f")
        if verbose:
            print("polymlp_energies.npy, polymlp_forces*.npy,", "and polymlp_stress_tensors.npy are generated.",
                  flush=True)
        return self

    def print_single(self):
        np.set_printoptions(suppress=True)
        print("Energy:", self.energies[0], "(eV/cell)", flush=True)
        print("Forces (eV/ang):", flush=True)
        for i, f in enumerate(self.forces[0].T):
            print("- atom", i, ":", f, flush=True)
        for label, s in (("eV/cell", self.stresses[0]), ("GPa", self.stresses_gpa[0])):
            print(f"Stress tensors ({label}):", flush=True)
            print("- xx, yy, zz:", s[0:3], flush=True)
            print("- xy, yz, zx:", s[3:6], flush=True)
        print("---------", flush=True)
        return self

    @property
    def elements(self):
        return self._models[0].params["elements"]

    @property
    def params(self):
        ps = [m.params for m in self._models]
        return ps[0] if len(ps) == 1 else ps

    @property
    def pot(self):
        return self._pot

    @property
    def energies(self):
        return self._e

    @property
    def forces(self):
        return self._f

    @property
    def stresses(self):
        return self._s

    @property
    def stresses_gpa(self):
        return convert_stresses_in_gpa(self._s, self._structures)
