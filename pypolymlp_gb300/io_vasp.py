"""VASP vasprun.xml datasets for the fit.

`Vasprun` and `VasprunMD` read what the reference's classes of the same names
read (src/pypolymlp/core/interface_vasp.py:108-345): from a single-point run
the energy without entropy (the second entry of the first calculation's energy
block), forces (3, n_atom) in eV/angstrom, the stress tensor in kbar and the
final structure (lattice vectors as columns, fractional positions, element and
type per atom); from an MD run (IBRION = 0) the same per ionic step.
`parse_properties_from_vaspruns` (interface_vasp.py:38-76) reads many files,
skips single-point runs that cannot be read or whose electronic steps did not
converge (last two e_0 energies 1e-3 eV or more apart, interface_vasp.py:516-532),
and returns the stresses in eV per cell (kbar x volume / 1602.1766208).
`split_ids_train_test` is the reference's split (core/utils.py:18-27): test
structures evenly spaced over the list.
"""

from __future__ import annotations

import xml.etree.ElementTree as ET
from typing import Sequence

import numpy as np

from pypolymlp_gb300.calculator import PolymlpStructure

EV_TO_KBAR = 1602.1766208


def _array(varray) -> np.ndarray:
    return np.array([[float(x) for x in v.text.split()] for v in varray])


def _rc_set(rcs):
    return [[c.text.replace(" ", "") for c in rc.findall("c")] for rc in rcs]


def _atoms(root):
    n_atoms = [int(r[0]) for r in _rc_set(root.findall(".//*[@name='atomtypes']/set/rc"))]
    rows = _rc_set(root.findall(".//*[@name='atoms']/set/rc"))
    elements = ["Zr" if r[0] == "r" else r[0] for r in rows]  # VASP truncates "Zr" to "r"
    types = [int(r[1]) - 1 for r in rows]
    return n_atoms, elements, types


def is_md(root) -> bool:
    tag = root.find(".//*[@name='IBRION']")
    try:
        return int(tag.text) == 0
    except (AttributeError, TypeError, ValueError):
        return False


class Vasprun:
    """A single-point vasprun.xml."""

    def __init__(self, name: str, root=None):
        self._root = ET.parse(name).getroot() if root is None else root
        self._calc = self._root.find("calculation")
        self._name = name

    @property
    def energy(self) -> float:
        return float(self._calc.find("energy")[1].text)

    @property
    def forces(self) -> np.ndarray:
        return _array(self._root.find(".//*[@name='forces']")).T

    @property
    def stress(self) -> np.ndarray:
        """(3, 3) in kbar."""
        return _array(self._root.find(".//*[@name='stress']"))

    @property
    def structure(self) -> PolymlpStructure:
        st = self._root.find(".//*[@name='finalpos']")
        n_atoms, elements, types = _atoms(self._root)
        return PolymlpStructure(_array(st.find(".//*[@name='basis']")).T,
                                _array(st.find(".//*[@name='positions']")).T, n_atoms, elements, types,
                                float(st.find(".//*[@name='volume']").text), name=self._name)

    def get_scstep(self) -> np.ndarray:
        return np.array([float(sc.find("energy").find(".//*[@name='e_0_energy']").text)
                         for sc in self._calc.findall("scstep")])


class VasprunMD:
    """A molecular-dynamics vasprun.xml: one structure per ionic step."""

    def __init__(self, name: str, root=None):
        self._root = ET.parse(name).getroot() if root is None else root
        self._calcs = self._root.findall("calculation")
        self._name = name

    @property
    def energies(self) -> np.ndarray:
        return np.array([float(c.find("energy")[1].text) for c in self._calcs])

    @property
    def forces(self) -> list:
        return [_array(c.find(".//*[@name='forces']")).T for c in self._calcs]

    @property
    def stresses(self) -> np.ndarray:
        return np.array([_array(c.find(".//*[@name='stress']")) for c in self._calcs])

    @property
    def structures(self) -> list:
        n_atoms, elements, types = _atoms(self._root)
        return [PolymlpStructure(_array(c.find(".//*[@name='basis']")).T, _array(c.find(".//*[@name='positions']")).T,
                                 n_atoms, elements, types, float(c.find(".//*[@name='volume']").text),
                                 name=self._name) for c in self._calcs]


def is_convergent(v: Vasprun, tol: float = 1e-3) -> bool:
    try:
        e = v.get_scstep()
        return bool(abs(e[-1] - e[-2]) < tol)
    except (AttributeError, IndexError, TypeError, ValueError):
        return True


def parse_properties_from_vaspruns(files: Sequence[str], verbose: bool = False):
    """(structures, (energies (n,), forces [(3, n_atom)], stresses (n, 3, 3) in eV per cell))."""
    structures, energies, forces, stresses = [], [], [], []
    for name in files:
        root = ET.parse(name).getroot()
        if is_md(root):
            v = VasprunMD(name, root)
            sts = v.structures
            structures += sts
            energies += list(v.energies)
            forces += v.forces
            stresses += [s * st.volume / EV_TO_KBAR for s, st in zip(v.stresses, sts)]
            continue
        try:
            v = Vasprun(name, root)
            st, e, f, s = v.structure, v.energy, v.forces, v.stress
        except (AttributeError, IndexError, TypeError, ValueError):
            if verbose:
                print("- Not readable:", name, flush=True)
            continue
        if not is_convergent(v):
            if verbose:
                print("- Not convergent:", name, flush=True)
            continue
        structures.append(st)
        energies.append(e)
        forces.append(f)
        stresses.append(s * st.volume / EV_TO_KBAR)
    return structures, (np.array(energies), forces, np.array(stresses))


def split_ids_train_test(n_data: int, train_ratio: float = 0.9):
    n_train = round(n_data * train_ratio)
    test_ids = np.round(np.linspace(0, n_data - 1, num=n_data - n_train)).astype(int)
    train = np.ones(n_data, dtype=bool)
    train[test_ids] = False
    return np.nonzero(train)[0], test_ids


def split_train_test(items: Sequence, train_ratio: float = 0.9):
    train_ids, test_ids = split_ids_train_test(len(items), train_ratio)
    return [items[i] for i in train_ids], [items[i] for i in test_ids]
