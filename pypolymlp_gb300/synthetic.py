"""Seeded synthetic structures and Morse labels for the benchmark workloads.

The reference publishes no dataset for this path, so every workload is a
seeded synthetic set with the shapes and distributions below:

* ``fcc_set``        : fcc 2x2x2 (32 atoms, a = 4.0 A), isotropic strain
                       U(0.95, 1.05), displacements N(0, 0.1 A), one element.
* ``binary_set``     : bcc or fcc conventional cells repeated to 64..128
                       atoms, a ~ U(2.8, 4.2) A, displacements N(0, 0.15 A),
                       species B with probability p ~ U(0, 1) per structure.
* ``ternary_set``    : N = round(exp(U(ln 8, ln 256))) (or uniform-int in a
                       given range), random lower-triangular cells with
                       volume N * U(15, 22) A^3 and shortest lattice vector
                       >= 2 A, fractional positions U(0, 1) with a 1.5 A
                       minimum distance (bounded retries), displacements
                       N(0, 0.2 A), three species.
* ``bcc_supercell``  : bcc n x n x n (2 n^3 atoms), a = 3.2 A, displacements
                       N(0, 0.1 A), species 50/50.

Labels come from a Morse pair potential
E = sum_{i<j, r<rc} D_ab (exp(-2 alpha (r - r0)) - 2 exp(-alpha (r - r0))),
forces F = -dE/dr, and stress in the reference's convention (eV per cell,
sum over pairs of (r_i - r_j)_a F_b, order xx, yy, zz, xy, yz, zx).
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np


@dataclass
class StructureSet:
    axis: List[np.ndarray] = field(default_factory=list)       # (3, 3), lattice vectors as columns
    positions: List[np.ndarray] = field(default_factory=list)  # (N, 3) Cartesian
    types: List[np.ndarray] = field(default_factory=list)      # (N,)
    energies: Optional[np.ndarray] = None
    forces: Optional[List[np.ndarray]] = None                  # (N, 3) each
    stresses: Optional[np.ndarray] = None                      # (n_st, 6), eV / cell

    def __len__(self):
        return len(self.types)

    @property
    def n_atoms(self):
        return np.array([len(t) for t in self.types], dtype=np.int64)

    def subset(self, idx):
        idx = list(idx)
        s = StructureSet([self.axis[i] for i in idx], [self.positions[i] for i in idx],
                         [self.types[i] for i in idx])
        if self.energies is not None:
            s.energies = self.energies[idx]
            s.forces = [self.forces[i] for i in idx]
            s.stresses = self.stresses[idx]
        return s


_FCC = np.array([[0, 0, 0], [0, 0.5, 0.5], [0.5, 0, 0.5], [0.5, 0.5, 0]], dtype=float)
_BCC = np.array([[0, 0, 0], [0.5, 0.5, 0.5]], dtype=float)


def _supercell(basis, reps, a):
    n1, n2, n3 = reps
    grid = np.array([[i, j, k] for i in range(n1) for j in range(n2) for k in range(n3)], dtype=float)
    cells = (grid[:, None, :] + basis[None, :, :]).reshape(-1, 3)  # in conventional-cell units
    axis = np.diag([n1 * a, n2 * a, n3 * a]).astype(float)
    return axis, cells * a


def fcc_set(n_struct=200, seed=1):
    rng = np.random.default_rng(seed)
    out = StructureSet()
    for _ in range(n_struct):
        axis, pos = _supercell(_FCC, (2, 2, 2), 4.0)
        s = rng.uniform(0.95, 1.05)
        axis = axis * s
        pos = pos * s + rng.normal(0.0, 0.1, pos.shape)
        out.axis.append(axis)
        out.positions.append(pos)
        out.types.append(np.zeros(len(pos), dtype=np.int32))
    return out


def _repeat_choices(n_basis, lo, hi):
    out = []
    for n1 in range(1, 9):
        for n2 in range(1, 9):
            for n3 in range(1, 9):
                if lo <= n_basis * n1 * n2 * n3 <= hi:
                    out.append((n1, n2, n3))
    return out


def binary_set(n_struct=5000, seed=2, n_min=64, n_max=128):
    rng = np.random.default_rng(seed)
    reps = {"bcc": _repeat_choices(2, n_min, n_max), "fcc": _repeat_choices(4, n_min, n_max)}
    out = StructureSet()
    for _ in range(n_struct):
        lat = "bcc" if rng.random() < 0.5 else "fcc"
        basis = _BCC if lat == "bcc" else _FCC
        choices = reps[lat]
        r = choices[rng.integers(len(choices))]
        a = rng.uniform(2.8, 4.2)
        axis, pos = _supercell(basis, r, a)
        pos = pos + rng.normal(0.0, 0.15, pos.shape)
        p = rng.random()
        types = (rng.random(len(pos)) < p).astype(np.int32)
        out.axis.append(axis)
        out.positions.append(pos)
        out.types.append(types)
    return out


def _min_dist_ok(frac, axis, dmin):
    """Whether every pair (minimum image) is at least dmin apart.  Atoms are
    added one at a time and the check stops at the first close pair: random
    cells of this family almost always have one, early."""
    n = len(frac)
    if n < 2:
        return True
    cart = frac @ axis.T
    inv_t = np.linalg.inv(axis).T
    for k in range(1, n):
        d = cart[:k] - cart[k]
        f = d @ inv_t
        f -= np.round(f)
        d = f @ axis.T
        if np.einsum("ij,ij->i", d, d).min() < dmin * dmin:
            return False
    return True


def ternary_set(n_struct=20000, seed=3, n_range=None, n_types=3, sigma=0.2):
    rng = np.random.default_rng(seed)
    out = StructureSet()
    for _ in range(n_struct):
        if n_range is None:
            n = int(round(math.exp(rng.uniform(math.log(8), math.log(256)))))
        else:
            n = int(rng.integers(n_range[0], n_range[1] + 1))
        vol = n * rng.uniform(15.0, 22.0)
        for _attempt in range(50):
            diag = rng.uniform(0.7, 1.3, 3)
            shear = rng.uniform(-0.3, 0.3, 3)
            L = np.array([[diag[0], 0, 0], [shear[0], diag[1], 0], [shear[1], shear[2], diag[2]]])
            axis = L.T  # columns are lattice vectors
            axis = axis * (vol / abs(np.linalg.det(axis))) ** (1 / 3)
            if np.linalg.norm(axis, axis=0).min() >= 2.0:
                break
        frac = None
        for _attempt in range(20):
            trial = rng.random((n, 3))
            if _min_dist_ok(trial, axis, 1.5):
                frac = trial
                break
        if frac is None:
            # lattice-seeded variant: points on a regular grid with jitter
            m = int(math.ceil(n ** (1 / 3)))
            g = np.array([[i, j, k] for i in range(m) for j in range(m) for k in range(m)], dtype=float)[:n]
            frac = (g + 0.5) / m + rng.normal(0, 0.02, (n, 3))
        pos = frac @ axis.T + rng.normal(0.0, sigma, (n, 3))
        out.axis.append(axis)
        out.positions.append(pos)
        out.types.append(rng.integers(0, n_types, n).astype(np.int32))
    return out


def bcc_supercell(n_rep, seed=4, a=3.2, sigma=0.1):
    rng = np.random.default_rng(seed)
    axis, pos = _supercell(_BCC, (n_rep, n_rep, n_rep), a)
    pos = pos + rng.normal(0.0, sigma, pos.shape)
    types = (rng.random(len(pos)) < 0.5).astype(np.int32)
    out = StructureSet()
    out.axis.append(axis)
    out.positions.append(pos)
    out.types.append(types)
    return out


def _translations(axis, rc):
    inv = np.linalg.inv(axis)
    h = 1.0 / np.linalg.norm(inv, axis=1)  # interplanar spacings
    m = np.ceil(rc / h).astype(int) + 1
    g = np.array([[i, j, k] for i in range(-m[0], m[0] + 1) for j in range(-m[1], m[1] + 1)
                  for k in range(-m[2], m[2] + 1)], dtype=float)
    return g @ axis.T


def morse_labels(sset: StructureSet, D, alpha=1.5, r0=2.85, rc=7.0, device=None):
    """Morse energies, forces and stresses for every structure (in place)."""
    import torch

    dev = torch.device(device) if device is not None else torch.device("cpu")
    Dm = torch.tensor(np.asarray(D, dtype=np.float64), device=dev)
    energies = np.zeros(len(sset))
    forces, stresses = [], np.zeros((len(sset), 6))
    for s in range(len(sset)):
        pos = torch.tensor(sset.positions[s], dtype=torch.float64, device=dev)
        typ = torch.tensor(sset.types[s], dtype=torch.int64, device=dev)
        tr = torch.tensor(_translations(sset.axis[s], rc), dtype=torch.float64, device=dev)
        n = pos.shape[0]
        # d[i, j, t] = r_i - r_j - t (vector from the image of j to i)
        d = pos[:, None, None, :] - pos[None, :, None, :] - tr[None, None, :, :]
        r = torch.linalg.norm(d, dim=-1)
        mask = (r < rc) & (r > 1e-8)
        rr = torch.where(mask, r, torch.full_like(r, rc))
        Dij = Dm[typ[:, None], typ[None, :]][:, :, None]
        ex = torch.exp(-alpha * (rr - r0))
        v = Dij * (ex * ex - 2.0 * ex)
        dv = Dij * (-2.0 * alpha * ex * ex + 2.0 * alpha * ex)
        v = torch.where(mask, v, torch.zeros_like(v))
        dv = torch.where(mask, dv, torch.zeros_like(dv))
        e = 0.5 * v.sum()
        # force on i: -sum_j,t V'(r) (r_i - r_j - t) / r
        g = (dv / rr)[..., None] * d
        f = -g.sum(dim=(1, 2))
        # stress: sum over pairs (each once) of d_a F_i,b = -0.5 sum_ijt V'/r d_a d_b
        sig = -0.5 * torch.einsum("ijt,ijta,ijtb->ab", dv / rr, d, d)
        energies[s] = float(e)
        forces.append(f.cpu().numpy())
        sg = sig.cpu().numpy()
        stresses[s] = [sg[0, 0], sg[1, 1], sg[2, 2], sg[0, 1], sg[1, 2], sg[2, 0]]
        del n
    sset.energies = energies
    sset.forces = forces
    sset.stresses = stresses
    return sset


def morse_D(n_types):
    """Per-pair well depths: 1 type 0.5; 2 types AA/BB/AB 0.4/0.6/0.5; 3 types
    0.4/0.5/0.6 on the diagonal and 0.5 off it."""
    if n_types == 1:
        return np.array([[0.5]])
    if n_types == 2:
        return np.array([[0.4, 0.5], [0.5, 0.6]])
    D = np.full((n_types, n_types), 0.5)
    for i, v in enumerate([0.4, 0.5, 0.6][:n_types]):
        D[i, i] = v
    return D
