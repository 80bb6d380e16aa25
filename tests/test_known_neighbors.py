"""Known answers of the reference's neighbour-list tests
(tests/test_cxx/test_neighbor.py, test_neighbor_variants.py: full and half
lists of rocksalt MgO and a 30-atom BiGd2 cell at a 6 angstrom cutoff, and the
number of lattice translations NeighborCell searches at 6, 8 and 16 angstrom;
structures and asserted values copied by tests/golden/make_known_answers.py).
The oracle's neighbour list, which the GPU lists match bit for bit, must
reproduce every asserted count, index sum, distance sum and difference vector,
with the reference test's comparisons (pytest.approx, np.isclose)."""

import json
import os

import numpy as np
import pytest

from pypolymlp_gb300.abi import Structures

KA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "known_answers")


def _cases():
    with open(os.path.join(KA, "known_neighbors.json")) as f:
        return json.load(f)["cases"]


def _structure(name):
    """Structures of one POSCAR, types in the file's element order."""
    from test_known_answers import read_poscar

    path = os.path.join(KA, name)
    elements = open(path).read().splitlines()[5].split()
    axis, pos, types = read_poscar(path, elements)
    return Structures([axis], [pos], [types]), types


def _lists(st, types, cutoff, half):
    """{distances, differences, neighbor_atoms} laid out as the reference's
    Neighbor classes return them: per atom, per neighbour type for the full
    list, one array per atom for the half list."""
    from oracle import oracle

    offs, nb, d = oracle.neighbor_list(st, 0, cutoff, half)
    n_type = int(types.max()) + 1
    out = {"distances": [], "differences": [], "neighbor_atoms": []}
    for i in range(len(types)):
        j, dv = nb[offs[i]:offs[i + 1]], d[offs[i]:offs[i + 1]]
        if half:
            groups = [(j, dv)]
        else:
            groups = [(j[types[j] == t], dv[types[j] == t]) for t in range(n_type)]
        dist = [np.linalg.norm(g[1], axis=1) for g in groups]
        out["distances"].append(dist[0] if half else dist)
        out["differences"].append(groups[0][1] if half else [g[1] for g in groups])
        out["neighbor_atoms"].append(groups[0][0] if half else [g[0] for g in groups])
    return out


def _value(obj, check):
    for k in check["idx"]:
        obj = obj[k]
    op = check["op"]
    if op == "len":
        return len(obj)
    if op == "sum":
        return float(np.sum(obj))
    if op == "sumsq":
        return float(np.sum(np.square(obj)))
    if op == "count_close":
        return int(np.count_nonzero(np.isclose(obj, check["arg"])))
    if op == "shape":
        return list(np.asarray(obj).shape)
    if op == "item":
        return float(obj)
    raise ValueError(op)


@pytest.mark.parametrize("name", sorted(_cases()))
def test_oracle_neighbors_reproduce_reference_known_answers(name):
    from oracle import oracle

    case = _cases()[name]
    st, types = _structure(case["structure"])
    lists = {}
    for c in case["checks"]:
        if c["attr"] == "translations":
            got = len(oracle.translations(st, 0, c["cutoff"])[0])
        else:
            key = (c["ctor"] == "NeighborHalf", c["cutoff"])
            if key not in lists:
                lists[key] = _lists(st, types, c["cutoff"], key[0])
            got = _value(lists[key][c["attr"]], c)
        want = pytest.approx(c["expect"]) if c["approx"] else c["expect"]
        assert got == want, (c, got)
