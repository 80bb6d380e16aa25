"""Polynomial-invariant tables (l combinations, m combinations, coefficients).

`Readgtinv` mirrors the reference's class of the same name
(src/pypolymlp/cxx/src/polymlp/polymlp_read_gtinv.cpp:12-57) and
`get_gtinv_attrs` its Python wrapper (src/pypolymlp/cxx/wrapper/api_gtinv_list.py:6):
for each order k = 1..order the invariants of that order whose largest l is at
most l_max[k-2] (0 for k = 1) are kept, in table order; the m combination of
each term is returned as lm indices l*l + l + m.  The tables themselves are the
reference's invariant basis (version 1: orders 1-6, version 2: orders 1-2),
stored in data/gtinv_v{version}.npz (written by tests/golden/make_gtinv_tables.py;
the layout is described there).  Errors follow polymlp_gtinv_data.cpp:34-40: an
order above the version's largest table or an unknown version raise
ValueError; a missing table raises RuntimeError.
"""

from __future__ import annotations

import functools
import os
from typing import Sequence

import numpy as np

_DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")


@functools.lru_cache(maxsize=None)
def _tables(version: int):
    if version not in (1, 2):
        raise ValueError("Invalid version")
    path = os.path.join(_DATA, f"gtinv_v{version}.npz")
    if not os.path.exists(path):
        raise RuntimeError(f"gtinv table not found: {path}")
    with np.load(path) as z:
        return {k: z[k] for k in z.files}


def _screen(order: int, maxl: int, version: int):
    t = _tables(version)
    if order > int(t["max_order"]):
        if order > 6:
            raise ValueError("Invalid order")
        raise RuntimeError(f"no version-{version} gtinv table of order {order}")
    ls, n_m, ms, cs = (t[f"o{order}_{k}"].astype(np.int64) if k != "coef" else t[f"o{order}_coef"]
                       for k in ("l", "n_m", "m", "coef"))
    starts = np.concatenate([[0], np.cumsum(n_m)])
    l_comb, lm_seq, lm_coeffs = [], [], []
    for i in np.nonzero(ls[:, -1] <= maxl)[0]:
        lc = ls[i]
        rows = slice(starts[i], starts[i + 1])
        l_comb.append(lc.tolist())
        lm_seq.append((lc * lc + lc + ms[rows]).tolist())
        lm_coeffs.append(cs[rows].tolist())
    return l_comb, lm_seq, lm_coeffs


class Readgtinv:
    """Invariants up to `gtinv_order` with l_max per order `gtinv_maxl`
    ([l_max of order 2, of order 3, ...])."""

    def __init__(self, gtinv_order: int, gtinv_maxl: Sequence[int], version: int = 1):
        if gtinv_order > 6:
            raise ValueError("Invalid order")
        maxl = [int(v) for v in gtinv_maxl]
        if len(maxl) < gtinv_order - 1:
            raise ValueError(f"gtinv_maxl needs {gtinv_order - 1} values, got {len(maxl)}")
        self._l, self._lm, self._c = [], [], []
        for k in range(1, gtinv_order + 1):
            lc, lm, c = _screen(k, 0 if k == 1 else maxl[k - 2], version)
            self._l += lc
            self._lm += lm
            self._c += c

    def get_lm_seq(self) -> list:
        return self._lm

    def get_l_comb(self) -> list:
        return self._l

    def get_lm_coeffs(self) -> list:
        return self._c


def get_gtinv_attrs(order: int, lmax: Sequence[int], version: int = 1):
    """(l_comb, lm_seq, lm_coeffs) of the invariants up to `order`."""
    r = Readgtinv(order, lmax, version)
    return r.get_l_comb(), r.get_lm_seq(), r.get_lm_coeffs()
