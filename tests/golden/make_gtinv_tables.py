"""Write the polynomial-invariant tables gtinv_v1.npz and gtinv_v2.npz.

The tables are the reference's invariant basis (version 1: orders 1-6,
version 2: orders 1-2), read in full through the reference's own reader
`Readgtinv` (src/pypolymlp/cxx/src/polymlp/polymlp_read_gtinv.cpp:12) built
under oracle/_ref from the reference's sources (make -C oracle ref; the
checkout is $PYPOLYMLP_REFERENCE, default /root/reference).  The tables are
written to pypolymlp_gb300/data/.
Asking for every order with an unbounded l_max returns every entry of the
reference's tables, in their order; `pypolymlp_gb300.gtinv` then screens them
by l_max as Readgtinv does.  The basis has to be the reference's: the
coefficients of a reference polymlp.yaml multiply these invariants.

Layout per order k (arrays named o{k}_...):
  l      (n_comb, k)  int8    l combination (ascending)
  n_m    (n_comb,)    int32   number of m combinations of each l combination
  m      (sum n_m, k) int8    m combinations, l combinations concatenated
  coef   (sum n_m,)   float64 coefficient of each m combination
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import ref  # noqa: E402

MAX_ORDER = {1: 6, 2: 2}


def tables(version):
    top = MAX_ORDER[version]
    l_comb, lm_seq, lm_coeffs = ref.readgtinv(top, [10**6] * (top - 1), version)
    out = {}
    for k in range(1, top + 1):
        idx = [i for i, lc in enumerate(l_comb) if len(lc) == k]
        ls = np.array([l_comb[i] for i in idx], dtype=np.int8).reshape(-1, k)
        n_m = np.array([len(lm_seq[i]) for i in idx], dtype=np.int32)
        m, coef = [], []
        for i in idx:
            lc = l_comb[i]
            for seq, c in zip(lm_seq[i], lm_coeffs[i]):
                m.append([lm - l * l - l for lm, l in zip(seq, lc)])
                coef.append(c)
        out[f"o{k}_l"] = ls
        out[f"o{k}_n_m"] = n_m
        out[f"o{k}_m"] = np.array(m, dtype=np.int8).reshape(-1, k)
        out[f"o{k}_coef"] = np.array(coef, dtype=np.float64)
    out["max_order"] = np.array(top, dtype=np.int32)
    return out


def main():
    for version in MAX_ORDER:
        path = os.path.join(REPO, "pypolymlp_gb300", "data", f"gtinv_v{version}.npz")
        np.savez_compressed(path, **tables(version))
        print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
