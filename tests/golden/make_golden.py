"""Generate the golden fixtures of tests/golden/ from the reference.

Run where the reference sources are available (they are compiled into
oracle/_ref by `make -C oracle ref`):

    python tests/golden/make_golden.py

Writes
  gtinv/gtinv_v1_order{o}_maxl{...}.json   the reference's invariant tables
                                           (Readgtinv) for the benchmark configs
  x_*.npz                                  signatures of the X rows computed by the
                                           reference's own C++ (Model::run via the
                                           PotentialModel glue): column sums, row
                                           sums, X @ R for a seeded Gaussian R
                                           (F x 16) and 4096 sampled elements
  eval_*.npz                               E/F/S from PotentialPropertiesFast glue
All inputs are seeded synthetic structures (pypolymlp_gb300.synthetic).
"""

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import ref  # noqa: E402
from pypolymlp_gb300 import synthetic as syn  # noqa: E402
from pypolymlp_gb300.abi import Structures, row_layout  # noqa: E402
from pypolymlp_gb300.params import make_params_dict, to_json  # noqa: E402

def gtinv_file(order, maxl, version=1):
    """Fixture path of the reference's Readgtinv output for (order, l_max per order)."""
    tag = "_".join(str(int(v)) for v in list(maxl)[: max(order - 1, 0)])
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "gtinv",
                        f"gtinv_v{version}_order{order}_maxl{tag}.json")


CONFIGS = {
    "cfg1": dict(n_type=1, cutoff=6.0, model_type=2, max_p=2, gaussian_params2=(0.0, 5.0, 8), gtinv_order=2,
                 gtinv_maxl=(4,)),
    "cfg2": dict(n_type=2, cutoff=7.0, model_type=3, max_p=2, gaussian_params2=(0.0, 5.0, 10), gtinv_order=3,
                 gtinv_maxl=(8, 4)),
    "cfg3": dict(n_type=3, cutoff=6.0, model_type=3, max_p=2, gaussian_params2=(0.0, 5.0, 8), gtinv_order=3,
                 gtinv_maxl=(6, 4)),
    "cfg5p": dict(n_type=3, cutoff=8.0, model_type=3, max_p=2, gaussian_params2=(0.0, 5.0, 4), gtinv_order=4,
                  gtinv_maxl=(8, 8, 2)),
}


# extra invariant tables used by the tests (small models)
EXTRA_GTINV = [(2, (2,)), (3, (4, 2)), (3, (6, 2)), (4, (4, 2, 1))]


def write_gtinv():
    tabs = [(c["gtinv_order"], c["gtinv_maxl"]) for c in CONFIGS.values()] + EXTRA_GTINV
    for order, maxl in tabs:
        l_comb, lm_seq, lm_coeffs = ref.readgtinv(order, maxl)
        path = gtinv_file(order, maxl)
        c = {"gtinv_order": order, "gtinv_maxl": maxl}
        with open(path, "w") as f:
            json.dump({"order": c["gtinv_order"], "maxl": list(c["gtinv_maxl"]), "version": 1,
                       "l_comb": l_comb, "lm_seq": lm_seq, "lm_coeffs": lm_coeffs}, f, separators=(",", ":"))
        print("wrote", path)


def params(name, **over):
    c = dict(CONFIGS[name])
    c.update(over)
    return make_params_dict(**c)


def write_x(name, p, sset, tag):
    st = Structures(sset.axis, sset.positions, sset.types)
    force = [True] * st.n_st
    e, f, s, n = row_layout(st.n_atoms, force)
    x = ref.features_x(p, st, e, f, s, n)
    sig = x_signature(x)
    np.savez_compressed(os.path.join(HERE, f"x_{tag}.npz"), params=to_json(p), axis=st.axis, positions=st.positions,
                        types=st.types, n_atoms=st.n_atoms, shape=np.array(x.shape), **sig)
    print("wrote", tag, x.shape)


def x_signature(x, seed=12345, n_proj=16, n_sample=4096):
    """Compact, size-independent fingerprint of X (shared with the tests)."""
    rng = np.random.default_rng(seed)
    R = rng.standard_normal((x.shape[1], n_proj))
    idx = rng.integers(0, x.size, n_sample)
    return {"colsum": x.sum(axis=0), "rowsum": x.sum(axis=1), "proj": x @ R, "sample_idx": idx,
            "sample": x.reshape(-1, order="F")[idx], "colmax": np.abs(x).max(axis=0)}


def write_potential_model(p, sets, force_dataset, tag):
    """X of several datasets with mixed force flags in PotentialModel's row
    layout (PyModel::set_index), computed by the reference build."""
    from pypolymlp_gb300.abi import row_layout_datasets

    axis, pos, types = [], [], []
    for ss in sets:
        axis += list(ss.axis)
        pos += list(ss.positions)
        types += list(ss.types)
    st = Structures(axis, pos, types)
    n_st_dataset = [len(ss.types) for ss in sets]
    e, f, s, n, fbegin, sbegin, n_data = row_layout_datasets(n_st_dataset, force_dataset, st.n_atoms)
    x = ref.features_x(p, st, e, f, s, n)
    sig = x_signature(x)
    np.savez_compressed(os.path.join(HERE, f"x_{tag}.npz"), params=to_json(p), axis=st.axis, positions=st.positions,
                        types=st.types, n_atoms=st.n_atoms, shape=np.array(x.shape), n_st_dataset=n_st_dataset,
                        force_dataset=np.array(force_dataset), fbegin=fbegin, sbegin=sbegin, n_data=n_data, **sig)
    print("wrote", tag, x.shape)


def write_eval(p, coeffs, sset, tag):
    st = Structures(sset.axis, sset.positions, sset.types)
    e, f, s = ref.evaluate(p, coeffs, st)
    np.savez_compressed(os.path.join(HERE, f"eval_{tag}.npz"), params=to_json(p), axis=st.axis,
                        positions=st.positions, types=st.types, n_atoms=st.n_atoms, coeffs=coeffs, energy=e,
                        forces=f, stress=s)
    print("wrote eval", tag)


def main():
    if not ref.available():
        raise SystemExit("oracle/_ref is not built (make -C oracle ref)")
    write_gtinv()
    write_x("cfg1", params("cfg1"), syn.fcc_set(4, seed=1), "cfg1")
    write_x("cfg2", params("cfg2"), syn.binary_set(2, seed=2), "cfg2")
    pair = make_params_dict(n_type=2, cutoff=6.0, model_type=2, max_p=3, feature_type="pair",
                            gaussian_params2=(0.0, 5.0, 6))
    write_x("pair", pair, syn.binary_set(2, seed=7, n_min=16, n_max=32), "pair_mt2_p3")
    tri = syn.ternary_set(3, seed=3, n_range=(8, 40))
    write_x("cfg3", params("cfg3"), tri, "cfg3")
    # the order-4 ternary model (F = 21,945) on two cells of its own family
    write_x("cfg5p", params("cfg5p"), syn.ternary_set(2, seed=5, n_range=(32, 40)), "cfg5p")
    # PotentialModel: three datasets, the middle one without forces
    write_potential_model(params("cfg2"), [syn.binary_set(2, seed=11), syn.binary_set(3, seed=12),
                                           syn.binary_set(1, seed=13)], [True, False, True], "potential_model")
    rng = np.random.default_rng(42)
    p2 = params("cfg2")
    c2 = rng.normal(size=ref.n_features(p2)) * 1e-3
    write_eval(p2, c2, syn.binary_set(2, seed=9), "cfg2")
    cp = rng.normal(size=ref.n_features(pair)) * 1e-2
    write_eval(pair, cp, syn.binary_set(2, seed=10, n_min=16, n_max=32), "pair")


if __name__ == "__main__":
    main()
