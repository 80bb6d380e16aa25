"""CPU tests: the C ABI library loads and exports every declared entry point,
and the host-side logic (parameter packing, row layout, weights, scales,
structure sharding) behaves as the reference's code it restates."""

import os
import re

import numpy as np
import pytest

from pypolymlp_gb300 import synthetic as syn
from pypolymlp_gb300.abi import FeatureParams, Structures, row_layout, row_layout_datasets
from pypolymlp_gb300.params import from_json, make_params_dict, to_json

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_functions():
    src = open(os.path.join(REPO, "include", "polymlp_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\bint\s+(pg_\w+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    import ctypes

    from pypolymlp_gb300 import build

    if not os.path.exists(build.LIB):
        build.build()
    lib = ctypes.CDLL(build.LIB)
    names = _declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_device_count_without_compute():
    from pypolymlp_gb300 import _ffi

    assert _ffi.device_count() >= 0


def test_last_error_reports_bad_arguments():
    """A null handle is rejected with a status and a message, not a crash."""
    import ctypes

    from pypolymlp_gb300 import _ffi

    L = _ffi.lib()
    assert L.pg_model_n_features(None, ctypes.byref(ctypes.c_int())) != 0
    buf = ctypes.create_string_buffer(256)
    L.pg_last_error(buf, 256)
    assert buf.value


def test_feature_params_packing():
    """cond_pair offsets follow the (i, j), i <= j row-major order of the
    reference's type-pair list; gtinv tables are flattened with running offsets."""
    p = make_params_dict(n_type=2, cutoff=6.0, model_type=3, max_p=2, gaussian_params2=(0.0, 5.0, 4),
                         gtinv_order=3, gtinv_maxl=(4, 2))
    fp = FeatureParams(p)
    s = fp.struct
    m = p["model"]
    assert s.n_type == 2 and s.feature_type == 1 and s.model_type == 3 and s.max_p == 2
    assert s.max_l == 4 and abs(s.cutoff - 6.0) < 1e-15 and s.n_fn == len(m["pair_params"])
    # (i, j) i <= j row-major: 3 type pairs for 2 types, offsets non-decreasing
    offs = [s.cond_offsets[q] for q in range(4)]
    assert offs[0] == 0 and offs == sorted(offs)
    assert s.n_lcomb > 0 and s.lcomb_offsets[s.n_lcomb] > 0
    # the JSON round trip keeps the packed form
    fq = FeatureParams(from_json(to_json(p))).struct
    assert (fq.n_lcomb, fq.n_fn, fq.max_l) == (s.n_lcomb, s.n_fn, s.max_l)
    assert [fq.cond_offsets[q] for q in range(4)] == offs


def test_row_layout_matches_reference_indexing():
    """Energies first, then 6 stress rows per force structure, then 3N force
    rows (PyModel::set_index, compute/py_model.cpp:58-106)."""
    n_atoms = [2, 3, 1]
    force = [True, False, True]
    e, f, s, n = row_layout(n_atoms, force)
    assert list(e) == [0, 1, 2]
    assert list(s) == [3, -1, 9]
    assert list(f) == [15, -1, 21]
    assert n == 3 + 12 + 3 * 3


def test_row_layout_datasets_begins():
    """Two datasets, the second without forces (PyModel::set_index)."""
    e, f, s, n, fbegin, sbegin, n_data = row_layout_datasets([2, 1], [True, False], [2, 3, 1])
    assert n == 3 + 6 * 2 + 3 * 5
    assert list(e) == [0, 1, 2]
    assert list(s) == [3, 9, -1] and list(f) == [15, 21, -1]
    assert list(sbegin) == [3, -1] and list(fbegin) == [15, -1]
    assert list(n_data) == [3, 15, 12]


def test_weights_and_scales_restatement():
    """apply_weights / compute_scales semantics on a small synthetic dataset."""
    from pypolymlp_gb300.regression import Dataset, compute_scales, get_min_energy, weights_and_targets

    ss = syn.binary_set(3, seed=5, n_min=8, n_max=16)
    syn.morse_labels(ss, syn.morse_D(2), device=None)
    d = Dataset.from_structure_set(ss)
    min_e = get_min_energy([d])
    assert np.isclose(min_e, min(np.asarray(d.energies) / np.array([len(t) for t in d.types])))
    e_row, f_row, s_row, n_rows, w, y = weights_and_targets(d, min_e)
    assert len(w) == len(y) == n_rows
    assert np.all(w >= 0) and np.all(np.isfinite(y))
    # columns: variance 2/3, constant (variance 0 -> zeroed, scale 1), variance 2/3
    xe_sum = np.array([3.0, 6.0, 6.0])
    xe_sq = np.array([5.0, 12.0, 14.0])
    scales, zero = compute_scales(None, xe_sum, xe_sq, 3, True)
    assert list(np.flatnonzero(zero)) == [1]
    np.testing.assert_allclose(scales, [np.sqrt(2 / 3), 1.0, np.sqrt(2 / 3)], rtol=1e-12)


def test_shard_ranges_cover_and_balance():
    from pypolymlp_gb300.distributed import shard_ranges, structure_rows

    rng = np.random.default_rng(3)
    n_atoms = rng.integers(8, 129, size=101)
    rows = structure_rows(n_atoms)
    for world in (1, 2, 3, 8):
        rg = shard_ranges(rows, world)
        assert rg[0][0] == 0 and rg[-1][1] == len(rows)
        assert all(a[1] == b[0] for a, b in zip(rg, rg[1:]))
        loads = [rows[a:b].sum() for a, b in rg]
        assert max(loads) - min(loads) <= 2 * rows.max()


def _gloo_worker(rank, world, port, result_path):
    import torch.distributed as dist

    from pypolymlp_gb300.distributed import allreduce_gram, shard_ranges

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    rng = np.random.default_rng(11)
    X = rng.normal(size=(40, 6))
    y = rng.normal(size=40)
    rows_per_struct = np.full(10, 4)
    a, b = shard_ranges(rows_per_struct, world)[rank]
    Xs, ys = X[4 * a:4 * b], y[4 * a:4 * b]
    part = (Xs.T @ Xs, Xs.T @ ys, float(ys @ ys), Xs.sum(0), (Xs ** 2).sum(0), len(ys))
    xtx, xty, yty, xe, xq, n = allreduce_gram(part)
    if rank == 0:
        np.savez(result_path, xtx=xtx, xty=xty, yty=yty, xe=xe, xq=xq, n=n, X=X, y=y)
    dist.destroy_process_group()


def test_gram_allreduce_two_gloo_ranks(tmp_path):
    """Two CPU ranks (gloo) each reduce a shard; the all-reduced sums equal the
    single-process X^T X, X^T y, y^T y and column sums."""
    import socket

    import torch.multiprocessing as mp

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = str(tmp_path / "r.npz")
    mp.spawn(_gloo_worker, args=(2, port, out), nprocs=2, join=True)
    r = np.load(out)
    X, y = r["X"], r["y"]
    np.testing.assert_allclose(r["xtx"], X.T @ X, rtol=1e-12)
    np.testing.assert_allclose(r["xty"], X.T @ y, rtol=1e-12)
    assert np.isclose(float(r["yty"]), y @ y)
    np.testing.assert_allclose(r["xe"], X.sum(0), rtol=1e-12)
    assert int(r["n"]) == 40
