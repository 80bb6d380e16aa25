import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(REPO, "tests", "golden")
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built extension")
    config.addinivalue_line("markers", "slow: CPU check of minutes; runs with PYPOLYMLP_SLOW=1")


def pytest_collection_modifyitems(config, items):
    if os.environ.get("PYPOLYMLP_SLOW") == "1":
        return
    skip = pytest.mark.skip(reason="slow CPU check (set PYPOLYMLP_SLOW=1 to run it)")
    for item in items:
        if "slow" in item.keywords:
            item.add_marker(skip)


def load_golden(name):
    from pypolymlp_gb300.abi import Structures
    from pypolymlp_gb300.params import from_json

    d = np.load(os.path.join(GOLDEN, name), allow_pickle=False)
    params = from_json(str(d["params"]))
    n_atoms = d["n_atoms"]
    off = np.concatenate([[0], np.cumsum(n_atoms)])
    pos = d["positions"]
    types = d["types"]
    st = Structures(d["axis"], [pos[off[i]:off[i + 1]] for i in range(len(n_atoms))],
                    [types[off[i]:off[i + 1]] for i in range(len(n_atoms))])
    return params, st, d


def x_signature(x, seed=12345, n_proj=16, n_sample=4096):
    rng = np.random.default_rng(seed)
    R = rng.standard_normal((x.shape[1], n_proj))
    idx = rng.integers(0, x.size, n_sample)
    return {"colsum": x.sum(axis=0), "rowsum": x.sum(axis=1), "proj": x @ R, "sample_idx": idx,
            "sample": x.reshape(-1, order="F")[idx], "colmax": np.abs(x).max(axis=0)}


def assert_signature(x, gold, rtol):
    """X against a reference signature.  Errors are scaled by the column (or
    row/projection) magnitude, since single elements can cancel to ~0."""
    sig = x_signature(x)
    colmax_raw = gold["colmax"]
    scale_all = np.abs(colmax_raw).max()
    # columns that vanish up to rounding carry only noise: floor at 1e-4 of max|X|
    colmax = np.maximum(colmax_raw, 1e-4 * scale_all)
    np.testing.assert_array_equal(np.asarray(x.shape), gold["shape"])
    # sampled elements: relative to their column magnitude
    idx = gold["sample_idx"]
    cols = idx // x.shape[0]
    err = np.abs(sig["sample"] - gold["sample"]) / np.maximum(colmax[cols], 1e-300)
    assert err.max() <= rtol, f"sampled elements: max rel err {err.max():.3e} > {rtol}"
    n_rows = x.shape[0]
    cs_scale = np.maximum(np.abs(colmax) * n_rows, 1e-300)
    err = np.abs(sig["colsum"] - gold["colsum"]) / cs_scale
    assert err.max() <= rtol, f"column sums: max rel err {err.max():.3e}"
    rs_scale = np.maximum(np.abs(x).sum(axis=1), 1e-300)
    err = np.abs(sig["rowsum"] - gold["rowsum"]) / rs_scale
    assert err.max() <= rtol * 10, f"row sums: max rel err {err.max():.3e}"
    pr_scale = (np.abs(x) @ np.abs(np.random.default_rng(12345).standard_normal((x.shape[1], 16)))) + 1e-300
    err = np.abs(sig["proj"] - gold["proj"]) / pr_scale
    assert err.max() <= rtol * 10, f"projections: max rel err {err.max():.3e}"
    return scale_all


def have_gpu():
    try:
        from pypolymlp_gb300 import _ffi

        return _ffi.device_count() > 0
    except Exception:
        return False
