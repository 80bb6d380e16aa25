"""The libmlpcpp drop-ins and the stream of the C ABI, on the GPU.

* compat.PotentialModel, called exactly as mlp_dev/core/features.py:120 calls
  libmlpcpp.PotentialModel (params dict, per-structure 3 x 3 axes, 3 x N
  positions, types, structures per dataset, force flags per dataset, atoms
  per structure), on three datasets with the middle one energy-only: X
  against the reference build's X of the same structures in PotentialModel's
  row layout (tests/golden/x_potential_model.npz, 1e-10 of the column
  magnitude), the first force/stress rows per dataset and n_data against the
  fixture, and get_x writable in Fortran order as the reference's view is.
* pg_set_stream: the entry points run on a caller's non-blocking torch stream,
  give the same results there, and are ordered after the caller's work on
  that stream (a 50 ms device sleep queued on it before the call delays the
  call's return).
"""

import time

import numpy as np
import pytest

from conftest import assert_signature, load_golden

pytestmark = pytest.mark.gpu


def test_potential_model_matches_reference_layout_and_rows():
    from pypolymlp_gb300.compat import PotentialModel

    params, st, gold = load_golden("x_potential_model.npz")
    offs = st.atom_offsets
    pos = st.positions.reshape(-1, 3)
    axis = [np.array(a) for a in st.axis]
    positions_c = [pos[offs[i]:offs[i + 1]].T.copy() for i in range(st.n_st)]
    types = [st.types[offs[i]:offs[i + 1]].copy() for i in range(st.n_st)]
    pm = PotentialModel(params, axis, positions_c, types, list(gold["n_st_dataset"]),
                        [bool(b) for b in gold["force_dataset"]], list(st.n_atoms))
    x = pm.get_x()
    assert x.flags["F_CONTIGUOUS"] and x.flags["WRITEABLE"] and x.dtype == np.float64
    assert_signature(x, gold, rtol=1e-10)
    assert pm.get_fbegin() == list(gold["fbegin"])
    assert pm.get_sbegin() == list(gold["sbegin"])
    assert pm.get_n_data() == list(gold["n_data"])
    assert pm.get_fbegin()[1] == -1 and pm.get_sbegin()[1] == -1  # energy-only dataset
    x *= 2.0  # the caller scales rows in place (utils_weights.py:76-92)
    assert pm.get_x()[0, 0] == x[0, 0]


def _x_case():
    from pypolymlp_gb300 import synthetic as syn
    from pypolymlp_gb300.abi import Structures, row_layout
    from pypolymlp_gb300.params import make_params_dict

    p = make_params_dict(n_type=2, cutoff=6.0, model_type=3, max_p=2, gaussian_params2=(0.0, 5.0, 6),
                         gtinv_order=3, gtinv_maxl=(6, 4))
    ss = syn.binary_set(4, seed=21)
    st = Structures(ss.axis, ss.positions, ss.types)
    return p, st, row_layout(st.n_atoms, [True] * st.n_st)


def test_entry_points_on_a_caller_stream_give_the_same_results():
    import torch

    from pypolymlp_gb300 import _ffi
    from pypolymlp_gb300.regression import solver_ridge

    p, st, (e, f, s, n) = _x_case()
    m = _ffi.Model(p)
    coefs = np.random.default_rng(1).normal(size=m.n_features) * 1e-3
    ref = {"x64": m.features_x(st, e, f, s, n, precision=_ffi.PG_FP64),
           "x32": m.features_x(st, e, f, s, n, precision=_ffi.PG_MIXED),
           "eval": _ffi.Evaluator(p, coefs, _ffi.PG_FP64).run(st)}
    xg = ref["x64"][:, :200]
    ref["gram"] = _ffi.gram_xtx(xg, _ffi.PG_MIXED)
    A = xg.T @ xg
    ref["solve"] = solver_ridge(A, xg.T @ np.ones(len(xg)), [1e-2, 1e-1])[0]
    for stream in (torch.cuda.Stream(), torch.cuda.Stream(priority=-1)):
        with _ffi.on_stream(stream):
            assert _ffi.get_stream() == stream.cuda_stream
            np.testing.assert_array_equal(m.features_x(st, e, f, s, n, precision=_ffi.PG_FP64), ref["x64"])
            np.testing.assert_array_equal(m.features_x(st, e, f, s, n, precision=_ffi.PG_MIXED), ref["x32"])
            for a, b in zip(_ffi.Evaluator(p, coefs, _ffi.PG_FP64).run(st), ref["eval"]):
                np.testing.assert_array_equal(a, b)
            np.testing.assert_array_equal(_ffi.gram_xtx(xg, _ffi.PG_MIXED), ref["gram"])
            np.testing.assert_array_equal(solver_ridge(A, xg.T @ np.ones(len(xg)), [1e-2, 1e-1])[0], ref["solve"])
    assert _ffi.get_stream() == 0


def test_calls_are_ordered_after_the_callers_work_on_its_stream():
    import torch

    from pypolymlp_gb300 import _ffi

    p, st, (e, f, s, n) = _x_case()
    m = _ffi.Model(p)
    m.features_x(st, e, f, s, n, precision=_ffi.PG_MIXED)  # warm-up
    torch.cuda.synchronize()
    # cycles for ~50 ms of device time at the current clock
    probe = torch.cuda.Stream()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(probe):
        ev0.record()
        torch.cuda._sleep(20_000_000)
        ev1.record()
    probe.synchronize()
    cycles = int(20_000_000 * 50.0 / ev0.elapsed_time(ev1))

    def call_time(sleep):
        caller = torch.cuda.Stream()
        if sleep:
            with torch.cuda.stream(caller):
                torch.cuda._sleep(cycles)
        t = time.time()
        with _ffi.on_stream(caller):
            m.features_x(st, e, f, s, n, precision=_ffi.PG_MIXED)
        dt = time.time() - t
        caller.synchronize()
        return dt

    plain = min(call_time(False) for _ in range(3))
    delayed = call_time(True)
    # the call returns only after the caller's queued 50 ms on that stream
    assert delayed >= plain + 0.025, (plain, delayed)
