"""pg_solve_ridge_noalloc: the ridge solve for callers that cannot allocate.

Some callers of this library cannot allocate GPU memory when they need a
solve - a server or framework whose own allocator owns the device's memory.
They own the input and output buffers; the entry point keeps its factor
workspace in a fixed array inside the library.  This test drives it through the C ABI with device buffers the
test allocates (with torch), and checks it against pg_solve_ridge, the
allocating entry point, on two calls in a row: the second call must not be
disturbed by what the first left in the shared array.  It lives in its own
file, collected last, and passes alone in a fresh process too.
"""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-8  # the tolerance of the ridge-solve tests


def _spd(F, seed):
    rng = np.random.default_rng(seed)
    B = rng.normal(size=(F + 17, F))
    return np.asfortranarray(B.T @ B), rng.normal(size=F)


def _noalloc(A, b, alpha):
    import torch

    from pypolymlp_gb300 import _ffi

    F = A.shape[0]
    dA = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()  # row-major of A^T == column-major of A
    db = torch.from_numpy(b.copy()).cuda()
    dx = torch.empty(F, dtype=torch.float64, device="cuda")
    info = C.c_int(-1)
    torch.cuda.synchronize()
    _ffi.check(_ffi.lib().pg_solve_ridge_noalloc(F, C.c_void_p(dA.data_ptr()), C.c_void_p(db.data_ptr()),
                                                 C.c_double(alpha), C.c_void_p(dx.data_ptr()), C.byref(info)))
    return dx.cpu().numpy(), info.value


def test_noalloc_matches_allocating_solve_twice():
    from pypolymlp_gb300.regression import solver_ridge

    # the largest size the fixed array holds, then a smaller call after it
    cases = [(_spd(1024, 1), 1e-2), (_spd(700, 3), 1e-2), (_spd(300, 2), 1e-3)]
    for (A, b), alpha in cases:
        ref, info_ref = solver_ridge(A, b, [alpha])
        got, info = _noalloc(A, b, alpha)
        assert info == 0 and info_ref[0] == 0
        assert np.abs(got - ref[:, 0]).max() <= RTOL * np.abs(ref).max()


def test_noalloc_reports_failure_and_rejects_oversize():
    from pypolymlp_gb300 import _ffi

    got, info = _noalloc(np.asfortranarray(-np.eye(16)), np.ones(16), 1e-3)
    assert info != 0 and np.all(got == 1e30)
    with pytest.raises(_ffi.GB300Error, match="exceeds the maximum"):
        _ffi.check(_ffi.lib().pg_solve_ridge_noalloc(1025, C.c_void_p(1), C.c_void_p(1), C.c_double(0.1),
                                                     C.c_void_p(1), C.byref(C.c_int())))
