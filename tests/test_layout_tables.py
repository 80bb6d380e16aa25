"""CPU tests of the host-built X-row layout tables (pypolymlp_gb300/csrc/host):
compiled with g++ together with tests/layout_checks.cpp, no GPU."""

import ctypes as C
import os
import subprocess

import pytest

from pypolymlp_gb300.abi import FeatureParams
from pypolymlp_gb300.params import make_params_dict

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(REPO, "pypolymlp_gb300", "csrc")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("layout") / "liblayout_checks.so")
    srcs = [os.path.join(REPO, "tests", "layout_checks.cpp")] + [
        os.path.join(CSRC, "host", f) for f in ("params.cpp", "model_tables.cpp", "flat_tables.cpp")]
    subprocess.run(["g++", "-O1", "-std=c++17", "-shared", "-fPIC", "-ffp-contract=off", "-I", CSRC, "-I",
                    os.path.join(REPO, "include"), *srcs, "-o", out], check=True)
    lib = C.CDLL(out)
    lib.check_layout.argtypes = [C.c_void_p, C.c_char_p, C.c_int]
    return lib


@pytest.mark.parametrize("kw", [
    dict(n_type=2, cutoff=7.0, model_type=3, max_p=2, gaussian_params2=(0.0, 5.0, 10), gtinv_order=3,
         gtinv_maxl=(8, 4)),
    dict(n_type=3, cutoff=6.0, model_type=3, max_p=2, gaussian_params2=(0.0, 5.0, 8), gtinv_order=3,
         gtinv_maxl=(6, 4)),
    dict(n_type=1, cutoff=6.0, model_type=2, max_p=2, gaussian_params2=(0.0, 5.0, 8), gtinv_order=2,
         gtinv_maxl=(4,)),
    dict(n_type=2, cutoff=6.0, model_type=2, max_p=3, gaussian_params2=(0.0, 5.0, 6), gtinv_order=2,
         gtinv_maxl=(4,)),
], ids=["binary", "ternary", "unary", "binary_p3"])
def test_layout_tables(checker, kw):
    fp = FeatureParams(make_params_dict(**kw))
    msg = C.create_string_buffer(512)
    rc = checker.check_layout(C.cast(fp.ref(), C.c_void_p), msg, 512)
    assert rc == 0, msg.value.decode()
    print(msg.value.decode())
