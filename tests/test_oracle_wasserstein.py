"""The oracle's Wasserstein transport cost against the reference's own solver.

The reference takes the cost from EMD_wrap (src/vendor/EMD_wrapper.h, POT's
network simplex); the oracle restates it with an independent exact method
(Hungarian assignment).  tests/golden/wasserstein_emd.json holds the
reference's costs on seeded cases, recorded by
tests/golden/make_wasserstein_goldens.py from the reference compiled in place
(oracle/_ref).  Equal lengths must give the reference's bits (its flows are
exactly 1/n) unless several plans are optimal (the same total summed in
another order, within 1e-15); unequal lengths agree to the rounding of the
network simplex's own flows (1e-14).  Where oracle/_ref is built, the same comparison also runs live on
more cases.
"""
import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest

import edm_oracle
from golden.wasserstein_cases import cases, tied

HERE = Path(__file__).resolve().parent
REF = HERE.parent / "oracle" / "_ref" / "libref_emd.so"
UNEQUAL_RTOL = 1e-14
TIED_RTOL = 1e-15


def _check(n1, n2, want, got, ties=False):
    if n1 == n2 and not ties:
        assert got == want, (n1, n2, got.hex(), want.hex())
    else:
        rtol = UNEQUAL_RTOL if n1 != n2 else TIED_RTOL
        assert abs(got - want) <= rtol * abs(want), (n1, n2, got, want)


def test_oracle_transport_cost_is_the_references():
    golden = json.loads((HERE / "golden" / "wasserstein_emd.json").read_text())["costs"]
    cs = cases()
    assert len(cs) == len(golden)
    for i, ((n1, n2, D), h) in enumerate(zip(cs, golden)):
        _check(n1, n2, float.fromhex(h), edm_oracle.emd_uniform(np.array(D).reshape(n1, n2)), tied(i))


@pytest.mark.skipif(not REF.exists(), reason="the reference checkout is not here (oracle/_ref not built)")
def test_oracle_transport_cost_against_the_reference_live():
    lib = C.CDLL(str(REF))
    lib.ref_emd_uniform.restype = C.c_double
    lib.ref_emd_uniform.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p]
    rng = np.random.default_rng(5)
    for n1 in range(1, 11):
        for n2 in range(1, 11):
            for _ in range(20):
                D = np.ascontiguousarray(rng.random((n1, n2)) * 10.0 ** rng.integers(-3, 4))
                ret = C.c_int()
                want = lib.ref_emd_uniform(D.ctypes.data, n1, n2, C.byref(ret))
                assert ret.value == 1
                _check(n1, n2, want, edm_oracle.emd_uniform(D))
