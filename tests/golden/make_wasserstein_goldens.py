"""Records the reference's own transport costs into wasserstein_emd.json.

The reference's Wasserstein distance takes its cost from EMD_wrap
(src/vendor/EMD_wrapper.h of EDM-Developers/fastEDM-r, POT's network simplex,
header-only).  oracle/Makefile compiles it in place, where the reference
checkout exists, into oracle/_ref/libref_emd.so; this script runs it on the
seeded cases of wasserstein_cases.py with the masses the reference passes
(1/n1, 1/n2) and stores each cost as a hexadecimal float.

    make -C oracle && python tests/golden/make_wasserstein_goldens.py
"""
import ctypes as C
import json
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
from wasserstein_cases import cases  # noqa: E402


def main():
    lib = C.CDLL(str(HERE.parent.parent / "oracle" / "_ref" / "libref_emd.so"))
    lib.ref_emd_uniform.restype = C.c_double
    lib.ref_emd_uniform.argtypes = [C.POINTER(C.c_double), C.c_int, C.c_int, C.POINTER(C.c_int)]
    out = []
    for n1, n2, D in cases():
        arr = (C.c_double * len(D))(*D)
        ret = C.c_int()
        cost = lib.ref_emd_uniform(arr, n1, n2, C.byref(ret))
        assert ret.value == 1, (n1, n2, ret.value)  # OPTIMAL
        out.append(float(cost).hex())
    (HERE / "wasserstein_emd.json").write_text(json.dumps({"generator": "wasserstein_cases.cases()", "costs": out}))


if __name__ == "__main__":
    main()
