"""CPU checks of the C ABI: the built library loads and exports every
function include/*.h declares (no compute call: there may be no GPU)."""
import ctypes
import re
from pathlib import Path

import pytest

from fedm_loader import PKG, build

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(fedm_[a-z_0-9]+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    path = build.build()
    return ctypes.CDLL(str(path))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("fedm_create", "fedm_run_command", "fedm_run_task", "fedm_free_result"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_create_without_device_fails_cleanly(lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    rc = lib.fedm_create(0, ctypes.byref(h))
    assert rc != 0 and not h.value


def _struct_fields(text, name):
    body = re.search(r"typedef struct " + name + r" \{(.*?)\} " + name + ";", text, flags=re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    fields = []
    for decl in body.split(";"):
        # "int a, b" declares a and b; the name is the last word of each part
        fields += [part.split()[-1].lstrip("*") for part in decl.split(",") if part.strip()]
    return fields


@pytest.mark.parametrize("struct, pyname", [("fedm_result", "Result"), ("fedm_timing", "Timing")])
def test_python_structs_follow_the_header(struct, pyname):
    """The ctypes mirrors in edm.py list the header's fields in its order."""
    from fedm_loader import fedm
    text = (ROOT / "include" / "fastedm_gb300.h").read_text()
    want = _struct_fields(text, struct)
    got = [f for f, _ in getattr(fedm, pyname)._fields_]
    assert got == want


def test_result_to_dict_splits_saved_manifolds():
    """saveManifolds: per task a row-major library block (rows x cols) and a
    prediction block, concatenated in task order, become the lists Ms / Mps."""
    from fedm_loader import fedm
    rows = (ctypes.c_int * 2)(3, 0)
    prows = (ctypes.c_int * 2)(2, 1)
    cols = (ctypes.c_int * 2)(2, 3)
    man = (ctypes.c_double * 6)(*range(6))
    pman = (ctypes.c_double * 7)(*[10 + v for v in range(7)])
    r = fedm.Result()
    r.rc, r.n_stats, r.kmin, r.kmax = 0, 0, -(2**31), -(2**31)
    r.missing_distance = r.dt_weight = float("nan")
    r.n_manifolds = 2
    r.manifold_rows = ctypes.cast(rows, ctypes.POINTER(ctypes.c_int))
    r.pred_manifold_rows = ctypes.cast(prows, ctypes.POINTER(ctypes.c_int))
    r.manifold_cols = ctypes.cast(cols, ctypes.POINTER(ctypes.c_int))
    r.manifolds = ctypes.cast(man, ctypes.POINTER(ctypes.c_double))
    r.pred_manifolds = ctypes.cast(pman, ctypes.POINTER(ctypes.c_double))
    d = fedm.result_to_dict(r)
    assert [m.shape for m in d["Ms"]] == [(3, 2), (0, 3)]
    assert [m.shape for m in d["Mps"]] == [(2, 2), (1, 3)]
    assert d["Ms"][0].tolist() == [[0, 1], [2, 3], [4, 5]]
    assert d["Mps"][0].tolist() == [[10, 11], [12, 13]] and d["Mps"][1].tolist() == [[14, 15, 16]]
