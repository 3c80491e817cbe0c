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
